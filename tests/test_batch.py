"""Formula batches: every formula of a batched round ends exactly as its own round
(the oracle's canonical final state, status and phase count), including formulas
that end UNSAT or have no clauses. CPU: the emulation build; GPU: the CUDA build."""
import numpy as np
import pytest

import oracle_runner as orr
from parafrost_gb300 import cnfgen, rounddump as rd
from parafrost_gb300.options import Options
from parafrost_gb300.sigma import PF_EINVAL, ResultBuffers, SigmaError, Simplifier


def mixed_batch(seed: int, n: int = 14) -> list:
    forms = []
    for i in range(n):
        s = seed * 100 + i
        kind = i % 5
        if kind == 0:
            forms.append(cnfgen.random_ksat(num_vars=200 + 37 * i, num_clauses=850 + 150 * i, k=3, seed=s))
        elif kind == 1:
            forms.append(cnfgen.aig_tseitin(num_inputs=40, num_and=300 + 25 * i, num_xor=30, seed=s))
        elif kind == 2:
            forms.append(cnfgen.random_mixed_ksat(600 + 40 * i, 3.6, seed=s))
        elif kind == 3:
            forms.append(cnfgen.random_ksat(num_vars=90, num_clauses=450, k=2, seed=s))  # mostly UNSAT
        else:
            forms.append(cnfgen.community(num_vars=500, num_clauses=2000, communities=5, seed=s))
    # a formula without clauses
    forms.insert(3, (7, np.empty(0, dtype=np.uint32), np.zeros(1, dtype=np.uint64)))
    return forms


def check_batch(lib, forms, opts, oracle=True):
    b = Simplifier(opts, library=lib)
    b.awaken_batch(forms)
    b.sigmify()
    got = b.batch_results()
    again = b.batch_results(out=ResultBuffers())  # the same through reused buffers
    b.close()
    for (st, _, res), (st2, _, res2) in zip(got, again):
        assert rd.canonical_result(st, res if st == 0 else None) == rd.canonical_result(st2, res2 if st2 == 0 else None)
    assert len(got) == len(forms)
    for i, ((nv, lits, off), (st, ph, res)) in enumerate(zip(forms, got)):
        s = Simplifier(opts, library=lib)
        s.awaken(nv, lits, off)
        one = s.sigmify()
        want = rd.canonical_result(one.status, s.result() if one.status == 0 else None)
        s.close()
        have = rd.canonical_result(st, res if st == 0 else None)
        assert have == want, f"formula {i}"
        assert ph == one.phases_run, f"formula {i}: phases"
        if oracle and off.size > 1:  # the oracle takes formulas with clauses
            ost, recs, _ = orr.run_oracle(nv, lits, off, opts, level=1)
            assert rd.canonical(recs) == have, f"formula {i} vs oracle"


OPTS = [dict(all=1), dict(all=1, phases=2, mu_pos=8, mu_neg=8), dict(all=1, gc_freq=1), dict()]


@pytest.mark.parametrize("opt", OPTS)
def test_batch_emu(built, opt):
    check_batch(built["emu"], mixed_batch(3), Options(**opt))


def test_batch_invalid_literal(built):
    forms = mixed_batch(4, n=3)
    nv, lits, off = forms[1]
    bad = lits.copy()
    bad[0] = 2 * nv + 2  # one past the formula's own variables
    forms[1] = (nv, bad, off)
    b = Simplifier(Options(all=1), library=built["emu"])
    with pytest.raises(SigmaError) as e:
        b.awaken_batch(forms)
    assert e.value.status == PF_EINVAL


@pytest.mark.gpu
@pytest.mark.parametrize("opt", OPTS)
def test_batch_gpu(cuda_lib, built, opt):
    check_batch(cuda_lib, mixed_batch(5), Options(**opt))


@pytest.mark.gpu
def test_batch_gpu_many(cuda_lib):
    """64 random k-SAT formulas with 1k-20k clauses (the batched workload's
    generator at a smaller size) against their own rounds and the oracle."""
    forms = list(cnfgen.batch_ksat(num_formulas=64, cmin=1_000, cmax=20_000, seed=9))
    check_batch(cuda_lib, forms, Options(all=1), oracle=True)


@pytest.mark.gpu
def test_batch_gpu_workload_slice(cuda_lib):
    """64 formulas of the batched benchmark's own generator and sizes (1k-200k
    clauses, k mixed 2-5), every one against the oracle."""
    forms = list(cnfgen.batch_ksat(num_formulas=4096, cmin=1_000, cmax=200_000, seed=1, indices=range(0, 4096, 64)))
    check_batch(cuda_lib, forms, Options(all=1), oracle=True)
