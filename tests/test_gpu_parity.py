"""GPU: the CUDA library (through its C ABI) against the golden fixtures of the
compiled reference and against the oracle restatement, stage by stage."""
import numpy as np
import pytest

import golden_cases as gc
import oracle_runner as orr
from parafrost_gb300 import build, cnfgen, rounddump as rd
from parafrost_gb300.options import Options
from parafrost_gb300.sigma import PF_EINVAL, PF_ESTATE, SigmaError, Simplifier
from test_emu import CASES, SUB_RERUN, run_lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(gc.index()))
def test_gpu_golden(cuda_lib, name):
    meta, arrays, (nv, lits, off), opts = gc.load(name)
    stats, recs, _ = run_lib(cuda_lib, nv, lits, off, opts, level=1, learnt=gc.learnt_mask(meta, off))
    assert stats.status == meta["status"]
    assert gc.check(meta, arrays, recs) == []


@pytest.mark.parametrize("seed", [21, 22])
@pytest.mark.parametrize("case", [c[0] for c in CASES])
@pytest.mark.parametrize("opt", [dict(all=1), dict(all=1, gc_freq=1, mu_pos=10, mu_neg=10), dict()])
def test_gpu_stagewise_vs_oracle(cuda_lib, built, case, seed, opt):
    nv, lits, off = dict(CASES)[case](seed)
    opts = Options(**opt)
    st, a, _ = orr.run_oracle(nv, lits, off, opts, level=2)
    stats, b, _ = run_lib(cuda_lib, nv, lits, off, opts, level=2)
    assert stats.status == st
    assert rd.compare(rd.normalize(a), rd.normalize(b)) == []


@pytest.mark.parametrize("gen", [
    lambda: cnfgen.aig_tseitin(num_inputs=5000, num_and=200_000, num_xor=20_000, seed=5),
    lambda: cnfgen.community(num_vars=200_000, num_clauses=800_000, seed=6),
    lambda: cnfgen.random_ksat(100_000, 426_000, 3, seed=7),
    lambda: cnfgen.random_mixed_ksat(300_000, 3.5, seed=8),
])
def test_gpu_canonical_medium(cuda_lib, built, gen):
    """Medium formulas: final canonical state equal to the oracle's."""
    nv, lits, off = gen()
    opts = Options(all=1)
    st, a, _ = orr.run_oracle(nv, lits, off, opts, level=1)
    stats, b, res = run_lib(cuda_lib, nv, lits, off, opts, level=1)
    assert stats.status == st
    assert rd.canonical(a) == rd.canonical(b)
    assert rd.compare(a, b, kinds=("pvs", "counts", "elim")) == []


def test_gpu_download_matches_dump(cuda_lib):
    nv, lits, off = cnfgen.random_ksat(2000, 8520, 3, seed=3)
    stats, recs, res = run_lib(cuda_lib, nv, lits, off, Options(all=1), level=1)
    fin = rd.final_state(recs)
    live = [lits_ for (f, _, lits_) in rd.cnf_clauses(fin["cnf"]) if (f & 3) != 2]
    assert res.clauses() == live
    assert np.array_equal(res.resolved, fin["resolved"])
    assert sorted(res.units.tolist()) == sorted(fin["trail"].tolist())
    assert np.nonzero(res.eliminated)[0].tolist() == fin["elim"].tolist()


def test_gpu_invalid_input(cuda_lib):
    with Simplifier(Options(all=1)) as s:
        with pytest.raises(SigmaError) as e:
            s.sigmify()
        assert e.value.status == PF_ESTATE
        bad = np.array([2, 4, 2], dtype=np.uint32)  # variable 1 repeated
        with pytest.raises(SigmaError) as e:
            s.awaken(3, bad, np.array([0, 3], dtype=np.uint64))
        assert e.value.status == PF_EINVAL
        oob = np.array([2, 40], dtype=np.uint32)  # literal of variable 20 > num_vars
        with pytest.raises(SigmaError) as e:
            s.awaken(3, oob, np.array([0, 2], dtype=np.uint64))
        assert e.value.status == PF_EINVAL


@pytest.mark.parametrize("case", [c[0] for c in SUB_RERUN])
@pytest.mark.parametrize("opt", [dict(all=1, mu_pos=10, mu_neg=10), dict(all=1)])
def test_gpu_sub_rerun(cuda_lib, built, case, opt):
    """The SUB units' fix-point with re-runs, stage by stage against the oracle."""
    nv, lits, off = dict(SUB_RERUN)[case]()
    opts = Options(**opt)
    st, a, _ = orr.run_oracle(nv, lits, off, opts, level=2)
    stats, b, _ = run_lib(cuda_lib, nv, lits, off, opts, level=2)
    assert stats.status == st
    assert rd.compare(rd.normalize(a), rd.normalize(b)) == []


@pytest.mark.parametrize("case", [c[0] for c in CASES])
def test_gpu_stagewise_bucketed_ot(cuda_lib, built, case):
    """The literal-bucket occurrence-table build (chosen by size for large formulas)
    forced on every formula, stage by stage against the oracle."""
    nv, lits, off = dict(CASES)[case](23)
    st, a, _ = orr.run_oracle(nv, lits, off, Options(all=1), level=2)
    stats, b, _ = run_lib(cuda_lib, nv, lits, off, Options(all=1, ot_buckets=1), level=2)
    assert stats.status == st
    assert rd.compare(rd.normalize(a), rd.normalize(b)) == []


@pytest.mark.parametrize("gen", [
    lambda: cnfgen.community(num_vars=200_000, num_clauses=800_000, seed=6),
    lambda: cnfgen.aig_tseitin(num_inputs=5000, num_and=200_000, num_xor=20_000, seed=5),
])
def test_gpu_canonical_bucketed_ot(cuda_lib, built, gen):
    nv, lits, off = gen()
    st, a, _ = orr.run_oracle(nv, lits, off, Options(all=1), level=1)
    stats, b, _ = run_lib(cuda_lib, nv, lits, off, Options(all=1, ot_buckets=1), level=1)
    assert stats.status == st
    assert rd.canonical(a) == rd.canonical(b)
    assert rd.compare(a, b, kinds=("pvs", "counts", "elim")) == []
