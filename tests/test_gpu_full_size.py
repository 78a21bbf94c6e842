"""GPU: bit-exact parity at the benchmarked sizes.

The full benchmark formulas go through the CUDA round and through the oracle
restatement (which equals the compiled reference on every golden fixture), and
their final states are compared: the simplified clauses (store order, statuses,
signatures), the witness stack, the eliminated variables, the units (as a set),
the live counts after every phase and the elected variables of every phase.
  * the 6.8M-clause Tseitin AIG (2M AND + 200k XOR gates over 50k inputs);
  * the 80M-clause, 20M-variable community-attachment formula;
  * an AIG round whose last 30% of clauses are learnt (an inprocessing input).
Store order is compared exactly first; a difference there falls back to the
canonical (sorted) clause multiset, the contract's comparison.
"""
import numpy as np
import pytest

import oracle_runner as orr
from parafrost_gb300 import cnfgen, rounddump as rd
from parafrost_gb300.options import Options
from test_emu import run_lib

pytestmark = pytest.mark.gpu


def _same_round(a: list, b: list) -> list:
    """Mismatches between two level-1 dumps of the same round."""
    errs = rd.compare(a, b, kinds=("pvs", "counts", "elim", "status"))
    fa, fb = rd.final_state(a), rd.final_state(b)
    if int(fa["status"][0]) != int(fb["status"][0]):
        return errs + ["status differs"]
    if int(fa["status"][0]) != 0:
        return errs
    for k in ("resolved", "elim"):
        if not np.array_equal(fa[k], fb[k]):
            errs.append(f"final {k} differs")
    if not np.array_equal(np.unique(fa["trail"]), np.unique(fb["trail"])):
        errs.append("final units differ")
    if not np.array_equal(fa["cnf"], fb["cnf"]):
        ca, cb = rd.canonical(a), rd.canonical(b)
        if ca["clauses"] != cb["clauses"]:
            errs.append("final clause multisets differ")
    return errs


def _run_both(lib, nv, lits, off, learnt=None):
    opts = Options(all=1)
    st, want, secs = orr.run_oracle(nv, lits, off, opts, level=1, learnt=learnt)
    stats, got, _ = run_lib(lib, nv, lits, off, opts, level=1, learnt=learnt)
    assert stats.status == st
    return want, got


def test_full_aig_round_equals_oracle(cuda_lib, built):
    nv, lits, off = cnfgen.aig_tseitin(num_inputs=50_000, num_and=2_000_000, num_xor=200_000, seed=1)
    want, got = _run_both(cuda_lib, nv, lits, off)
    assert _same_round(want, got) == []


def test_full_community_round_equals_oracle(cuda_lib, built):
    nv, lits, off = cnfgen.community(seed=1)
    assert off.size - 1 == 80_000_000 and nv == 20_000_000
    want, got = _run_both(cuda_lib, nv, lits, off)
    assert _same_round(want, got) == []


def test_aig_learnt_tail_equals_oracle(cuda_lib, built):
    nv, lits, off = cnfgen.aig_tseitin(num_inputs=5_000, num_and=200_000, num_xor=20_000, seed=11)
    learnt = np.zeros(off.size - 1, dtype=np.uint8)
    learnt[int(learnt.size * 0.7):] = 1
    want, got = _run_both(cuda_lib, nv, lits, off, learnt)
    assert _same_round(want, got) == []
