"""CPU: the oracle restatement against the reference's golden fixtures."""
import ctypes

import pytest

import golden_cases as gc
import oracle_runner as orr
from make_golden import digest


@pytest.mark.parametrize("name", sorted(gc.index()))
def test_oracle_matches_reference_golden(built, name):
    meta, arrays, (nv, lits, off), opts = gc.load(name)
    assert digest(lits, off) == meta["input_hash"], "generator output changed"
    st, recs, _ = orr.run_oracle(nv, lits, off, opts, level=1, learnt=gc.learnt_mask(meta, off))
    assert st == meta["status"]
    assert gc.check(meta, arrays, recs) == []


def test_introsort_replica_matches_libstdcxx(built):
    lib = orr.oracle_lib()
    lib.oracle_check_introsort.restype = ctypes.c_long
    lib.oracle_check_introsort.argtypes = [ctypes.c_uint64, ctypes.c_int]
    assert lib.oracle_check_introsort(7, 20000) == 0
