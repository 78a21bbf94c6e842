"""The library's DIMACS reader (pf_dimacs_parse; ParaFROST::parser,
src/cpu/dimacs.cpp:25-176). CPU: the emulation build exports the same reader."""
import os
import tempfile

import numpy as np
import pytest

import oracle_runner as orr
from parafrost_gb300 import cnfgen, rounddump as rd
from parafrost_gb300.options import Options
from parafrost_gb300.sigma import PF_EINVAL, SigmaError, Simplifier, read_dimacs


def _write(text: str) -> str:
    fd, path = tempfile.mkstemp(suffix=".cnf")
    with os.fdopen(fd, "w") as f:
        f.write(text)
    return path


def test_dimacs_round_trip(built):
    nv, lits, off = cnfgen.random_mixed_ksat(3000, 3.5, seed=4)
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "f.cnf")
        cnfgen.to_dimacs(p, nv, lits, off)
        rnv, rl, ro, empty = read_dimacs(p, library=built["emu"])
    assert rnv == nv and not empty
    assert np.array_equal(ro, off) and np.array_equal(rl, lits)


def test_dimacs_normalisation(built):
    # comments, a repeated literal, a tautology, a unit, clauses over several lines
    p = _write("c a comment\np cnf 5 6\n1 -2 1 0\n2 -2 3 0\n4 0\n-5\n 3 0\nc trailing\n1 2 3 4 5 0\n-1 -3 0\n")
    try:
        nv, lits, off, empty = read_dimacs(p, library=built["emu"])
    finally:
        os.unlink(p)
    clauses = [tuple(lits[off[i]:off[i + 1]].tolist()) for i in range(off.size - 1)]
    assert nv == 5 and not empty
    assert clauses == [(2, 5), (8,), (11, 6), (2, 4, 6, 8, 10), (3, 7)]


def test_dimacs_errors(built):
    for text in ("p cnf 3 1\n1 4 0\n", "1 2 0\n", "p cnf 3 1\n1 2\n", "p cnf 3 1\n1 x 0\n"):
        p = _write(text)
        try:
            with pytest.raises(SigmaError) as e:
                read_dimacs(p, library=built["emu"])
            assert e.value.status == PF_EINVAL
        finally:
            os.unlink(p)
    p = _write("p cnf 3 2\n1 2 0\n0\n")
    try:
        nv, lits, off, empty = read_dimacs(p, library=built["emu"])
    finally:
        os.unlink(p)
    assert empty and off.size == 2


@pytest.mark.skipif(not orr.reference_available(), reason="compiled reference not built here")
def test_dimacs_round_matches_reference(built):
    """A file read by the library and simplified gives the reference's round on
    the same file (the reference reads it with its own parser)."""
    nv, lits, off = cnfgen.aig_tseitin(num_inputs=300, num_and=4000, num_xor=400, seed=8)
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "f.cnf")
        cnfgen.to_dimacs(p, nv, lits, off)
        rnv, rl, ro, _ = read_dimacs(p, library=built["emu"])
    with Simplifier(Options(all=1, dump_level=1), library=built["emu"]) as s:
        s.awaken(rnv, rl, ro)
        s.sigmify()
        with tempfile.TemporaryDirectory() as td:
            dp = os.path.join(td, "d")
            s.write_dump(dp)
            ours = rd.read(dp)
    ref = orr.run_reference(nv, lits, off, Options(all=1), level=1)
    assert rd.canonical(ours) == rd.canonical(ref)
