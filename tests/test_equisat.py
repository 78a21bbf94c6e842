"""Equisatisfiability through the reference solver (CPU; needs the compiled
reference, oracle/_ref, built where the reference sources are).

For each formula, the round's result (simplified clauses plus units) is solved by
the reference CDCL solver with its own simplifier off. A SAT answer's model, with
the eliminated variables cleared, is extended through the round's witness stack
as the reference's MODEL::extend does (src/cpu/model.cpp:104-138) and must satisfy
every original clause (MODEL::verify, model.cpp:140-212). An UNSAT answer, or a
round that proves UNSAT itself, must agree with the reference solver on the
original formula. The round runs through the kernel-logic emulation build (the
same item functions the CUDA kernels run).
"""
import numpy as np
import pytest

import oracle_runner as orr
from parafrost_gb300 import cnfgen
from parafrost_gb300.options import Options
from parafrost_gb300.sigma import Simplifier

pytestmark = pytest.mark.skipif(not orr.solver_available(), reason="compiled reference solver not built here")

FORMULAS = {
    "aig_33k": lambda: cnfgen.aig_tseitin(num_inputs=2000, num_and=30_000, num_xor=3000, seed=2),
    "aig_unrolled": lambda: cnfgen.aig_unrolled(2000, 8, seed=5),
    "community_80k": lambda: cnfgen.community(num_vars=20_000, num_clauses=80_000, communities=20, seed=3),
    "community_100k": lambda: cnfgen.community(num_vars=25_000, num_clauses=100_000, communities=25, seed=9),
    "ksat3_easy": lambda: cnfgen.random_ksat(5000, 18_000, 3, seed=4),
    "mixed_sat": lambda: cnfgen.random_mixed_ksat(20_000, 3.0, seed=6),
    "ksat3_unsat": lambda: cnfgen.random_ksat(150, 900, 3, seed=3),
    "ksat2_unsat": lambda: cnfgen.random_ksat(300, 600, 2, seed=1),
}


def _round(lib, nv, lits, off, opts):
    with Simplifier(opts, library=lib) as s:
        s.awaken(nv, lits, off)
        st = s.sigmify()
        return st.status, (s.result() if st.status == 0 else None)


@pytest.mark.parametrize("name", sorted(FORMULAS))
@pytest.mark.parametrize("opt", [dict(all=1), dict(all=1, phases=3, mu_pos=8, mu_neg=8, gc_freq=1)])
def test_round_is_equisatisfiable(built, name, opt):
    nv, lits, off = FORMULAS[name]()
    status, res = _round(built["emu"], nv, lits, off, Options(**opt))
    if status != 0:  # the round proved UNSAT: the reference solver must agree
        assert orr.reference_solve(nv, lits, off)[0] == "UNSAT"
        return
    answer, model = orr.reference_solve(nv, res.lits, res.offsets, res.units)
    if answer == "UNSAT":
        assert orr.reference_solve(nv, lits, off)[0] == "UNSAT"
        return
    assert orr.check_models(nv, lits, off, status, res, model) == []
