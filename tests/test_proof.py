"""DRAT proof of a round (pf_sigma_proof; the reference's -proof output,
src/cpu/proof.cpp).

* Every addition line follows by unit propagation from the input and the lines
  before it (the oracle's forward RUP checker); an UNSAT round's proof ends with
  the empty clause, so it refutes the formula.
* Against the compiled reference (CPU, where it is built), for a round that ends
  SAT: every line of the reference's proof of the same round (addition and
  deletion lines after the parser's) is in ours, and each extra line of ours
  contains a literal of the round's final units (the reference leaves out an added
  clause that a unit assigned before it satisfies). For a round that ends UNSAT,
  which units are derived before the contradiction depends on the order the units
  propagate in (the reference walks its trail; a sweep wave here checks the whole
  store against the assignment), so both proofs must refute the formula, not hold
  the same lines.
* GPU: the CUDA build's proof holds the same lines as the emulation build's (for
  a round that ends UNSAT, only the refutation is checked: the lines that the
  other variables of the contradicting stage add depend on timing).
"""
from collections import Counter

import numpy as np
import pytest

import oracle_runner as orr
from parafrost_gb300 import cnfgen
from parafrost_gb300.options import Options
from parafrost_gb300.sigma import Simplifier

FORMULAS = {
    "aig_33k": lambda: cnfgen.aig_tseitin(num_inputs=2000, num_and=30_000, num_xor=3000, seed=2),
    "community_80k": lambda: cnfgen.community(num_vars=20_000, num_clauses=80_000, communities=20, seed=3),
    "ksat3_10k": lambda: cnfgen.random_ksat(10_000, 42_600, 3, seed=1),
    "mixed_5k": lambda: cnfgen.random_mixed_ksat(5000, 4.0, seed=1),
    "ksat2_unsat": lambda: cnfgen.random_ksat(300, 600, 2, seed=1),
}


def _proof(lib, nv, lits, off, opts=None):
    with Simplifier(opts or Options(all=1, proof=1), library=lib) as s:
        s.awaken(nv, lits, off)
        st = s.sigmify()
        pr = s.proof()
        units = set(s.result().units.tolist()) if st.status == 0 else set()
    return st.status, pr, units


@pytest.mark.parametrize("name", sorted(FORMULAS))
def test_proof_is_rup_emu(built, name):
    nv, lits, off = FORMULAS[name]()
    status, pr, _ = _proof(built["emu"], nv, lits, off)
    bad, refutes = orr.check_drat(nv, lits, off, pr)
    assert bad == -1, f"line {bad} is not implied"
    assert refutes == (status == 1)


@pytest.mark.skipif(not orr.reference_available(), reason="compiled reference not built here")
@pytest.mark.parametrize("name", sorted(FORMULAS))
@pytest.mark.parametrize("opt", [dict(all=1), dict(all=1, phases=3, mu_pos=10, mu_neg=10, gc_freq=1)])
def test_proof_lines_match_reference(built, name, opt):
    nv, lits, off = FORMULAS[name]()
    status, pr, units = _proof(built["emu"], nv, lits, off, Options(**opt, proof=1))
    _, ref = orr.run_reference(nv, lits, off, Options(**opt), level=1, proof=True)
    ours, theirs = Counter(orr.drat_lines(pr)), Counter(ref)
    if status == 1:
        assert ("a", ()) in theirs, "the reference's proof of an UNSAT round ends with the empty clause"
        bad, refutes = orr.check_drat(nv, lits, off, pr)
        assert bad == -1 and refutes
        return
    assert not (theirs - ours), "a reference line is missing"
    extra = ours - theirs
    assert all(any(x in units for x in lits_) for (_, lits_) in extra), "an extra line is not satisfied"


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(FORMULAS))
def test_proof_gpu(cuda_lib, built, name):
    nv, lits, off = FORMULAS[name]()
    status, pr, _ = _proof(cuda_lib, nv, lits, off)
    bad, refutes = orr.check_drat(nv, lits, off, pr)
    assert bad == -1 and refutes == (status == 1)
    if status == 0:  # after a contradiction, what the stage's other variables add is timing
        _, pe, _ = _proof(built["emu"], nv, lits, off)
        assert Counter(orr.drat_lines(pr)) == Counter(orr.drat_lines(pe))
