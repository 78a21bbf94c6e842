"""The drop-in boundary in C++ (CPU; needs the reference sources where it is built):
oracle/_ref/sigma_dropin is the unmodified reference solver whose preprocessing
sigmify round goes through include/sigma_gb300.hpp and the C ABI (here the
emulation build of the library), followed by the reference's own write-back and
CDCL search. Its answer must equal the reference solver's own, and a SAT answer's
model, extended through the witness stack the library produced, must pass the
reference's own MODEL::verify on the input file.

No input here has a clause that earlier one-literal clauses falsify: the
reference's DIMACS parser drops such a clause instead of answering UNSAT
(src/cpu/dimacs.cpp:145-176, a clause left with no literal falls through), so
the reference itself answers SAT with a model that its own verification rejects
(an unrolled AIG whose asserted output is unreachable does this)."""
import os
import re
import subprocess
import tempfile

import pytest

from parafrost_gb300 import build, cnfgen

DROPIN = os.path.join(build.ROOT, "oracle", "_ref", "sigma_dropin")
SOLVER = os.path.join(build.ROOT, "oracle", "_ref", "parafrost")

pytestmark = pytest.mark.skipif(not (os.path.exists(DROPIN) and os.path.exists(SOLVER)),
                                reason="drop-in harness not built here (needs the reference sources)")

FORMULAS = {
    "aig_33k": lambda: cnfgen.aig_tseitin(num_inputs=2000, num_and=30_000, num_xor=3000, seed=2),
    "aig_units": lambda: cnfgen.with_units_of("aig_tseitin", 40, num_inputs=2000, num_and=30000, num_xor=3000,
                                              seed=7),
    "community_80k": lambda: cnfgen.community(num_vars=20_000, num_clauses=80_000, communities=20, seed=3),
    "ksat3_easy": lambda: cnfgen.random_ksat(5000, 18_000, 3, seed=4),
    "ksat3_unsat": lambda: cnfgen.random_ksat(150, 900, 3, seed=3),
    "mixed_sat": lambda: cnfgen.random_mixed_ksat(20_000, 3.0, seed=6),
}


def _run(binary, cnf, extra=()):
    # the harness is always quiet; the reference's -quiet flag lives in its own main()
    quiet = ["-quiet"] if binary == SOLVER else []
    out = subprocess.run([binary, cnf, *quiet, "-model", "-modelverify", *extra], stdout=subprocess.PIPE,
                         stderr=subprocess.STDOUT, text=True, timeout=600).stdout
    return re.sub(r"\x1b\[[0-9;]*m", "", out)


@pytest.mark.parametrize("name", sorted(FORMULAS))
def test_dropin_solver_agrees_with_reference(built, name):
    nv, lits, off = FORMULAS[name]()
    with tempfile.TemporaryDirectory() as td:
        cnf = os.path.join(td, "f.cnf")
        cnfgen.to_dimacs(cnf, nv, lits, off)
        ours = _run(DROPIN, cnf)
        ref = _run(SOLVER, cnf)
    answer = [l for l in ours.splitlines() if l.startswith("s ")]
    assert answer == [l for l in ref.splitlines() if l.startswith("s ")]
    rounds = [l for l in ours.splitlines() if l.startswith("c sigma_gb300 round")]
    assert len(rounds) == 1 or "orgs" in ours, ours[-2000:]
    if answer == ["s SATISFIABLE"]:
        assert "c model VERIFIED" in ours, ours[-2000:]
        assert "NOT VERIFIED" not in ours
