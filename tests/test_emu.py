"""CPU: the kernel item functions, run serially by the emulation build, against the
oracle stage by stage and against the golden fixtures. This checks kernel logic
without a GPU; the GPU tests run the same code as CUDA kernels."""
import os
import tempfile

import pytest

import golden_cases as gc
import oracle_runner as orr
from parafrost_gb300 import build, cnfgen, rounddump as rd
from parafrost_gb300.options import Options
from parafrost_gb300.sigma import Simplifier


def run_lib(library, nv, lits, off, opts, level=2, learnt=None):
    op = Options(**{**opts.__dict__, "dump_level": level})
    with Simplifier(op, library=library) as s:
        s.awaken(nv, lits, off, learnt)
        stats = s.sigmify()
        with tempfile.TemporaryDirectory() as td:
            p = os.path.join(td, "d.bin")
            s.write_dump(p)
            recs = rd.read(p)
        res = s.result() if stats.status == 0 else None
    return stats, recs, res


@pytest.mark.parametrize("name", sorted(gc.index()))
def test_emu_golden(built, name):
    meta, arrays, (nv, lits, off), opts = gc.load(name)
    if meta.get("num_clauses", 0) > 60000 or nv > 50000:
        pytest.skip("large case: GPU test only")
    stats, recs, _ = run_lib(build.EMU, nv, lits, off, opts, level=1, learnt=gc.learnt_mask(meta, off))
    assert stats.status == meta["status"]
    assert gc.check(meta, arrays, recs) == []


CASES = [
    ("ksat3", lambda s: cnfgen.random_ksat(300, 1278, 3, seed=s)),
    ("aig", lambda s: cnfgen.aig_tseitin(num_inputs=150, num_and=2000, num_xor=300, seed=s)),
    ("mixed", lambda s: cnfgen.random_mixed_ksat(2500, 3.2, seed=s)),
    ("community", lambda s: cnfgen.community(num_vars=3000, num_clauses=9000, communities=10, seed=s)),
]


@pytest.mark.parametrize("seed", [11, 12])
@pytest.mark.parametrize("case", [c[0] for c in CASES])
@pytest.mark.parametrize("opt", [dict(all=1), dict(all=1, gc_freq=1, mu_pos=10, mu_neg=10)])
def test_emu_stagewise(built, case, seed, opt):
    gen = dict(CASES)[case]
    nv, lits, off = gen(seed)
    opts = Options(**opt)
    st, a, _ = orr.run_oracle(nv, lits, off, opts, level=2)
    stats, b, _ = run_lib(build.EMU, nv, lits, off, opts, level=2)
    assert stats.status == st
    assert rd.compare(rd.normalize(a), rd.normalize(b)) == []


# Formulas whose SUB pass finds units in a variable that an earlier variable's unit
# reaches, so the producers' fix-point re-runs some of them (the rare path).
SUB_RERUN = [
    ("ksat2_60_s5", lambda: cnfgen.random_ksat(60, 75, 2, seed=5)),
    ("ksat2_60_s36", lambda: cnfgen.random_ksat(60, 106, 2, seed=36)),
    ("ksat2_150_s63", lambda: cnfgen.random_ksat(150, 213, 2, seed=63)),
    ("ksat2_150_s161", lambda: cnfgen.random_ksat(150, 311, 2, seed=161)),
]


@pytest.mark.parametrize("case", [c[0] for c in SUB_RERUN])
@pytest.mark.parametrize("opt", [dict(all=1, mu_pos=10, mu_neg=10), dict(all=1)])
def test_emu_sub_rerun(built, case, opt):
    nv, lits, off = dict(SUB_RERUN)[case]()
    opts = Options(**opt)
    st, a, _ = orr.run_oracle(nv, lits, off, opts, level=2)
    stats, b, _ = run_lib(build.EMU, nv, lits, off, opts, level=2)
    assert stats.status == st
    assert rd.compare(rd.normalize(a), rd.normalize(b)) == []
