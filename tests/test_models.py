"""Size-independent properties of a round, with a model of the original formula
(evaluated AIG inputs, or the community generator's planted assignment):
  - every clause and unit of the result holds under that model (all are implied
    by the original);
  - the model restricted to the variables not eliminated, extended through the
    witness stack as the reference's MODEL::extend does, satisfies every original
    clause.
At full size (6.8M-clause AIG) these stand in for the oracle comparison, which is
run at smaller sizes. The checker itself is tested by planting mistakes on the CPU."""
import numpy as np
import pytest

import oracle_runner as orr
from parafrost_gb300 import cnfgen
from parafrost_gb300.options import Options
from parafrost_gb300.sigma import Simplifier

AIG_SMALL = dict(num_inputs=400, num_and=8000, num_xor=800, seed=12)
COMM_SMALL = dict(num_vars=4000, num_clauses=16000, communities=20, seed=13)


def run(lib, nv, lits, off, opts=None):
    s = Simplifier(opts or Options(all=1), library=lib)
    s.awaken(nv, lits, off)
    st = s.sigmify()
    res = s.result() if st.status == 0 else None
    s.close()
    return st.status, res


@pytest.mark.parametrize("opt", [dict(all=1), dict(all=1, phases=3, mu_pos=8, mu_neg=8)])
def test_models_emu(built, opt):
    nv, lits, off = cnfgen.aig_tseitin(**AIG_SMALL)
    st, res = run(built["emu"], nv, lits, off, Options(**opt))
    assert orr.check_models(nv, lits, off, st, res, cnfgen.aig_model(**AIG_SMALL)) == []
    nv, lits, off = cnfgen.community(**COMM_SMALL)
    st, res = run(built["emu"], nv, lits, off, Options(**opt))
    model = cnfgen.community_planted(COMM_SMALL["num_vars"], COMM_SMALL["seed"])
    assert orr.check_models(nv, lits, off, st, res, model) == []


def test_model_checker_catches_mistakes(built):
    """Mistakes planted in a correct result (on the CPU) are reported."""
    nv, lits, off = cnfgen.aig_tseitin(**AIG_SMALL)
    model = cnfgen.aig_model(**AIG_SMALL)
    st, res = run(built["emu"], nv, lits, off)
    assert res.resolved.size > 4 and res.lits.size > 0
    # a result clause made false: negate every literal of clause 0
    bad = res.lits.copy()
    o0, o1 = int(res.offsets[0]), int(res.offsets[1])
    truth = model[bad[o0:o1] >> 1] == (1 - (bad[o0:o1] & 1))
    bad[o0:o1] ^= truth.astype(np.uint32)  # flip exactly the true literals
    r2 = type(res)(res.num_vars, bad, res.offsets, res.learnt, res.units, res.resolved, res.eliminated)
    assert any("result clauses false" in f for f in orr.check_models(nv, lits, off, st, r2, model))
    # a lost witness stack: eliminated variables stay false and gates break
    r3 = type(res)(res.num_vars, res.lits, res.offsets, res.learnt, res.units, res.resolved[:0], res.eliminated)
    assert any("extended model falsifies" in f for f in orr.check_models(nv, lits, off, st, r3, model))


@pytest.mark.gpu
def test_models_gpu_full_size(cuda_lib):
    """The 6.8M-clause AIG round (the benchmark's workload) and a 16M-clause
    community formula."""
    kw = dict(num_inputs=50_000, num_and=2_000_000, num_xor=200_000, seed=1)
    nv, lits, off = cnfgen.aig_tseitin(**kw)
    st, res = run(cuda_lib, nv, lits, off)
    assert orr.check_models(nv, lits, off, st, res, cnfgen.aig_model(**kw)) == []
    kc = dict(num_vars=4_000_000, num_clauses=16_000_000, seed=2)
    nv, lits, off = cnfgen.community(**kc)
    st, res = run(cuda_lib, nv, lits, off)
    assert orr.check_models(nv, lits, off, st, res, cnfgen.community_planted(kc["num_vars"], kc["seed"])) == []
