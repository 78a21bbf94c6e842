"""Model extension on the device (pf_sigma_extend; MODEL::extend, src/cpu/model.cpp:
104-138): the extended values equal the oracle's host walk byte for byte, and a
model of the original formula, restricted to the variables the round kept,
extends to a model of the original formula. Single formulas and batches (each
formula of a batch walked by its own thread); CPU: the emulation build; GPU: the
CUDA build."""
import numpy as np
import pytest

import oracle_runner as orr
from parafrost_gb300 import cnfgen
from parafrost_gb300.options import Options
from parafrost_gb300.sigma import Simplifier

AIG = dict(num_inputs=400, num_and=8000, num_xor=800, seed=12)
COMM = dict(num_vars=4000, num_clauses=16000, communities=20, seed=13)


def host_extend(res, values) -> np.ndarray:
    """The oracle's walk from the same start: eliminated variables false, units set."""
    v = np.array(values, dtype=np.uint8, copy=True)
    v[np.asarray(res.eliminated, dtype=bool)] = 0
    u = res.units
    v[u >> 1] = (1 - (u & 1)).astype(np.uint8)
    r = np.ascontiguousarray(res.resolved, dtype=np.uint32)
    z = np.zeros(1, np.uint64)
    assert orr.oracle_lib().oracle_extend_and_check(res.num_vars, v.ctypes.data, r.ctypes.data, r.size,
                                                    z.ctypes.data, z.ctypes.data, 0) == 0
    return v


def known_models():
    return [(cnfgen.aig_tseitin(**AIG), cnfgen.aig_model(**AIG)),
            (cnfgen.community(**COMM), cnfgen.community_planted(COMM["num_vars"], COMM["seed"])),
            (cnfgen.aig_tseitin(num_inputs=60, num_and=900, num_xor=90, seed=3),
             cnfgen.aig_model(num_inputs=60, num_and=900, num_xor=90, seed=3))]


def _check_single(lib):
    for (nv, lits, off), model in known_models():
        with Simplifier(Options(all=1), library=lib) as s:
            s.awaken(nv, lits, off)
            assert s.sigmify().status == 0
            res = s.result()
            got = s.extend(model)
        assert np.array_equal(got, host_extend(res, model))
        z = np.zeros(1, np.uint64)
        l, o = np.ascontiguousarray(lits), np.ascontiguousarray(off)
        g = got.copy()
        assert orr.oracle_lib().oracle_extend_and_check(nv, g.ctypes.data, z.ctypes.data, 0, l.ctypes.data,
                                                        o.ctypes.data, o.size - 1) == 0, "original clause falsified"


def _check_batch(lib, forms, models):
    b = Simplifier(Options(all=1), library=lib)
    b.awaken_batch(forms)
    b.sigmify()
    results = b.batch_results()
    got = b.batch_extend(models)
    b.close()
    for (nv, lits, off), (st, _, res), model, g in zip(forms, results, models, got):
        if st != 0:
            continue
        assert np.array_equal(g, host_extend(res, model))


def _batch_case():
    pairs = known_models()
    forms = [f for f, _ in pairs]
    models = [m for _, m in pairs]
    # formulas without a known model: any start values, the walk is still compared
    for i in range(5):
        f = cnfgen.random_mixed_ksat(600 + 90 * i, 3.4, seed=40 + i)
        forms.append(f)
        models.append(np.random.default_rng(i).integers(0, 2, f[0] + 1).astype(np.uint8))
    return forms, models


def test_extend_single_emu(built):
    _check_single(built["emu"])


def test_extend_batch_emu(built):
    _check_batch(built["emu"], *_batch_case())


@pytest.mark.gpu
def test_extend_single_gpu(cuda_lib):
    _check_single(cuda_lib)


@pytest.mark.gpu
def test_extend_batch_gpu(cuda_lib):
    _check_batch(cuda_lib, *_batch_case())
    forms = list(cnfgen.batch_ksat(num_formulas=4096, cmin=1_000, cmax=200_000, seed=1, indices=range(0, 4096, 64)))
    models = [np.random.default_rng(i).integers(0, 2, f[0] + 1).astype(np.uint8) for i, f in enumerate(forms)]
    _check_batch(cuda_lib, forms, models)
