"""The autotuner (parafrost_gb300.tune): every candidate setting gives the same
round result, and the chosen options are one of the candidates. CPU: the
emulation build (its timings are the host's); GPU: the CUDA build on a batch."""
import pytest

from parafrost_gb300 import cnfgen, tune
from parafrost_gb300.options import Options


def _check(lib, formulas):
    best, seen = tune.tune(formulas, Options(all=1), library=lib, repeats=1)
    for knob, values in tune.CANDIDATES.items():
        assert getattr(best, knob) in (0,) + tuple(values)
        assert set(values) <= set(seen[knob]) | {0}
    return best, seen


def test_tune_emu(built):
    _check(built["emu"], cnfgen.community(num_vars=3000, num_clauses=9000, communities=10, seed=2))
    _check(built["emu"], [cnfgen.random_ksat(300, 1200, 3, seed=i) for i in range(4)])


@pytest.mark.gpu
def test_tune_gpu(cuda_lib):
    forms = list(cnfgen.batch_ksat(num_formulas=4096, cmin=1_000, cmax=200_000, seed=1, indices=range(0, 4096, 128)))
    _check(cuda_lib, forms)
    _check(cuda_lib, cnfgen.community(num_vars=200_000, num_clauses=800_000, seed=6))
