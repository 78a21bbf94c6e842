"""The standalone occurrence-table build (pf_create_ot): emulation on CPU, CUDA on GPU."""
import numpy as np
import pytest

from parafrost_gb300 import build, cnfgen
from parafrost_gb300.sigma import PF_EINVAL, SigmaError, create_ot, occurrence_lists


def _sorted_lists(off, size, refs):
    out = refs.copy()
    for l in range(size.size):
        a, b = int(off[l]), int(off[l]) + int(size[l])
        out[a:b] = np.sort(out[a:b])
    return out


def _check(num_vars, lits, offsets, off, size, refs):
    eoff, esize, erefs = occurrence_lists(num_vars, lits, offsets)
    assert np.array_equal(off, eoff)
    assert np.array_equal(size, esize)
    assert np.array_equal(_sorted_lists(off, size, refs), erefs)


def test_create_ot_emulation(built):
    nv, lits, offsets = cnfgen.random_mixed_ksat(20000, 4.0, seed=9)
    D = 2 * (nv + 1)
    off = np.zeros(D + 1, np.uint32)
    size = np.zeros(D, np.uint32)
    refs = np.zeros(lits.size, np.uint32)
    create_ot(nv, lits.ctypes.data, offsets.ctypes.data, offsets.size - 1, off.ctypes.data, size.ctypes.data,
              refs.ctypes.data, None, library=build.EMU)
    _check(nv, lits, offsets, off, size, refs)
    bad = lits.copy()
    bad[5] = 2 * nv + 7
    with pytest.raises(SigmaError) as e:
        create_ot(nv, bad.ctypes.data, offsets.ctypes.data, offsets.size - 1, off.ctypes.data, size.ctypes.data,
                  refs.ctypes.data, None, library=build.EMU)
    assert e.value.status == PF_EINVAL


@pytest.mark.gpu
@pytest.mark.parametrize("gen", [lambda: cnfgen.random_mixed_ksat(200_000, 4.0, seed=3),
                                 lambda: cnfgen.community(num_vars=100_000, num_clauses=400_000, seed=4)])
def test_create_ot_gpu(cuda_lib, gen):
    import torch
    nv, lits, offsets = gen()
    D = 2 * (nv + 1)
    dl = torch.from_numpy(lits.view(np.int32)).cuda()
    do = torch.from_numpy(offsets.view(np.int64)).cuda()
    off = torch.zeros(D + 1, dtype=torch.int32, device="cuda")
    size = torch.zeros(D, dtype=torch.int32, device="cuda")
    refs = torch.zeros(lits.size, dtype=torch.int32, device="cuda")
    create_ot(nv, dl.data_ptr(), do.data_ptr(), offsets.size - 1, off.data_ptr(), size.data_ptr(), refs.data_ptr(),
              torch.cuda.current_stream().cuda_stream)
    _check(nv, lits, offsets, off.cpu().numpy().view(np.uint32), size.cpu().numpy().view(np.uint32),
           refs.cpu().numpy().view(np.uint32))
