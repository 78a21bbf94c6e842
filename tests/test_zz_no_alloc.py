"""The no-allocation occurrence-table build, pf_create_ot_noalloc.

It exists for callers that must not allocate device memory (a serving process
whose HBM is fully reserved by its own pool or a framework's caching allocator,
or a caller that cannot take a cudaFree's device-wide synchronisation). Its
output must equal the allocating entry point's, pf_create_ot, on consecutive
calls (the fixed scratch keeps the previous call's contents), and after a
warm-up call it must make no device allocation at all (the library's own
allocation counter, pf_device_alloc_count, stays put). Lists compare as sets:
the order inside one occurrence list is unspecified for both.

This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from parafrost_gb300 import cnfgen
from parafrost_gb300.sigma import PF_EINVAL, PF_OK, load_library

pytestmark = pytest.mark.gpu

_VP, _U32, _U64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64
MAX_VARS = 67_106_815  # (65,536 - 2) scan blocks of 2048 literal slots, minus the slots 0 and 1


def _lib(path):
    lib = load_library(path)
    for name in ("pf_create_ot", "pf_create_ot_noalloc"):
        fn = getattr(lib, name)
        fn.argtypes = [_U32, _VP, _VP, _U64, _VP, _VP, _VP, _VP]
        fn.restype = ctypes.c_int
    return lib


def _table(fn, nv, dl, do, ncls, nlits, stream):
    import torch
    D = 2 * (nv + 1)
    off = torch.full((D + 1,), -1, dtype=torch.int32, device="cuda")
    size = torch.full((D,), -1, dtype=torch.int32, device="cuda")
    refs = torch.full((nlits,), -1, dtype=torch.int32, device="cuda")
    st = fn(nv, dl.data_ptr(), do.data_ptr(), ncls, off.data_ptr(), size.data_ptr(), refs.data_ptr(), stream)
    assert st == PF_OK
    off_h = off.cpu().numpy().view(np.uint32)
    size_h = size.cpu().numpy().view(np.uint32)
    refs_h = refs.cpu().numpy().view(np.uint32).copy()
    for l in range(D):
        a, b = int(off_h[l]), int(off_h[l]) + int(size_h[l])
        refs_h[a:b] = np.sort(refs_h[a:b])
    return off_h, size_h, refs_h


def test_noalloc_matches_allocating_entry_point(cuda_lib):
    import torch
    lib = _lib(cuda_lib)
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row, on formulas of different sizes
    for gen in (lambda: cnfgen.community(num_vars=300_000, num_clauses=1_200_000, seed=12),
                lambda: cnfgen.random_mixed_ksat(100_000, 4.0, seed=13)):
        nv, lits, offsets = gen()
        dl = torch.from_numpy(lits.view(np.int32)).cuda()
        do = torch.from_numpy(offsets.view(np.int64)).cuda()
        ncls = offsets.size - 1
        want = _table(lib.pf_create_ot, nv, dl, do, ncls, lits.size, stream)
        before = lib.pf_device_alloc_count()
        got = _table(lib.pf_create_ot_noalloc, nv, dl, do, ncls, lits.size, stream)
        assert lib.pf_device_alloc_count() == before, "the no-allocation call allocated device memory"
        for w, g in zip(want, got):
            assert np.array_equal(w, g)


def test_noalloc_variable_limit(cuda_lib):
    """One variable past the limit is refused on the host; the limit itself is
    accepted (a two-clause formula over the largest variable numbers)."""
    import torch
    lib = _lib(cuda_lib)
    dummy = torch.zeros(4, dtype=torch.int64, device="cuda")
    p = dummy.data_ptr()
    st = lib.pf_create_ot_noalloc(MAX_VARS + 1, p, p, 1, p, p, p, None)
    assert st == PF_EINVAL
    assert b"67,106,815" in lib.pf_last_error()
    v = MAX_VARS
    lits = np.array([2, 2 * v + 1, 2 * v, 2 * (v - 1)], dtype=np.uint32)
    offsets = np.array([0, 2, 4], dtype=np.uint64)
    dl = torch.from_numpy(lits.view(np.int32)).cuda()
    do = torch.from_numpy(offsets.view(np.int64)).cuda()
    D = 2 * (v + 1)
    off = torch.empty(D + 1, dtype=torch.int32, device="cuda")
    size = torch.empty(D, dtype=torch.int32, device="cuda")
    refs = torch.full((4,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    before = lib.pf_device_alloc_count()
    st = lib.pf_create_ot_noalloc(v, dl.data_ptr(), do.data_ptr(), 2, off.data_ptr(), size.data_ptr(),
                                  refs.data_ptr(), stream)
    assert st == PF_OK, lib.pf_last_error()
    assert lib.pf_device_alloc_count() == before
    o = off.cpu().numpy().view(np.uint32)
    sz = size.cpu().numpy().view(np.uint32)
    assert o[D] == 4 and sz.sum() == 4
    for lit, cl in ((2, 0), (2 * v + 1, 0), (2 * v, 1), (2 * (v - 1), 1)):
        assert sz[lit] == 1 and int(refs[int(o[lit])].item()) == cl
