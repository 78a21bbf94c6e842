"""Malformed inputs end in PF_EINVAL before any literal is read out of range, and
a device-side loop that reaches its bound ends the round with PF_ETIMEOUT (the
loop bound is lowered through the loop_limit option, so nothing waits): the
context stays usable and is destroyed cleanly. CPU: the emulation build; GPU: the
CUDA build (every case here is one the kernels' own checks turn into an error)."""
import numpy as np
import pytest

from parafrost_gb300 import build, cnfgen
from parafrost_gb300.options import Options
from parafrost_gb300.sigma import PF_EINVAL, PF_ETIMEOUT, SigmaError, Simplifier, create_ot


def _bad_offsets():
    nv, lits, off = cnfgen.random_ksat(200, 850, 3, seed=4)
    down = off.copy()
    down[300] = down[298]  # goes down in the middle: clause 299 would end before it starts
    past = off.copy()
    past[400] = off[-1] + 64  # an inner offset beyond the last literal
    under = off.copy()
    under[10] = 0
    under[0] = 3  # an inner offset below the first
    return nv, lits, off, [down, past, under]


def _check_upload(lib):
    nv, lits, off, bads = _bad_offsets()
    for bad in bads:
        with Simplifier(Options(all=1), library=lib) as s:
            with pytest.raises(SigmaError) as e:
                s.awaken(nv, lits, bad)
            assert e.value.status == PF_EINVAL
            s.awaken(nv, lits, off)  # the context takes a good formula afterwards
            assert s.sigmify().status == 0


def test_upload_rejects_bad_offsets_emu(built):
    _check_upload(built["emu"])


def test_create_ot_rejects_bad_offsets_emu(built):
    nv, lits, off, bads = _bad_offsets()
    D = 2 * (nv + 1)
    o = np.zeros(D + 1, np.uint32)
    sz = np.zeros(D, np.uint32)
    refs = np.zeros(lits.size, np.uint32)
    for bad in bads[:2]:  # offsets[0] must be 0, so only the inner ones are bad here
        with pytest.raises(SigmaError) as e:
            create_ot(nv, lits.ctypes.data, bad.ctypes.data, bad.size - 1, o.ctypes.data, sz.ctypes.data,
                      refs.ctypes.data, None, library=build.EMU)
        assert e.value.status == PF_EINVAL


def _check_loop_limit(lib):
    nv, lits, off = cnfgen.aig_tseitin(num_inputs=200, num_and=3000, num_xor=300, seed=3)
    s = Simplifier(Options(all=1, loop_limit=1), library=lib)
    s.awaken(nv, lits, off)
    with pytest.raises(SigmaError) as e:
        s.sigmify()
    assert e.value.status == PF_ETIMEOUT
    s.close()
    # the default bound is never reached by a correct round
    with Simplifier(Options(all=1), library=lib) as s:
        s.awaken(nv, lits, off)
        assert s.sigmify().status == 0


def test_loop_limit_times_out_emu(built):
    _check_loop_limit(built["emu"])


@pytest.mark.gpu
def test_upload_rejects_bad_offsets_gpu(cuda_lib):
    _check_upload(cuda_lib)


@pytest.mark.gpu
def test_create_ot_rejects_bad_offsets_gpu(cuda_lib):
    import torch
    nv, lits, off, bads = _bad_offsets()
    D = 2 * (nv + 1)
    dl = torch.from_numpy(lits.view(np.int32)).cuda()
    o = torch.zeros(D + 1, dtype=torch.int32, device="cuda")
    sz = torch.zeros(D, dtype=torch.int32, device="cuda")
    refs = torch.zeros(lits.size, dtype=torch.int32, device="cuda")
    for bad in bads[:2]:
        do = torch.from_numpy(bad.view(np.int64)).cuda()
        with pytest.raises(SigmaError) as e:
            create_ot(nv, dl.data_ptr(), do.data_ptr(), bad.size - 1, o.data_ptr(), sz.data_ptr(), refs.data_ptr(),
                      torch.cuda.current_stream().cuda_stream)
        assert e.value.status == PF_EINVAL


@pytest.mark.gpu
def test_loop_limit_times_out_gpu(cuda_lib):
    _check_loop_limit(cuda_lib)


def _check_conflicting_units(lib):
    """(x) and (-x) among the input clauses: the round proves UNSAT. (The reference's
    parser drops a clause that earlier units falsify, src/cpu/dimacs.cpp:153-176, and
    goes on as if it were absent; a round here never drops a clause.)"""
    nv, lits, off = cnfgen.random_ksat(200, 600, 3, seed=2)
    lits = np.concatenate([lits, np.array([2 * 17, 2 * 17 + 1], dtype=np.uint32)])
    off = np.concatenate([off, off[-1] + np.array([1, 2], dtype=np.uint64)])
    with Simplifier(Options(all=1), library=lib) as s:
        s.awaken(nv, lits, off)
        assert s.sigmify().status == 1


def test_conflicting_input_units_emu(built):
    _check_conflicting_units(built["emu"])


@pytest.mark.gpu
def test_conflicting_input_units_gpu(cuda_lib):
    _check_conflicting_units(cuda_lib)
