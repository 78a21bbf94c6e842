"""Python binding of libsigma_gb300.so (the ctypes form of the C ABI in
include/sigma_gb300.h).

``Simplifier`` mirrors the reference's simplifier entry points: construct it
with the reference option names (``Options``), ``awaken()`` uploads a formula
(ParaFROST::awaken/extract, src/cpu/simplify.cpp:95-155), ``sigmify()`` runs one
round (ParaFROST::sigmify, simplify.cpp:115-129) and ``result()`` returns the
simplified formula, units, witness stack and eliminated flags. Errors raise
``SigmaError`` with the library's status; a proved contradiction is reported as
``status == PF_UNSAT`` (the reference's learnEmpty + killSolver path).

The product path loads the CUDA library only and raises when it is missing or
no GPU is visible; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from .options import Options, PfOptions

PF_OK, PF_UNSAT, PF_EINVAL, PF_ENOMEM, PF_ETIMEOUT, PF_EDEVICE, PF_ESTATE = 0, 1, -1, -2, -3, -4, -5
STATUS_NAMES = {0: "PF_OK", 1: "PF_UNSAT", -1: "PF_EINVAL", -2: "PF_ENOMEM", -3: "PF_ETIMEOUT",
                -4: "PF_EDEVICE", -5: "PF_ESTATE"}
STAGES = ["ot", "prop", "lcve", "sort", "sub", "ve", "bce", "ere", "gc", "count", "upload", "download"]


class SigmaError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


# The kernels pf_round_stats times one by one (ms_kernel / bytes_kernel order).
HOT_KERNELS = ("mis_rounds", "bve_decide", "sub", "bve_write")


class RoundStats(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("phases_run", ctypes.c_int32),
                ("clauses_before", ctypes.c_uint64), ("literals_before", ctypes.c_uint64),
                ("clauses_after", ctypes.c_uint64), ("literals_after", ctypes.c_uint64),
                ("eliminated_vars", ctypes.c_uint64), ("units", ctypes.c_uint64),
                ("resolved_words", ctypes.c_uint64), ("ms_total", ctypes.c_double),
                ("ms_stage", ctypes.c_double * 12), ("algorithmic_bytes", ctypes.c_uint64),
                ("kernel_launches", ctypes.c_uint32), ("mis_rounds", ctypes.c_uint32),
                ("prop_waves", ctypes.c_uint32), ("host_syncs", ctypes.c_uint32), ("ms_kernel", ctypes.c_double * 4),
                ("bytes_kernel", ctypes.c_uint64 * 4), ("launches_kernel", ctypes.c_uint32 * 4),
                ("phase_elected", ctypes.c_uint32 * 8), ("phase_clauses", ctypes.c_uint64 * 8),
                ("phase_literals", ctypes.c_uint64 * 8), ("phase_bytes", ctypes.c_uint64 * 8),
                ("phase_ms", ctypes.c_double * 8)]

    PHASE_FIELDS = ("phase_elected", "phase_clauses", "phase_literals", "phase_bytes", "phase_ms")

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_
             if f not in ("ms_stage", "ms_kernel", "bytes_kernel", "launches_kernel")
             and f not in self.PHASE_FIELDS}
        d["ms_stage"] = {s: self.ms_stage[i] for i, s in enumerate(STAGES)}
        d["kernels"] = {k: {"ms": self.ms_kernel[i], "bytes": int(self.bytes_kernel[i]),
                            "launches": int(self.launches_kernel[i])} for i, k in enumerate(HOT_KERNELS)}
        d["phases"] = [{"phase": p, "clauses": int(self.phase_clauses[p]), "literals": int(self.phase_literals[p]),
                        "elected": int(self.phase_elected[p]), "bytes": int(self.phase_bytes[p]),
                        "ms": self.phase_ms[p]} for p in range(min(int(self.phases_run) + 1, 8))
                       if self.phase_ms[p] > 0 or self.phase_clauses[p] > 0]
        return d


_VP, _U32, _U64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64


def _bind(lib: ctypes.CDLL) -> ctypes.CDLL:
    lib.pf_default_options.argtypes = [_VP]
    lib.pf_derive_options.argtypes = [_VP]
    lib.pf_sigma_create.argtypes = [_VP, ctypes.POINTER(_VP)]
    lib.pf_sigma_create.restype = ctypes.c_int
    lib.pf_sigma_upload.argtypes = [_VP, _U32, _VP, _VP, _U64, _VP]
    lib.pf_sigma_upload.restype = ctypes.c_int
    lib.pf_sigma_upload_device.argtypes = [_VP, _U32, _VP, _VP, _U64, _VP]
    lib.pf_sigma_upload_device.restype = ctypes.c_int
    lib.pf_sigma_round.argtypes = [_VP, _VP]
    lib.pf_sigma_round.restype = ctypes.c_int
    lib.pf_sigma_result_sizes.argtypes = [_VP, _VP, _VP, _VP, _VP]
    lib.pf_sigma_result_sizes.restype = ctypes.c_int
    lib.pf_sigma_download.argtypes = [_VP, _VP, _VP, _VP, _VP, _VP, _VP]
    lib.pf_sigma_download.restype = ctypes.c_int
    lib.pf_sigma_proof.argtypes = [_VP, _VP, _VP]
    lib.pf_sigma_proof.restype = ctypes.c_int
    lib.pf_sigma_extend.argtypes = [_VP, _VP]
    lib.pf_sigma_extend.restype = ctypes.c_int
    lib.pf_sigma_write_dump.argtypes = [_VP, ctypes.c_char_p]
    lib.pf_sigma_write_dump.restype = ctypes.c_int
    lib.pf_sigma_upload_batch.argtypes = [_VP, _U32, _VP, _VP, _VP, _VP]
    lib.pf_sigma_upload_batch.restype = ctypes.c_int
    lib.pf_sigma_upload_batch_parts.argtypes = [_VP, _U32, _VP, _VP, _VP, _VP]
    lib.pf_sigma_upload_batch_parts.restype = ctypes.c_int
    lib.pf_sigma_upload_batch_device.argtypes = [_VP, _U32, _VP, _VP, _VP, _VP]
    lib.pf_sigma_upload_batch_device.restype = ctypes.c_int
    lib.pf_sigma_batch_result_sizes.argtypes = [_VP, _VP, _VP, _VP, _VP, _VP, _VP]
    lib.pf_sigma_batch_result_sizes.restype = ctypes.c_int
    lib.pf_sigma_batch_download.argtypes = [_VP, _VP, _VP, _VP, _VP, _VP, _VP]
    lib.pf_sigma_batch_download.restype = ctypes.c_int
    lib.pf_sigma_footprint.argtypes = [_VP, _VP]
    lib.pf_sigma_footprint.restype = ctypes.c_int
    lib.pf_sigma_destroy.argtypes = [_VP]
    lib.pf_sigma_destroy.restype = None
    lib.pf_create_ot.argtypes = [_U32, _VP, _VP, _U64, _VP, _VP, _VP, _VP]
    lib.pf_create_ot.restype = ctypes.c_int
    lib.pf_device_alloc_count.argtypes = []
    lib.pf_device_alloc_count.restype = ctypes.c_uint64
    lib.pf_dimacs_parse.argtypes = [ctypes.c_char_p, _VP]
    lib.pf_dimacs_parse.restype = ctypes.c_int
    lib.pf_formula_free.argtypes = [_VP]
    lib.pf_formula_free.restype = None
    lib.pf_last_error.argtypes = []
    lib.pf_last_error.restype = ctypes.c_char_p
    return lib


_LIBS: dict = {}


def load_library(path: str | None = None) -> ctypes.CDLL:
    """Load the CUDA library (default) or an explicit library path."""
    from . import build
    path = path or build.LIB
    if path not in _LIBS:
        if not os.path.exists(path):
            raise SigmaError(PF_EDEVICE, f"CUDA library not built: {path} (run __graft_entry__.build())")
        _LIBS[path] = _bind(ctypes.CDLL(path))
    return _LIBS[path]


class PfFormula(ctypes.Structure):
    _fields_ = [("num_vars", ctypes.c_uint32), ("num_clauses", ctypes.c_uint64),
                ("lits", ctypes.POINTER(ctypes.c_uint32)), ("offsets", ctypes.POINTER(ctypes.c_uint64)),
                ("empty_clause", ctypes.c_int32)]


def read_dimacs(path: str, library: str | None = None):
    """(num_vars, lits, offsets, empty_clause) of a DIMACS file, read by the library's
    reader (pf_dimacs_parse)."""
    lib = load_library(library)
    f = PfFormula()
    st = lib.pf_dimacs_parse(path.encode(), ctypes.byref(f))
    if st not in (PF_OK, PF_UNSAT):
        raise SigmaError(st, lib.pf_last_error().decode(errors="replace"))
    try:
        n, nl = int(f.num_clauses), 0
        off = np.ctypeslib.as_array(f.offsets, shape=(n + 1,)).copy()
        nl = int(off[-1])
        lits = np.ctypeslib.as_array(f.lits, shape=(max(nl, 1),))[:nl].copy()
    finally:
        lib.pf_formula_free(ctypes.byref(f))
    return int(f.num_vars), lits.astype(np.uint32), off.astype(np.uint64), bool(f.empty_clause)


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def create_ot(num_vars: int, d_lits: int, d_offsets: int, num_clauses: int, d_ot_off: int, d_ot_size: int,
              d_ot_refs: int, stream: int | None = None, library: str | None = None) -> None:
    """Occurrence table of a clause list held in device memory (pf_create_ot)."""
    lib = load_library(library)
    st = lib.pf_create_ot(num_vars, d_lits, d_offsets, num_clauses, d_ot_off, d_ot_size, d_ot_refs, stream)
    if st != PF_OK:
        raise SigmaError(st, lib.pf_last_error().decode(errors="replace"))


def occurrence_lists(num_vars: int, lits: np.ndarray, offsets: np.ndarray):
    """Host restatement of the table's content: per literal, the sorted clause indices."""
    owner = np.repeat(np.arange(offsets.size - 1, dtype=np.uint32), np.diff(offsets.astype(np.int64)))
    order = np.lexsort((owner, lits))
    D = 2 * (num_vars + 1)
    size = np.bincount(lits, minlength=D).astype(np.uint32)
    off = np.concatenate([[0], np.cumsum(size)]).astype(np.uint32)
    return off, size, owner[order]


class ResultBuffers:
    """Host buffers reused across Simplifier.result(out=...) calls: each grows to the
    largest result seen, so repeated downloads write into memory that is already
    mapped. `alloc(nbytes)` returns a uint8 array (default np.empty); a caller can
    pass one that returns page-locked memory, which the device copies into directly."""

    def __init__(self, alloc=None):
        self._alloc = alloc or (lambda n: np.empty(n, dtype=np.uint8))
        self._bufs: dict = {}

    def take(self, name: str, count: int, dtype) -> np.ndarray:
        dt = np.dtype(dtype)
        need = max(int(count), 1) * dt.itemsize
        b = self._bufs.get(name)
        if b is None or b.nbytes < need:
            b = self._alloc(need)
            self._bufs[name] = b
        return b[:need].view(dt)[:count]


@dataclass
class Result:
    num_vars: int
    lits: np.ndarray       # uint32, clause literals in clause-store order
    offsets: np.ndarray    # uint64, num_clauses + 1
    learnt: np.ndarray     # uint8 per clause
    units: np.ndarray      # uint32, assigned literals
    resolved: np.ndarray   # uint32, witness stack (model.resolved)
    eliminated: np.ndarray # uint8 per variable (index 0 unused)

    def clauses(self) -> list:
        o = self.offsets.astype(np.int64)
        return [tuple(int(x) for x in self.lits[o[i]:o[i + 1]]) for i in range(o.size - 1)]


def pack_batch(formulas):
    """Concatenate (num_vars, lits, offsets) formulas: (num_vars[], lits, offsets)."""
    nv = np.array([f[0] for f in formulas], dtype=np.uint32)
    lits = np.concatenate([np.asarray(f[1], dtype=np.uint32) for f in formulas]) if formulas else np.empty(0, np.uint32)
    parts, base = [np.zeros(1, dtype=np.uint64)], 0
    for f in formulas:
        o = np.asarray(f[2], dtype=np.uint64)
        parts.append(o[1:] - o[0] + np.uint64(base))
        base += int(o[-1] - o[0])
    return nv, lits, np.concatenate(parts)


def lits_offsets_begin(formulas, lits, offsets):
    """clause_begin, lits, offsets of a packed batch."""
    cb = np.zeros(len(formulas) + 1, dtype=np.uint64)
    cb[1:] = np.cumsum([np.asarray(f[2]).size - 1 for f in formulas])
    return cb, lits, offsets


class Simplifier:
    """One resident formula on the current GPU (a pf_sigma_ctx)."""

    def __init__(self, opts: Options | None = None, library: str | None = None):
        self.lib = load_library(library)
        self.opts = (opts or Options()).derived()
        self._o = self.opts.to_struct()
        h = _VP()
        st = self.lib.pf_sigma_create(ctypes.addressof(self._o), ctypes.byref(h))
        self._check(st)
        self.h = h
        self.num_vars = 0

    def _check(self, st: int) -> int:
        if st not in (PF_OK, PF_UNSAT):
            raise SigmaError(st, self.lib.pf_last_error().decode(errors="replace"))
        return st

    def awaken(self, num_vars: int, lits: np.ndarray, offsets: np.ndarray, learnt: np.ndarray | None = None) -> None:
        """Upload a formula from host arrays (ParaFROST::awaken/extract)."""
        lits = np.ascontiguousarray(lits, dtype=np.uint32)
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        if learnt is not None:
            learnt = np.ascontiguousarray(learnt, dtype=np.uint8)
        self._check(self.lib.pf_sigma_upload(self.h, num_vars, _ptr(lits), _ptr(offsets), offsets.size - 1,
                                             _ptr(learnt)))
        self.num_vars = num_vars

    def awaken_device(self, num_vars: int, d_lits: int, d_offsets: int, num_clauses: int, d_learnt: int | None = None):
        """Upload from device pointers (e.g. torch tensors' data_ptr())."""
        self._check(self.lib.pf_sigma_upload_device(self.h, num_vars, d_lits, d_offsets, num_clauses, d_learnt))
        self.num_vars = num_vars

    def sigmify(self) -> RoundStats:
        """One sigmify round. stats.status is PF_OK or PF_UNSAT."""
        stats = RoundStats()
        self._check(self.lib.pf_sigma_round(self.h, ctypes.byref(stats)))
        return stats

    def result(self, out: ResultBuffers | None = None) -> Result:
        """The simplified formula. With `out`, the arrays are views into its reusable
        buffers (valid until they are used again); otherwise fresh arrays."""
        nc, nl, nu, nr = _U64(), _U64(), _U64(), _U64()
        self._check(self.lib.pf_sigma_result_sizes(self.h, ctypes.byref(nc), ctypes.byref(nl), ctypes.byref(nu),
                                                   ctypes.byref(nr)))
        take = out.take if out is not None else (lambda _name, count, dtype: np.empty(count, dtype=dtype))
        lits = take("lits", nl.value, np.uint32)
        offsets = take("offsets", nc.value + 1, np.uint64)
        learnt = take("learnt", nc.value, np.uint8)
        units = take("units", nu.value, np.uint32)
        resolved = take("resolved", nr.value, np.uint32)
        elim = take("eliminated", self.num_vars + 1, np.uint8)
        self._check(self.lib.pf_sigma_download(self.h, _ptr(lits), _ptr(offsets), _ptr(learnt), _ptr(units),
                                               _ptr(resolved), _ptr(elim)))
        return Result(self.num_vars, lits, offsets, learnt, units, resolved, elim)

    # ---- formula batches
    def awaken_batch(self, formulas) -> None:
        """Upload a batch: formulas is a sequence of (num_vars, lits, offsets) in each
        formula's own numbering (each formula copied from its own arrays)."""
        nf = len(formulas)
        arrs = [(np.ascontiguousarray(l, dtype=np.uint32), np.ascontiguousarray(o, dtype=np.uint64))
                for _, l, o in formulas]
        nv = np.array([f[0] for f in formulas], dtype=np.uint32)
        nc = np.array([o.size - 1 for _, o in arrs], dtype=np.uint64)
        dummy = np.zeros(1, np.uint32)  # stands for an empty formula's literal array
        lp = (ctypes.c_void_p * nf)(*[l.ctypes.data if l.size else dummy.ctypes.data for l, _ in arrs])
        op = (ctypes.c_void_p * nf)(*[o.ctypes.data for _, o in arrs])
        self._keep = (arrs, dummy)  # the arrays must live through the call
        self._check(self.lib.pf_sigma_upload_batch_parts(self.h, nf, _ptr(nv), _ptr(nc), lp, op))
        self._keep = None
        self.batch_vars = nv.copy()

    def upload_batch(self, num_vars: np.ndarray, clause_begin: np.ndarray, lits: np.ndarray,
                     offsets: np.ndarray) -> None:
        num_vars = np.ascontiguousarray(num_vars, dtype=np.uint32)
        clause_begin = np.ascontiguousarray(clause_begin, dtype=np.uint64)
        lits = np.ascontiguousarray(lits, dtype=np.uint32)
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        self._check(self.lib.pf_sigma_upload_batch(self.h, num_vars.size, _ptr(num_vars), _ptr(clause_begin),
                                                   _ptr(lits), _ptr(offsets)))
        self.batch_vars = num_vars.copy()

    def upload_batch_device(self, num_vars: np.ndarray, clause_begin: np.ndarray, d_lits: int, d_offsets: int):
        num_vars = np.ascontiguousarray(num_vars, dtype=np.uint32)
        clause_begin = np.ascontiguousarray(clause_begin, dtype=np.uint64)
        self._check(self.lib.pf_sigma_upload_batch_device(self.h, num_vars.size, _ptr(num_vars), _ptr(clause_begin),
                                                          d_lits, d_offsets))
        self.batch_vars = num_vars.copy()

    def batch_results(self, out: ResultBuffers | None = None) -> list:
        """[(status, phases, Result)] per formula of the last batched round. With
        `out`, the arrays are views into its reusable buffers."""
        nf = self.batch_vars.size
        st = np.empty(nf, dtype=np.int32)
        ph = np.empty(nf, dtype=np.uint32)
        nc, nl, nu, nr = (np.empty(nf, dtype=np.uint64) for _ in range(4))
        self._check(self.lib.pf_sigma_batch_result_sizes(self.h, _ptr(st), _ptr(ph), _ptr(nc), _ptr(nl), _ptr(nu),
                                                         _ptr(nr)))
        C, Lt, U, R = int(nc.sum()), int(nl.sum()), int(nu.sum()), int(nr.sum())
        take = out.take if out is not None else (lambda _name, count, dtype: np.empty(count, dtype=dtype))
        lits = take("lits", Lt, np.uint32)
        offsets = take("offsets", C + 1, np.uint64)
        learnt = take("learnt", C, np.uint8)
        units = take("units", U, np.uint32)
        resolved = take("resolved", R, np.uint32)
        elim = take("eliminated", int(self.batch_vars.astype(np.uint64).sum()) + nf, np.uint8)
        self._check(self.lib.pf_sigma_batch_download(self.h, _ptr(lits), _ptr(offsets), _ptr(learnt), _ptr(units),
                                                     _ptr(resolved), _ptr(elim)))
        out = []
        c0 = u0 = r0 = e0 = 0
        for f in range(nf):
            c1, u1, r1 = c0 + int(nc[f]), u0 + int(nu[f]), r0 + int(nr[f])
            e1 = e0 + int(self.batch_vars[f]) + 1
            o = offsets[c0:c1 + 1]
            res = Result(int(self.batch_vars[f]), lits[int(o[0]):int(o[-1])], o - o[0],
                         learnt[c0:c1], units[u0:u1], resolved[r0:r1], elim[e0:e1])
            out.append((int(st[f]), int(ph[f]), res))
            c0, u0, r0, e0 = c1, u1, r1, e1
        return out

    def proof(self) -> bytes:
        """The last round's DRAT proof (binary format); needs Options(proof=1)."""
        n = _U64(0)
        self._check(self.lib.pf_sigma_proof(self.h, None, ctypes.byref(n)))
        buf = np.empty(max(n.value, 1), dtype=np.uint8)
        self._check(self.lib.pf_sigma_proof(self.h, _ptr(buf), ctypes.byref(n)))
        return buf[:n.value].tobytes()

    def extend(self, values: np.ndarray) -> np.ndarray:
        """MODEL::extend on the device for the single formula of the last round:
        values (uint8 per variable 0..num_vars, 1 = true) is a model of the simplified
        formula; returns a model of the original formula."""
        v = np.array(values, dtype=np.uint8, copy=True)
        assert v.size == self.num_vars + 1
        self._check(self.lib.pf_sigma_extend(self.h, _ptr(v)))
        return v

    def batch_extend(self, models: list) -> list:
        """MODEL::extend on the device for every formula of the last batched round:
        models[f] (uint8 per variable 0..num_vars[f]) is a model of formula f's
        simplified result; returns the extended models, formulas walked side by side."""
        nf = self.batch_vars.size
        assert len(models) == nf
        packed = np.concatenate([np.asarray(m, dtype=np.uint8) for m in models]) if nf else np.zeros(0, np.uint8)
        assert packed.size == int(self.batch_vars.astype(np.uint64).sum()) + nf
        self._check(self.lib.pf_sigma_extend(self.h, _ptr(packed)))
        out, e0 = [], 0
        for f in range(nf):
            e1 = e0 + int(self.batch_vars[f]) + 1
            out.append(packed[e0:e1])
            e0 = e1
        return out

    def write_dump(self, path: str) -> None:
        self._check(self.lib.pf_sigma_write_dump(self.h, path.encode()))

    def footprint(self) -> int:
        b = _U64()
        self._check(self.lib.pf_sigma_footprint(self.h, ctypes.byref(b)))
        return b.value

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.pf_sigma_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
