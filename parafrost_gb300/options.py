"""Simplifier options: the reference's option names, defaults and derivation rules.

Names and defaults follow ParaFROST's CPU option table (src/cpu/options.cpp:24-46);
``derived()`` applies its derivation rules (options.cpp:281-311). ``to_struct()``
gives the ``pf_options`` C struct of include/sigma_gb300.h.
"""
from __future__ import annotations

import ctypes
import dataclasses


class PfOptions(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in (
        "phases", "all", "ve", "ve_plus", "sub", "bce", "ere", "ve_lbound", "ve_clause_max",
        "ve_phase_min", "mu_pos", "mu_neg", "xor_max_arity", "sub_max", "bce_max", "ere_max",
        "ere_clause_max", "lcve_min", "gc_freq", "dump_level", "loop_limit", "proof", "ot_buckets", "sweep_div",
        "pv_blocks")] + [("reserved", ctypes.c_int32 * 2)]


# python field -> (reference option name, kind)
_REF_NAMES = {
    "phases": ("phases", int), "all": ("all", bool), "ve": ("ve", bool), "ve_plus": ("ve+", bool),
    "sub": ("sub", bool), "bce": ("bce", bool), "ere": ("ere", bool), "ve_lbound": ("velbound", bool),
    "ve_clause_max": ("veclausemax", int), "ve_phase_min": ("vephasemin", int), "mu_pos": ("mupos", int),
    "mu_neg": ("muneg", int), "xor_max_arity": ("xormaxarity", int), "sub_max": ("submax", int),
    "bce_max": ("bcemax", int), "ere_max": ("eremax", int), "ere_clause_max": ("ereclausemax", int),
    "lcve_min": ("lcvemin", int), "gc_freq": ("gcfreq", int),
}


@dataclasses.dataclass
class Options:
    phases: int = 5
    all: int = 0
    ve: int = 1
    ve_plus: int = 1
    sub: int = 1
    bce: int = 0
    ere: int = 1
    ve_lbound: int = 0
    ve_clause_max: int = 100
    ve_phase_min: int = 500
    mu_pos: int = 32
    mu_neg: int = 32
    xor_max_arity: int = 10
    sub_max: int = 3000
    bce_max: int = 3000
    ere_max: int = 3000
    ere_clause_max: int = 1000
    lcve_min: int = 1
    gc_freq: int = 2
    dump_level: int = 0
    loop_limit: int = 0  # device-side loop rounds before PF_ETIMEOUT (0: variables + 2)
    proof: int = 0  # 1: record the round's DRAT proof (reference option "proof")
    ot_buckets: int = 0  # occurrence-table build: 0 by size, 1 literal buckets, -1 atomics
    sweep_div: int = 0  # propagation sweeps when pending lists exceed 1/sweep_div of the store (0: 64, -1: never)
    pv_blocks: int = 0  # blocks per SM of the per-variable warp kernels (0: 8)

    def derived(self) -> "Options":
        """Option derivation of the reference (src/cpu/options.cpp:281-311)."""
        o = dataclasses.replace(self)
        o.ve = int(bool(o.ve or o.ve_plus))
        if o.all:
            o.ve, o.ve_plus, o.bce, o.ere = 1, 1, 1, 1
        if not o.phases and (o.ve or o.sub or o.bce):
            o.phases = 1
        if o.phases and not (o.ve or o.sub or o.bce):
            o.phases = 0
        if o.phases > 1 and not o.ve:
            o.phases = 1
        return o

    def to_struct(self) -> PfOptions:
        s = PfOptions()
        for f in dataclasses.fields(self):
            setattr(s, f.name, int(getattr(self, f.name)))
        return s

    def reference_flags(self) -> list:
        """The same settings as command-line flags of the reference solver."""
        flags = []
        for name, (ref, kind) in _REF_NAMES.items():
            val = getattr(self, name)
            if kind is bool:
                flags.append(f"-{ref}" if val else f"-no-{ref}")
            else:
                flags.append(f"--{ref}={val}")
        return flags
