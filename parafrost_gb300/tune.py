"""Autotuner for the launch-shape knobs of a round (no counterpart in the reference).

The round's results do not depend on these knobs, only its speed does:
  * ``ot_buckets``: occurrence-table build by per-occurrence atomics (-1) or by
    literal buckets with staged, contiguous writes (1);
  * ``sweep_div``: how large a propagation wave must be (its pending literals'
    lists against the store) before it sweeps the whole store instead of walking
    the lists (-1 never);
  * ``pv_blocks``: blocks per SM of the per-variable warp kernels (SUB, the BVE
    decision and write, BCE), i.e. how many elected variables are in flight.

``tune(formulas, opts)`` runs rounds of a sample (one formula, or a batch) on a
context with each candidate setting, one knob at a time starting from the
defaults (coordinate descent), keeps the fastest by the device time of the round
(``pf_round_stats.ms_total``, the median of ``repeats`` rounds), and returns the
options with the chosen knobs and the timings it saw. Every candidate round must
give the same result as the defaults; a candidate that does not is an error.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import rounddump as rd
from .options import Options
from .sigma import Simplifier

CANDIDATES = {
    "ot_buckets": (-1, 1),
    "sweep_div": (16, 64, 256, -1),
    "pv_blocks": (4, 8, 16),
}


def _round_ms(lib, formulas, opts: Options, repeats: int):
    """(median round ms, canonical result of the last round)."""
    times = []
    with Simplifier(opts, library=lib) as s:
        for _ in range(repeats):
            if len(formulas) == 1:
                s.awaken(*formulas[0])
            else:
                s.awaken_batch(formulas)
            st = s.sigmify()
            times.append(st.ms_total)
        if len(formulas) == 1:
            res = [rd.canonical_result(st.status, s.result() if st.status == 0 else None)]
        else:
            res = [rd.canonical_result(f_st, r if f_st == 0 else None) for f_st, _, r in s.batch_results()]
    return float(np.median(times)), res


def tune(formulas, opts: Options | None = None, library: str | None = None, repeats: int = 3,
         candidates: dict | None = None) -> tuple:
    """(tuned Options, {knob: {value: ms}}) for a sample: one (num_vars, lits,
    offsets) formula or a list of them (run as one batch)."""
    if isinstance(formulas, tuple):
        formulas = [formulas]
    best = dataclasses.replace(opts or Options(all=1))
    cand = candidates or CANDIDATES
    base_ms, want = _round_ms(library, formulas, best, repeats)
    seen = {}
    for knob, values in cand.items():
        seen[knob] = {getattr(best, knob): base_ms}
        for v in values:
            if v == getattr(best, knob):
                continue
            trial = dataclasses.replace(best, **{knob: v})
            ms, got = _round_ms(library, formulas, trial, repeats)
            if got != want:
                raise RuntimeError(f"tuning knob {knob}={v} changed the round's result")
            seen[knob][v] = ms
            if ms < base_ms:
                best, base_ms = trial, ms
    return best, seen
