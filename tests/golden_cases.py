"""Loader for the golden fixtures made by tests/golden/make_golden.py."""
import json
import os

import numpy as np

from parafrost_gb300 import cnfgen, rounddump
from parafrost_gb300.options import Options

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def index() -> dict:
    with open(os.path.join(HERE, "index.json")) as f:
        return json.load(f)


def load(name: str):
    meta = index()[name]
    arrays = dict(np.load(os.path.join(HERE, f"{name}.npz")))
    nv, lits, off = getattr(cnfgen, meta["generator"])(**meta["kwargs"])
    return meta, arrays, (nv, lits, off), Options(**meta["options"])


def learnt_mask(meta: dict, off: np.ndarray):
    """Learnt flag per clause of a case (None when every clause is original): the
    last learnt_tail clauses are learnt."""
    n = int(meta.get("learnt_tail", 0))
    if not n:
        return None
    m = np.zeros(off.size - 1, dtype=np.uint8)
    m[m.size - n:] = 1
    return m


def check(meta: dict, arrays: dict, recs: list) -> list:
    """Compare a round dump (level >= 1) against a golden case; returns mismatches."""
    import sys
    sys.path.insert(0, HERE)
    from make_golden import summarize
    got = summarize(recs)
    errs = []
    if got["status"] != meta["status"]:
        return [f"status {got['status']} != {meta['status']}"]
    if got["pv_counts"] != meta["pv_counts"]:
        errs.append(f"pv counts {got['pv_counts']} != {meta['pv_counts']}")
    if got["pv_hash"] != meta["pv_hash"]:
        errs.append("elected variables differ")
    if meta["status"] == 0:
        for k in ("elim", "resolved", "units"):
            if not np.array_equal(got[k], arrays[k]):
                errs.append(f"{k} differs")
        if got["clauses_hash"] != meta["clauses_hash"]:
            errs.append("simplified clauses differ")
    return errs
