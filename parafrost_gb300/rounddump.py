"""Reader and comparator for round dumps.

A round dump is the per-stage state of one sigmify round written as records
``kind, phase, stage, n, data[n]`` (little-endian uint32). The GPU library
writes it when asked (``dump_path``/``dump_level`` options); the test oracles
write the same records, so parity is checked record by record.
"""
from __future__ import annotations

import numpy as np

KIND = {1: "cnf", 2: "otsize", 3: "scores", 4: "eligible", 5: "pvs", 6: "pvlists",
        7: "trail", 8: "resolved", 9: "elim", 10: "counts", 11: "status", 12: "timing", 13: "proofmark"}
STAGE = {0: "input", 1: "prop", 2: "lcve", 3: "sort", 4: "sub", 5: "ve", 6: "bce", 7: "ere", 8: "final"}


def read(path_or_bytes) -> list:
    """Return [(kind_name, phase, stage_name, np.ndarray[uint32])] in file order."""
    if isinstance(path_or_bytes, (bytes, bytearray, memoryview)):
        buf = np.frombuffer(path_or_bytes, dtype="<u4")
    else:
        buf = np.fromfile(path_or_bytes, dtype="<u4")
    out, i = [], 0
    while i + 4 <= buf.size:
        kind, phase, stage, n = (int(x) for x in buf[i:i + 4])
        out.append((KIND.get(kind, str(kind)), phase, STAGE.get(stage, str(stage)), buf[i + 4:i + 4 + n].copy()))
        i += 4 + n
    return out


def cnf_clauses(data: np.ndarray) -> list:
    """Decode a cnf record into [(flags, sig, lits_tuple)]."""
    n = int(data[0])
    res, i = [], 1
    for _ in range(n):
        flags, sig, size = int(data[i]), int(data[i + 1]), int(data[i + 2])
        res.append((flags, sig, tuple(int(x) for x in data[i + 3:i + 3 + size])))
        i += 3 + size
    return res


def final_state(recs: list) -> dict:
    """Collect the final-stage records into a dict keyed by kind name."""
    return {k: d for (k, ph, st, d) in recs if st == "final"}


def canonical(recs: list) -> dict:
    """Final state in canonical form: clause multiset, witness stack, units set, eliminated set."""
    fin = final_state(recs)
    res = {"status": int(fin["status"][0]) if "status" in fin else None}
    if res["status"] != 0:
        return res
    live = [(f & 3, lits) for (f, _, lits) in cnf_clauses(fin["cnf"]) if (f & 3) != 2]
    res["clauses"] = sorted(live)
    res["resolved"] = fin["resolved"].tolist()
    res["units"] = sorted(set(fin["trail"].tolist()))
    res["elim"] = fin["elim"].tolist()
    return res


def canonical_result(status: int, res) -> dict:
    """The form of ``canonical`` for a downloaded result (sigma.Result)."""
    out = {"status": int(status)}
    if out["status"] != 0:
        return out
    o = res.offsets.astype(np.int64)
    cls = [(int(res.learnt[i]) & 1, tuple(int(x) for x in res.lits[o[i]:o[i + 1]])) for i in range(o.size - 1)]
    out["clauses"] = sorted(cls)
    out["resolved"] = res.resolved.tolist()
    out["units"] = sorted(set(res.units.tolist()))
    out["elim"] = [v for v in range(1, res.eliminated.size) if res.eliminated[v]]
    return out


def normalize(recs: list) -> list:
    """Mask what parallel unit propagation may legitimately change.

    The reference strips false literals one trail literal at a time, so a clause
    that ends up deleted keeps whichever false literals it still had when a true
    literal reached it; the GPU's wave-parallel propagation can strip a different
    subset. Live clauses, statuses, units and every later decision are the same.
    Deleted clauses therefore compare by status only, and sorted occurrence lists
    compare without their deleted entries (whose position follows their content).
    """
    out, deleted = [], {}
    for kind, phase, stage, d in recs:
        if kind == "cnf":
            cl = cnf_clauses(d)
            flat = [len(cl)]
            dele = set()
            for i, (f, sig, lits) in enumerate(cl):
                if (f & 3) == 2:
                    flat += [2, 0, 0]
                    dele.add(i)
                else:
                    flat += [f, sig, len(lits)] + list(lits)
            deleted[(phase, stage)] = dele
            d = np.array(flat, dtype=np.uint32)
        elif kind == "pvlists":
            dele = deleted.get((phase, "prop"), set())
            flat, i = [], 0
            while i < d.size:
                n = int(d[i])
                keep = [int(x) for x in d[i + 1:i + 1 + n] if int(x) not in dele]
                flat += [len(keep)] + keep
                i += 1 + n
            d = np.array(flat, dtype=np.uint32)
        out.append((kind, phase, stage, d))
    return out


def _key(rec):
    kind, phase, stage, _ = rec
    return (kind, phase, stage)


def compare(a: list, b: list, kinds=None, set_kinds=("trail",)) -> list:
    """Compare two dumps record by record; returns a list of mismatch strings (empty = equal).

    Records are matched by (kind, phase, stage). ``trail`` records compare as sets
    (the order of units found by one propagation pass is not part of the contract).
    Timing records are ignored.
    """
    ia = {_key(r): r[3] for r in a if r[0] != "timing"}
    ib = {_key(r): r[3] for r in b if r[0] != "timing"}
    errs = []
    keys = [k for k in ia if k in ib and (kinds is None or k[0] in kinds)]
    for k in sorted(set(ia) ^ set(ib)):
        if kinds is None or k[0] in kinds:
            errs.append(f"record {k} only in {'first' if k in ia else 'second'}")
    order = {"input": 0, "prop": 1, "lcve": 2, "sort": 3, "sub": 4, "ve": 5, "bce": 6, "ere": 7, "final": 8}
    keys.sort(key=lambda k: (k[1], order.get(k[2], 99), k[0]))
    for k in keys:
        x, y = ia[k], ib[k]
        if k[0] in set_kinds:
            if set(x.tolist()) != set(y.tolist()):
                errs.append(f"{k}: sets differ (|a|={x.size}, |b|={y.size})")
            continue
        if x.size != y.size or not np.array_equal(x, y):
            where = int(np.argmax(x[:min(x.size, y.size)] != y[:min(x.size, y.size)])) if min(x.size, y.size) else 0
            errs.append(f"{k}: differ (len {x.size} vs {y.size}, first diff at word {where})")
    return errs
