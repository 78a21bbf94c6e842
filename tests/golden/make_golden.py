"""Generate the golden fixtures from the compiled reference simplifier.

Runs oracle/_ref/sigma_ref (the reference ParaFROST CPU simplifier built from its
own sources by oracle/ref.mk) on seeded synthetic formulas and stores, per case,
the generator call, a hash of the input and the reference's outputs: status,
per-phase elected-variable counts and hashes, eliminated variables, witness stack,
units and the canonical (sorted) simplified clause multiset. Small cases also keep
the full clause list. Regenerate with:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from parafrost_gb300 import cnfgen, rounddump  # noqa: E402
from parafrost_gb300.options import Options  # noqa: E402

CASES = [
    # name, generator, kwargs, options
    ("ksat3_10k_s1", "random_ksat", dict(num_vars=10_000, num_clauses=42_600, k=3, seed=1), dict(all=1)),
    ("ksat3_10k_s2_default", "random_ksat", dict(num_vars=10_000, num_clauses=42_600, k=3, seed=2), dict()),
    ("ksat3_200_s3", "random_ksat", dict(num_vars=200, num_clauses=852, k=3, seed=3), dict(all=1)),
    ("ksat2_400_s4", "random_ksat", dict(num_vars=400, num_clauses=300, k=2, seed=4), dict(all=1)),
    ("ksat2_300_unsat_s1", "random_ksat", dict(num_vars=300, num_clauses=600, k=2, seed=1), dict(all=1)),
    ("aig_3k_s1", "aig_tseitin", dict(num_inputs=200, num_and=3000, num_xor=400, seed=1), dict(all=1)),
    ("aig_30k_s2", "aig_tseitin", dict(num_inputs=2000, num_and=30000, num_xor=3000, seed=2), dict(all=1)),
    ("aig_3k_s3_tight", "aig_tseitin", dict(num_inputs=200, num_and=3000, num_xor=400, seed=3),
     dict(all=1, gc_freq=1, mu_pos=10, mu_neg=10)),
    ("mixed_5k_s1", "random_mixed_ksat", dict(num_clauses=5000, ratio=4.0, seed=1), dict(all=1)),
    ("mixed_5k_s2_lbound", "random_mixed_ksat", dict(num_clauses=5000, ratio=2.5, seed=2), dict(all=1, ve_lbound=1)),
    ("community_12k_s1", "community", dict(num_vars=4000, num_clauses=12000, communities=10, seed=1), dict(all=1)),
    ("community_12k_s2", "community", dict(num_vars=4000, num_clauses=12000, communities=10, seed=2),
     dict(all=1, phases=3)),
    ("community_80k_s3", "community", dict(num_vars=20000, num_clauses=80000, communities=20, seed=3), dict(all=1)),
    # inprocessing inputs: the last clauses enter the round as learnt clauses (after
    # the original ones, the order awaken() extracts them in)
    ("ksat3_10k_s5_learnt", "random_ksat", dict(num_vars=10_000, num_clauses=42_600, k=3, seed=5), dict(all=1),
     8_000),
    ("aig_30k_s6_learnt", "aig_tseitin", dict(num_inputs=2000, num_and=30000, num_xor=3000, seed=6), dict(all=1),
     20_000),
    ("community_12k_s7_learnt", "community", dict(num_vars=4000, num_clauses=12000, communities=10, seed=7),
     dict(all=1, phases=3), 3_000),
    # root-level units among the input clauses (propagated before the first phase)
    ("aig_33k_s7_units", "with_units_of",
     dict(gen="aig_tseitin", count=40, num_inputs=2000, num_and=30000, num_xor=3000, seed=7), dict(all=1)),
    ("community_80k_s8_units", "with_units_of",
     dict(gen="community", count=100, num_vars=20000, num_clauses=80000, communities=20, seed=8), dict(all=1)),
    ("ksat3_2k_s9_units", "with_units_of", dict(gen="random_ksat", count=120, unit_seed=6, num_vars=2000,
                                                num_clauses=7000, k=3, seed=9), dict(all=1)),
]

SMALL = 20_000  # keep full clause lists below this many output clauses


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def canonical_clause_array(clauses: list) -> np.ndarray:
    """[n, (status, size, lits...)*] of the sorted clause multiset."""
    flat = [len(clauses)]
    for st, lits in clauses:
        flat += [st, len(lits)] + list(lits)
    return np.array(flat, dtype=np.uint32)


def summarize(recs: list) -> dict:
    canon = rounddump.canonical(recs)
    out = {"status": canon["status"]}
    pvs = [(ph, d) for (k, ph, st, d) in recs if k == "pvs"]
    out["pv_counts"] = [int(d.size) for _, d in pvs]
    out["pv_hash"] = digest(*[d for _, d in pvs]) if pvs else ""
    if canon["status"] == 0:
        out["elim"] = np.array(canon["elim"], dtype=np.uint32)
        out["resolved"] = np.array(canon["resolved"], dtype=np.uint32)
        out["units"] = np.array(canon["units"], dtype=np.uint32)
        cls = canonical_clause_array(canon["clauses"])
        out["clauses_hash"] = digest(cls)
        out["num_clauses"] = len(canon["clauses"])
        out["clauses"] = cls if len(canon["clauses"]) <= SMALL else None
    return out


def main() -> None:
    import oracle_runner as orr
    if not orr.reference_available():
        raise SystemExit("compiled reference missing: run __graft_entry__.build() where the reference sources are")
    index = {}
    for name, gen, kw, opt, *tail in CASES:
        learnt_tail = tail[0] if tail else 0
        nv, lits, off = getattr(cnfgen, gen)(**kw)
        recs = orr.run_reference(nv, lits, off, Options(**opt), level=1, learnt_tail=learnt_tail)
        s = summarize(recs)
        arrays = {k: v for k, v in s.items() if isinstance(v, np.ndarray)}
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
        meta = {k: v for k, v in s.items() if not isinstance(v, np.ndarray) and v is not None}
        meta.update(generator=gen, kwargs=kw, options=opt, input_hash=digest(lits, off), num_vars=nv)
        if learnt_tail:
            meta["learnt_tail"] = learnt_tail
        index[name] = meta
        print(name, meta["status"], meta.get("num_clauses"), meta["pv_counts"])
    with open(os.path.join(HERE, "index.json"), "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
