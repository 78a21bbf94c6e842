"""Seeded synthetic CNF generators for the sigmify workloads.

No public benchmark suite is used: each generator builds a formula with the
shape, size and value distribution of one workload and is fully determined by
its seed (a counter-based splitmix64 stream, so x86 and Arm hosts and every
numpy version produce the same formula).

Formulas are returned as ``(num_vars, lits, offsets)`` in the solver's literal
encoding ``lit = 2*var + sign`` (sign 1 = negative, variables 1..num_vars), the
encoding of ParaFROST's clause store (src/cpu/const.h:73-78). ``lits`` is a
uint32 array, ``offsets`` a uint64 array of length ``num_clauses + 1``.
Literals inside a clause are in generation order (the upload normalises them,
as ``extract`` does in src/cpu/simplify.cpp:95-113); no clause repeats a
variable, so the reference parser keeps every clause unchanged.
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    """Vectorised splitmix64 finaliser over a uint64 counter array."""
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


class Stream:
    """Counter-based random stream: draw i of stream (seed, tag) = splitmix64(...)."""

    def __init__(self, seed: int, tag: int = 0):
        with np.errstate(over="ignore"):
            self.key = _splitmix64(np.array([(seed * 0x100000001B3 + tag) & 0xFFFFFFFFFFFFFFFF], dtype=np.uint64))[0]
        self.pos = 0

    def u64(self, n: int) -> np.ndarray:
        ctr = np.arange(self.pos, self.pos + n, dtype=np.uint64)
        self.pos += n
        with np.errstate(over="ignore"):
            return _splitmix64(ctr * np.uint64(0xD1B54A32D192ED03) + self.key)

    def below(self, bound, n: int) -> np.ndarray:
        """n integers uniform in [0, bound) (bound scalar or array, < 2**32)."""
        r = self.u64(n) >> np.uint64(32)
        return ((r * np.asarray(bound, dtype=np.uint64)) >> np.uint64(32)).astype(np.int64)

    def unit(self, n: int) -> np.ndarray:
        """n floats uniform in [0, 1)."""
        return (self.u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _pack(num_vars: int, var_rows: list, sign_rows: list) -> tuple:
    """Concatenate clause rows (arrays of equal-length clauses) into lits/offsets."""
    sizes, lits = [], []
    for vars_, signs in zip(var_rows, sign_rows):
        k = vars_.shape[1]
        sizes.append(np.full(vars_.shape[0], k, dtype=np.uint64))
        lits.append(((vars_.astype(np.uint32) << 1) | signs.astype(np.uint32)).reshape(-1))
    return num_vars, np.concatenate(lits), np.concatenate([[0], np.cumsum(np.concatenate(sizes))]).astype(np.uint64)


def _plant(st: Stream, planted: np.ndarray, var: np.ndarray, sign: np.ndarray, owner: np.ndarray, n: int) -> np.ndarray:
    """Flip one random literal of every clause that the planted assignment falsifies.

    A literal (var, sign) is true under the assignment when sign == 1 - planted[var].
    """
    true_lit = (sign ^ 1) == planted[var]
    sat = np.bincount(owner, weights=true_lit.astype(np.float64), minlength=n) > 0
    dead = np.nonzero(~sat)[0]
    if dead.size:
        starts = np.searchsorted(owner, dead)
        sizes = np.searchsorted(owner, dead, side="right") - starts
        pos = starts + st.below(sizes, dead.size)
        sign = sign.copy()
        sign[pos] ^= 1
    return sign


def _distinct_rows(st: Stream, draw, rows: np.ndarray) -> np.ndarray:
    """Redraw rows that repeat a variable until every row is duplicate-free."""
    while True:
        s = np.sort(rows, axis=1)
        bad = np.nonzero((s[:, 1:] == s[:, :-1]).any(axis=1))[0]
        if bad.size == 0:
            return rows
        rows[bad] = draw(bad.size)


def random_ksat(num_vars: int, num_clauses: int, k: int = 3, seed: int = 1) -> tuple:
    """Uniform random k-SAT: k distinct variables per clause, fair signs."""
    st = Stream(seed, 1)
    draw = lambda n: 1 + st.below(num_vars, n * k).reshape(n, k)
    vars_ = _distinct_rows(st, draw, draw(num_clauses))
    signs = st.below(2, num_clauses * k).reshape(num_clauses, k)
    return _pack(num_vars, [vars_], [signs])


def random_mixed_ksat(num_clauses: int, ratio: float, kmin: int = 2, kmax: int = 5, seed: int = 1,
                      plant: bool = True) -> tuple:
    """Random CNF with clause length uniform in [kmin, kmax] (batched workload).

    With ``plant`` the formula is kept satisfiable as in ``community``."""
    num_vars = max(kmax + 1, int(round(num_clauses / ratio)))
    st = Stream(seed, 4)
    ks = kmin + st.below(kmax - kmin + 1, num_clauses)
    cols = np.arange(kmax)
    used = cols[None, :] < ks[:, None]
    sentinel = -(cols[None, :] + 1)

    def draw(rows_k):
        v = 1 + st.below(num_vars, rows_k.size * kmax).reshape(rows_k.size, kmax)
        return np.where(cols[None, :] < rows_k[:, None], v, sentinel)

    vars_ = draw(ks)
    while True:
        s = np.sort(vars_, axis=1)
        bad = np.nonzero((s[:, 1:] == s[:, :-1]).any(axis=1))[0]
        if bad.size == 0:
            break
        vars_[bad] = draw(ks[bad])
    signs = st.below(2, num_clauses * kmax).reshape(num_clauses, kmax)
    if plant:
        # keep the formula satisfiable: flip one literal of each clause falsified by a seeded assignment
        planted = st.below(2, num_vars + 1).astype(np.int64)
        v = np.where(used, vars_, 0)
        sat = ((signs ^ 1) == planted[v]) & used   # literal true under the planted assignment
        dead = np.nonzero(~sat.any(axis=1))[0]
        pick = st.below(ks[dead], dead.size)
        signs[dead, pick] ^= 1
    lits = ((vars_.astype(np.int64) << 1) | signs)[used].astype(np.uint32)
    off = np.concatenate([[0], np.cumsum(ks)]).astype(np.uint64)
    return num_vars, lits, off


def _aig_structure(num_inputs: int, num_and: int, num_xor: int, window: float, seed: int) -> tuple:
    """Gate nodes, fan-in nodes with polarities, and XOR flags of the random AIG."""
    st = Stream(seed, 2)
    num_gates = num_and + num_xor
    num_vars = num_inputs + num_gates
    g = np.arange(num_inputs + 1, num_vars + 1, dtype=np.int64)
    lo = np.maximum(1, g - np.maximum(2, (window * (g - 1)).astype(np.int64)))
    span = g - lo
    a = lo + st.below(span, num_gates)
    b = lo + st.below(span, num_gates)
    while True:
        same = np.nonzero(a == b)[0]
        if same.size == 0:
            break
        b[same] = lo[same] + st.below(span[same], same.size)
    pa = st.below(2, num_gates)
    pb = st.below(2, num_gates)
    is_xor = np.zeros(num_gates, dtype=bool)
    # choose exactly num_xor XOR positions: rank gates by a random key
    key = st.u64(num_gates)
    is_xor[np.argsort(key, kind="stable")[:num_xor]] = True
    return g, a, b, pa, pb, is_xor


def aig_tseitin(num_inputs: int = 50_000, num_and: int = 2_000_000, num_xor: int = 200_000,
                window: float = 0.10, seed: int = 1) -> tuple:
    """Tseitin encoding of a seeded random and-inverter graph with XOR gates.

    Node n (variables 1..num_inputs are primary inputs) takes two distinct fan-in
    nodes from the most recent ``window`` fraction of nodes before it, each with a
    random polarity. AND: (-g a)(-g b)(g -a -b); XOR: (-g a b)(-g -a -b)(g -a b)(g a -b).
    """
    g, a, b, pa, pb, is_xor = _aig_structure(num_inputs, num_and, num_xor, window, seed)
    num_gates = num_and + num_xor
    num_vars = num_inputs + num_gates
    la = (a << 1) | pa
    lb = (b << 1) | pb
    lg = g << 1
    sizes = np.where(is_xor, 4 * 3, 2 + 2 + 3).astype(np.int64)  # literals per gate block
    ncls = np.where(is_xor, 4, 3)
    total = int(sizes.sum())
    out = np.empty(total, dtype=np.uint32)
    csz = np.empty(int(ncls.sum()), dtype=np.uint64)
    start = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    cstart = np.concatenate([[0], np.cumsum(ncls)[:-1]])
    A = ~is_xor
    s, c = start[A], cstart[A]
    ga, aa, bb = lg[A], la[A], lb[A]
    out[s + 0], out[s + 1] = ga | 1, aa
    out[s + 2], out[s + 3] = ga | 1, bb
    out[s + 4], out[s + 5], out[s + 6] = ga, aa ^ 1, bb ^ 1
    csz[c + 0], csz[c + 1], csz[c + 2] = 2, 2, 3
    X = is_xor
    s, c = start[X], cstart[X]
    gx, ax, bx = lg[X], la[X], lb[X]
    out[s + 0], out[s + 1], out[s + 2] = gx | 1, ax, bx
    out[s + 3], out[s + 4], out[s + 5] = gx | 1, ax ^ 1, bx ^ 1
    out[s + 6], out[s + 7], out[s + 8] = gx, ax ^ 1, bx
    out[s + 9], out[s + 10], out[s + 11] = gx, ax, bx ^ 1
    csz[c + 0] = csz[c + 1] = csz[c + 2] = csz[c + 3] = 3
    off = np.concatenate([[0], np.cumsum(csz)]).astype(np.uint64)
    return num_vars, out, off


def aig_unrolled(num_gates: int = 5_000, steps: int = 5, num_inputs: int | None = None,
                 num_latches: int | None = None, window: float = 0.10, seed: int = 1) -> tuple:
    """Bounded unrolling of a seeded random sequential AIG (serving requests).

    One frame has ``num_inputs`` inputs, ``num_latches`` latches and ``num_gates``
    AND gates; gate fan-ins are two distinct earlier nodes of the frame (inputs,
    latches, gates) from the most recent ``window`` fraction, with random
    polarity. Frame 0's latches are fresh variables reset to 0 by unit clauses; frame
    t's latches are the next-state literals (distinct gates, random polarity) of
    frame t-1. Tseitin per gate: (-g a)(-g b)(g -a -b); the last frame asserts one
    gate output (the property's bad state) as a unit clause.
    """
    ni = num_inputs if num_inputs is not None else max(2, num_gates // 10)
    nl = num_latches if num_latches is not None else max(1, num_gates // 10)
    nl = min(nl, num_gates)
    st = Stream(seed, 7)
    nodes = ni + nl + num_gates
    g = np.arange(ni + nl + 1, nodes + 1, dtype=np.int64)  # gate node ids of a frame
    lo = np.maximum(1, g - np.maximum(2, (window * (g - 1)).astype(np.int64)))
    span = g - lo
    next_var = 1
    lits_parts, size_parts = [], []
    latch_lits = None
    for t in range(steps):
        lit_of = np.zeros(nodes + 1, dtype=np.int64)
        lit_of[1:ni + 1] = (np.arange(next_var, next_var + ni, dtype=np.int64) << 1)
        next_var += ni
        if t == 0:
            lv = np.arange(next_var, next_var + nl, dtype=np.int64)
            next_var += nl
            lit_of[ni + 1:ni + nl + 1] = lv << 1
            lits_parts.append(((lv << 1) | 1).astype(np.uint32))  # reset: latch = 0
            size_parts.append(np.ones(nl, dtype=np.uint64))
        else:
            lit_of[ni + 1:ni + nl + 1] = latch_lits
        gv = np.arange(next_var, next_var + num_gates, dtype=np.int64)
        next_var += num_gates
        lit_of[ni + nl + 1:] = gv << 1
        a = lo + st.below(span, num_gates)
        b = lo + st.below(span, num_gates)
        while True:
            same = np.nonzero(a == b)[0]
            if same.size == 0:
                break
            b[same] = lo[same] + st.below(span[same], same.size)
        la = lit_of[a] ^ st.below(2, num_gates)
        lb = lit_of[b] ^ st.below(2, num_gates)
        lg = gv << 1
        blk = np.empty((num_gates, 7), dtype=np.int64)
        blk[:, 0], blk[:, 1] = lg | 1, la
        blk[:, 2], blk[:, 3] = lg | 1, lb
        blk[:, 4], blk[:, 5], blk[:, 6] = lg, la ^ 1, lb ^ 1
        lits_parts.append(blk.reshape(-1).astype(np.uint32))
        size_parts.append(np.tile(np.array([2, 2, 3], dtype=np.uint64), num_gates))
        # next-state literals: distinct gates of this frame
        pick = np.argsort(st.u64(num_gates), kind="stable")[:nl]
        latch_lits = (gv[pick] << 1) ^ st.below(2, nl)
    bad = (int(next_var - 1 - st.below(num_gates, 1)[0]) << 1)
    lits_parts.append(np.array([bad], dtype=np.uint32))
    size_parts.append(np.ones(1, dtype=np.uint64))
    off = np.concatenate([[0], np.cumsum(np.concatenate(size_parts))]).astype(np.uint64)
    return next_var - 1, np.concatenate(lits_parts), off


def serving_requests(num: int, seed: int = 1, cmin: int = 10_000, cmax: int = 5_000_000):
    """Serving requests: unrolled AIGs with gates log-uniform in [5k, 50k] and steps
    log-uniform in [5, 100], kept when the clause count is within [cmin, cmax]."""
    st = Stream(seed, 8)
    out, i = [], 0
    while len(out) < num:
        u = st.unit(2)
        gates = int(np.exp(np.log(5_000) + u[0] * np.log(10.0)))
        steps = int(np.exp(np.log(5) + u[1] * np.log(20.0)))
        ncls = steps * 3 * gates + gates // 10 + 1
        i += 1
        if cmin <= ncls <= cmax:
            out.append(aig_unrolled(gates, steps, seed=seed * 1_000_003 + i))
    return out


def community(num_vars: int = 20_000_000, num_clauses: int = 80_000_000, communities: int = 200,
              modularity: float = 0.8, mean_len: float = 3.5, max_len: int = 64,
              exponent: float = 2.5, seed: int = 1, chunk: int = 8_000_000, plant: bool = True) -> tuple:
    """Community-attachment industrial-like CNF.

    Clause length is 1 + Geometric(p) with mean ``mean_len`` clipped to
    [2, max_len]. With probability ``modularity`` all literals of a clause come
    from one community, otherwise each literal picks its community uniformly.
    Inside a community, the variable of frequency rank r (0-based) is drawn with
    probability proportional to (r+1)^(-1/(exponent-1)) (a power law in variable
    frequency with the given exponent); ranks map to variables through a seeded
    permutation. With ``plant`` a seeded assignment is drawn first and one random
    literal of every clause it falsifies is flipped, so the formula stays
    satisfiable (dense binaries among hub variables otherwise make it trivially
    UNSAT in the first phase).
    """
    st = Stream(seed, 3)
    planted = (st.below(2, num_vars + 1).astype(np.int64)) if plant else None
    per = num_vars // communities
    assert per * communities == num_vars
    beta = 1.0 / (exponent - 1.0)
    w = np.arange(1, per + 1, dtype=np.float64) ** (-beta)
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    perm = np.argsort(st.u64(num_vars), kind="stable").astype(np.uint32) + 1  # rank -> variable
    p = 1.0 / (mean_len - 1.0)
    lits_parts, sizes_parts = [], []
    done = 0
    while done < num_clauses:
        n = min(chunk, num_clauses - done)
        u = st.unit(n)
        k = 1 + np.ceil(np.log1p(-u) / np.log1p(-p)).astype(np.int64)
        k = np.clip(k, 2, max_len)
        total = int(k.sum())
        owner = np.repeat(np.arange(n), k)
        local = st.below(communities, n)
        modular = st.unit(n) < modularity
        lit_comm = np.where(modular[owner], local[owner], st.below(communities, total))
        rank = np.searchsorted(cdf, st.unit(total), side="right")
        rank = np.minimum(rank, per - 1)
        var = perm[lit_comm * per + rank].astype(np.int64)
        # redraw repeated variables inside a clause; after the first pass only the
        # clauses that had a repeat can have one, so later passes look at those alone
        # (their positions keep the same relative order, so the redraws are the same)
        starts = np.concatenate([[0], np.cumsum(k)[:-1]])
        idx = None
        while True:
            o = owner if idx is None else owner[idx]
            key = o * np.int64(num_vars + 1) + (var if idx is None else var[idx])
            order = np.argsort(key, kind="stable")
            sk = key[order]
            dup = order[1:][sk[1:] == sk[:-1]]
            if idx is not None:
                dup = idx[dup]
            if dup.size == 0:
                break
            rr = np.minimum(np.searchsorted(cdf, st.unit(dup.size), side="right"), per - 1)
            var[dup] = perm[lit_comm[dup] * per + rr]
            own = np.unique(owner[dup])
            lens = k[own]
            first = np.cumsum(lens) - lens
            idx = np.repeat(starts[own] - first, lens) + np.arange(int(lens.sum()), dtype=np.int64)
        sign = st.below(2, total)
        if planted is not None:
            sign = _plant(st, planted, var, sign, owner, n)
        lits_parts.append(((var.astype(np.uint32) << 1) | sign.astype(np.uint32)))
        sizes_parts.append(k.astype(np.uint64))
        del starts
        done += n
    lits = np.concatenate(lits_parts)
    off = np.concatenate([[0], np.cumsum(np.concatenate(sizes_parts))]).astype(np.uint64)
    return num_vars, lits, off


def community_planted(num_vars: int = 20_000_000, seed: int = 1) -> np.ndarray:
    """The assignment ``community(..., plant=True)`` plants (uint8 per variable,
    1 = true, index 0 unused): the first draw of the generator's stream."""
    return Stream(seed, 3).below(2, num_vars + 1).astype(np.uint8)


def aig_model(num_inputs: int = 50_000, num_and: int = 2_000_000, num_xor: int = 200_000,
              window: float = 0.10, seed: int = 1, input_seed: int = 7) -> np.ndarray:
    """A satisfying assignment of ``aig_tseitin`` with the same arguments: seeded
    random inputs, every gate evaluated in order (uint8 per variable, 1 = true)."""
    g, a, b, pa, pb, is_xor = _aig_structure(num_inputs, num_and, num_xor, window, seed)
    val = np.zeros(num_inputs + num_and + num_xor + 1, dtype=np.uint8)
    val[1:num_inputs + 1] = Stream(input_seed, 9).below(2, num_inputs).astype(np.uint8)
    av, bv, xv = a.tolist(), b.tolist(), is_xor.tolist()
    pav, pbv = pa.tolist(), pb.tolist()
    vl = val.tolist()
    for t, node in enumerate(g.tolist()):
        x = vl[av[t]] ^ (1 if pav[t] else 0)
        y = vl[bv[t]] ^ (1 if pbv[t] else 0)
        vl[node] = (x ^ y) if xv[t] else (x & y)
    return np.array(vl, dtype=np.uint8)


def with_units(num_vars: int, lits: np.ndarray, offsets: np.ndarray, count: int, seed: int = 1,
               model: np.ndarray | None = None) -> tuple:
    """The formula with ``count`` one-literal clauses appended (seeded random
    variables, repeats allowed; random signs, or the signs that make them true
    under ``model``, uint8 per variable): the root-level units an incremental or
    BMC front end passes along with its clauses."""
    st = Stream(seed, 11)
    var = 1 + st.below(num_vars, count)
    sign = st.below(2, count) if model is None else (1 - np.asarray(model, dtype=np.int64)[var])
    units = ((var << 1) | sign).astype(np.uint32)
    off = np.concatenate([offsets, offsets[-1] + 1 + np.arange(count, dtype=np.uint64)]).astype(np.uint64)
    return num_vars, np.concatenate([lits, units]), off


def with_units_of(gen: str, count: int, unit_seed: int = 1, **kw) -> tuple:
    """``with_units`` over the formula ``gen(**kw)`` of this module, with units true
    under the formula's known model (AIG inputs evaluated, or the community
    formula's planted assignment)."""
    model = None
    if gen == "aig_tseitin":
        model = aig_model(**kw)
    elif gen == "community":
        model = community_planted(kw["num_vars"], kw.get("seed", 1))
    return with_units(*globals()[gen](**kw), count=count, seed=unit_seed, model=model)


def batch_ksat(num_formulas: int = 4096, cmin: int = 1_000, cmax: int = 200_000, seed: int = 1,
               indices=None):
    """Batched workload: clause counts log-uniform in [cmin, cmax], ratio U[3.0, 4.5], k in 2..5.
    ``indices`` picks formulas of the batch (each is generated on its own seed)."""
    st = Stream(seed, 5)
    u = st.unit(num_formulas)
    counts = np.exp(np.log(cmin) + u * (np.log(cmax) - np.log(cmin))).astype(np.int64)
    ratios = 3.0 + 1.5 * st.unit(num_formulas)
    for i in (range(num_formulas) if indices is None else indices):
        yield random_mixed_ksat(int(counts[i]), float(ratios[i]), seed=seed * 1_000_003 + i)


WORKLOADS = {
    "ksat3-10k": dict(fn=random_ksat, kw=dict(num_vars=10_000, num_clauses=42_600, k=3)),
    "aig-2.2m": dict(fn=aig_tseitin, kw=dict()),
    "community-20m": dict(fn=community, kw=dict()),
}


def make(name: str, seed: int = 1, **overrides):
    spec = WORKLOADS[name]
    kw = dict(spec["kw"])
    kw.update(overrides)
    return spec["fn"](seed=seed, **kw)


def to_dimacs(path: str, num_vars: int, lits: np.ndarray, offsets: np.ndarray) -> None:
    """Write a DIMACS file (used to feed the reference solver's own parser)."""
    lits = np.asarray(lits, dtype=np.int64)
    ints = (lits >> 1) * np.where(lits & 1, -1, 1)
    n = offsets.size - 1
    with open(path, "w") as f:
        f.write(f"p cnf {num_vars} {n}\n")
        step = 1 << 20
        off = offsets.astype(np.int64)
        for c0 in range(0, n, step):
            c1 = min(n, c0 + step)
            seg = ints[off[c0]:off[c1]]
            sizes = np.diff(off[c0:c1 + 1])
            # insert a 0 terminator after every clause
            ends = np.cumsum(sizes)
            out = np.insert(seg, ends, 0)
            txt = " ".join(map(str, out.tolist()))
            f.write(txt.replace(" 0 ", " 0\n"))
            f.write("\n")
