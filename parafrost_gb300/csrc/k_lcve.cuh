// LCVE election: ParaFROST::LCVE + depFreeze (src/cpu/lcve.cpp:46-100), with the
// variable order of varReorder (lcve.cpp:25-44, histogram.h:32-41, key.h:57-66).
//
// The reference walks candidates in (score, variable) order, skips eliminated,
// zero-occurrence and frozen ones, stops at the first candidate whose two lists
// reach the freezing temperatures (pt, nt), elects the rest and freezes every
// neighbour v with ps[v] < pt or ns[v] < nt. Writing F for those freezable
// variables, the elected set is the lexicographically-first independent set of
// the co-occurrence graph restricted to F, in rank order, cut at the break
// candidate B = the first valid candidate that is either outside F (it is never
// frozen and its lists are necessarily long) or an independent-set member whose
// lists reach the temperatures. The independent set is the greedy one in rank
// order (a vertex joins when every lower-ranked neighbour is out, leaves when one
// lower-ranked neighbour is in), decided by push/pull rounds over the graph
// (mis_rounds_k below).
#pragma once

#include "cnf.cuh"

namespace sigma {

// Independent-set word of a variable, read by every neighbour test: bits 0-29 the
// variable's rank if it is a vertex of the graph (MIS_NO_RANK otherwise; never
// changes while the set is decided), bits 30-31 the decision. Four bytes a
// variable keep the words of a 20M-variable graph (80 MB) in L2 while the walks
// stream clause records past them. Where a vertex's last pull walk stopped (an
// index into its two lists) is a separate word that only the vertex's walk reads.
enum : u32 { MIS_UNDECIDED = 0, MIS_IN = 1, MIS_OUT = 2 };
constexpr u32 MIS_NO_RANK = 0x3FFFFFFFu;
HD u32 mis_rank(u32 w) { return w & MIS_NO_RANK; }
HD u32 mis_dec(u32 w) { return w >> 30; }
HD u32 mis_dec_bits(u32 d) { return d << 30; }

struct LcveArgs {
    Ctx c;
    u32 pt, nt;           // mu_pos << mu_inc, mu_neg << mu_inc
    u32* score;           // nvars+1
    u32* order;           // nvars: variables in (score, var) order
    u32* rank;            // nvars+1
    u32* word;            // nvars+1: independent-set words
    u32* resume;          // nvars+1: where each vertex's last pull walk stopped
    const Q4* crec;       // per clause: its first three literals and size | deleted << 31
    u64* ws_bytes;        // kSpreadSlots words summing the graph's working set (4*occ + sum(8 + 4*len))
    u32* gbits;           // graph membership, one bit per variable (zeroed before k_mis_init)
    u32* bound;           // per formula f: [2f] = B0 (first valid non-F rank), [2f+1] = B
    const u32* f_active;  // batches: formulas taking part in this election (null: all)
    u32* f_npvs;          // batches: elected variables per formula
    u32* pvs;             // elected variables in rank order
    u64 pf = 0, pl = 0;   // L2 policies in the rounds kernel: streams go first, words last
    u32* cmin;            // per clause: the least rank of its graph vertices (MIS_NO_RANK when
                          // it has none or is deleted), built with the clause records
    bool r0 = false;      // the first round's pull: walks test cmin instead of the neighbours
};

// write_scores (histogram.h:32-41): eligible[v-1] = v, scores[v] = ps*ns (32-bit wrap).
// The largest score goes to max_score (it sets how many radix passes the order needs).
HD void k_scores(const LcveArgs& a, u32* max_score, u32 v) {
    u32 sc = 0;
    if (v) {
        sc = a.c.ps[v] * a.c.ns[v];
        a.score[v] = sc;
        a.order[v - 1] = v;
    }
    warp_max_atomic(max_score, sc);
}

HD bool lcve_valid(const Ctx& c, u32 v) {
    if (c.vstate[v]) return false;
    return !(c.ps[v] == 0 && c.ns[v] == 0);
}
HD bool lcve_freezable(const LcveArgs& a, u32 v) { return a.c.ps[v] < a.pt || a.c.ns[v] < a.nt; }
HD bool lcve_big(const LcveArgs& a, u32 v) {
    return a.c.ot_size[V2L(v)] >= a.pt && a.c.ot_size[NEG(V2L(v))] >= a.nt;
}

// rank[v] and B0 = first valid candidate outside F.
HD void k_rank(const LcveArgs& a, u32 p) {
    const u32 v = a.order[p];
    a.rank[v] = p;
    if (lcve_valid(a.c, v) && !lcve_freezable(a, v)) atom_min(&a.bound[2 * fid_of(a.c, v)], p);
}

// The independent set is decided in rounds of two phases:
//   push: every vertex that went in during the last round marks its undecided
//         higher-ranked neighbours out;
//   pull: every undecided vertex walks its live clauses, from where its last walk
//         stopped, looking at its lower-ranked graph neighbours; the first one
//         that is not out stops the walk (the vertex stays undecided and resumes
//         there), and a walk that reaches the end finds every lower neighbour out,
//         so the vertex goes in.
// A vertex goes in exactly when all its lower neighbours are out, and out when a
// lower neighbour is in, as in the greedy walk in rank order. Out is final, so the
// clauses a walk has passed never need another look. Vertices with more than
// MIS_WARP_MIN_OCC clauses are walked by a whole warp; the others by one thread,
// or by a group of lanes when few of them are left (mis_lanes).
constexpr u32 MIS_WARP_MIN_OCC = 32;

struct MisFront {
    u32* small;   // list of small-adjacency vertices
    u32* nsmall;
    u32* big;     // list of large-adjacency vertices
    u32* nbig;
};

HD bool mis_is_big(const Ctx& c, u32 v) { return c.ot_size[V2L(v)] + c.ot_size[NEG(V2L(v))] > MIS_WARP_MIN_OCC; }

HD void mis_append(const MisFront& f, const Ctx& c, u32 v, bool pred) {
    const bool big = pred && mis_is_big(c, v);
    const u32 ps = warp_append(f.nsmall, pred && !big);
    const u32 pb = warp_append(f.nbig, big);
    if (pred && !big) f.small[ps] = v;
    if (big) f.big[pb] = v;
}

// Graph membership; every graph vertex starts on the undecided lists.
HD void k_mis_init(const LcveArgs& a, const MisFront& und, u32 v) {
    const u32 f = v ? fid_of(a.c, v) : 0u;
    const bool in_graph = v && (!a.f_active || a.f_active[f]) && lcve_valid(a.c, v) && lcve_freezable(a, v) &&
                          a.rank[v] < a.bound[2 * f];
    a.word[v] = in_graph ? a.rank[v] : MIS_NO_RANK;
    a.resume[v] = 0;
    bitmap_set(a.gbits, v, in_graph);
    mis_append(und, a.c, v, in_graph);
}

#if SIGMA_CUDA
// k_mis_init over variables 0..n-1 with block-wide appends: a block takes 256
// consecutive variables a step, ranks its small and big vertices by warp ballots and
// reserves both lists' places with one atomic each (the lists' two counters would
// otherwise take one atomic per warp step over 20M variables); lane 0 of a warp
// writes its 32 variables' membership word.
__global__ void __launch_bounds__(256) mis_init_k(LcveArgs a, MisFront und, u32 n) {
    __shared__ u32 ws[8], wb[8], base_s, base_b;
    const u32 lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (u32 v0 = blockIdx.x * 256u; v0 < n; v0 += gridDim.x * 256u) {
        const u32 v = v0 + threadIdx.x;
        bool in_graph = false, big = false;
        if (v < n) {
            const u32 f = v ? fid_of(a.c, v) : 0u;
            in_graph = v && (!a.f_active || a.f_active[f]) && lcve_valid(a.c, v) && lcve_freezable(a, v) &&
                       a.rank[v] < a.bound[2 * f];
            a.word[v] = in_graph ? a.rank[v] : MIS_NO_RANK;
            a.resume[v] = 0;
            big = in_graph && mis_is_big(a.c, v);
        }
        const u32 gm = __ballot_sync(kFull, in_graph);
        if (lane == 0 && v < n) a.gbits[v >> 5] = gm;
        const u32 ms = __ballot_sync(kFull, in_graph && !big), mb = __ballot_sync(kFull, big);
        if (lane == 0) {
            ws[warp] = (u32)__popc(ms);
            wb[warp] = (u32)__popc(mb);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            u32 ts = 0, tb = 0;
            for (u32 k = 0; k < 8; k++) {
                const u32 xs = ws[k], xb = wb[k];
                ws[k] = ts;
                wb[k] = tb;
                ts += xs;
                tb += xb;
            }
            base_s = ts ? atomicAdd(und.nsmall, ts) : 0u;
            base_b = tb ? atomicAdd(und.nbig, tb) : 0u;
        }
        __syncthreads();
        const u32 below = (1u << lane) - 1u;
        if (in_graph && !big) und.small[base_s + ws[warp] + (u32)__popc(ms & below)] = v;
        if (big) und.big[base_b + wb[warp] + (u32)__popc(mb & below)] = v;
        __syncthreads();
    }
}
#endif

// The clause walks read literals four at a time, so the loads (and the pushes'
// atomics) of a chunk are in flight together. Clauses and lists are not written
// while the independent set is decided.
constexpr u32 MIS_CHUNK = 4;

// A clause as the election reads it: one 16-byte record holding its first three
// literals and its size and deleted bit (built once per election by k_mis_rec), so
// clauses of up to three literals cost one load; longer ones read the rest of
// their literals from the store.
// In the first round no vertex is out yet, so a clause stops a walk of v exactly when
// one of its graph vertices ranks below v: when its least rank (cmin) is below v's.
// The first round's walks then load one word per clause (kept in q.x) instead of the
// record and the neighbours' words.
struct MisCl {
    Q4 q;
    u32 r;
    bool r0;
    HD bool deleted() const { return !r0 && (q.w >> 31) != 0; }
    HD u32 size() const { return q.w & 0x7FFFFFFFu; }
};
HD MisCl mis_cl(const LcveArgs& a, u32 r) {
    MisCl cl;
    cl.r = r;
    cl.r0 = a.r0;
    if (a.r0) {
        cl.q.x = ldro_hint(&a.cmin[r], a.pf);
        cl.q.y = cl.q.z = cl.q.w = 0;
    } else {
        cl.q = ldro4_hint(&a.crec[r], a.pf);
    }
    return cl;
}
// Literal k of the clause; L is the clause's literal array (read only for k >= 3).
HD u32 mis_lit(const MisCl& cl, const u32* L, u32 k) {
    return k == 0 ? cl.q.x : k == 1 ? cl.q.y : k == 2 ? cl.q.z : ldro(L + k);
}
HD const u32* mis_long_lits(const LcveArgs& a, const MisCl& cl) {
    return cl.size() > 3 ? a.c.lits + hdr_ro(&a.c.hdr[cl.r]).start : nullptr;
}

// The record of clause i, and the graph's working set: every graph vertex's list
// entry (4 bytes) and, for a live clause, its header and literals (8 + 4*len) once
// per graph vertex in it. Runs after k_mis_init.
HD void k_mis_rec(const LcveArgs& a, Q4* rec, u32 i) {
    const Ctx& c = a.c;
    const Hdr h = c.hdr[i];
    const u32* l = c.lits + h.start;
    Q4 q;
    q.x = h.size > 0 ? l[0] : 0u;
    q.y = h.size > 1 ? l[1] : 0u;
    q.z = h.size > 2 ? l[2] : 0u;
    q.w = h.size | (h_deleted(h.flags) ? 0x80000000u : 0u);
    rec[i] = q;
    u32 ng = 0, m = MIS_NO_RANK;
    for (u32 k = 0; k < h.size; k++) {
        const u32 x = ABS(l[k]);
        ng += (ldro(&a.gbits[x >> 5]) >> (x & 31u)) & 1u;
        const u32 rk = mis_rank(a.word[x]);
        if (rk < m) m = rk;
    }
    a.cmin[i] = h_deleted(h.flags) ? MIS_NO_RANK : m;
    spread_sum_add64(a.ws_bytes, (u64)ng * (4ull + (h_deleted(h.flags) ? 0ull : 8ull + 4ull * h.size)));
}

#if SIGMA_CUDA
// k_mis_rec for 32 clauses per warp: lane i writes the record of clause id0 + i
// (coalesced 16-byte stores), and the graph working set is summed over the warp's
// literals with consecutive lanes on consecutive literals (coalesced reads), each
// literal of a graph vertex adding 4 bytes and, in a live clause, the clause's
// 8 + 4 * len bytes.
__global__ void __launch_bounds__(256) mis_rec_warp_k(LcveArgs a, Q4* rec) {
    __shared__ u32 s_min[256];  // per lane of the block: the least rank of its clause
    const u32 lane = threadIdx.x & 31u;
    const u32 nw = (gridDim.x * blockDim.x) >> 5;
    const u32 ngroups = (a.c.ncls + 31u) / 32u;
    u64 sum = 0;
    for (u32 g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < ngroups; g += nw) {
        const u32 id0 = g * 32u;
        const u32 n = a.c.ncls - id0 < 32u ? a.c.ncls - id0 : 32u;
        u32 start = 0, sz = 0, weight = 0;
        bool dead = true;
        s_min[threadIdx.x] = MIS_NO_RANK;
        __syncwarp();
        if (lane < n) {
            const Hdr h = hdr_ro(&a.c.hdr[id0 + lane]);
            const u32* l = a.c.lits + h.start;
            Q4 q;
            q.x = h.size > 0 ? __ldg(&l[0]) : 0u;
            q.y = h.size > 1 ? __ldg(&l[1]) : 0u;
            q.z = h.size > 2 ? __ldg(&l[2]) : 0u;
            q.w = h.size | (h_deleted(h.flags) ? 0x80000000u : 0u);
            rec[id0 + lane] = q;
            start = h.start;
            sz = h.size;
            weight = 4u + (h_deleted(h.flags) ? 0u : 8u + 4u * h.size);
            dead = h_deleted(h.flags);
        }
        u32 incl = sz;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u32 t = __shfl_up_sync(0xffffffffu, incl, o);
            if ((int)lane >= o) incl += t;
        }
        const u32 excl = incl - sz;
        const u32 total = __shfl_sync(0xffffffffu, incl, 31);
        for (u32 base = 0; base < total; base += 32) {
            const u32 j = base + lane;
            u32 k = 0;
#pragma unroll
            for (u32 step = 16; step; step >>= 1) {
                const u32 v = __shfl_sync(0xffffffffu, incl, k + step - 1);
                if (v <= j) k += step;
            }
            const u32 st = __shfl_sync(0xffffffffu, start, k & 31u), ex = __shfl_sync(0xffffffffu, excl, k & 31u);
            const u32 wt = __shfl_sync(0xffffffffu, weight, k & 31u);
            if (j < total) {
                const u32 x = ABS(__ldg(&a.c.lits[st + (j - ex)]));
                if ((ldro(&a.gbits[x >> 5]) >> (x & 31u)) & 1u) {
                    sum += wt;
                    atomicMin(&s_min[(threadIdx.x & ~31u) + (k & 31u)], mis_rank(ldro(&a.word[x])));
                }
            }
        }
        __syncwarp();
        if (lane < n) a.cmin[id0 + lane] = dead ? MIS_NO_RANK : s_min[threadIdx.x];
    }
    for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0 && sum) atomicAdd((unsigned long long*)(a.ws_bytes + (blockIdx.x & (kSpreadSlots - 1u))),
                                    (unsigned long long)sum);
}
#endif

// Whether clause cl holds a graph neighbour of v ranked below rv that is not out
// (decisions are read through to the cache level other SMs write).
HD bool mis_blocked_in(const LcveArgs& a, u32 v, u32 rv, const MisCl& cl) {
    if (cl.r0) return cl.q.x < rv;
    if (cl.deleted()) return false;
    const u32 size = cl.size();
    const u32* L = mis_long_lits(a, cl);
    for (u32 k0 = 0; k0 < size; k0 += MIS_CHUNK) {
        u32 w[MIS_CHUNK];
#pragma unroll
        for (u32 j = 0; j < MIS_CHUNK; j++) w[j] = k0 + j < size ? ABS(mis_lit(cl, L, k0 + j)) : v;
        bool b = false;
#pragma unroll
        for (u32 j = 0; j < MIS_CHUNK; j++) {
            if (w[j] == v) continue;
            const u32 g = ldcg_hint(&a.word[w[j]], a.pl);
            b |= mis_rank(g) < rv && mis_dec(g) != MIS_OUT;
        }
        if (b) return true;
    }
    return false;
}

// Pull walk of undecided vertex v by one thread: true when v went in; otherwise the
// resume point is stored (v stays undecided). The next clause's record is loaded
// before the current one is examined.
HD bool mis_pull_one(const LcveArgs& a, u32 v, u32 wv) {
    const u32 rv = mis_rank(wv);
    const u32 p = V2L(v), np = a.c.ot_size[p], n = np + a.c.ot_size[p + 1];
    const u32 op = a.c.ot_off[p], on = a.c.ot_off[p + 1] - np;
    u32 t = vload(&a.resume[v]);
    if (t < n) {
        MisCl cl = mis_cl(a, ldro_hint(&a.c.ot_refs[t < np ? op + t : on + t], a.pf));
        for (; t < n; t++) {
            MisCl nx = cl;
            if (t + 1 < n) nx = mis_cl(a, ldro_hint(&a.c.ot_refs[t + 1 < np ? op + t + 1 : on + t + 1], a.pf));
            if (mis_blocked_in(a, v, rv, cl)) {
                a.resume[v] = t;
                return false;
            }
            cl = nx;
        }
    }
    atom_or(&a.word[v], mis_dec_bits(MIS_IN));
    return true;
}

// Push of in vertex u (rank ru) through clause cl: undecided higher neighbours go
// out. The rank in a neighbour's word never changes and a decision is final, so a
// plain (possibly older) load decides whether the atomic is needed.
HD void mis_push_clause(const LcveArgs& a, u32 u, u32 ru, const MisCl& cl) {
    if (cl.deleted()) return;
    const u32 size = cl.size();
    const u32* L = mis_long_lits(a, cl);
    for (u32 k0 = 0; k0 < size; k0 += MIS_CHUNK) {
        u32 w[MIS_CHUNK];
#pragma unroll
        for (u32 j = 0; j < MIS_CHUNK; j++) w[j] = k0 + j < size ? ABS(mis_lit(cl, L, k0 + j)) : u;
#pragma unroll
        for (u32 j = 0; j < MIS_CHUNK; j++) {
            if (w[j] == u) continue;
            const u32 g = ldcg_hint(&a.word[w[j]], a.pl);
            if (mis_rank(g) != MIS_NO_RANK && mis_rank(g) > ru && mis_dec(g) == MIS_UNDECIDED)
                atom_or(&a.word[w[j]], mis_dec_bits(MIS_OUT));
        }
    }
}

HD void mis_push_vertex(const LcveArgs& a, u32 u) {
    const u32 ru = mis_rank(a.word[u]);
    const u32 p = V2L(u), np = a.c.ot_size[p], n = np + a.c.ot_size[p + 1];
    const u32 op = a.c.ot_off[p], on = a.c.ot_off[p + 1] - np;
    if (!n) return;
    MisCl cl = mis_cl(a, ldro_hint(&a.c.ot_refs[op], a.pf));
    for (u32 t = 0; t < n; t++) {
        MisCl nx = cl;
        if (t + 1 < n) nx = mis_cl(a, ldro_hint(&a.c.ot_refs[t + 1 < np ? op + t + 1 : on + t + 1], a.pf));
        mis_push_clause(a, u, ru, cl);
        cl = nx;
    }
}

#if !SIGMA_CUDA
// Serial rounds of the emulation build: the same phases over the same lists.
HD void k_mis_push(const LcveArgs& a, const u32* in, u32 idx) { mis_push_vertex(a, in[idx]); }
HD void k_mis_pull(const LcveArgs& a, const u32* in, const MisFront& und, const MisFront& ins, u32 idx) {
    const u32 v = in[idx];
    const u32 wv = a.word[v];
    if (mis_dec(wv) != MIS_UNDECIDED) return;
    const bool big = mis_is_big(a.c, v);
    if (mis_pull_one(a, v, wv)) {
        if (big) ins.big[atom_add(ins.nbig, 1u)] = v;
        else ins.small[atom_add(ins.nsmall, 1u)] = v;
    } else {
        if (big) und.big[atom_add(und.nbig, 1u)] = v;
        else und.small[atom_add(und.nsmall, 1u)] = v;
    }
}
#else
// All rounds in one cooperative launch. Round r reads the undecided and new-in
// lists u[r&1], in[r&1] (lengths in counter set r%3: undecided small, large, in
// small, large) and writes u[(r+1)&1], in[(r+1)&1] through counter set (r+1)%3;
// set (r+2)%3, last read in round r-1, is cleared for round r+1. Grid barriers
// separate the push phase, the pull phase and the rounds.
struct MisRounds {
    u32* u_small[2];
    u32* u_big[2];
    u32* in_small[2];
    u32* in_big[2];
    u32* ctr;        // three sets of four counters
    u32* bar;        // grid barrier: [0] arrivals, [1] generation
    u32* rounds;     // out: rounds run
    u32 max_rounds;
    u32* trace;      // optional: per round [undecided small, big, went-in small, big, start ns / 1024]
    u32 trace_cap;   // rounds the trace holds
};

// Vertices leaving a pull phase are staged per block in shared memory and copied
// to the next lists with one reservation per block (a vertex that finds its
// block's queue full goes to the list directly).
constexpr u32 MIS_QCAP = 1024;

struct MisBlockQueue {
    u32 small[MIS_QCAP], big[MIS_QCAP];
    u32 ns, nb, base_s, base_b;
};

DEV void mis_queue_push(MisBlockQueue& q, const MisFront& f, bool big, u32 w) {
    if (big) {
        const u32 k = atomicAdd(&q.nb, 1u);
        if (k < MIS_QCAP) q.big[k] = w;
        else f.big[atomicAdd(f.nbig, 1u)] = w;
    } else {
        const u32 k = atomicAdd(&q.ns, 1u);
        if (k < MIS_QCAP) q.small[k] = w;
        else f.small[atomicAdd(f.nsmall, 1u)] = w;
    }
}

// Append of the lanes with pred by one reservation per warp: to the block's queue
// while it has room, the rest to the list. All lanes of the warp take part.
DEV void mis_queue_warp(u32* qa, u32& qn, u32* list, u32* nlist, bool pred, u32 v) {
    const u32 lane = threadIdx.x & 31u;
    const u32 m = __ballot_sync(kFull, pred);
    if (!m) return;
    const u32 cnt = (u32)__popc(m), rank = (u32)__popc(m & ((1u << lane) - 1u));
    u32 k = 0;
    if (lane == 0) k = atomicAdd(&qn, cnt);
    k = __shfl_sync(kFull, k, 0);
    const u32 fit = k < MIS_QCAP ? (cnt < MIS_QCAP - k ? cnt : MIS_QCAP - k) : 0u;
    u32 g = 0;
    if (lane == 0 && cnt > fit) g = atomicAdd(nlist, cnt - fit);
    g = __shfl_sync(kFull, g, 0);
    if (pred) {
        if (rank < fit) qa[k + rank] = v;
        else list[g + rank - fit] = v;
    }
}

// Lanes per vertex for a phase over n small vertices and nth threads: when the list
// is short, each vertex's clauses are spread over a group of up to 32 lanes, so the
// phase waits for one clause walk per vertex instead of a whole list walked by one
// thread.
DEV u32 mis_lanes(u32 n, u32 nth) {
    u32 L = 1;
    while (L < 32u && (u64)n * (2u * L) <= nth) L *= 2u;
    return L;
}

DEV void mis_queue_flush(MisBlockQueue& q, const MisFront& f) {
    __syncthreads();
    const u32 ns = q.ns < MIS_QCAP ? q.ns : MIS_QCAP, nb = q.nb < MIS_QCAP ? q.nb : MIS_QCAP;
    if (threadIdx.x == 0) {
        q.base_s = ns ? atomicAdd(f.nsmall, ns) : 0u;
        q.base_b = nb ? atomicAdd(f.nbig, nb) : 0u;
    }
    __syncthreads();
    for (u32 i = threadIdx.x; i < ns; i += blockDim.x) f.small[q.base_s + i] = q.small[i];
    for (u32 i = threadIdx.x; i < nb; i += blockDim.x) f.big[q.base_b + i] = q.big[i];
    __syncthreads();
    if (threadIdx.x == 0) q.ns = q.nb = 0;
}

__global__ void __launch_bounds__(256, 6) mis_rounds_k(LcveArgs a0, MisRounds w) {
    LcveArgs a = a0;
    a.pf = l2_policy_first();
    a.pl = l2_policy_last();
    __shared__ MisBlockQueue qu, qi;
    const u32 tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const u32 lane = threadIdx.x & 31u, nwarps = nth >> 5;
    if (threadIdx.x == 0) qu.ns = qu.nb = qi.ns = qi.nb = 0;
    __syncthreads();
    for (u32 r = 0;; r++) {
        a.r0 = r == 0;
        const u32 cur = r % 3, nxt = (r + 1) % 3, old = (r + 2) % 3;
        const u32 us = vload(&w.ctr[4 * cur]), ub = vload(&w.ctr[4 * cur + 1]);
        const u32 is = vload(&w.ctr[4 * cur + 2]), ib = vload(&w.ctr[4 * cur + 3]);
        if (!us && !ub && !is && !ib) {
            if (tid == 0) *w.rounds = r;
            return;
        }
        if (r >= w.max_rounds) {
            if (tid == 0) atomicOr(a.c.err, ERR_ITER);
            return;
        }
        if (tid == 0)
            for (u32 k = 0; k < 4; k++) w.ctr[4 * old + k] = 0;
        if (tid == 0 && w.trace && r < w.trace_cap) {
            u32* t = w.trace + 5 * r;
            t[0] = us;
            t[1] = ub;
            t[2] = is;
            t[3] = ib;
            t[4] = (u32)(global_ns() >> 10);
        }
        // push: the vertices that went in last round (lists written by other blocks: uncached reads)
        const u32* pin_b = w.in_big[r & 1];
        for (u32 idx = tid >> 5; idx < ib; idx += nwarps) {
            const u32 u = vload(&pin_b[idx]);
            const u32 ru = mis_rank(a.word[u]);
            const u32 p = V2L(u), np = a.c.ot_size[p], nn = a.c.ot_size[p + 1];
            const u32 op = a.c.ot_off[p], on = a.c.ot_off[p + 1];
            for (u32 t = lane; t < np + nn; t += 32)
                mis_push_clause(a, u, ru, mis_cl(a, ldro_hint(&a.c.ot_refs[t < np ? op + t : on + (t - np)], a.pf)));
            __syncwarp();
        }
        const u32* pin_s = w.in_small[r & 1];
        const u32 li = mis_lanes(is, nth);
        if (li == 1) {
            for (u32 idx = tid; idx < is; idx += nth) mis_push_vertex(a, vload(&pin_s[idx]));
        } else {
            // a group of li lanes per vertex, clauses strided over the group
            const u32 sub = lane & (li - 1u);
            for (u32 idx = tid / li; idx < is; idx += nth / li) {
                const u32 u = vload(&pin_s[idx]);
                const u32 ru = mis_rank(a.word[u]);
                const u32 p = V2L(u), np = a.c.ot_size[p], n = np + a.c.ot_size[p + 1];
                const u32 op = a.c.ot_off[p], on = a.c.ot_off[p + 1] - np;
                for (u32 t = sub; t < n; t += li)
                    mis_push_clause(a, u, ru, mis_cl(a, ldro_hint(&a.c.ot_refs[t < np ? op + t : on + t], a.pf)));
            }
        }
        if (!grid_barrier(w.bar, a.c.err)) return;
        // pull: the undecided vertices
        MisFront fu, fi;
        fu.small = w.u_small[(r + 1) & 1];
        fu.nsmall = &w.ctr[4 * nxt];
        fu.big = w.u_big[(r + 1) & 1];
        fu.nbig = &w.ctr[4 * nxt + 1];
        fi.small = w.in_small[(r + 1) & 1];
        fi.nsmall = &w.ctr[4 * nxt + 2];
        fi.big = w.in_big[(r + 1) & 1];
        fi.nbig = &w.ctr[4 * nxt + 3];
        const u32* pu_b = w.u_big[r & 1];
        for (u32 idx = tid >> 5; idx < ub; idx += nwarps) {
            const u32 v = vload(&pu_b[idx]);
            const u32 wv = vload(&a.word[v]);
            if (mis_dec(wv) != MIS_UNDECIDED) continue;  // warp-uniform
            const u32 rv = mis_rank(wv);
            const u32 p = V2L(v), np = a.c.ot_size[p], n = np + a.c.ot_size[p + 1];
            const u32 op = a.c.ot_off[p], on = a.c.ot_off[p + 1];
            u32 stop = NONE;
            for (u32 b0 = vload(&a.resume[v]); b0 < n && stop == NONE; b0 += 32) {
                const u32 t = b0 + lane;
                const bool blk = t < n && mis_blocked_in(a, v, rv, mis_cl(a, ldro_hint(&a.c.ot_refs[t < np ? op + t : on + (t - np)], a.pf)));
                const u32 m = __ballot_sync(0xffffffffu, blk);
                if (m) stop = b0 + (u32)(__ffs(m) - 1);
            }
            if (lane == 0) {
                if (stop != NONE) {
                    a.resume[v] = stop;
                    mis_queue_push(qu, fu, true, v);
                } else {
                    atomicOr(&a.word[v], mis_dec_bits(MIS_IN));
                    mis_queue_push(qi, fi, true, v);
                }
            }
            __syncwarp();
        }
        const u32* pu_s = w.u_small[r & 1];
        const u32 lu = mis_lanes(us, nth);
        if (lu == 1) {
            // warp-uniform trip count: the appends below take every lane
            for (u32 base = tid - lane; base < us; base += nth) {
                const u32 idx = base + lane;
                u32 v = 0;
                bool in = false, und = false;
                if (idx < us) {
                    v = vload(&pu_s[idx]);
                    const u32 wv = vload(&a.word[v]);
                    if (mis_dec(wv) == MIS_UNDECIDED) {
                        in = mis_pull_one(a, v, wv);
                        und = !in;
                    }
                }
                mis_queue_warp(qi.small, qi.ns, fi.small, fi.nsmall, in, v);
                mis_queue_warp(qu.small, qu.ns, fu.small, fu.nsmall, und, v);
            }
        } else {
            // a group of lu lanes per vertex: batches of lu clauses in list order,
            // the first blocking clause of a batch (lowest lane) stops the walk
            const u32 sub = lane & (lu - 1u), gbase = lane - sub;
            const u32 gmask = lu == 32u ? kFull : ((1u << lu) - 1u) << gbase;
            const u32 gpw = 32u / lu;
            for (u32 base = (tid >> 5) * gpw; base < us; base += nwarps * gpw) {
                const u32 idx = base + lane / lu;
                u32 v = 0;
                bool in = false, und = false;
                if (idx < us) {
                    v = vload(&pu_s[idx]);
                    const u32 wv = vload(&a.word[v]);
                    if (mis_dec(wv) == MIS_UNDECIDED) {  // the same word for the whole group
                        const u32 rv = mis_rank(wv);
                        const u32 p = V2L(v), np = a.c.ot_size[p], n = np + a.c.ot_size[p + 1];
                        const u32 op = a.c.ot_off[p], on = a.c.ot_off[p + 1] - np;
                        u32 stop = NONE;
                        for (u32 b0 = vload(&a.resume[v]); b0 < n; b0 += lu) {
                            const u32 t = b0 + sub;
                            const bool blk =
                                t < n && mis_blocked_in(a, v, rv, mis_cl(a, ldro_hint(&a.c.ot_refs[t < np ? op + t : on + t], a.pf)));
                            const u32 m = (__ballot_sync(gmask, blk) & gmask) >> gbase;
                            if (m) {
                                stop = b0 + (u32)(__ffs(m) - 1);
                                break;
                            }
                        }
                        if (sub == 0) {
                            if (stop != NONE) {
                                a.resume[v] = stop;
                                und = true;
                            } else {
                                atom_or(&a.word[v], mis_dec_bits(MIS_IN));
                                in = true;
                            }
                        }
                    }
                }
                mis_queue_warp(qi.small, qi.ns, fi.small, fi.nsmall, in, v);
                mis_queue_warp(qu.small, qu.ns, fu.small, fu.nsmall, und, v);
            }
        }
        mis_queue_flush(qu, fu);
        mis_queue_flush(qi, fi);
        if (!grid_barrier(w.bar, a.c.err)) return;
    }
}
#endif

// B starts at B0, per formula.
HD void k_bound_init(const LcveArgs& a, u32 f) { a.bound[2 * f + 1] = a.bound[2 * f]; }

// B = min(B0, first member whose lists reach the temperatures).
HD void k_mis_bound(const LcveArgs& a, u32 v) {
    if (v == 0) return;
    const u32 w = a.word[v];
    if (mis_rank(w) != MIS_NO_RANK && mis_dec(w) == MIS_IN && lcve_big(a, v)) atom_min(&a.bound[2 * fid_of(a.c, v) + 1], a.rank[v]);
}

// Election flags over rank positions below B (compacted by the caller in rank order).
HD void k_elect_flag(const LcveArgs& a, u32* flags, u32 p) {
    const u32 v = a.order[p];
    const u32 w = a.word[v];
    flags[p] = (p < a.bound[2 * fid_of(a.c, v) + 1] && mis_rank(w) != MIS_NO_RANK && mis_dec(w) == MIS_IN) ? 1u : 0u;
}

HD void k_elect_write(const LcveArgs& a, const u32* flags, const u32* scan, u32 p) {
    if (!flags[p]) return;
    const u32 v = a.order[p];
    a.pvs[scan[p]] = v;
    a.c.pvrank[v] = scan[p];
    if (a.f_npvs) atom_add(&a.f_npvs[fid_of(a.c, v)], 1u);
}

}  // namespace sigma
