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
// lower-ranked neighbour is in), decided by frontier waves over the graph.
#pragma once

#include "cnf.cuh"

namespace sigma {

// Independent-set word of a variable (one 64-bit word, so a neighbour test and its
// update touch one sector): bits 0-31 the variable's rank if it is a vertex of the
// graph (NONE otherwise, which never changes while the set is decided), bits 32-61
// the count of lower-neighbour occurrences not yet out, bits 62-63 the decision.
enum : u32 { MIS_UNDECIDED = 0, MIS_IN = 1, MIS_OUT = 2 };
constexpr u64 MIS_CNT_ONE = 1ull << 32;
constexpr u32 MIS_CNT_MAX = (1u << 30) - 1u;
HD u32 mis_rank(u64 w) { return (u32)w; }
HD u32 mis_cnt(u64 w) { return (u32)(w >> 32) & MIS_CNT_MAX; }
HD u32 mis_dec(u64 w) { return (u32)(w >> 62); }
HD u64 mis_dec_bits(u32 d) { return (u64)d << 62; }

struct LcveArgs {
    Ctx c;
    u32 pt, nt;           // mu_pos << mu_inc, mu_neg << mu_inc
    u32* score;           // nvars+1
    u32* order;           // nvars: variables in (score, var) order
    u32* rank;            // nvars+1
    u64* word;            // nvars+1: independent-set words
    const Q4* crec;       // per clause: its first three literals and size | deleted << 31
    u64* ws_bytes;        // accumulates the graph's working set (4*occ + sum(8 + 4*len))
    u32* bound;           // per formula f: [2f] = B0 (first valid non-F rank), [2f+1] = B
    const u32* f_active;  // batches: formulas taking part in this election (null: all)
    u32* f_npvs;          // batches: elected variables per formula
    u32* pvs;             // elected variables in rank order
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

// The independent set is decided by pushing decisions along edges to higher ranks:
// every graph vertex counts the occurrences of lower-ranked graph neighbours in its
// live clauses; a vertex with none is in. A vertex that goes in sends every higher
// neighbour out; a vertex that goes out decrements its higher neighbours' counts, and
// a count reaching zero means every lower neighbour is out, so that vertex goes in.
// Each wave processes only the vertices decided in the previous one. A neighbour
// shared through several clauses is counted and decremented once per clause.
// Vertices with more than MIS_WARP_MIN_OCC clauses are handled by a whole warp.
constexpr u32 MIS_WARP_MIN_OCC = 32;

struct MisFront {
    u32* small;   // next frontier, small adjacency
    u32* nsmall;
    u32* big;     // next frontier, large adjacency
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

// Graph membership, and the list of large graph vertices for the warp count.
HD void k_mis_init(const LcveArgs& a, const MisFront& bigs, u32 v) {
    const u32 f = v ? fid_of(a.c, v) : 0u;
    const bool in_graph = v && (!a.f_active || a.f_active[f]) && lcve_valid(a.c, v) && lcve_freezable(a, v) &&
                          a.rank[v] < a.bound[2 * f];
    a.word[v] = in_graph ? a.rank[v] : NONE;
    const bool big = in_graph && mis_is_big(a.c, v);
    const u32 pb = warp_append(bigs.nbig, big);
    if (big) bigs.big[pb] = v;
}

// The clause walks read literals four at a time, so the loads (and the pushes'
// atomics) of a chunk are in flight together. Clauses and lists are not written
// while the independent set is decided.
constexpr u32 MIS_CHUNK = 4;

// A clause as the election reads it: one 16-byte record holding its first three
// literals and its size and deleted bit (built once per election by k_mis_rec), so
// clauses of up to three literals cost one load; longer ones read the rest of
// their literals from the store.
HD void k_mis_rec(const Ctx& c, Q4* rec, u32 i) {
    const Hdr h = c.hdr[i];
    const u32* l = c.lits + h.start;
    Q4 q;
    q.x = h.size > 0 ? l[0] : 0u;
    q.y = h.size > 1 ? l[1] : 0u;
    q.z = h.size > 2 ? l[2] : 0u;
    q.w = h.size | (h_deleted(h.flags) ? 0x80000000u : 0u);
    rec[i] = q;
}
struct MisCl {
    Q4 q;
    u32 r;
    HD bool deleted() const { return (q.w >> 31) != 0; }
    HD u32 size() const { return q.w & 0x7FFFFFFFu; }
};
HD MisCl mis_cl(const LcveArgs& a, u32 r) {
    MisCl cl;
    cl.q = ldro4(&a.crec[r]);
    cl.r = r;
    return cl;
}
// Literal k of the clause; L is the clause's literal array (read only for k >= 3).
HD u32 mis_lit(const MisCl& cl, const u32* L, u32 k) {
    return k == 0 ? cl.q.x : k == 1 ? cl.q.y : k == 2 ? cl.q.z : ldro(L + k);
}
HD const u32* mis_long_lits(const LcveArgs& a, const MisCl& cl) {
    return cl.size() > 3 ? a.c.lits + hdr_ro(&a.c.hdr[cl.r]).start : nullptr;
}

// Occurrences of graph vertices ranked below rv (other than v) in clause r, and
// the clause's bytes (8 + 4*len when live) added to ws.
HD u32 mis_lower_in_hdr(const LcveArgs& a, u32 v, u32 rv, const MisCl& cl, u64& ws) {
    if (cl.deleted()) return 0;
    const u32 size = cl.size();
    ws += 8ull + 4ull * size;
    const u32* L = mis_long_lits(a, cl);
    u32 n = 0;
    for (u32 k0 = 0; k0 < size; k0 += MIS_CHUNK) {
        u32 w[MIS_CHUNK];
#pragma unroll
        for (u32 j = 0; j < MIS_CHUNK; j++) w[j] = k0 + j < size ? ABS(mis_lit(cl, L, k0 + j)) : v;
#pragma unroll
        for (u32 j = 0; j < MIS_CHUNK; j++) n += (w[j] != v && mis_rank(a.word[w[j]]) < rv) ? 1u : 0u;
    }
    return n;
}
HD u32 mis_lower_in_clause(const LcveArgs& a, u32 v, u32 rv, u32 r, u64& ws) {
    return mis_lower_in_hdr(a, v, rv, mis_cl(a, r), ws);
}

// Stores the lower-neighbour count of graph vertex v; a vertex with none goes in
// and is returned true (the caller puts it on the first frontier).
HD bool mis_set_count(const LcveArgs& a, u32 v, u32 rv, u32 n) {
    if (n > MIS_CNT_MAX) {  // cannot be held: stop the election with an error
        atom_or(a.c.err, ERR_CAP_SCRATCH);
        n = MIS_CNT_MAX;
    }
    a.word[v] = (u64)rv | ((u64)n << 32) | (n ? 0ull : mis_dec_bits(MIS_IN));
    return n == 0;
}

// The next clause's header is loaded before the current clause's literals are
// examined, so two clause walks overlap.
HD bool mis_count_one(const LcveArgs& a, u32 v, u64& ws) {
    const u32 rv = mis_rank(a.word[v]);
    const u32 p = V2L(v), np = a.c.ot_size[p], n_all = np + a.c.ot_size[p + 1];
    const u32 op = a.c.ot_off[p], on = a.c.ot_off[p + 1] - np;
    ws += 4ull * n_all;
    u32 n = 0;
    if (n_all) {
        MisCl h = mis_cl(a, ldro(&a.c.ot_refs[op]));
        for (u32 t = 0; t < n_all; t++) {
            MisCl hn = h;
            if (t + 1 < n_all) hn = mis_cl(a, ldro(&a.c.ot_refs[t + 1 < np ? op + t + 1 : on + t + 1]));
            n += mis_lower_in_hdr(a, v, rv, h, ws);
            h = hn;
        }
    }
    return mis_set_count(a, v, rv, n);
}

// Count for the small graph vertices (the large ones go through the warp kernel).
HD void k_mis_count(const LcveArgs& a, const MisFront& f, u32 v) {
    u64 ws = 0;
    const bool in0 = v && mis_rank(a.word[v]) != NONE && !mis_is_big(a.c, v) && mis_count_one(a, v, ws);
    mis_append(f, a.c, v, in0);
    warp_sum_add64(a.ws_bytes, ws);
}

// Frontier vertex u (rank ru, in or out) pushes its decision to its higher
// neighbours in clause r; app(w) is called for each neighbour w this decides. An
// in vertex marks them out; an out vertex decrements their counts unconditionally
// (a decided neighbour's count no longer matters; a count cannot fall below the
// occurrences of a lower neighbour that is in, which never decrements), and the
// push that takes a count from one to zero marks that neighbour in: no other push
// can reach it any more.
template <class App>
HD void mis_push_clause(const LcveArgs& a, u32 u, u32 ru, bool in, const MisCl& cl, App app) {
    if (cl.deleted()) return;
    const u32 size = cl.size();
    const u32* L = mis_long_lits(a, cl);
    for (u32 k0 = 0; k0 < size; k0 += MIS_CHUNK) {
        u32 w[MIS_CHUNK];
        u64 old[MIS_CHUNK];
        bool up[MIS_CHUNK];
#pragma unroll
        for (u32 j = 0; j < MIS_CHUNK; j++) w[j] = k0 + j < size ? ABS(mis_lit(cl, L, k0 + j)) : u;
#pragma unroll
        for (u32 j = 0; j < MIS_CHUNK; j++) {
            const u32 g = w[j] != u ? mis_rank(a.word[w[j]]) : NONE;
            up[j] = g != NONE && g > ru;
        }
#pragma unroll
        for (u32 j = 0; j < MIS_CHUNK; j++)
            if (up[j]) old[j] = in ? atom_or64(&a.word[w[j]], mis_dec_bits(MIS_OUT)) : atom_add64(&a.word[w[j]], 0ull - MIS_CNT_ONE);
#pragma unroll
        for (u32 j = 0; j < MIS_CHUNK; j++) {
            if (!up[j] || mis_dec(old[j]) != MIS_UNDECIDED) continue;
            if (in) {
                app(w[j]);
            } else if (mis_cnt(old[j]) == 1u) {
                atom_or64(&a.word[w[j]], mis_dec_bits(MIS_IN));
                app(w[j]);
            }
        }
    }
}

// Frontier vertex u pushes through all its clauses. The next clause's header is
// loaded before the current clause's atomics, so two clause walks overlap.
template <class App>
HD void mis_push_vertex(const LcveArgs& a, u32 u, App app) {
    const u64 wu = vload64(&a.word[u]);
    const bool in = mis_dec(wu) == MIS_IN;
    const u32 ru = mis_rank(wu);
    const u32 p = V2L(u), np = a.c.ot_size[p], n = np + a.c.ot_size[p + 1];
    const u32 op = a.c.ot_off[p], on = a.c.ot_off[p + 1] - np;
    if (!n) return;
    MisCl h = mis_cl(a, ldro(&a.c.ot_refs[op]));
    for (u32 t = 0; t < n; t++) {
        MisCl hn = h;
        if (t + 1 < n) hn = mis_cl(a, ldro(&a.c.ot_refs[t + 1 < np ? op + t + 1 : on + t + 1]));
        mis_push_clause(a, u, ru, in, h, app);
        h = hn;
    }
}

#if !SIGMA_CUDA
HD void k_mis_count_big(const LcveArgs& a, const u32* in, const MisFront& f, u32 idx) {
    const u32 v = in[idx];
    u64 ws = 0;
    if (mis_count_one(a, v, ws)) f.big[atom_add(f.nbig, 1u)] = v;
    *a.ws_bytes += ws;
}
// One wave step of the serial build: frontier vertex in[idx] pushes, decided
// vertices go straight to the next lists.
HD void k_mis_push(const LcveArgs& a, const u32* in, const MisFront& f, u32 idx) {
    mis_push_vertex(a, in[idx], [&](u32 w) {
        if (mis_is_big(a.c, w)) f.big[atom_add(f.nbig, 1u)] = w;
        else f.small[atom_add(f.nsmall, 1u)] = w;
    });
}
#else
// Count for the small graph vertices with a warp per 32 consecutive variables: the
// clauses of the 32 are spread over the lanes (as in the waves), each lane adds its
// clauses' lower-neighbour occurrences to the owner's counter in shared memory.
__global__ void __launch_bounds__(256) mis_count_flat_k(LcveArgs a, MisFront f, u32 nvars) {
    __shared__ u32 acc[8][32];
    const u32 lane = threadIdx.x & 31u, wl = threadIdx.x >> 5;
    const u32 nwarps = (gridDim.x * blockDim.x) >> 5;
    for (u32 base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32u; base <= nvars; base += nwarps * 32u) {
        const u32 v = base + lane;
        const u64 wv = (v && v <= nvars) ? a.word[v] : (u64)NONE;
        const bool counted = mis_rank(wv) != NONE && !mis_is_big(a.c, v);
        const u32 p = V2L(v);
        const u32 np = counted ? a.c.ot_size[p] : 0u, cnt = counted ? np + a.c.ot_size[p + 1] : 0u;
        const u32 op = counted ? a.c.ot_off[p] : 0u, on = counted ? a.c.ot_off[p + 1] : 0u;
        u64 ws = 4ull * cnt;
        acc[wl][lane] = 0;
        u32 incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u32 t = __shfl_up_sync(0xffffffffu, incl, o);
            if ((int)lane >= o) incl += t;
        }
        const u32 start = incl - cnt;
        const u32 total = __shfl_sync(0xffffffffu, incl, 31);
        __syncwarp();
        for (u32 t0 = 0; t0 < total; t0 += 32u) {
            const u32 t = t0 + lane;
            u32 lo = 0;
#pragma unroll
            for (u32 step = 16; step; step >>= 1) {
                const u32 s_mid = __shfl_sync(0xffffffffu, start, (int)(lo + step));
                if (lo + step < 32u && s_mid <= t) lo += step;
            }
            const u32 ov = __shfl_sync(0xffffffffu, v, (int)lo);
            const u64 owv = __shfl_sync(0xffffffffu, wv, (int)lo);
            const u32 onp = __shfl_sync(0xffffffffu, np, (int)lo);
            const u32 oop = __shfl_sync(0xffffffffu, op, (int)lo);
            const u32 oon = __shfl_sync(0xffffffffu, on, (int)lo);
            const u32 ost = __shfl_sync(0xffffffffu, start, (int)lo);
            if (t < total) {
                const u32 k = t - ost;
                const u32 r = ldro(&a.c.ot_refs[k < onp ? oop + k : oon + (k - onp)]);
                const u32 nl = mis_lower_in_hdr(a, ov, mis_rank(owv), mis_cl(a, r), ws);
                if (nl) atomicAdd(&acc[wl][lo], nl);
            }
        }
        __syncwarp();
        const bool in0 = counted && mis_set_count(a, v, mis_rank(wv), acc[wl][lane]);
        mis_append(f, a.c, v, in0);
        warp_sum_add64(a.ws_bytes, ws);
        __syncwarp();
    }
}

// Count for the large graph vertices, one warp each (lanes take its clauses). The
// list length is read from device memory (no host round trip).
__global__ void mis_count_warp_k(LcveArgs a, const u32* in, const u32* n_ptr, MisFront f) {
    const u32 lane = threadIdx.x & 31u, nw = (gridDim.x * blockDim.x) >> 5;
    const u32 n = *n_ptr;
    for (u32 idx = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; idx < n; idx += nw) {
        const u32 v = in[idx];
        const u32 rv = mis_rank(a.word[v]);
        const u32 p = V2L(v), np = a.c.ot_size[p], nn = a.c.ot_size[p + 1];
        const u32 op = a.c.ot_off[p], on = a.c.ot_off[p + 1];
        u32 cnt = 0;
        u64 ws = 0;
        for (u32 t = lane; t < np + nn; t += 32)
            cnt += mis_lower_in_clause(a, v, rv, ldro(&a.c.ot_refs[t < np ? op + t : on + (t - np)]), ws);
        cnt = __reduce_add_sync(0xffffffffu, cnt);
        for (int o = 16; o; o >>= 1) ws += __shfl_xor_sync(0xffffffffu, ws, o);
        if (lane == 0) {
            atomicAdd((unsigned long long*)a.ws_bytes, (unsigned long long)(ws + 4ull * (np + nn)));
            if (mis_set_count(a, v, rv, cnt)) f.big[atomicAdd(f.nbig, 1u)] = v;
        }
        __syncwarp();
    }
}

// All frontier waves in one cooperative launch. Wave k reads the lists small[k&1],
// big[k&1] with lengths in counter pair k%3 and appends to the other lists through
// pair (k+1)%3; pair (k+2)%3, last read in wave k-1, is cleared for wave k+1. A
// grid barrier separates the waves.
struct MisWaves {
    u32* small[2];
    u32* big[2];
    u32* ctr;        // three (small, big) length pairs; pair 0 holds the first frontier
    u32* bar;        // grid barrier: [0] arrivals, [1] generation
    u32* waves;      // out: number of waves run
    u32 max_waves;
};

// Vertices decided in a wave are staged per block in shared memory and copied to
// the next lists with one reservation per block (a vertex that finds its block's
// queue full goes to the list directly).
constexpr u32 MIS_QCAP = 2048;

struct MisBlockQueue {
    u32 small[MIS_QCAP], big[MIS_QCAP];
    u32 ns, nb, base_s, base_b;
};

DEV void mis_queue_push(MisBlockQueue& q, const MisFront& f, const Ctx& c, u32 w) {
    if (mis_is_big(c, w)) {
        const u32 k = atomicAdd(&q.nb, 1u);
        if (k < MIS_QCAP) q.big[k] = w;
        else f.big[atomicAdd(f.nbig, 1u)] = w;
    } else {
        const u32 k = atomicAdd(&q.ns, 1u);
        if (k < MIS_QCAP) q.small[k] = w;
        else f.small[atomicAdd(f.nsmall, 1u)] = w;
    }
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

__global__ void __launch_bounds__(256) mis_waves_k(LcveArgs a, MisWaves w) {
    __shared__ MisBlockQueue q;
    const u32 tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const u32 lane = threadIdx.x & 31u, nwarps = nth >> 5;
    if (threadIdx.x == 0) q.ns = q.nb = 0;
    __syncthreads();
    for (u32 wave = 0;; wave++) {
        const u32 cur = wave % 3, nxt = (wave + 1) % 3, old = (wave + 2) % 3;
        const u32 ns = vload(&w.ctr[2 * cur]), nb = vload(&w.ctr[2 * cur + 1]);
        if (!ns && !nb) {
            if (tid == 0) *w.waves = wave;
            return;
        }
        if (wave >= w.max_waves) {
            if (tid == 0) atomicOr(a.c.err, ERR_ITER);
            return;
        }
        if (tid == 0) {
            w.ctr[2 * old] = 0;
            w.ctr[2 * old + 1] = 0;
        }
        MisFront f;
        f.small = w.small[(wave + 1) & 1];
        f.nsmall = &w.ctr[2 * nxt];
        f.big = w.big[(wave + 1) & 1];
        f.nbig = &w.ctr[2 * nxt + 1];
        const auto app = [&](u32 v) { mis_queue_push(q, f, a.c, v); };
        // the lists were written in the previous wave by other blocks: read them uncached
        const u32* in_b = w.big[wave & 1];
        for (u32 idx = tid >> 5; idx < nb; idx += nwarps) {
            const u32 u = vload(&in_b[idx]);
            const u64 wu = vload64(&a.word[u]);
            const bool uin = mis_dec(wu) == MIS_IN;
            const u32 ru = mis_rank(wu);
            const u32 p = V2L(u), np = a.c.ot_size[p], nn = a.c.ot_size[p + 1];
            const u32 op = a.c.ot_off[p], on = a.c.ot_off[p + 1];
            for (u32 t = lane; t < np + nn; t += 32)
                mis_push_clause(a, u, ru, uin, mis_cl(a, ldro(&a.c.ot_refs[t < np ? op + t : on + (t - np)])), app);
            __syncwarp();
        }
        // small vertices: a warp takes 32 of them and spreads all their clauses over
        // its lanes (a prefix of the clause counts maps each lane's clause to its
        // vertex), so every lane walks about as many clauses as the others
        const u32* in_s = w.small[wave & 1];
        for (u32 base = (tid >> 5) * 32u; base < ns; base += nwarps * 32u) {
            const u32 idx = base + lane;
            const u32 u = idx < ns ? vload(&in_s[idx]) : 0u;
            const u64 wu = u ? vload64(&a.word[u]) : 0ull;
            const u32 p = V2L(u);
            const u32 np = u ? a.c.ot_size[p] : 0u, cnt = u ? np + a.c.ot_size[p + 1] : 0u;
            const u32 op = u ? a.c.ot_off[p] : 0u, on = u ? a.c.ot_off[p + 1] : 0u;
            u32 incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const u32 t = __shfl_up_sync(0xffffffffu, incl, o);
                if ((int)lane >= o) incl += t;
            }
            const u32 start = incl - cnt;
            const u32 total = __shfl_sync(0xffffffffu, incl, 31);
            for (u32 t0 = 0; t0 < total; t0 += 32u) {
                const u32 t = t0 + lane;
                // owner: the last lane whose start is <= t
                u32 lo = 0;
#pragma unroll
                for (u32 step = 16; step; step >>= 1) {
                    const u32 s_mid = __shfl_sync(0xffffffffu, start, (int)(lo + step));
                    if (lo + step < 32u && s_mid <= t) lo += step;
                }
                const u32 ou = __shfl_sync(0xffffffffu, u, (int)lo);
                const u64 owu = __shfl_sync(0xffffffffu, wu, (int)lo);
                const u32 onp = __shfl_sync(0xffffffffu, np, (int)lo);
                const u32 oop = __shfl_sync(0xffffffffu, op, (int)lo);
                const u32 oon = __shfl_sync(0xffffffffu, on, (int)lo);
                const u32 ost = __shfl_sync(0xffffffffu, start, (int)lo);
                if (t < total) {
                    const u32 k = t - ost;
                    const u32 r = ldro(&a.c.ot_refs[k < onp ? oop + k : oon + (k - onp)]);
                    mis_push_clause(a, ou, mis_rank(owu), mis_dec(owu) == MIS_IN, mis_cl(a, r), app);
                }
                __syncwarp();
            }
        }
        mis_queue_flush(q, f);
        if (!grid_barrier(w.bar, a.c.err)) return;
    }
}
#endif

// B starts at B0, per formula.
HD void k_bound_init(const LcveArgs& a, u32 f) { a.bound[2 * f + 1] = a.bound[2 * f]; }

// B = min(B0, first member whose lists reach the temperatures).
HD void k_mis_bound(const LcveArgs& a, u32 v) {
    if (v == 0) return;
    const u64 w = a.word[v];
    if (mis_rank(w) != NONE && mis_dec(w) == MIS_IN && lcve_big(a, v)) atom_min(&a.bound[2 * fid_of(a.c, v) + 1], a.rank[v]);
}

// Election flags over rank positions below B (compacted by the caller in rank order).
HD void k_elect_flag(const LcveArgs& a, u32* flags, u32 p) {
    const u32 v = a.order[p];
    const u64 w = a.word[v];
    flags[p] = (p < a.bound[2 * fid_of(a.c, v) + 1] && mis_rank(w) != NONE && mis_dec(w) == MIS_IN) ? 1u : 0u;
}

HD void k_elect_write(const LcveArgs& a, const u32* flags, const u32* scan, u32 p) {
    if (!flags[p]) return;
    const u32 v = a.order[p];
    a.pvs[scan[p]] = v;
    a.c.pvrank[v] = scan[p];
    if (a.f_npvs) atom_add(&a.f_npvs[fid_of(a.c, v)], 1u);
}

}  // namespace sigma
