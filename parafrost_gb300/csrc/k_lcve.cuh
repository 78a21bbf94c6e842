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
// lists reach the temperatures. The independent set is decided in parallel
// rounds: a vertex joins when every lower-ranked neighbour is out, leaves when
// one lower-ranked neighbour is in (Blelloch-Fineman-Shun deterministic greedy MIS).
#pragma once

#include "cnf.cuh"

namespace sigma {

enum : uint8_t { MIS_NONE = 0, MIS_UNDECIDED = 1, MIS_IN = 2, MIS_OUT = 3 };

struct LcveArgs {
    Ctx c;
    u32 pt, nt;           // mu_pos << mu_inc, mu_neg << mu_inc
    u32* score;           // nvars+1
    u32* order;           // nvars: variables in (score, var) order
    u32* rank;            // nvars+1
    uint8_t* state;       // nvars+1
    u32* bound;           // [0] = B0 (first valid non-F rank), [1] = B
    u32* changed;         // round counter of undecided vertices
    u32* pvs;             // elected variables in rank order
};

// write_scores (histogram.h:32-41): eligible[v-1] = v, scores[v] = ps*ns (32-bit wrap).
HD void k_scores(const LcveArgs& a, u32 v) {
    if (v == 0) return;
    a.score[v] = a.c.ps[v] * a.c.ns[v];
    a.order[v - 1] = v;
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
    if (lcve_valid(a.c, v) && !lcve_freezable(a, v)) atom_min(&a.bound[0], p);
}

// Work lists of undecided vertices and, per vertex, where its last scan met the first
// undecided lower neighbour (side:1 | list index:23 | literal index:8). Everything
// before that point was out or irrelevant, and "out" is final, so the next round
// resumes there. Indices are capped, which only makes a scan start earlier.
struct MisList {
    u32* resume;
    u32* in;
    u32* out;
    u32* nout;
};

HD u32 mis_pos(u32 side, u32 i, u32 k) {
    if (i >= 0x7FFFFFu) return (side << 31) | (0x7FFFFFu << 8);  // restart that clause from its first literal
    return (side << 31) | (i << 8) | (k < 255u ? k : 255u);
}

// Vertices whose two lists hold more than this many clauses are scanned by a whole
// warp (one clause per lane) instead of one thread.
constexpr u32 MIS_WARP_MIN_OCC = 12;

HD void k_mis_init(const LcveArgs& a, const MisList& small, const MisList& big, u32 v) {
    if (v == 0) { a.state[0] = MIS_NONE; return; }
    const bool in_graph = lcve_valid(a.c, v) && lcve_freezable(a, v) && a.rank[v] < a.bound[0];
    a.state[v] = in_graph ? MIS_UNDECIDED : MIS_NONE;
    if (in_graph) small.resume[v] = 0;
    const bool is_big = in_graph && a.c.ot_size[V2L(v)] + a.c.ot_size[NEG(V2L(v))] > MIS_WARP_MIN_OCC;
    const u32 ps = warp_append(small.nout, in_graph && !is_big);
    const u32 pb = warp_append(big.nout, is_big);
    if (in_graph && !is_big) small.out[ps] = v;
    if (is_big) big.out[pb] = v;
}

// One round for an undecided vertex: scan its live clauses from the resume point.
HD void k_mis_round(const LcveArgs& a, const MisList& w, u32 idx) {
    const u32 v = w.in[idx];
    volatile uint8_t* st = (volatile uint8_t*)a.state;
    if (st[v] != MIS_UNDECIDED) return;
    const Ctx& c = a.c;
    const u32 rv = a.rank[v];
    const u32 pos = w.resume[v];
    const u32 side0 = pos >> 31, i0 = (pos >> 8) & 0x7FFFFFu, k0 = pos & 0xFFu;
    u32 first = NONE;
    for (u32 side = side0; side < 2; side++) {
        const u32 l = V2L(v) + side;
        const u32 o = c.ot_off[l], s = c.ot_size[l];
        for (u32 i = side == side0 ? i0 : 0u; i < s; i++) {
            const Hdr h = c.hdr[c.ot_refs[o + i]];
            if (h_deleted(h.flags)) continue;
            const u32* lits = c.lits + h.start;
            const u32 kstart = (side == side0 && i == i0) ? k0 : 0u;
            for (u32 k = kstart; k < h.size; k++) {
                const u32 u = ABS(lits[k]);
                if (u == v) continue;
                const uint8_t su = st[u];
                if (su == MIS_NONE || a.rank[u] > rv) continue;
                if (su == MIS_IN) { st[v] = MIS_OUT; return; }
                if (su == MIS_UNDECIDED && first == NONE) first = mis_pos(side, i, k);
            }
        }
    }
    if (first == NONE) {
        st[v] = MIS_IN;
    } else {
        w.resume[v] = first;
        w.out[warp_append(w.nout, true)] = v;
    }
}

#if SIGMA_CUDA
// The same round with one warp per vertex: lanes take consecutive clauses of the
// two lists (from the resume point, at clause granularity), ballots give "some lower
// neighbour is in" and the first clause holding an undecided lower neighbour.
__global__ void mis_round_warp_k(LcveArgs a, MisList w, u32 n) {
    const u32 lane = threadIdx.x & 31u;
    const u32 nwarps = (gridDim.x * blockDim.x) >> 5;
    volatile uint8_t* st = (volatile uint8_t*)a.state;
    const Ctx& c = a.c;
    for (u32 idx = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; idx < n; idx += nwarps) {
        const u32 v = w.in[idx];
        if (st[v] != MIS_UNDECIDED) continue;
        const u32 rv = a.rank[v];
        const u32 pos = w.resume[v];
        const u32 side0 = pos >> 31, i0 = (pos >> 8) & 0x7FFFFFu;
        const u32 np = c.ot_size[V2L(v)], nn = c.ot_size[NEG(V2L(v))];
        const u32 op = c.ot_off[V2L(v)], on = c.ot_off[NEG(V2L(v))];
        const u32 total = np + nn;
        const u32 t0 = side0 ? np + (i0 < nn ? i0 : nn) : (i0 < np ? i0 : np);
        u32 first = NONE;
        bool out = false;
        for (u32 base = t0; base < total; base += 32) {
            const u32 t = base + lane;
            bool has_in = false, has_und = false;
            if (t < total) {
                const Hdr h = c.hdr[c.ot_refs[t < np ? op + t : on + (t - np)]];
                if (!h_deleted(h.flags)) {
                    const u32* L = c.lits + h.start;
                    for (u32 k = 0; k < h.size; k++) {
                        const u32 u = ABS(L[k]);
                        if (u == v) continue;
                        const uint8_t su = st[u];
                        if (su == MIS_NONE || a.rank[u] > rv) continue;
                        if (su == MIS_IN) { has_in = true; break; }
                        if (su == MIS_UNDECIDED) has_und = true;
                    }
                }
            }
            if (__ballot_sync(0xffffffffu, has_in)) { out = true; break; }
            const u32 und = __ballot_sync(0xffffffffu, has_und);
            if (und && first == NONE) {
                const u32 tt = base + (u32)(__ffs(und) - 1);
                first = tt < np ? mis_pos(0, tt, 0) : mis_pos(1, tt - np, 0);
            }
        }
        if (lane == 0) {
            if (out) st[v] = MIS_OUT;
            else if (first == NONE) st[v] = MIS_IN;
            else {
                w.resume[v] = first;
                w.out[atomicAdd(w.nout, 1u)] = v;
            }
        }
        __syncwarp();
    }
}
#endif

// B = min(B0, first member whose lists reach the temperatures).
HD void k_mis_bound(const LcveArgs& a, u32 v) {
    if (v == 0) return;
    if (a.state[v] == MIS_IN && lcve_big(a, v)) atom_min(&a.bound[1], a.rank[v]);
}

// Election flags over rank positions below B (compacted by the caller in rank order).
HD void k_elect_flag(const LcveArgs& a, u32* flags, u32 p) {
    const u32 v = a.order[p];
    flags[p] = (p < a.bound[1] && a.state[v] == MIS_IN) ? 1u : 0u;
}

HD void k_elect_write(const LcveArgs& a, const u32* flags, const u32* scan, u32 p) {
    if (!flags[p]) return;
    const u32 v = a.order[p];
    a.pvs[scan[p]] = v;
    a.c.pvrank[v] = scan[p];
}

}  // namespace sigma
