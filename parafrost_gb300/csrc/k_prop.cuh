// In-round unit propagation: ParaFROST::prop (src/cpu/elimination.cpp:41-99;
// GPU reference elimbcp.cu:103-192, which runs it on the host).
//
// The reference walks the trail in order; for each assigned literal t it strips
// -t from the clauses of ot[-t] (deleting those satisfied by a literal already
// true), enqueues the units this creates, then empties ot[-t] and deletes every
// clause of ot[t]. Here the pending literals of one wave are processed together:
//   wave A (per pending literal t): delete ot[t], collect ot[-t] into a worklist;
//   wave B (per collected clause): delete it if any literal is true, else remove
//          every false literal; an empty clause is a conflict, a unit is claimed
//          with a compare-and-swap on its variable and appended to the trail.
// Waves repeat until no new unit appears. The final state is the propagation
// fixpoint the reference reaches: the same clauses deleted, the same live-clause
// contents and signatures, the same set of assigned literals, the same emptied
// lists, and a conflict exactly when the reference finds one. Only the order of
// the trail and the literal contents of clauses that end up deleted can differ.
#pragma once

#include "cnf.cuh"

namespace sigma {

struct PropArgs {
    Ctx c;
    u32 head;        // first pending trail index of this wave
    u32 stamp;       // wave stamp (never reused within a context)
    u32* cl_stamp;   // per clause: last wave that collected it
    u32* work;       // collected clause ids
    u32* nwork;      // device counter
    u32 cap_work;
};

// Loads of data that earlier waves of the same launch may have written (the
// persistent wave kernel): read at L2, past this SM's L1.
template <bool Fresh, class T>
HD T ldw(const T* p) {
#if defined(__CUDA_ARCH__)
    if (Fresh) return __ldcg(p);
#endif
    return *p;
}
template <bool Fresh>
HD Hdr ldw_hdr(const Hdr* p) {
#if defined(__CUDA_ARCH__)
    if (Fresh) {
        const uint4 v = __ldcg(reinterpret_cast<const uint4*>(p));
        Hdr h;
        h.start = v.x;
        h.size = v.y;
        h.sig = v.z;
        h.flags = v.w;
        return h;
    }
#endif
    return *p;
}

// Wave A: one item per pending literal.
template <bool Fresh>
HD void prop_lists(const PropArgs& a, u32 k) {
    const Ctx& c = a.c;
    const u32 t = ldw<Fresh>(&c.trail[a.head + k]);
    const u32 f = FLIP(t);
    // collect ot[-t]
    const u32 fo = c.ot_off[f], fs = ldw<Fresh>(&c.ot_size[f]);
    for (u32 i = 0; i < fs; i++) {
        const u32 r = c.ot_refs[fo + i];
        const bool take = !h_deleted(ldw<Fresh>(&c.hdr[r].flags)) && atom_exch(&a.cl_stamp[r], a.stamp) != a.stamp;
        const u32 pos = warp_append(a.nwork, take);  // one reservation per group of lanes
        if (!take) continue;
        if (pos < a.cap_work) a.work[pos] = r;
        else set_err(c, ERR_CAP_SCRATCH);
    }
    // toblivion(ot[t])
    const u32 to = c.ot_off[t], ts = ldw<Fresh>(&c.ot_size[t]);
    for (u32 i = 0; i < ts; i++) {
        const u32 r = c.ot_refs[to + i];
        c.hdr[r].flags = (ldw<Fresh>(&c.hdr[r].flags) & ~3u) | ST_DELETED;
        touch(c, r);
    }
    c.ot_size[t] = 0;
    c.ot_size[f] = 0;
}

// Wave B: one item per collected clause.
constexpr u32 PROP_SHORT = 4;
template <bool Fresh>
HD void prop_clause(const PropArgs& a, u32 k) {
    const Ctx& c = a.c;
    const u32 r = ldw<Fresh>(&a.work[k]);
    Hdr h = ldw_hdr<Fresh>(&c.hdr[r]);
    if (h_deleted(h.flags)) return;
    u32* l = c.lits + h.start;
    const u32 v0 = ABS(ldw<Fresh>(&l[0]));  // names the formula if the clause empties
    u32 n = 0, sig = 0;
    if (h.size <= PROP_SHORT) {
        // short clause: all literals and their values loaded together
        u32 L[PROP_SHORT];
        int val[PROP_SHORT];
#pragma unroll
        for (u32 j = 0; j < PROP_SHORT; j++) L[j] = j < h.size ? ldw<Fresh>(&l[j]) : 0u;
#pragma unroll
        for (u32 j = 0; j < PROP_SHORT; j++) val[j] = j < h.size ? lit_value(c, L[j]) : 0;
        bool sat = false;
#pragma unroll
        for (u32 j = 0; j < PROP_SHORT; j++) sat |= val[j] == 1;
        if (sat) {
            c.hdr[r].flags = (h.flags & ~3u) | ST_DELETED;
            touch(c, r);
            return;
        }
#pragma unroll
        for (u32 j = 0; j < PROP_SHORT; j++) {
            if (j < h.size && val[j] != 0) {
                l[n++] = L[j];
                sig |= MAPHASH(L[j]);
            }
        }
    } else {
        // satisfied?
        for (u32 i = 0; i < h.size; i++) {
            if (lit_value(c, ldw<Fresh>(&l[i])) == 1) {
                c.hdr[r].flags = (h.flags & ~3u) | ST_DELETED;
                touch(c, r);
                return;
            }
        }
        for (u32 i = 0; i < h.size; i++) {
            const u32 lit = ldw<Fresh>(&l[i]);
            if (lit_value(c, lit) == 0) continue;
            l[n++] = lit;
            sig |= MAPHASH(lit);
        }
    }
    h.size = n;
    h.sig = sig;
    c.hdr[r] = h;
    touch(c, r);
    if (n == 0) {
        set_unsat(c, v0);
        // in a batch the other formulas go on: keep no empty live clause around
        if (c.var_fid) {
            c.hdr[r].flags = (h.flags & ~3u) | ST_DELETED;
            touch(c, r);
        }
        return;
    }
    if (n == 1) claim_unit(c, l[0]);
}

HD void k_prop_lists(const PropArgs& a, u32 k) { prop_lists<false>(a, k); }

#if SIGMA_CUDA
// A warp's run of reserved work-list slots [at, end) (the same in every lane). The
// collected clauses go to the run; a run that cannot take a step's clauses is
// closed (its free slots hold NONE, which the clause pass skips) and a new run of
// PROP_SLOTS is reserved, so the list's counter takes one atomic per run rather
// than one per step of every warp.
constexpr u32 PROP_SLOTS = 256;
struct WarpSlots {
    u32 at = 0, end = 0;
};
DEV void slots_close(const PropArgs& a, WarpSlots& ws) {
    for (u32 i = ws.at + (threadIdx.x & 31u); i < ws.end; i += 32)
        if (i < a.cap_work) a.work[i] = NONE;
    ws.at = ws.end = 0;
}
DEV u32 slots_append(const PropArgs& a, WarpSlots& ws, bool pred) {
    const u32 lane = threadIdx.x & 31u;
    const u32 m = __ballot_sync(0xffffffffu, pred);
    if (!m) return 0;
    const u32 cnt = (u32)__popc(m);
    if (ws.at + cnt > ws.end) {
        slots_close(a, ws);
        u32 nb = 0;
        if (lane == 0) nb = atomicAdd(a.nwork, PROP_SLOTS);
        nb = __shfl_sync(0xffffffffu, nb, 0);
        ws.at = nb;
        ws.end = nb + PROP_SLOTS;
    }
    const u32 pos = ws.at + (u32)__popc(m & ((1u << lane) - 1u));
    ws.at += cnt;
    return pos;
}

// Wave A by warps over one pending literal's two lists seen as one range: entries
// [0, fs) collect ot[-t], entries [fs, fs + ts) delete the clauses of ot[t]. A warp
// takes entries [s0, s1) of pending literal k, lanes on consecutive entries. The
// lists are emptied by the wave's clause pass, once every part has been walked.
DEV void prop_lists_part(const PropArgs& a, WarpSlots& ws, u32 k, u32 s0, u32 s1) {
    const Ctx& c = a.c;
    const u32 lane = threadIdx.x & 31u;
    const u32 t = __ldcg(&c.trail[a.head + k]);
    const u32 f = FLIP(t);
    const u32 fo = c.ot_off[f], fs = __ldcg(&c.ot_size[f]);
    const u32 to = c.ot_off[t];
    const u32 e = s1 < fs ? s1 : fs;
    for (u32 i0 = s0; i0 < e; i0 += 32) {
        const u32 i = i0 + lane;
        const u32 r = i < e ? c.ot_refs[fo + i] : 0u;
        const bool take = i < e && !h_deleted(__ldcg(&c.hdr[r].flags)) && atomicExch(&a.cl_stamp[r], a.stamp) != a.stamp;
        const u32 pos = slots_append(a, ws, take);
        if (!take) continue;
        if (pos < a.cap_work) a.work[pos] = r;
        else set_err(c, ERR_CAP_SCRATCH);
    }
    for (u32 i = (s0 > fs ? s0 : fs) + lane; i < s1; i += 32) {
        const u32 r = c.ot_refs[to + (i - fs)];
        c.hdr[r].flags = (__ldcg(&c.hdr[r].flags) & ~3u) | ST_DELETED;
        touch(c, r);
    }
}
// Pending literal k by one warp: its first PROP_PART entries here, the rest as parts
// of PROP_PART entries on the part list, walked by all warps after the wave's
// first barrier (one long list is then never one warp's critical path).
constexpr u32 PROP_PART = 2048;
DEV void prop_lists_warp(const PropArgs& a, WarpSlots& ws, u32 k, u64* parts, u32* nparts, u32 cap_parts) {
    const Ctx& c = a.c;
    const u32 lane = threadIdx.x & 31u;
    const u32 t = __ldcg(&c.trail[a.head + k]);
    const u32 n = __ldcg(&c.ot_size[FLIP(t)]) + __ldcg(&c.ot_size[t]);
    for (u32 s0 = PROP_PART * (lane + 1u); s0 < n; s0 += 32u * PROP_PART) {
        const u32 q = atomicAdd(nparts, 1u);
        if (q < cap_parts) parts[q] = (u64)k << 32 | s0;
        else set_err(c, ERR_CAP_SCRATCH);
    }
    prop_lists_part(a, ws, k, 0, n < PROP_PART ? n : PROP_PART);
}
#endif
HD void k_prop_clause(const PropArgs& a, u32 k) { prop_clause<false>(a, k); }

// Sweep wave: when the pending literals' lists cover a large part of the store (a
// propagation cascade), every clause of the store is checked against the current
// assignment instead, in store order (streaming reads, no list walk, no collection):
// a clause with a true literal is deleted, one with false literals loses them (a
// unit is claimed, an empty clause is a conflict); a clause without an assigned
// literal is left alone. Literals assigned during the sweep are pending for the next
// wave, so the fixpoint is the one the list waves reach.
template <bool Fresh>
HD void prop_sweep_clause(const PropArgs& a, u32 r) {
    const Ctx& c = a.c;
    Hdr h = ldw_hdr<Fresh>(&c.hdr[r]);
    if (h_deleted(h.flags)) return;
    u32* l = c.lits + h.start;
    u32 nfalse = 0;
    for (u32 i = 0; i < h.size; i++) {
        const int v = lit_value(c, ldw<Fresh>(&l[i]));
        if (v == 1) {
            c.hdr[r].flags = (h.flags & ~3u) | ST_DELETED;
            touch(c, r);
            return;
        }
        nfalse += v == 0;
    }
    if (!nfalse) return;
    const u32 v0 = ABS(ldw<Fresh>(&l[0]));
    u32 n = 0, sig = 0;
    for (u32 i = 0; i < h.size; i++) {
        const u32 lit = ldw<Fresh>(&l[i]);
        if (lit_value(c, lit) == 0) continue;
        l[n++] = lit;
        sig |= MAPHASH(lit);
    }
    h.size = n;
    h.sig = sig;
    c.hdr[r] = h;
    touch(c, r);
    if (n == 0) {
        set_unsat(c, v0);
        if (c.var_fid) {
            c.hdr[r].flags = (h.flags & ~3u) | ST_DELETED;
            touch(c, r);
        }
        return;
    }
    if (n == 1) claim_unit(c, l[0]);
}
HD void k_prop_sweep(const PropArgs& a, u32 r) { prop_sweep_clause<false>(a, r); }
// The lists of a swept wave's literals end empty, as the list waves leave them.
HD void k_prop_sweep_lists(const PropArgs& a, u32 k) {
    const u32 t = a.c.trail[a.head + k];
    a.c.ot_size[t] = 0;
    a.c.ot_size[FLIP(t)] = 0;
}
// Sweep rather than walk: the pending literals' lists (estimated from the mean list
// length) exceed a fraction of the store; scale = mean list length x the divisor of
// that fraction (0: never sweep).
HD bool prop_use_sweep(u32 pending, u32 scale, u32 ncls) { return scale && (u64)pending * scale > (u64)ncls; }

#if SIGMA_CUDA
// prop_clause (Always) or prop_sweep_clause (not Always) for up to 32 clauses by one
// warp: lane i loads the header of clause r (has: lane i holds one); the live
// clauses' literals are then read and valued by consecutive lanes, 32 literals of the
// warp's clauses per step, and each literal's value is read once. Every literal that
// is not false moves down to its place among its clause's kept literals (it is
// written only when its place changes, so a clause without false literals is not
// written), its signature bit goes to the clause's word in shared memory, and lane i
// learns from the step's ballots whether its clause has a true literal and how many
// false ones. A clause with a true literal is deleted (its literal contents do not
// matter then); otherwise, when it had false literals (or always, for Always), its
// header takes the kept size and signature, as the per-thread versions leave it.
// sm: 3 words per thread of the block (signature, unit, first variable of a clause).
template <bool Always>
DEV void prop_warp_clauses(const PropArgs& a, u32* sm, u32 r, bool has) {
    const Ctx& c = a.c;
    const u32 lane = threadIdx.x & 31u, wb = threadIdx.x & ~31u;
    u32* s_sig = sm;
    u32* s_unit = sm + blockDim.x;
    u32* s_v0 = sm + 2 * blockDim.x;
    Hdr h;
    h.start = h.size = h.sig = h.flags = 0;
    if (has) h = ldw_hdr<true>(&c.hdr[r]);
    const bool live = has && !h_deleted(h.flags);
    const u32 sz = live ? h.size : 0u;
    u32 incl = sz;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const u32 t = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)lane >= o) incl += t;
    }
    const u32 excl = incl - sz;
    const u32 total = __shfl_sync(0xffffffffu, incl, 31);
    s_sig[wb + lane] = 0;
    __syncwarp();
    bool sat = false;
    u32 nfalse = 0, kept = 0;
    for (u32 base = 0; base < total; base += 32) {
        const u32 j = base + lane;
        u32 k = 0;  // the lane whose clause holds literal j: the first with incl > j
#pragma unroll
        for (u32 step = 16; step; step >>= 1) {
            const u32 v = __shfl_sync(0xffffffffu, incl, k + step - 1);
            if (v <= j) k += step;
        }
        k &= 31u;
        const u32 st = __shfl_sync(0xffffffffu, h.start, k), ex = __shfl_sync(0xffffffffu, excl, k);
        const u32 kc = __shfl_sync(0xffffffffu, kept, k);  // the clause's literals kept in earlier steps
        const bool in = j < total;
        const u32 lit = in ? ldw<true>(&c.lits[st + (j - ex)]) : 0u;
        const int val = in ? lit_value(c, lit) : VAL_UNDEF;
        const bool keep = in && val != 0;
        const u32 bt = __ballot_sync(0xffffffffu, in && val == 1), bf = __ballot_sync(0xffffffffu, in && val == 0);
        const u32 bk = __ballot_sync(0xffffffffu, keep);
        if (in) {
            const u32 pos = j - ex;  // place in the clause
            if (pos == 0) s_v0[wb + k] = ABS(lit);
            if (keep) {
                // the clause's lanes of this step start at lane max(ex - base, 0)
                const u32 lo = ex > base ? ex - base : 0u;
                const u32 below = bk & ((1u << lane) - 1u) & ~((1u << lo) - 1u);
                const u32 p = kc + (u32)__popc(below);
                if (p != pos) c.lits[st + p] = lit;
                if (p == 0) s_unit[wb + k] = lit;
                atomicOr(&s_sig[wb + k], MAPHASH(lit));
            }
        }
        // this lane's literals in the step: [excl - base, incl - base) clipped to the warp
        const int lo = max((int)excl - (int)base, 0), hi = min((int)incl - (int)base, 32);
        if (lo < hi) {
            const u32 m = (hi - lo == 32 ? 0xffffffffu : ((1u << (hi - lo)) - 1u)) << lo;
            sat |= (bt & m) != 0;
            nfalse += (u32)__popc(bf & m);
            kept += (u32)__popc(bk & m);
        }
    }
    __syncwarp();
    if (!live) return;
    if (sat) {
        c.hdr[r].flags = (h.flags & ~3u) | ST_DELETED;
        touch(c, r);
        return;
    }
    if (!Always && !nfalse) return;
    const u32 n = kept;
    h.size = n;
    h.sig = s_sig[wb + lane];
    c.hdr[r] = h;
    touch(c, r);
    if (n == 0) {
        set_unsat(c, s_v0[wb + lane]);  // names the formula the clause emptied in
        if (c.var_fid) {
            c.hdr[r].flags = (h.flags & ~3u) | ST_DELETED;
            touch(c, r);
        }
        return;
    }
    if (n == 1) claim_unit(c, s_unit[wb + lane]);
}

// Every wave of one propagation in one cooperative launch: wave A over the trail
// literals [head, tail), a grid barrier, wave B over the collected clauses, a
// barrier, then the literals wave B appended. Wave w uses work counter w & 1 and
// clears the other one (last read in wave w-1, before its closing barrier).
struct PropWaves {
    u32* nwork2;     // two work counters
    u32* bar;        // grid barrier words
    u32* waves;      // out: waves run
    u32 max_waves;
    u32 sweep_scale; // mean occurrences per literal x sweep divisor (0: never sweep)
    u32* trace;      // optional: per wave [pending, collected | sweep << 31, start, clause pass start (ns / 1024)]
    u32 trace_cap;   // waves the trace holds
    u32* tail;       // the trail length every block uses for the wave (set before the
                     // launch and by the barrier that ends each wave)
    u64* parts;      // list parts past a pending literal's first PROP_PART entries:
    u32* nparts2;    // pending index << 32 | first entry; two counters (wave & 1)
    u32 cap_parts;
};

__global__ void __launch_bounds__(256, 4) prop_waves_k(PropArgs a, PropWaves w) {
    __shared__ u32 sm[3 * 256];
    const u32 tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    u32 head = a.head;
    for (u32 wave = 0;; wave++) {
        // a sweep claims units while slower blocks may still be starting the wave, so
        // the wave's end of the trail is the copy the last barrier took
        const u32 tail = vload(w.tail);
        if (tail == head) {
            if (tid == 0) *w.waves = wave;
            return;
        }
        if (wave >= w.max_waves) {
            if (tid == 0) atomicOr(a.c.err, ERR_ITER);
            return;
        }
        PropArgs b = a;
        b.head = head;
        b.stamp = a.stamp + wave;
        b.nwork = &w.nwork2[wave & 1];
        if (tid == 0) {
            w.nwork2[(wave + 1) & 1] = 0;
            w.nparts2[(wave + 1) & 1] = 0;
        }
        const bool sweep = prop_use_sweep(tail - head, w.sweep_scale, a.c.ncls);
        if (tid == 0 && w.trace && wave < w.trace_cap) {
            w.trace[4 * wave] = tail - head;
            w.trace[4 * wave + 1] = sweep ? 1u << 31 : 0u;
            w.trace[4 * wave + 2] = (u32)(global_ns() >> 10);
            w.trace[4 * wave + 3] = 0;
        }
        const u32 warp = tid >> 5, nwarps = nth >> 5;
        if (sweep) {
            for (u32 g = warp; g < (a.c.ncls + 31u) / 32u; g += nwarps) {
                const u32 r = g * 32u + (tid & 31u);
                prop_warp_clauses<false>(b, sm, r, r < a.c.ncls);
            }
            for (u32 i = tid; i < tail - head; i += nth) k_prop_sweep_lists(b, i);
            if (!grid_barrier(w.bar, a.c.err, a.c.ntrail, w.tail)) return;
            head = tail;
            continue;
        }
        u32* nparts = &w.nparts2[wave & 1];
        WarpSlots ws;
        for (u32 i = warp; i < tail - head; i += nwarps) prop_lists_warp(b, ws, i, w.parts, nparts, w.cap_parts);
        slots_close(b, ws);
        if (!grid_barrier(w.bar, a.c.err)) return;
        const u32 np = vload(nparts);
        if (np) {
            const u32 npc = np < w.cap_parts ? np : w.cap_parts;
            for (u32 i = warp; i < npc; i += nwarps) {
                const u64 q = __ldcg(&w.parts[i]);
                const u32 k = (u32)(q >> 32), s0 = (u32)q;
                const u32 t = __ldcg(&a.c.trail[head + k]);
                const u32 n = __ldcg(&a.c.ot_size[FLIP(t)]) + __ldcg(&a.c.ot_size[t]);
                prop_lists_part(b, ws, k, s0, n - s0 < PROP_PART ? n : s0 + PROP_PART);
            }
            slots_close(b, ws);
            if (!grid_barrier(w.bar, a.c.err)) return;
        }
        const u32 n = vload(b.nwork);
        const u32 nw = n < a.cap_work ? n : a.cap_work;
        if (tid == 0 && w.trace && wave < w.trace_cap) {
            w.trace[4 * wave + 1] = n;
            w.trace[4 * wave + 3] = (u32)(global_ns() >> 10);
        }
        for (u32 g = warp; g < (nw + 31u) / 32u; g += nwarps) {
            const u32 k = g * 32u + (tid & 31u);
            const u32 r = k < nw ? __ldcg(&b.work[k]) : NONE;  // NONE: a free slot of a closed run
            prop_warp_clauses<true>(b, sm, r, r != NONE);
        }
        for (u32 i = tid; i < tail - head; i += nth) k_prop_sweep_lists(b, i);
        if (!grid_barrier(w.bar, a.c.err, a.c.ntrail, w.tail)) return;
        head = tail;
    }
}
#endif

// reduceOT (src/cpu/simplify.cpp:58-79), run after propagation when SUB is off:
// drop deleted clauses from every list.
HD void k_reduce_list(const Ctx& c, u32 l) {
    const u32 o = c.ot_off[l], s = c.ot_size[l];
    u32 j = 0;
    for (u32 i = 0; i < s; i++) {
        const u32 r = c.ot_refs[o + i];
        if (!h_deleted(c.hdr[r].flags)) c.ot_refs[o + j++] = r;
    }
    c.ot_size[l] = j;
}

}  // namespace sigma
