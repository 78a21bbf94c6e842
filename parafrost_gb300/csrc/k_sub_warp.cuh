// SUB with one warp per elected variable (self_sub_x, src/cpu/subsume.h:144-179).
//
// The candidate loop stays in list order: whether a candidate is strengthened or
// deleted depends on what happened to the earlier ones. The two searches inside
// one candidate step are split over the lanes: the self-subsumption search over
// the opposite list (subsume.h:123-142: first clause that strengthens the
// candidate, stopping at the first clause longer than it) and the subsumption
// search over the earlier candidates (subsume.h:105-121: first clause that
// subsumes it). Each takes the first hit in list order, so the outcome is the
// sequential one. Writes to the clauses happen on lane 0 between warp barriers.
#pragma once

#include "k_sub.cuh"

namespace sigma {

// Candidates of list lx against the opposite list lo (x: the candidates' literal of
// the elected variable, fx its negation).
HD void sub_warp_side(const SubArgs& a, u32 k, u32 p, u32 lx, u32 lo, SubLocal& L) {
    const Ctx& c = a.c;
    const u32* cands = c.ot_refs + c.ot_off[lx];
    const u32* opp = c.ot_refs + c.ot_off[lo];
    const u32 cs = c.ot_size[lx];
    for (u32 i = 0; i < cs; i++) {
        const u32 r = cands[i];
        const Hdr h = c.hdr[r];
        if (h.size > HSE_MAX_CL_SIZE) break;
        if (h_deleted(h.flags)) continue;
        // self-subsumption: first opposite clause that strengthens r, or the first
        // one longer than r (where the reference's scan stops)
        const u32 ls = c.ot_size[lo];
        const u32* cl = c.lits + h.start;
        const u32 js = wfirst(ls, [&](u32 j) {
            const Hdr s = c.hdr[opp[j]];
            if (s.size > h.size) return true;
            return !h_deleted(s.flags) && s.size > 1 && sig_selfsub(s.sig, h.sig) &&
                   clause_selfsub(lx, lo, c.lits + s.start, s.size, cl, h.size);
        });
        if (js != NONE_IDX && c.hdr[opp[js]].size <= h.size) {
            wone([&] {
                sub_strengthen(a, k, p, r, lx, L);
                set_molten(c, r, true);
            });
        }
        // subsumption by an earlier candidate
        const Hdr cand = c.hdr[r];
        const u32* cl2 = c.lits + cand.start;
        const u32 jb = wfirst(i, [&](u32 j) {
            const Hdr s = c.hdr[cands[j]];
            if (h_deleted(s.flags)) return false;
            if (h_molten(cand.flags) && s.size > cand.size) return false;
            return s.size > 1 && sig_sub(s.sig, cand.sig) && clause_sub(c.lits + s.start, s.size, cl2, cand.size);
        });
        if (jb != NONE_IDX) {
            wone([&] {
                const u32 sr = cands[jb];
                const Hdr s = c.hdr[sr];
                if (h_learnt(s.flags) && h_original(cand.flags)) c.hdr[sr].flags = (s.flags & ~3u) | ST_ORIGINAL;
                mark_deleted(c, r);
            });
        }
    }
    wone([&] { sub_update_list(c, lx); });
}

HD void sub_warp_pv(const SubArgs& a, u32 k) {
    if (a.run && !a.run[k]) return;
    const Ctx& c = a.c;
    const u32 v = a.pvs[k];
    const u32 p = V2L(v), n = NEG(p);
    if (c.ot_size[p] > a.sub_max || c.ot_size[n] > a.sub_max) return;
    SubLocal L;  // lane 0's (only lane 0 strengthens)
    L.n = 0;
    if (a.pre_off) {
        wone([&] {
            for (u32 i = a.pre_off[k]; i < a.pre_off[k + 1]; i++) sub_local_oblivion(c, p, a.pre_lits[i]);
        });
    }
    sub_warp_side(a, k, p, p, n, L);
    sub_warp_side(a, k, p, n, p, L);
}

// ---------------------------------------------------------------- staged lists
// The exact pass (no elected variable can derive a unit) with the variable's two
// lists staged in the warp's shared-memory slot: ids, sizes, signatures, flags and
// literals, loaded once by all lanes. The candidate loop then reads only the slot;
// every change (strengthened literals, size, signature, flags, list compaction) is
// made in the slot and written through to the store, so the slot and the store
// agree at every step and the outcome is the one above.
constexpr u32 SUBW_KC = 64;   // clauses (both lists)
constexpr u32 SUBW_KL = 384;  // literals
constexpr u32 SUBW_WORDS = 5 * SUBW_KC + SUBW_KL;

struct SubSlot {
    u32* id;
    u32* size;
    u32* sig;
    u32* flags;
    u32* start;  // offset of the clause's literals in lits
    u32* lits;
    HD void bind(u32* s) {
        id = s;
        size = id + SUBW_KC;
        sig = size + SUBW_KC;
        flags = sig + SUBW_KC;
        start = flags + SUBW_KC;
        lits = start + SUBW_KC;
    }
    HD u32* L(u32 i) const { return lits + start[i]; }
};

// Stage list p as entries [0, np) and list n as [np, np + nn); false when they do
// not fit the slot.
HD bool sub_stage(SubSlot& w, const Ctx& c, u32 p, u32 np, u32 nn) {
    const u32 tot = np + nn;
    if (tot > SUBW_KC) return false;
    const u32* lp = c.ot_refs + c.ot_off[p];
    const u32* ln = c.ot_refs + c.ot_off[p + 1];
#if defined(__CUDA_ARCH__)
    static_assert(SUBW_KC <= 64, "two clauses per lane");
    const u32 lane = threadIdx.x & 31u;
    u32 gstart[2] = {0, 0}, carry = 0;
#pragma unroll
    for (u32 rr = 0; rr < 2; rr++) {
        const u32 i = rr * 32u + lane;
        u32 sz = 0;
        if (i < tot) {
            const u32 r = i < np ? lp[i] : ln[i - np];
            const Hdr h = c.hdr[r];
            w.id[i] = r;
            w.size[i] = h.size;
            w.sig[i] = h.sig;
            w.flags[i] = h.flags;
            gstart[rr] = h.start;
            sz = h.size;
        }
        u32 incl = sz;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u32 t = __shfl_up_sync(kFull, incl, o);
            if ((int)lane >= o) incl += t;
        }
        if (i < tot) w.start[i] = carry + incl - sz;
        carry += __shfl_sync(kFull, incl, 31);
    }
    __syncwarp();
    if (carry > SUBW_KL) return false;
#pragma unroll
    for (u32 rr = 0; rr < 2; rr++) {
        const u32 i = rr * 32u + lane;
        if (i < tot) {
            const u32* src = c.lits + gstart[rr];
            u32* dst = w.lits + w.start[i];
            for (u32 k = 0; k < w.size[i]; k++) dst[k] = src[k];
        }
    }
    __syncwarp();
#else
    u32 total = 0;
    for (u32 i = 0; i < tot; i++) {
        const u32 r = i < np ? lp[i] : ln[i - np];
        const Hdr h = c.hdr[r];
        w.id[i] = r;
        w.size[i] = h.size;
        w.sig[i] = h.sig;
        w.flags[i] = h.flags;
        w.start[i] = total;
        total += h.size;
    }
    if (total > SUBW_KL) return false;
    for (u32 i = 0; i < tot; i++) {
        const u32* src = c.lits + c.hdr[w.id[i]].start;
        for (u32 k = 0; k < w.size[i]; k++) w.lits[w.start[i] + k] = src[k];
    }
#endif
    return true;
}

HD void sub_slot_flags(const Ctx& c, SubSlot& w, u32 i, u32 f) {
    w.flags[i] = f;
    c.hdr[w.id[i]].flags = f;
}

// ParaFROST::strengthen (elimination.cpp:199-234) of staged entry i, in the slot and
// the store, then molten (subsume.h:135). Only the exact pass runs staged, where no
// strengthening leaves one literal; the unit branch keeps the reference's error and
// conflict outcomes all the same.
HD void sub_slot_strengthen(const Ctx& c, SubSlot& w, u32 i, u32 me) {
    const u32 r = w.id[i];
    u32* gl = c.lits + c.hdr[r].start;
    u32* sl = w.L(i);
    const u32 size = w.size[i];
    u32 n = 0, sig = 0;
    for (u32 k = 0; k < size; k++) {
        const u32 lit = sl[k];
        if (lit != me) {
            sl[n] = lit;
            gl[n] = lit;
            n++;
            sig |= MAPHASH(lit);
        }
    }
    w.size[i] = size - 1;
    w.sig[i] = sig;
    c.hdr[r].sig = sig;
    c.hdr[r].size = size - 1;
    if (n == 1) {
        const int val = lit_value(c, sl[0]);
        if (val == VAL_UNDEF) set_err(c, ERR_CAP_SCRATCH);
        else if (val == 0) set_unsat(c, ABS(sl[0]));
    }
    sub_slot_flags(c, w, i, w.flags[i] | F_MOLTEN);
}

// sub_warp_side over staged entries: candidates [cb, cb + cn) with literal x against
// the opposite entries [ob, ob + on) (literal fx).
HD void sub_slot_side(const Ctx& c, SubSlot& w, u32 cb, u32 cn, u32 ob, u32 on, u32 x, u32 fx) {
    for (u32 t = 0; t < cn; t++) {
        const u32 i = cb + t;
        const u32 size = w.size[i];
        if (size > HSE_MAX_CL_SIZE) break;
        if (h_deleted(w.flags[i])) continue;
        const u32 sig = w.sig[i];
        const u32 js = wfirst(on, [&](u32 q) {
            const u32 j = ob + q;
            const u32 sj = w.size[j];
            if (sj > size) return true;
            return !h_deleted(w.flags[j]) && sj > 1 && sig_selfsub(w.sig[j], sig) &&
                   clause_selfsub(x, fx, w.L(j), sj, w.L(i), size);
        });
        if (js != NONE_IDX && w.size[ob + js] <= size) wone([&] { sub_slot_strengthen(c, w, i, x); });
        const u32 cs = w.size[i], cf = w.flags[i], csig = w.sig[i];
        const u32 jb = wfirst(t, [&](u32 q) {
            const u32 j = cb + q;
            if (h_deleted(w.flags[j])) return false;
            if (h_molten(cf) && w.size[j] > cs) return false;
            return w.size[j] > 1 && sig_sub(w.sig[j], csig) && clause_sub(w.L(j), w.size[j], w.L(i), cs);
        });
        if (jb != NONE_IDX) {
            wone([&] {
                const u32 j = cb + jb;
                if (h_learnt(w.flags[j]) && h_original(cf)) sub_slot_flags(c, w, j, (w.flags[j] & ~3u) | ST_ORIGINAL);
                sub_slot_flags(c, w, i, (w.flags[i] & ~3u) | ST_DELETED);
            });
        }
    }
}

// updateOL (subsume.h:27-37) of list l from its staged entries [b, b + n): molten
// entries are unmelted and dropped, deleted ones dropped; the kept entries move to
// the front of the range. Returns the new list size.
HD u32 sub_slot_update(const Ctx& c, SubSlot& w, u32 l, u32 b, u32 n) {
    u32 j = 0;
    wone([&] {
        const u32 o = c.ot_off[l];
        for (u32 q = 0; q < n; q++) {
            const u32 i = b + q, f = w.flags[i];
            if (h_molten(f)) {
                sub_slot_flags(c, w, i, f & ~F_MOLTEN);
            } else if (!h_deleted(f)) {
                const u32 d = b + j;
                c.ot_refs[o + j] = w.id[i];
                w.id[d] = w.id[i];
                w.size[d] = w.size[i];
                w.sig[d] = w.sig[i];
                w.flags[d] = f;
                w.start[d] = w.start[i];
                j++;
            }
        }
        c.ot_size[l] = j;
    });
    return wbcast(j, 0);
}

// self_sub_x with staged lists; lists that do not fit run sub_warp_pv.
HD void sub_slot_pv(const SubArgs& a, u32 k, u32* slot) {
    const Ctx& c = a.c;
    const u32 v = a.pvs[k];
    const u32 p = V2L(v), n = NEG(p);
    const u32 np = c.ot_size[p], nn = c.ot_size[n];
    if (np > a.sub_max || nn > a.sub_max) return;
    SubSlot w;
    w.bind(slot);
    if (!sub_stage(w, c, p, np, nn)) {
        sub_warp_pv(a, k);
        return;
    }
    sub_slot_side(c, w, 0, np, np, nn, p, n);
    const u32 np2 = sub_slot_update(c, w, p, 0, np);
    sub_slot_side(c, w, np, nn, 0, np2, n, p);
    sub_slot_update(c, w, n, np, nn);
}

// Emulation entry of the staged path: a local slot, lanes in turn.
HD void k_sub_slot(const SubArgs& a, u32 k) {
    u32 slot[SUBW_WORDS];
    sub_slot_pv(a, k, slot);
}

#if SIGMA_CUDA
constexpr u32 kSubWarpChunk = 4;

// Warps take elected variables in work order (perm), a few at a time. With
// `staged`, each warp's slot is SUBW_WORDS words of the dynamic shared memory.
__global__ void __launch_bounds__(256) sub_warp_k(SubArgs a, const u32* perm, u32 n, u32* next, int staged) {
    extern __shared__ u32 smem[];
    u32* slot = smem + (threadIdx.x >> 5) * SUBW_WORDS;
    const u32 lane = threadIdx.x & 31u;
    while (true) {
        u32 j0 = 0;
        if (lane == 0) j0 = atomicAdd(next, kSubWarpChunk);
        j0 = __shfl_sync(0xffffffffu, j0, 0);
        if (j0 >= n) break;
        const u32 j1 = j0 + kSubWarpChunk < n ? j0 + kSubWarpChunk : n;
        for (u32 j = j0; j < j1; j++) {
            if (staged) sub_slot_pv(a, perm[j], slot);
            else sub_warp_pv(a, perm[j]);
        }
    }
}
#endif

}  // namespace sigma
