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
                if (h_learnt(s.flags) && h_original(cand.flags)) {
                    c.hdr[sr].flags = (s.flags & ~3u) | ST_ORIGINAL;
                    touch(c, sr);
                }
                proof_delete(c, r);
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

#if SIGMA_CUDA
// Warps take elected variables in work order (perm), a few at a time.
__global__ void __launch_bounds__(256, 8) sub_warp_k(SubArgs a, const u32* perm, u32 n, u32* next) {
    const u32 lane = threadIdx.x & 31u;
    u32 chunk = warp_chunk(n);
    while (true) {
        u32 j0 = 0;
        if (lane == 0) j0 = atomicAdd(next, chunk);
        j0 = __shfl_sync(0xffffffffu, j0, 0);
        if (j0 >= n) break;
        const u32 j1 = j0 + chunk < n ? j0 + chunk : n;
        for (u32 j = j0; j < j1; j++) sub_warp_pv(a, perm[j]);
        chunk = warp_chunk(n - j1);
    }
}
#endif

}  // namespace sigma
