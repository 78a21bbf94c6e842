// Blocked-clause elimination (ParaFROST::BCE, src/cpu/elimination.cpp:131-167;
// GPU bce_k, kernels.cu:675-694, blocked.cuh) and eager redundancy elimination
// (ParaFROST::ERE, elimination.cpp:169-197, forward_equ/merge_ere in
// src/cpu/redundancy.h:25-142; GPU ere_k, kernels.cu:696-730, redundancy.cuh).
#pragma once

#include "cnf.cuh"
#include "k_bve.cuh"

namespace sigma {

// isTautology (src/cpu/simplify.h:119-137).
HD bool is_tautology(u32 x, const u32* a, u32 n1, const u32* b, u32 n2) {
    u32 i = 0, j = 0;
    while (i < n1 && j < n2) {
        const u32 l1 = a[i], l2 = b[j];
        const u32 v1 = ABS(l1), v2 = ABS(l2);
        if (v1 == x) i++;
        else if (v2 == x) j++;
        else if ((l1 ^ l2) == 1u) return true;
        else if (v1 < v2) i++;
        else if (v2 < v1) j++;
        else { i++; j++; }
    }
    return false;
}

struct BceArgs {
    Ctx c;
    const u32* pvs;
    u32 bce_max;
    u32* nwit;           // count step output
    const u64* wit_scan; // write step input
    u64 wit_base;
};

HD bool bce_blocked(const Ctx& c, u32 v, const Hdr& neg, const ListRef& poss) {
    for (u32 j = 0; j < poss.n; j++) {
        const Hdr pos = c.hdr[poss.ids[j]];
        if (h_original(pos.flags) && !is_tautology(v, c.lits + neg.start, neg.size, c.lits + pos.start, pos.size))
            return false;
    }
    return true;
}

// Count step (witness words of the negative clauses blocked on v), one warp per
// elected variable: the lanes take the negative clauses, each checking its own
// against the whole positive list. A variable eliminated by VE in this phase is
// skipped (PVs[i] == 0 in the reference).
HD void bce_count_warp(const BceArgs& a, u32 k) {
    const Ctx& c = a.c;
    const u32 v = a.pvs[k];
    const u32 p = V2L(v), n = NEG(p);
    const bool skip = c.vstate[v] || c.ot_size[p] > a.bce_max || c.ot_size[n] > a.bce_max;
    u32 w = 0;
    if (!skip) {
        const ListRef poss = list_of(c, p), negs = list_of(c, n);
        w = wsum(negs.n, [&](u32 i) {
            const Hdr neg = c.hdr[negs.ids[i]];
            return (h_original(neg.flags) && bce_blocked(c, v, neg, poss)) ? neg.size + 1 : 0u;
        });
    }
    wone([&] { a.nwit[k] = w; });
}

#if SIGMA_CUDA
// Warps take elected variables in work order (perm), a few at a time.
__global__ void __launch_bounds__(256) bce_count_warp_k(BceArgs a, const u32* perm, u32 npos, u32* next) {
    const u32 lane = threadIdx.x & 31u;
    u32 chunk = warp_chunk(npos);
    while (true) {
        u32 j0 = 0;
        if (lane == 0) j0 = atomicAdd(next, chunk);
        j0 = __shfl_sync(0xffffffffu, j0, 0);
        if (j0 >= npos) break;
        const u32 j1 = j0 + chunk < npos ? j0 + chunk : npos;
        for (u32 j = j0; j < j1; j++) bce_count_warp(a, perm[j]);
        chunk = warp_chunk(npos - j1);
    }
}
#endif

// Write step: save each blocked clause with witness -v, then delete it.
HD void k_bce_write(const BceArgs& a, u32 k) {
    const Ctx& c = a.c;
    const u32 v = a.pvs[k];
    if (c.vstate[v]) return;
    const u32 p = V2L(v), n = NEG(p);
    if (c.ot_size[p] > a.bce_max || c.ot_size[n] > a.bce_max) return;
    const ListRef poss = list_of(c, p), negs = list_of(c, n);
    u64 w = a.wit_base + a.wit_scan[k];
    for (u32 i = 0; i < negs.n; i++) {
        const u32 r = negs.ids[i];
        const Hdr neg = c.hdr[r];
        if (!h_original(neg.flags)) continue;
        if (bce_blocked(c, v, neg, poss)) {
            w = save_clause(c, w, c.lits + neg.start, neg.size, n);
            mark_deleted(c, r);
        }
    }
}

// ---------------------------------------------------------------- ERE
// merge_ere (redundancy.h:38-85).
HD bool merge_ere(u32 x, const u32* a, u32 n1, const u32* b, u32 n2, const u32* t, u32 n) {
    u32 i = 0, j = 0, it = 0;
    while (it < n && i < n1 && j < n2) {
        const u32 lit = t[it];
        if (ABS(lit) == x) return false;
        const u32 l1 = a[i], l2 = b[j];
        const u32 v1 = ABS(l1), v2 = ABS(l2);
        if (v1 == x) i++;
        else if (v2 == x) j++;
        else if (v1 < v2) { if (l1 != lit) return false; i++; it++; }
        else if (v2 < v1) { if (l2 != lit) return false; j++; it++; }
        else { if (l1 != lit) return false; i++; j++; it++; }
    }
    while (it < n && i < n1) {
        const u32 l1 = a[i];
        if (ABS(l1) != x && l1 != t[it++]) return false;
        i++;
    }
    while (it < n && j < n2) {
        const u32 l2 = b[j];
        if (ABS(l2) != x && l2 != t[it++]) return false;
        j++;
    }
    return true;
}

struct EreArgs {
    Ctx c;
    const u32* pvs;
    u32 npvs;
    u32 ere_max;
    int ere_clause_max;
    // parallel pass: (target, key) records and per-clause claims
    u64* claim;     // per clause: smallest key that picked it (all ones = none)
    u32* rec_target;
    u64* rec_key;
    u32* nrec;
    u32 cap_rec;
    // resolution of the records
    u32* losers;    // indices of records that lost their target
    u32* nlosers;
};

// The (pv rank, i, j) order of forward_equ calls in ERE(): one 64-bit key.
HD u64 ere_key(u32 k, u32 i, u32 j) { return ((u64)k << 32) | ((u64)i << 16) | (u64)j; }

// forward_equ (redundancy.h:87-142) up to the target search: the smallest clause
// id in ot[best] equal to the resolvent (NONE if none). With `live_only`, targets
// deleted so far are skipped through their status, exactly as the reference
// (its status test fails on deleted clauses); the parallel pass passes false and
// sees the statuses ERE started with.
HD u32 ere_find(const Ctx& c, u32 x, const Hdr& h1, const Hdr& h2, int maxsize) {
    const u32* a = c.lits + h1.start;
    const u32* b = c.lits + h2.start;
    const u32 n1 = h1.size, n2 = h2.size;
    int len = (int)(n1 + n2) - 2;
    u32 i = 0, j = 0, minsize = 0xFFFFFFFFu, msig = 0, best = 0;
    while (i < n1 && j < n2) {
        const u32 l1 = a[i], l2 = b[j];
        const u32 v1 = ABS(l1), v2 = ABS(l2);
        if (v1 == x) i++;
        else if (v2 == x) j++;
        else if ((l1 ^ l2) == 1u) return NONE;
        else if (v1 < v2) {
            i++;
            if (c.ot_size[l1] < minsize) { minsize = c.ot_size[l1]; best = l1; }
            msig |= MAPHASH(l1);
        } else if (v2 < v1) {
            j++;
            if (c.ot_size[l2] < minsize) { minsize = c.ot_size[l2]; best = l2; }
            msig |= MAPHASH(l2);
        } else {
            i++; j++; len--;
            if (c.ot_size[l1] < minsize) { minsize = c.ot_size[l1]; best = l1; }
            msig |= MAPHASH(l1);
        }
    }
    // The reference reads ot[0] with an unbounded count when no literal precedes the
    // end of the shorter antecedent (undefined behaviour); such pairs are skipped.
    if (minsize == 0xFFFFFFFFu) return NONE;
    if (!(len > 1 && (!maxsize || len <= maxsize))) return NONE;
    const u32 type = (h_learnt(h1.flags) || h_learnt(h2.flags)) ? ST_LEARNT : ST_ORIGINAL;
    const ListRef L = list_of(c, best);
    u32 found = NONE;
    for (u32 t = 0; t < L.n; t++) {
        const u32 r = L.ids[t];
        if (r >= found) continue;
        const Hdr h = c.hdr[r];
        if ((u32)len == h.size && (h_learnt(h.flags) || (h.flags & 3u) == type) && sig_sub(msig, h.sig) &&
            merge_ere(x, a, n1, b, n2, c.lits + h.start, h.size))
            found = r;
    }
    return found;
}

// Parallel pass: every resolvent finds its first target; targets are claimed by the
// smallest key.
HD void k_ere_pv(const EreArgs& a, u32 k) {
    const Ctx& c = a.c;
    const u32 v = a.pvs[k];
    u32 dx = V2L(v), fx = NEG(dx);
    if (c.ot_size[dx] > c.ot_size[fx]) swap_t(dx, fx);
    const ListRef me = list_of(c, dx), other = list_of(c, fx);
    if (me.n > a.ere_max || other.n > a.ere_max) return;
    for (u32 i = 0; i < me.n; i++) {
        const Hdr hi = c.hdr[me.ids[i]];
        if (h_deleted(hi.flags)) continue;
        for (u32 j = 0; j < other.n; j++) {
            const Hdr hj = c.hdr[other.ids[j]];
            if (h_deleted(hj.flags)) continue;
            const u32 t = ere_find(c, v, hi, hj, a.ere_clause_max);
            if (t == NONE) continue;
            const u64 key = ere_key(k, i, j);
            atom_min64(&a.claim[t], key);
            const u32 pos = atom_add(a.nrec, 1u);
            if (pos < a.cap_rec) { a.rec_target[pos] = t; a.rec_key[pos] = key; }
            else set_err(c, ERR_CAP_SCRATCH);
        }
    }
}

// The same pass with one item per (elected variable, i, j) pair, so a variable
// with long lists is spread over many threads. perm lists the variables' ranks,
// cnt/off are per position of perm (pair counts and their exclusive scan).
HD void k_ere_count(const EreArgs& a, const u32* perm, u64* cnt, u32 q) {
    const Ctx& c = a.c;
    const u32 v = a.pvs[perm[q]];
    const u32 p = V2L(v), n = NEG(p);
    const u32 sp = c.ot_size[p], sn = c.ot_size[n];
    cnt[q] = (sp > a.ere_max || sn > a.ere_max) ? 0ull : (u64)sp * sn;
}
HD void k_ere_pair(const EreArgs& a, const u32* perm, const u64* off, u32 npos, u32 item) {
    const Ctx& c = a.c;
    const u32 q = upper_segment(off, npos, (u64)item);
    const u32 k = perm[q];
    const u32 v = a.pvs[k];
    u32 dx = V2L(v), fx = NEG(dx);
    if (c.ot_size[dx] > c.ot_size[fx]) swap_t(dx, fx);
    const ListRef me = list_of(c, dx), other = list_of(c, fx);
    const u32 r = item - (u32)off[q];
    const u32 i = r / other.n, j = r - i * other.n;
    const Hdr hi = c.hdr[me.ids[i]];
    if (h_deleted(hi.flags)) return;
    const Hdr hj = c.hdr[other.ids[j]];
    if (h_deleted(hj.flags)) return;
    const u32 t = ere_find(c, v, hi, hj, a.ere_clause_max);
    if (t == NONE) return;
    const u64 key = ere_key(k, i, j);
    atom_min64(&a.claim[t], key);
    const u32 pos = atom_add(a.nrec, 1u);
    if (pos < a.cap_rec) { a.rec_target[pos] = t; a.rec_key[pos] = key; }
    else set_err(c, ERR_CAP_SCRATCH);
}

// Winners delete their target; losers (an earlier resolvent took the same clause)
// are collected for the ordered fix-up.
HD void k_ere_resolve(const EreArgs& a, u32 q) {
    const u32 t = a.rec_target[q];
    if (a.claim[t] == a.rec_key[q]) {
        proof_delete(a.c, t);
        mark_deleted(a.c, t);
    } else {
        const u32 pos = atom_add(a.nlosers, 1u);
        a.losers[pos] = q;
    }
}

// Ordered fix-up, one thread: losers in key order redo forward_equ on the current
// statuses (no clause is claimed twice: every earlier resolvent of the same
// literal set already holds its target).
HD void ere_fixup(const EreArgs& a, const u64* keys, u32 nkeys) {
    const Ctx& c = a.c;
    for (u32 q = 0; q < nkeys; q++) {
        const u64 key = keys[q];
        const u32 k = (u32)(key >> 32), i = (u32)((key >> 16) & 0xFFFFu), j = (u32)(key & 0xFFFFu);
        const u32 v = a.pvs[k];
        u32 dx = V2L(v), fx = NEG(dx);
        if (c.ot_size[dx] > c.ot_size[fx]) swap_t(dx, fx);
        const ListRef me = list_of(c, dx), other = list_of(c, fx);
        const u32 t = ere_find(c, v, c.hdr[me.ids[i]], c.hdr[other.ids[j]], a.ere_clause_max);
        if (t != NONE) {
            proof_delete(c, t);
            mark_deleted(c, t);
        }
    }
}

// Whole ERE in reference order on one thread (used when the formula has learnt
// clauses, where resolvent types make first-choice claims order dependent).
HD void ere_sequential(const EreArgs& a) {
    const Ctx& c = a.c;
    for (u32 k = 0; k < a.npvs; k++) {
        const u32 v = a.pvs[k];
        u32 dx = V2L(v), fx = NEG(dx);
        if (c.ot_size[dx] > c.ot_size[fx]) swap_t(dx, fx);
        const ListRef me = list_of(c, dx), other = list_of(c, fx);
        if (me.n > a.ere_max || other.n > a.ere_max) continue;
        for (u32 i = 0; i < me.n; i++) {
            if (h_deleted(c.hdr[me.ids[i]].flags)) continue;
            for (u32 j = 0; j < other.n; j++) {
                if (h_deleted(c.hdr[other.ids[j]].flags)) continue;
                const u32 t = ere_find(c, v, c.hdr[me.ids[i]], c.hdr[other.ids[j]], a.ere_clause_max);
                if (t != NONE) {
                    proof_delete(c, t);
                    mark_deleted(c, t);
                }
            }
        }
    }
}

}  // namespace sigma
