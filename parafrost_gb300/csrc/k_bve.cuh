// Bounded variable elimination with gate substitution: ParaFROST::bve
// (src/cpu/bve.cpp:28-221) and the gate finders (src/cpu/and.h, equivalence.h,
// ifthenelse.h, xor.h), merge/count helpers (src/cpu/simplify.h:119-332).
// GPU reference: in_ve_k_1/ve_k_1 + 2x scan + ve_k_2 (src/gpu/kernels.cu:375-651).
//
// Three steps, as in the GPU reference: (1) per elected variable, decide how it
// goes (pure, equivalence, AND/OR, ITE, XOR, plain resolution, or kept) and count
// the resolvents with more than one literal, their literals and the witness words;
// (2) exclusive scans over the elected order give every variable its clause slots,
// literal range and witness range, so resolvents land in the reference's order
// (appended in elected order, bve.cpp:218); (3) per variable, write witness and
// resolvents, substitute equivalences, delete the antecedents, mark eliminated.
// Units go straight to the trail through a compare-and-swap on their variable.
//
// Elected variables share no clause, so molten flags and in-place edits stay
// private. The decision lives in k_bve_warp.cuh (warp form) and k_bve_analyze.cuh.
#pragma once

#include "cnf.cuh"
#include "introsort.cuh"
#include "k_bve_analyze.cuh"
#include "k_bve_warp.cuh"
#include "k_sub.cuh"

namespace sigma {

struct BveArgs {
    Ctx c;
    const u32* pvs;
    u32 npvs;
    int ve_clause_max;
    int ve_lbound;
    int xor_max_arity;
    // analysis results, one per elected variable
    uint8_t* type;
    u32* porgs;
    u32* norgs;
    u32* ncls;     // resolvents with more than one literal
    u32* nlits;    // their literals
    u32* nwit;     // witness words
    u32* def;      // equivalence definition literal
    // per-variable scratch (AND/OR fan-in list)
    const u64* scr_off;
    u32* scr;
    // write step: exclusive scans over ncls / nlits / nwit and the bases they add to
    const u32* cls_scan;
    const u64* lit_scan;
    const u64* wit_scan;
    u32 cls_base;
    u64 lit_base;
    u64 wit_base;
    // per variable: the stamp of its last KEEP decision (0: none) and the lists it
    // saw then (positive size | negative size << 8 | originals << 16, << 24);
    // null: every variable is decided
    u32* keep_at;
    u32* keep_shape;
};

struct ListRef {
    const u32* ids;
    u32 n;
};
HD ListRef list_of(const Ctx& c, u32 l) {
    ListRef r;
    r.ids = c.ot_refs + c.ot_off[l];
    r.n = c.ot_size[l];
    return r;
}

HD bool merge_into(u32 x, const u32* a, u32 n1, const u32* b, u32 n2, u32* out, u32& on) {
    u32 i = 0, j = 0;
    on = 0;
    while (i < n1 && j < n2) {
        const u32 l1 = a[i], l2 = b[j];
        const u32 v1 = ABS(l1), v2 = ABS(l2);
        if (v1 == x) i++;
        else if (v2 == x) j++;
        else if ((l1 ^ l2) == 1u) return false;
        else if (v1 < v2) { i++; out[on++] = l1; }
        else if (v2 < v1) { j++; out[on++] = l2; }
        else { i++; j++; out[on++] = l1; }
    }
    while (i < n1) { const u32 l = a[i++]; if (ABS(l) != x) out[on++] = l; }
    while (j < n2) { const u32 l = b[j++]; if (ABS(l) != x) out[on++] = l; }
    return true;
}

// Step 1 with one warp per elected variable (k_bve_warp.cuh); variables too large
// for the warp slot take the per-thread decision on lane 0.
// A variable decided KEEP whose two lists have the same sizes and whose clauses
// have not changed since (no clause stamped after that decision: every change of
// literals or status, deletion included, stamps the clause, and a clause that joins
// a list is new or changed) sees the same lists in the same order (lists are
// rebuilt and sorted from the same clauses in the same store order), and decides
// KEEP again: the decision depends on
// the lists' clauses and order alone (other literals' list sizes only pick between
// identical matches of a gate, which KEEP does not use). Its result is written
// without staging the lists.
HD bool bve_keep_again(const BveArgs& a, u32 k) {
    if (!a.keep_at) return false;
    const Ctx& c = a.c;
    const u32 v = a.pvs[k];
    const u32 at = a.keep_at[v];
    if (!at) return false;
    const u32 p = V2L(v), np = c.ot_size[p], nn = c.ot_size[p + 1];
    const u32 sh = a.keep_shape[v];
    if ((sh & 0xFFu) != np || ((sh >> 8) & 0xFFu) != nn) return false;
    const u32* lp = c.ot_refs + c.ot_off[p];
    const u32* ln = c.ot_refs + c.ot_off[p + 1];
    const u32 changed = wsum(np + nn, [&](u32 i) { return c.cstamp[i < np ? lp[i] : ln[i - np]] > at ? 1u : 0u; });
    if (changed) return false;
    if (lane_id() == 0) {
        a.type[k] = VE_KEEP;
        a.porgs[k] = (sh >> 16) & 0xFFu;
        a.norgs[k] = sh >> 24;
        a.def[k] = 0;
        a.ncls[k] = 0;
        a.nlits[k] = 0;
        a.nwit[k] = 0;
    }
    wsync();
    return true;
}

HD void bve_warp_one(const BveArgs& a, u32 k, u32* slot) {
    if (bve_keep_again(a, k)) return;
    VeOpts o;
    o.ve_clause_max = a.ve_clause_max;
    o.ve_lbound = a.ve_lbound;
    o.xor_max_arity = a.xor_max_arity;
    WarpPv w;
    w.bind(a.c, slot);
    VeResult r;
    const bool staged = wpv_stage(w, a.c, a.pvs[k]);
    if (staged) r = wpv_bve_decide(w, o);
    if (lane_id() == 0) {
        if (!staged) {
            GlobalPv g;
            g.init(a.c, a.pvs[k], a.scr + a.scr_off[k]);
            r = pv_bve_decide(g, o);
        }
        a.type[k] = r.type;
        a.porgs[k] = r.porgs;
        a.norgs[k] = r.norgs;
        a.def[k] = r.def;
        a.ncls[k] = r.ncls;
        a.nlits[k] = r.nlits;
        a.nwit[k] = r.nwit;
        if (a.keep_at) {
            const u32 v = a.pvs[k];
            const bool keep = staged && r.type == VE_KEEP;
            a.keep_at[v] = keep ? a.c.stamp : 0u;
            if (keep) a.keep_shape[v] = w.np | (w.nn << 8) | (r.porgs << 16) | (r.norgs << 24);
        }
    }
    wsync();
}

#if SIGMA_CUDA
constexpr int kBveWarpThreads = 256;
__global__ void __launch_bounds__(kBveWarpThreads, 6) bve_warp_k(BveArgs a, const u32* perm, u32* next) {
    extern __shared__ u32 smem[];
    u32* slot = smem + (threadIdx.x >> 5) * WPV_WORDS;
    const u32 lane = threadIdx.x & 31u;
    u32 chunk = warp_chunk(a.npvs);
    while (true) {
        u32 j0 = 0;
        if (lane == 0) j0 = atomicAdd(next, chunk);
        j0 = __shfl_sync(0xffffffffu, j0, 0);
        if (j0 >= a.npvs) break;
        const u32 j1 = j0 + chunk < a.npvs ? j0 + chunk : a.npvs;
        for (u32 j = j0; j < j1; j++) bve_warp_one(a, perm[j], slot);
        chunk = warp_chunk(a.npvs - j1);
    }
}
#endif

// Emulation entry of the warp path: the slot is a local array, lanes run in turn.
HD void k_bve_warp(const BveArgs& a, u32 k) {
    u32 slot[WPV_WORDS];
    bve_warp_one(a, k, slot);
}

// ---------------------------------------------------------------- write step
// MODEL::saveClause (src/cpu/model.cpp:363-379) at w; returns the next position.
HD u64 save_clause(const Ctx& c, u64 w, const u32* l, u32 size, u32 witlit) {
    const u64 first = w;
    u32 pos = 0;
    for (u32 i = 0; i < size; i++) {
        c.resolved[w++] = l[i];
        if (l[i] == witlit) pos = i;
    }
    if (pos) { const u32 t = c.resolved[first + pos]; c.resolved[first + pos] = c.resolved[first]; c.resolved[first] = t; }
    c.resolved[w++] = size;
    if (c.res_mark) c.res_mark[w - 1] = 1;
    return w;
}
HD u64 save_witness(const Ctx& c, u64 w, u32 lit) {
    c.resolved[w++] = lit;
    c.resolved[w++] = 1;
    if (c.res_mark) c.res_mark[w - 1] = 1;
    return w;
}

HD void enqueue_unit(const Ctx& c, u32 u) { claim_unit(c, u); }

// toblivion(p, pOrgs, nOrgs, poss, negs, model) (simplify.h:305-332).
HD void oblivion_var(const Ctx& c, u32 p, u32 pOrgs, u32 nOrgs, u64 w) {
    const u32 n = NEG(p);
    const u32 save = pOrgs > nOrgs ? n : p;
    const u32 other = pOrgs > nOrgs ? p : n;
    const ListRef S = list_of(c, save);
    for (u32 i = 0; i < S.n; i++) {
        const u32 r = S.ids[i];
        const Hdr h = c.hdr[r];
        if (h_original(h.flags)) w = save_clause(c, w, c.lits + h.start, h.size, save);
        mark_deleted(c, r);
    }
    w = save_witness(c, w, pOrgs > nOrgs ? p : n);
    const ListRef O = list_of(c, other);
    for (u32 i = 0; i < O.n; i++) mark_deleted(c, O.ids[i]);
    c.ot_size[save] = 0;
    c.ot_size[other] = 0;
}

// substitute_single(dx, org, def) (equivalence.h:24-42): 0 or the unit left.
HD u32 substitute_clause(const Ctx& c, u32 r, u32 dx, u32 def) {
    Hdr h = c.hdr[r];
    u32* l = c.lits + h.start;
    u32 n = 0;
    for (u32 i = 0; i < h.size; i++) {
        const u32 lit = l[i];
        if (lit == dx) l[n++] = def;
        else if (lit != def) l[n++] = lit;
    }
    h.size = n;
    touch(c, r);
    if (n == 1) { c.hdr[r].size = 1; return l[0]; }
    reference_list_sort(l, (int)n, LitLess());
    h.sig = calc_sig(l, n);
    c.hdr[r].size = h.size;
    c.hdr[r].sig = h.sig;
    proof_line(c, l, n);
    return 0;
}

// substitute_single(p, def, ot) (equivalence.h:44-86).
HD void substitute_var(const Ctx& c, u32 p, u32 def) {
    const u32 n = NEG(p), def_f = FLIP(def);
    for (u32 side = 0; side < 2; side++) {
        const u32 l = side ? p : n;           // negatives first
        const u32 dx = l, d = side ? def : def_f;
        const u32 kill = side ? def_f : def;  // has(def) on negatives, has(def_f) on positives
        const ListRef L = list_of(c, l);
        for (u32 i = 0; i < L.n; i++) {
            const u32 r = L.ids[i];
            const Hdr h = c.hdr[r];
            if (h_learnt(h.flags) || h_molten(h.flags) || sorted_has(c.lits + h.start, h.size, kill)) {
                mark_deleted(c, r);
            } else if (h_original(h.flags)) {
                const u32 unit = substitute_clause(c, r, dx, d);
                if (unit) enqueue_unit(c, unit);
            }
        }
    }
}

// Step 3 for one elected variable.
HD void k_bve_write(const BveArgs& a, u32 k) {
    const Ctx& c = a.c;
    const uint8_t type = a.type[k];
    if (type == VE_KEEP) return;
    const u32 v = a.pvs[k];
    const u32 p = V2L(v), n = NEG(p);
    const u32 pOrgs = a.porgs[k], nOrgs = a.norgs[k];
    u64 w = a.wit_base + a.wit_scan[k];
    if (type == VE_EQU) {
        // save_BN_gate (equivalence.h:132-153), then substitute in place.
        const u32 save = pOrgs > nOrgs ? n : p;
        const ListRef S = list_of(c, save);
        for (u32 i = 0; i < S.n; i++) {
            const Hdr h = c.hdr[S.ids[i]];
            if (h_original(h.flags)) w = save_clause(c, w, c.lits + h.start, h.size, save);
        }
        save_witness(c, w, pOrgs > nOrgs ? p : n);
        substitute_var(c, p, a.def[k]);
    } else {
        if ((type == VE_RES || type == VE_SUBST) && a.ncls[k]) {
            // xresolve / xsubstitute (bve.cpp:144-186): "me" is the shorter list.
            u32 dx = p, fx = n;
            if (c.ot_size[dx] > c.ot_size[fx]) swap_t(dx, fx);
            const ListRef me = list_of(c, dx), other = list_of(c, fx);
            const bool gate = type == VE_SUBST;
            u32 id = a.cls_base + a.cls_scan[k];
            u64 ls = a.lit_base + a.lit_scan[k];
            const u32 id_end = id + a.ncls[k];
            const u64 ls_end = ls + a.nlits[k];
            for (u32 i = 0; i < me.n; i++) {
                const Hdr hi = c.hdr[me.ids[i]];
                if (!h_original(hi.flags)) continue;
                const bool mi = h_molten(hi.flags);
                for (u32 j = 0; j < other.n; j++) {
                    const Hdr hj = c.hdr[other.ids[j]];
                    if (!h_original(hj.flags)) continue;
                    if (gate && mi == h_molten(hj.flags)) continue;
                    const int rs = merge_size(v, c.lits + hi.start, hi.size, c.lits + hj.start, hj.size);
                    if (rs == 0) continue;
                    if (rs == 1) {
                        // unit resolvent (newResolvent, bve.cpp:200-211): one literal survives
                        u32 buf[1];
                        u32 on = 0;
                        merge_into(v, c.lits + hi.start, hi.size, c.lits + hj.start, hj.size, buf, on);
                        enqueue_unit(c, buf[0]);
                        continue;
                    }
                    if (id >= id_end || ls + (u64)rs > ls_end) { set_err(c, ERR_INTERNAL); return; }
                    u32 on = 0;
                    merge_into(v, c.lits + hi.start, hi.size, c.lits + hj.start, hj.size, c.lits + ls, on);
                    Hdr nh;
                    nh.start = (u32)ls;
                    nh.size = on;
                    nh.sig = calc_sig(c.lits + ls, on);
                    nh.flags = ST_ORIGINAL | F_ADDED;
                    c.hdr[id] = nh;
                    touch(c, id);
                    id++;
                    ls += on;
                }
            }
            if (id != id_end || ls != ls_end) { set_err(c, ERR_INTERNAL); return; }
        }
        oblivion_var(c, p, pOrgs, nOrgs, w);
    }
    c.vstate[v] = 1;  // markEliminated (src/cpu/solve.h:535-541)
}

#if SIGMA_CUDA
// oblivion_var over the lanes: the saved list's original clauses get their witness
// records at offsets from a warp prefix of their lengths (the sequential loop's
// order), every clause of both lists is deleted, and the variable's own witness
// closes the records.
__device__ void oblivion_var_warp(const Ctx& c, u32 p, u32 pOrgs, u32 nOrgs, u64 w) {
    const u32 lane = threadIdx.x & 31u;
    const u32 n = NEG(p);
    const u32 save = pOrgs > nOrgs ? n : p;
    const u32 other = pOrgs > nOrgs ? p : n;
    const ListRef S = list_of(c, save);
    for (u32 b0 = 0; b0 < S.n; b0 += 32u) {
        const u32 i = b0 + lane;
        u32 r = 0, words = 0;
        Hdr h;
        if (i < S.n) {
            r = S.ids[i];
            h = c.hdr[r];
            words = h_original(h.flags) ? h.size + 1u : 0u;
        }
        u64 incl = words;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u64 t = __shfl_up_sync(0xffffffffu, incl, o);
            if ((int)lane >= o) incl += t;
        }
        if (words) save_clause(c, w + incl - words, c.lits + h.start, h.size, save);
        if (i < S.n) mark_deleted(c, r);
        w += __shfl_sync(0xffffffffu, incl, 31);
    }
    const ListRef O = list_of(c, other);
    for (u32 i = lane; i < O.n; i += 32u) mark_deleted(c, O.ids[i]);
    __syncwarp();
    if (lane == 0) {
        save_witness(c, w, pOrgs > nOrgs ? p : n);
        c.ot_size[save] = 0;
        c.ot_size[other] = 0;
    }
}

// Step 2 with one warp per elected variable: the resolvent pairs, in the
// reference's (i, j) order, go over the lanes 32 at a time; a warp prefix of the
// kept ones gives each its id and literal offset, so the clauses land where the
// sequential loop puts them. Equivalences and the witness/deletion part run on
// lane 0 as in k_bve_write.
__device__ void bve_write_warp(const BveArgs& a, u32 k) {
    const Ctx& c = a.c;
    const u32 lane = threadIdx.x & 31u;
    const uint8_t type = a.type[k];
    if (type == VE_KEEP) return;
    if (type == VE_EQU || !a.ncls[k]) {
        if (lane == 0) k_bve_write(a, k);
        __syncwarp();
        return;
    }
    const u32 v = a.pvs[k];
    const u32 p = V2L(v), n = NEG(p);
    u32 dx = p, fx = n;
    if (c.ot_size[dx] > c.ot_size[fx]) swap_t(dx, fx);
    const ListRef me = list_of(c, dx), other = list_of(c, fx);
    const bool gate = type == VE_SUBST;
    u32 id = a.cls_base + a.cls_scan[k];
    u64 ls = a.lit_base + a.lit_scan[k];
    const u32 id_end = id + a.ncls[k];
    const u64 ls_end = ls + a.nlits[k];
    const u32 pairs = me.n * other.n;
    bool bad = false;
    for (u32 b0 = 0; b0 < pairs; b0 += 32u) {
        const u32 q = b0 + lane;
        int rs = 0;
        Hdr hi, hj;
        if (q < pairs) {
            hi = c.hdr[me.ids[q / other.n]];
            hj = c.hdr[other.ids[q % other.n]];
            if (h_original(hi.flags) && h_original(hj.flags) && !(gate && h_molten(hi.flags) == h_molten(hj.flags)))
                rs = merge_size(v, c.lits + hi.start, hi.size, c.lits + hj.start, hj.size);
        }
        if (rs == 1) {
            u32 buf[1];
            u32 on = 0;
            merge_into(v, c.lits + hi.start, hi.size, c.lits + hj.start, hj.size, buf, on);
            enqueue_unit(c, buf[0]);
        }
        const bool keep = rs >= 2;
        const u32 kept = __ballot_sync(0xffffffffu, keep);
        u64 lits = keep ? (u64)rs : 0ull;
        u64 incl = lits;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u64 t = __shfl_up_sync(0xffffffffu, incl, o);
            if ((int)lane >= o) incl += t;
        }
        const u32 my_id = id + (u32)__popc(kept & ((1u << lane) - 1u));
        const u64 my_ls = ls + incl - lits;
        if (keep) {
            if (my_id >= id_end || my_ls + lits > ls_end) {
                bad = true;
            } else {
                u32 on = 0;
                merge_into(v, c.lits + hi.start, hi.size, c.lits + hj.start, hj.size, c.lits + my_ls, on);
                Hdr nh;
                nh.start = (u32)my_ls;
                nh.size = on;
                nh.sig = calc_sig(c.lits + my_ls, on);
                nh.flags = ST_ORIGINAL | F_ADDED;
                c.hdr[my_id] = nh;
                touch(c, my_id);
            }
        }
        id += (u32)__popc(kept);
        ls += __shfl_sync(0xffffffffu, incl, 31);
    }
    bad = __any_sync(0xffffffffu, bad) || id != id_end || ls != ls_end;
    __syncwarp();
    if (bad) {
        if (lane == 0) set_err(c, ERR_INTERNAL);
        __syncwarp();
        return;
    }
    oblivion_var_warp(c, p, a.porgs[k], a.norgs[k], a.wit_base + a.wit_scan[k]);
    if (lane == 0) c.vstate[v] = 1;  // markEliminated (src/cpu/solve.h:535-541)
    __syncwarp();
}

__global__ void __launch_bounds__(256, 6) bve_write_warp_k(BveArgs a, const u32* perm, u32 npos, u32* next) {
    const u32 lane = threadIdx.x & 31u;
    u32 chunk = warp_chunk(npos);
    while (true) {
        u32 j0 = 0;
        if (lane == 0) j0 = atomicAdd(next, chunk);
        j0 = __shfl_sync(0xffffffffu, j0, 0);
        if (j0 >= npos) break;
        const u32 j1 = j0 + chunk < npos ? j0 + chunk : npos;
        for (u32 j = j0; j < j1; j++) bve_write_warp(a, perm[j]);
        chunk = warp_chunk(npos - j1);
    }
}
#endif

// Per-variable scratch words for the AND/OR fan-in list.
HD void k_bve_scratch_need(const Ctx& c, const u32* pvs, u64* need, u32 k) {
    const u32 p = V2L(pvs[k]);
    need[k] = (u64)c.ot_size[p] + c.ot_size[NEG(p)] + 2;
}

}  // namespace sigma
