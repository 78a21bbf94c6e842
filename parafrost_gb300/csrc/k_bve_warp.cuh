// BVE step 1 (ParaFROST::bve's decision, src/cpu/bve.cpp:37-142) with one warp per
// elected variable.
//
// The warp stages the variable's two lists in its shared-memory slot (ids, headers,
// literals; all lanes loading), then runs the reference's decision sequence with
// warp-uniform control flow: every list scan, every pair enumeration and every
// resolvent count is spread over the lanes and combined with ballots or reductions,
// taking the same first match / same counts the sequential code takes. Molten flags
// are written through to the clause store for the write step. Variables whose lists
// exceed the slot run the per-thread decision (k_bve_analyze.cuh) on lane 0.
#pragma once

#include "cnf.cuh"
#include "introsort.cuh"
#include "k_bve_analyze.cuh"

namespace sigma {

constexpr u32 WPV_KC = 64;   // clauses per variable (both lists)
constexpr u32 WPV_KL = 384;  // literals per variable
constexpr u32 WPV_XL = 24;   // XOR literal set (arity <= 20)
// words per warp slot
constexpr u32 WPV_HIST = 16;  // original clauses per size (< 16) per list, counted when staging
constexpr u32 WPV_WORDS = 5 * WPV_KC + WPV_KL + (WPV_KC + 2) + WPV_XL + 8 + 2 * WPV_HIST;

struct WarpPv {
    const Ctx* c;
    u32 v, np, nn;
    u32* id;
    u32* size;
    u32* sig;
    u32* flags;
    u32* start;
    u32* lits;
    u32* out;   // AND/OR fan-in list
    u32* xl;    // XOR literal set
    u32* ctl;   // [side]: original clauses, [2 + side]: their literals (counted when staging)
    u32* hist;  // [side * WPV_HIST + size]

    HD void bind(const Ctx& cc, u32* slot) {
        c = &cc;
        id = slot;
        size = id + WPV_KC;
        sig = size + WPV_KC;
        flags = sig + WPV_KC;
        start = flags + WPV_KC;
        lits = start + WPV_KC;
        out = lits + WPV_KL;
        xl = out + WPV_KC + 2;
        ctl = xl + WPV_XL;
        hist = ctl + 8;
    }
    // original clauses of `size` in one side's list (sizes >= WPV_HIST: the list length)
    HD u32 count_size(u32 side, u32 size) const { return size < WPV_HIST ? hist[side * WPV_HIST + size] : n(side); }
    HD u32 n(u32 side) const { return side ? nn : np; }
    HD u32 base(u32 side) const { return side ? np : 0u; }
    HD const u32* L(u32 i) const { return lits + start[i]; }
    // list size of a literal: the staged lists for the variable's own literals
    HD u32 lsize(u32 lit) const { return ABS(lit) == v ? n(lit & 1u) : c->ot_size[lit]; }
};

// Stage the lists; false when they exceed the slot.
HD bool wpv_stage(WarpPv& w, const Ctx& c, u32 var) {
    w.v = var;
    const u32 p = V2L(var);
    w.np = c.ot_size[p];
    w.nn = c.ot_size[p + 1];
    const u32 tot = w.np + w.nn;
    if (tot > WPV_KC) return false;
    const u32* lp = c.ot_refs + c.ot_off[p];
    const u32* ln = c.ot_refs + c.ot_off[p + 1];
    const u32 np = w.np;
    wfor(2 * WPV_HIST, [&](u32 i) { w.hist[i] = 0; });
#if defined(__CUDA_ARCH__)
    // lane l stages clauses l and l + 32 (tot <= 64): headers, the exclusive prefix
    // of the sizes by a warp scan, then the literals from the starts kept in registers
    static_assert(WPV_KC <= 64, "two clauses per lane");
    const u32 lane = threadIdx.x & 31u;
    u32 gstart[2] = {0, 0}, carry = 0, org[2] = {0, 0}, olit[2] = {0, 0};
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
            if (h_original(h.flags)) {
                if (h.size < WPV_HIST) atomicAdd(&w.hist[(i < np ? 0u : WPV_HIST) + h.size], 1u);
                org[i < np ? 0 : 1]++;
                olit[i < np ? 0 : 1] += h.size;
            }
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
    {
        const u32 o0 = __reduce_add_sync(kFull, org[0]), o1 = __reduce_add_sync(kFull, org[1]);
        const u32 l0 = __reduce_add_sync(kFull, olit[0]), l1 = __reduce_add_sync(kFull, olit[1]);
        if (lane == 0) {
            w.ctl[0] = o0;
            w.ctl[1] = o1;
            w.ctl[2] = l0;
            w.ctl[3] = l1;
        }
    }
    __syncwarp();
    if (carry > WPV_KL) return false;
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
    for (u32 k = 0; k < 4; k++) w.ctl[k] = 0;
    for (u32 i = 0; i < tot; i++) {
        const u32 r = i < np ? lp[i] : ln[i - np];
        const Hdr h = c.hdr[r];
        w.id[i] = r;
        w.size[i] = h.size;
        w.sig[i] = h.sig;
        w.flags[i] = h.flags;
        w.start[i] = total;
        total += h.size;
        if (h_original(h.flags)) {
            if (h.size < WPV_HIST) w.hist[(i < np ? 0u : WPV_HIST) + h.size]++;
            w.ctl[i < np ? 0 : 1]++;
            w.ctl[i < np ? 2 : 3] += h.size;
        }
    }
    if (total > WPV_KL) return false;
    for (u32 i = 0; i < tot; i++) {
        const u32* src = c.lits + c.hdr[w.id[i]].start;
        u32* dst = w.lits + w.start[i];
        for (u32 k = 0; k < w.size[i]; k++) dst[k] = src[k];
    }
#endif
    return true;
}

HD void wpv_set_molten(WarpPv& w, u32 i, bool m) {
    wone([&]() {
        const u32 f = w.flags[i];
        const u32 nf = m ? (f | F_MOLTEN) : (f & ~F_MOLTEN);
        w.flags[i] = nf;
        w.c->hdr[w.id[i]].flags = nf;
    });
}

// Unmelt the entries of [b, e) selected by pred (freezeBinaries / freezeArities).
template <class P>
HD void wpv_unmelt_if(WarpPv& w, u32 b, u32 e, P pred) {
    wfor(e - b, [&](u32 t) {
        const u32 i = b + t;
        const u32 f = w.flags[i];
        if (h_molten(f) && pred(i)) {
            w.flags[i] = f & ~F_MOLTEN;
            w.c->hdr[w.id[i]].flags = f & ~F_MOLTEN;
        }
    });
}

// Original clauses of a side and their literals (fixed while the variable is
// decided: only molten flags change).
HD u32 wpv_orgs(const WarpPv& w, u32 side) { return w.ctl[side]; }
HD u32 wpv_lits_before(const WarpPv& w, u32 side) { return w.ctl[2 + side]; }

// countResolvents / countSubstituted (simplify.h:237-295) over all pairs at once:
// the rejection test (count > clsbefore, any size above the limit, literal bound)
// does not depend on the enumeration order; nAdded is the full count (>= 1 when
// rejected, exact when accepted).
HD bool wpv_count_added(const WarpPv& w, const VeOpts& o, int clsbefore, u32 sme, int& nAdded, u32& nLits,
                        bool gate) {
    const u32 so = sme ^ 1u;
    const u32 bm = w.base(sme), nm = w.n(sme), bo = w.base(so), no = w.n(so);
    const u32 pairs = nm * no;
    const int rlimit = o.ve_clause_max;
    const u32 x = w.v;
    // one pass, packed per pair: resolvent (bit 0), over the size limit (bit 16),
    // its literals (bits 32..63)
    const u64 s = wsum64(pairs, [&](u32 t) -> u64 {
        const u32 i = bm + t / no, j = bo + t % no;
        const u32 fi = w.flags[i], fj = w.flags[j];
        if (!h_original(fi) || !h_original(fj)) return 0ull;
        if (gate && h_molten(fi) == h_molten(fj)) return 0ull;
        const int rs = merge_size(x, w.L(i), w.size[i], w.L(j), w.size[j]);
        if (rs <= 1) return 0ull;
        return 1ull | ((rlimit && rs > rlimit) ? (1ull << 16) : 0ull) | ((u64)rs << 32);
    });
    const u32 cnt = (u32)(s & 0xFFFFu), over = (u32)((s >> 16) & 0xFFFFu), lit = (u32)(s >> 32);
    nAdded = (int)cnt;
    nLits = lit;
    if ((int)cnt > clsbefore || over) return true;
    if (o.ve_lbound && lit > wpv_lits_before(w, 0) + wpv_lits_before(w, 1)) return true;
    return false;
}

// find_sfanin + find_BN_gate (equivalence.h:88-130). Lists enter with no molten
// clause; a failed search leaves none.
HD u32 wpv_find_bn_gate(WarpPv& w) {
    const u32 p = V2L(w.v), n = NEG(p);
    auto is_bin = [&](u32 i) { return h_original(w.flags[i]) && w.size[i] == 2; };
    const u32 nb = w.count_size(0, 2);  // original binaries of the positive list
    if (nb == 1) {
        const u32 bi = wfirst(w.np, [&](u32 i) { return is_bin(i); });
        const u32* l = w.L(bi);
        u32 first = FLIP(l[0] ^ l[1] ^ p);
        u32 second = n;
        const u32 def = first;
        if (second < first) { first = second; second = def; }
        const u32 nj = wfirst(w.nn, [&](u32 t) {
            const u32 i = w.np + t;
            return is_bin(i) && w.L(i)[0] == first && w.L(i)[1] == second;
        });
        if (nj != NONE_IDX) {
            wpv_set_molten(w, bi, true);
            wpv_set_molten(w, w.np + nj, true);
            return def;
        }
    }
    wpv_unmelt_if(w, 0, w.np, [&](u32 i) { return is_bin(i); });
    return 0;
}

// find_fanin + find_AO_gate (and.h:25-86).
HD bool wpv_find_ao_gate(WarpPv& w, const VeOpts& o, u32 dx, int nOrgCls, int& nAdded, u32& nLits) {
    const u32 side = dx & 1u, fside = side ^ 1u;
    const u32 b = w.base(side), ns = w.n(side);
    auto is_bin = [&](u32 i) { return h_original(w.flags[i]) && w.size[i] == 2; };
    // The fan-in is every original binary of the side; the gate needs at least two
    // and an original clause of one more literal on the other side. Without them the
    // search below melts the binaries and unmelts them again.
    const u32 nbin = w.count_size(side, 2);
    if (nbin < 2 || w.count_size(fside, nbin + 1) == 0) {
        wpv_unmelt_if(w, b, b + ns, [&](u32 i) { return is_bin(i); });
        return false;
    }
    // fan-in literals in list order, binaries melted
    u32 on = 0;
    for (u32 base = 0; base < ns; base += 32) {
        const u32 m = wballot([&](u32 l) { return base + l < ns && is_bin(b + base + l); });
        const u32 on0 = on;
        wfor(32, [&](u32 l) {
            if ((m >> l) & 1u) {
                const u32 i = b + base + l;
                const u32* L = w.L(i);
                w.out[on0 + (u32)popc32(m & ((1u << l) - 1u))] = FLIP(L[0] ^ L[1] ^ dx);
                const u32 nf = w.flags[i] | F_MOLTEN;
                w.flags[i] = nf;
                w.c->hdr[w.id[i]].flags = nf;
            }
        });
        on += (u32)popc32(m);
    }
    if (on > 1) {
        const u32 f_dx = FLIP(dx);
        wone([&]() {
            w.out[on] = f_dx;
            reference_list_sort(w.out, (int)(on + 1), LitLess());
        });
        on++;
        u32 sig = 0;
        for (u32 t = 0; t < on; t++) sig |= MAPHASH(w.out[t]);
        const u32 fb = w.base(fside);
        const u32 j = wfirst(w.n(fside), [&](u32 t) {
            const u32 i = fb + t;
            if (!(h_original(w.flags[i]) && w.size[i] == on && sig_sub(w.sig[i], sig))) return false;
            const u32* L = w.L(i);
            for (u32 k = 0; k < on; k++) if (L[k] != w.out[k]) return false;
            return true;
        });
        if (j != NONE_IDX) {
            wpv_set_molten(w, fb + j, true);
            nAdded = 0;
            if (!wpv_count_added(w, o, nOrgCls, side, nAdded, nLits, true)) return true;
            wpv_set_molten(w, fb + j, false);
        }
    }
    wpv_unmelt_if(w, b, b + ns, [&](u32 i) { return is_bin(i); });
    return false;
}

// fast_equality_check (ifthenelse.h:25-40) on the own list (see pv_fast_equality_check):
// the reference takes the first match in list order when the own literal's list is
// no longer than the others', else the match of smallest id. The two agree unless
// two or more clauses match, so the list sizes are only read then.
HD u32 wpv_feq_lane(const WarpPv& w, u32 x, u32 y, u32 z) {
    u32 q0 = x, q1 = y, q2 = z;
    { const u32 lo = q1 < q2 ? q1 : q2, hi = q1 < q2 ? q2 : q1; q1 = lo; q2 = hi; }
    { const u32 lo = q0 < q2 ? q0 : q2, hi = q0 < q2 ? q2 : q0; q0 = lo; q2 = hi; }
    { const u32 lo = q0 < q1 ? q0 : q1, hi = q0 < q1 ? q1 : q0; q0 = lo; q1 = hi; }
    const u32 side = x & 1u, b = w.base(side), e = b + w.n(side);
    u32 first = NONE, best = NONE, best_id = NONE;
    for (u32 i = b; i < e; i++) {
        const u32 f = w.flags[i];
        if (h_molten(f) || !(h_original(f) && w.size[i] == 3)) continue;
        const u32* L = w.L(i);
        if (L[0] == q0 && L[1] == q1 && L[2] == q2) {
            if (first == NONE) first = i;
            if (w.id[i] < best_id) { best_id = w.id[i]; best = i; }
        }
    }
    if (first == best) return first;
    u32 sy = w.lsize(y);
    const u32 sz = w.lsize(z);
    if (sy > sz) sy = sz;
    return !(w.lsize(x) > sy) ? first : best;
}

// The ITE candidate pair test of find_ITE_gate (ifthenelse.h:48-70); d1/d2 out.
HD bool wpv_ite_pair(const WarpPv& w, u32 dx, u32 i, u32 j, u32& d1, u32& d2) {
    const u32 fx = FLIP(dx);
    if (!(h_original(w.flags[i]) && w.size[i] == 3)) return false;
    if (!(h_original(w.flags[j]) && w.size[j] == 3)) return false;
    const u32* li = w.L(i);
    u32 xi = li[0], yi = li[1], zi = li[2];
    if (yi == dx) swap_t(xi, yi);
    if (zi == dx) swap_t(xi, zi);
    const u32* lj = w.L(j);
    u32 xj = lj[0], yj = lj[1], zj = lj[2];
    if (yj == dx) swap_t(xj, yj);
    if (zj == dx) swap_t(xj, zj);
    if (ABS(yi) == ABS(zj)) swap_t(yj, zj);
    if (ABS(zi) == ABS(zj)) return false;
    if (yi != FLIP(yj)) return false;
    d1 = wpv_feq_lane(w, fx, yi, FLIP(zi));
    if (d1 == NONE) return false;
    d2 = wpv_feq_lane(w, fx, yj, FLIP(zj));
    return d2 != NONE;
}

// find_ITE_gate (ifthenelse.h:42-97): first successful pair in (i, j) order.
HD bool wpv_find_ite_gate(WarpPv& w, const VeOpts& o, u32 dx, int nOrgCls, int& nAdded, u32& nLits) {
    const u32 side = dx & 1u, b = w.base(side), ns = w.n(side);
    // a gate needs a pair of original ternary clauses in this list; without one the
    // search below fails with no effect
    if (w.count_size(side, 3) < 2) return false;
    for (u32 a = 0; a < ns; a++) {
        const u32 i = b + a;
        if (!(h_original(w.flags[i]) && w.size[i] == 3)) continue;
        const u32 t = wfirst(ns - a - 1, [&](u32 q) {
            u32 d1, d2;
            return wpv_ite_pair(w, dx, i, i + 1 + q, d1, d2);
        });
        if (t == NONE_IDX) continue;
        const u32 j = i + 1 + t;
        u32 d1 = NONE, d2 = NONE;
        wpv_ite_pair(w, dx, i, j, d1, d2);
        wpv_set_molten(w, i, true);
        wpv_set_molten(w, j, true);
        wpv_set_molten(w, d1, true);
        wpv_set_molten(w, d2, true);
        nAdded = 0;
        if (wpv_count_added(w, o, nOrgCls, side, nAdded, nLits, true)) {
            wpv_set_molten(w, i, false);
            wpv_set_molten(w, j, false);
            wpv_set_molten(w, d1, false);
            wpv_set_molten(w, d2, false);
            return false;
        }
        return true;
    }
    return false;
}

// makeArity (xor.h:52-84): flip by the next even-parity counter, find the arity
// clause in the own list: the first in list order when the reference scans the own
// list (its literal has the shortest list), else the smallest id. The two agree
// unless two or more clauses match, so the list sizes are only read then.
HD bool wpv_make_arity(WarpPv& w, u32& parity, u32 size) {
    const u32 oldparity = parity;
    do { ++parity; } while (popc32(parity) & 1);
    wone([&]() {
        for (u32 k = 0; k < size; k++) {
            const u32 bit = 1u << k;
            if ((parity & bit) != (oldparity & bit)) w.xl[k] = FLIP(w.xl[k]);
        }
    });
    u32 ownlit = w.xl[0];
    for (u32 k = 0; k < size; k++) if (ABS(w.xl[k]) == w.v) ownlit = w.xl[k];
    const u32 side = ownlit & 1u, b = w.base(side), ns = w.n(side);
    auto match = [&](u32 t) {
        const u32 i = b + t;
        if (!(h_original(w.flags[i]) && w.size[i] == size)) return false;
        const u32* L = w.L(i);
        for (u32 a = 0; a < size; a++) {
            bool in = false;
            for (u32 q = 0; q < size; q++) if (L[a] == w.xl[q]) { in = true; break; }
            if (!in) return false;
        }
        return true;
    };
    u32 mid = NONE_IDX;
    const u32 t = wfirst_min(ns, match, [&](u32 q) { return w.id[b + q]; }, mid);
    if (t == NONE_IDX) return false;
    u32 found = b + t;
    if (w.id[found] != mid) {
        u32 best = w.xl[0], minsize = w.lsize(w.xl[0]);
        for (u32 k = 1; k < size; k++) {
            const u32 sk = w.lsize(w.xl[k]);
            if (sk < minsize) { minsize = sk; best = w.xl[k]; }
        }
        if (best != ownlit) found = b + wfirst(ns, [&](u32 q) { return w.id[b + q] == mid; });
    }
    wpv_set_molten(w, found, true);
    return true;
}

// find_XOR_gate (xor.h:86-131).
HD bool wpv_find_xor_gate(WarpPv& w, const VeOpts& o, u32 dx, int nOrgCls, int& nAdded, u32& nLits) {
    const u32 side = dx & 1u, b = w.base(side), ns = w.n(side);
    auto freeze_arities = [&]() {
        wpv_unmelt_if(w, 0, w.np + w.nn, [&](u32 i) { return w.size[i] > 2; });
    };
    // An XOR of arity k has 2^k clauses of size k+1, half of them in each list. A
    // candidate whose size has fewer originals than that in either list cannot
    // complete; its search would only melt and then unmelt clauses longer than two,
    // which freeze_arities does directly (once while nothing melts in between).
    bool frozen = false;
    for (u32 a = 0; a < ns; a++) {
        const u32 i = b + a;
        if (!h_original(w.flags[i])) continue;
        const u32 size = w.size[i];
        const int arity = (int)size - 1;
        if (size < 3 || arity > o.xor_max_arity) continue;
        const u32 need = arity - 1 < 31 ? (1u << (arity - 1)) : 0xFFFFFFFFu;
        if (w.count_size(side, size) < need || w.count_size(side ^ 1u, size) < need) {
            if (!frozen) freeze_arities();  // a repeat would change nothing
            frozen = true;
            continue;
        }
        frozen = false;  // this candidate's search melts clauses
        wfor(size, [&](u32 k) { w.xl[k] = w.L(i)[k]; });
        u32 parity = 0;
        int itargets = 1 << arity;
        while (--itargets && wpv_make_arity(w, parity, size)) {}
        if (itargets) freeze_arities();
        else {
            wpv_set_molten(w, i, true);
            nAdded = 0;
            if (wpv_count_added(w, o, nOrgCls, side, nAdded, nLits, true)) {
                freeze_arities();
                break;
            }
            return true;
        }
    }
    return false;
}

// The decision of bve() for the staged variable.
HD VeResult wpv_bve_decide(WarpPv& w, const VeOpts& o) {
    const u32 p = V2L(w.v), n = NEG(p);
    const u32 pOrgs = wpv_orgs(w, 0), nOrgs = wpv_orgs(w, 1);
    uint8_t type = VE_KEEP;
    int nAdded = 0;
    u32 nLits = 0, def = 0;
    if (!pOrgs || !nOrgs) {
        type = VE_PURE;
    } else if ((def = wpv_find_bn_gate(w)) != 0) {
        type = VE_EQU;
    } else {
        const int nOrgCls = (int)(pOrgs + nOrgs);
        if (nOrgCls > 2) {
            if (wpv_find_ao_gate(w, o, n, nOrgCls, nAdded, nLits)) type = VE_SUBST;
            else if (!nAdded && wpv_find_ao_gate(w, o, p, nOrgCls, nAdded, nLits)) type = VE_SUBST;
        }
        if (type == VE_KEEP && nOrgCls > 3) {
            if (wpv_find_ite_gate(w, o, p, nOrgCls, nAdded, nLits)) type = VE_SUBST;
            else if (!nAdded && wpv_find_ite_gate(w, o, n, nOrgCls, nAdded, nLits)) type = VE_SUBST;
            else if (wpv_find_xor_gate(w, o, p, nOrgCls, nAdded, nLits)) type = VE_SUBST;
            else if (!nAdded && wpv_find_xor_gate(w, o, n, nOrgCls, nAdded, nLits)) type = VE_SUBST;
        }
        if (type == VE_KEEP && !nAdded && !wpv_count_added(w, o, nOrgCls, 0, nAdded, nLits, false)) type = VE_RES;
    }
    VeResult r;
    r.type = type;
    r.porgs = pOrgs;
    r.norgs = nOrgs;
    r.def = def;
    const bool adds = type == VE_RES || type == VE_SUBST;
    r.ncls = adds ? (u32)nAdded : 0u;
    r.nlits = adds ? nLits : 0u;
    if (type == VE_KEEP) r.nwit = 0;
    else {
        const u32 s = pOrgs > nOrgs ? 1u : 0u;
        r.nwit = 2 + wpv_lits_before(w, s) + wpv_orgs(w, s);
    }
    return r;
}

}  // namespace sigma
