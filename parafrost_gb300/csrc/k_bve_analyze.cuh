// BVE step 1 (the decision of ParaFROST::bve, src/cpu/bve.cpp:37-142) over a view
// of one elected variable's two occurrence lists.
//
// This is the per-thread form of the decision, reading the lists straight from the
// clause store (GlobalPv). The kernel runs the warp form (k_bve_warp.cuh); a
// variable whose lists do not fit the warp's shared-memory slot runs this one on
// lane 0.
//
// View entries are numbered 0..np-1 (the positive list ot[2v]) and np..np+nn-1 (the
// negative list ot[2v+1]); side s of literal l is l & 1.
#pragma once

#include "cnf.cuh"
#include "introsort.cuh"
#include "k_sub.cuh"

namespace sigma {

// ---------------------------------------------------------------- views
struct GlobalPv {
    const Ctx* c;
    u32 v, np, nn;
    const u32* lp;  // ot[2v] entries
    const u32* ln;  // ot[2v+1] entries
    u32* scr;       // scratch of at least np+nn+2 words (AND/OR fan-in list)

    HD void init(const Ctx& cc, u32 var, u32* scratch) {
        c = &cc;
        v = var;
        const u32 p = V2L(var);
        np = cc.ot_size[p];
        nn = cc.ot_size[p + 1];
        lp = cc.ot_refs + cc.ot_off[p];
        ln = cc.ot_refs + cc.ot_off[p + 1];
        scr = scratch;
    }
    HD u32 n(u32 side) const { return side ? nn : np; }
    HD u32 base(u32 side) const { return side ? np : 0u; }
    HD u32 id(u32 i) const { return i < np ? lp[i] : ln[i - np]; }
    HD u32 size(u32 i) const { return c->hdr[id(i)].size; }
    HD u32 sig(u32 i) const { return c->hdr[id(i)].sig; }
    HD u32 flags(u32 i) const { return c->hdr[id(i)].flags; }
    HD const u32* lits(u32 i) const { return c->lits + c->hdr[id(i)].start; }
    HD void set_molten(u32 i, bool m) const { sigma::set_molten(*c, id(i), m); }
    HD u32* scratch() const { return scr; }
};

// ---------------------------------------------------------------- helpers
// merge(x, c1, c2) -> resolvent size, 0 for a tautology (simplify.h:175-202).
HD int merge_size(u32 x, const u32* a, u32 n1, const u32* b, u32 n2) {
    u32 i = 0, j = 0;
    int len = (int)(n1 + n2) - 2;
    while (i < n1 && j < n2) {
        const u32 l1 = a[i], l2 = b[j];
        const u32 v1 = ABS(l1), v2 = ABS(l2);
        if (v1 == x) i++;
        else if (v2 == x) j++;
        else if ((l1 ^ l2) == 1u) return 0;
        else if (v1 < v2) i++;
        else if (v2 < v1) j++;
        else { i++; j++; len--; }
    }
    return len;
}

struct VeOpts {
    int ve_clause_max;
    int ve_lbound;
    int xor_max_arity;
};

template <class A>
HD u32 pv_count_orgs(const A& a, u32 side) {
    u32 n = 0;
    const u32 b = a.base(side), e = b + a.n(side);
    for (u32 i = b; i < e; i++) if (h_original(a.flags(i))) n++;
    return n;
}

template <class A>
HD u32 pv_lits_before(const A& a, u32 side) {
    u32 n = 0;
    const u32 b = a.base(side), e = b + a.n(side);
    for (u32 i = b; i < e; i++) if (h_original(a.flags(i))) n += a.size(i);
    return n;
}

// countResolvents / countSubstituted (simplify.h:237-295): "me" = side sme.
template <class A>
HD bool pv_count_added(const A& a, const VeOpts& o, int clsbefore, u32 sme, int& nAdded, u32& nLits, bool gate) {
    const u32 x = a.v;
    const u32 so = sme ^ 1u;
    const u32 bm = a.base(sme), em = bm + a.n(sme), bo = a.base(so), eo = bo + a.n(so);
    u32 added = 0;
    const int rlimit = o.ve_clause_max;
    for (u32 i = bm; i < em; i++) {
        const u32 fi = a.flags(i);
        if (!h_original(fi)) continue;
        const bool mi = h_molten(fi);
        const u32* li = a.lits(i);
        const u32 si = a.size(i);
        for (u32 j = bo; j < eo; j++) {
            const u32 fj = a.flags(j);
            if (!h_original(fj)) continue;
            if (gate && mi == h_molten(fj)) continue;
            const int rsize = merge_size(x, li, si, a.lits(j), a.size(j));
            if (rsize > 1) {
                if (++nAdded > clsbefore || (rlimit && rsize > rlimit)) { nLits = added; return true; }
                added += (u32)rsize;
            }
        }
    }
    nLits = added;
    if (o.ve_lbound) {
        if (added > pv_lits_before(a, 0) + pv_lits_before(a, 1)) return true;
    }
    return false;
}

template <class A>
HD void pv_freeze_binaries(A& a, u32 side) {
    const u32 b = a.base(side), e = b + a.n(side);
    for (u32 i = b; i < e; i++)
        if (h_original(a.flags(i)) && a.size(i) == 2 && h_molten(a.flags(i))) a.set_molten(i, false);
}

// find_sfanin + find_BN_gate (equivalence.h:88-130).
template <class A>
HD u32 pv_find_bn_gate(A& a) {
    const u32 p = V2L(a.v), n = NEG(p);
    u32 first = 0;
    {
        u32 imp = 0;
        int nImps = 0;
        bool multi = false;
        for (u32 i = 0; i < a.np; i++) {
            if (h_original(a.flags(i)) && a.size(i) == 2) {
                const u32* l = a.lits(i);
                imp = FLIP(l[0] ^ l[1] ^ p);
                a.set_molten(i, true);
                nImps++;
            }
            if (nImps > 1) { multi = true; break; }
        }
        first = multi ? 0u : imp;
    }
    if (first) {
        u32 second = n, def = first;
        if (second < first) { first = second; second = def; }
        for (u32 i = a.np; i < a.np + a.nn; i++) {
            if (!(h_original(a.flags(i)) && a.size(i) == 2)) continue;
            const u32* l = a.lits(i);
            if (l[0] == first && l[1] == second) {
                a.set_molten(i, true);
                return def;
            }
        }
    }
    pv_freeze_binaries(a, 0);
    return 0;
}

// find_fanin + find_AO_gate (and.h:25-86) for gate output literal dx.
template <class A>
HD bool pv_find_ao_gate(A& a, const VeOpts& o, u32 dx, int nOrgCls, int& nAdded, u32& nLits) {
    const u32 side = dx & 1u, fside = side ^ 1u;
    u32* out = a.scratch();
    u32 on = 0, sig = 0;
    const u32 b = a.base(side), e = b + a.n(side);
    for (u32 i = b; i < e; i++) {
        if (h_original(a.flags(i)) && a.size(i) == 2) {
            const u32* l = a.lits(i);
            const u32 imp = FLIP(l[0] ^ l[1] ^ dx);
            out[on++] = imp;
            sig |= MAPHASH(imp);
            a.set_molten(i, true);
        }
    }
    if (on > 1) {
        const u32 f_dx = FLIP(dx);
        out[on++] = f_dx;
        sig |= MAPHASH(f_dx);
        reference_list_sort(out, (int)on, LitLess());
        const u32 fb = a.base(fside), fe = fb + a.n(fside);
        for (u32 i = fb; i < fe; i++) {
            const u32 f = a.flags(i);
            if (!(h_original(f) && a.size(i) == on && sig_sub(a.sig(i), sig))) continue;
            const u32* l = a.lits(i);
            bool eq = true;
            for (u32 t = 0; t < on; t++) if (l[t] != out[t]) { eq = false; break; }
            if (!eq) continue;
            a.set_molten(i, true);
            nAdded = 0;
            if (pv_count_added(a, o, nOrgCls, side, nAdded, nLits, true)) {
                a.set_molten(i, false);
                break;
            }
            return true;
        }
    }
    pv_freeze_binaries(a, side);
    return false;
}

// fast_equality_check (ifthenelse.h:25-40): index of the original, unmolten ternary
// (x y z) in the shortest of the three lists; NONE if absent. x is the variable's own
// literal; every clause that can match holds it, so the own list is scanned: first
// match in its order when the reference picks the own list, else the smallest
// matching id (the reference's first match in a neighbour list, which it keeps in
// clause-store order, among the same live matching clauses).
template <class A>
HD u32 pv_fast_equality_check(const A& a, u32 x, u32 y, u32 z) {
    const Ctx& c = *a.c;
    const u32 ownlit = x;
    if (c.ot_size[y] > c.ot_size[z]) swap_t(y, z);
    const u32 sx = a.n(ownlit & 1u);  // own list size
    const u32 sy = c.ot_size[y];
    const bool own = !(sx > sy);      // the reference keeps x when ot[x] is not longer than ot[y]
    // sort3 (simplify.h:105-117) of the three literals
    u32 q0 = x, q1 = y, q2 = z;
    { const u32 lo = q1 < q2 ? q1 : q2, hi = q1 < q2 ? q2 : q1; q1 = lo; q2 = hi; }
    { const u32 lo = q0 < q2 ? q0 : q2, hi = q0 < q2 ? q2 : q0; q0 = lo; q2 = hi; }
    { const u32 lo = q0 < q1 ? q0 : q1, hi = q0 < q1 ? q1 : q0; q0 = lo; q1 = hi; }
    const u32 side = ownlit & 1u;
    const u32 b = a.base(side), e = b + a.n(side);
    u32 best = NONE, best_id = NONE;
    for (u32 i = b; i < e; i++) {
        const u32 f = a.flags(i);
        if (h_molten(f)) continue;
        if (!(h_original(f) && a.size(i) == 3)) continue;
        const u32* l = a.lits(i);
        if (l[0] == q0 && l[1] == q1 && l[2] == q2) {
            if (own) return i;
            const u32 id = a.id(i);
            if (id < best_id) { best_id = id; best = i; }
        }
    }
    return best;
}

// find_ITE_gate (ifthenelse.h:42-97).
template <class A>
HD bool pv_find_ite_gate(A& a, const VeOpts& o, u32 dx, int nOrgCls, int& nAdded, u32& nLits) {
    const u32 fx = FLIP(dx);
    const u32 side = dx & 1u;
    const u32 b = a.base(side), e = b + a.n(side);
    for (u32 i = b; i < e; i++) {
        if (!(h_original(a.flags(i)) && a.size(i) == 3)) continue;
        const u32* li = a.lits(i);
        u32 xi = li[0], yi = li[1], zi = li[2];
        if (yi == dx) swap_t(xi, yi);
        if (zi == dx) swap_t(xi, zi);
        for (u32 j = i + 1; j < e; j++) {
            if (!(h_original(a.flags(j)) && a.size(j) == 3)) continue;
            const u32* lj = a.lits(j);
            u32 xj = lj[0], yj = lj[1], zj = lj[2];
            if (yj == dx) swap_t(xj, yj);
            if (zj == dx) swap_t(xj, zj);
            if (ABS(yi) == ABS(zj)) swap_t(yj, zj);
            if (ABS(zi) == ABS(zj)) continue;
            if (yi != FLIP(yj)) continue;
            const u32 d1 = pv_fast_equality_check(a, fx, yi, FLIP(zi));
            if (d1 == NONE) continue;
            const u32 d2 = pv_fast_equality_check(a, fx, yj, FLIP(zj));
            if (d2 == NONE) continue;
            a.set_molten(i, true); a.set_molten(j, true);
            a.set_molten(d1, true); a.set_molten(d2, true);
            nAdded = 0;
            if (pv_count_added(a, o, nOrgCls, side, nAdded, nLits, true)) {
                a.set_molten(i, false); a.set_molten(j, false);
                a.set_molten(d1, false); a.set_molten(d2, false);
                return false;
            }
            return true;
        }
    }
    return false;
}

constexpr int XOR_MAX_SIZE = 21;  // xormaxarity <= 20 (src/cpu/options.cpp:46)

// freezeArities (xor.h:13-25).
template <class A>
HD void pv_freeze_arities(A& a) {
    for (u32 i = 0; i < a.np + a.nn; i++)
        if (a.size(i) > 2 && h_molten(a.flags(i))) a.set_molten(i, false);
}

// makeArity (xor.h:52-84) with COUNTFLIPS (xor.h:23-27). Matches hold the own
// literal: the own list is scanned (see pv_fast_equality_check).
template <class A>
HD bool pv_make_arity(A& a, u32& parity, u32* lits, int size) {
    const Ctx& c = *a.c;
    const u32 oldparity = parity;
    do { ++parity; } while (popc32(parity) & 1);
    for (int k = 0; k < size; k++) {
        const u32 bit = 1u << k;
        if ((parity & bit) != (oldparity & bit)) lits[k] = FLIP(lits[k]);
    }
    u32 best = lits[0], ownlit = lits[0];
    u32 minsize = ABS(lits[0]) == a.v ? a.n(lits[0] & 1u) : c.ot_size[lits[0]];
    for (int k = 0; k < size; k++) if (ABS(lits[k]) == a.v) ownlit = lits[k];
    for (int k = 1; k < size; k++) {
        const u32 ls = ABS(lits[k]) == a.v ? a.n(lits[k] & 1u) : c.ot_size[lits[k]];
        if (ls < minsize) { minsize = ls; best = lits[k]; }
    }
    const bool own = best == ownlit;
    const u32 side = ownlit & 1u;
    const u32 b = a.base(side), e = b + a.n(side);
    u32 found = NONE, found_id = NONE;
    for (u32 i = b; i < e; i++) {
        if (!(h_original(a.flags(i)) && a.size(i) == (u32)size)) continue;
        const u32* l = a.lits(i);
        bool all = true;
        for (int t = 0; t < size && all; t++) {  // checkArity (xor.h:35-50)
            bool in = false;
            for (int q = 0; q < size; q++) if (l[t] == lits[q]) { in = true; break; }
            all = in;
        }
        if (!all) continue;
        if (own) { found = i; break; }
        const u32 id = a.id(i);
        if (id < found_id) { found_id = id; found = i; }
    }
    if (found == NONE) return false;
    a.set_molten(found, true);
    return true;
}

// find_XOR_gate (xor.h:86-131).
template <class A>
HD bool pv_find_xor_gate(A& a, const VeOpts& o, u32 dx, int nOrgCls, int& nAdded, u32& nLits) {
    const u32 side = dx & 1u;
    const u32 b = a.base(side), e = b + a.n(side);
    u32 out[XOR_MAX_SIZE];
    for (u32 i = b; i < e; i++) {
        if (!h_original(a.flags(i))) continue;
        const int size = (int)a.size(i);
        const int arity = size - 1;
        if (size < 3 || arity > o.xor_max_arity) continue;
        const u32* li = a.lits(i);
        for (int t = 0; t < size; t++) out[t] = li[t];
        u32 parity = 0;
        int itargets = 1 << arity;
        while (--itargets && pv_make_arity(a, parity, out, size)) {}
        if (itargets) pv_freeze_arities(a);
        else {
            a.set_molten(i, true);
            nAdded = 0;
            if (pv_count_added(a, o, nOrgCls, side, nAdded, nLits, true)) {
                pv_freeze_arities(a);
                break;
            }
            return true;
        }
    }
    return false;
}

// Witness words of toblivion / save_BN_gate (simplify.h:305-332, equivalence.h:132-153).
template <class A>
HD u32 pv_witness_words(const A& a, u32 pOrgs, u32 nOrgs) {
    const u32 side = pOrgs > nOrgs ? 1u : 0u;
    const u32 b = a.base(side), e = b + a.n(side);
    u32 w = 2;
    for (u32 i = b; i < e; i++) if (h_original(a.flags(i))) w += a.size(i) + 1;
    return w;
}

struct VeResult {
    uint8_t type;
    u32 porgs, norgs, ncls, nlits, nwit, def;
};

enum : uint8_t { VE_KEEP = 0, VE_PURE = 1, VE_EQU = 2, VE_RES = 3, VE_SUBST = 4 };

// The decision of bve() (bve.cpp:37-142) for one elected variable.
template <class A>
HD VeResult pv_bve_decide(A& a, const VeOpts& o) {
    const u32 p = V2L(a.v), n = NEG(p);
    const u32 pOrgs = pv_count_orgs(a, 0), nOrgs = pv_count_orgs(a, 1);
    uint8_t type = VE_KEEP;
    int nAdded = 0;
    u32 nLits = 0, def = 0;
    if (!pOrgs || !nOrgs) {
        type = VE_PURE;
    } else if ((def = pv_find_bn_gate(a)) != 0) {
        type = VE_EQU;
    } else {
        const int nOrgCls = (int)(pOrgs + nOrgs);
        if (nOrgCls > 2) {
            if (pv_find_ao_gate(a, o, n, nOrgCls, nAdded, nLits)) type = VE_SUBST;
            else if (!nAdded && pv_find_ao_gate(a, o, p, nOrgCls, nAdded, nLits)) type = VE_SUBST;
        }
        if (type == VE_KEEP && nOrgCls > 3) {
            if (pv_find_ite_gate(a, o, p, nOrgCls, nAdded, nLits)) type = VE_SUBST;
            else if (!nAdded && pv_find_ite_gate(a, o, n, nOrgCls, nAdded, nLits)) type = VE_SUBST;
            else if (pv_find_xor_gate(a, o, p, nOrgCls, nAdded, nLits)) type = VE_SUBST;
            else if (!nAdded && pv_find_xor_gate(a, o, n, nOrgCls, nAdded, nLits)) type = VE_SUBST;
        }
        if (type == VE_KEEP && !nAdded && !pv_count_added(a, o, nOrgCls, 0, nAdded, nLits, false)) type = VE_RES;
    }
    VeResult r;
    r.type = type;
    r.porgs = pOrgs;
    r.norgs = nOrgs;
    r.def = def;
    const bool adds = type == VE_RES || type == VE_SUBST;
    r.ncls = adds ? (u32)nAdded : 0u;
    r.nlits = adds ? nLits : 0u;
    r.nwit = type == VE_KEEP ? 0u : pv_witness_words(a, pOrgs, nOrgs);
    return r;
}

}  // namespace sigma
