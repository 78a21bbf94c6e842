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
// private. Gate finders also read lists of neighbour literals (never elected);
// where the reference takes the first match of such a list (which it keeps in
// clause-store order) the smallest matching clause id is taken instead.
#pragma once

#include "cnf.cuh"
#include "introsort.cuh"
#include "k_sub.cuh"

namespace sigma {

enum : uint8_t { VE_KEEP = 0, VE_PURE = 1, VE_EQU = 2, VE_RES = 3, VE_SUBST = 4 };

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

HD u32 count_orgs(const Ctx& c, u32 l) {
    const ListRef L = list_of(c, l);
    u32 n = 0;
    for (u32 i = 0; i < L.n; i++) if (h_original(c.hdr[L.ids[i]].flags)) n++;
    return n;
}

HD u32 lits_before(const Ctx& c, u32 l) {
    const ListRef L = list_of(c, l);
    u32 n = 0;
    for (u32 i = 0; i < L.n; i++) {
        const Hdr h = c.hdr[L.ids[i]];
        if (h_original(h.flags)) n += h.size;
    }
    return n;
}

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

// merge(x, c1, c2, out) (simplify.h:139-173); false for a tautology.
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

// countResolvents / countSubstituted (simplify.h:237-295). Returns true when the
// elimination is rejected; nAdded/nLits hold the counts (exact when accepted).
HD bool count_added(const BveArgs& a, u32 x, int clsbefore, u32 lme, u32 lother, int& nAdded, u32& nLits, bool gate) {
    const Ctx& c = a.c;
    const ListRef me = list_of(c, lme), other = list_of(c, lother);
    u32 added_lits = 0;
    const int rlimit = a.ve_clause_max;
    for (u32 i = 0; i < me.n; i++) {
        const Hdr hi = c.hdr[me.ids[i]];
        if (!h_original(hi.flags)) continue;
        const bool mi = h_molten(hi.flags);
        const u32* li = c.lits + hi.start;
        for (u32 j = 0; j < other.n; j++) {
            const Hdr hj = c.hdr[other.ids[j]];
            if (!h_original(hj.flags)) continue;
            if (gate && mi == h_molten(hj.flags)) continue;
            const int rsize = merge_size(x, li, hi.size, c.lits + hj.start, hj.size);
            if (rsize > 1) {
                if (++nAdded > clsbefore || (rlimit && rsize > rlimit)) { nLits = added_lits; return true; }
                added_lits += (u32)rsize;
            }
        }
    }
    nLits = added_lits;
    if (a.ve_lbound) {
        if (added_lits > lits_before(c, lme) + lits_before(c, lother)) return true;
    }
    return false;
}

HD void freeze_binaries(const Ctx& c, u32 l) {
    const ListRef L = list_of(c, l);
    for (u32 i = 0; i < L.n; i++) {
        const u32 r = L.ids[i];
        const Hdr h = c.hdr[r];
        if (h_original(h.flags) && h.size == 2) set_molten(c, r, false);
    }
}

// ---------------------------------------------------------------- EQU
// find_sfanin + find_BN_gate (equivalence.h:88-130).
HD u32 find_bn_gate(const Ctx& c, u32 p) {
    const u32 n = NEG(p);
    u32 first = 0;
    {
        const ListRef L = list_of(c, p);
        u32 imp = 0;
        int nImps = 0;
        bool multi = false;
        for (u32 i = 0; i < L.n; i++) {
            const u32 r = L.ids[i];
            const Hdr h = c.hdr[r];
            if (h_original(h.flags) && h.size == 2) {
                const u32* l = c.lits + h.start;
                imp = FLIP(l[0] ^ l[1] ^ p);
                set_molten(c, r, true);
                nImps++;
            }
            if (nImps > 1) { multi = true; break; }
        }
        first = multi ? 0u : imp;
    }
    if (first) {
        u32 second = n, def = first;
        if (second < first) { first = second; second = def; }
        const ListRef N = list_of(c, n);
        for (u32 i = 0; i < N.n; i++) {
            const u32 r = N.ids[i];
            const Hdr h = c.hdr[r];
            if (!(h_original(h.flags) && h.size == 2)) continue;
            const u32* l = c.lits + h.start;
            if (l[0] == first && l[1] == second) {
                set_molten(c, r, true);
                return def;
            }
        }
    }
    freeze_binaries(c, p);
    return 0;
}

// ---------------------------------------------------------------- AND/OR
// find_fanin + find_AO_gate (and.h:25-86). out: scratch of at least |ot[dx]|+1 words.
HD bool find_ao_gate(const BveArgs& a, u32 dx, int nOrgCls, u32* out, int& nAdded, u32& nLits) {
    const Ctx& c = a.c;
    const u32 x = ABS(dx);
    const ListRef I = list_of(c, dx);
    u32 on = 0, sig = 0;
    for (u32 i = 0; i < I.n; i++) {
        const u32 r = I.ids[i];
        const Hdr h = c.hdr[r];
        if (h_original(h.flags) && h.size == 2) {
            const u32* l = c.lits + h.start;
            const u32 imp = FLIP(l[0] ^ l[1] ^ dx);
            out[on++] = imp;
            sig |= MAPHASH(imp);
            set_molten(c, r, true);
        }
    }
    if (on > 1) {
        const u32 f_dx = FLIP(dx);
        out[on++] = f_dx;
        sig |= MAPHASH(f_dx);
        reference_list_sort(out, (int)on, LitLess());
        const ListRef O = list_of(c, f_dx);
        for (u32 i = 0; i < O.n; i++) {
            const u32 r = O.ids[i];
            const Hdr h = c.hdr[r];
            if (!(h_original(h.flags) && h.size == on && sig_sub(h.sig, sig))) continue;
            const u32* l = c.lits + h.start;
            bool eq = true;
            for (u32 t = 0; t < on; t++) if (l[t] != out[t]) { eq = false; break; }
            if (!eq) continue;
            set_molten(c, r, true);
            nAdded = 0;
            if (count_added(a, x, nOrgCls, dx, f_dx, nAdded, nLits, true)) {
                set_molten(c, r, false);
                break;
            }
            return true;
        }
    }
    freeze_binaries(c, dx);
    return false;
}

// ---------------------------------------------------------------- ITE
// fast_equality_check (ifthenelse.h:25-40): the original, unmolten ternary (x y z)
// in the shortest of the three lists; NONE if absent. The first argument is always
// the elected variable's own literal, so every clause that can match is in that
// literal's own list: the search scans the own list and returns the first match in
// its order when the reference picks the own list, else the smallest matching id
// (the reference's first match in a neighbour list, which it keeps in clause-store
// order, among the same set of live matching clauses).
HD u32 fast_equality_check(const Ctx& c, u32 v, u32 x, u32 y, u32 z) {
    const u32 ownlit = x;
    if (c.ot_size[y] > c.ot_size[z]) swap_t(y, z);
    if (c.ot_size[x] > c.ot_size[y]) swap_t(x, y);
    const u32 ll = x;
    // sort3 (simplify.h:105-117)
    { const u32 lo = y < z ? y : z, hi = y < z ? z : y; y = lo; z = hi; }
    { const u32 lo = x < z ? x : z, hi = x < z ? z : x; x = lo; z = hi; }
    { const u32 lo = x < y ? x : y, hi = x < y ? y : x; x = lo; y = hi; }
    const ListRef L = list_of(c, ownlit);
    const bool own = ll == ownlit;
    (void)v;
    u32 best = NONE;
    for (u32 i = 0; i < L.n; i++) {
        const u32 r = L.ids[i];
        const Hdr h = c.hdr[r];
        if (h_molten(h.flags)) continue;
        if (!(h_original(h.flags) && h.size == 3)) continue;
        const u32* l = c.lits + h.start;
        if (l[0] == x && l[1] == y && l[2] == z) {
            if (own) return r;
            if (r < best) best = r;
        }
    }
    return best;
}

// find_ITE_gate (ifthenelse.h:42-97).
HD bool find_ite_gate(const BveArgs& a, u32 dx, int nOrgCls, int& nAdded, u32& nLits) {
    const Ctx& c = a.c;
    const u32 fx = FLIP(dx), v = ABS(dx);
    const ListRef I = list_of(c, dx);
    for (u32 i = 0; i < I.n; i++) {
        const u32 ri = I.ids[i];
        const Hdr hi = c.hdr[ri];
        if (!(h_original(hi.flags) && hi.size == 3)) continue;
        const u32* li = c.lits + hi.start;
        u32 xi = li[0], yi = li[1], zi = li[2];
        if (yi == dx) swap_t(xi, yi);
        if (zi == dx) swap_t(xi, zi);
        for (u32 j = i + 1; j < I.n; j++) {
            const u32 rj = I.ids[j];
            const Hdr hj = c.hdr[rj];
            if (!(h_original(hj.flags) && hj.size == 3)) continue;
            const u32* lj = c.lits + hj.start;
            u32 xj = lj[0], yj = lj[1], zj = lj[2];
            if (yj == dx) swap_t(xj, yj);
            if (zj == dx) swap_t(xj, zj);
            if (ABS(yi) == ABS(zj)) swap_t(yj, zj);
            if (ABS(zi) == ABS(zj)) continue;
            if (yi != FLIP(yj)) continue;
            const u32 d1 = fast_equality_check(c, v, fx, yi, FLIP(zi));
            if (d1 == NONE) continue;
            const u32 d2 = fast_equality_check(c, v, fx, yj, FLIP(zj));
            if (d2 == NONE) continue;
            set_molten(c, ri, true); set_molten(c, rj, true);
            set_molten(c, d1, true); set_molten(c, d2, true);
            nAdded = 0;
            if (count_added(a, v, nOrgCls, dx, fx, nAdded, nLits, true)) {
                set_molten(c, ri, false); set_molten(c, rj, false);
                set_molten(c, d1, false); set_molten(c, d2, false);
                return false;
            }
            return true;
        }
    }
    return false;
}

// ---------------------------------------------------------------- XOR
constexpr int XOR_MAX_SIZE = 21;  // xormaxarity <= 20 (src/cpu/options.cpp:46)

HD void freeze_arities(const Ctx& c, u32 l1, u32 l2) {
    for (u32 side = 0; side < 2; side++) {
        const ListRef L = list_of(c, side ? l2 : l1);
        for (u32 i = 0; i < L.n; i++) {
            const u32 r = L.ids[i];
            const Hdr h = c.hdr[r];
            if (h.size > 2 && h_molten(h.flags)) set_molten(c, r, false);
        }
    }
}

// makeArity (xor.h:52-84), COUNTFLIPS (xor.h:23-27).
HD bool make_arity(const Ctx& c, u32 v, u32& parity, u32* lits, int size) {
    const u32 oldparity = parity;
    do { ++parity; } while (popc32(parity) & 1);
    for (int k = 0; k < size; k++) {
        const u32 bit = 1u << k;
        if ((parity & bit) != (oldparity & bit)) lits[k] = FLIP(lits[k]);
    }
    u32 best = lits[0];
    u32 minsize = c.ot_size[best];
    u32 ownlit = lits[0];
    for (int k = 1; k < size; k++) {
        const u32 ls = c.ot_size[lits[k]];
        if (ls < minsize) { minsize = ls; best = lits[k]; }
    }
    for (int k = 0; k < size; k++) if (ABS(lits[k]) == v) ownlit = lits[k];
    // Every clause that can match holds the variable's own literal: scan that list
    // (see fast_equality_check for why the result is the reference's).
    const ListRef L = list_of(c, ownlit);
    const bool own = best == ownlit;
    u32 found = NONE;
    for (u32 i = 0; i < L.n; i++) {
        const u32 r = L.ids[i];
        const Hdr h = c.hdr[r];
        if (!(h_original(h.flags) && h.size == (u32)size)) continue;
        const u32* l = c.lits + h.start;
        bool all = true;
        for (int t = 0; t < size && all; t++) {  // checkArity (xor.h:35-50)
            bool in = false;
            for (int q = 0; q < size; q++) if (l[t] == lits[q]) { in = true; break; }
            all = in;
        }
        if (!all) continue;
        if (own) { found = r; break; }
        if (r < found) found = r;
    }
    if (found == NONE) return false;
    set_molten(c, found, true);
    return true;
}

// find_XOR_gate (xor.h:86-131).
HD bool find_xor_gate(const BveArgs& a, u32 dx, int nOrgCls, int& nAdded, u32& nLits) {
    const Ctx& c = a.c;
    const u32 fx = FLIP(dx), v = ABS(dx);
    const ListRef I = list_of(c, dx);
    u32 out[XOR_MAX_SIZE];
    for (u32 i = 0; i < I.n; i++) {
        const u32 ri = I.ids[i];
        const Hdr hi = c.hdr[ri];
        if (!h_original(hi.flags)) continue;
        const int size = (int)hi.size;
        const int arity = size - 1;
        if (size < 3 || arity > a.xor_max_arity) continue;
        const u32* li = c.lits + hi.start;
        for (int t = 0; t < size; t++) out[t] = li[t];
        u32 parity = 0;
        int itargets = 1 << arity;
        while (--itargets && make_arity(c, v, parity, out, size)) {}
        if (itargets) freeze_arities(c, dx, fx);
        else {
            set_molten(c, ri, true);
            nAdded = 0;
            if (count_added(a, v, nOrgCls, dx, fx, nAdded, nLits, true)) {
                freeze_arities(c, dx, fx);
                break;
            }
            return true;
        }
    }
    return false;
}

// Witness words of toblivion / save_BN_gate (simplify.h:305-332, equivalence.h:132-153).
HD u32 witness_words(const Ctx& c, u32 p, u32 pOrgs, u32 nOrgs) {
    const u32 l = pOrgs > nOrgs ? NEG(p) : p;
    const ListRef L = list_of(c, l);
    u32 w = 2;
    for (u32 i = 0; i < L.n; i++) {
        const Hdr h = c.hdr[L.ids[i]];
        if (h_original(h.flags)) w += h.size + 1;
    }
    return w;
}

// Step 1: the decision of bve() (bve.cpp:37-142) for one elected variable.
HD void k_bve_analyze(const BveArgs& a, u32 k) {
    const Ctx& c = a.c;
    const u32 v = a.pvs[k];
    const u32 p = V2L(v), n = NEG(p);
    const u32 pOrgs = count_orgs(c, p), nOrgs = count_orgs(c, n);
    uint8_t type = VE_KEEP;
    int nAdded = 0;
    u32 nLits = 0, def = 0;
    if (!pOrgs || !nOrgs) {
        type = VE_PURE;
    } else if ((def = find_bn_gate(c, p)) != 0) {
        type = VE_EQU;
    } else {
        const int nOrgCls = (int)(pOrgs + nOrgs);
        u32* scr = a.scr + a.scr_off[k];
        if (nOrgCls > 2) {
            if (find_ao_gate(a, n, nOrgCls, scr, nAdded, nLits)) type = VE_SUBST;
            else if (!nAdded && find_ao_gate(a, p, nOrgCls, scr, nAdded, nLits)) type = VE_SUBST;
        }
        if (type == VE_KEEP && nOrgCls > 3) {
            if (find_ite_gate(a, p, nOrgCls, nAdded, nLits)) type = VE_SUBST;
            else if (!nAdded && find_ite_gate(a, n, nOrgCls, nAdded, nLits)) type = VE_SUBST;
            else if (find_xor_gate(a, p, nOrgCls, nAdded, nLits)) type = VE_SUBST;
            else if (!nAdded && find_xor_gate(a, n, nOrgCls, nAdded, nLits)) type = VE_SUBST;
        }
        if (type == VE_KEEP && !nAdded && !count_added(a, v, nOrgCls, p, n, nAdded, nLits, false)) type = VE_RES;
    }
    a.type[k] = type;
    a.porgs[k] = pOrgs;
    a.norgs[k] = nOrgs;
    a.def[k] = def;
    const bool adds = type == VE_RES || type == VE_SUBST;
    a.ncls[k] = adds ? (u32)nAdded : 0u;
    a.nlits[k] = adds ? nLits : 0u;
    a.nwit[k] = type == VE_KEEP ? 0u : witness_words(c, p, pOrgs, nOrgs);
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
    return w;
}
HD u64 save_witness(const Ctx& c, u64 w, u32 lit) {
    c.resolved[w++] = lit;
    c.resolved[w++] = 1;
    return w;
}

// A unit found inside the round goes to the trail unless its variable is already
// assigned; the opposite assignment is a conflict (enqueueUnit / learnEmpty paths of
// bve.cpp:200-211, equivalence.h:56-80).
HD void enqueue_unit(const Ctx& c, u32 u) {
    const u32 old = atom_cas(&c.asg[ABS(u)], 0u, u);
    if (old == 0) {
        const u32 pos = atom_add(c.ntrail, 1u);
        c.trail[pos] = u;
    } else if (old != u) {
        set_err(c, ERR_UNSAT);
    }
}

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
    if (n == 1) { c.hdr[r].size = 1; return l[0]; }
    reference_list_sort(l, (int)n, LitLess());
    h.sig = calc_sig(l, n);
    c.hdr[r].size = h.size;
    c.hdr[r].sig = h.sig;
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

// Per-variable scratch words for the AND/OR fan-in list.
HD void k_bve_scratch_need(const Ctx& c, const u32* pvs, u64* need, u32 k) {
    const u32 p = V2L(pvs[k]);
    need[k] = (u64)c.ot_size[p] + c.ot_size[NEG(p)] + 2;
}

}  // namespace sigma
