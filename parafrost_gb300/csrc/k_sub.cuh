// SUB: self-subsuming strengthening and backward subsumption over the two lists
// of every elected variable (ParaFROST::SUB, src/cpu/elimination.cpp:110-129;
// self_sub_x and helpers, src/cpu/subsume.h:27-179; GPU reference sub_k,
// kernels.cu:653-673, subsume.cuh).
//
// Elected variables never share a clause, so each one works on its own clauses
// in place. The one effect that crosses variables is a strengthened binary that
// becomes a unit: the reference enqueues it and at once deletes every clause of
// ot[unit] (elimination.cpp:214-226), which later variables then see deleted.
// Units can only come from a binary (x u) next to a binary (-x u) at the start of
// SUB (SUB only removes x from a clause, and only deletes clauses otherwise); when
// no elected variable has such a pair the parallel pass is exact. When some do
// (the producers), the driver settles the producers first: it checkpoints their
// lists, runs them, and re-runs (from the checkpoint, with the earlier producers'
// units' clauses pre-deleted) every producer whose set of such units changed,
// until none does. The other variables yield no unit, so one run of each, with the
// units of the producers before it pre-deleted, is exact. Inside one variable the
// reference's immediate deletion is applied to its own clauses. The bookkeeping
// (which units reach which variable, sorted and compared per variable) runs on the
// device.
#pragma once

#include "cnf.cuh"

namespace sigma {

constexpr int SUB_MAX_LOCAL_UNITS = 16;
constexpr u32 HSE_MAX_CL_SIZE = 1000;  // subsume.h:21

HD bool sig_sub(u32 A, u32 B) { return !(A & ~B); }
HD bool sig_selfsub(u32 A, u32 B) {
    const u32 Bt = B | ((B & 0xAAAAAAAAu) >> 1) | ((B & 0x55555555u) << 1);
    return !(A & ~Bt);
}

// sub(SCLAUSE&, SCLAUSE&) (subsume.h:39-56).
HD bool clause_sub(const u32* sm, u32 n1, const u32* lr, u32 n2) {
    u32 it1 = 0, it2 = 0, s = 0;
    while (it1 < n1 && it2 < n2) {
        const u32 a = sm[it1], b = lr[it2];
        if (a < b) it1++;
        else if (b < a) it2++;
        else { s++; it1++; it2++; }
    }
    return s == n1;
}

// selfsub(x, fx, sm, lr) (subsume.h:75-103).
HD bool clause_selfsub(u32 x, u32 fx, const u32* sm, u32 n1, const u32* lr, u32 n2) {
    u32 it1 = 0, it2 = 0, s = 0;
    bool self = false;
    while (it1 < n1 && it2 < n2) {
        const u32 a = sm[it1], b = lr[it2];
        if (a == fx) it1++;
        else if (b == x) { self = true; it2++; }
        else if (a < b) it1++;
        else if (b < a) it2++;
        else { s++; it1++; it2++; }
    }
    if (s + 1 == n1) {
        if (self) return true;
        while (it2 < n2) { if (lr[it2] == x) return true; it2++; }
    }
    return false;
}

HD bool sorted_has(const u32* l, u32 n, u32 lit) {
    u32 lo = 0, hi = n;
    while (lo < hi) {
        const u32 mid = (lo + hi) >> 1;
        if (l[mid] < lit) lo = mid + 1;
        else hi = mid;
    }
    return lo < n && l[lo] == lit;
}

HD void mark_deleted(const Ctx& c, u32 r) {
    c.hdr[r].flags = (c.hdr[r].flags & ~3u) | ST_DELETED;
    touch(c, r);
}
HD void set_molten(const Ctx& c, u32 r, bool m) {
    const u32 f = c.hdr[r].flags;
    c.hdr[r].flags = m ? (f | F_MOLTEN) : (f & ~F_MOLTEN);
}

struct SubArgs {
    Ctx c;
    const u32* pvs;
    u32 npvs;
    u32 sub_max;
    // units found: (pv rank, literal) pairs
    U2* units;
    u32* nunits;
    u32 cap_units;
    // per-PV literals whose clauses an earlier variable's unit deletes (re-runs only)
    const u32* pre_off;   // npvs + 1, or null
    const u32* pre_lits;
    const uint8_t* run;   // per PV: 1 = run this PV (null = all)
};

struct SubLocal {
    u32 units[SUB_MAX_LOCAL_UNITS];
    int n;
};

// toblivion(ot[unit]) restricted to this variable's own clauses.
HD void sub_local_oblivion(const Ctx& c, u32 p, u32 u) {
    for (u32 side = 0; side < 2; side++) {
        const u32 l = p + side;
        const u32 o = c.ot_off[l], s = c.ot_size[l];
        for (u32 i = 0; i < s; i++) {
            const u32 r = c.ot_refs[o + i];
            const Hdr h = c.hdr[r];
            if (sorted_has(c.lits + h.start, h.size, u)) mark_deleted(c, r);
        }
    }
}

// ParaFROST::strengthen (elimination.cpp:199-234).
HD void sub_strengthen(const SubArgs& a, u32 k, u32 p, u32 r, u32 me, SubLocal& L) {
    const Ctx& c = a.c;
    Hdr h = c.hdr[r];
    u32* l = c.lits + h.start;
    u32 n = 0, sig = 0;
    for (u32 i = 0; i < h.size; i++) {
        const u32 lit = l[i];
        if (lit != me) { l[n++] = lit; sig |= MAPHASH(lit); }
    }
    h.sig = sig;
    h.size = h.size - 1;
    c.hdr[r].sig = h.sig;
    c.hdr[r].size = h.size;
    touch(c, r);
    if (n > 1) proof_line(c, l, n);
    if (n == 1) {
        const u32 unit = l[0];
        int val = lit_value(c, unit);
        for (int i = 0; i < L.n; i++) {
            if (L.units[i] == unit) val = 1;
            else if (L.units[i] == FLIP(unit)) val = 0;
        }
        if (val == VAL_UNDEF) {
            if (L.n >= SUB_MAX_LOCAL_UNITS) { set_err(c, ERR_CAP_SCRATCH); return; }
            L.units[L.n++] = unit;
            const u32 pos = atom_add(a.nunits, 1u);
            if (pos < a.cap_units) a.units[pos] = mk_u2(k, unit);
            else set_err(c, ERR_CAP_SCRATCH);
            sub_local_oblivion(c, p, unit);
        } else if (val == 0) {
            set_unsat(c, ABS(unit));
        }
    }
}

// subsume(list, end, cand) (subsume.h:105-121).
HD bool sub_subsume(const Ctx& c, const u32* list, u32 end, u32 cr) {
    const Hdr cand = c.hdr[cr];
    const u32* cl = c.lits + cand.start;
    for (u32 j = 0; j < end; j++) {
        const u32 sr = list[j];
        const Hdr s = c.hdr[sr];
        if (h_deleted(s.flags)) continue;
        if (h_molten(cand.flags) && s.size > cand.size) continue;
        if (s.size > 1 && sig_sub(s.sig, cand.sig) && clause_sub(c.lits + s.start, s.size, cl, cand.size)) {
            if (h_learnt(s.flags) && h_original(cand.flags)) {
                c.hdr[sr].flags = (s.flags & ~3u) | ST_ORIGINAL;
                touch(c, sr);
            }
            proof_delete(c, cr);
            mark_deleted(c, cr);
            return true;
        }
    }
    return false;
}

// selfsubsume(x, fx, list, cand) (subsume.h:123-142).
HD bool sub_selfsubsume(const SubArgs& a, u32 k, u32 p, u32 x, u32 fx, const u32* list, u32 ls, u32 cr, SubLocal& L) {
    const Ctx& c = a.c;
    const Hdr cand = c.hdr[cr];
    const u32* cl = c.lits + cand.start;
    for (u32 j = 0; j < ls; j++) {
        const Hdr s = c.hdr[list[j]];
        if (s.size > cand.size) break;
        if (h_deleted(s.flags)) continue;
        if (s.size > 1 && sig_selfsub(s.sig, cand.sig) && clause_selfsub(x, fx, c.lits + s.start, s.size, cl, cand.size)) {
            sub_strengthen(a, k, p, cr, x, L);
            set_molten(c, cr, true);
            return true;
        }
    }
    return false;
}

// updateOL (subsume.h:27-37).
HD void sub_update_list(const Ctx& c, u32 l) {
    const u32 o = c.ot_off[l], s = c.ot_size[l];
    u32 j = 0;
    for (u32 i = 0; i < s; i++) {
        const u32 r = c.ot_refs[o + i];
        const u32 f = c.hdr[r].flags;
        if (h_molten(f)) c.hdr[r].flags = f & ~F_MOLTEN;
        else if (!h_deleted(f)) c.ot_refs[o + j++] = r;
    }
    c.ot_size[l] = j;
}

// self_sub_x (subsume.h:144-179), one elected variable per item.
HD void k_sub_pv(const SubArgs& a, u32 k) {
    if (a.run && !a.run[k]) return;
    const Ctx& c = a.c;
    const u32 v = a.pvs[k];
    const u32 p = V2L(v), n = NEG(p);
    if (c.ot_size[p] > a.sub_max || c.ot_size[n] > a.sub_max) return;
    SubLocal L;
    L.n = 0;
    if (a.pre_off) {
        for (u32 i = a.pre_off[k]; i < a.pre_off[k + 1]; i++) sub_local_oblivion(c, p, a.pre_lits[i]);
    }
    const u32* poss = c.ot_refs + c.ot_off[p];
    const u32* negs = c.ot_refs + c.ot_off[n];
    u32 ps = c.ot_size[p];
    for (u32 i = 0; i < ps; i++) {
        const u32 r = poss[i];
        const Hdr h = c.hdr[r];
        if (h.size > HSE_MAX_CL_SIZE) break;
        if (h_deleted(h.flags)) continue;
        sub_selfsubsume(a, k, p, p, n, negs, c.ot_size[n], r, L);
        sub_subsume(c, poss, i, r);
    }
    sub_update_list(c, p);
    ps = c.ot_size[p];
    const u32 ns = c.ot_size[n];
    for (u32 i = 0; i < ns; i++) {
        const u32 r = negs[i];
        const Hdr h = c.hdr[r];
        if (h.size > HSE_MAX_CL_SIZE) break;
        if (h_deleted(h.flags)) continue;
        sub_selfsubsume(a, k, p, n, p, poss, c.ot_size[p], r, L);
        sub_subsume(c, negs, i, r);
    }
    sub_update_list(c, n);
}

// Whether SUB on this variable can produce a unit: some binary (x u) in the
// positive list next to a binary (-x u) in the negative list. Counts producers in
// *flag and, with prod, sets prod[k] (cleared first).
HD void k_sub_unit_possible(const SubArgs& a, u32* flag, u32* prod, u32 k) {
    const Ctx& c = a.c;
    const u32 v = a.pvs[k];
    const u32 p = V2L(v), n = NEG(p);
    if (prod) prod[k] = 0;
    if (c.ot_size[p] > a.sub_max || c.ot_size[n] > a.sub_max) return;
    const u32 po = c.ot_off[p], ps = c.ot_size[p], no = c.ot_off[n], ns = c.ot_size[n];
    for (u32 i = 0; i < ps; i++) {
        const Hdr hi = c.hdr[c.ot_refs[po + i]];
        if (hi.size != 2 || h_deleted(hi.flags)) continue;
        const u32* li = c.lits + hi.start;
        const u32 ui = li[0] == p ? li[1] : li[0];
        for (u32 j = 0; j < ns; j++) {
            const Hdr hj = c.hdr[c.ot_refs[no + j]];
            if (hj.size != 2 || h_deleted(hj.flags)) continue;
            const u32* lj = c.lits + hj.start;
            const u32 uj = lj[0] == n ? lj[1] : lj[0];
            if (ui == uj) {
                atom_add(flag, 1u);
                if (prod) prod[k] = 1;
                return;
            }
        }
    }
}

// ---------------------------------------------------------------- checkpoint
// Per elected variable: its two lists (ids) and every clause in them (header +
// literals), so a re-run starts from the state SUB started with.
struct SubCkptArgs {
    Ctx c;
    const u32* pvs;
    const u32* ent_off;   // npvs+1: list entries (both lists)
    const u64* word_off;  // npvs+1: literal words
    u32* ids;             // saved list entries
    Hdr* hdrs;            // saved headers, one per entry
    u32* words;           // saved literals
    u32* sizes;           // 2 per PV: saved list sizes
    const uint8_t* run;   // restore only these (null = all)
};

HD void k_sub_need(const Ctx& c, const u32* pvs, const uint8_t* only, u32* ent, u64* words, u32 k) {
    if (only && !only[k]) {
        ent[k] = 0;
        words[k] = 0;
        return;
    }
    const u32 p = V2L(pvs[k]);
    u32 e = 0;
    u64 w = 0;
    for (u32 side = 0; side < 2; side++) {
        const u32 l = p + side, o = c.ot_off[l], s = c.ot_size[l];
        e += s;
        for (u32 i = 0; i < s; i++) w += c.hdr[c.ot_refs[o + i]].size;
    }
    ent[k] = e;
    words[k] = w;
}

HD void k_sub_save(const SubCkptArgs& a, u32 k) {
    if (a.run && !a.run[k]) return;
    const Ctx& c = a.c;
    const u32 p = V2L(a.pvs[k]);
    u32 e = a.ent_off[k];
    u64 w = a.word_off[k];
    for (u32 side = 0; side < 2; side++) {
        const u32 l = p + side, o = c.ot_off[l], s = c.ot_size[l];
        a.sizes[2 * k + side] = s;
        for (u32 i = 0; i < s; i++) {
            const u32 r = c.ot_refs[o + i];
            const Hdr h = c.hdr[r];
            a.ids[e] = r;
            a.hdrs[e] = h;
            e++;
            for (u32 t = 0; t < h.size; t++) a.words[w++] = c.lits[h.start + t];
        }
    }
}

HD void k_sub_restore(const SubCkptArgs& a, u32 k) {
    if (a.run && !a.run[k]) return;
    const Ctx& c = a.c;
    const u32 p = V2L(a.pvs[k]);
    u32 e = a.ent_off[k];
    u64 w = a.word_off[k];
    for (u32 side = 0; side < 2; side++) {
        const u32 l = p + side, o = c.ot_off[l], s = a.sizes[2 * k + side];
        c.ot_size[l] = s;
        for (u32 i = 0; i < s; i++) {
            const u32 r = a.ids[e];
            const Hdr h = a.hdrs[e];
            e++;
            c.ot_refs[o + i] = r;
            c.hdr[r] = h;
            touch(c, r);
            for (u32 t = 0; t < h.size; t++) c.lits[h.start + t] = a.words[w++];
        }
    }
}

// Which later variables does a unit reach? For unit q (found by PV rank `from`),
// every clause of ot[lit] owned by an elected variable of higher rank.
struct SubReachArgs {
    Ctx c;
    const U2* units;   // (rank, lit)
    U2* pairs;         // (target rank, unit index)
    u32* npairs;
    u32 cap_pairs;
    const uint8_t* target;  // targets considered (per rank); null = all
};
// One item per (unit, clause of the unit's list): a unit's list can be long (hub
// variables), so its clauses are spread over threads. item_off is the exclusive
// scan of the units' list sizes.
HD void k_sub_reach(const SubReachArgs& a, const u32* item_off, u32 nunits, u32 item) {
    const Ctx& c = a.c;
    u32 lo = 0, hi = nunits;  // unit q: item_off[q] <= item < item_off[q+1]
    while (hi - lo > 1) {
        const u32 mid = (lo + hi) >> 1;
        if (item_off[mid] <= item) lo = mid;
        else hi = mid;
    }
    const u32 q = lo;
    const U2 u = a.units[q];
    const Hdr h = c.hdr[c.ot_refs[c.ot_off[u.y] + (item - item_off[q])]];
    const u32* l = c.lits + h.start;
    for (u32 t = 0; t < h.size; t++) {
        const u32 owner = c.pvrank[ABS(l[t])];
        if (owner != NONE && owner > u.x) {
            if (a.target && !a.target[owner]) break;
            const u32 pos = atom_add(a.npairs, 1u);
            if (pos < a.cap_pairs) a.pairs[pos] = mk_u2(owner, q);
            else set_err(c, ERR_CAP_SCRATCH);
            break;
        }
    }
}
HD void k_sub_reach_size(const Ctx& c, const U2* units, u32* size, u32 q) { size[q] = c.ot_size[units[q].y]; }

// ---------------------------------------------------------------- unit sets
// The units every variable must see pre-deleted: reach pairs (target rank, unit)
// become the sorted set of distinct (rank, literal) pairs, segmented per rank; a
// variable re-runs when its segment differs from the one its last run used.
HD void k_subfx_pairlit(const U2* pairs, const U2* units, u32* rank, u32* lit, u32 i) {
    rank[i] = pairs[i].x;
    lit[i] = units[pairs[i].y].y;
}
HD void k_subfx_first(const u32* rank, const u32* lit, u32* flag, u32 i) {
    flag[i] = (i == 0 || rank[i] != rank[i - 1] || lit[i] != lit[i - 1]) ? 1u : 0u;
}
HD void k_subfx_scatter(const u32* rank, const u32* lit, const u32* flag, const u32* scan, u32* orank, u32* olit,
                        u32* count, u32 i) {
    if (!flag[i]) return;
    orank[scan[i]] = rank[i];
    olit[scan[i]] = lit[i];
    atom_add(&count[rank[i]], 1u);
}
HD void k_subfx_diff(const u32* woff, const u32* wlit, const u32* uoff, const u32* ulit, const uint8_t* cand,
                     u32* flag, uint8_t* run, u32 k) {
    bool d = false;
    if (cand[k]) {
        const u32 a0 = woff[k], n = woff[k + 1] - a0, b0 = uoff[k];
        d = n != uoff[k + 1] - b0;
        for (u32 i = 0; !d && i < n; i++) d = wlit[a0 + i] != ulit[b0 + i];
    }
    flag[k] = d ? 1u : 0u;
    run[k] = d ? 1 : 0;
}
// units of the variables that do not re-run stay
HD void k_subfx_keep(const U2* units, const uint8_t* run, u32* flag, u32 i) { flag[i] = run[units[i].x] ? 0u : 1u; }
HD void k_subfx_keep_scatter(const U2* units, const u32* flag, const u32* scan, U2* out, u32 i) {
    if (flag[i]) out[scan[i]] = units[i];
}
HD void k_subfx_to8(const u32* f, uint8_t* b, bool invert, u32 k) { b[k] = (f[k] != 0) != invert ? 1 : 0; }

// Commit of the units, spread over the clauses of their lists (a hub literal's
// list is long): item i is clause i - item_off[q] of ot[lits[q]]; the lists are
// emptied afterwards (k_sub_commit_clear).
HD void k_sub_commit_size(const Ctx& c, const u32* lits_, u32* size, u32 q) { size[q] = c.ot_size[lits_[q]]; }
HD void k_sub_commit_item(const Ctx& c, const u32* lits_, const u32* item_off, u32 nunits, u32 item) {
    u32 lo = 0, hi = nunits;
    while (hi - lo > 1) {
        const u32 mid = (lo + hi) >> 1;
        if (item_off[mid] <= item) lo = mid;
        else hi = mid;
    }
    const u32 lit = lits_[lo];
    mark_deleted(c, c.ot_refs[c.ot_off[lit] + (item - item_off[lo])]);
}
HD void k_sub_commit_clear(const Ctx& c, const u32* lits_, u32 q) { c.ot_size[lits_[q]] = 0; }

}  // namespace sigma
