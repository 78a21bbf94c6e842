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

// Wave A: one item per pending literal.
HD void k_prop_lists(const PropArgs& a, u32 k) {
    const Ctx& c = a.c;
    const u32 t = c.trail[a.head + k];
    const u32 f = FLIP(t);
    // collect ot[-t]
    const u32 fo = c.ot_off[f], fs = c.ot_size[f];
    for (u32 i = 0; i < fs; i++) {
        const u32 r = c.ot_refs[fo + i];
        if (h_deleted(c.hdr[r].flags)) continue;
        if (atom_exch(&a.cl_stamp[r], a.stamp) == a.stamp) continue;
        const u32 pos = atom_add(a.nwork, 1u);
        if (pos < a.cap_work) a.work[pos] = r;
        else set_err(c, ERR_CAP_SCRATCH);
    }
    // toblivion(ot[t])
    const u32 to = c.ot_off[t], ts = c.ot_size[t];
    for (u32 i = 0; i < ts; i++) {
        const u32 r = c.ot_refs[to + i];
        c.hdr[r].flags = (c.hdr[r].flags & ~3u) | ST_DELETED;
    }
    c.ot_size[t] = 0;
    c.ot_size[f] = 0;
}

// Wave B: one item per collected clause.
HD void k_prop_clause(const PropArgs& a, u32 k) {
    const Ctx& c = a.c;
    const u32 r = a.work[k];
    Hdr h = c.hdr[r];
    if (h_deleted(h.flags)) return;
    u32* l = c.lits + h.start;
    const u32 v0 = ABS(l[0]);  // names the formula if the clause empties
    // satisfied?
    for (u32 i = 0; i < h.size; i++) {
        if (lit_value(c, l[i]) == 1) {
            c.hdr[r].flags = (h.flags & ~3u) | ST_DELETED;
            return;
        }
    }
    u32 n = 0, sig = 0;
    for (u32 i = 0; i < h.size; i++) {
        const u32 lit = l[i];
        if (lit_value(c, lit) == 0) continue;
        l[n++] = lit;
        sig |= MAPHASH(lit);
    }
    h.size = n;
    h.sig = sig;
    c.hdr[r] = h;
    if (n == 0) {
        set_unsat(c, v0);
        // in a batch the other formulas go on: keep no empty live clause around
        if (c.var_fid) c.hdr[r].flags = (h.flags & ~3u) | ST_DELETED;
        return;
    }
    if (n == 1) {
        const u32 u = l[0];
        const u32 old = atom_cas(&c.asg[ABS(u)], 0u, u);
        if (old == 0) {
            const u32 pos = atom_add(c.ntrail, 1u);
            c.trail[pos] = u;
        } else if (old != u) {
            set_unsat(c, ABS(u));
        }
    }
}

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
