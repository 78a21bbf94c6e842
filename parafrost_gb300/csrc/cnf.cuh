// Device data model of one resident formula (the reference's SCNF / OT / VARS,
// src/gpu/simptypes.cuh:78-318, sclause.h:37-186; CPU twin src/cpu/sclause.h:29-161).
//
// Clause store (SCNF): clause id = position in clause-store order. Each clause has
// a 16-byte header {start, size, sig, flags} (one 128-bit load) and its literals at
// lits[start .. start+size), sorted ascending. flags: bits 0-1 status
// (0 original, 1 learnt, 2 deleted), bit 2 molten, bit 3 added.
//
// Occurrence table (OT): CSR. List of literal l occupies
// ot_refs[ot_off[l] .. ot_off[l] + ot_size[l]) (capacity up to ot_off[l+1]); entries
// are clause ids. Lists are built in arbitrary order; the lists of elected
// variables are put into the reference's order by the sort stage, and every scan
// of another list that the reference stops at its "first match" looks for the
// smallest matching clause id instead (the reference's lists of non-elected
// literals are in clause-store order).
#pragma once

#include "device.cuh"

namespace sigma {

// Literal helpers (src/cpu/const.h:72-80).
HD u32 ABS(u32 x) { return x >> 1; }
HD u32 V2L(u32 v) { return v << 1; }
HD u32 NEG(u32 x) { return x | 1u; }
HD u32 FLIP(u32 x) { return x ^ 1u; }
HD u32 SIGN(u32 x) { return x & 1u; }
HD u32 MAPHASH(u32 x) { return 1u << (x & 31u); }

enum : u32 { ST_ORIGINAL = 0, ST_LEARNT = 1, ST_DELETED = 2, F_MOLTEN = 4, F_ADDED = 8 };

struct __align__(16) Hdr {
    u32 start, size, sig, flags;
};

HD bool h_original(u32 f) { return (f & 3u) == ST_ORIGINAL; }
HD bool h_learnt(u32 f) { return (f & ST_LEARNT) != 0; }
HD bool h_deleted(u32 f) { return (f & ST_DELETED) != 0; }
HD bool h_molten(u32 f) { return (f & F_MOLTEN) != 0; }

// Values: asg[v] = the literal of v that is true, 0 when v is unassigned.
enum : int { VAL_UNDEF = -1 };

// Pointer view of one context, passed by value to every kernel.
struct Ctx {
    u32 nvars;     // variables 1..nvars
    u32 D;         // literal slots: 2*(nvars+1)
    // clause store
    Hdr* hdr;
    u32* lits;
    u32 ncls;      // clauses in the store (ids 0..ncls-1)
    u32 cap_cls;   // header capacity
    u64 nlits_used;
    u64 cap_lits;
    // occurrence table
    u32* ot_off;   // D+1
    u32* ot_size;  // D
    u32* ot_refs;
    u32* ot_cursor;  // D, scatter cursors
    u32 ot_cap;      // capacity of ot_refs
    // variables
    u32* asg;      // nvars+1
    uint8_t* vstate;  // nvars+1, 1 = eliminated
    u32* ps;       // occurrences of +v in live clauses (occurs[v].ps)
    u32* ns;       // occurrences of -v
    u32* pvrank;   // nvars+1: rank in the elected list, or NONE
    // trail and witness stack
    u32* trail;
    u32* ntrail;   // device counter
    u32* resolved;
    u64* nresolved;  // device counter
    u64 cap_resolved;
    // error word
    u32* err;
    // formula batches (null for a single formula): formula of each variable, and
    // one error word per formula (an empty clause ends that formula only)
    const u32* var_fid;
    u32* f_err;
    uint8_t* res_mark;  // batches: 1 on the last word (the length) of every witness record
    // per clause: the phase stamp of its last change of literals or status
    // (deletion and creation included), and this phase's stamp
    u32* cstamp;
    u32 stamp;
    // DRAT proof lines of the round (null when no proof is recorded): words
    // [n, lit_0 .. lit_{n-1}] per added clause, appended at a device counter
    u32* proof;
    u64* nproof;
    u64 cap_proof;
};

constexpr u32 NONE = 0xFFFFFFFFu;

// Clause r's literals or status changed in this phase.
// One line of the proof: an added clause (the reference's proof.addResolvent /
// addUnit, src/cpu/proof.cpp:181-228, for a strengthened, substituted or resolved
// clause or a unit) or, with del, a deleted one (proof.deleteClause, proof.cpp:
// 193, through removeClause, src/cpu/sclause.cpp:67-84). Header word: the size,
// with bit 31 set for a deletion.
constexpr u32 PROOF_DELETE = 0x80000000u;
HD void proof_line(const Ctx& c, const u32* lits, u32 n, bool del = false) {
    if (!c.proof) return;
    const u64 pos = atom_add64(c.nproof, (u64)n + 1);
    if (pos + n + 1 > c.cap_proof) {
        atom_or(c.err, ERR_CAP_SCRATCH);  // the proof buffer was sized too small
        return;
    }
    c.proof[pos] = n | (del ? PROOF_DELETE : 0u);
    for (u32 i = 0; i < n; i++) c.proof[pos + 1 + i] = lits[i];
}
// removeClause's proof line for live clause r (subsumed, or made redundant by ERE).
HD void proof_delete(const Ctx& c, u32 r) {
    if (!c.proof) return;
    const Hdr h = c.hdr[r];
    proof_line(c, c.lits + h.start, h.size, true);
}

HD void touch(const Ctx& c, u32 r) {
    if (c.cstamp) c.cstamp[r] = c.stamp;
}

HD int lit_value(const Ctx& c, u32 lit) {
    const u32 a = vload(&c.asg[ABS(lit)]);
    if (!a) return VAL_UNDEF;
    return a == lit ? 1 : 0;
}

HD void set_err(const Ctx& c, u32 bits) { atom_or(c.err, bits); }

// The formula holding variable v derived the empty clause.
HD void set_unsat(const Ctx& c, u32 v) {
    if (c.var_fid) atom_or(&c.f_err[c.var_fid[v]], ERR_UNSAT);
    else set_err(c, ERR_UNSAT);
}
HD u32 fid_of(const Ctx& c, u32 v) { return c.var_fid ? c.var_fid[v] : 0u; }

// A unit found inside the round goes to the trail unless its variable is already
// assigned; the opposite assignment is a conflict (enqueueUnit / learnEmpty paths of
// bve.cpp:200-211, equivalence.h:56-80). The variable is claimed with a
// compare-and-swap.
HD void claim_unit(const Ctx& c, u32 u) {
    const u32 old = atom_cas(&c.asg[ABS(u)], 0u, u);
    if (old == 0) {
        c.trail[atom_add(c.ntrail, 1u)] = u;
        proof_line(c, &u, 1);  // learnUnit's proof.addUnit (src/cpu/solve.h:475-479)
    } else if (old != u) {
        set_unsat(c, ABS(u));
    }
}

// Header load through the read-only path (for launches that write no header).
HD Hdr hdr_ro(const Hdr* p) {
#if defined(__CUDA_ARCH__)
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(p));
    Hdr h;
    h.start = v.x;
    h.size = v.y;
    h.sig = v.z;
    h.flags = v.w;
    return h;
#else
    return *p;
#endif
}
HD const u32* clause_lits(const Ctx& c, const Hdr& h) { return c.lits + h.start; }

// Signature of a literal array.
HD u32 calc_sig(const u32* l, u32 n) {
    u32 s = 0;
    for (u32 i = 0; i < n; i++) s |= MAPHASH(l[i]);
    return s;
}

}  // namespace sigma
