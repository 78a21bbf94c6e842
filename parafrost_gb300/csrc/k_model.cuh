// Model extension on the device: MODEL::extend (src/cpu/model.cpp:104-138).
//
// The witness stack holds records [witness, other literals..., length]. Walking the
// stack from its end, a record whose other literals are all false under the current
// values sets its witness true. Each record may read values that the records after
// it set, so one formula's walk is one dependent chain; the formulas of a batch are
// walked side by side, one thread per formula.
#pragma once

#include "cnf.cuh"

namespace sigma {

struct ExtendArgs {
    const u32* resolved;  // witness stack (the store's numbering)
    uint8_t* value;       // per variable of the store: 1 true, 0 false
    u64 nres;             // single formula: stack length
    // formula batches: records in formula order (stack order inside a formula)
    const u32* rec_start;  // stack position of every record's witness
    const u64* rec_words;  // words of every record (its literals and the length word)
    const u32* order;      // records sorted by formula
    const u32* f_first;    // nf + 1: formula f owns order[f_first[f] .. f_first[f+1])
    u32* err;
};

HD bool ext_true(const uint8_t* value, u32 lit) { return value[ABS(lit)] == (SIGN(lit) ? 0 : 1); }

// One record: literals resolved[st .. st+len), the witness first.
HD void ext_record(const ExtendArgs& a, u64 st, u32 len) {
    for (u32 j = len - 1; j >= 1; j--)
        if (ext_true(a.value, a.resolved[st + j])) return;
    const u32 w = a.resolved[st];
    a.value[ABS(w)] = SIGN(w) ? 0 : 1;
}

// The single formula: records from the end of the stack, found by their length words.
HD void k_extend_single(const ExtendArgs& a) {
    u64 x = a.nres;
    while (x) {
        const u32 len = a.resolved[x - 1];
        if (len == 0 || len > x - 1) {  // malformed stack
            atom_or(a.err, ERR_INTERNAL);
            return;
        }
        const u64 st = x - 1 - len;
        ext_record(a, st, len);
        x = st;
    }
}

// Formula f of a batch: its records from the last to the first.
HD void k_extend_formula(const ExtendArgs& a, u32 f) {
    for (u32 i = a.f_first[f + 1]; i-- > a.f_first[f];) {
        const u32 r = a.order[i];
        ext_record(a, a.rec_start[r], (u32)a.rec_words[r] - 1u);
    }
}

// Values before the walk: eliminated variables start false (the solver never
// assigns them; MODEL::extend starts them at 0), the round's units hold.
HD void k_extend_clear(const Ctx& c, uint8_t* value, u32 v) {
    if (c.vstate[v]) value[v] = 0;
}
HD void k_extend_unit(const Ctx& c, uint8_t* value, u32 i) {
    const u32 u = c.trail[i];
    value[ABS(u)] = SIGN(u) ? 0 : 1;
}

// Batch values between the caller's layout (formula after formula, num_vars[f] + 1
// entries each, the first unused) and the store's numbering.
struct ExtendMap {
    const u64* p_first;  // nf + 1: first packed position of every formula
    const u32* f_var;    // nf + 1: variable offset of every formula in the store
    u32 nf;
};
HD void k_extend_in(const ExtendMap& m, const uint8_t* packed, uint8_t* value, u32 p) {
    const u32 f = upper_segment(m.p_first, m.nf, (u64)p);
    const u32 local = (u32)(p - m.p_first[f]);
    if (local) value[m.f_var[f] + local] = packed[p] ? 1 : 0;
}
HD void k_extend_out(const ExtendMap& m, const uint8_t* value, uint8_t* packed, u32 p) {
    const u32 f = upper_segment(m.p_first, m.nf, (u64)p);
    const u32 local = (u32)(p - m.p_first[f]);
    if (local) packed[p] = value[m.f_var[f] + local];  // the unused first entry keeps the caller's value
}

}  // namespace sigma
