/*
 * Round-dump record writer shared by the oracle restatement and the compiled
 * reference harness (test infrastructure only; nothing in the product uses it).
 *
 * A dump is a sequence of records, each five-or-more little-endian uint32 words:
 *     kind, phase, stage, n, data[n]
 * The GPU library writes the same records (see include/sigma_gb300.h, "round
 * dump"), so parity tests compare the three producers record by record.
 */
#ifndef SIGMA_ORACLE_DUMP_H
#define SIGMA_ORACLE_DUMP_H

#include <cstdint>
#include <cstdio>
#include <vector>

namespace sigdump {

enum Kind : uint32_t {
    K_CNF = 1,      // clause snapshot: n_clauses, then per clause: flags, sig, size, lits[size]
    K_OTSIZE = 2,   // occurrence-list sizes, one per literal slot (2V+2)
    K_SCORES = 3,   // scores[0..V]
    K_ELIGIBLE = 4, // eligible order after the LCV sort (V entries)
    K_PVS = 5,      // elected variables in election order
    K_PVLISTS = 6,  // per PV: |pos|, pos clause indices, |neg|, neg clause indices
    K_TRAIL = 7,    // assigned literals (compared as a set)
    K_RESOLVED = 8, // witness stack (model.resolved), exact order
    K_ELIM = 9,     // eliminated variables, ascending
    K_COUNTS = 10,  // n_cls_after, n_lits_after
    K_STATUS = 11,  // 0 = round finished, 1 = UNSAT proved inside the round
    K_TIMING = 12,  // microseconds (not compared)
    K_PROOFMARK = 13,  // proof lines written before the round (reference harness with -proof)
};

enum Stage : uint32_t {
    S_INPUT = 0, S_PROP = 1, S_LCVE = 2, S_SORT = 3, S_SUB = 4, S_VE = 5,
    S_BCE = 6, S_ERE = 7, S_FINAL = 8,
};

// Clause flag word inside a K_CNF record.
inline uint32_t clause_flags(uint32_t status, bool molten, bool added) {
    return (status & 3u) | (molten ? 4u : 0u) | (added ? 8u : 0u);
}

struct Writer {
    FILE* f = nullptr;
    bool open(const char* path) { f = std::fopen(path, "wb"); return f != nullptr; }
    void rec(uint32_t kind, uint32_t phase, uint32_t stage, const std::vector<uint32_t>& d) {
        if (!f) return;
        uint32_t h[4] = {kind, phase, stage, (uint32_t)d.size()};
        std::fwrite(h, 4, 4, f);
        if (!d.empty()) std::fwrite(d.data(), 4, d.size(), f);
        std::fflush(f);
    }
    void close() { if (f) std::fclose(f); f = nullptr; }
};

}  // namespace sigdump

#endif
