// DIMACS CNF reader (host code): ParaFROST's parser, src/cpu/dimacs.cpp:25-176.
//
// The file is read whole; "c" lines are comments, "p cnf V C" is the header, and
// every clause is a run of non-zero integers ended by 0. Each clause is normalised
// as the reference's toClause() does: a repeated literal is dropped, a clause with
// a literal and its negation (a tautology) is dropped, and a literal whose variable
// exceeds V is an error. Unlike the reference, which also applies the units read so
// far while parsing, every clause is kept as written (one-literal clauses included:
// the upload puts them on the trail and the round propagates them first), and an
// empty clause is reported as a contradiction instead of being dropped.
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

namespace sigma {

struct DimacsFormula {
    uint32_t num_vars = 0;
    std::vector<uint32_t> lits;      // 2v + sign
    std::vector<uint64_t> offsets{0};
    bool empty_clause = false;       // the file holds an empty clause
};

// Parses path into f; returns "" or the error text.
inline std::string dimacs_read(const char* path, DimacsFormula& f) {
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return std::string("cannot open ") + path;
    std::vector<char> buf;
    {
        char chunk[1 << 16];
        size_t n;
        while ((n = std::fread(chunk, 1, sizeof chunk, fp)) > 0) buf.insert(buf.end(), chunk, chunk + n);
        std::fclose(fp);
    }
    buf.push_back('\0');
    const char* p = buf.data();
    const char* end = p + buf.size() - 1;
    bool header = false;
    uint64_t declared = 0;
    std::vector<uint32_t> clause;
    std::vector<int8_t> mark;  // per variable: 0 unseen, 1 positive, -1 negative in this clause
    auto skip_line = [&]() {
        while (p < end && *p != '\n') p++;
    };
    while (p < end) {
        const char ch = *p;
        if (ch == ' ' || ch == '\t' || ch == '\r' || ch == '\n') {
            p++;
            continue;
        }
        if (ch == 'c' || ch == '%') {
            skip_line();
            continue;
        }
        if (ch == 'p') {
            if (header) return "second header";
            unsigned long long v = 0, c = 0;
            if (std::sscanf(p, "p cnf %llu %llu", &v, &c) != 2) return "malformed header";
            if (v == 0 || v >= (1ull << 30)) return "number of variables in the header out of range";
            f.num_vars = (uint32_t)v;
            declared = c;
            mark.assign(f.num_vars + 1, 0);
            header = true;
            skip_line();
            continue;
        }
        if (!header) return "clause before the header";
        // one integer
        bool neg = false;
        if (*p == '-') {
            neg = true;
            p++;
        }
        if (p >= end || *p < '0' || *p > '9') return "unexpected character";
        uint64_t v = 0;
        while (p < end && *p >= '0' && *p <= '9') {
            v = v * 10 + (uint64_t)(*p - '0');
            if (v > f.num_vars) return "literal of a variable above the header's count";
            p++;
        }
        if (v == 0) {
            // end of clause: drop tautologies, keep the rest
            bool taut = false;
            for (uint32_t lit : clause) {
                const uint32_t x = lit >> 1;
                if (mark[x] == 2) taut = true;
            }
            for (uint32_t lit : clause) mark[lit >> 1] = 0;
            if (!taut) {
                if (clause.empty()) f.empty_clause = true;
                else {
                    f.lits.insert(f.lits.end(), clause.begin(), clause.end());
                    f.offsets.push_back(f.lits.size());
                }
            }
            clause.clear();
            continue;
        }
        const uint32_t x = (uint32_t)v;
        const int8_t s = neg ? -1 : 1;
        if (mark[x] == 0) {
            mark[x] = s;
            clause.push_back(2u * x + (neg ? 1u : 0u));
        } else if (mark[x] != s && mark[x] != 2) {
            mark[x] = 2;  // both signs: a tautology
        }
    }
    if (!clause.empty()) return "last clause not ended by 0";
    if (!header) return "no header";
    (void)declared;  // the reference warns on a count mismatch; the clauses read are what counts
    return "";
}

}  // namespace sigma
