// Header-only C++ host mirror of ParaFROST's simplifier entry points over the C ABI
// of sigma_gb300.h. A solver keeps its own CDCL state and hands the round to the GPU:
//
//   pfrost_gb300::Sigma sigma(opts);                 // optSimp()        (src/gpu/simplify.cu:254-270)
//   sigma.awaken(maxVar, lits, offsets, learnt);     // awaken/extract   (src/cpu/simplify.cpp:95-155)
//   int st = sigma.sigmify();                        // sigmifying loop  (src/cpu/simplify.cpp:157-209)
//   sigma.result(out);                               // cacheCNF/units/resolved (src/gpu/transfer.cu:68-165)
//
// Errors throw pfrost_gb300::Error carrying the pf_status; a proved contradiction
// is returned as PF_UNSAT (the reference's learnEmpty + killSolver path).
#pragma once

#include "sigma_gb300.h"

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace pfrost_gb300 {

struct Error : std::runtime_error {
    pf_status status;
    Error(pf_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(pf_status s) {
    if (s != PF_OK && s != PF_UNSAT) throw Error(s, pf_last_error());
}

struct Simplified {
    std::vector<uint32_t> lits;      // surviving clauses, clause-store order
    std::vector<uint64_t> offsets;   // num_clauses + 1
    std::vector<uint8_t> learnt;     // per clause
    std::vector<uint32_t> units;     // assigned literals (the trail)
    std::vector<uint32_t> resolved;  // witness stack, MODEL::resolved format
    std::vector<uint8_t> eliminated; // per variable, index 0 unused
};

class Sigma {
public:
    explicit Sigma(const pf_options* opts = nullptr) {
        pf_options o;
        if (opts) o = *opts;
        else pf_default_options(&o);
        pf_derive_options(&o);
        check(pf_sigma_create(&o, &ctx_));
    }
    ~Sigma() { pf_sigma_destroy(ctx_); }
    Sigma(const Sigma&) = delete;
    Sigma& operator=(const Sigma&) = delete;

    void awaken(uint32_t max_var, const uint32_t* lits, const uint64_t* offsets, uint64_t num_clauses,
                const uint8_t* learnt = nullptr) {
        check(pf_sigma_upload(ctx_, max_var, lits, offsets, num_clauses, learnt));
        max_var_ = max_var;
    }
    int sigmify(pf_round_stats* stats = nullptr) {
        pf_round_stats s;
        const pf_status st = pf_sigma_round(ctx_, &s);
        check(st);
        if (stats) *stats = s;
        return st;
    }
    void result(Simplified& out) {
        uint64_t nc = 0, nl = 0, nu = 0, nr = 0;
        check(pf_sigma_result_sizes(ctx_, &nc, &nl, &nu, &nr));
        out.lits.resize(nl);
        out.offsets.resize(nc + 1);
        out.learnt.resize(nc);
        out.units.resize(nu);
        out.resolved.resize(nr);
        out.eliminated.resize(max_var_ + 1);
        check(pf_sigma_download(ctx_, out.lits.data(), out.offsets.data(), out.learnt.data(), out.units.data(),
                                out.resolved.data(), out.eliminated.data()));
    }
    pf_sigma_ctx* handle() const { return ctx_; }

private:
    pf_sigma_ctx* ctx_ = nullptr;
    uint32_t max_var_ = 0;
};

}  // namespace pfrost_gb300
