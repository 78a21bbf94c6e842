/*
 * Drop-in harness: the UNMODIFIED reference ParaFROST solver (compiled from its own
 * sources by oracle/ref.mk) with its preprocessing sigmify round handed to this
 * repository's C ABI through the C++ mirror include/sigma_gb300.hpp, in place of the
 * round's phase loop inside sigmifying(). Test infrastructure only.
 *
 * sigmify_gb300() is ParaFROST::sigmifying() (src/cpu/simplify.cpp:157-232) with its
 * phase loop (lines 184-197) replaced by pfrost_gb300::Sigma: the solver's own
 * rootify/shrinkTop/awaken build the simplifying CNF, the library runs the round,
 * and the result is written back into the solver (clauses, units, witness stack,
 * eliminated variables) before the reference's own tail runs: countFinal,
 * shrinkSimp, map/newBeginning, rebuildWT, retrail. solve_gb300() is
 * ParaFROST::solve() (src/cpu/solve.cpp:138-158) with that call as its
 * preprocessing step and no in-processing rounds; wrapup() then prints the answer
 * and, with -model -modelverify, extends the model through the witness stack and
 * verifies it on the input file with the reference's own MODEL::verify.
 *
 * usage: sigma_dropin <cnf.dimacs> [reference options...]
 */
#include "solve.h"
#include "sigma_gb300.hpp"

#include <cstdio>
#include <vector>

bool quiet_en = true;
bool competition_en = false;
int verbose = 0;

using namespace pFROST;

struct Dropin : public ParaFROST {
    explicit Dropin(const string& path) : ParaFROST(path) {}

    // The reference's option set, in the library's option struct.
    pf_options library_options() const {
        pf_options o;
        pf_default_options(&o);
        o.phases = opts.phases;
        o.all = opts.all_en;
        o.ve = opts.ve_en;
        o.ve_plus = opts.ve_plus_en;
        o.sub = opts.sub_en;
        o.bce = opts.bce_en;
        o.ere = opts.ere_en;
        o.ve_lbound = opts.ve_lbound_en;
        o.ve_clause_max = opts.ve_clause_limit;
        o.ve_phase_min = (int32_t)opts.lits_min;
        o.mu_pos = (int32_t)opts.mu_pos;
        o.mu_neg = (int32_t)opts.mu_neg;
        o.xor_max_arity = opts.xor_max_arity;
        o.sub_max = opts.sub_limit;
        o.bce_max = opts.bce_limit;
        o.ere_max = opts.ere_limit;
        o.ere_clause_max = opts.ere_max_resolvent;
        o.lcve_min = (int32_t)opts.lcve_min;
        o.gc_freq = opts.shrink_rate;
        return o;
    }

    void sigmify_gb300() {
        rootify();
        shrinkTop(false);
        if (orgs.empty()) {
            recycleWT();
            return;
        }
        awaken();
        if (simpstate == AWAKEN_FAIL) {
            recycle();
            return;
        }
        // the simplifying CNF, flattened (clause-store order: originals, then learnts)
        std::vector<uint32_t> lits;
        std::vector<uint64_t> offs{0};
        std::vector<uint8_t> learnt;
        for (uint32 i = 0; i < scnf.size(); i++) {
            S_REF c = scnf[i];
            for (int k = 0; k < c->size(); k++) lits.push_back((*c)[k]);
            offs.push_back(lits.size());
            learnt.push_back(c->learnt() ? 1 : 0);
        }
        const pf_options o = library_options();
        pfrost_gb300::Sigma sigma(&o);
        sigma.awaken(inf.maxVar, lits.data(), offs.data(), scnf.size(), learnt.data());
        pf_round_stats st;
        const int status = sigma.sigmify(&st);
        std::printf("c sigma_gb300 round: status %d, %llu -> %llu clauses, %d phases, %llu variables eliminated\n",
                    status, (unsigned long long)st.clauses_before, (unsigned long long)st.clauses_after,
                    st.phases_run, (unsigned long long)st.eliminated_vars);
        if (status == PF_UNSAT) {
            learnEmpty();
            killSolver();
        }
        pfrost_gb300::Simplified r;
        sigma.result(r);
        // write-back: the simplified clauses replace the simplifying CNF
        for (uint32 i = 0; i < scnf.size(); i++) scnf[i]->markDeleted();
        shrinkSimp();
        for (size_t i = 0; i + 1 < r.offsets.size(); i++) {
            Lits_t lc;
            for (uint64_t k = r.offsets[i]; k < r.offsets[i + 1]; k++) lc.push(r.lits[k]);
            const size_t bytes = hc_scsize + (lc.size() - 1) * hc_isize;
            S_REF s = (S_REF) new Byte[bytes];
            s->init(lc);
            s->set_status(r.learnt[i] ? LEARNT : ORIGINAL);
            s->calcSig();
            scnf.push(s);
        }
        // units: root-level assignments, already propagated by the round
        for (uint32_t u : r.units)
            if (UNASSIGNED(sp->value[u])) enqueueUnit(u);
        sp->propagated = trail.size();
        // witness stack: records [witness, literals..., length], literals through vorg
        // (MODEL::saveLiteral, src/cpu/model.cpp:273-279)
        std::vector<uint32_t> w(r.resolved);
        for (size_t x = w.size(); x > 0;) {
            const uint32_t len = w[x - 1];
            for (size_t j = x - 1 - len; j < x - 1; j++) w[j] = V2DEC(vorg[ABS(w[j])], SIGN(w[j]));
            x = x - 1 - len;
        }
        for (uint32_t word : w) model.resolved.push(word);
        for (uint32 v = 1; v <= inf.maxVar; v++)
            if (r.eliminated[v] && !sp->vstate[v].state) markEliminated(v);
        // the reference's own tail of sigmifying() (src/cpu/simplify.cpp:203-231)
        occurs.clear(true), ot.clear(true);
        countFinal();
        shrinkSimp();
        if (!inf.unassigned || !inf.nClauses) {
            cnfstate = SAT;
            return;
        }
        if (canMap()) map(true);
        else newBeginning();
        rebuildWT(opts.sigma_priorbins);
        retrail();
    }

    void solve_gb300() {
        timer.start();
        initLimits();
        if (canPreSigmify()) sigmify_gb300();
        if (UNSOLVED(cnfstate)) {
            MDMInit();
            while (UNSOLVED(cnfstate) && !runningout()) {
                if (BCP()) analyze();
                else if (!inf.unassigned) cnfstate = SAT;
                else if (canReduce()) reduce();
                else if (canRestart()) restart();
                else if (canRephase()) rephase();
                else if (canProbe()) probe();
                else if (canMMD()) MDM();
                else decide();
            }
        }
        timer.stop(), timer.solve += timer.cpuTime();
        wrapup();
    }
};

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <cnf> [options]\n", argv[0]);
        return 2;
    }
    parseArguments(argc, argv);
    Dropin* d = new Dropin(argv[1]);
    pfrost = d;
    d->solve_gb300();
    return 0;
}
