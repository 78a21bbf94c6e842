/*
 * Reference harness: drives the UNMODIFIED reference ParaFROST CPU simplifier
 * (compiled from its own sources by oracle/ref.mk) through one sigmify round and
 * records its state after every stage. Test infrastructure only.
 *
 * The round replays ParaFROST::sigmifying() (src/cpu/simplify.cpp:157-232) step
 * by step through the solver's own member functions, so every decision is taken
 * by reference code; the harness only adds snapshots between the steps and a
 * wall-clock timer around the phase loop (src/cpu/simplify.cpp:182-209).
 *
 * usage: sigma_ref <cnf.dimacs> <dump.bin> <level> [--learnt-tail=N] [reference options...]
 *   with the reference options -proof --proofout=<file>, the reference writes its
 *   binary DRAT proof; the dump then records how many lines precede the round.
 *   level 0: input + final state + timing; 1: + per-phase summaries; 2: + every stage.
 *   --learnt-tail=N: the last N parsed clauses become learnt clauses before the
 *   round (an inprocessing call's input: awaken() extracts the original clauses,
 *   then the learnt ones, src/cpu/simplify.cpp:147-148).
 */
#include "solve.h"
#include "dump.h"

#include <chrono>
#include <cstdlib>
#include <cstring>
#include <unordered_map>

bool quiet_en = true;
bool competition_en = false;
int verbose = 0;

using namespace pFROST;
using sigdump::Writer;

static Writer g_dump;
static bool g_round_done = false;

static void on_exit_hook() {
    // killSolver() exits the process when the simplifier proves UNSAT.
    if (!g_round_done) g_dump.rec(sigdump::K_STATUS, 0, sigdump::S_FINAL, {1u});
    g_dump.close();
}

struct Harness : public ParaFROST {
    int level = 0;
    uint32_t learnt_tail = 0;
    explicit Harness(const string& path) : ParaFROST(path) {}

    std::unordered_map<const SCLAUSE*, uint32_t> index_of() {
        std::unordered_map<const SCLAUSE*, uint32_t> m;
        m.reserve(scnf.size() * 2 + 1);
        for (uint32_t i = 0; i < scnf.size(); i++) m[scnf[i]] = i;
        return m;
    }
    void dump_cnf(uint32_t ph, uint32_t st) {
        std::vector<uint32_t> d;
        d.push_back((uint32_t)scnf.size());
        for (uint32_t i = 0; i < scnf.size(); i++) {
            SCLAUSE& c = *scnf[i];
            d.push_back(sigdump::clause_flags((uint32_t)c.status(), c.molten(), c.added()));
            d.push_back(c.sig());
            d.push_back((uint32_t)c.size());
            for (int k = 0; k < c.size(); k++) d.push_back(c[k]);
        }
        g_dump.rec(sigdump::K_CNF, ph, st, d);
    }
    void dump_trail(uint32_t ph, uint32_t st) {
        std::vector<uint32_t> d(trail.data(), trail.data() + trail.size());
        g_dump.rec(sigdump::K_TRAIL, ph, st, d);
    }
    void dump_resolved(uint32_t ph, uint32_t st) {
        std::vector<uint32_t> d(model.resolved.data(), model.resolved.data() + model.resolved.size());
        g_dump.rec(sigdump::K_RESOLVED, ph, st, d);
    }
    void dump_elim(uint32_t ph, uint32_t st) {
        std::vector<uint32_t> d;
        for (uint32_t v = 1; v <= inf.maxVar; v++)
            if (MELTED(sp->vstate[v].state)) d.push_back(v);
        g_dump.rec(sigdump::K_ELIM, ph, st, d);
    }
    void dump_otsizes(uint32_t ph, uint32_t st) {
        std::vector<uint32_t> d(inf.nDualVars, 0);
        for (uint32_t l = 2; l < inf.nDualVars && l < ot.size(); l++) d[l] = (uint32_t)ot[l].size();
        g_dump.rec(sigdump::K_OTSIZE, ph, st, d);
    }
    void dump_lcve(uint32_t ph) {
        // scores live in sp->tmpstack until depFreeze reuses it as the frozen stack;
        // recompute them from occurs exactly as write_scores does (histogram.h:32-41).
        std::vector<uint32_t> s(inf.maxVar + 1, 0);
        for (uint32_t v = 1; v <= inf.maxVar; v++) s[v] = occurs[v].ps * occurs[v].ns;
        g_dump.rec(sigdump::K_SCORES, ph, sigdump::S_LCVE, s);
        std::vector<uint32_t> e(eligible.data(), eligible.data() + eligible.size());
        g_dump.rec(sigdump::K_ELIGIBLE, ph, sigdump::S_LCVE, e);
    }
    void dump_pvs(uint32_t ph, uint32_t st) {
        std::vector<uint32_t> d(PVs.data(), PVs.data() + PVs.size());
        g_dump.rec(sigdump::K_PVS, ph, st, d);
    }
    void dump_pvlists(uint32_t ph, uint32_t st) {
        auto idx = index_of();
        std::vector<uint32_t> d;
        for (uint32_t i = 0; i < PVs.size(); i++) {
            const uint32_t p = V2L(PVs[i]);
            for (uint32_t l = p; l <= p + 1; l++) {
                OL& ol = ot[l];
                d.push_back((uint32_t)ol.size());
                for (int k = 0; k < ol.size(); k++) d.push_back(idx[ol[k]]);
            }
        }
        g_dump.rec(sigdump::K_PVLISTS, ph, st, d);
    }
    void dump_counts(uint32_t ph, uint32_t st) {
        g_dump.rec(sigdump::K_COUNTS, ph, st, {(uint32_t)inf.n_cls_after, (uint32_t)inf.n_lits_after});
    }
    void stage(uint32_t ph, uint32_t st) {
        if (level < 2) return;
        dump_cnf(ph, st);
        dump_trail(ph, st);
        if (st >= sigdump::S_VE) dump_resolved(ph, st);
    }

    // ParaFROST::sigmifying() (src/cpu/simplify.cpp:157-232) up to the write-back.
    void round() {
        // with -proof, the lines written so far (the parser's) are not the round's
        if (opts.proof_en) g_dump.rec(sigdump::K_PROOFMARK, 0, sigdump::S_INPUT, {(uint32_t)proof.numClauses()});
        rootify();
        shrinkTop(false);
        if (orgs.empty()) {
            g_dump.rec(sigdump::K_STATUS, 0, sigdump::S_FINAL, {2u});
            g_round_done = true;
            return;
        }
        if (learnt_tail) {
            // the last clauses of orgs move to the learnt list, marked learnt as the
            // CDCL loop marks the clauses it learns (src/cpu/clause.h:151)
            const uint32_t n = learnt_tail < orgs.size() ? learnt_tail : (uint32_t)orgs.size();
            const uint32_t first = (uint32_t)orgs.size() - n;
            for (uint32_t i = first; i < orgs.size(); i++) {
                cm[orgs[i]].markLearnt();
                learnts.push(orgs[i]);
            }
            orgs.resize(first);
        }
        awaken();
        dump_cnf(0, sigdump::S_INPUT);
        dump_trail(0, sigdump::S_INPUT);
        auto t0 = std::chrono::steady_clock::now();
        int64 litsbefore = inf.nLiterals, diff = INT64_MAX;
        while (litsbefore) {
            resizeCNF();
            createOT();
            if (!prop()) killSolver();
            if (level >= 2) { dump_otsizes(phase, sigdump::S_PROP); stage(phase, sigdump::S_PROP); }
            if (!LCVE()) break;
            if (level >= 2) dump_lcve(phase);
            if (level >= 1) dump_pvs(phase, sigdump::S_LCVE);
            sortOT();
            if (level >= 2) dump_pvlists(phase, sigdump::S_SORT);
            if (stop(diff)) {
                ERE();
                stage(phase, sigdump::S_ERE);
                break;
            }
            SUB();
            stage(phase, sigdump::S_SUB);
            VE();
            stage(phase, sigdump::S_VE);
            BCE();
            stage(phase, sigdump::S_BCE);
            countAll(), filterPVs();
            if (level >= 1) { dump_counts(phase, sigdump::S_BCE); dump_elim(phase, sigdump::S_BCE); }
            inf.nClauses = inf.n_cls_after, inf.nLiterals = inf.n_lits_after;
            diff = litsbefore - inf.nLiterals, litsbefore = inf.nLiterals;
            phase++, mu_inc++;
            mu_inc += phase == opts.phases;
        }
        if (!prop()) killSolver();
        occurs.clear(true), ot.clear(true);
        countFinal();
        shrinkSimp();
        auto t1 = std::chrono::steady_clock::now();
        g_round_done = true;
        const uint64_t us = (uint64_t)std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count();
        dump_cnf(phase, sigdump::S_FINAL);
        dump_trail(phase, sigdump::S_FINAL);
        dump_resolved(phase, sigdump::S_FINAL);
        dump_elim(phase, sigdump::S_FINAL);
        dump_counts(phase, sigdump::S_FINAL);
        g_dump.rec(sigdump::K_TIMING, 0, sigdump::S_FINAL, {(uint32_t)(us & 0xffffffffu), (uint32_t)(us >> 32)});
        g_dump.rec(sigdump::K_STATUS, 0, sigdump::S_FINAL, {0u});
    }
};

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s <cnf> <dump> <level> [options]\n", argv[0]);
        return 2;
    }
    if (!g_dump.open(argv[2])) { std::perror("dump"); return 2; }
    std::atexit(on_exit_hook);
    const int level = std::atoi(argv[3]);
    // parseArguments() reads options from argv[2..]; hand it the formula plus the
    // reference options only.
    std::vector<char*> args;
    args.push_back(argv[0]);
    args.push_back(argv[1]);
    uint32_t learnt_tail = 0;
    for (int i = 4; i < argc; i++) {
        if (!std::strncmp(argv[i], "--learnt-tail=", 14)) learnt_tail = (uint32_t)std::strtoul(argv[i] + 14, nullptr, 10);
        else args.push_back(argv[i]);
    }
    int n = (int)args.size();
    parseArguments(n, args.data());
    Harness* h = new Harness(argv[1]);
    pfrost = h;
    h->level = level;
    h->learnt_tail = learnt_tail;
    h->round();
    return 0;
}
