/*
 * ORACLE — test infrastructure, never part of the product.
 *
 * CPU restatement of one ParaFROST SIGmA round (the CPU simplifier,
 * src/cpu/simplify.cpp:157-232 and the files it calls), used to check the
 * GB300 kernels bit for bit and as the CPU baseline ("port") on hosts where
 * the reference itself is not compiled. Every function cites the reference
 * lines it follows. It is pinned against the compiled reference (oracle/_ref,
 * built by oracle/ref.mk) through the golden fixtures in tests/golden/.
 *
 * Written in C++ because the reference's occurrence-list sort is libstdc++'s
 * std::sort (src/cpu/sort.h:98-109): calling the same library routine keeps
 * the order of equal-key clauses identical to the reference's.
 *
 * Clause references are indices into an arena that never moves; the clause
 * store order (scnf) is a vector of those indices, as in the reference where
 * S_REF is a pointer (src/cpu/sclause.h:161, simptypes.h:28-30).
 */
#include "../include/sigma_gb300.h"
#include "dump.h"

#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

typedef uint32_t u32;
typedef int64_t i64;

// Literal helpers (src/cpu/const.h:72-80).
inline u32 ABS(u32 x) { return x >> 1; }
inline u32 V2L(u32 v) { return v << 1; }
inline u32 NEG(u32 x) { return x | 1u; }
inline u32 FLIP(u32 x) { return x ^ 1u; }
inline u32 SIGN(u32 x) { return x & 1u; }
inline u32 MAPHASH(u32 x) { return 1u << (x & 31u); }

enum : uint8_t { ST_ORIGINAL = 0, ST_LEARNT = 1, ST_DELETED = 2 };
enum : int8_t { V_UNDEF = -1 };

// SCLAUSE (src/cpu/sclause.h:29-160): status, molten, added flags, signature, literals.
struct Clause {
    uint8_t st = ST_ORIGINAL;
    bool molten = false, added = false;
    u32 sig = 0;
    std::vector<u32> lits;
    int size() const { return (int)lits.size(); }
    bool original() const { return st == ST_ORIGINAL; }
    bool learnt() const { return (st & ST_LEARNT) != 0; }
    bool deleted() const { return (st & ST_DELETED) != 0; }
    void calcSig() { sig = 0; for (u32 l : lits) sig |= MAPHASH(l); }
    // SCLAUSE::has (sclause.h:126-145): membership in a sorted clause.
    bool has(u32 lit) const { return std::binary_search(lits.begin(), lits.end(), lit); }
};

typedef std::vector<u32> OL;  // occurrence list of clause indices

struct Unsat {};  // learnEmpty() + killSolver() in the reference

struct Round {
    pf_options opts;
    u32 maxVar = 0;
    std::vector<Clause> arena;
    std::vector<u32> scnf;
    std::vector<OL> ot;
    std::vector<int8_t> value;    // per literal: 1 true, 0 false, -1 unassigned
    std::vector<uint8_t> vstate;  // per var: 1 = eliminated (MELTED_M)
    std::vector<uint8_t> frozen;
    std::vector<u32> trail;
    size_t propagated = 0;
    std::vector<u32> resolved;    // MODEL::resolved
    std::vector<u32> PVs, eligible;
    std::vector<u32> ps, ns;      // occurs[v].ps / .ns
    std::vector<u32> scores;
    u32 mu_inc = 0;
    int phase = 0;
    i64 nClauses = 0, nLiterals = 0, n_cls_after = 0, n_lits_after = 0;
    sigdump::Writer dump;
    int level = 0;

    Clause& C(u32 r) { return arena[r]; }

    // ---------------------------------------------------------------- dumps
    std::vector<u32> index_of() {
        std::vector<u32> idx(arena.size(), UINT32_MAX);
        for (u32 i = 0; i < scnf.size(); i++) idx[scnf[i]] = i;
        return idx;
    }
    void dump_cnf(u32 ph, u32 st) {
        std::vector<u32> d;
        d.push_back((u32)scnf.size());
        for (u32 r : scnf) {
            Clause& c = C(r);
            d.push_back(sigdump::clause_flags(c.st, c.molten, c.added));
            d.push_back(c.sig);
            d.push_back((u32)c.size());
            d.insert(d.end(), c.lits.begin(), c.lits.end());
        }
        dump.rec(sigdump::K_CNF, ph, st, d);
    }
    void dump_trail(u32 ph, u32 st) { dump.rec(sigdump::K_TRAIL, ph, st, trail); }
    void dump_resolved(u32 ph, u32 st) { dump.rec(sigdump::K_RESOLVED, ph, st, resolved); }
    void dump_elim(u32 ph, u32 st) {
        std::vector<u32> d;
        for (u32 v = 1; v <= maxVar; v++) if (vstate[v]) d.push_back(v);
        dump.rec(sigdump::K_ELIM, ph, st, d);
    }
    void dump_otsizes(u32 ph, u32 st) {
        std::vector<u32> d(V2L(maxVar + 1), 0);
        for (u32 l = 2; l < d.size(); l++) d[l] = (u32)ot[l].size();
        dump.rec(sigdump::K_OTSIZE, ph, st, d);
    }
    void dump_pvlists(u32 ph, u32 st) {
        std::vector<u32> idx = index_of(), d;
        for (u32 v : PVs) {
            for (u32 l = V2L(v); l <= V2L(v) + 1; l++) {
                d.push_back((u32)ot[l].size());
                for (u32 r : ot[l]) d.push_back(idx[r]);
            }
        }
        dump.rec(sigdump::K_PVLISTS, ph, st, d);
    }
    void stage(u32 ph, u32 st) {
        if (level < 2) return;
        dump_cnf(ph, st);
        dump_trail(ph, st);
        if (st >= sigdump::S_VE) dump_resolved(ph, st);
    }

    // ---------------------------------------------------------------- solver state
    // ParaFROST::enqueueUnit (src/cpu/solve.h:430-445), root level only.
    void enqueueUnit(u32 lit) {
        value[lit] = 1;
        value[FLIP(lit)] = 0;
        trail.push_back(lit);
    }
    bool unassigned(u32 lit) const { return value[lit] == V_UNDEF; }

    // MODEL::saveWitness / saveClause (src/cpu/model.cpp:334-379); vorg is the identity
    // before any variable mapping (solve.h:234-240).
    void saveWitness(u32 w) { resolved.push_back(w); resolved.push_back(1); }
    void saveClause(const Clause& c, u32 witlit) {
        const size_t last = resolved.size();
        int pos = -1;
        for (int i = 0; i < c.size(); i++) {
            resolved.push_back(c.lits[i]);
            if (c.lits[i] == witlit) pos = i;
        }
        if (pos > 0) std::swap(resolved[last + pos], resolved[last]);
        resolved.push_back((u32)c.size());
    }

    // ---------------------------------------------------------------- extract / OT
    // ParaFROST::extract (src/cpu/simplify.cpp:95-113). A one-literal clause is a unit
    // the reference's parser puts on the trail (src/cpu/dimacs.cpp:153-159): it is
    // enqueued (the opposite literal already there: UNSAT) and kept as a deleted slot.
    bool input_unsat = false;
    void extract(const u32* lits, const uint64_t* off, uint64_t n, const uint8_t* learnt) {
        arena.reserve(n + n / 4);
        scnf.reserve(n + n / 4);
        for (uint64_t i = 0; i < n; i++) {
            Clause c;
            c.st = (learnt && learnt[i]) ? ST_LEARNT : ST_ORIGINAL;
            c.lits.assign(lits + off[i], lits + off[i + 1]);
            c.calcSig();
            std::sort(c.lits.begin(), c.lits.end());
            if (c.size() == 1) {
                const u32 u = c.lits[0];
                if (unassigned(u)) enqueueUnit(u);
                else if (value[u] == 0) input_unsat = true;
                c.st = ST_DELETED;
            } else {
                nLiterals += c.size();
                nClauses++;
            }
            scnf.push_back((u32)arena.size());
            arena.push_back(std::move(c));
        }
    }

    // rootify() + shrinkTop() at the start of sigmifying() (src/cpu/simplify.cpp:163-164,
    // shrink.cpp:152-216): the input units propagated at the root, satisfied clauses
    // dropped and false literals removed before the first occurrence table. Here the
    // same fixpoint by prop() over a table of the input, then shrinkSimp(). Returns
    // false when no clause is left (the reference then skips the round).
    bool rootUnits() {
        if (input_unsat) throw Unsat();
        if (propagated >= trail.size()) return true;
        createOT();
        prop();
        shrinkSimp();
        countAll();
        nClauses = n_cls_after;
        nLiterals = n_lits_after;
        return !scnf.empty();
    }

    // ParaFROST::createOT (simplify.cpp:35-56).
    void createOT() {
        for (u32 v = 1; v <= maxVar; v++) { ot[V2L(v)].clear(); ot[NEG(V2L(v))].clear(); }
        for (u32 r : scnf) {
            const Clause& c = C(r);
            if (c.learnt() || c.original())
                for (u32 l : c.lits) ot[l].push_back(r);
        }
    }

    // toblivion(OL&) (simplify.h:297-303).
    void toblivion(OL& list) {
        for (u32 r : list) C(r).st = ST_DELETED;
        list.clear();
        list.shrink_to_fit();
    }

    // ParaFROST::reduceOL / reduceOT (simplify.cpp:58-79).
    void reduceOT() {
        for (u32 l = 2; l < V2L(maxVar + 1); l++) {
            OL& ol = ot[l];
            size_t j = 0;
            for (size_t i = 0; i < ol.size(); i++) if (!C(ol[i]).deleted()) ol[j++] = ol[i];
            ol.resize(j);
        }
    }

    // ParaFROST::shrinkSimp (simplify.cpp:234-245).
    void shrinkSimp() {
        size_t j = 0;
        for (size_t i = 0; i < scnf.size(); i++) {
            if (C(scnf[i]).deleted()) { C(scnf[i]).lits.clear(); C(scnf[i]).lits.shrink_to_fit(); }
            else scnf[j++] = scnf[i];
        }
        scnf.resize(j);
    }

    // resizeCNF (src/cpu/solve.h:684-688).
    void resizeCNF() {
        const int times = phase + 1;
        if (opts.gc_freq > 0 && times > 1 && times != opts.phases && (times % opts.gc_freq) == 0) shrinkSimp();
    }

    // ---------------------------------------------------------------- prop
    // ParaFROST::propClause (src/cpu/elimination.cpp:41-62).
    bool propClause(u32 lit, Clause& c) {
        u32 sig = 0;
        size_t j = 0;
        for (size_t i = 0; i < c.lits.size(); i++) {
            const u32 other = c.lits[i];
            if (other != lit) {
                if (value[other] > 0) return true;
                c.lits[j++] = other;
                sig |= MAPHASH(other);
            }
        }
        c.sig = sig;
        c.lits.pop_back();
        return false;
    }

    // ParaFROST::prop (src/cpu/elimination.cpp:64-99).
    void prop() {
        const size_t before = propagated;
        while (propagated < trail.size()) {
            const u32 assign = trail[propagated++], f_assign = FLIP(assign);
            OL& fl = ot[f_assign];
            for (size_t i = 0; i < fl.size(); i++) {
                Clause& c = C(fl[i]);
                if (c.deleted()) continue;
                if (propClause(f_assign, c)) c.st = ST_DELETED;
                else {
                    const int size = c.size();
                    if (!size) throw Unsat();
                    if (size == 1) {
                        const u32 unit = c.lits[0];
                        if (unassigned(unit)) enqueueUnit(unit);
                        else throw Unsat();
                    }
                }
            }
            fl.clear();
            fl.shrink_to_fit();
            toblivion(ot[assign]);
        }
        if (propagated != before && !opts.sub) reduceOT();
    }

    // ---------------------------------------------------------------- LCVE
    // histSimp (src/cpu/histogram.cpp:82-96) + write_scores (histogram.h:32-41) + the
    // LCV order (lcve.cpp:34 with key.h:57-66,203-209: score ascending, variable ascending).
    void varReorder() {
        std::fill(ps.begin(), ps.end(), 0);
        std::fill(ns.begin(), ns.end(), 0);
        for (u32 r : scnf) {
            const Clause& c = C(r);
            if (c.deleted()) continue;
            for (u32 l : c.lits) { if (SIGN(l)) ns[ABS(l)]++; else ps[ABS(l)]++; }
        }
        eligible.resize(maxVar);
        for (u32 v = 1; v <= maxVar; v++) { eligible[v - 1] = v; scores[v] = ps[v] * ns[v]; }
        // rSort (sort.h:123-133): insertion sort / std::sort with LCV_CMP, or a stable LSD
        // radix on the score over the ascending initial order; all three give this order.
        std::stable_sort(eligible.begin(), eligible.end(), [&](u32 a, u32 b) { return scores[a] < scores[b]; });
    }

    // ParaFROST::depFreeze (src/cpu/lcve.cpp:83-100).
    void depFreeze(const OL& ol, u32 cand, u32 pt, u32 nt) {
        for (u32 r : ol) {
            const Clause& c = C(r);
            if (c.deleted()) continue;
            for (u32 l : c.lits) {
                const u32 v = ABS(l);
                if (!frozen[v] && v != cand && (ps[v] < pt || ns[v] < nt)) frozen[v] = 1;
            }
        }
    }

    // ParaFROST::LCVE (src/cpu/lcve.cpp:46-81).
    bool LCVE() {
        varReorder();
        PVs.clear();
        const u32 pt = (u32)opts.mu_pos << mu_inc, nt = (u32)opts.mu_neg << mu_inc;
        for (u32 i = 0; i < eligible.size(); i++) {
            const u32 cand = eligible[i];
            if (vstate[cand]) continue;
            if (frozen[cand]) continue;
            const u32 p = V2L(cand), n = NEG(p);
            const u32 psz = (u32)ot[p].size(), nsz = (u32)ot[n].size();
            if (ps[cand] == 0 && ns[cand] == 0) continue;
            if (psz >= pt && nsz >= nt) break;
            PVs.push_back(cand);
            depFreeze(ot[p], cand, pt, nt);
            depFreeze(ot[n], cand, pt, nt);
        }
        std::fill(frozen.begin(), frozen.end(), 0);
        const bool go = PVs.size() >= (size_t)opts.lcve_min;
        // the reference harness records the order only for an election that goes on
        if (go && level >= 2) {
            dump.rec(sigdump::K_SCORES, phase, sigdump::S_LCVE, scores);
            dump.rec(sigdump::K_ELIGIBLE, phase, sigdump::S_LCVE, eligible);
        }
        return go;
    }

    // ---------------------------------------------------------------- sortOT
    // CNF_CMP_KEY (src/cpu/simplify.h:29-42).
    struct KeyCmp {
        Round* R;
        bool operator()(u32 a, u32 b) const {
            const Clause& x = R->C(a);
            const Clause& y = R->C(b);
            if (x.size() != y.size()) return x.size() < y.size();
            if (x.lits[0] != y.lits[0]) return x.lits[0] < y.lits[0];
            if (x.lits.back() != y.lits.back()) return x.lits.back() < y.lits.back();
            return x.sig < y.sig;
        }
    };
    // Sort(Vec, CMP) (src/cpu/sort.h:97-109): insertion sort up to 20 entries, else std::sort.
    void sortList(OL& ol) {
        KeyCmp cmp{this};
        const size_t sz = ol.size();
        if (sz <= 20) {
            // insertionSort (sort.h:43-57)
            if (sz == 2 && cmp(ol[1], ol[0])) std::swap(ol[0], ol[1]);
            else if (sz > 2) {
                for (size_t i = 1; i < sz; i++) {
                    u32 tmp = ol[i];
                    size_t j = i;
                    for (; j > 0 && cmp(tmp, ol[j - 1]); j--) ol[j] = ol[j - 1];
                    ol[j] = tmp;
                }
            }
        } else {
            std::sort(ol.begin(), ol.end(), cmp);
        }
    }
    // ParaFROST::sortOT (simplify.cpp:81-93).
    void sortOT() {
        for (u32 v : PVs) {
            OL& poss = ot[V2L(v)];
            OL& negs = ot[NEG(V2L(v))];
            if (poss.size() > 1) sortList(poss);
            if (negs.size() > 1) sortList(negs);
        }
    }

    // ---------------------------------------------------------------- SUB
    // sub / selfsub signature filters (src/cpu/simplify.h:84-90).
    static bool subSig(u32 A, u32 B) { return !(A & ~B); }
    static bool selfsubSig(u32 A, u32 B) {
        const u32 Bt = B | ((B & 0xAAAAAAAAu) >> 1) | ((B & 0x55555555u) << 1);
        return !(A & ~Bt);
    }
    // sub(SCLAUSE&, SCLAUSE&) (src/cpu/subsume.h:39-56).
    static bool subClause(const Clause& sm, const Clause& lr) {
        int it1 = 0, it2 = 0, s = 0;
        const int n1 = sm.size(), n2 = lr.size();
        while (it1 < n1 && it2 < n2) {
            const u32 a = sm.lits[it1], b = lr.lits[it2];
            if (a < b) it1++;
            else if (b < a) it2++;
            else { s++; it1++; it2++; }
        }
        return s == n1;
    }
    // selfsub(x, fx, sm, lr) (src/cpu/subsume.h:75-103).
    static bool selfsubClause(u32 x, u32 fx, const Clause& sm, const Clause& lr) {
        int it1 = 0, it2 = 0, s = 0;
        const int n1 = sm.size(), n2 = lr.size();
        bool self = false;
        while (it1 < n1 && it2 < n2) {
            const u32 a = sm.lits[it1], b = lr.lits[it2];
            if (a == fx) it1++;
            else if (b == x) { self = true; it2++; }
            else if (a < b) it1++;
            else if (b < a) it2++;
            else { s++; it1++; it2++; }
        }
        if (s + 1 == n1) {
            if (self) return true;
            while (it2 < n2) { if (lr.lits[it2] == x) return true; it2++; }
        }
        return false;
    }
    // ParaFROST::strengthen (src/cpu/elimination.cpp:199-234); learnt-clause LBD bumping
    // (bumpShrunken) only feeds the CDCL search and is not restated.
    void strengthen(Clause& c, u32 me) {
        u32 sig = 0;
        size_t n = 0;
        for (size_t k = 0; k < c.lits.size(); k++) {
            const u32 lit = c.lits[k];
            if (lit != me) { c.lits[n++] = lit; sig |= MAPHASH(lit); }
        }
        c.sig = sig;
        c.lits.pop_back();
        if (n == 1) {
            const u32 unit = c.lits[0];
            if (unassigned(unit)) { enqueueUnit(unit); toblivion(ot[unit]); }
            else if (value[unit] == 0) throw Unsat();
        }
    }
    // subsume(list, end, cand) (src/cpu/subsume.h:105-121).
    bool subsume(OL& list, size_t end, Clause& cand) {
        const int candsz = cand.size();
        for (size_t j = 0; j < end; j++) {
            Clause& s = C(list[j]);
            if (s.deleted()) continue;
            if (cand.molten && s.size() > candsz) continue;
            if (s.size() > 1 && subSig(s.sig, cand.sig) && subClause(s, cand)) {
                if (s.learnt() && cand.original()) s.st = ST_ORIGINAL;
                cand.st = ST_DELETED;  // removeClause (src/cpu/sclause.cpp:77-84)
                return true;
            }
        }
        return false;
    }
    // selfsubsume (src/cpu/subsume.h:123-142).
    bool selfsubsume(u32 x, u32 fx, OL& list, Clause& cand) {
        const int candsz = cand.size();
        const u32 candsig = cand.sig;
        for (size_t j = 0; j < list.size(); j++) {
            Clause& s = C(list[j]);
            const int subsize = s.size();
            if (subsize > candsz) break;
            if (s.deleted()) continue;
            if (subsize > 1 && selfsubSig(s.sig, candsig) && selfsubClause(x, fx, s, cand)) {
                strengthen(cand, x);
                cand.molten = true;
                return true;
            }
        }
        return false;
    }
    // updateOL (src/cpu/subsume.h:27-37).
    void updateOL(OL& ol) {
        size_t j = 0;
        for (size_t i = 0; i < ol.size(); i++) {
            Clause& c = C(ol[i]);
            if (c.molten) c.molten = false;
            else if (!c.deleted()) ol[j++] = ol[i];
        }
        ol.resize(j);
    }
    // self_sub_x (src/cpu/subsume.h:144-179).
    void self_sub_x(u32 p) {
        const u32 n = NEG(p);
        OL& poss = ot[p];
        OL& negs = ot[n];
        for (size_t i = 0; i < poss.size(); i++) {
            Clause& pos = C(poss[i]);
            if (pos.size() > 1000) break;  // HSE_MAX_CL_SIZE
            if (pos.deleted()) continue;
            selfsubsume(p, n, negs, pos);
            subsume(poss, i, pos);
        }
        updateOL(poss);
        for (size_t i = 0; i < negs.size(); i++) {
            Clause& neg = C(negs[i]);
            if (neg.size() > 1000) break;
            if (neg.deleted()) continue;
            selfsubsume(n, p, poss, neg);
            subsume(negs, i, neg);
        }
        updateOL(negs);
    }
    // ParaFROST::SUB (src/cpu/elimination.cpp:110-129).
    void SUB() {
        if (!(opts.sub || opts.ve_plus)) return;
        for (u32 v : PVs) {
            const u32 p = V2L(v), n = NEG(p);
            if (ot[p].size() <= (size_t)opts.sub_max && ot[n].size() <= (size_t)opts.sub_max) self_sub_x(p);
        }
    }

    // ---------------------------------------------------------------- VE helpers
    // merge(x, c1, c2, out) (src/cpu/simplify.h:139-173).
    static bool merge(u32 x, const Clause& c1, const Clause& c2, std::vector<u32>& out) {
        out.clear();
        const int n1 = c1.size(), n2 = c2.size();
        int it1 = 0, it2 = 0;
        while (it1 < n1 && it2 < n2) {
            const u32 l1 = c1.lits[it1], l2 = c2.lits[it2];
            const u32 v1 = ABS(l1), v2 = ABS(l2);
            if (v1 == x) it1++;
            else if (v2 == x) it2++;
            else if ((l1 ^ l2) == 1u) return false;
            else if (v1 < v2) { it1++; out.push_back(l1); }
            else if (v2 < v1) { it2++; out.push_back(l2); }
            else { it1++; it2++; out.push_back(l1); }
        }
        while (it1 < n1) { const u32 l = c1.lits[it1++]; if (ABS(l) != x) out.push_back(l); }
        while (it2 < n2) { const u32 l = c2.lits[it2++]; if (ABS(l) != x) out.push_back(l); }
        return true;
    }
    // merge(x, c1, c2) -> resolvent size or 0 for a tautology (simplify.h:175-202).
    static int mergeSize(u32 x, const Clause& c1, const Clause& c2) {
        const int n1 = c1.size(), n2 = c2.size();
        int it1 = 0, it2 = 0, len = n1 + n2 - 2;
        while (it1 < n1 && it2 < n2) {
            const u32 l1 = c1.lits[it1], l2 = c2.lits[it2];
            const u32 v1 = ABS(l1), v2 = ABS(l2);
            if (v1 == x) it1++;
            else if (v2 == x) it2++;
            else if ((l1 ^ l2) == 1u) return 0;
            else if (v1 < v2) it1++;
            else if (v2 < v1) it2++;
            else { it1++; it2++; len--; }
        }
        return len;
    }
    // isTautology (simplify.h:119-137).
    static bool isTautology(u32 x, const Clause& c1, const Clause& c2) {
        const int n1 = c1.size(), n2 = c2.size();
        int it1 = 0, it2 = 0;
        while (it1 < n1 && it2 < n2) {
            const u32 l1 = c1.lits[it1], l2 = c2.lits[it2];
            const u32 v1 = ABS(l1), v2 = ABS(l2);
            if (v1 == x) it1++;
            else if (v2 == x) it2++;
            else if ((l1 ^ l2) == 1u) return true;
            else if (v1 < v2) it1++;
            else if (v2 < v1) it2++;
            else { it1++; it2++; }
        }
        return false;
    }
    int countOrgs(const OL& l) { int n = 0; for (u32 r : l) if (C(r).original()) n++; return n; }
    int countLitsBefore(const OL& l) { int n = 0; for (u32 r : l) if (C(r).original()) n += C(r).size(); return n; }

    // countSubstituted / countResolvents (simplify.h:237-295); molten-aware when gate is set.
    bool countAdded(u32 x, int clsbefore, const OL& me, const OL& other, int& nAddedCls, bool gate) {
        int nAddedLits = 0;
        const int rlimit = opts.ve_clause_max;
        for (u32 ri : me) {
            const Clause& ci = C(ri);
            if (!ci.original()) continue;
            for (u32 rj : other) {
                const Clause& cj = C(rj);
                if (!cj.original()) continue;
                if (gate && ci.molten == cj.molten) continue;
                int rsize;
                if ((rsize = mergeSize(x, ci, cj)) > 1) {
                    if (++nAddedCls > clsbefore || (rlimit && rsize > rlimit)) return true;
                    nAddedLits += rsize;
                }
            }
        }
        if (opts.ve_lbound) {
            if (nAddedLits > countLitsBefore(me) + countLitsBefore(other)) return true;
        }
        return false;
    }

    void freezeBinaries(OL& l) { for (u32 r : l) { Clause& c = C(r); if (c.original() && c.size() == 2) c.molten = false; } }

    // toblivion(p, pOrgs, nOrgs, poss, negs, model) (simplify.h:305-332).
    void toblivionVar(u32 p, int pOrgs, int nOrgs) {
        const u32 n = NEG(p);
        OL& poss = ot[p];
        OL& negs = ot[n];
        if (pOrgs > nOrgs) {
            for (u32 r : negs) { Clause& c = C(r); if (c.original()) saveClause(c, n); c.st = ST_DELETED; }
            saveWitness(p);
            negs.clear(); negs.shrink_to_fit();
            toblivion(poss);
        } else {
            for (u32 r : poss) { Clause& c = C(r); if (c.original()) saveClause(c, p); c.st = ST_DELETED; }
            saveWitness(n);
            poss.clear(); poss.shrink_to_fit();
            toblivion(negs);
        }
    }

    // ---------------------------------------------------------------- EQU gate
    // find_sfanin (src/cpu/equivalence.h:88-106).
    u32 find_sfanin(u32 gate_out, OL& list) {
        u32 imp = 0;
        int nImps = 0;
        for (u32 r : list) {
            Clause& c = C(r);
            if (c.original() && c.size() == 2) {
                imp = FLIP(c.lits[0] ^ c.lits[1] ^ gate_out);
                c.molten = true;
                nImps++;
            }
            if (nImps > 1) return 0;
        }
        return imp;
    }
    // find_BN_gate (equivalence.h:108-130).
    u32 find_BN_gate(u32 p) {
        const u32 n = NEG(p);
        OL& poss = ot[p];
        OL& negs = ot[n];
        u32 first = find_sfanin(p, poss);
        if (first) {
            u32 second = n, def = first;
            if (second < first) { first = second; second = def; }
            for (u32 r : negs) {
                Clause& c = C(r);
                if (c.original() && c.size() == 2 && c.lits[0] == first && c.lits[1] == second) {
                    c.molten = true;
                    return def;
                }
            }
        }
        freezeBinaries(poss);
        return 0;
    }
    // save_BN_gate (equivalence.h:132-153).
    void save_BN_gate(u32 p, int pOrgs, int nOrgs) {
        const u32 n = NEG(p);
        if (pOrgs > nOrgs) {
            for (u32 r : ot[n]) if (C(r).original()) saveClause(C(r), n);
            saveWitness(p);
        } else {
            for (u32 r : ot[p]) if (C(r).original()) saveClause(C(r), p);
            saveWitness(n);
        }
    }
    // substitute_single(dx, org, def) (equivalence.h:24-42): returns a unit or 0.
    u32 substituteClause(u32 dx, Clause& org, u32 def) {
        size_t n = 0;
        for (size_t i = 0; i < org.lits.size(); i++) {
            const u32 lit = org.lits[i];
            if (lit == dx) org.lits[n++] = def;
            else if (lit != def) org.lits[n++] = lit;
        }
        org.lits.resize(n);
        if (org.size() == 1) return org.lits[0];
        // Sort(data, size, LESS) (sort.h:59-69): plain ascending order of distinct literals.
        std::sort(org.lits.begin(), org.lits.end());
        org.calcSig();
        return 0;
    }
    // substitute_single(p, def, ot) (equivalence.h:44-86); true = contradiction.
    bool substitute_single(u32 p, u32 def) {
        const u32 n = NEG(p), def_f = FLIP(def);
        OL& poss = ot[p];
        OL& negs = ot[n];
        for (u32 r : negs) {
            Clause& neg = C(r);
            if (neg.learnt() || neg.molten || neg.has(def)) neg.st = ST_DELETED;
            else if (neg.original()) {
                const u32 unit = substituteClause(n, neg, def_f);
                if (unit) {
                    if (unassigned(unit)) enqueueUnit(unit);
                    else if (value[unit] == 0) return true;
                }
            }
        }
        for (u32 r : poss) {
            Clause& pos = C(r);
            if (pos.learnt() || pos.molten || pos.has(def_f)) pos.st = ST_DELETED;
            else if (pos.original()) {
                const u32 unit = substituteClause(p, pos, def);
                if (unit) {
                    if (unassigned(unit)) enqueueUnit(unit);
                    else if (value[unit] == 0) return true;
                }
            }
        }
        return false;
    }

    // ---------------------------------------------------------------- AND/OR gate
    // find_fanin (src/cpu/and.h:25-41).
    void find_fanin(u32 gate_out, OL& list, std::vector<u32>& out_c, u32& sig) {
        out_c.clear();
        sig = 0;
        for (u32 r : list) {
            Clause& c = C(r);
            if (c.original() && c.size() == 2) {
                const u32 imp = FLIP(c.lits[0] ^ c.lits[1] ^ gate_out);
                out_c.push_back(imp);
                sig |= MAPHASH(imp);
                c.molten = true;
            }
        }
    }
    // find_AO_gate (and.h:43-86).
    bool find_AO_gate(u32 dx, int nOrgCls, std::vector<u32>& out_c, int& nAddedCls) {
        out_c.clear();
        u32 sig;
        const u32 x = ABS(dx);
        OL& itarget = ot[dx];
        find_fanin(dx, itarget, out_c, sig);
        if (out_c.size() > 1) {
            const u32 f_dx = FLIP(dx);
            out_c.push_back(f_dx);
            sig |= MAPHASH(f_dx);
            std::sort(out_c.begin(), out_c.end());
            OL& otarget = ot[f_dx];
            for (u32 r : otarget) {
                Clause& c = C(r);
                if (c.original() && (size_t)c.size() == out_c.size() && subSig(c.sig, sig) && c.lits == out_c) {
                    c.molten = true;
                    nAddedCls = 0;
                    if (countAdded(x, nOrgCls, itarget, otarget, nAddedCls, true)) {
                        c.molten = false;
                        break;
                    }
                    return true;
                }
            }
        }
        freezeBinaries(itarget);
        return false;
    }

    // ---------------------------------------------------------------- ITE gate
    // fast_equality_check (src/cpu/ifthenelse.h:25-40).
    u32 fast_equality_check(u32 x, u32 y, u32 z) {
        if (ot[y].size() > ot[z].size()) std::swap(y, z);
        if (ot[x].size() > ot[y].size()) std::swap(x, y);
        OL& list = ot[x];
        // sort3 (simplify.h:105-117)
        auto cswap = [](u32& a, u32& b) { const u32 lo = std::min(a, b), hi = std::max(a, b); a = lo; b = hi; };
        cswap(y, z); cswap(x, z); cswap(x, y);
        for (u32 r : list) {
            Clause& c = C(r);
            if (c.molten) continue;
            if (c.original() && c.size() == 3 && c.lits[0] == x && c.lits[1] == y && c.lits[2] == z) return r;
        }
        return UINT32_MAX;
    }
    // find_ITE_gate (ifthenelse.h:42-97).
    bool find_ITE_gate(u32 dx, int nOrgCls, int& nAddedCls) {
        const u32 fx = FLIP(dx);
        OL& itarget = ot[dx];
        const size_t sz = itarget.size();
        for (size_t i = 0; i < sz; i++) {
            Clause& ci = C(itarget[i]);
            if (!(ci.original() && ci.size() == 3)) continue;
            u32 xi = ci.lits[0], yi = ci.lits[1], zi = ci.lits[2];
            if (yi == dx) std::swap(xi, yi);
            if (zi == dx) std::swap(xi, zi);
            for (size_t j = i + 1; j < sz; j++) {
                Clause& cj = C(itarget[j]);
                if (!(cj.original() && cj.size() == 3)) continue;
                u32 xj = cj.lits[0], yj = cj.lits[1], zj = cj.lits[2];
                if (yj == dx) std::swap(xj, yj);
                if (zj == dx) std::swap(xj, zj);
                if (ABS(yi) == ABS(zj)) std::swap(yj, zj);
                if (ABS(zi) == ABS(zj)) continue;
                if (yi != FLIP(yj)) continue;
                const u32 d1 = fast_equality_check(fx, yi, FLIP(zi));
                if (d1 == UINT32_MAX) continue;
                const u32 d2 = fast_equality_check(fx, yj, FLIP(zj));
                if (d2 == UINT32_MAX) continue;
                ci.molten = cj.molten = C(d1).molten = C(d2).molten = true;
                OL& otarget = ot[fx];
                nAddedCls = 0;
                if (countAdded(ABS(dx), nOrgCls, itarget, otarget, nAddedCls, true)) {
                    ci.molten = cj.molten = C(d1).molten = C(d2).molten = false;
                    return false;
                }
                return true;
            }
        }
        return false;
    }

    // ---------------------------------------------------------------- XOR gate
    // freezeArities (src/cpu/xor.h:13-25).
    void freezeArities(OL& me, OL& other) {
        for (u32 r : me) { Clause& c = C(r); if (c.size() > 2 && c.molten) c.molten = false; }
        for (u32 r : other) { Clause& c = C(r); if (c.size() > 2 && c.molten) c.molten = false; }
    }
    // checkArity (xor.h:35-50).
    static bool checkArity(const Clause& c, const std::vector<u32>& lits) {
        for (u32 lit : c.lits)
            if (std::find(lits.begin(), lits.end(), lit) == lits.end()) return false;
        return true;
    }
    // makeArity (xor.h:52-84) with COUNTFLIPS (xor.h:23-27).
    bool makeArity(u32& parity, std::vector<u32>& lits) {
        const int size = (int)lits.size();
        const u32 oldparity = parity;
        while (__builtin_parity(++parity)) {}
        for (int k = 0; k < size; k++) {
            const u32 bit = 1u << k;
            if ((parity & bit) != (oldparity & bit)) lits[k] = FLIP(lits[k]);
        }
        u32 best = lits[0];
        size_t minsize = ot[best].size();
        for (int k = 1; k < size; k++) {
            const size_t lsize = ot[lits[k]].size();
            if (lsize < minsize) { minsize = lsize; best = lits[k]; }
        }
        for (u32 r : ot[best]) {
            Clause& c = C(r);
            if (c.original() && c.size() == size && checkArity(c, lits)) {
                c.molten = true;
                return true;
            }
        }
        return false;
    }
    // find_XOR_gate (xor.h:86-131).
    bool find_XOR_gate(u32 dx, int nOrgCls, std::vector<u32>& out_c, int& nAddedCls) {
        const u32 fx = FLIP(dx), v = ABS(dx);
        OL& itarget = ot[dx];
        OL& otarget = ot[fx];
        for (size_t i = 0; i < itarget.size(); i++) {
            Clause& ci = C(itarget[i]);
            if (!ci.original()) continue;
            const int size = ci.size();
            const int arity = size - 1;
            if (size < 3 || arity > opts.xor_max_arity) continue;
            out_c = ci.lits;  // copyClause
            u32 parity = 0;
            int itargets = 1 << arity;
            while (--itargets && makeArity(parity, out_c)) {}
            if (itargets) freezeArities(itarget, otarget);
            else {
                ci.molten = true;
                nAddedCls = 0;
                if (countAdded(v, nOrgCls, itarget, otarget, nAddedCls, true)) {
                    freezeArities(itarget, otarget);
                    break;
                }
                return true;
            }
        }
        return false;
    }

    // ---------------------------------------------------------------- resolvents
    // ParaFROST::newResolvent (src/cpu/bve.cpp:188-220).
    void newResolvent(const std::vector<u32>& res) {
        if (res.size() == 1) {
            const u32 unit = res[0];
            if (unassigned(unit)) enqueueUnit(unit);
            else if (value[unit] == 0) throw Unsat();
            return;
        }
        Clause c;
        c.lits = res;
        c.calcSig();
        c.added = true;
        scnf.push_back((u32)arena.size());
        arena.push_back(std::move(c));
    }
    // xsubstitute / xresolve (bve.cpp:144-186): "me" is the shorter list, positive on ties.
    void addResolvents(u32 x, std::vector<u32>& out_c, bool gate) {
        u32 dx = V2L(x), fx = NEG(dx);
        if (ot[dx].size() > ot[fx].size()) std::swap(dx, fx);
        // arena may grow inside the loop: index by reference number, never keep Clause&.
        const OL& me = ot[dx];
        const OL& other = ot[fx];
        for (u32 ri : me) {
            if (!C(ri).original()) continue;
            const bool a = C(ri).molten;
            for (u32 rj : other) {
                if (!C(rj).original()) continue;
                if (gate && a == C(rj).molten) continue;
                if (merge(x, C(ri), C(rj), out_c)) newResolvent(out_c);
            }
        }
    }

    // ParaFROST::bve (src/cpu/bve.cpp:28-142).
    void bve() {
        std::vector<u32> out_c;
        for (size_t i = 0; i < PVs.size(); i++) {
            u32 v = PVs[i];
            const u32 p = V2L(v), n = NEG(p);
            const int pOrgs = countOrgs(ot[p]), nOrgs = countOrgs(ot[n]);
            if (!pOrgs || !nOrgs) {
                toblivionVar(p, pOrgs, nOrgs);
                v = 0;
            } else if (u32 def = find_BN_gate(p)) {
                save_BN_gate(p, pOrgs, nOrgs);
                if (substitute_single(p, def)) throw Unsat();
                v = 0;
            } else {
                out_c.clear();
                const int nOrgCls = pOrgs + nOrgs;
                int nAddedCls = 0;
                int type = 0;  // 1 = RESOLUTION, 2 = SUBSTITUTION (simplify.h:25-27)
                if (nOrgCls > 2) {
                    if (find_AO_gate(n, nOrgCls, out_c, nAddedCls)) type = 2;
                    else if (!nAddedCls && find_AO_gate(p, nOrgCls, out_c, nAddedCls)) type = 2;
                }
                if (!type && nOrgCls > 3) {
                    if (find_ITE_gate(p, nOrgCls, nAddedCls)) type = 2;
                    else if (!nAddedCls && find_ITE_gate(n, nOrgCls, nAddedCls)) type = 2;
                    else if (find_XOR_gate(p, nOrgCls, out_c, nAddedCls)) type = 2;
                    else if (!nAddedCls && find_XOR_gate(n, nOrgCls, out_c, nAddedCls)) type = 2;
                }
                if (!type && !nAddedCls && !countAdded(v, nOrgCls, ot[p], ot[n], nAddedCls, false)) type = 1;
                if (type) {
                    if (nAddedCls) addResolvents(v, out_c, type == 2);
                    toblivionVar(p, pOrgs, nOrgs);
                    v = 0;
                }
            }
            if (!v) {
                vstate[PVs[i]] = 1;  // markEliminated (solve.h:535-541)
                PVs[i] = 0;
            }
        }
    }

    void VE() { if (opts.ve) bve(); }

    // ---------------------------------------------------------------- BCE
    // ParaFROST::BCE (src/cpu/elimination.cpp:131-167).
    void BCE() {
        if (!opts.bce) return;
        for (u32 v : PVs) {
            if (!v) continue;
            const u32 p = V2L(v), n = NEG(p);
            OL& poss = ot[p];
            OL& negs = ot[n];
            if (poss.size() <= (size_t)opts.bce_max && negs.size() <= (size_t)opts.bce_max) {
                for (u32 rn : negs) {
                    Clause& neg = C(rn);
                    if (!neg.original()) continue;
                    bool allTautology = true;
                    for (u32 rp : poss) {
                        const Clause& pos = C(rp);
                        if (pos.original() && !isTautology(v, neg, pos)) { allTautology = false; break; }
                    }
                    if (allTautology) {
                        saveClause(neg, n);
                        neg.st = ST_DELETED;
                    }
                }
            }
        }
    }

    // ---------------------------------------------------------------- ERE
    // merge_ere (src/cpu/redundancy.h:38-85).
    static bool merge_ere(u32 x, const Clause& c1, const Clause& c2, const Clause& target) {
        const int n1 = c1.size(), n2 = c2.size(), n = target.size();
        int it1 = 0, it2 = 0, it = 0;
        while (it < n && it1 < n1 && it2 < n2) {
            const u32 lit = target.lits[it];
            if (ABS(lit) == x) return false;
            const u32 l1 = c1.lits[it1], l2 = c2.lits[it2];
            const u32 v1 = ABS(l1), v2 = ABS(l2);
            if (v1 == x) it1++;
            else if (v2 == x) it2++;
            else if (v1 < v2) { if (l1 != lit) return false; it1++; it++; }
            else if (v2 < v1) { if (l2 != lit) return false; it2++; it++; }
            else { if (l1 != lit) return false; it1++; it2++; it++; }
        }
        while (it < n && it1 < n1) {
            const u32 l1 = c1.lits[it1];
            if (ABS(l1) != x && l1 != target.lits[it++]) return false;
            it1++;
        }
        while (it < n && it2 < n2) {
            const u32 l2 = c2.lits[it2];
            if (ABS(l2) != x && l2 != target.lits[it++]) return false;
            it2++;
        }
        return true;
    }
    // forward_equ (redundancy.h:87-142).
    void forward_equ(u32 x, const Clause& c1, const Clause& c2) {
        const int n1 = c1.size(), n2 = c2.size();
        int len = n1 + n2 - 2;
        int it1 = 0, it2 = 0;
        size_t minsize = SIZE_MAX;
        u32 msig = 0, best = 0;
        while (it1 < n1 && it2 < n2) {
            const u32 l1 = c1.lits[it1], l2 = c2.lits[it2];
            const u32 v1 = ABS(l1), v2 = ABS(l2);
            if (v1 == x) it1++;
            else if (v2 == x) it2++;
            else if ((l1 ^ l2) == 1u) return;
            else if (v1 < v2) {
                it1++;
                if (ot[l1].size() < minsize) { minsize = ot[l1].size(); best = l1; }
                msig |= MAPHASH(l1);
            } else if (v2 < v1) {
                it2++;
                if (ot[l2].size() < minsize) { minsize = ot[l2].size(); best = l2; }
                msig |= MAPHASH(l2);
            } else {
                it1++; it2++; len--;
                if (ot[l1].size() < minsize) { minsize = ot[l1].size(); best = l1; }
                msig |= MAPHASH(l1);
            }
        }
        const int maxsize = opts.ere_clause_max;
        // The reference indexes ot[0] with an unbounded count when no literal precedes the
        // end of the shorter antecedent (undefined behaviour); such pairs are skipped here.
        if (minsize == SIZE_MAX) return;
        if (len > 1 && (!maxsize || len <= maxsize)) {
            const uint8_t type = (c1.learnt() || c2.learnt()) ? ST_LEARNT : ST_ORIGINAL;
            const OL& minlist = ot[best];
            for (size_t i = 0; i < minsize; i++) {
                Clause& c = C(minlist[i]);
                if (len == c.size() && (c.learnt() || c.st == type) && subSig(msig, c.sig) && merge_ere(x, c1, c2, c)) {
                    c.st = ST_DELETED;  // removeClause
                    break;
                }
            }
        }
    }
    // ParaFROST::ERE (src/cpu/elimination.cpp:169-197).
    void ERE() {
        if (!opts.ere) return;
        for (u32 v : PVs) {
            u32 dx = V2L(v), fx = NEG(dx);
            if (ot[dx].size() > ot[fx].size()) std::swap(dx, fx);
            const OL& me = ot[dx];
            const OL& other = ot[fx];
            if (me.size() <= (size_t)opts.ere_max && other.size() <= (size_t)opts.ere_max) {
                for (u32 ri : me) {
                    if (C(ri).deleted()) continue;
                    for (u32 rj : other) {
                        if (C(rj).deleted()) continue;
                        forward_equ(v, C(ri), C(rj));
                    }
                }
            }
        }
    }

    // ---------------------------------------------------------------- counts
    // countAll (src/cpu/solve.h:724-734).
    void countAll() {
        n_cls_after = n_lits_after = 0;
        for (u32 r : scnf) {
            const Clause& c = C(r);
            if (c.original() || c.learnt()) { n_cls_after++; n_lits_after += c.size(); }
        }
    }
    // filterPVs (solve.h:697-707).
    void filterPVs() {
        size_t n = 0;
        for (u32 x : PVs) if (x && !vstate[x]) PVs[n++] = x;
        PVs.resize(n);
    }
    bool stop(i64 lr) const { return phase == opts.phases || (lr <= opts.ve_phase_min && phase > 2); }

    // ParaFROST::sigmifying (src/cpu/simplify.cpp:182-209), after awaken().
    void run() {
        i64 litsbefore = nLiterals, diff = INT64_MAX;
        while (litsbefore) {
            resizeCNF();
            createOT();
            prop();
            if (level >= 2) { dump_otsizes(phase, sigdump::S_PROP); stage(phase, sigdump::S_PROP); }
            if (!LCVE()) break;
            if (level >= 1) dump.rec(sigdump::K_PVS, phase, sigdump::S_LCVE, PVs);
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
            countAll();
            filterPVs();
            if (level >= 1) {
                dump.rec(sigdump::K_COUNTS, phase, sigdump::S_BCE, {(u32)n_cls_after, (u32)n_lits_after});
                dump_elim(phase, sigdump::S_BCE);
            }
            nClauses = n_cls_after;
            nLiterals = n_lits_after;
            diff = litsbefore - nLiterals;
            litsbefore = nLiterals;
            phase++;
            mu_inc++;
            mu_inc += (phase == opts.phases);
        }
        prop();
        countAll();
        nClauses = n_cls_after;
        nLiterals = n_lits_after;
        shrinkSimp();
    }
};

}  // namespace

extern "C" {

void pf_default_options(pf_options* o) {
    std::memset(o, 0, sizeof(*o));
    o->phases = 5; o->all = 0; o->ve = 1; o->ve_plus = 1; o->sub = 1; o->bce = 0; o->ere = 1;
    o->ve_lbound = 0; o->ve_clause_max = 100; o->ve_phase_min = 500; o->mu_pos = 32; o->mu_neg = 32;
    o->xor_max_arity = 10; o->sub_max = 3000; o->bce_max = 3000; o->ere_max = 3000;
    o->ere_clause_max = 1000; o->lcve_min = 1; o->gc_freq = 2; o->dump_level = 0;
}

// Option derivation (src/cpu/options.cpp:281-311).
void pf_derive_options(pf_options* o) {
    o->ve = (o->ve || o->ve_plus) ? 1 : 0;
    if (o->all) { o->ve = 1; o->ve_plus = 1; o->bce = 1; o->ere = 1; }
    if (!o->phases && (o->ve || o->sub || o->bce)) o->phases = 1;
    if (o->phases && !(o->ve || o->sub || o->bce)) o->phases = 0;
    if (o->phases > 1 && !o->ve) o->phases = 1;
}

/* Runs one round of the restated simplifier. Options must already be derived.
 * Returns 0 (round finished), 1 (UNSAT proved), 2 (formula empty / no round). */
int oracle_sigmify(const pf_options* opts, uint32_t num_vars, const uint32_t* lits, const uint64_t* offsets,
                   uint64_t num_clauses, const uint8_t* learnt, const char* dump_path, int dump_level,
                   double* seconds) {
    Round* R = new Round();
    R->opts = *opts;
    R->maxVar = num_vars;
    R->level = dump_level;
    if (dump_path) R->dump.open(dump_path);
    const u32 D = V2L(num_vars + 1);
    R->ot.assign(D, OL());
    R->value.assign(D, V_UNDEF);
    R->vstate.assign(num_vars + 1, 0);
    R->frozen.assign(num_vars + 1, 0);
    R->ps.assign(num_vars + 1, 0);
    R->ns.assign(num_vars + 1, 0);
    R->scores.assign(num_vars + 1, 0);
    int status = 0;
    if (num_clauses == 0 || (!opts->phases && !(opts->all || opts->ere))) status = 2;
    if (status == 0) {
        R->extract(lits, offsets, num_clauses, learnt);
        R->dump_cnf(0, sigdump::S_INPUT);
        R->dump_trail(0, sigdump::S_INPUT);
        auto t0 = std::chrono::steady_clock::now();
        try {
            // with nothing left after the root propagation the reference skips the
            // round; its state (units, no clause) is the final state dumped here
            if (R->rootUnits()) R->run();
        } catch (Unsat&) {
            status = 1;
        }
        auto t1 = std::chrono::steady_clock::now();
        const double s = std::chrono::duration<double>(t1 - t0).count();
        if (seconds) *seconds = s;
        if (status == 0) {
            R->dump_cnf(R->phase, sigdump::S_FINAL);
            R->dump_trail(R->phase, sigdump::S_FINAL);
            R->dump_resolved(R->phase, sigdump::S_FINAL);
            R->dump_elim(R->phase, sigdump::S_FINAL);
            R->dump.rec(sigdump::K_COUNTS, R->phase, sigdump::S_FINAL, {(u32)R->n_cls_after, (u32)R->n_lits_after});
            const uint64_t us = (uint64_t)(s * 1e6);
            R->dump.rec(sigdump::K_TIMING, 0, sigdump::S_FINAL, {(u32)(us & 0xffffffffu), (u32)(us >> 32)});
        }
    }
    R->dump.rec(sigdump::K_STATUS, 0, sigdump::S_FINAL, {(u32)status});
    R->dump.close();
    delete R;
    return status;
}

}  // extern "C"

// ---------------------------------------------------------------- sort replica check
// Checks the product's replica of libstdc++'s std::sort (parafrost_gb300/csrc/
// introsort.cuh, used on the device for occurrence lists longer than 20) against
// std::sort itself on random keys with many ties: returns the number of trials
// whose permutation differs.
#include "../parafrost_gb300/csrc/introsort.cuh"
#include <random>

extern "C" long oracle_check_introsort(uint64_t seed, int trials) {
    struct E { uint32_t key, id; };
    std::mt19937_64 rng(seed);
    long bad = 0;
    for (int t = 0; t < trials; t++) {
        const int n = (t % 7 == 0) ? (int)(rng() % 3000) : (int)(rng() % 200);
        const uint32_t kmax = 1 + (uint32_t)(rng() % ((t % 3 == 0) ? 3 : 50));
        std::vector<E> a(n);
        for (int i = 0; i < n; i++) a[i] = E{(uint32_t)(rng() % kmax), (uint32_t)i};
        if (t % 11 == 0) std::sort(a.begin(), a.end(), [](E x, E y) { return x.key < y.key; });
        if (t % 13 == 0) std::reverse(a.begin(), a.end());
        std::vector<E> b = a;
        auto cmp = [](const E& x, const E& y) { return x.key < y.key; };
        std::sort(a.begin(), a.end(), cmp);
        sigma::std_sort_replica(b.data(), b.data() + n, cmp);
        for (int i = 0; i < n; i++) if (a[i].id != b[i].id) { bad++; break; }
    }
    return bad;
}

// ---------------------------------------------------------------- model extension
// MODEL::extend (src/cpu/model.cpp:104-138) over a witness stack, then a count of
// the clauses of (lits, offsets) that the extended model falsifies. value[v] is 1
// for true; the stack is walked from its end: a record [first, ..., last, length]
// whose literals after the first are all false sets its first literal true.
extern "C" long oracle_extend_and_check(uint32_t num_vars, uint8_t* value, const uint32_t* resolved, uint64_t nres,
                                        const uint32_t* lits, const uint64_t* offsets, uint64_t num_clauses) {
    auto sat = [&](uint32_t lit) { return value[lit >> 1] == ((lit & 1u) ? 0 : 1); };
    if (nres) {
        uint64_t x = nres - 1;  // the last record's length word
        while (true) {
            const uint64_t k = resolved[x];
            if (k == 0 || k > x) return -1;  // malformed stack
            const uint64_t first = x - k;
            bool unsat = true;
            for (uint64_t j = x - 1; j > first; j--) {
                if (sat(resolved[j])) {
                    unsat = false;
                    break;
                }
            }
            if (unsat) {
                const uint32_t lit = resolved[first];
                if ((lit >> 1) > num_vars) return -1;
                value[lit >> 1] = (lit & 1u) ? 0 : 1;
            }
            if (first == 0) break;
            x = first - 1;
        }
    }
    long bad = 0;
    for (uint64_t c = 0; c < num_clauses; c++) {
        bool ok = false;
        for (uint64_t i = offsets[c]; i < offsets[c + 1] && !ok; i++) ok = sat(lits[i]);
        bad += !ok;
    }
    return bad;
}

// ---------------------------------------------------------------- DRAT check
// A forward checker for the addition lines of a binary DRAT proof (the format of
// src/cpu/proof.cpp:95-135): every added clause must follow by unit propagation
// (RUP) from the input clauses and the clauses added before it. Deletion lines are
// skipped (a round adds none). Watched-literal propagation, root assignments kept.
namespace {
struct RupChecker {
    std::vector<std::vector<u32>> cls;
    std::vector<std::vector<u32>> watch;  // per literal: clause indices watching it
    std::vector<int8_t> val;              // per literal: 1 true, 0 false, -1 unassigned
    std::vector<u32> trail;
    size_t head = 0;
    bool root_conflict = false;

    explicit RupChecker(uint32_t nv) : watch(2 * (size_t)nv + 2), val(2 * (size_t)nv + 2, -1) {}
    bool assign(u32 lit) {
        if (val[lit] == 1) return true;
        if (val[lit] == 0) return false;
        val[lit] = 1;
        val[lit ^ 1u] = 0;
        trail.push_back(lit);
        return true;
    }
    // unit propagation from trail[head]; false on a conflict
    bool propagate() {
        while (head < trail.size()) {
            const u32 f = trail[head++] ^ 1u;  // the literal that became false
            std::vector<u32>& ws = watch[f];
            size_t j = 0;
            bool conflict = false;
            for (size_t i = 0; i < ws.size(); i++) {
                const u32 ci = ws[i];
                if (conflict) { ws[j++] = ci; continue; }
                std::vector<u32>& c = cls[ci];
                if (c[0] == f) std::swap(c[0], c[1]);
                if (val[c[0]] == 1) { ws[j++] = ci; continue; }
                bool moved = false;
                for (size_t k = 2; k < c.size(); k++) {
                    if (val[c[k]] != 0) {
                        std::swap(c[1], c[k]);
                        watch[c[1]].push_back(ci);
                        moved = true;
                        break;
                    }
                }
                if (moved) continue;
                ws[j++] = ci;
                if (val[c[0]] == 0) conflict = true;
                else assign(c[0]);
            }
            ws.resize(j);
            if (conflict) return false;
        }
        return true;
    }
    void add(const std::vector<u32>& lits) {
        if (root_conflict) return;
        if (lits.empty()) { root_conflict = true; return; }
        if (lits.size() == 1) {
            if (!assign(lits[0]) || !propagate()) root_conflict = true;
            return;
        }
        std::vector<u32> c(lits);
        // watch two literals that are not false where possible
        for (size_t k = 0; k < 2; k++)
            for (size_t m = k; m < c.size(); m++)
                if (val[c[m]] != 0) { std::swap(c[k], c[m]); break; }
        const u32 ci = (u32)cls.size();
        cls.push_back(c);
        watch[c[0]].push_back(ci);
        watch[c[1]].push_back(ci);
        if (val[c[0]] == 0) root_conflict = true;  // every literal false at the root
        else if (val[c[1]] == 0 && val[c[0]] != 1) {
            if (!assign(c[0]) || !propagate()) root_conflict = true;
        }
    }
    bool rup(const std::vector<u32>& lits) {
        if (root_conflict) return true;
        const size_t mark = trail.size(), mhead = head;
        bool ok = false;
        for (u32 l : lits) {
            if (val[l] == 1) { ok = true; break; }
            if (val[l] == -1) assign(l ^ 1u);
        }
        if (!ok) ok = !propagate();
        for (size_t i = trail.size(); i-- > mark;) { val[trail[i]] = -1; val[trail[i] ^ 1u] = -1; }
        trail.resize(mark);
        head = mhead;
        return ok;
    }
};
}  // namespace

/* Checks every addition line of a binary DRAT proof by RUP against the formula and
 * the earlier lines. Returns -1 when all hold (sets *empty to 1 when an empty clause
 * is added, i.e. the proof refutes the formula), else the index of the first line
 * that fails; -2 for a malformed proof. */
extern "C" long oracle_check_drat(uint32_t num_vars, const uint32_t* lits, const uint64_t* offsets,
                                  uint64_t num_clauses, const uint8_t* proof, uint64_t nbytes, int* empty) {
    RupChecker ck(num_vars);
    std::vector<u32> c;
    for (uint64_t i = 0; i < num_clauses; i++) {
        c.assign(lits + offsets[i], lits + offsets[i + 1]);
        ck.add(c);
    }
    if (empty) *empty = 0;
    uint64_t p = 0;
    long line = 0;
    while (p < nbytes) {
        const uint8_t tag = proof[p++];
        if (tag != 'a' && tag != 'd') return -2;
        c.clear();
        while (true) {
            if (p >= nbytes) return -2;
            u32 r = 0, shift = 0;
            uint8_t b;
            do {
                if (p >= nbytes || shift > 28) return -2;
                b = proof[p++];
                r |= (u32)(b & 127u) << shift;
                shift += 7;
            } while (b & 128u);
            if (r == 0) break;
            if ((r >> 1) > num_vars || r < 2) return -2;
            c.push_back(r);
        }
        if (tag == 'a') {
            if (!ck.rup(c)) return line;
            if (c.empty() && empty) *empty = 1;
            ck.add(c);
        }
        line++;
    }
    return -1;
}
