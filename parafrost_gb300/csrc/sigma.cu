// sigma_gb300 host driver: one context = one resident formula. Implements the
// C ABI of include/sigma_gb300.h and runs ParaFROST's sigmify round
// (ParaFROST::sigmifying, src/cpu/simplify.cpp:157-232; GPU twin
// src/gpu/simplify.cu:155-234) as a sequence of device stages.
#include "../../include/sigma_gb300.h"

#include "cnf.cuh"
#include "dimacs.h"
#include "k_bce_ere.cuh"
#include "k_bve.cuh"
#include "k_lcve.cuh"
#include "k_model.cuh"
#include "k_otb.cuh"
#include "k_prop.cuh"
#include "k_sortot.cuh"
#include "k_store.cuh"
#include "k_sub.cuh"
#include "k_sub_warp.cuh"
#include "prims.cuh"
#include "runtime.h"

#include <algorithm>
#include <array>
#include <climits>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <vector>

using namespace sigma;

namespace {

thread_local std::string g_last_error;

// ---------------------------------------------------------------- functors
struct FUpload { UploadArgs a; HD void operator()(u32 i) const { k_upload_clause(a, i); } };
struct FHist { Ctx c; HD void operator()(u32 i) const { k_hist_clause(c, i); } };
struct FScatter { Ctx c; HD void operator()(u32 i) const { k_scatter_clause(c, i); } };
struct FOccursCl { Ctx c; HD void operator()(u32 i) const { k_occurs_clause(c, i); } };
struct FOccursOt { Ctx c; HD void operator()(u32 i) const { k_occurs_from_ot(c, i); } };
struct FCount { CountArgs a; HD void operator()(u32 i) const { k_count_clause(a, i); } };
struct FGcFlags { Ctx c; u32* keep; u64* sizes; HD void operator()(u32 i) const { k_gc_flags(c, keep, sizes, i); } };
struct FGcMove { GcArgs a; HD void operator()(u32 i) const { k_gc_move(a, i); } };
struct FPropLists { PropArgs a; HD void operator()(u32 i) const { k_prop_lists(a, i); } };
struct FPropClause { PropArgs a; HD void operator()(u32 i) const { k_prop_clause(a, i); } };
struct FPropSweep { PropArgs a; HD void operator()(u32 i) const { k_prop_sweep(a, i); } };
struct FPropSweepLists { PropArgs a; HD void operator()(u32 i) const { k_prop_sweep_lists(a, i); } };
struct FReduce { Ctx c; HD void operator()(u32 i) const { k_reduce_list(c, i); } };
struct FScores { LcveArgs a; u32* max_score; HD void operator()(u32 i) const { k_scores(a, max_score, i); } };
struct FRank { LcveArgs a; HD void operator()(u32 i) const { k_rank(a, i); } };
struct FMisRec { LcveArgs a; Q4* rec; HD void operator()(u32 i) const { k_mis_rec(a, rec, i); } };
#if !SIGMA_CUDA
struct FMisPush { LcveArgs a; const u32* in; HD void operator()(u32 i) const { k_mis_push(a, in, i); } };
struct FMisPull {
    LcveArgs a; const u32* in; MisFront und, ins;
    HD void operator()(u32 i) const { k_mis_pull(a, in, und, ins, i); }
};
#endif
struct FMisInit { LcveArgs a; MisFront b; HD void operator()(u32 i) const { k_mis_init(a, b, i); } };
struct FMisBound { LcveArgs a; HD void operator()(u32 i) const { k_mis_bound(a, i); } };
struct FElectFlag { LcveArgs a; u32* flags; HD void operator()(u32 i) const { k_elect_flag(a, flags, i); } };
struct FElectWrite { LcveArgs a; const u32* flags; const u32* scan; HD void operator()(u32 i) const { k_elect_write(a, flags, scan, i); } };
struct FFill32 { u32* p; u32 v; HD void operator()(u32 i) const { p[i] = v; } };
// Proof line of clause from + i (a resolvent just written).
struct FProofClause {
    Ctx c; u32 from;
    HD void operator()(u32 i) const {
        const Hdr h = c.hdr[from + i];
        if (!h_deleted(h.flags) && h.size > 1) proof_line(c, c.lits + h.start, h.size);
    }
};
struct FSortList { SortArgs a; HD void operator()(u32 i) const { k_sort_list(a, i); } };
struct FSubPossible { SubArgs a; u32* flag; u32* prod; HD void operator()(u32 i) const { k_sub_unit_possible(a, flag, prod, i); } };
struct FSubPv { SubArgs a; HD void operator()(u32 i) const { k_sub_pv(a, i); } };
struct FSubNeed {
    Ctx c; const u32* pvs; const uint8_t* only; u32* ent; u64* words;
    HD void operator()(u32 i) const { k_sub_need(c, pvs, only, ent, words, i); }
};
struct FSubfxPairLit {
    const U2* pairs; const U2* units; u32* rank; u32* lit;
    HD void operator()(u32 i) const { k_subfx_pairlit(pairs, units, rank, lit, i); }
};
struct FSubfxFirst { const u32* rank; const u32* lit; u32* flag; HD void operator()(u32 i) const { k_subfx_first(rank, lit, flag, i); } };
struct FSubfxScatter {
    const u32* rank; const u32* lit; const u32* flag; const u32* scan; u32* orank; u32* olit; u32* count;
    HD void operator()(u32 i) const { k_subfx_scatter(rank, lit, flag, scan, orank, olit, count, i); }
};
struct FSubfxDiff {
    const u32* woff; const u32* wlit; const u32* uoff; const u32* ulit; const uint8_t* cand; u32* flag; uint8_t* run;
    HD void operator()(u32 k) const { k_subfx_diff(woff, wlit, uoff, ulit, cand, flag, run, k); }
};
struct FSubfxKeep { const U2* units; const uint8_t* run; u32* flag; HD void operator()(u32 i) const { k_subfx_keep(units, run, flag, i); } };
struct FSubfxKeepScatter {
    const U2* units; const u32* flag; const u32* scan; U2* out;
    HD void operator()(u32 i) const { k_subfx_keep_scatter(units, flag, scan, out, i); }
};
struct FSubfxTo8 { const u32* f; uint8_t* b; bool invert; HD void operator()(u32 k) const { k_subfx_to8(f, b, invert, k); } };
struct FSubSave { SubCkptArgs a; HD void operator()(u32 i) const { k_sub_save(a, i); } };
struct FSubRestore { SubCkptArgs a; HD void operator()(u32 i) const { k_sub_restore(a, i); } };
struct FSubReach { SubReachArgs a; const u32* off; u32 nq; HD void operator()(u32 i) const { k_sub_reach(a, off, nq, i); } };
struct FSubReachSize { Ctx c; const U2* units; u32* size; HD void operator()(u32 q) const { k_sub_reach_size(c, units, size, q); } };
struct FSubWarp { SubArgs a; HD void operator()(u32 k) const { sub_warp_pv(a, k); } };
struct FSubCommitSize { Ctx c; const u32* lits; u32* size; HD void operator()(u32 q) const { k_sub_commit_size(c, lits, size, q); } };
struct FSubCommitItem {
    Ctx c; const u32* lits; const u32* off; u32 n;
    HD void operator()(u32 i) const { k_sub_commit_item(c, lits, off, n, i); }
};
struct FSubCommitClear { Ctx c; const u32* lits; HD void operator()(u32 q) const { k_sub_commit_clear(c, lits, q); } };
struct FSubAssign { Ctx c; const U2* units; HD void operator()(u32 i) const { enqueue_unit(c, units[i].y); } };
struct FBveNeed { Ctx c; const u32* pvs; u64* need; HD void operator()(u32 i) const { k_bve_scratch_need(c, pvs, need, i); } };
struct FBveWarp { BveArgs a; HD void operator()(u32 i) const { k_bve_warp(a, i); } };
struct FBveWrite { BveArgs a; HD void operator()(u32 i) const { k_bve_write(a, i); } };
struct FBceCountWarp { BceArgs a; HD void operator()(u32 i) const { bce_count_warp(a, i); } };
struct FBceWrite { BceArgs a; HD void operator()(u32 i) const { k_bce_write(a, i); } };
struct FEre { EreArgs a; HD void operator()(u32 i) const { k_ere_pv(a, i); } };
struct FEreCount { EreArgs a; const u32* perm; u64* cnt; HD void operator()(u32 q) const { k_ere_count(a, perm, cnt, q); } };
struct FErePair { EreArgs a; const u32* perm; const u64* off; u32 n; HD void operator()(u32 i) const { k_ere_pair(a, perm, off, n, i); } };
struct FEreResolve { EreArgs a; HD void operator()(u32 i) const { k_ere_resolve(a, i); } };
struct FEreFix { EreArgs a; const u64* keys; u32 n; HD void operator()() const { ere_fixup(a, keys, n); } };
// Sort keys of the ERE losers: loser order[i]'s low key word (hi = false; order[i] =
// i set first) or high key word (hi = true), and the keys in sorted order.
struct FEreLoserKey {
    const u64* key; const u32* losers; u32* order; u32* out; bool hi;
    HD void operator()(u32 i) const {
        if (!hi) order[i] = i;
        const u64 k = key[losers[order[i]]];
        out[i] = hi ? (u32)(k >> 32) : (u32)k;
    }
};
struct FEreLoserGather {
    const u64* key; const u32* losers; const u32* order; u64* out;
    HD void operator()(u32 i) const { out[i] = key[losers[order[i]]]; }
};
struct FEreSeq { EreArgs a; HD void operator()() const { ere_sequential(a); } };
// Item i of a permuted launch runs f(perm[i]).
template <class F>
struct Perm {
    F f;
    const u32* perm;
    HD void operator()(u32 i) const { f(perm[i]); }
};
// Work-order key of elected variable k: descending clause count.
// Elected variables from n_first on (a batch's stopping formulas) come after the
// others; clause counts from 127 up share the first place (one 8-bit radix pass).
struct FPvKey {
    Ctx c; const u32* pvs; u32* key; u32* val; u32 n_first;
    HD void operator()(u32 k) const {
        const u32 p = V2L(pvs[k]);
        const u32 occ = c.ot_size[p] + c.ot_size[p + 1];
        key[k] = (k >= n_first ? 0x80u : 0u) | (0x7Fu - (occ < 0x7Fu ? occ : 0x7Fu));
        val[k] = k;
    }
};
struct FBoundInit { LcveArgs a; HD void operator()(u32 f) const { k_bound_init(a, f); } };
struct FVarFid { u32* var_fid; const u32* f_var; u32 nf; HD void operator()(u32 v) const { k_var_fid(var_fid, f_var, nf, v); } };
struct FCountFormula { FormulaCountArgs a; HD void operator()(u32 i) const { k_count_formula(a, i); } };
// Batch partition of the elected list: group of each elected variable's formula
// (0 dropped, 1 goes on, 2 stops this phase).
struct FPvGroup {
    Ctx c; const u32* pvs; const u32* f_group; u32* go; u32* stop;
    HD void operator()(u32 k) const {
        const u32 g = f_group[fid_of(c, pvs[k])];
        go[k] = g == 1u;
        stop[k] = g == 2u;
    }
};
struct FPvPartition {
    Ctx c; const u32* pvs; const u32* go; const u32* go_scan; const u32* stop; const u32* stop_scan; u32 n_go;
    u32* out;
    HD void operator()(u32 k) const {
        const u32 v = pvs[k];
        u32 pos = NONE;
        if (go[k]) pos = go_scan[k];
        else if (stop[k]) pos = n_go + stop_scan[k];
        if (pos != NONE) out[pos] = v;
        c.pvrank[v] = pos;
    }
};

// Batch upload from separate arrays: offsets moved from each formula's own base
// to its place in the store.
struct FRebase {
    u64* off; const u64* cb; const u64* first; const u64* base; u32 nf;
    HD void operator()(u32 i) const {
        const u32 f = upper_segment(cb, nf, (u64)i);
        off[i] = off[i] - first[f] + base[f];
    }
};

// Batch witness split: record starts (the word after a record's length word).
struct FRecStart {
    const uint8_t* mark; u32* flag;
    HD void operator()(u32 i) const { flag[i] = (i == 0 || mark[i - 1]) ? 1u : 0u; }
};
struct FRecScatter {
    const u32* flag; const u32* scan; u32* rstart;
    HD void operator()(u32 i) const { if (flag[i]) rstart[scan[i]] = i; }
};
// Formula (key), index (value) and word count of every record; words per formula.
struct FRecFid {
    Ctx c; const u32* rstart; u32 nrec; u32 nwords; u32* key; u32* val; u64* words; u64* f_words;
    HD void operator()(u32 r) const {
        const u32 st = rstart[r], en = r + 1 < nrec ? rstart[r + 1] : nwords;
        const u32 f = c.var_fid[ABS(c.resolved[st])];
        key[r] = f;
        val[r] = r;
        words[r] = en - st;
        atom_add64(&f_words[f], (u64)(en - st));
    }
};
struct FRecSize {
    const u64* words; const u32* order; u64* size;
    HD void operator()(u32 k) const { size[k] = words[order[k]]; }
};
// Records in formula order, literals in the formula's numbering, lengths kept.
struct FRecGather {
    Ctx c; const u32* rstart; const u32* order; const u32* fid; const u64* words; const u64* off; const u32* f_var;
    u32* out;
    HD void operator()(u32 k) const {
        const u32 r = order[k];
        const u32 st = rstart[r];
        const u32 n = (u32)words[r];
        const u32 shift = 2u * f_var[fid[k]];
        u32* o = out + off[k];
        for (u32 j = 0; j + 1 < n; j++) o[j] = c.resolved[st + j] - shift;
        o[n - 1] = c.resolved[st + n - 1];
    }
};
// Model extension: records per formula, and the walks.
struct FRecCount {
    Ctx c; const u32* rstart; u32* f_recs;
    HD void operator()(u32 r) const { atom_add(&f_recs[c.var_fid[ABS(c.resolved[rstart[r]])]], 1u); }
};
struct FExtendFormula { ExtendArgs a; HD void operator()(u32 f) const { k_extend_formula(a, f); } };
struct FExtendSingle { ExtendArgs a; HD void operator()() const { k_extend_single(a); } };
struct FExtendClear { Ctx c; uint8_t* value; HD void operator()(u32 v) const { k_extend_clear(c, value, v); } };
struct FExtendUnit { Ctx c; uint8_t* value; HD void operator()(u32 i) const { k_extend_unit(c, value, i); } };
struct FExtendIn {
    ExtendMap m; const uint8_t* packed; uint8_t* value;
    HD void operator()(u32 p) const { k_extend_in(m, packed, value, p); }
};
struct FExtendOut {
    ExtendMap m; const uint8_t* value; uint8_t* packed;
    HD void operator()(u32 p) const { k_extend_out(m, value, packed, p); }
};

// Trail split: formula and index of every unit; units per formula.
struct FUnitFid {
    Ctx c; u32* key; u32* val; u64* f_units;
    HD void operator()(u32 i) const {
        const u32 f = c.var_fid[ABS(c.trail[i])];
        key[i] = f;
        val[i] = i;
        atom_add64(&f_units[f], 1ull);
    }
};
struct FUnitGather {
    Ctx c; const u32* order; const u32* fid; const u32* f_var; u32* out;
    HD void operator()(u32 k) const { out[k] = c.trail[order[k]] - 2u * f_var[fid[k]]; }
};

// Download of a compacted store: clause offsets and learnt flags.
struct FDownOffsets {
    const Hdr* hdr; u64* off; uint8_t* learnt;
    HD void operator()(u32 i) const {
        const Hdr h = hdr[i];
        off[i] = h.start;
        learnt[i] = h_learnt(h.flags) ? 1 : 0;
    }
};

// Batch download: formula of every clause (key) with its index (value).
struct FClauseFid {
    Ctx c; u32* key; u32* val;
    HD void operator()(u32 i) const {
        key[i] = c.var_fid[ABS(c.lits[c.hdr[i].start])];
        val[i] = i;
    }
};
// Sizes and learnt flags in formula order.
struct FClauseSize {
    Ctx c; const u32* order; u64* size; uint8_t* learnt;
    HD void operator()(u32 k) const {
        const Hdr h = c.hdr[order[k]];
        size[k] = h.size;
        learnt[k] = h_learnt(h.flags) ? 1 : 0;
    }
};
// Literals in formula order, in each formula's own numbering.
struct FClauseGather {
    Ctx c; const u32* order; const u32* fid; const u64* off; const u32* f_var; u32* out;
    HD void operator()(u32 k) const {
        const Hdr h = c.hdr[order[k]];
        const u32 shift = 2u * f_var[fid[k]];
        const u32* l = c.lits + h.start;
        u32* o = out + off[k];
        for (u32 j = 0; j < h.size; j++) o[j] = l[j] - shift;
    }
};

enum Stage { ST_OT = 0, ST_PROP, ST_LCVE, ST_SORT, ST_SUB, ST_VE, ST_BCE, ST_ERE, ST_GC, ST_COUNT, ST_UP, ST_DOWN };

}  // namespace

struct pf_sigma_ctx {
    pf_options opt;
    Runtime rt;
    StageTimer tm;
    // DRAT proof of the round (opt.proof): lines [n, lits...] written by the kernels
    // into `proof` at the device counter counters64[4] (units as they are assigned);
    // proof_bound bounds the words reserved so far
    DBuf<u32> proof;
    u64 proof_bound = 0;
    bool uploaded = false, has_learnt = false;
    u32 rounds_run = 0;  // rounds since the last upload
    u32 nvars = 0, D = 0;
    u32 ncls = 0;
    u64 nlits_used = 0;
    u32 ntrail = 0, prop_head = 0;
    u64 nresolved = 0;
    u32 wave_stamp = 0;
    // clause store (double-buffered for compaction)
    DBuf<Hdr> hdr, hdr2;
    DBuf<u32> cstamp, cstamp2;  // per clause: phase stamp of its last change (Ctx::cstamp)
    DBuf<u32> keep_at, keep_shape;  // per variable: the last KEEP decision (BveArgs)
    DBuf<u32> lits, lits2;
    // occurrence table
    DBuf<u32> ot_off, ot_size, ot_refs, ot_cursor;
    // variables
    DBuf<u32> asg, ps, ns, pvrank;
    DBuf<uint8_t> vstate;
    DBuf<u32> trail, resolved;
    DBuf<u32> counters;   // [0] ntrail, [1] err, [2..] scratch counters
    DBuf<u64> counters64; // [0] nresolved, [2..3] counts
    DBuf<u64> ws_slots;   // [0, 32): elected lists' working set, [32, 64): graph working set (summed slots)
    // stage scratch
    DBuf<u32> score, order, order_k2, order_v2, rank, bound, pvs, flags, flags_scan;
    DBuf<u32> mis_big_a, mis_big_b;
    DBuf<u32> mis_word, mis_resume, mis_cmin;
    DBuf<u32> mis_in[4];  // new-in lists of the election rounds (small x2, large x2)
    DBuf<Q4> mis_rec;  // the election's 16-byte clause records
    DBuf<u32> mis_gbits;  // the election's graph membership bitmap
    DBuf<u32> pv_perm, pv_key;
    DBuf<u32> work, cl_stamp;
    DBuf<u32> radix_hist, radix_hscan, scan_tmp32;
    DBuf<u64> scan_tmp64;
    DBuf<u64> big64a, big64b;
    DBuf<uint8_t> down_learnt;  // learnt flags of the downloaded clauses
    DBuf<u64> up_off;           // offsets of an upload from host buffers
    DBuf<uint8_t> up_learnt;    // learnt flags of an upload from host buffers
    DBuf<u32> big32a, big32b;
    // BVE
    DBuf<uint8_t> ve_type;
    DBuf<u32> ve_porgs, ve_norgs, ve_ncls, ve_nlits, ve_nwit, ve_def, ve_cls_scan, ve_scr;
    DBuf<u64> ve_scr_off, ve_lit_scan, ve_wit_scan;
    // SUB safe path
    DBuf<U2> sub_units, sub_pairs;
    DBuf<u32> sub_ent, sub_ent_off, sub_ids, sub_words, sub_sizes, sub_pre_off, sub_pre_lits, sub_ulits;
    DBuf<u64> sub_wrd, sub_wrd_off;
    DBuf<Hdr> sub_hdrs;
    DBuf<uint8_t> sub_run;
    // SUB unit fix-point (device bookkeeping)
    DBuf<u32> fx_prod, fx_rank, fx_lit, fx_k2, fx_v2, fx_flag, fx_scan;
    DBuf<u32> want_rank, want_lit, want_cnt, want_off, used_lit, used_off;
    DBuf<uint8_t> fx_prod8, fx_other8;
    DBuf<U2> sub_units2;
    // ERE
    DBuf<u64> ere_claim, ere_key;
    DBuf<u32> ere_target, ere_losers;
    // formula batch (nf = 0: one formula). Formula f owns variables
    // h_f_var[f]+1 .. h_f_var[f+1] of the store's numbering.
    u32 nf = 0;
    std::vector<u32> h_f_var, h_f_nv;
    DBuf<u32> f_var, var_fid, f_err, f_active, f_npvs, f_group;
    DBuf<uint8_t> res_mark;  // witness record ends (batches)
    DBuf<u64> f_count;  // [f] live clauses, [nf + f] live literals
    std::vector<int> f_status;
    std::vector<u32> f_phases;
    // host state
    u32 npvs = 0;
    bool compact = false;          // clause i's literals start at the sum of the earlier sizes
    u32 n_go = 0;                  // elected variables of the formulas that go on (front of pvs)
    u32 perm_off = 0, perm_n = 0;  // range of pv_perm the per-variable stages run over
    bool ot_dirty = false;  // clauses changed since the OT build
    int phase = 0;
    u32 mu_inc = 0;
    i64 n_cls_after = 0, n_lits_after = 0;
    pf_round_stats st;
    std::vector<uint32_t> dump;
    u64 alg_bytes = 0;
    // hottest kernels, timed one by one: election rounds, BVE decision, SUB, BVE write
    enum { K_MIS, K_BVE, K_SUB, K_BVEW, K_COUNT };
    KernelClock kclock[K_COUNT];
    u64 kbytes[K_COUNT] = {};
    u64 phase_ws = 0;  // elected lists' working set of the current phase
    u32 mis_rounds = 0;
    u32 prop_waves = 0;

    Ctx view() {
        Ctx c;
        c.nvars = nvars;
        c.D = D;
        c.hdr = hdr.p;
        c.lits = lits.p;
        c.ncls = ncls;
        c.cap_cls = (u32)hdr.n;
        c.nlits_used = nlits_used;
        c.cap_lits = lits.n;
        c.ot_off = ot_off.p;
        c.ot_size = ot_size.p;
        c.ot_refs = ot_refs.p;
        c.ot_cursor = ot_cursor.p;
        c.ot_cap = (u32)ot_refs.n;
        c.asg = asg.p;
        c.vstate = vstate.p;
        c.ps = ps.p;
        c.ns = ns.p;
        c.pvrank = pvrank.p;
        c.trail = trail.p;
        c.ntrail = counters.p + 0;
        c.resolved = resolved.p;
        c.nresolved = counters64.p + 0;
        c.cap_resolved = resolved.n;
        c.err = counters.p + 1;
        c.var_fid = nf ? var_fid.p : nullptr;
        c.f_err = nf ? f_err.p : nullptr;
        c.res_mark = nf ? res_mark.p : nullptr;
        c.cstamp = cstamp.p;
        c.stamp = (u32)phase + 1u;
        c.proof = opt.proof ? proof.p : nullptr;
        c.nproof = opt.proof ? counters64.p + 4 : nullptr;
        c.cap_proof = proof.n;
        return c;
    }

    // Values the host needs together (scan totals, counters, the error word) are
    // gathered into device slots on the stream and read back with one copy, so a
    // stage waits for the device once instead of once per value.
    DBuf<u64> hread;
    u64 hr[8] = {};
    u64* hslot(int k) {
        hread.reserve(rt, 8);
        return hread.p + k;
    }
    // scan with its total into slot k
    template <class Tin, class T>
    void scan_to(const Tin* in, T* out, size_t n, int k) {
#if SIGMA_CUDA
        rt.zero(hslot(k), 8);
        scan1_launch(in, out, n, (T*)hslot(k));
#else
        u64 t;
        if constexpr (sizeof(T) == 4) t = scan32(in, out, n);
        else t = scan64(in, out, n);
        rt.h2d(hslot(k), &t, 8);
#endif
    }
    // a device word into slot k (zero-extended)
    void word_to(const u32* d, int k) {
        rt.zero(hslot(k), 8);
        rt.d2d(hslot(k), d, 4);
    }
    // all slots into hr; the error word rides along in slot 7 and is checked
    void read_slots_checked(u32 stage_err_mask = ~0u) {
        word_to(counters.p + 1, 7);
        rt.d2h(hr, hslot(0), 8 * sizeof(u64));
        check_err((u32)hr[7] & stage_err_mask);
    }
    u32 read_err() {
        u32 e = 0;
        rt.d2h(&e, counters.p + 1, 4);
        return e;
    }
    u32 read_u32(const u32* d) {
        u32 v = 0;
        rt.d2h(&v, d, 4);
        return v;
    }
    u64 read_slots(const u64* d) {
        u64 v[kSpreadSlots];
        rt.d2h(v, d, sizeof v);
        u64 t = 0;
        for (u64 x : v) t += x;
        return t;
    }
    u64 read_u64(const u64* d) {
        u64 v = 0;
        rt.d2h(&v, d, 8);
        return v;
    }
    void write_u32(u32* d, u32 v) { rt.h2d(d, &v, 4); }
#if SIGMA_CUDA
    // Blocks of a cooperative wave kernel (256 threads): every block resident at once.
    int mis_grid = 0;
    template <class K>
    int coop_grid(K kernel, int& cache) {
        if (!cache) {
            int per_sm = 0;
            ck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0), "occupancy");
            if (per_sm < 1) throw std::runtime_error("a wave kernel cannot be resident");
            cache = per_sm * rt.sms;
        }
        return cache;
    }
    int mis_rounds_grid() { return coop_grid(mis_rounds_k, mis_grid); }
#endif
    void write_u64(u64* d, u64 v) { rt.h2d(d, &v, 8); }

    // exclusive scans
#if SIGMA_CUDA
    // single-pass scans: tile state kept across scans (flags tagged with an epoch)
    DBuf<u64> scan1_agg, scan1_incl, scan1_total;
    DBuf<u32> scan1_flag, scan1_ctl;
    u32 scan1_epoch = 0, scan1_base = 0;
    template <class Tin, class T>
    T scan1(const Tin* in, T* out, size_t n) {
        scan1_total.reserve(rt, 2);
        T* total = (T*)scan1_total.p;
        scan1_launch(in, out, n, total);
        T h = 0;
        rt.d2h(&h, total, sizeof(T));
        return h;
    }
    // the scan, its total written to the device word `total` (no synchronisation)
    template <class Tin, class T>
    void scan1_launch(const Tin* in, T* out, size_t n, T* total) {
        const size_t tiles = scan1_tiles(n);
        if (!scan1_ctl.p || scan1_base > 0x7FFFFFFFu || scan1_epoch >= 0x3FFFFFFFu) {
            scan1_ctl.reserve(rt, 4);
            rt.zero(scan1_ctl.p, 16);
            scan1_base = 0;
            if (scan1_flag.p) rt.zero(scan1_flag.p, scan1_flag.bytes());
            scan1_epoch = 0;
        }
        if (tiles > scan1_flag.n) {
            const size_t cap = tiles + tiles / 2 + 64;
            scan1_agg.reserve(rt, cap);
            scan1_incl.reserve(rt, cap);
            scan1_flag.reserve(rt, cap);
            rt.zero(scan1_flag.p, scan1_flag.bytes());
        }
        if (n == 0) {
            rt.zero(total, sizeof(T));
        } else {
            Scan1State st{scan1_agg.p, scan1_incl.p, scan1_flag.p, scan1_ctl.p, counters.p + 1};
            rt.launches++;
            scan1_k<Tin, T><<<(unsigned)tiles, kScanThreads, 0, rt.stream>>>(in, out, n, total, st, scan1_base,
                                                                             ++scan1_epoch);
            ck(cudaGetLastError(), "launch");
            scan1_base += (u32)tiles;
        }
    }
    u32 scan32(const u32* in, u32* out, size_t n) { return scan1<u32, u32>(in, out, n); }
    template <class Tin>
    u64 scan64(const Tin* in, u64* out, size_t n) { return scan1<Tin, u64>(in, out, n); }
#else
    u32 scan32(const u32* in, u32* out, size_t n) {
        scan_tmp32.reserve(rt, scan_tmp_elems(n) + 2);
        u32* total = scan_tmp32.p + scan_tmp32.n - 1;
        excl_scan<u32, u32>(in, out, n, total, scan_tmp32.p, rt.stream);
        rt.launches += 3;
        return read_u32(total);
    }
    template <class Tin>
    u64 scan64(const Tin* in, u64* out, size_t n) {
        scan_tmp64.reserve(rt, scan_tmp_elems(n) + 2);
        u64* total = scan_tmp64.p + scan_tmp64.n - 1;
        excl_scan<Tin, u64>(in, out, n, total, scan_tmp64.p, rt.stream);
        rt.launches += 3;
        return read_u64(total);
    }
#endif

    // ------------------------------------------------------------ dumps
    void rec(u32 kind, u32 ph, u32 stage, const std::vector<u32>& d) {
        dump.push_back(kind);
        dump.push_back(ph);
        dump.push_back(stage);
        dump.push_back((u32)d.size());
        dump.insert(dump.end(), d.begin(), d.end());
    }
    template <class T>
    std::vector<T> fetch(const T* d, size_t n) {
        std::vector<T> h(n);
        if (n) rt.d2h(h.data(), d, n * sizeof(T));
        return h;
    }
    void dump_cnf(u32 ph, u32 stage) {
        auto H = fetch(hdr.p, ncls);
        auto L = fetch(lits.p, nlits_used);
        std::vector<u32> d;
        d.push_back(ncls);
        for (u32 i = 0; i < ncls; i++) {
            d.push_back(H[i].flags & 15u);
            d.push_back(H[i].sig);
            d.push_back(H[i].size);
            for (u32 k = 0; k < H[i].size; k++) d.push_back(L[H[i].start + k]);
        }
        rec(1, ph, stage, d);
    }
    void dump_trail(u32 ph, u32 stage) { rec(7, ph, stage, fetch(trail.p, ntrail)); }
    void dump_resolved(u32 ph, u32 stage) { rec(8, ph, stage, fetch(resolved.p, nresolved)); }
    void dump_elim(u32 ph, u32 stage) {
        auto vs = fetch(vstate.p, nvars + 1);
        std::vector<u32> d;
        for (u32 v = 1; v <= nvars; v++) if (vs[v]) d.push_back(v);
        rec(9, ph, stage, d);
    }
    void dump_stage(u32 ph, u32 stage) {
        if (opt.dump_level < 2) return;
        dump_cnf(ph, stage);
        dump_trail(ph, stage);
        if (stage >= 5) dump_resolved(ph, stage);
    }
    void dump_pvlists(u32 ph) {
        auto P = fetch(pvs.p, npvs);
        auto off = fetch(ot_off.p, D + 1);
        auto sz = fetch(ot_size.p, D);
        auto refs = fetch(ot_refs.p, off[D]);
        std::vector<u32> d;
        for (u32 v : P) {
            for (u32 l = V2L(v); l <= V2L(v) + 1; l++) {
                d.push_back(sz[l]);
                for (u32 i = 0; i < sz[l]; i++) d.push_back(refs[off[l] + i]);
            }
        }
        rec(6, ph, 3, d);
    }

    void check(u32 stage_err_mask = ~0u) { check_err(read_err() & stage_err_mask); }
    void check_err(u32 e) {
        if (e & ERR_UNSAT) throw int(PF_UNSAT);
        if (e & (ERR_CAP_CLAUSES | ERR_CAP_LITS | ERR_CAP_WITNESS | ERR_CAP_SCRATCH)) throw std::runtime_error("capacity exceeded (internal sizing bug)");
        if (e & ERR_ITER) throw int(PF_ETIMEOUT);
        if (e & ERR_INPUT) throw int(PF_EINVAL);
        if (e & ERR_INTERNAL) throw std::runtime_error("internal invariant violated");
    }

    // ------------------------------------------------------------ proof
    // Room for `words` more proof words (the buffer keeps what is written).
    void proof_reserve(u64 words) {
        if (!opt.proof) return;
        proof_bound += words;
        if (proof_bound > proof.n) proof.grow(rt, (size_t)(proof_bound + proof_bound / 2 + 4096), proof.n);
    }
    // Resolvents written in [from, ncls): each a proof line, in store order.
    void proof_clauses(u32 from) {
        if (!opt.proof || from >= ncls) return;
        rt.each(FProofClause{view(), from}, ncls - from);
    }

    // ------------------------------------------------------------ capacity
    void ensure_clauses(u64 need) {
        if (need <= hdr.n) return;
        const size_t cap = (size_t)(need + need / 4 + 1024);
        if (cap > 0xFFFFFFF0ull) throw OomError("clause count exceeds 32-bit ids");
        hdr.grow(rt, cap, ncls);
        cstamp.grow(rt, cap, ncls);
    }
    void ensure_lits(u64 need) {
        if (need <= lits.n) return;
        const size_t cap = (size_t)(need + need / 4 + 4096);
        if (cap > 0xFFFFFFF0ull) throw OomError("literal pool exceeds 32-bit offsets");
        lits.grow(rt, cap, nlits_used);
    }
    void ensure_resolved(u64 need) {
        if (need <= resolved.n) return;
        resolved.grow(rt, (size_t)(need + need / 4 + 4096), nresolved);
        if (nf) {
            res_mark.grow(rt, resolved.n, nresolved);
            rt.zero(res_mark.p + nresolved, res_mark.n - nresolved);
        }
    }

    // ------------------------------------------------------------ stages
#if SIGMA_CUDA
    // Occurrence table by literal buckets (k_otb.cuh): buckets of 2^shift literal
    // slots, at most OTB_MAX_BUCKETS of them (so up to 134M literal slots). Used when
    // the per-literal counters (4 bytes a slot) outgrow the L2 cache, where the
    // atomic histogram and scatter turn into random device-memory traffic.
    static constexpr u64 kOtbMinSlots = 1ull << 24;
    DBuf<u32> otb_count, otb_base, otb_cursor;
    DBuf<u64> otb_pair;
    bool otb_plan(u32& shift, u32& nb) const {
        if (opt.ot_buckets < 0 || (opt.ot_buckets == 0 && D < kOtbMinSlots)) return false;
        u32 s = 8;
        while (s < OTB_MAX_SHIFT && ((u64)D >> s) > 1024) s++;
        shift = s;
        nb = (u32)(((u64)D + (1ull << s) - 1) >> s);
        return nb <= OTB_MAX_BUCKETS;
    }
    void create_ot_buckets(u32 shift, u32 nb) {
        otb_count.reserve(rt, nb + 1);
        otb_base.reserve(rt, nb + 1);
        otb_cursor.reserve(rt, nb + 1);
        otb_pair.reserve(rt, (size_t)nlits_used + 1);
        rt.zero(otb_count.p, (size_t)nb * 4);
        // pass-1 tiles: about 7/8 of the stage at the store's mean clause length
        const u64 mean_x8 = std::max<u64>(8ull * nlits_used / std::max<u32>(ncls, 1), 8);
        const u32 fill_tile = (u32)std::min<u64>(std::max<u64>(7ull * OTB_FILL_CAP / mean_x8, 32), 4096) & ~31u;
        OtbArgs a{view(), shift, nb, otb_count.p, otb_cursor.p, otb_base.p, otb_pair.p, fill_tile};
        const u32 fill_smem = OTB_FILL_CAP * 8 + 3 * nb * 4;
        static bool attr_set = false;
        if (!attr_set) {
            ck(cudaFuncSetAttribute(ot_bucket_lists_k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)((1u << OTB_MAX_SHIFT) * 4)),
               "smem attr");
            ck(cudaFuncSetAttribute(ot_bucket_fill_k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(OTB_FILL_CAP * 8 + 3 * OTB_MAX_BUCKETS * 4)),
               "smem attr");
            attr_set = true;
        }
        const u32 grid = (u32)rt.sms * 8u;
        if (ncls) {
            rt.launches++;
            ot_bucket_count_k<<<grid, 256, nb * 4, rt.stream>>>(a);
            ck(cudaGetLastError(), "launch");
        }
        scan1_launch(otb_count.p, otb_base.p, nb, otb_base.p + nb);
        rt.d2d(otb_cursor.p, otb_base.p, (size_t)nb * 4);
        const u32 ntiles = (ncls + fill_tile - 1) / fill_tile;
        if (ntiles) {
            rt.launches++;
            int per_sm = 0;
            ck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ot_bucket_fill_k, OTB_FILL_THREADS, fill_smem),
               "occupancy");
            const u32 fill_grid = std::min((u32)rt.sms * (u32)std::max(per_sm, 1), ntiles);
            ot_bucket_fill_k<<<fill_grid, OTB_FILL_THREADS, fill_smem, rt.stream>>>(a);
            ck(cudaGetLastError(), "launch");
        }
        rt.launches++;
        ot_bucket_lists_k<<<nb, OTB_LIST_THREADS, (1u << shift) * 4, rt.stream>>>(a);
        ck(cudaGetLastError(), "launch");
        rt.d2d(ot_off.p + D, otb_base.p + nb, 4);
    }
#endif

    // createOT (simplify.cpp:35-56).
    void create_ot() {
        // the occurrences (live clauses' literals) never exceed the literal pool in
        // use, so the table is sized before its total is known
        if (nlits_used > ot_refs.n) ot_refs.reserve(rt, (size_t)nlits_used + nlits_used / 4 + 1024);
#if SIGMA_CUDA
        u32 shift = 0, nb = 0;
        if (otb_plan(shift, nb)) {
            create_ot_buckets(shift, nb);
            word_to(ot_off.p + D, 0);
            read_slots_checked();
            ot_dirty = false;
            alg_bytes += 2ull * (4ull * nlits_used + 8ull * ncls) + 8ull * D + 4ull * (u32)hr[0];
            return;
        }
#endif
        Ctx c = view();
        rt.zero(ot_size.p, (size_t)D * 4);
        rt.each(FHist{c}, ncls);
#if SIGMA_CUDA
        scan1_launch(ot_size.p, ot_off.p, D, ot_off.p + D);
#else
        write_u32(ot_off.p + D, scan32(ot_size.p, ot_off.p, D));
#endif
        rt.d2d(ot_cursor.p, ot_off.p, (size_t)D * 4);
        c = view();
        rt.each(FScatter{c}, ncls);
        word_to(ot_off.p + D, 0);
        read_slots_checked();
        const u32 total = (u32)hr[0];
        ot_dirty = false;
        alg_bytes += 2ull * (4ull * nlits_used + 8ull * ncls) + 8ull * D + 4ull * total;
    }

    // The mean occurrence-list length (literals in use per literal slot) times the
    // sweep divisor, 0 when sweeps are off (prop_use_sweep).
    u32 sweep_scale() const {
        if (opt.sweep_div < 0) return 0;
        const u64 div = opt.sweep_div ? (u64)opt.sweep_div : 64ull;
        return (u32)std::min<u64>(std::max<u64>(div * nlits_used / std::max<u32>(D, 1), 1), 0xFFFFFFFFull);
    }
    // Blocks of the per-variable warp kernels.
    u32 pv_grid() const { return (u32)rt.sms * (opt.pv_blocks > 0 ? (u32)opt.pv_blocks : 8u); }

#if SIGMA_CUDA
    // Traces of the persistent launches, printed to stderr when the environment sets
    // PF_TRACE: per propagation wave the pending literals, the clauses collected (or
    // "sweep") and the wave's device time; per election round the undecided and
    // went-in vertex lists (small and big adjacency) and the round's device time.
    static constexpr u32 kPropTraceWaves = 4096;
    const bool trace_on = std::getenv("PF_TRACE") != nullptr;
    DBuf<u32> prop_trace;
    DBuf<u64> prop_parts;
    void print_mis_trace(u32 rounds) {
        const u32 n = std::min(rounds, kPropTraceWaves);
        std::vector<u32> t(5 * (size_t)n + 5);
        if (n) rt.d2h(t.data(), prop_trace.p, 5 * (size_t)n * 4);
        std::fprintf(stderr, "election phase %u: %u rounds\n", phase, rounds);
        for (u32 i = 0; i < n; i++) {
            const double us = i + 1 < n ? (double)(u32)(t[5 * i + 9] - t[5 * i + 4]) * 1.024 : 0.0;
            std::fprintf(stderr, "  round %u undecided %u+%u in %u+%u %.1f us\n", i, t[5 * i], t[5 * i + 1],
                         t[5 * i + 2], t[5 * i + 3], us);
        }
    }
    void print_prop_trace(u32 waves) {
        const u32 n = std::min(waves, kPropTraceWaves);
        std::vector<u32> t(4 * (size_t)n + 4);
        if (n) rt.d2h(t.data(), prop_trace.p, 4 * (size_t)n * 4);
        std::fprintf(stderr, "prop phase %u: %u waves, ncls %u\n", phase, waves, ncls);
        for (u32 i = 0; i < n; i++) {
            const u32* w = &t[4 * i];
            const double us = i + 1 < n ? (double)(u32)(w[6] - w[2]) * 1.024 : 0.0;
            if (w[1] >> 31) {
                std::fprintf(stderr, "  wave %u pending %u sweep %.1f us\n", i, w[0], us);
            } else {
                const double la = w[3] ? (double)(u32)(w[3] - w[2]) * 1.024 : 0.0;
                std::fprintf(stderr, "  wave %u pending %u collected %u %.1f us (lists %.1f us)\n", i, w[0], w[1], us,
                             la);
            }
        }
    }
#endif

    // prop (elimination.cpp:64-99).
    void prop() {
        if (prop_head >= ntrail) return;
#if SIGMA_CUDA
        // collected clauses plus the free slots of the warps' closed runs (at most 31
        // per run of PROP_SLOTS, and two partly used runs per warp and wave)
        const size_t nwarps = (size_t)rt.sms * 4 * 256 / 32;
        work.reserve(rt, (size_t)ot_refs.n + ot_refs.n / 8 + 2 * nwarps * PROP_SLOTS + 1024);
#else
        work.reserve(rt, (size_t)std::max<u64>(ot_refs.n, 1024));
#endif
        if (cl_stamp.n < hdr.n) {
            cl_stamp.reserve(rt, hdr.n);
            rt.zero(cl_stamp.p, cl_stamp.bytes());
            wave_stamp = 0;
        }
#if SIGMA_CUDA
        {
            PropArgs a;
            a.c = view();
            a.head = prop_head;
            a.stamp = wave_stamp + 1;
            a.cl_stamp = cl_stamp.p;
            a.work = work.p;
            a.nwork = nullptr;
            a.cap_work = (u32)work.n;
            // parts of long lists: at most one per PROP_PART occurrences of the table
            prop_parts.reserve(rt, (size_t)(nlits_used / PROP_PART) + 1024);
            PropWaves w{counters.p + 22, counters.p + 24, counters.p + 26, loop_bound(), sweep_scale(),
                        nullptr, 0, counters.p + 28, prop_parts.p, counters.p + 29, (u32)prop_parts.n};
            if (trace_on) {
                prop_trace.reserve(rt, 5 * kPropTraceWaves);
                w.trace = prop_trace.p;
                w.trace_cap = kPropTraceWaves - 1;
            }
            rt.zero(counters.p + 22, 5 * 4);  // [22..23] work counters, [24..25] barrier, [26] waves
            rt.d2d(counters.p + 28, counters.p + 0, 4);  // [28] the trail's end for the first wave
            rt.zero(counters.p + 29, 2 * 4);             // [29..30] list-part counters
            void* args[] = {&a, &w};
            rt.launches++;
            // four blocks per SM: most waves of a propagation are small, and the grid
            // barrier between them costs one arrival per block
            ck(cudaLaunchCooperativeKernel((const void*)prop_waves_k, dim3(rt.sms * 4), dim3(256), args, 0,
                                           rt.stream),
               "cooperative launch");
            check();
            const u32 waves = read_u32(counters.p + 26);
            if (trace_on) print_prop_trace(waves);
            wave_stamp += waves;
            prop_waves += waves;
            ntrail = read_u32(counters.p + 0);
            prop_head = ntrail;
        }
#else
        u32 guard = 0;
        while (prop_head < ntrail) {
            if (++guard > loop_bound()) throw int(PF_ETIMEOUT);
            prop_waves++;
            const u32 pend = ntrail - prop_head;
            PropArgs a;
            a.c = view();
            a.head = prop_head;
            a.stamp = ++wave_stamp;
            a.cl_stamp = cl_stamp.p;
            a.work = work.p;
            a.nwork = counters.p + 2;
            a.cap_work = (u32)work.n;
            if (prop_use_sweep(pend, sweep_scale(), ncls)) {
                rt.each(FPropSweep{a}, ncls);
                rt.each(FPropSweepLists{a}, pend);
                prop_head = ntrail;
                ntrail = read_u32(counters.p + 0);
                check();
                continue;
            }
            write_u32(counters.p + 2, 0);
            rt.each(FPropLists{a}, pend);
            const u32 nw = read_u32(counters.p + 2);
            prop_head = ntrail;
            rt.each(FPropClause{a}, nw);
            ntrail = read_u32(counters.p + 0);
            check();
        }
#endif
        ot_dirty = true;
        if (!opt.sub) rt.each(FReduce{view()}, D);
    }

    // LCVE (lcve.cpp:46-81).
    bool lcve() {
        Ctx c = view();
        rt.zero(ps.p, (size_t)(nvars + 1) * 4);
        rt.zero(ns.p, (size_t)(nvars + 1) * 4);
        if (ot_dirty) rt.each(FOccursCl{c}, ncls);
        else rt.each(FOccursOt{c}, nvars + 1);
        LcveArgs a;
        a.c = c;
        a.pt = (u32)opt.mu_pos << mu_inc;
        a.nt = (u32)opt.mu_neg << mu_inc;
        a.score = score.p;
        a.order = order.p;
        a.rank = rank.p;
        a.word = mis_word.p;
        a.resume = mis_resume.p;
        mis_rec.reserve(rt, (size_t)ncls + 1);
        a.crec = mis_rec.p;
        mis_cmin.reserve(rt, (size_t)ncls + 1);
        a.cmin = mis_cmin.p;
        mis_gbits.reserve(rt, (size_t)nvars / 32 + 1);
        rt.zero(mis_gbits.p, ((size_t)nvars / 32 + 1) * 4);
        a.gbits = mis_gbits.p;
        a.ws_bytes = ws_slots.p + kSpreadSlots;
        a.bound = bound.p;
        a.pvs = pvs.p;
        a.f_active = nf ? f_active.p : nullptr;
        a.f_npvs = nf ? f_npvs.p : nullptr;
        const u32 nform = nf ? nf : 1u;
        rt.zero(score.p, (size_t)(nvars + 1) * 4);
        write_u32(counters.p + 27, 0);
        rt.each(FScores{a, counters.p + 27}, nvars + 1);
        // LCV order: stable by score over ascending variables (rSort, sort.h:123-133);
        // radix passes only over the bytes the largest score uses
        const u32 max_score = read_u32(counters.p + 27);
        int bits = 8;
        while (bits < 32 && (max_score >> bits)) bits += 8;
        rt.d2d(order_k2.p, score.p + 1, (size_t)nvars * 4);  // keys = score[1..]
        radix_sort_pairs(order_k2.p, order.p, order_v2.p, rank.p, nvars, bits, radix_hist.p, radix_hscan.p,
                         scan_tmp32.p, rt.stream);
        rt.launches += 5 * (bits / 8);
        rt.zero(bound.p, (size_t)nform * 8, 0xFF);
        rt.each(FRank{a}, nvars);
        // Independent set by push/pull rounds. Undecided lists: flags|mis_big_a and
        // flags_scan|mis_big_b; new-in lists: mis_in[0..3].
        mis_big_a.reserve(rt, nvars + 1);
        mis_big_b.reserve(rt, nvars + 1);
        for (auto& b : mis_in) b.reserve(rt, nvars + 1);
        u32* ctr = counters.p + 12;  // [12..23] three sets of list lengths, [24..25] barrier, [26] rounds
        rt.zero(ctr, 15 * 4);
#if SIGMA_CUDA
        rt.launches++;
        mis_init_k<<<rt.grid(nvars + 1), 256, 0, rt.stream>>>(
            a, MisFront{flags.p, ctr, mis_big_a.p, ctr + 1}, nvars + 1);
        ck(cudaGetLastError(), "launch");
#else
        rt.each(FMisInit{a, MisFront{flags.p, ctr, mis_big_a.p, ctr + 1}}, nvars + 1);
#endif
#if SIGMA_CUDA
        if (ncls) {
            rt.launches++;
            mis_rec_warp_k<<<rt.grid((ncls + 7u) / 8u, 8), 256, 0, rt.stream>>>(a, mis_rec.p);
            ck(cudaGetLastError(), "launch");
        }
#else
        rt.each(FMisRec{a, mis_rec.p}, ncls);
#endif
        u32 rounds = 0;
#if SIGMA_CUDA
        MisRounds w;
        w.u_small[0] = flags.p;
        w.u_small[1] = flags_scan.p;
        w.u_big[0] = mis_big_a.p;
        w.u_big[1] = mis_big_b.p;
        w.in_small[0] = mis_in[0].p;
        w.in_small[1] = mis_in[1].p;
        w.in_big[0] = mis_in[2].p;
        w.in_big[1] = mis_in[3].p;
        w.ctr = ctr;
        w.bar = ctr + 12;
        w.rounds = ctr + 14;
        w.max_rounds = loop_bound();
        w.trace = nullptr;
        w.trace_cap = 0;
        if (trace_on) {
            prop_trace.reserve(rt, 5 * kPropTraceWaves);
            w.trace = prop_trace.p;
            w.trace_cap = kPropTraceWaves;
        }
        void* args[] = {&a, &w};
        kclock[K_MIS].start(rt);
        ck(cudaLaunchCooperativeKernel((const void*)mis_rounds_k, dim3(mis_rounds_grid()), dim3(256), args, 0,
                                       rt.stream),
           "cooperative launch");
        kclock[K_MIS].stop(rt);
        rt.launches++;
#else
        MisFront und[2] = {{flags.p, ctr, mis_big_a.p, ctr + 1}, {flags_scan.p, ctr + 4, mis_big_b.p, ctr + 5}};
        MisFront ins[2] = {{mis_in[0].p, ctr + 2, mis_in[2].p, ctr + 3}, {mis_in[1].p, ctr + 6, mis_in[3].p, ctr + 7}};
        kclock[K_MIS].start(rt);
        for (u32 cur = 0;; cur ^= 1u) {
            u32 n[4];
            rt.d2h(n, ctr + 4 * cur, 16);
            if (!n[0] && !n[1] && !n[2] && !n[3]) break;
            if (++rounds > loop_bound()) throw int(PF_ETIMEOUT);
            if (n[2]) rt.each(FMisPush{a, ins[cur].small}, n[2]);
            if (n[3]) rt.each(FMisPush{a, ins[cur].big}, n[3]);
            rt.zero(ctr + 4 * (cur ^ 1u), 16);
            LcveArgs ar = a;
            ar.r0 = rounds == 1;  // the first round's walks test the clauses' least ranks
            if (n[0]) rt.each(FMisPull{ar, und[cur].small, und[cur ^ 1u], ins[cur ^ 1u]}, n[0]);
            if (n[1]) rt.each(FMisPull{ar, und[cur].big, und[cur ^ 1u], ins[cur ^ 1u]}, n[1]);
        }
        kclock[K_MIS].stop(rt);
#endif
        rt.each(FBoundInit{a}, nform);
        rt.each(FMisBound{a}, nvars + 1);
        rt.each(FFill32{pvrank.p, NONE}, nvars + 1);
        rt.each(FElectFlag{a, flags.p}, nvars);
        if (nf) rt.zero(f_npvs.p, (size_t)nf * 4);
        // one read: the elected count, the rounds run and the error word (a round
        // that ran out of time is caught here; the kernels since only read words)
        scan_to(flags.p, flags_scan.p, nvars, 0);
#if SIGMA_CUDA
        word_to(ctr + 14, 1);
#endif
        read_slots_checked();
        npvs = (u32)hr[0];
#if SIGMA_CUDA
        rounds = (u32)hr[1];
        if (trace_on) print_mis_trace(rounds);
#endif
        mis_rounds += rounds;
        rt.each(FElectWrite{a, flags.p, flags_scan.p}, nvars);
        n_go = npvs;
        perm_off = 0;
        perm_n = npvs;
        alg_bytes += 4ull * D + 24ull * nvars;
        const bool go = npvs >= (u32)opt.lcve_min;
        // stage dumps record an election that goes on (as the reference harness does)
        if (go && opt.dump_level >= 2) {
            rec(3, phase, 2, fetch(score.p, nvars + 1));
            rec(4, phase, 2, fetch(order.p, nvars));
        }
        if (go && opt.dump_level >= 1) rec(5, phase, 2, fetch(pvs.p, npvs));
        return go;
    }

    void sort_ot() {
        rt.zero(ws_slots.p, kSpreadSlots * 8);
        SortArgs a{view(), pvs.p, ws_slots.p};
        rt.each(FSortList{a}, 2 * npvs);
        // work order of the per-variable kernels: most clauses first (longest
        // processing time first), so similar variables share a warp and the longest
        // ones do not start last. Results still go to each variable's elected rank.
        pv_perm.reserve(rt, nvars + 1);
        pv_key.reserve(rt, nvars + 1);
        rt.each(FPvKey{view(), pvs.p, pv_key.p, pv_perm.p, n_go}, npvs);
        radix_sort_pairs(pv_key.p, pv_perm.p, order_k2.p, order_v2.p, npvs, 8, radix_hist.p, radix_hscan.p,
                         scan_tmp32.p, rt.stream);
        rt.launches += 5;
    }

    // f(k) for every elected variable, in work order, dynamically scheduled.
    template <class F>
    void pv_each(const F& f) {
        rt.each_dyn(Perm<F>{f, pv_perm.p + perm_off}, perm_n, counters.p + 11);
    }

    // working set of the elected lists, accumulated by the sort kernel
    u64 pv_bytes() { return read_slots(ws_slots.p); }

    // One SUB pass over the elected variables (warp per variable).
    void sub_pass(const SubArgs& a) {
#if SIGMA_CUDA
        if (!perm_n) return;
        ck(cudaMemsetAsync(counters.p + 11, 0, 4, rt.stream), "memset");
        rt.launches++;
        sub_warp_k<<<pv_grid(), 256, 0, rt.stream>>>(a, pv_perm.p + perm_off, perm_n, counters.p + 11);
        ck(cudaGetLastError(), "launch");
#else
        pv_each(FSubWarp{a});
#endif
    }

    // SUB (elimination.cpp:110-129).
    void sub() {
        if (!(opt.sub || opt.ve_plus) || !npvs) return;
        proof_reserve(phase_ws / 2 + 16);  // at most two lines per clause of the elected lists
        SubArgs a;
        a.c = view();
        a.pvs = pvs.p;
        a.npvs = npvs;
        a.sub_max = (u32)opt.sub_max;
        a.units = nullptr;
        a.nunits = counters.p + 4;
        a.cap_units = 0;
        a.pre_off = nullptr;
        a.pre_lits = nullptr;
        a.run = nullptr;
        write_u32(counters.p + 5, 0);
        fx_prod.reserve(rt, npvs + 1);
        rt.each(FSubPossible{a, counters.p + 5, fx_prod.p}, npvs);
        kbytes[K_SUB] += phase_ws;
        if (read_u32(counters.p + 5) == 0) {
            kclock[K_SUB].start(rt);
            sub_pass(a);
            kclock[K_SUB].stop(rt);
            // the exact pass derives no unit; its error word is read with the next
            // stage's values (the VE preparation and the counts only read the store)
            // unless stage dumps are being recorded
            if (opt.dump_level) check();
            return;
        }
        sub_safe(a);
    }

    // Bits a radix key needs for values below n (multiples of 8).
    static int key_bits(u64 n) {
        int b = 8;
        while (b < 32 && (n >> b)) b += 8;
        return b;
    }

    // The sorted sets of unit literals (sub_units[0, nu)) that reach every target
    // variable from an earlier one: want_off (npvs + 1 segment starts, by rank) and
    // want_lit.
    void sub_unit_sets(u32 nu, const uint8_t* target) {
        want_cnt.reserve(rt, npvs + 1);
        want_off.reserve(rt, npvs + 1);
        rt.zero(want_cnt.p, ((size_t)npvs + 1) * 4);
        u32 nwant = 0;
        if (nu) {
            big32a.reserve(rt, (size_t)nu + 1);
            big32b.reserve(rt, (size_t)nu + 1);
            rt.each(FSubReachSize{view(), sub_units.p, big32a.p}, nu);
            const u32 items = scan32(big32a.p, big32b.p, nu);
            sub_pairs.reserve(rt, (size_t)items + 16);
            write_u32(counters.p + 6, 0);
            SubReachArgs ra{view(), sub_units.p, sub_pairs.p, counters.p + 6, (u32)sub_pairs.n, target};
            if (items) rt.each(FSubReach{ra, big32b.p, nu}, items);
            const u32 np = read_u32(counters.p + 6);
            if (np) {
                fx_rank.reserve(rt, (size_t)np + 1);
                fx_lit.reserve(rt, (size_t)np + 1);
                fx_k2.reserve(rt, (size_t)np + 1);
                fx_v2.reserve(rt, (size_t)np + 1);
                fx_flag.reserve(rt, (size_t)np + 1);
                fx_scan.reserve(rt, (size_t)np + 1);
                rt.each(FSubfxPairLit{sub_pairs.p, sub_units.p, fx_rank.p, fx_lit.p}, np);
                radix_hist.reserve(rt, radix_hist_elems(np));
                radix_hscan.reserve(rt, radix_hist_elems(np));
                scan_tmp32.reserve(rt, scan_tmp_elems(radix_hist_elems(np)) + 4);
                // by literal, then stable by rank: (rank, literal) order
                const int lb = key_bits(D), rb = key_bits(npvs);
                radix_sort_pairs(fx_lit.p, fx_rank.p, fx_k2.p, fx_v2.p, np, lb, radix_hist.p, radix_hscan.p,
                                 scan_tmp32.p, rt.stream);
                radix_sort_pairs(fx_rank.p, fx_lit.p, fx_k2.p, fx_v2.p, np, rb, radix_hist.p, radix_hscan.p,
                                 scan_tmp32.p, rt.stream);
                rt.launches += 5 * (lb / 8 + rb / 8);
                rt.each(FSubfxFirst{fx_rank.p, fx_lit.p, fx_flag.p}, np);
                nwant = scan32(fx_flag.p, fx_scan.p, np);
                want_rank.reserve(rt, (size_t)nwant + 1);
                want_lit.reserve(rt, (size_t)nwant + 1);
                rt.each(FSubfxScatter{fx_rank.p, fx_lit.p, fx_flag.p, fx_scan.p, want_rank.p, want_lit.p, want_cnt.p}, np);
            }
        }
        want_lit.reserve(rt, (size_t)nwant + 1);
        write_u32(want_off.p + npvs, scan32(want_cnt.p, want_off.p, npvs));
    }

    // SUB when units are possible (see k_sub.cuh): the producers settle by re-runs
    // from their checkpoint, then every other variable runs once with the
    // producers' units pre-deleted.
    void sub_safe(SubArgs a) {
        Ctx c = view();
        fx_prod8.reserve(rt, npvs + 1);
        fx_other8.reserve(rt, npvs + 1);
        sub_run.reserve(rt, npvs + 1);
        rt.each(FSubfxTo8{fx_prod.p, fx_prod8.p, false}, npvs);
        rt.each(FSubfxTo8{fx_prod.p, fx_other8.p, true}, npvs);
        // checkpoint of the producers
        sub_ent.reserve(rt, npvs + 1);
        sub_ent_off.reserve(rt, npvs + 1);
        sub_wrd.reserve(rt, npvs + 1);
        sub_wrd_off.reserve(rt, npvs + 1);
        rt.each(FSubNeed{c, pvs.p, fx_prod8.p, sub_ent.p, sub_wrd.p}, npvs);
        const u32 ents = scan32(sub_ent.p, sub_ent_off.p, npvs);
        const u64 words = scan64(sub_wrd.p, sub_wrd_off.p, npvs);
        sub_ids.reserve(rt, ents + 1);
        sub_hdrs.reserve(rt, ents + 1);
        sub_words.reserve(rt, (size_t)words + 1);
        sub_sizes.reserve(rt, 2 * npvs + 2);
        SubCkptArgs ck{c, pvs.p, sub_ent_off.p, sub_wrd_off.p, sub_ids.p, sub_hdrs.p, sub_words.p, sub_sizes.p,
                       fx_prod8.p};
        rt.each(FSubSave{ck}, npvs);
        // the producers' first run
        sub_units.reserve(rt, (size_t)ents + 16);
        sub_units2.reserve(rt, sub_units.n);
        a.units = sub_units.p;
        a.cap_units = (u32)sub_units.n;
        a.run = fx_prod8.p;
        write_u32(counters.p + 4, 0);
        kclock[K_SUB].start(rt);
        sub_pass(a);
        kclock[K_SUB].stop(rt);
        check();
        u32 nu = read_u32(counters.p + 4);
        // fix-point among the producers: a producer re-runs when the set of earlier
        // producers' units that reach it differs from the set its last run used
        used_off.reserve(rt, npvs + 1);
        used_lit.reserve(rt, 1);
        rt.zero(used_off.p, ((size_t)npvs + 1) * 4);
        fx_flag.reserve(rt, npvs + 1);
        fx_scan.reserve(rt, npvs + 1);
        for (u32 iter = 0;; iter++) {
            if (iter > npvs + 2) throw int(PF_ETIMEOUT);
            sub_unit_sets(nu, fx_prod8.p);
            fx_flag.reserve(rt, npvs + 1);
            fx_scan.reserve(rt, npvs + 1);
            rt.each(FSubfxDiff{want_off.p, want_lit.p, used_off.p, used_lit.p, fx_prod8.p, fx_flag.p, sub_run.p}, npvs);
            const u32 nrerun = scan32(fx_flag.p, fx_scan.p, npvs);
            if (!nrerun) break;
            // restore the re-runs; they use the new sets
            SubCkptArgs rk = ck;
            rk.c = view();
            rk.run = sub_run.p;
            rt.each(FSubRestore{rk}, npvs);
            std::swap(used_lit, want_lit);
            std::swap(used_off, want_off);
            // their old units go, the others' stay
            fx_flag.reserve(rt, (size_t)nu + 1);
            fx_scan.reserve(rt, (size_t)nu + 1);
            u32 nkeep = 0;
            if (nu) {
                rt.each(FSubfxKeep{sub_units.p, sub_run.p, fx_flag.p}, nu);
                nkeep = scan32(fx_flag.p, fx_scan.p, nu);
                rt.each(FSubfxKeepScatter{sub_units.p, fx_flag.p, fx_scan.p, sub_units2.p}, nu);
                std::swap(sub_units, sub_units2);
            }
            SubArgs b = a;
            b.c = view();
            b.units = sub_units.p;
            b.cap_units = (u32)sub_units.n;
            b.pre_off = used_off.p;
            b.pre_lits = used_lit.p;
            b.run = sub_run.p;
            write_u32(counters.p + 4, nkeep);
            sub_pass(b);
            check();
            nu = read_u32(counters.p + 4);
        }
        // every other variable once, with the units of the producers before it pre-deleted
        sub_unit_sets(nu, fx_other8.p);
        SubArgs b = a;
        b.c = view();
        b.units = sub_units.p;
        b.cap_units = (u32)sub_units.n;
        b.pre_off = want_off.p;
        b.pre_lits = want_lit.p;
        b.run = fx_other8.p;
        write_u32(counters.p + 4, nu);
        sub_pass(b);
        check();
        nu = read_u32(counters.p + 4);
        // commit: enqueueUnit + toblivion(ot[unit]). The reference commits in producer
        // order; the outcome does not depend on it (the same literals end assigned, an
        // opposite pair is a conflict either way), so the units go to the trail in
        // parallel, first claim wins, and the newly assigned ones empty their lists.
        if (!nu) return;
        const u32 before = ntrail;
        rt.each(FSubAssign{view(), sub_units.p}, nu);
        ntrail = read_u32(counters.p + 0);
        if (ntrail > before) {
            const u32 na = ntrail - before;
            const u32* ul = trail.p + before;
            big32a.reserve(rt, (size_t)na + 1);
            big32b.reserve(rt, (size_t)na + 1);
            rt.each(FSubCommitSize{view(), ul, big32a.p}, na);
            const u32 items = scan32(big32a.p, big32b.p, na);
            if (items) rt.each(FSubCommitItem{view(), ul, big32b.p, na}, items);
            rt.each(FSubCommitClear{view(), ul}, na);
        }
        check();
    }

    // VE (elimination.cpp:101-108) = bve (bve.cpp:28-142).
    void ve() {
        if (!opt.ve || !npvs) return;
        Ctx c = view();
        ve_type.reserve(rt, npvs);
        ve_porgs.reserve(rt, npvs);
        ve_norgs.reserve(rt, npvs);
        ve_ncls.reserve(rt, npvs);
        ve_nlits.reserve(rt, npvs);
        ve_nwit.reserve(rt, npvs);
        ve_def.reserve(rt, npvs);
        ve_cls_scan.reserve(rt, npvs);
        ve_scr_off.reserve(rt, npvs + 1);
        ve_lit_scan.reserve(rt, npvs);
        ve_wit_scan.reserve(rt, npvs);
        big64a.reserve(rt, npvs + 1);
        rt.each(FBveNeed{c, pvs.p, big64a.p}, npvs);
        scan_to(big64a.p, ve_scr_off.p, npvs, 0);
        read_slots_checked();
        const u64 scr_words = hr[0];
        ve_scr.reserve(rt, (size_t)scr_words + 16);
        BveArgs a;
        a.c = c;
        a.pvs = pvs.p;
        a.npvs = npvs;
        a.ve_clause_max = opt.ve_clause_max;
        a.ve_lbound = opt.ve_lbound;
        a.xor_max_arity = opt.xor_max_arity;
        a.type = ve_type.p;
        a.porgs = ve_porgs.p;
        a.norgs = ve_norgs.p;
        a.ncls = ve_ncls.p;
        a.nlits = ve_nlits.p;
        a.nwit = ve_nwit.p;
        a.def = ve_def.p;
        a.scr_off = ve_scr_off.p;
        a.scr = ve_scr.p;
        a.keep_at = keep_at.p;
        a.keep_shape = keep_shape.p;
#if SIGMA_CUDA
        {
            const int smem = kBveWarpThreads / 32 * (int)WPV_WORDS * 4;
            static bool attr_set = false;
            if (!attr_set) {
                ck(cudaFuncSetAttribute(bve_warp_k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem), "smem attr");
                attr_set = true;
            }
            ck(cudaMemsetAsync(counters.p + 11, 0, 4, rt.stream), "memset");
            rt.launches++;
            kclock[K_BVE].start(rt);
            bve_warp_k<<<pv_grid(), kBveWarpThreads, smem, rt.stream>>>(a, pv_perm.p, counters.p + 11);
            kclock[K_BVE].stop(rt);
            ck(cudaGetLastError(), "launch");
        }
#else
        kclock[K_BVE].start(rt);
        pv_each(FBveWarp{a});
        kclock[K_BVE].stop(rt);
#endif
        kbytes[K_BVE] += phase_ws;
        scan_to(ve_ncls.p, ve_cls_scan.p, npvs, 0);
        scan_to(ve_nlits.p, ve_lit_scan.p, npvs, 1);
        scan_to(ve_nwit.p, ve_wit_scan.p, npvs, 2);
        read_slots_checked();
        const u32 add_cls = (u32)hr[0];
        const u64 add_lits = hr[1], add_wit = hr[2];
        ensure_clauses((u64)ncls + add_cls);
        ensure_lits(nlits_used + add_lits);
        ensure_resolved(nresolved + add_wit);
        // substituted clauses (one line each) and the resolvents
        proof_reserve(phase_ws / 4 + add_lits + add_cls + 16);
        a.c = view();
        a.cls_scan = ve_cls_scan.p;
        a.lit_scan = ve_lit_scan.p;
        a.wit_scan = ve_wit_scan.p;
        a.cls_base = ncls;
        a.lit_base = nlits_used;
        a.wit_base = nresolved;
        kclock[K_BVEW].start(rt);
#if SIGMA_CUDA
        if (perm_n) {
            ck(cudaMemsetAsync(counters.p + 11, 0, 4, rt.stream), "memset");
            rt.launches++;
            bve_write_warp_k<<<pv_grid(), 256, 0, rt.stream>>>(a, pv_perm.p + perm_off, perm_n,
                                                                       counters.p + 11);
            ck(cudaGetLastError(), "launch");
        }
#else
        pv_each(FBveWrite{a});
#endif
        kclock[K_BVEW].stop(rt);
        kbytes[K_BVEW] += phase_ws + 4ull * add_lits + 8ull * add_cls + 4ull * add_wit;
        const u32 first_new = ncls;
        ncls += add_cls;
        nlits_used += add_lits;
        proof_clauses(first_new);
        nresolved += add_wit;
        word_to(counters.p + 0, 0);
        read_slots_checked();
        ntrail = (u32)hr[0];
        alg_bytes += 4ull * add_lits + 8ull * add_cls + 4ull * add_wit;
    }

    // BCE (elimination.cpp:131-167).
    void bce() {
        if (!opt.bce || !npvs) return;
        BceArgs a;
        a.c = view();
        a.pvs = pvs.p;
        a.bce_max = (u32)opt.bce_max;
        ve_nwit.reserve(rt, npvs);
        ve_wit_scan.reserve(rt, npvs);
        a.nwit = ve_nwit.p;
#if SIGMA_CUDA
        if (perm_n) {
            ck(cudaMemsetAsync(counters.p + 11, 0, 4, rt.stream), "memset");
            rt.launches++;
            bce_count_warp_k<<<pv_grid(), 256, 0, rt.stream>>>(a, pv_perm.p + perm_off, perm_n, counters.p + 11);
            ck(cudaGetLastError(), "launch");
        }
#else
        pv_each(FBceCountWarp{a});
#endif
        scan_to(ve_nwit.p, ve_wit_scan.p, npvs, 0);
        read_slots_checked();
        const u64 add = hr[0];
        if (!add) return;
        ensure_resolved(nresolved + add);
        a.c = view();
        a.wit_scan = ve_wit_scan.p;
        a.wit_base = nresolved;
        pv_each(FBceWrite{a});
        nresolved += add;
        alg_bytes += 4ull * add;
    }

    // ERE (elimination.cpp:169-197).
    void ere() {
        if (!opt.ere || !npvs) return;
        proof_reserve(nlits_used + ncls + 16);  // a deletion line per clause at most
        if (opt.ere_max > 65535) throw std::runtime_error("eremax above 65535 is not supported");
        EreArgs a;
        a.c = view();
        a.pvs = pvs.p;
        a.npvs = npvs;
        a.ere_max = (u32)opt.ere_max;
        a.ere_clause_max = opt.ere_clause_max;
        if (has_learnt) {
            rt.one(FEreSeq{a});
            rt.sync();
            return;
        }
        ere_claim.reserve(rt, hdr.n);
        rt.zero(ere_claim.p, (size_t)ncls * 8, 0xFF);
        const size_t cap_rec = (size_t)ncls + (1u << 20);
        ere_target.reserve(rt, cap_rec);
        ere_key.reserve(rt, cap_rec);
        ere_losers.reserve(rt, cap_rec);
        a.claim = ere_claim.p;
        a.rec_target = ere_target.p;
        a.rec_key = ere_key.p;
        a.nrec = counters.p + 7;
        a.cap_rec = (u32)cap_rec;
        a.losers = ere_losers.p;
        a.nlosers = counters.p + 8;
        write_u32(counters.p + 7, 0);
        write_u32(counters.p + 8, 0);
        // one item per (variable, i, j) pair when the pair count fits 32-bit items
        big64a.reserve(rt, (size_t)perm_n + 1);
        big64b.reserve(rt, (size_t)perm_n + 1);
        rt.each(FEreCount{a, pv_perm.p + perm_off, big64a.p}, perm_n);
        const u64 pairs = scan64(big64a.p, big64b.p, perm_n);
        if (pairs < 0xFFFFFFF0ull) rt.each(FErePair{a, pv_perm.p + perm_off, big64b.p, perm_n}, (u32)pairs);
        else pv_each(FEre{a});
        check();
        const u32 nrec = read_u32(counters.p + 7);
        rt.each(FEreResolve{a}, nrec);
        const u32 nl = read_u32(counters.p + 8);
        if (nl) {
            // the losers' keys in ascending order, sorted on the device: by the low
            // word (pair), then stably by the high word (elected rank)
            big32a.reserve(rt, (size_t)nl + 1);
            big32b.reserve(rt, (size_t)nl + 1);
            work.reserve(rt, 2 * (size_t)nl + 2);
            big64b.reserve(rt, (size_t)nl + 1);
            radix_hist.reserve(rt, radix_hist_elems(nl));
            radix_hscan.reserve(rt, radix_hist_elems(nl));
            scan_tmp32.reserve(rt, scan_tmp_elems(radix_hist_elems(nl)) + 4);
            rt.each(FEreLoserKey{ere_key.p, ere_losers.p, big32b.p, big32a.p, false}, nl);
            radix_sort_pairs(big32a.p, big32b.p, work.p, work.p + nl + 1, nl, 32, radix_hist.p, radix_hscan.p,
                             scan_tmp32.p, rt.stream);
            rt.each(FEreLoserKey{ere_key.p, ere_losers.p, big32b.p, big32a.p, true}, nl);
            const int rb = key_bits(npvs);
            radix_sort_pairs(big32a.p, big32b.p, work.p, work.p + nl + 1, nl, rb, radix_hist.p, radix_hscan.p,
                             scan_tmp32.p, rt.stream);
            rt.launches += 5 * (4 + rb / 8);
            rt.each(FEreLoserGather{ere_key.p, ere_losers.p, big32b.p, big64b.p}, nl);
            rt.one(FEreFix{a, big64b.p, nl});
        }
    }

    // countAll (solve.h:724-734).
    void count_all() {
        rt.zero(counters64.p + 2, 16);
        CountArgs a{view(), counters64.p + 2};
#if SIGMA_CUDA
        if (ncls) {
            rt.launches++;
            count_live_k<<<rt.grid(ncls, 4), 256, 0, rt.stream>>>(a.c.hdr, ncls, a.out);
            ck(cudaGetLastError(), "launch");
        }
#else
        rt.each(FCount{a}, ncls);
#endif
        rt.d2d(hslot(0), counters64.p + 2, 16);
        read_slots_checked();
        n_cls_after = (i64)hr[0];
        n_lits_after = (i64)hr[1];
    }

    // shrinkSimp (simplify.cpp:234-245).
    void gc() {
        if (!ncls) {
            compact = true;
            return;
        }
        big32a.reserve(rt, (size_t)ncls + 1);
        big32b.reserve(rt, (size_t)ncls + 1);
        big64a.reserve(rt, (size_t)ncls + 1);
        big64b.reserve(rt, (size_t)ncls + 1);
        Ctx c = view();
        rt.each(FGcFlags{c, big32a.p, big64a.p}, ncls);
        scan_to(big32a.p, big32b.p, ncls, 0);
        scan_to(big64a.p, big64b.p, ncls, 1);
        read_slots_checked();
        const u32 keep = (u32)hr[0];
        const u64 keep_lits = hr[1];
        hdr2.reserve(rt, hdr.n);
        cstamp2.reserve(rt, hdr.n);
        lits2.reserve(rt, std::max<size_t>(lits.n, (size_t)keep_lits + 16));
        GcArgs g{c, big32b.p, big64b.p, hdr2.p, lits2.p, cstamp2.p};
        rt.each(FGcMove{g}, ncls);
        std::swap(hdr, hdr2);
        std::swap(cstamp, cstamp2);
        std::swap(lits, lits2);
        alg_bytes += (4ull * nlits_used + 8ull * ncls) + (4ull * keep_lits + 8ull * keep);
        ncls = keep;
        nlits_used = keep_lits;
        compact = true;
    }

    // resizeCNF (solve.h:684-688). Besides the reference's schedule, a large store
    // whose live clauses fill less than a quarter of its slots is compacted too: the
    // compaction keeps the clauses' order, so no result of the round changes, and the
    // next phase's passes over the store (table build, sweeps, clause records) stop
    // walking dead slots. Not while stage dumps are written (they name clauses by
    // their place in the store).
    void resize_cnf() {
        const int times = phase + 1;
        const bool sched = opt.gc_freq > 0 && times > 1 && times != opt.phases && (times % opt.gc_freq) == 0;
        const bool sparse = opt.dump_level == 0 && ncls >= kSparseGcMin && (u64)n_cls_after * 4 < ncls;
        if (sched || sparse) gc();
    }
    static constexpr u32 kSparseGcMin = 1u << 20;

    // Rounds a device-side loop may run (election rounds, propagation waves).
    u32 loop_bound() const { return opt.loop_limit > 0 ? (u32)opt.loop_limit : nvars + 2; }

    bool stop(i64 lr) const { return phase == opt.phases || (lr <= opt.ve_phase_min && phase > 2); }

    // Per-phase figures of the round (pf_round_stats phase_*): opened at the top of
    // a phase with the live counts entering it, closed where the phase ends.
    u64 ph_bytes0 = 0;
    double ph_ms0 = 0;
    double stage_ms_sum() const {
        double t = 0;
        for (double x : st.ms_stage) t += x;
        return t;
    }
    void phase_open(i64 cls, i64 lits) {
        if (phase >= 8) return;
        st.phase_clauses[phase] = (u64)cls;
        st.phase_literals[phase] = (u64)lits;
        ph_bytes0 = alg_bytes;
        ph_ms0 = stage_ms_sum();
    }
    void phase_close() {
        if (phase >= 8) return;
        st.phase_elected[phase] = npvs;
        st.phase_bytes[phase] = alg_bytes - ph_bytes0;
        st.phase_ms[phase] = stage_ms_sum() - ph_ms0;
    }

    double timed(int stage, void (pf_sigma_ctx::*fn)()) {
        tm.start(rt);
        (this->*fn)();
        const double ms = tm.stop(rt);
        st.ms_stage[stage] += ms;
        return ms;
    }

    // Units of the input (one-literal clauses) before the first phase: the
    // reference's sigmifying() starts with rootify() + shrinkTop() (root-level
    // propagation, then satisfied clauses dropped and false literals removed,
    // src/cpu/simplify.cpp:163-164, shrink.cpp:152-216), so its first occurrence
    // table holds only the clauses that survive them. Here: a table, the
    // propagation, then a compaction of the store.
    void root_units() {
        if (prop_head >= ntrail) return;
        timed(ST_OT, &pf_sigma_ctx::create_ot);
        timed(ST_PROP, &pf_sigma_ctx::prop);
        timed(ST_GC, &pf_sigma_ctx::gc);
        compact = false;
    }

    // sigmifying (simplify.cpp:182-209).
    void round() {
        phase = 0;
        mu_inc = 0;
        root_units();
        count_all();
        i64 litsbefore = n_lits_after, diff = INT64_MAX;
        st.clauses_before = (u64)n_cls_after;
        st.literals_before = (u64)n_lits_after;
        while (litsbefore) {
            phase_open(n_cls_after, litsbefore);
            timed(ST_GC, &pf_sigma_ctx::resize_cnf);
            timed(ST_OT, &pf_sigma_ctx::create_ot);
            timed(ST_PROP, &pf_sigma_ctx::prop);
            if (opt.dump_level >= 2) {
                rec(2, phase, 1, fetch(ot_size.p, D));
                dump_stage(phase, 1);
            }
            tm.start(rt);
            const bool go = lcve();
            st.ms_stage[ST_LCVE] += tm.stop(rt);
            if (!go) {
                phase_close();
                break;
            }
            timed(ST_SORT, &pf_sigma_ctx::sort_ot);
            if (opt.dump_level >= 2) dump_pvlists(phase);
            const u64 W = pv_bytes();
            phase_ws = W;
            alg_bytes += 2ull * W;  // sort reads and writes the lists (8*occ) ~ bounded by W
            if (stop(diff)) {
                timed(ST_ERE, &pf_sigma_ctx::ere);
                alg_bytes += W;
                dump_stage(phase, 7);
                phase_close();
                break;
            }
            timed(ST_SUB, &pf_sigma_ctx::sub);
            dump_stage(phase, 4);
            timed(ST_VE, &pf_sigma_ctx::ve);
            dump_stage(phase, 5);
            timed(ST_BCE, &pf_sigma_ctx::bce);
            dump_stage(phase, 6);
            alg_bytes += 4ull * W;
            timed(ST_COUNT, &pf_sigma_ctx::count_all);
            phase_close();
            if (opt.dump_level >= 1) {
                rec(10, phase, 6, {(u32)n_cls_after, (u32)n_lits_after});
                dump_elim(phase, 6);
            }
            diff = litsbefore - n_lits_after;
            litsbefore = n_lits_after;
            phase++;
            mu_inc++;
            mu_inc += (phase == opt.phases);
        }
        timed(ST_PROP, &pf_sigma_ctx::prop);
        timed(ST_COUNT, &pf_sigma_ctx::count_all);
        timed(ST_GC, &pf_sigma_ctx::gc);
        st.phases_run = phase;
    }

    // Clauses of a batch's store grouped by formula (store order inside a formula,
    // literals in the formula's numbering) straight into host buffers.
    void batch_clauses_to(u32* h_lits, u64* h_off, uint8_t* h_learnt) {
        const u32 n = ncls;
        if (!n) {
            if (h_off) h_off[0] = 0;
            return;
        }
        big32a.reserve(rt, (size_t)n + 1);
        big32b.reserve(rt, (size_t)n + 1);
        work.reserve(rt, 2 * (size_t)n + 2);
        radix_hist.reserve(rt, radix_hist_elems(n));
        radix_hscan.reserve(rt, radix_hist_elems(n));
        scan_tmp32.reserve(rt, scan_tmp_elems(radix_hist_elems(n)) + 4);
        const Ctx c = view();
        rt.each(FClauseFid{c, big32a.p, big32b.p}, n);
        int bits = 8;
        while (bits < 32 && (nf >> bits)) bits += 8;
        radix_sort_pairs(big32a.p, big32b.p, work.p, work.p + n + 1, n, bits, radix_hist.p, radix_hscan.p,
                         scan_tmp32.p, rt.stream);
        rt.launches += 3 * (bits / 8);
        big64a.reserve(rt, (size_t)n + 1);
        big64b.reserve(rt, (size_t)n + 1);
        DBuf<uint8_t> lrn;
        lrn.reserve(rt, n);
        rt.each(FClauseSize{c, big32b.p, big64a.p, lrn.p}, n);
        const u64 total = scan64(big64a.p, big64b.p, n);
        write_u64(big64b.p + n, total);
        lits2.reserve(rt, (size_t)total + 1);
        rt.each(FClauseGather{c, big32b.p, big32a.p, big64b.p, f_var.p, lits2.p}, n);
        if (h_lits) rt.d2h(h_lits, lits2.p, (size_t)total * 4);
        if (h_off) rt.d2h(h_off, big64b.p, ((size_t)n + 1) * 8);
        if (h_learnt) rt.d2h(h_learnt, lrn.p, n);
        lrn.free();
    }

    int fid_bits() const {
        int bits = 8;
        while (bits < 32 && (nf >> bits)) bits += 8;
        return bits;
    }

    // Witness records grouped per formula (records in order inside a formula): the
    // word count per formula, and with h_out the words in each formula's numbering.
    void batch_witness(std::vector<u64>& f_words_out, u32* h_out) {
        const u64 W = nresolved;
        f_words_out.assign(nf, 0);
        if (!W) return;
        if (W >= 0xFFFFFFF0ull) throw std::runtime_error("witness stack too large for 32-bit positions");
        const u32 w = (u32)W;
        DBuf<u32> flag, scan, rstart, key, val, k2, v2, out;
        DBuf<u64> words, size, off, fw;
        flag.reserve(rt, w);
        scan.reserve(rt, w);
        rt.each(FRecStart{res_mark.p, flag.p}, w);
        const u32 R = scan32(flag.p, scan.p, w);
        rstart.reserve(rt, R + 1);
        rt.each(FRecScatter{flag.p, scan.p, rstart.p}, w);
        key.reserve(rt, R + 1);
        val.reserve(rt, R + 1);
        words.reserve(rt, R + 1);
        fw.reserve(rt, nf);
        rt.zero(fw.p, (size_t)nf * 8);
        const Ctx c = view();
        rt.each(FRecFid{c, rstart.p, R, w, key.p, val.p, words.p, fw.p}, R);
        rt.d2h(f_words_out.data(), fw.p, (size_t)nf * 8);
        if (!h_out) return;
        k2.reserve(rt, R + 1);
        v2.reserve(rt, R + 1);
        radix_hist.reserve(rt, radix_hist_elems(R));
        radix_hscan.reserve(rt, radix_hist_elems(R));
        scan_tmp32.reserve(rt, scan_tmp_elems(radix_hist_elems(R)) + 4);
        const int bits = fid_bits();
        radix_sort_pairs(key.p, val.p, k2.p, v2.p, R, bits, radix_hist.p, radix_hscan.p, scan_tmp32.p, rt.stream);
        rt.launches += 5 * (bits / 8);
        size.reserve(rt, R + 1);
        off.reserve(rt, R + 1);
        rt.each(FRecSize{words.p, val.p, size.p}, R);
        scan64(size.p, off.p, R);
        out.reserve(rt, w);
        rt.each(FRecGather{c, rstart.p, val.p, key.p, words.p, off.p, f_var.p, out.p}, R);
        rt.d2h(h_out, out.p, (size_t)w * 4);
    }

    // MODEL::extend (src/cpu/model.cpp:104-138) on the device for the last round's
    // result: h_values holds the caller's model of the simplified formula(s) and
    // receives the model of the original one(s). A batch's formulas are walked side
    // by side, one thread each.
    void extend(uint8_t* h_values) {
        DBuf<uint8_t> val, packed;
        DBuf<u64> pfirst;
        val.reserve(rt, (size_t)nvars + 1);
        ExtendMap m{nullptr, nf ? f_var.p : nullptr, nf};
        u64 npacked = 0;
        if (!nf) {
            rt.h2d(val.p, h_values, (size_t)nvars + 1);
        } else {
            std::vector<u64> first(nf + 1, 0);
            for (u32 f = 0; f < nf; f++) first[f + 1] = first[f] + h_f_nv[f] + 1;
            npacked = first[nf];
            if (npacked >= 0xFFFFFFF0ull) throw std::runtime_error("batch values exceed 32-bit positions");
            pfirst.reserve(rt, nf + 1);
            rt.h2d(pfirst.p, first.data(), (size_t)(nf + 1) * 8);
            packed.reserve(rt, npacked);
            rt.h2d(packed.p, h_values, npacked);
            rt.zero(val.p, (size_t)nvars + 1);
            m.p_first = pfirst.p;
            rt.each(FExtendIn{m, packed.p, val.p}, (u32)npacked);
        }
        const Ctx c = view();
        rt.each(FExtendClear{c, val.p}, nvars + 1);
        if (ntrail) rt.each(FExtendUnit{c, val.p}, ntrail);
        ExtendArgs a{};
        a.resolved = resolved.p;
        a.value = val.p;
        a.nres = nresolved;
        a.err = counters.p + 1;
        DBuf<u32> flag, scan, rstart, key, ord, k2, v2, frec, ffirst;
        DBuf<u64> words, fw;
        if (!nf) {
            if (nresolved) rt.one(FExtendSingle{a});
        } else if (nresolved) {
            if (nresolved >= 0xFFFFFFF0ull) throw std::runtime_error("witness stack too large for 32-bit positions");
            const u32 w = (u32)nresolved;
            flag.reserve(rt, w);
            scan.reserve(rt, w);
            rt.each(FRecStart{res_mark.p, flag.p}, w);
            const u32 R = scan32(flag.p, scan.p, w);
            rstart.reserve(rt, R + 1);
            rt.each(FRecScatter{flag.p, scan.p, rstart.p}, w);
            key.reserve(rt, R + 1);
            ord.reserve(rt, R + 1);
            words.reserve(rt, R + 1);
            fw.reserve(rt, nf);
            rt.zero(fw.p, (size_t)nf * 8);
            rt.each(FRecFid{c, rstart.p, R, w, key.p, ord.p, words.p, fw.p}, R);
            k2.reserve(rt, R + 1);
            v2.reserve(rt, R + 1);
            radix_hist.reserve(rt, radix_hist_elems(R));
            radix_hscan.reserve(rt, radix_hist_elems(R));
            scan_tmp32.reserve(rt, scan_tmp_elems(radix_hist_elems(R)) + 4);
            const int bits = fid_bits();
            radix_sort_pairs(key.p, ord.p, k2.p, v2.p, R, bits, radix_hist.p, radix_hscan.p, scan_tmp32.p, rt.stream);
            rt.launches += 5 * (bits / 8);
            frec.reserve(rt, nf + 1);
            ffirst.reserve(rt, nf + 1);
            rt.zero(frec.p, (size_t)(nf + 1) * 4);
            rt.each(FRecCount{c, rstart.p, frec.p}, R);
            write_u32(ffirst.p + nf, scan32(frec.p, ffirst.p, nf));
            a.rec_start = rstart.p;
            a.rec_words = words.p;
            a.order = ord.p;
            a.f_first = ffirst.p;
            rt.each(FExtendFormula{a}, nf);
        }
        check();
        if (!nf) {
            rt.d2h(h_values, val.p, (size_t)nvars + 1);
        } else {
            rt.each(FExtendOut{m, val.p, packed.p}, (u32)npacked);
            rt.d2h(h_values, packed.p, npacked);
        }
    }

    // Trail units grouped per formula, in the formula's numbering.
    void batch_units(std::vector<u64>& f_units_out, u32* h_out) {
        f_units_out.assign(nf, 0);
        const u32 n = ntrail;
        if (!n) return;
        DBuf<u32> key, val, k2, v2, out;
        DBuf<u64> fu;
        key.reserve(rt, n);
        val.reserve(rt, n);
        fu.reserve(rt, nf);
        rt.zero(fu.p, (size_t)nf * 8);
        const Ctx c = view();
        rt.each(FUnitFid{c, key.p, val.p, fu.p}, n);
        rt.d2h(f_units_out.data(), fu.p, (size_t)nf * 8);
        if (!h_out) return;
        k2.reserve(rt, n);
        v2.reserve(rt, n);
        radix_hist.reserve(rt, radix_hist_elems(n));
        radix_hscan.reserve(rt, radix_hist_elems(n));
        scan_tmp32.reserve(rt, scan_tmp_elems(radix_hist_elems(n)) + 4);
        const int bits = fid_bits();
        radix_sort_pairs(key.p, val.p, k2.p, v2.p, n, bits, radix_hist.p, radix_hscan.p, scan_tmp32.p, rt.stream);
        rt.launches += 5 * (bits / 8);
        out.reserve(rt, n);
        rt.each(FUnitGather{c, val.p, key.p, f_var.p, out.p}, n);
        rt.d2h(h_out, out.p, (size_t)n * 4);
    }

    // Formula of a literal of the store, on the host.
    u32 host_fid(u32 lit) const {
        const u32 v = ABS(lit);
        u32 lo = 0, hi = nf;
        while (hi - lo > 1) {
            const u32 mid = (lo + hi) >> 1;
            if (h_f_var[mid] < v) lo = mid;
            else hi = mid;
        }
        return lo;
    }

    // ------------------------------------------------------------ formula batches
    // Each formula of a batch runs its own sigmifying loop; the formulas share the
    // store, so one phase does the stage kernels once for all formulas still in their
    // loop. Formulas never share variables or clauses, so every stage's result for a
    // formula is the one it would have alone: the election's order restricted to a
    // formula is that formula's own (score, variable) order, its bounds are kept per
    // formula, and new clauses and witness words keep each formula's relative order.
    // A formula leaves the loop exactly where its own would end; its final
    // propagation then happens in the next phase's (or the closing) propagation.
    std::vector<u64> fc_cls, fc_lits;

    void count_formulas() {
        rt.zero(f_count.p, (size_t)nf * 16);
        FormulaCountArgs a{view(), f_count.p, f_count.p + nf};
#if SIGMA_CUDA
        if (ncls) {
            rt.launches++;
            count_formula_k<<<rt.grid(ncls, 4), 256, 0, rt.stream>>>(a, ncls);
            ck(cudaGetLastError(), "launch");
        }
#else
        rt.each(FCountFormula{a}, ncls);
#endif
        std::vector<u64> h = fetch(f_count.p, 2 * (size_t)nf);
        fc_cls.assign(h.begin(), h.begin() + nf);
        fc_lits.assign(h.begin() + nf, h.end());
        n_cls_after = n_lits_after = 0;
        for (u32 f = 0; f < nf; f++) {
            n_cls_after += (i64)fc_cls[f];
            n_lits_after += (i64)fc_lits[f];
        }
    }

    // Formulas that derived the empty clause leave the loop with status UNSAT.
    void mark_unsat(std::vector<uint8_t>& done) {
        const std::vector<u32> e = fetch(f_err.p, nf);
        for (u32 f = 0; f < nf; f++) {
            if ((e[f] & ERR_UNSAT) && f_status[f] != PF_UNSAT) {
                f_status[f] = PF_UNSAT;
                f_phases[f] = 0;  // as a single round stopped by the empty clause reports
                done[f] = 1;
            }
        }
    }

    // Orders the elected list as [formulas that go on | formulas that stop this
    // phase]; elected variables of dropped formulas leave it. group: per formula.
    void partition_pvs(const std::vector<u32>& group) {
        rt.h2d(f_group.p, group.data(), (size_t)nf * 4);
        big32a.reserve(rt, (size_t)npvs + 1);
        big32b.reserve(rt, (size_t)npvs + 1);
        const Ctx c = view();
        rt.each(FPvGroup{c, pvs.p, f_group.p, flags.p, big32a.p}, npvs);
        const u32 ngo = scan32(flags.p, flags_scan.p, npvs);
        const u32 nstop = scan32(big32a.p, big32b.p, npvs);
        pv_key.reserve(rt, nvars + 1);
        rt.each(FPvPartition{c, pvs.p, flags.p, flags_scan.p, big32a.p, big32b.p, ngo, pv_key.p}, npvs);
        rt.d2d(pvs.p, pv_key.p, (size_t)(ngo + nstop) * 4);
        npvs = ngo + nstop;
        n_go = ngo;
    }

    void round_batch() {
        phase = 0;
        mu_inc = 0;
        std::fill(f_status.begin(), f_status.end(), (int)PF_OK);
        std::fill(f_phases.begin(), f_phases.end(), 0u);
        std::vector<uint8_t> done(nf, 0);
        root_units();
        count_formulas();
        st.clauses_before = (u64)n_cls_after;
        st.literals_before = (u64)n_lits_after;
        const pf_options& o = opt;
        if (!o.phases && !(o.all || o.ere)) return;
        std::vector<i64> litsbefore(nf), diff(nf, INT64_MAX);
        for (u32 f = 0; f < nf; f++) {
            litsbefore[f] = (i64)fc_lits[f];
            if (!litsbefore[f]) done[f] = 1;
        }
        std::vector<u32> active(nf), group(nf);
        for (;;) {
            bool any = false;
            for (u32 f = 0; f < nf; f++) any |= !done[f];
            if (!any) break;
            phase_open(n_cls_after, n_lits_after);
            timed(ST_GC, &pf_sigma_ctx::resize_cnf);
            timed(ST_OT, &pf_sigma_ctx::create_ot);
            timed(ST_PROP, &pf_sigma_ctx::prop);
            mark_unsat(done);
            for (u32 f = 0; f < nf; f++) active[f] = !done[f];
            rt.h2d(f_active.p, active.data(), (size_t)nf * 4);
            tm.start(rt);
            lcve();
            const std::vector<u32> fn = fetch(f_npvs.p, nf);
            u32 going = 0;
            for (u32 f = 0; f < nf; f++) {
                group[f] = 0;
                if (done[f]) continue;
                if (fn[f] < (u32)o.lcve_min) {  // LCVE() false: leave the loop
                    done[f] = 1;
                    f_phases[f] = (u32)phase;
                } else {
                    group[f] = stop(diff[f]) ? 2u : 1u;
                    going++;
                }
            }
            partition_pvs(group);
            st.ms_stage[ST_LCVE] += tm.stop(rt);
            if (!going) {
                phase_close();
                continue;
            }
            timed(ST_SORT, &pf_sigma_ctx::sort_ot);
            const u64 W = pv_bytes();
            phase_ws = W;
            alg_bytes += 2ull * W;
            const u32 all = npvs;
            if (n_go < all) {  // stop(diff): ERE, then leave the loop
                perm_off = n_go;
                perm_n = all - n_go;
                timed(ST_ERE, &pf_sigma_ctx::ere);
            }
            if (n_go) {
                npvs = n_go;
                perm_off = 0;
                perm_n = n_go;
                timed(ST_SUB, &pf_sigma_ctx::sub);
                timed(ST_VE, &pf_sigma_ctx::ve);
                timed(ST_BCE, &pf_sigma_ctx::bce);
                npvs = all;
            }
            alg_bytes += 4ull * W;
            timed(ST_COUNT, &pf_sigma_ctx::count_formulas);
            phase_close();
            mark_unsat(done);
            for (u32 f = 0; f < nf; f++) {
                if (done[f]) continue;
                if (group[f] == 2) {
                    done[f] = 1;
                    f_phases[f] = (u32)phase;
                } else if (group[f] == 1) {
                    diff[f] = litsbefore[f] - (i64)fc_lits[f];
                    litsbefore[f] = (i64)fc_lits[f];
                    if (!litsbefore[f]) {
                        done[f] = 1;
                        f_phases[f] = (u32)phase + 1;
                    }
                }
            }
            phase++;
            mu_inc++;
            mu_inc += (phase == o.phases);
        }
        timed(ST_PROP, &pf_sigma_ctx::prop);
        timed(ST_COUNT, &pf_sigma_ctx::count_formulas);
        mark_unsat(done);
        timed(ST_GC, &pf_sigma_ctx::gc);
        st.phases_run = phase;
    }
};

// ---------------------------------------------------------------- C ABI
static pf_status fail(const std::string& m, pf_status s) {
    g_last_error = m;
    return s;
}

template <class F>
static pf_status guarded(F f) {
    try {
        return f();
    } catch (int code) {
        if (code == PF_UNSAT) return PF_UNSAT;
        return fail("stopped with status " + std::to_string(code), (pf_status)code);
    } catch (OomError& e) {
        return fail(e.what(), PF_ENOMEM);
    } catch (CudaError& e) {
        return fail(e.what(), PF_EDEVICE);
    } catch (std::exception& e) {
        return fail(e.what(), PF_EDEVICE);
    }
}

extern "C" {

void pf_default_options(pf_options* o) {
    std::memset(o, 0, sizeof(*o));
    o->phases = 5; o->all = 0; o->ve = 1; o->ve_plus = 1; o->sub = 1; o->bce = 0; o->ere = 1;
    o->ve_lbound = 0; o->ve_clause_max = 100; o->ve_phase_min = 500; o->mu_pos = 32; o->mu_neg = 32;
    o->xor_max_arity = 10; o->sub_max = 3000; o->bce_max = 3000; o->ere_max = 3000;
    o->ere_clause_max = 1000; o->lcve_min = 1; o->gc_freq = 2; o->dump_level = 0;
}

void pf_derive_options(pf_options* o) {
    o->ve = (o->ve || o->ve_plus) ? 1 : 0;
    if (o->all) { o->ve = 1; o->ve_plus = 1; o->bce = 1; o->ere = 1; }
    if (!o->phases && (o->ve || o->sub || o->bce)) o->phases = 1;
    if (o->phases && !(o->ve || o->sub || o->bce)) o->phases = 0;
    if (o->phases > 1 && !o->ve) o->phases = 1;
}

pf_status pf_sigma_create(const pf_options* opts, pf_sigma_ctx** out) {
    if (!out) return fail("null output pointer", PF_EINVAL);
    *out = nullptr;
    pf_sigma_ctx* c = new pf_sigma_ctx();
    try {
        if (opts) c->opt = *opts;
        else pf_default_options(&c->opt);
        if (c->opt.xor_max_arity > 20 || c->opt.xor_max_arity < 2) {
            delete c;
            return fail("xormaxarity must be in [2, 20]", PF_EINVAL);
        }
        c->rt.init();
        c->tm.init();
        c->counters.reserve(c->rt, 32);
        c->counters64.reserve(c->rt, 8);
        c->rt.zero(c->counters.p, 32 * 4);
        c->rt.zero(c->counters64.p, 8 * 8);
        c->rt.sync();
    } catch (std::exception& e) {
        delete c;
        return fail(e.what(), PF_EDEVICE);
    }
    *out = c;
    return PF_OK;
}

// Variable offsets of a batch's formulas in the store's numbering. Each formula's
// range starts at a multiple of 16 variables, so its literals move by a multiple of
// 32 and keep their signature bits (1 << (lit & 31)): clause signatures, and the
// occurrence-list order they take part in, are the formula's own.
static std::vector<u32> batch_var_offsets(u32 nf, const uint32_t* num_vars) {
    std::vector<u32> off(nf + 1, 0);
    for (u32 f = 0; f < nf; f++) off[f + 1] = off[f] + ((num_vars[f] + 15u) & ~15u);
    return off;
}

// Formula batch of an upload: nf formulas with their variable counts and clause
// ranges (host arrays).
struct BatchSpec {
    u32 nf;
    const uint32_t* num_vars;
    const uint64_t* clause_begin;
    // formulas in separate host arrays (null: one concatenated lits/offsets pair)
    const uint32_t* const* part_lits = nullptr;
    const uint64_t* const* part_offsets = nullptr;
};

static pf_status upload_common(pf_sigma_ctx* ctx, uint32_t num_vars, const uint32_t* lits, const uint64_t* offsets,
                               uint64_t num_clauses, const uint8_t* learnt, bool device,
                               const BatchSpec* batch = nullptr) {
    if (!ctx) return fail("null context", PF_EINVAL);
    if (!lits || !offsets || num_vars == 0) return fail("null formula", PF_EINVAL);
    if (num_vars >= (1u << 30)) return fail("too many variables", PF_EINVAL);
    if (num_clauses >= 0xFFFFFF00ull) return fail("too many clauses", PF_EINVAL);
    return guarded([&]() -> pf_status {
        pf_sigma_ctx& c = *ctx;
        Runtime& rt = c.rt;
        u64 off0 = 0, offn = 0;
        const bool parts = batch && batch->part_lits;
        if (parts) {
            for (u32 f = 0; f < batch->nf; f++) {
                const u64 nc = batch->clause_begin[f + 1] - batch->clause_begin[f];
                const u64* o = batch->part_offsets[f];
                if (o[nc] < o[0]) return fail("offsets not ascending", PF_EINVAL);
                offn += o[nc] - o[0];
            }
        } else if (device) {
            rt.d2h(&off0, offsets, 8);
            rt.d2h(&offn, offsets + num_clauses, 8);
        } else {
            off0 = offsets[0];
            offn = offsets[num_clauses];
        }
        if (offn < off0) return fail("offsets not ascending", PF_EINVAL);
        const u64 L = offn - off0;
        if (L >= 0xF0000000ull) return fail("too many literals", PF_EINVAL);
        c.nvars = num_vars;
        c.D = 2 * (num_vars + 1);
        c.nf = batch ? batch->nf : 0u;
            c.fc_cls.clear();
        c.fc_lits.clear();
        c.ncls = (u32)num_clauses;
        c.nlits_used = L;
        c.ntrail = c.prop_head = 0;
        c.nresolved = 0;
        c.has_learnt = false;
        const size_t cap_cls = (size_t)num_clauses + num_clauses / 2 + 1024;
        const size_t cap_lits = (size_t)L + L / 2 + 4096;
        c.hdr.reserve(rt, cap_cls);
        c.cstamp.reserve(rt, cap_cls);
        rt.zero(c.cstamp.p, cap_cls * 4);
        c.lits.reserve(rt, cap_lits);
        c.cl_stamp.reserve(rt, cap_cls);
        rt.zero(c.cl_stamp.p, cap_cls * 4);
        c.wave_stamp = 0;
        c.ot_off.reserve(rt, c.D + 1);
        c.ot_size.reserve(rt, c.D);
        c.ot_cursor.reserve(rt, c.D);
        c.ot_refs.reserve(rt, cap_lits);
        c.asg.reserve(rt, num_vars + 1);
        c.vstate.reserve(rt, num_vars + 1);
        c.ps.reserve(rt, num_vars + 1);
        c.ns.reserve(rt, num_vars + 1);
        c.pvrank.reserve(rt, num_vars + 1);
        c.trail.reserve(rt, num_vars + 1);
        c.resolved.reserve(rt, (size_t)L + 2 * (size_t)num_vars + 4096);
        c.score.reserve(rt, num_vars + 1);
        c.order.reserve(rt, num_vars + 1);
        c.order_k2.reserve(rt, num_vars + 1);
        c.order_v2.reserve(rt, num_vars + 1);
        c.rank.reserve(rt, num_vars + 1);
        c.bound.reserve(rt, 4);  // a batch upload widens it to two words per formula
        c.pvs.reserve(rt, num_vars + 1);
        c.flags.reserve(rt, num_vars + 1);
        c.flags_scan.reserve(rt, num_vars + 1);
        c.mis_word.reserve(rt, num_vars + 1);
        c.mis_resume.reserve(rt, num_vars + 1);
        c.radix_hist.reserve(rt, radix_hist_elems(num_vars + 1));
        c.radix_hscan.reserve(rt, radix_hist_elems(num_vars + 1));
        c.scan_tmp32.reserve(rt, scan_tmp_elems(std::max<size_t>(radix_hist_elems(num_vars + 1), cap_cls)) + 4);
        rt.zero(c.asg.p, (size_t)(num_vars + 1) * 4);
        rt.zero(c.vstate.p, num_vars + 1);
        rt.zero(c.counters.p, 32 * 4);
        rt.zero(c.counters64.p, 8 * 8);
        // literals and offsets
        // offsets and learnt flags from host buffers land in buffers the context keeps
        // (an upload of the same size allocates nothing)
        DBuf<u64>& doff = c.up_off;
        DBuf<uint8_t>& dlearnt = c.up_learnt;
        const u64* off_ptr = offsets;
        const uint8_t* learnt_ptr = learnt;
        if (parts) {
            // each formula's literals and offsets straight to their place; offsets
            // are rebased on the device
            doff.reserve(rt, num_clauses + 1);
            std::vector<u64> first(batch->nf), base(batch->nf);
            u64 at = 0;
            for (u32 f = 0; f < batch->nf; f++) {
                const u64 cb = batch->clause_begin[f], nc = batch->clause_begin[f + 1] - cb;
                const u64* o = batch->part_offsets[f];
                const u64 len = o[nc] - o[0];
                first[f] = o[0];
                base[f] = at;
                if (len) rt.h2d(c.lits.p + at, batch->part_lits[f] + o[0], len * 4);
                if (nc) rt.h2d(doff.p + cb, o, nc * 8);
                at += len;
            }
            c.write_u64(doff.p + num_clauses, at);
            DBuf<u64> dfirst, dbase, dcb;
            dfirst.reserve(rt, batch->nf);
            dbase.reserve(rt, batch->nf);
            dcb.reserve(rt, batch->nf + 1);
            rt.h2d(dfirst.p, first.data(), batch->nf * 8);
            rt.h2d(dbase.p, base.data(), batch->nf * 8);
            rt.h2d(dcb.p, batch->clause_begin, (batch->nf + 1) * 8);
            if (num_clauses) rt.each(FRebase{doff.p, dcb.p, dfirst.p, dbase.p, batch->nf}, (u32)num_clauses);
            rt.sync();
            off_ptr = doff.p;
        } else if (device) {
            rt.d2d(c.lits.p, lits + off0, L * 4);
        } else {
            doff.reserve(rt, num_clauses + 1);
            rt.h2d(c.lits.p, lits + off0, L * 4);
            rt.h2d(doff.p, offsets, (num_clauses + 1) * 8);
            off_ptr = doff.p;
            if (learnt) {
                dlearnt.reserve(rt, num_clauses + 1);
                rt.h2d(dlearnt.p, learnt, num_clauses);
                learnt_ptr = dlearnt.p;
            }
        }
        if (learnt) {
            std::vector<uint8_t> h(num_clauses);
            if (device) rt.d2h(h.data(), learnt, num_clauses);
            else std::memcpy(h.data(), learnt, num_clauses);
            for (u64 i = 0; i < num_clauses; i++) if (h[i]) { c.has_learnt = true; break; }
        }
        DBuf<u64> dcls;
        DBuf<u32> dnv;
        UploadArgs a{c.view(), off_ptr, learnt_ptr, off0, L, 0u, nullptr, nullptr, nullptr};
        if (batch) {
            const u32 nf = batch->nf;
            c.h_f_var = batch_var_offsets(nf, batch->num_vars);
            c.h_f_nv.assign(batch->num_vars, batch->num_vars + nf);
            c.f_var.reserve(rt, nf + 1);
            rt.h2d(c.f_var.p, c.h_f_var.data(), (size_t)(nf + 1) * 4);
            dnv.reserve(rt, nf);
            rt.h2d(dnv.p, batch->num_vars, (size_t)nf * 4);
            dcls.reserve(rt, nf + 1);
            rt.h2d(dcls.p, batch->clause_begin, (size_t)(nf + 1) * 8);
            c.var_fid.reserve(rt, num_vars + 1);
            rt.each(FVarFid{c.var_fid.p, c.f_var.p, nf}, num_vars + 1);
            c.f_err.reserve(rt, nf);
            rt.zero(c.f_err.p, (size_t)nf * 4);
            c.f_active.reserve(rt, nf);
            c.f_npvs.reserve(rt, nf);
            c.f_group.reserve(rt, nf);
            c.f_count.reserve(rt, 2 * (size_t)nf);
            c.bound.reserve(rt, 2 * (size_t)nf + 2);
            c.f_status.assign(nf, PF_OK);
            c.f_phases.assign(nf, 0);
            c.res_mark.reserve(rt, c.resolved.n);
            rt.zero(c.res_mark.p, c.res_mark.n);
            a = UploadArgs{c.view(), off_ptr, learnt_ptr, parts ? 0ull : off0, L, nf, dcls.p, c.f_var.p, dnv.p};
        }
        rt.each(FUpload{a}, (u32)num_clauses);
        rt.sync();
        dcls.free();
        dnv.free();
        const u32 e = c.read_err();
        if (e & ERR_INPUT) {
            c.uploaded = false;
            return fail("invalid clause (empty, literal out of range or repeated variable)", PF_EINVAL);
        }
        c.ntrail = c.read_u32(c.counters.p + 0);  // units of one-literal clauses
        c.uploaded = true;
        c.rounds_run = 0;
        c.compact = false;
        return PF_OK;
    });
}

pf_status pf_sigma_upload(pf_sigma_ctx* ctx, uint32_t num_vars, const uint32_t* lits, const uint64_t* offsets,
                          uint64_t num_clauses, const uint8_t* learnt) {
    return upload_common(ctx, num_vars, lits, offsets, num_clauses, learnt, false);
}

pf_status pf_sigma_upload_device(pf_sigma_ctx* ctx, uint32_t num_vars, const uint32_t* d_lits,
                                 const uint64_t* d_offsets, uint64_t num_clauses, const uint8_t* d_learnt) {
    return upload_common(ctx, num_vars, d_lits, d_offsets, num_clauses, d_learnt, true);
}

static pf_status upload_batch(pf_sigma_ctx* ctx, uint32_t num_formulas, const uint32_t* num_vars,
                              const uint64_t* clause_begin, const uint32_t* lits, const uint64_t* offsets, bool device) {
    if (!ctx) return fail("null context", PF_EINVAL);
    if (!num_formulas || !num_vars || !clause_begin) return fail("empty batch", PF_EINVAL);
    if (clause_begin[0] != 0) return fail("clause_begin[0] must be 0", PF_EINVAL);
    u64 total_vars = 0;
    for (u32 f = 0; f < num_formulas; f++) {
        if (clause_begin[f + 1] < clause_begin[f]) return fail("clause ranges not ascending", PF_EINVAL);
        if (num_vars[f] >= (1u << 30)) return fail("too many variables", PF_EINVAL);
        total_vars += (num_vars[f] + 15u) & ~15u;
    }
    if (total_vars == 0) return fail("batch without variables", PF_EINVAL);
    if (total_vars >= (1u << 30)) return fail("too many variables", PF_EINVAL);
    BatchSpec b{num_formulas, num_vars, clause_begin};
    return upload_common(ctx, (u32)total_vars, lits, offsets, clause_begin[num_formulas], nullptr, device, &b);
}

pf_status pf_sigma_upload_batch(pf_sigma_ctx* ctx, uint32_t num_formulas, const uint32_t* num_vars,
                                const uint64_t* clause_begin, const uint32_t* lits, const uint64_t* offsets) {
    return upload_batch(ctx, num_formulas, num_vars, clause_begin, lits, offsets, false);
}

pf_status pf_sigma_upload_batch_parts(pf_sigma_ctx* ctx, uint32_t num_formulas, const uint32_t* num_vars,
                                      const uint64_t* num_clauses, const uint32_t* const* lits,
                                      const uint64_t* const* offsets) {
    if (!ctx) return fail("null context", PF_EINVAL);
    if (!num_formulas || !num_vars || !num_clauses || !lits || !offsets) return fail("empty batch", PF_EINVAL);
    std::vector<uint64_t> cb(num_formulas + 1, 0);
    u64 total_vars = 0;
    for (u32 f = 0; f < num_formulas; f++) {
        if (!lits[f] || !offsets[f]) return fail("null formula", PF_EINVAL);
        if (num_vars[f] >= (1u << 30)) return fail("too many variables", PF_EINVAL);
        cb[f + 1] = cb[f] + num_clauses[f];
        total_vars += (num_vars[f] + 15u) & ~15u;
    }
    if (total_vars == 0) return fail("batch without variables", PF_EINVAL);
    if (total_vars >= (1u << 30)) return fail("too many variables", PF_EINVAL);
    BatchSpec b{num_formulas, num_vars, cb.data(), lits, offsets};
    // lits/offsets of the concatenated form are unused with parts; pass non-null markers
    return upload_common(ctx, (u32)total_vars, lits[0], offsets[0], cb[num_formulas], nullptr, false, &b);
}

pf_status pf_sigma_upload_batch_device(pf_sigma_ctx* ctx, uint32_t num_formulas, const uint32_t* num_vars,
                                       const uint64_t* clause_begin, const uint32_t* d_lits,
                                       const uint64_t* d_offsets) {
    return upload_batch(ctx, num_formulas, num_vars, clause_begin, d_lits, d_offsets, true);
}

pf_status pf_sigma_round(pf_sigma_ctx* ctx, pf_round_stats* stats) {
    if (!ctx) return fail("null context", PF_EINVAL);
    if (!ctx->uploaded) return fail("round before upload", PF_ESTATE);
    pf_sigma_ctx& c = *ctx;
    std::memset(&c.st, 0, sizeof(c.st));
    c.dump.clear();
    c.proof_bound = 0;
    if (c.opt.proof) {
        c.rt.zero(c.counters64.p + 4, 8);
        c.proof_reserve(2ull * c.nvars + 4096);  // every unit of the round: [1, lit]
    }
    c.alg_bytes = 0;
    c.mis_rounds = 0;
    c.prop_waves = 0;
    c.rt.launches = 0;
    c.rt.syncs = 0;
    c.compact = false;
    for (int k = 0; k < pf_sigma_ctx::K_COUNT; k++) {
        c.kclock[k].reset();
        c.kbytes[k] = 0;
    }
    pf_status status = PF_OK;
    try {
        c.keep_at.reserve(c.rt, (size_t)c.nvars + 1);
        c.keep_shape.reserve(c.rt, (size_t)c.nvars + 1);
        c.rt.zero(c.keep_at.p, ((size_t)c.nvars + 1) * 4);
        c.ws_slots.reserve(c.rt, 2 * kSpreadSlots);
        c.rt.zero(c.ws_slots.p + kSpreadSlots, kSpreadSlots * 8);
        pf_options& o = c.opt;
        if (c.opt.dump_level > 0) {
            c.dump_cnf(0, 0);
            c.dump_trail(0, 0);
        }
        StageTimer whole;
        whole.init();
        whole.start(c.rt);
        if (c.nf) {
            if (c.opt.dump_level > 0) throw std::runtime_error("round dumps are not written for formula batches");
            if (c.opt.proof) throw std::runtime_error("proofs are recorded for single formulas only");
            c.round_batch();
        } else if (!(!o.phases && !(o.all || o.ere))) {
            c.round();
        }
        c.st.ms_total = whole.stop(c.rt);
        whole.destroy();
        if (c.opt.dump_level > 0) {
            c.dump_cnf(c.phase, 8);
            c.dump_trail(c.phase, 8);
            c.dump_resolved(c.phase, 8);
            c.dump_elim(c.phase, 8);
            c.rec(10, c.phase, 8, {(u32)c.n_cls_after, (u32)c.n_lits_after});
        }
    } catch (int code) {
        status = (pf_status)code;
        if (code != PF_UNSAT) g_last_error = "round stopped with status " + std::to_string(code);
    } catch (OomError& e) {
        status = fail(e.what(), PF_ENOMEM);
    } catch (std::exception& e) {
        status = fail(e.what(), PF_EDEVICE);
    }
    if (c.opt.dump_level > 0) c.rec(11, 0, 8, {status == PF_OK ? 0u : (status == PF_UNSAT ? 1u : 3u)});
    c.st.status = status;
    c.rounds_run++;
    c.st.clauses_after = (u64)c.n_cls_after;
    c.st.literals_after = (u64)c.n_lits_after;
    c.st.units = c.ntrail;
    c.st.resolved_words = c.nresolved;
    c.st.algorithmic_bytes = c.alg_bytes;
    c.st.kernel_launches = c.rt.launches;
    c.st.mis_rounds = c.mis_rounds;
    c.st.prop_waves = c.prop_waves;
    c.st.host_syncs = c.rt.syncs;
    if (status == PF_OK || status == PF_UNSAT) {
        try {
            c.rt.sync();
            c.kbytes[pf_sigma_ctx::K_MIS] = c.read_slots(c.ws_slots.p + kSpreadSlots);
            for (int k = 0; k < pf_sigma_ctx::K_COUNT; k++) {
                c.st.ms_kernel[k] = c.kclock[k].total_ms();
                c.st.bytes_kernel[k] = c.kbytes[k];
                c.st.launches_kernel[k] = c.kclock[k].launches();
            }
        } catch (std::exception&) {
        }
    }
    if (stats) *stats = c.st;
    return status;
}

pf_status pf_sigma_result_sizes(pf_sigma_ctx* ctx, uint64_t* num_clauses, uint64_t* num_literals, uint64_t* num_units,
                                uint64_t* num_resolved) {
    if (!ctx || !ctx->uploaded) return fail("no formula", PF_ESTATE);
    if (ctx->nf) return fail("a formula batch: use pf_sigma_batch_result_sizes", PF_ESTATE);
    if (num_clauses) *num_clauses = ctx->ncls;
    if (num_literals) *num_literals = ctx->nlits_used;
    if (num_units) *num_units = ctx->ntrail;
    if (num_resolved) *num_resolved = ctx->nresolved;
    return PF_OK;
}

pf_status pf_sigma_download(pf_sigma_ctx* ctx, uint32_t* lits, uint64_t* offsets, uint8_t* learnt, uint32_t* units,
                            uint32_t* resolved, uint8_t* eliminated) {
    if (!ctx || !ctx->uploaded) return fail("no formula", PF_ESTATE);
    if (ctx->nf) return fail("a formula batch: use pf_sigma_batch_download", PF_ESTATE);
    return guarded([&]() -> pf_status {
        pf_sigma_ctx& c = *ctx;
        if ((lits || offsets || learnt) && c.compact) {
            // compacted store: the literals are already contiguous in clause order; all
            // copies are queued, then one synchronisation
            c.big64a.reserve(c.rt, (size_t)c.ncls + 1);
            c.down_learnt.reserve(c.rt, (size_t)c.ncls + 1);
            if (c.ncls) c.rt.each(FDownOffsets{c.hdr.p, c.big64a.p, c.down_learnt.p}, c.ncls);
            c.write_u64(c.big64a.p + c.ncls, c.nlits_used);
            if (lits && c.nlits_used) c.rt.d2h_async(lits, c.lits.p, (size_t)c.nlits_used * 4);
            if (offsets) c.rt.d2h_async(offsets, c.big64a.p, ((size_t)c.ncls + 1) * 8);
            if (learnt && c.ncls) c.rt.d2h_async(learnt, c.down_learnt.p, c.ncls);
        } else if (lits || offsets || learnt) {
            auto H = c.fetch(c.hdr.p, c.ncls);
            std::vector<u32> L;
            if (lits) L = c.fetch(c.lits.p, c.nlits_used);
            u64 o = 0;
            for (u32 i = 0; i < c.ncls; i++) {
                if (offsets) offsets[i] = o;
                if (learnt) learnt[i] = h_learnt(H[i].flags) ? 1 : 0;
                if (lits) std::memcpy(lits + o, L.data() + H[i].start, H[i].size * 4);
                o += H[i].size;
            }
            if (offsets) offsets[c.ncls] = o;
        }
        if (units && c.ntrail) c.rt.d2h_async(units, c.trail.p, (size_t)c.ntrail * 4);
        if (resolved && c.nresolved) c.rt.d2h_async(resolved, c.resolved.p, (size_t)c.nresolved * 4);
        if (eliminated) c.rt.d2h_async(eliminated, c.vstate.p, c.nvars + 1);
        c.rt.sync();
        return PF_OK;
    });
}

// ---------------------------------------------------------------- batch results
// Clauses are grouped per formula on the device (a stable sort of the store by
// formula); the trail and the witness stack are split on the host, with literals
// back in each formula's own numbering.
pf_status pf_sigma_batch_result_sizes(pf_sigma_ctx* ctx, int32_t* status, uint32_t* phases, uint64_t* num_clauses,
                                      uint64_t* num_literals, uint64_t* num_units, uint64_t* num_resolved) {
    if (!ctx || !ctx->uploaded) return fail("no formula", PF_ESTATE);
    if (!ctx->nf) return fail("not a formula batch", PF_ESTATE);
    return guarded([&]() -> pf_status {
        pf_sigma_ctx& c = *ctx;
        if (c.fc_cls.size() != c.nf) c.count_formulas();
        std::vector<u64> nunit, nres;
        if (num_units) c.batch_units(nunit, nullptr);
        if (num_resolved) c.batch_witness(nres, nullptr);
        for (u32 f = 0; f < c.nf; f++) {
            if (status) status[f] = c.f_status[f];
            if (phases) phases[f] = c.f_phases[f];
            if (num_clauses) num_clauses[f] = c.fc_cls[f];
            if (num_literals) num_literals[f] = c.fc_lits[f];
            if (num_units) num_units[f] = nunit[f];
            if (num_resolved) num_resolved[f] = nres[f];
        }
        return PF_OK;
    });
}

pf_status pf_sigma_batch_download(pf_sigma_ctx* ctx, uint32_t* lits, uint64_t* offsets, uint8_t* learnt,
                                  uint32_t* units, uint32_t* resolved, uint8_t* eliminated) {
    if (!ctx || !ctx->uploaded) return fail("no formula", PF_ESTATE);
    if (!ctx->nf) return fail("not a formula batch", PF_ESTATE);
    return guarded([&]() -> pf_status {
        pf_sigma_ctx& c = *ctx;
        const u32 nf = c.nf;
        if (lits || offsets || learnt) c.batch_clauses_to(lits, offsets, learnt);
        std::vector<u64> counts;
        if (units) c.batch_units(counts, units);
        if (resolved) c.batch_witness(counts, resolved);
        if (eliminated) {
            const std::vector<uint8_t> vs = c.fetch(c.vstate.p, c.nvars + 1);
            u64 w = 0;
            for (u32 f = 0; f < nf; f++) {
                eliminated[w++] = 0;
                std::memcpy(eliminated + w, vs.data() + c.h_f_var[f] + 1, c.h_f_nv[f]);
                w += c.h_f_nv[f];
            }
        }
        return PF_OK;
    });
}

// One binary DRAT line (src/cpu/proof.cpp:95-135): 'a' or 'd', every literal in
// 7-bit groups (low group first, high bit set on all but the last), a 0 byte.
static void drat_line(std::vector<uint8_t>& out, char tag, const u32* lits, u32 n) {
    out.push_back((uint8_t)tag);
    for (u32 i = 0; i < n; i++) {
        u32 r = lits[i];
        while (r & ~127u) {
            out.push_back((uint8_t)((r & 127u) | 128u));
            r >>= 7;
        }
        out.push_back((uint8_t)r);
    }
    out.push_back(0);
}

pf_status pf_sigma_proof(pf_sigma_ctx* ctx, uint8_t* out, uint64_t* bytes) {
    if (!ctx || !bytes) return fail("null argument", PF_EINVAL);
    if (!ctx->opt.proof) return fail("the context records no proof (option proof = 0)", PF_ESTATE);
    if (!ctx->rounds_run || (ctx->st.status != PF_OK && ctx->st.status != PF_UNSAT))
        return fail("no finished round", PF_ESTATE);
    return guarded([&]() -> pf_status {
        pf_sigma_ctx& c = *ctx;
        u64 words = 0;
        c.rt.d2h(&words, c.counters64.p + 4, 8);
        if (words > c.proof.n) throw std::runtime_error("proof buffer overflow");
        std::vector<u32> w = c.fetch(c.proof.p, (size_t)words);
        std::vector<uint8_t> enc;
        enc.reserve((size_t)words * 3 + 8);
        for (u64 i = 0; i < words;) {
            const u32 n = w[i] & ~PROOF_DELETE;
            if (i + 1 + n > words) throw std::runtime_error("malformed proof buffer");
            drat_line(enc, (w[i] & PROOF_DELETE) ? 'd' : 'a', w.data() + i + 1, n);
            i += 1 + n;
        }
        if (c.st.status == PF_UNSAT) drat_line(enc, 'a', nullptr, 0);
        if (out) {
            if (*bytes < enc.size()) {
                *bytes = enc.size();
                return fail("proof buffer too small", PF_EINVAL);
            }
            std::memcpy(out, enc.data(), enc.size());
        }
        *bytes = enc.size();
        return PF_OK;
    });
}

pf_status pf_sigma_extend(pf_sigma_ctx* ctx, uint8_t* values) {
    if (!ctx || !values) return fail("null argument", PF_EINVAL);
    if (!ctx->uploaded || ctx->st.status != PF_OK || !ctx->rounds_run)
        return fail("model extension needs a finished round without contradiction", PF_ESTATE);
    return guarded([&]() -> pf_status {
        ctx->extend(values);
        return PF_OK;
    });
}

pf_status pf_sigma_write_dump(pf_sigma_ctx* ctx, const char* path) {
    if (!ctx || !path) return fail("null argument", PF_EINVAL);
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(std::string("cannot open ") + path, PF_EINVAL);
    if (!ctx->dump.empty()) std::fwrite(ctx->dump.data(), 4, ctx->dump.size(), f);
    std::fclose(f);
    return PF_OK;
}

struct FHistCsr { CsrOtArgs a; HD void operator()(u32 i) const { k_hist_csr(a, i); } };
struct FScatterCsr { CsrOtArgs a; HD void operator()(u32 i) const { k_scatter_csr(a, i); } };

// Histogram -> scan -> scatter over caller buffers; `tmp` holds the scan block sums
// (scan_tmp_elems(D) words) followed by one error word.
static void create_ot_into(Runtime& rt, u32 num_vars, const u32* d_lits, const u64* d_offsets, u64 num_clauses,
                           u32* d_ot_off, u32* d_ot_size, u32* d_ot_refs, u32* tmp, size_t tmp_words) {
    const u32 D = 2 * (num_vars + 1);
    u32* err = tmp + tmp_words - 1;
    u64 off0 = 0, offn = 0;
    rt.d2h(&off0, d_offsets, 8);
    rt.d2h(&offn, d_offsets + num_clauses, 8);
    CsrOtArgs a{d_lits, d_offsets, d_ot_off, d_ot_size, d_ot_refs, offn - off0, D, err};
    if (off0 != 0) throw int(PF_EINVAL);
    rt.zero(err, 4);
    rt.zero(d_ot_size, (size_t)D * 4);
    rt.each(FHistCsr{a}, (u32)num_clauses);
    excl_scan<u32, u32>(d_ot_size, d_ot_off, D, d_ot_off + D, tmp, rt.stream);
    rt.zero(d_ot_size, (size_t)D * 4);
    rt.each(FScatterCsr{a}, (u32)num_clauses);
    u32 e = 0;
    rt.d2h(&e, err, 4);
    if (e & ERR_INPUT) throw int(PF_EINVAL);
    if (e) throw std::runtime_error("occurrence table build failed");
}

pf_status pf_create_ot(uint32_t num_vars, const uint32_t* d_lits, const uint64_t* d_offsets, uint64_t num_clauses,
                       uint32_t* d_ot_off, uint32_t* d_ot_size, uint32_t* d_ot_refs, void* stream) {
    if (!d_lits || !d_offsets || !d_ot_off || !d_ot_size || !d_ot_refs || !num_vars) return fail("null argument", PF_EINVAL);
    if (num_vars >= (1u << 30) || num_clauses >= 0xFFFFFF00ull) return fail("formula too large", PF_EINVAL);
    Runtime rt;
    return guarded([&]() -> pf_status {
        rt.init();
#if SIGMA_CUDA
        cudaStreamDestroy(rt.stream);
        rt.stream = (cudaStream_t)stream;
#endif
        const u32 D = 2 * (num_vars + 1);
        const size_t words = scan_tmp_elems(D) + 1;
        u32* tmp = (u32*)rt.alloc(words * 4);
        try {
            create_ot_into(rt, num_vars, d_lits, d_offsets, num_clauses, d_ot_off, d_ot_size, d_ot_refs, tmp, words);
        } catch (...) {
            rt.sync();
            rt.release(tmp, words * 4);
            throw;
        }
        rt.sync();
        rt.release(tmp, words * 4);
        return PF_OK;
    });
}

// ---------------------------------------------------------------- no-allocation variant
// pf_create_ot_noalloc: the scan scratch (block sums + one error word) is this
// fixed array instead of a cudaMalloc. In host code its name only stands in for
// the device symbol; the device address comes from cudaGetSymbolAddress, looked
// up once per device on that device's first call.
constexpr u32 kNoallocWords = 1u << 16;  // 256 KiB
// The scan over D = 2*num_vars+2 literal slots keeps ceil(D / 2048) + 1 block sums,
// followed by one error word, so the largest accepted num_vars is 67,106,815.
constexpr u64 kNoallocScanTile = 2048;
constexpr u64 kNoallocMaxVars = (u64)(kNoallocWords - 2) * kNoallocScanTile / 2 - 1;
static_assert(kNoallocMaxVars == 67106815ull, "no-allocation limit");
#if SIGMA_CUDA
static_assert(kScanTile == (int)kNoallocScanTile, "scan tile of the no-allocation limit");
#endif
#if SIGMA_CUDA
static __device__ __align__(256) u32 g_noalloc_scratch[kNoallocWords];
#else
alignas(256) static u32 g_noalloc_scratch[kNoallocWords];
#endif
static std::mutex g_noalloc_mu;
static u32* g_noalloc_dev[256];  // per device ordinal

static u32* noalloc_scratch_ptr() {
#if SIGMA_CUDA
    int dev = 0;
    ck(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= 256) throw std::runtime_error("device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_dev[dev]) {
        void* p = nullptr;
        ck(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress");
        g_noalloc_dev[dev] = (u32*)p;
    }
    return g_noalloc_dev[dev];
#else
    return g_noalloc_scratch;
#endif
}

pf_status pf_create_ot_noalloc(uint32_t num_vars, const uint32_t* d_lits, const uint64_t* d_offsets,
                               uint64_t num_clauses, uint32_t* d_ot_off, uint32_t* d_ot_size, uint32_t* d_ot_refs,
                               void* stream) {
    if (!d_lits || !d_offsets || !d_ot_off || !d_ot_size || !d_ot_refs || !num_vars) return fail("null argument", PF_EINVAL);
    if (num_clauses >= 0xFFFFFF00ull) return fail("too many clauses", PF_EINVAL);
    if (num_vars > kNoallocMaxVars)
        return fail("pf_create_ot_noalloc: num_vars above 67,106,815 exceeds the fixed scratch", PF_EINVAL);
    return guarded([&]() -> pf_status {
        Runtime rt;  // no init(): this call creates no stream and allocates nothing
#if SIGMA_CUDA
        int dev = 0;
        ck(cudaGetDevice(&dev), "cudaGetDevice");
        ck(cudaDeviceGetAttribute(&rt.sms, cudaDevAttrMultiProcessorCount, dev), "attr");
        rt.stream = (cudaStream_t)stream;
#endif
        u32* scratch = noalloc_scratch_ptr();
        create_ot_into(rt, num_vars, d_lits, d_offsets, num_clauses, d_ot_off, d_ot_size, d_ot_refs, scratch,
                       kNoallocWords);
        rt.sync();
        return PF_OK;
    });
}

uint64_t pf_device_alloc_count(void) { return device_alloc_count().load(); }

pf_status pf_dimacs_parse(const char* path, pf_formula* out) {
    if (!path || !out) return fail("null argument", PF_EINVAL);
    std::memset(out, 0, sizeof(*out));
    return guarded([&]() -> pf_status {
        DimacsFormula f;
        const std::string err = dimacs_read(path, f);
        if (!err.empty()) return fail(std::string("DIMACS: ") + err, PF_EINVAL);
        const size_t nc = f.offsets.size() - 1;
        out->num_vars = f.num_vars;
        out->num_clauses = nc;
        out->lits = (uint32_t*)std::malloc(std::max<size_t>(f.lits.size(), 1) * 4);
        out->offsets = (uint64_t*)std::malloc((nc + 1) * 8);
        if (!out->lits || !out->offsets) {
            pf_formula_free(out);
            return fail("out of host memory", PF_ENOMEM);
        }
        if (!f.lits.empty()) std::memcpy(out->lits, f.lits.data(), f.lits.size() * 4);
        std::memcpy(out->offsets, f.offsets.data(), (nc + 1) * 8);
        out->empty_clause = f.empty_clause ? 1 : 0;
        return f.empty_clause ? PF_UNSAT : PF_OK;
    });
}

void pf_formula_free(pf_formula* f) {
    if (!f) return;
    std::free(f->lits);
    std::free(f->offsets);
    f->lits = nullptr;
    f->offsets = nullptr;
}

pf_status pf_sigma_footprint(pf_sigma_ctx* ctx, uint64_t* bytes) {
    if (!ctx || !bytes) return fail("null argument", PF_EINVAL);
    *bytes = ctx->rt.bytes_live;
    return PF_OK;
}

void pf_sigma_destroy(pf_sigma_ctx* ctx) {
    if (!ctx) return;
    // DBuf members release themselves through the runtime
    pf_sigma_ctx& c = *ctx;
    DBuf<Hdr>* hb[] = {&c.hdr, &c.hdr2, &c.sub_hdrs};
    for (auto* b : hb) b->free();
    DBuf<u32>* b32[] = {&c.lits, &c.lits2, &c.ot_off, &c.ot_size, &c.ot_refs, &c.ot_cursor, &c.asg, &c.ps, &c.ns,
                        &c.pvrank, &c.trail, &c.resolved, &c.counters, &c.score, &c.order, &c.order_k2,
                        &c.order_v2, &c.rank, &c.bound, &c.pvs, &c.flags, &c.flags_scan, &c.work, &c.cl_stamp,
                        &c.radix_hist, &c.radix_hscan, &c.scan_tmp32, &c.big32a, &c.big32b, &c.ve_porgs,
                        &c.ve_norgs, &c.ve_ncls, &c.ve_nlits, &c.ve_nwit, &c.ve_def, &c.ve_cls_scan, &c.ve_scr,
                        &c.sub_ent, &c.sub_ent_off, &c.sub_ids, &c.sub_words, &c.sub_sizes, &c.sub_pre_off,
                        &c.sub_pre_lits, &c.sub_ulits, &c.ere_target, &c.ere_losers, &c.cstamp, &c.cstamp2,
                        &c.keep_at, &c.keep_shape};
    for (auto* b : b32) b->free();
    DBuf<u64>* b64[] = {&c.counters64, &c.ws_slots, &c.hread, &c.scan_tmp64, &c.big64a, &c.big64b, &c.ve_scr_off, &c.ve_lit_scan,
                        &c.ve_wit_scan, &c.sub_wrd, &c.sub_wrd_off, &c.ere_claim, &c.ere_key};
    for (auto* b : b64) b->free();
    DBuf<uint8_t>* b8[] = {&c.vstate, &c.ve_type, &c.sub_run};
    c.mis_word.free();
    c.mis_resume.free();
    c.mis_cmin.free();
    for (auto& b : c.mis_in) b.free();
    c.mis_rec.free();
    c.mis_gbits.free();
    c.down_learnt.free();
    c.up_off.free();
    c.up_learnt.free();
    c.res_mark.free();
#if SIGMA_CUDA
    c.scan1_agg.free();
    c.scan1_incl.free();
    c.scan1_total.free();
    c.scan1_flag.free();
    c.scan1_ctl.free();
#endif
    c.mis_big_a.free();
    c.mis_big_b.free();
#if SIGMA_CUDA
    c.otb_count.free();
    c.otb_base.free();
    c.otb_cursor.free();
    c.otb_pair.free();
    c.prop_trace.free();
    c.prop_parts.free();
#endif
    c.pv_perm.free();
    c.pv_key.free();
    for (auto* b : b8) b->free();
    c.sub_units.free();
    c.sub_units2.free();
    c.sub_pairs.free();
    DBuf<u32>* fx[] = {&c.fx_prod, &c.fx_rank, &c.fx_lit, &c.fx_k2, &c.fx_v2, &c.fx_flag, &c.fx_scan, &c.want_rank,
                       &c.want_lit, &c.want_cnt, &c.want_off, &c.used_lit, &c.used_off};
    for (auto* b : fx) b->free();
    c.fx_prod8.free();
    c.fx_other8.free();
    c.proof.free();
    c.tm.destroy();
    for (auto& k : c.kclock) k.destroy();
    c.rt.destroy();
    delete ctx;
}

const char* pf_last_error(void) { return g_last_error.c_str(); }

}  // extern "C"
