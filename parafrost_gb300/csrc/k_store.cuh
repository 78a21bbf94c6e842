// Clause-store kernels: upload normalisation, occurrence-table build, survivor
// counts and compaction. Item functions run once per clause / literal slot.
#pragma once

#include "cnf.cuh"
#include "introsort.cuh"

namespace sigma {

// ---------------------------------------------------------------- upload
// extract() (src/cpu/simplify.cpp:95-113; GPU: transfer.cu:24-42 + prep_cnf_k,
// kernels.cu:61-70): literals sorted ascending, signature over the clause,
// status from the learnt flag. Rejects literals out of range and clauses that
// repeat a variable. A one-literal clause is not a clause of the store: as the
// reference's parser does (src/cpu/dimacs.cpp:153-159), its literal goes to the
// trail (first claim of the variable wins; the opposite literal already there is
// a contradiction) and the clause is kept as a deleted slot; the round then
// propagates these units before its first phase.
struct UploadArgs {
    Ctx c;
    const u64* off;      // num_clauses + 1
    const uint8_t* learnt;  // may be null
    u64 base;            // literal offset of off[0]
    u64 nlits;           // literals uploaded: every clause must lie in [base, base + nlits)
    // formula batches: nf formulas, formula f holds clauses [f_cls[f], f_cls[f+1])
    // and f_nv[f] variables from f_var[f]+1 on; its literals arrive in its own
    // numbering and are moved to the batch's (nf = 0: a single formula)
    u32 nf;
    const u64* f_cls;
    const u32* f_var;
    const u32* f_nv;
};

HD void k_upload_clause(const UploadArgs& a, u32 i) {
    const u64 o0 = a.off[i], o1 = a.off[i + 1];
    // offsets that go down, or leave the uploaded literals, are rejected before
    // any literal is touched
    if (o0 < a.base || o1 < o0 || o1 - a.base > a.nlits) { set_err(a.c, ERR_INPUT); return; }
    const u64 s = o0 - a.base, e = o1 - a.base;
    u32* l = a.c.lits + s;
    const u32 n = (u32)(e - s);
    if (n == 0) { set_err(a.c, ERR_INPUT); return; }
    if (a.nf) {
        const u32 f = upper_segment(a.f_cls, a.nf, (u64)i);
        const u32 shift = 2u * a.f_var[f], lim = 2u * a.f_nv[f] + 2u;
        for (u32 k = 0; k < n; k++) {
            if (l[k] < 2 || l[k] >= lim) { set_err(a.c, ERR_INPUT); return; }
            l[k] += shift;
        }
    }
    if (n <= 32) ref_insertion_sort(l, (int)n, LitLess());
    else std_sort_replica(l, l + n, LitLess());
    u32 sig = 0;
    for (u32 k = 0; k < n; k++) {
        const u32 lit = l[k];
        if (lit < 2 || lit >= a.c.D) { set_err(a.c, ERR_INPUT); return; }
        if (k && ABS(lit) == ABS(l[k - 1])) { set_err(a.c, ERR_INPUT); return; }
        sig |= MAPHASH(lit);
    }
    Hdr h;
    h.start = (u32)s;
    h.size = n;
    h.sig = sig;
    h.flags = (a.learnt && a.learnt[i]) ? ST_LEARNT : ST_ORIGINAL;
    if (n == 1) {
        h.flags = ST_DELETED;
        const u32 u = l[0];
        const u32 old = atom_cas(&a.c.asg[ABS(u)], 0u, u);
        if (old == 0) a.c.trail[atom_add(a.c.ntrail, 1u)] = u;
        else if (old != u) set_unsat(a.c, ABS(u));
    }
    a.c.hdr[i] = h;
}

// ---------------------------------------------------------------- OT build
// createOT (src/cpu/simplify.cpp:35-56) as histogram -> exclusive scan -> scatter
// (GPU reference: histogram.cu:34-52, memory.cu:271-312, create_ot_k kernels.cu:81-96).
HD void k_hist_clause(const Ctx& c, u32 i) {
    const Hdr h = c.hdr[i];
    if (h_deleted(h.flags)) return;
    const u32* l = c.lits + h.start;
    for (u32 k = 0; k < h.size; k++) atom_add(&c.ot_size[l[k]], 1u);
}

HD void k_scatter_clause(const Ctx& c, u32 i) {
    const Hdr h = c.hdr[i];
    if (h_deleted(h.flags)) return;
    const u32* l = c.lits + h.start;
    for (u32 k = 0; k < h.size; k++) {
        const u32 pos = atom_add(&c.ot_cursor[l[k]], 1u);
        if (pos < c.ot_cap) c.ot_refs[pos] = i;
        else set_err(c, ERR_INTERNAL);
    }
}

// Standalone occurrence-table build over a clause list in CSR form (all clauses
// live): histogram into ot_size, exclusive scan into ot_off, then a scatter that
// reuses ot_size (zeroed after the scan) as the per-literal cursor, which leaves
// the list sizes in ot_size again.
struct CsrOtArgs {
    const u32* lits;
    const u64* off;
    u32* ot_off;
    u32* ot_size;
    u32* ot_refs;
    u64 nlits;
    u32 D;
    u32* err;
};
// A clause whose offsets go down or leave [0, nlits) is an input error; neither
// pass reads its literals.
HD bool csr_clause_ok(const CsrOtArgs& a, u32 i) {
    const u64 s = a.off[i], e = a.off[i + 1];
    return s <= e && e <= a.nlits;
}
HD void k_hist_csr(const CsrOtArgs& a, u32 i) {
    if (!csr_clause_ok(a, i)) { atom_or(a.err, ERR_INPUT); return; }
    for (u64 k = a.off[i]; k < a.off[i + 1]; k++) {
        const u32 lit = a.lits[k];
        if (lit < 2 || lit >= a.D) { atom_or(a.err, ERR_INPUT); continue; }
        atom_add(&a.ot_size[lit], 1u);
    }
}
HD void k_scatter_csr(const CsrOtArgs& a, u32 i) {
    if (!csr_clause_ok(a, i)) return;
    for (u64 k = a.off[i]; k < a.off[i + 1]; k++) {
        const u32 lit = a.lits[k];
        if (lit < 2 || lit >= a.D) continue;
        const u32 pos = a.ot_off[lit] + atom_add(&a.ot_size[lit], 1u);
        if (pos < a.nlits) a.ot_refs[pos] = i;
        else atom_or(a.err, ERR_INTERNAL);
    }
}

// occurs[v] = (ps, ns) over live clauses (histSimp, src/cpu/histogram.cpp:82-96).
HD void k_occurs_clause(const Ctx& c, u32 i) {
    const Hdr h = c.hdr[i];
    if (h_deleted(h.flags)) return;
    const u32* l = c.lits + h.start;
    for (u32 k = 0; k < h.size; k++) {
        const u32 lit = l[k];
        atom_add(SIGN(lit) ? &c.ns[ABS(lit)] : &c.ps[ABS(lit)], 1u);
    }
}

// occurs straight from the occurrence-list sizes (valid when no clause changed since
// the OT build): ps = |ot[2v]|, ns = |ot[2v+1]|.
HD void k_occurs_from_ot(const Ctx& c, u32 v) {
    if (v == 0) { c.ps[0] = c.ns[0] = 0; return; }
    c.ps[v] = c.ot_size[V2L(v)];
    c.ns[v] = c.ot_size[NEG(V2L(v))];
}

// ---------------------------------------------------------------- counts
// countAll (src/cpu/solve.h:724-734): live clauses and their literals.
struct CountArgs {
    Ctx c;
    u64* out;  // [0] clauses, [1] literals
};
HD void k_count_clause(const CountArgs& a, u32 i) {
    const Hdr h = a.c.hdr[i];
    if (h_deleted(h.flags)) return;
    atom_add64(&a.out[0], 1ull);
    atom_add64(&a.out[1], (u64)h.size);
}

// Formula of every variable of a batch (variable 0 belongs to none).
HD void k_var_fid(u32* var_fid, const u32* f_var, u32 nf, u32 v) {
    var_fid[v] = v ? upper_segment(f_var, nf, v - 1) : NONE;
}

// Live clauses and literals per formula of a batch (countAll per formula); a
// clause's formula is that of its first literal's variable.
struct FormulaCountArgs {
    Ctx c;
    u64* f_cls;   // nf
    u64* f_lits;  // nf
};
HD void k_count_formula(const FormulaCountArgs& a, u32 i) {
    const Hdr h = a.c.hdr[i];
    if (h_deleted(h.flags)) return;
    const u32 f = a.c.var_fid[ABS(a.c.lits[h.start])];
    atom_add64(&a.f_cls[f], 1ull);
    atom_add64(&a.f_lits[f], (u64)h.size);
}

#if SIGMA_CUDA
// Same count; lanes of a warp that share a formula (a formula's clauses are
// mostly adjacent) add once.
__global__ void count_formula_k(FormulaCountArgs a, u32 n) {
    const u32 lane = threadIdx.x & 31u;
    for (u32 base = blockIdx.x * blockDim.x; base < n; base += blockDim.x * gridDim.x) {
        const u32 i = base + threadIdx.x;
        u32 f = NONE, cls = 0, lits = 0;
        if (i < n) {
            const Hdr h = a.c.hdr[i];
            if (!h_deleted(h.flags)) {
                f = a.c.var_fid[ABS(a.c.lits[h.start])];
                cls = 1;
                lits = h.size;
            }
        }
        const u32 peers = __match_any_sync(0xffffffffu, f);
        cls = __reduce_add_sync(peers, cls);
        lits = __reduce_add_sync(peers, lits);
        if (f != NONE && lane == (u32)(__ffs(peers) - 1)) {
            atomicAdd((unsigned long long*)&a.f_cls[f], (unsigned long long)cls);
            atomicAdd((unsigned long long*)&a.f_lits[f], (unsigned long long)lits);
        }
    }
}

// Same counts with a warp/block reduction and one pair of atomics per block.
__global__ void count_live_k(const Hdr* __restrict__ hdr, u32 n, u64* out) {
    u64 cls = 0, lits = 0;
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += blockDim.x * gridDim.x) {
        const Hdr h = hdr[i];
        if (!h_deleted(h.flags)) { cls++; lits += h.size; }
    }
    for (int o = 16; o; o >>= 1) {
        cls += __shfl_down_sync(0xffffffffu, cls, o);
        lits += __shfl_down_sync(0xffffffffu, lits, o);
    }
    __shared__ u64 s_cls[32], s_lits[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { s_cls[warp] = cls; s_lits[warp] = lits; }
    __syncthreads();
    if (threadIdx.x == 0) {
        u64 c = 0, l = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) { c += s_cls[w]; l += s_lits[w]; }
        atomicAdd((unsigned long long*)&out[0], (unsigned long long)c);
        atomicAdd((unsigned long long*)&out[1], (unsigned long long)l);
    }
}
#endif

// ---------------------------------------------------------------- compaction
// shrinkSimp (src/cpu/simplify.cpp:234-245; GPU: recycle.cu:30-97): drop deleted
// clauses, keep order. Two exclusive scans (kept clauses, kept literals) give the
// new id and the new literal start of every survivor.
struct GcArgs {
    Ctx c;
    const u32* keep_scan;    // exclusive scan of keep flags
    const u64* lit_scan;     // exclusive scan of kept sizes
    Hdr* new_hdr;
    u32* new_lits;
    u32* new_stamp;  // the clause stamps move with the headers
};
HD void k_gc_flags(const Ctx& c, u32* keep, u64* sizes, u32 i) {
    const Hdr h = c.hdr[i];
    const bool k = !h_deleted(h.flags);
    keep[i] = k ? 1u : 0u;
    sizes[i] = k ? (u64)h.size : 0ull;
}
HD void k_gc_move(const GcArgs& a, u32 i) {
    const Hdr h = a.c.hdr[i];
    if (h_deleted(h.flags)) return;
    const u32 id = a.keep_scan[i];
    const u64 st = a.lit_scan[i];
    Hdr nh = h;
    nh.start = (u32)st;
    a.new_hdr[id] = nh;
    if (a.c.cstamp) a.new_stamp[id] = a.c.cstamp[i];
    const u32* src = a.c.lits + h.start;
    u32* dst = a.new_lits + st;
    for (u32 k = 0; k < h.size; k++) dst[k] = src[k];
}

}  // namespace sigma
