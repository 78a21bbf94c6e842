/*
 * sigma_gb300 — GB300-native (sm_103a) SIGmA inprocessing round of ParaFROST.
 *
 * C ABI of libsigma_gb300.so: plain pointers and sizes, no C++ or torch types.
 * One context holds one formula resident in device memory (clause store,
 * occurrence table, per-variable state) and runs sigmify rounds on it.
 *
 * Literal encoding is the reference solver's: lit = 2*var + sign, variables
 * 1..num_vars, sign 1 = negative (src/cpu/const.h:73-78). Literal slots 0 and 1
 * are unused.
 *
 * Every entry point returns a pf_status; none exits the process or resets the
 * device. Errors are sticky per context until pf_sigma_destroy.
 */
#ifndef SIGMA_GB300_H
#define SIGMA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. Replaces the reference's simpstate codes and exit paths
 * (src/gpu/const.cuh:29-32, definitions.cuh:51-74). */
typedef enum {
    PF_OK = 0,
    PF_UNSAT = 1,     /* the round proved the formula unsatisfiable (learnEmpty) */
    PF_EINVAL = -1,   /* bad argument (literal out of range, null pointer, ...) */
    PF_ENOMEM = -2,   /* device memory budget exceeded (CNFALLOC_FAIL/OTALLOC_FAIL) */
    PF_ETIMEOUT = -3, /* a bounded device wait gave up */
    PF_EDEVICE = -4,  /* CUDA error; pf_last_error() has the text */
    PF_ESTATE = -5,   /* call out of order (e.g. round before upload) */
} pf_status;

/* Simplifier options: the reference's option names and defaults
 * (src/cpu/options.cpp:24-46, derivation rules at options.cpp:281-311).
 * Fill with pf_default_options() and pass to pf_sigma_create. */
typedef struct {
    int32_t phases;          /* "phases"       = 5     */
    int32_t all;             /* "all"          = 0  (=> ve, ve+, bce, ere) */
    int32_t ve;              /* "ve"           = 1     */
    int32_t ve_plus;         /* "ve+"          = 1     */
    int32_t sub;             /* "sub"          = 1     */
    int32_t bce;             /* "bce"          = 0     */
    int32_t ere;             /* "ere"          = 1     */
    int32_t ve_lbound;       /* "velbound"     = 0     */
    int32_t ve_clause_max;   /* "veclausemax"  = 100 (0: no limit) */
    int32_t ve_phase_min;    /* "vephasemin"   = 500   */
    int32_t mu_pos;          /* "mupos"        = 32    */
    int32_t mu_neg;          /* "muneg"        = 32    */
    int32_t xor_max_arity;   /* "xormaxarity"  = 10    */
    int32_t sub_max;         /* "submax"       = 3000  */
    int32_t bce_max;         /* "bcemax"       = 3000  */
    int32_t ere_max;         /* "eremax"       = 3000  */
    int32_t ere_clause_max;  /* "ereclausemax" = 1000 (0: no limit) */
    int32_t lcve_min;        /* "lcvemin"      = 1     */
    int32_t gc_freq;         /* "gcfreq"       = 2 (0: never compact inside the round) */
    /* GB300 extras (no counterpart in the reference) */
    int32_t dump_level;      /* 0: off, 1: per-phase summaries, 2: every stage */
    int32_t loop_limit;      /* rounds a device-side loop may run (election rounds, propagation
                              * waves) before the round gives up with PF_ETIMEOUT; 0: the
                              * default bound, variables + 2, which a correct round never reaches.
                              * A small value exercises the give-up path without any wait. */
    int32_t proof;           /* "proof" = 0: 1 records the round's DRAT proof (pf_sigma_proof);
                              * single formulas only */
    int32_t ot_buckets;      /* occurrence-table build: 0 by size (literal buckets once the
                              * per-literal counters outgrow the L2 cache), 1 always literal
                              * buckets, -1 always per-occurrence atomics */
    int32_t sweep_div;       /* propagation sweeps the whole store when the pending literals'
                              * lists exceed 1/sweep_div of it: 0 = 64, -1 never sweeps */
    int32_t pv_blocks;       /* blocks per SM of the per-variable warp kernels: 0 = 8 */
    int32_t reserved[2];
} pf_options;

/* Per-round statistics (the reference's stage report, src/cpu/statistics.cpp:28-41,
 * plus the device-side measurements). Times are device milliseconds. */
typedef struct {
    int32_t status;           /* pf_status of the round */
    int32_t phases_run;
    uint64_t clauses_before, literals_before;
    uint64_t clauses_after, literals_after;
    uint64_t eliminated_vars; /* variables eliminated by this round */
    uint64_t units;           /* assigned literals on the trail after the round */
    uint64_t resolved_words;  /* witness-stack length */
    double ms_total;          /* device time of the round */
    double ms_stage[12];      /* ot, prop, lcve, sort, sub, ve, bce, ere, gc, count, upload, download */
    uint64_t algorithmic_bytes; /* bytes the round's kernels must move (HBM roofline numerator) */
    uint32_t kernel_launches;   /* kernels launched by the round */
    uint32_t mis_rounds;        /* push/pull rounds of the independent-set elections */
    uint32_t prop_waves;        /* waves of the in-round unit propagations */
    uint32_t host_syncs;        /* times the host waited for the device during the round */
    /* The hottest kernels, timed with CUDA events on the context stream:
     * [0] independent-set rounds (LCVE), [1] BVE decision, [2] SUB, [3] BVE write. */
    double ms_kernel[4];        /* device time summed over the round's launches */
    uint64_t bytes_kernel[4];   /* algorithmic bytes those launches processed */
    uint32_t launches_kernel[4];
    /* Per phase p < 8 of the round (a batch: the batch's shared phase p): live
     * clauses and literals entering it, variables elected in it, the algorithmic
     * bytes and device time of its stages (the closing propagation, count and
     * compaction after the last phase are in neither). */
    uint32_t phase_elected[8];
    uint64_t phase_clauses[8], phase_literals[8];
    uint64_t phase_bytes[8];
    double phase_ms[8];
} pf_round_stats;

typedef struct pf_sigma_ctx pf_sigma_ctx;

/* Fills *o with the reference defaults. */
void pf_default_options(pf_options* o);

/* Applies the reference's option derivation (options.cpp:304-311) in place. */
void pf_derive_options(pf_options* o);

/* Creates a context on the current CUDA device. Replaces ParaFROST::optSimp()
 * + cuMM pool set-up (src/gpu/simplify.cu:254-270, memory.cu). *out is NULL on error. */
pf_status pf_sigma_create(const pf_options* opts, pf_sigma_ctx** out);

/* Uploads a formula: clause c has literals lits[offsets[c] .. offsets[c+1]).
 * learnt may be NULL (all original). Literal order inside a clause is free; the
 * upload sorts literals and computes signatures, as extract() does
 * (src/cpu/simplify.cpp:95-113, src/gpu/transfer.cu:24-42 + kernels.cu:61-70).
 * Host buffers; copies are issued on the context stream. */
pf_status pf_sigma_upload(pf_sigma_ctx* ctx, uint32_t num_vars,
                          const uint32_t* lits, const uint64_t* offsets, uint64_t num_clauses,
                          const uint8_t* learnt);

/* Same as pf_sigma_upload, with lits/offsets/learnt already in device memory. */
pf_status pf_sigma_upload_device(pf_sigma_ctx* ctx, uint32_t num_vars,
                                 const uint32_t* d_lits, const uint64_t* d_offsets, uint64_t num_clauses,
                                 const uint8_t* d_learnt);

/* Runs one sigmify round (ParaFROST::sigmifying(), src/cpu/simplify.cpp:157-232,
 * GPU twin src/gpu/simplify.cu:155-234) on the resident formula. */
pf_status pf_sigma_round(pf_sigma_ctx* ctx, pf_round_stats* stats);

/* Sizes of the simplified formula, for sizing pf_sigma_download buffers. */
pf_status pf_sigma_result_sizes(pf_sigma_ctx* ctx, uint64_t* num_clauses, uint64_t* num_literals,
                                uint64_t* num_units, uint64_t* num_resolved);

/* Copies the simplified formula back to host buffers (any pointer may be NULL):
 * surviving clauses in clause-store order (lits/offsets/learnt), the trail of
 * assigned literals, the witness stack (the reference's model.resolved words,
 * src/cpu/model.cpp:334-379) and one eliminated flag per variable (index 0 unused).
 * Replaces cacheCNF/cacheUnits/cacheResolved/markEliminated (src/gpu/transfer.cu:68-165). */
pf_status pf_sigma_download(pf_sigma_ctx* ctx, uint32_t* lits, uint64_t* offsets, uint8_t* learnt,
                            uint32_t* units, uint32_t* resolved, uint8_t* eliminated);

/* Model extension on the device (MODEL::extend, src/cpu/model.cpp:104-138) after a
 * round that ended PF_OK: values holds, per variable, the caller's model of the
 * simplified formula (1 true, 0 false) and receives a model of the original formula.
 * The round's units are set and eliminated variables start false (as the reference,
 * whose solver never assigns them), then the witness stack is walked from its end:
 * a record whose other literals are all false sets its witness true. Single formula:
 * values[0 .. num_vars] (index 0 unused); its records form one dependent chain,
 * walked by one device thread. Formula batch: formula after formula, num_vars[f] + 1
 * entries each (the first unused; the layout of pf_sigma_batch_download's eliminated
 * flags), every formula walked by its own thread, side by side. For the batched
 * SAT answers of many formulas; one large formula is faster on a host core. */
pf_status pf_sigma_extend(pf_sigma_ctx* ctx, uint8_t* values);

/* The last round's DRAT proof in the reference's binary format (src/cpu/proof.cpp:
 * 95-135, the file ParaFROST writes with -proof): one addition line per clause the
 * round derived (strengthened by SUB, substituted by an equivalence, resolvents of
 * VE) and per unit it assigned, and one deletion line per clause that SUB found
 * subsumed or ERE redundant, as they happen, then the empty clause when the round
 * proved UNSAT. Literals are in the caller's numbering. The reference leaves out an
 * added clause that a unit assigned before it satisfies; this one keeps it. Lines of one stage come in any order (the stage's
 * variables are independent); every line is implied by unit propagation over the
 * input and the lines before it. Needs the option proof = 1. out may be NULL: *bytes
 * receives the size; otherwise *bytes is out's capacity on entry and the size on
 * return. */
pf_status pf_sigma_proof(pf_sigma_ctx* ctx, uint8_t* out, uint64_t* bytes);

/* Writes the per-stage round dump of the last round to path (dump_level > 0). */
pf_status pf_sigma_write_dump(pf_sigma_ctx* ctx, const char* path);

/* Builds the occurrence table of a clause list (createOTAsync, src/gpu/kernels.cu:949-982
 * with resizeOTAsync's scan, memory.cu:271-312; CPU createOT, simplify.cpp:35-56).
 * All pointers are device memory: clause c has literals d_lits[d_offsets[c] ..
 * d_offsets[c+1]) (offsets relative to d_lits), literals in [2, 2*num_vars+2).
 * Outputs: d_ot_off[2*num_vars+3] (list starts, last = total), d_ot_size[2*num_vars+2]
 * (list sizes), d_ot_refs[total literals] (clause indices; order inside a list is
 * unspecified). stream is a cudaStream_t (NULL = legacy default stream). The scan
 * scratch is allocated and freed inside the call; the call returns after the
 * stream has finished. */
pf_status pf_create_ot(uint32_t num_vars, const uint32_t* d_lits, const uint64_t* d_offsets, uint64_t num_clauses,
                       uint32_t* d_ot_off, uint32_t* d_ot_size, uint32_t* d_ot_refs, void* stream);

/* pf_create_ot without any allocation. No counterpart in the reference.
 *
 * For callers that must not allocate device memory: a serving process whose HBM
 * is fully reserved up front by its own pool or by a framework's caching
 * allocator (where a cudaMalloc can fail or escape the budget), or a caller that
 * cannot take the device-wide synchronisation a cudaFree implies. Inputs and
 * outputs are the caller's device buffers, exactly as for pf_create_ot; the scan
 * scratch lives in a fixed 256 KiB array inside the library (held by every GPU
 * that loads the library until the process exits). Limit: num_vars <= 67,106,815
 * (2*num_vars+2 literal slots in at most 65,534 scan blocks of 2048); larger
 * formulas get PF_EINVAL before any GPU work. The first call on a device looks up
 * the array's device address (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture. With lazy module loading (the
 * CUDA default, CUDA_MODULE_LOADING=LAZY) that first call, and the first launch of
 * each kernel it uses, also load code onto the device, which takes device memory:
 * make one warm-up call (or set CUDA_MODULE_LOADING=EAGER) before the caller's pool
 * reserves all of HBM; later calls take none. All calls share the one array:
 * calls that overlap on the GPU (other streams, other threads) race; serialise
 * them. Calls no cudaMalloc, cudaFree or other allocating routine (see
 * pf_device_alloc_count), and creates no stream. */
pf_status pf_create_ot_noalloc(uint32_t num_vars, const uint32_t* d_lits, const uint64_t* d_offsets,
                               uint64_t num_clauses, uint32_t* d_ot_off, uint32_t* d_ot_size, uint32_t* d_ot_refs,
                               void* stream);

/* ---- Formula batches (no counterpart in the reference: ParaFROST simplifies one
 * formula per solver object; many small formulas are simplified here by one context).
 * Formula f has num_vars[f] variables and the clauses [clause_begin[f], clause_begin[f+1])
 * of lits/offsets (clause_begin[0] = 0), its literals in its own numbering
 * (2v + sign, 1 <= v <= num_vars[f]); num_vars and clause_begin are host arrays of
 * num_formulas and num_formulas + 1 entries. pf_sigma_round then runs every formula's
 * own round (its own phases, stop rule and bounds, as pf_sigma_round on that formula
 * alone would) on the one resident store; a formula that derives the empty clause
 * ends with status PF_UNSAT while the others go on. No learnt clauses, no dumps. */
pf_status pf_sigma_upload_batch(pf_sigma_ctx* ctx, uint32_t num_formulas, const uint32_t* num_vars,
                                const uint64_t* clause_begin, const uint32_t* lits, const uint64_t* offsets);

/* Same as pf_sigma_upload_batch with every formula in its own host arrays: formula f
 * has num_clauses[f] clauses, literals lits[f][offsets[f][c] .. offsets[f][c+1])
 * (offsets[f][0] need not be 0). Nothing is concatenated on the host: each array is
 * copied to its place in the store. */
pf_status pf_sigma_upload_batch_parts(pf_sigma_ctx* ctx, uint32_t num_formulas, const uint32_t* num_vars,
                                      const uint64_t* num_clauses, const uint32_t* const* lits,
                                      const uint64_t* const* offsets);

/* Same as pf_sigma_upload_batch with lits/offsets in device memory. */
pf_status pf_sigma_upload_batch_device(pf_sigma_ctx* ctx, uint32_t num_formulas, const uint32_t* num_vars,
                                       const uint64_t* clause_begin, const uint32_t* d_lits,
                                       const uint64_t* d_offsets);

/* Per formula of the last batched round (arrays of num_formulas; any may be NULL):
 * status (PF_OK or PF_UNSAT), phases run, and the sizes pf_sigma_batch_download
 * writes for that formula. */
pf_status pf_sigma_batch_result_sizes(pf_sigma_ctx* ctx, int32_t* status, uint32_t* phases, uint64_t* num_clauses,
                                      uint64_t* num_literals, uint64_t* num_units, uint64_t* num_resolved);

/* Every formula's result, formula after formula, in its own numbering (any pointer
 * may be NULL): clauses (lits, offsets with sum(num_clauses) + 1 entries into lits,
 * learnt), trail units, witness stack, and num_vars[f] + 1 eliminated flags per
 * formula (the first of each unused), with the layouts of pf_sigma_download. */
pf_status pf_sigma_batch_download(pf_sigma_ctx* ctx, uint32_t* lits, uint64_t* offsets, uint8_t* learnt,
                                  uint32_t* units, uint32_t* resolved, uint8_t* eliminated);

/* A formula in host memory, as pf_dimacs_parse returns it: clause c has literals
 * lits[offsets[c] .. offsets[c+1]) (2*var + sign); the arrays belong to the library
 * and are released by pf_formula_free. */
typedef struct {
    uint32_t num_vars;
    uint64_t num_clauses;
    uint32_t* lits;
    uint64_t* offsets;  /* num_clauses + 1 */
    int32_t empty_clause; /* 1: the file holds an empty clause (the formula is unsatisfiable) */
} pf_formula;

/* Reads a DIMACS CNF file (ParaFROST::parser, src/cpu/dimacs.cpp:25-176): comments,
 * the "p cnf V C" header, clauses ended by 0. As the reference's toClause() does, a
 * repeated literal is dropped, a tautological clause is dropped and a variable above
 * V is an error (PF_EINVAL, text in pf_last_error). Every other clause is kept as
 * written, one-literal clauses included (pf_sigma_upload turns them into units); an
 * empty clause sets empty_clause and returns PF_UNSAT (the reference drops a clause
 * that its earlier units falsify; this reader keeps the contradiction). */
pf_status pf_dimacs_parse(const char* path, pf_formula* out);

/* Releases the arrays of a formula from pf_dimacs_parse. */
void pf_formula_free(pf_formula* f);

/* Device bytes held by the context. */
pf_status pf_sigma_footprint(pf_sigma_ctx* ctx, uint64_t* bytes);

/* Device allocations (cudaMalloc calls) this library has made in this process, over
 * all contexts and calls. No counterpart in the reference: lets a caller that
 * budgets device memory check that a call allocated nothing. */
uint64_t pf_device_alloc_count(void);

void pf_sigma_destroy(pf_sigma_ctx* ctx);

/* Text of the last error on this thread. */
const char* pf_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* SIGMA_GB300_H */
