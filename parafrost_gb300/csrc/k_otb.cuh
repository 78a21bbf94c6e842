// Occurrence-table build by literal buckets (createOT, src/cpu/simplify.cpp:35-56;
// GPU reference: histogram.cu:34-52, memory.cu:271-312, create_ot_k kernels.cu:81-96).
//
// The literal slots are cut into buckets of 2^shift consecutive slots. No pass
// issues one device-memory atomic per occurrence, and no pass writes outside the
// range of the bucket it works on:
//   pass 0 (ot_bucket_count_k): every occurrence (a literal of a live clause) adds
//     one to its bucket in a per-block shared histogram; one atomic per bucket per
//     block at the end. An exclusive scan of the bucket counts gives every bucket
//     its range of the table (all its literals' lists, side by side).
//   pass 1 (ot_bucket_fill_k): per tile of clauses, every occurrence (literal,
//     clause id, one 8-byte word) is staged in shared memory and counted per
//     bucket; a block scan orders the tile by bucket, one reservation per non-empty
//     bucket gives each run its place, and the runs are written out contiguously
//     (consecutive threads on consecutive words).
//   pass 2 (ot_bucket_lists_k): one block per bucket: per-slot counts in shared
//     memory, a block scan gives the list sizes and starts of the bucket's slots,
//     then every occurrence lands in its list inside the bucket's range.
// Clause headers and literals are read by whole warps, consecutive lanes on
// consecutive literals. The order inside one list is unspecified, as for the
// atomic build: the elected lists are sorted into the reference's order later.
#pragma once

#include "cnf.cuh"

namespace sigma {

#if SIGMA_CUDA

constexpr u32 OTB_TILE = 4096;      // clauses per block tile in pass 0
constexpr u32 OTB_FILL_CAP = 6144;   // occurrences of a pass-1 tile ordered in shared memory
                                     // (48 KB: three 512-thread blocks per SM)
constexpr u32 OTB_MAX_BUCKETS = 4096;
constexpr u32 OTB_MAX_SHIFT = 15;   // 32,768 slots: 128 KiB of shared counters in pass 2
constexpr u32 OTB_LIST_THREADS = 1024;  // one block a bucket, 32 warps to keep its loads in flight
constexpr unsigned OTB_FULL = 0xffffffffu;

struct OtbArgs {
    Ctx c;
    u32 shift;        // bucket of literal l: l >> shift
    u32 nb;           // buckets
    u32* count;       // nb: occurrences per bucket (pass 0)
    u32* cursor;      // nb: next free position of every bucket (pass 1; starts at base)
    const u32* base;  // nb + 1: first position of every bucket, base[nb] = occurrences
    u64* tpair;       // occurrences grouped by bucket: clause id << 32 | literal
    u32 fill_tile;    // clauses per pass-1 tile (a multiple of 32)
};

// The literals of the live clauses id0 .. id0+n-1 (n <= 32), walked by one warp with
// consecutive lanes on consecutive literals (clauses are mostly adjacent in the
// literal array, so the loads coalesce). f(valid, literal, clause id) is called by
// every lane of the warp in every step, valid false past the end.
template <class F>
DEV void warp_clause_literals(const Ctx& c, u32 id0, u32 n, F&& f) {
    const u32 lane = threadIdx.x & 31u;
    u32 start = 0, sz = 0;
    if (lane < n) {
        const Hdr h = hdr_ro(&c.hdr[id0 + lane]);
        if (!h_deleted(h.flags)) {
            start = h.start;
            sz = h.size;
        }
    }
    u32 incl = sz;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const u32 t = __shfl_up_sync(OTB_FULL, incl, o);
        if ((int)lane >= o) incl += t;
    }
    const u32 excl = incl - sz;
    const u32 total = __shfl_sync(OTB_FULL, incl, 31);
    for (u32 base = 0; base < total; base += 32) {
        const u32 j = base + lane;
        // owner: the first lane k whose inclusive end is past j
        u32 k = 0;
#pragma unroll
        for (u32 step = 16; step; step >>= 1) {
            const u32 v = __shfl_sync(OTB_FULL, incl, k + step - 1);
            if (v <= j) k += step;
        }
        const u32 st = __shfl_sync(OTB_FULL, start, k & 31u), ex = __shfl_sync(OTB_FULL, excl, k & 31u);
        const bool valid = j < total;
        const u32 lit = valid ? __ldg(&c.lits[st + (j - ex)]) : 0u;
        f(valid, lit, id0 + k);
    }
}

// Pass 0: occurrences per bucket.
__global__ void __launch_bounds__(256) ot_bucket_count_k(OtbArgs a) {
    extern __shared__ u32 otb_hist[];
    for (u32 b = threadIdx.x; b < a.nb; b += blockDim.x) otb_hist[b] = 0;
    __syncthreads();
    const u32 warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const u32 ngroups = (a.c.ncls + 31u) / 32u;
    for (u32 g = blockIdx.x * nw + warp; g < ngroups; g += gridDim.x * nw) {
        const u32 id0 = g * 32u;
        const u32 n = a.c.ncls - id0 < 32u ? a.c.ncls - id0 : 32u;
        warp_clause_literals(a.c, id0, n, [&](bool valid, u32 lit, u32) {
            if (valid) atomicAdd(&otb_hist[lit >> a.shift], 1u);
        });
    }
    __syncthreads();
    for (u32 b = threadIdx.x; b < a.nb; b += blockDim.x)
        if (otb_hist[b]) atomicAdd(&a.count[b], otb_hist[b]);
}

// Block-wide exclusive scan of cnt[0, n) in place; returns the total. Every thread
// of the block calls it.
DEV u32 otb_block_scan(u32* cnt, u32 n, u32* warp_tot, u32* carry) {
    const u32 tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) *carry = 0;
    __syncthreads();
    for (u32 i0 = 0; i0 < n; i0 += blockDim.x) {
        const u32 i = i0 + tid;
        const u32 v = i < n ? cnt[i] : 0u;
        u32 incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u32 t = __shfl_up_sync(OTB_FULL, incl, o);
            if ((int)lane >= o) incl += t;
        }
        if (lane == 31) warp_tot[warp] = incl;
        __syncthreads();
        u32 before = *carry;
        for (u32 w = 0; w < warp; w++) before += warp_tot[w];
        if (i < n) cnt[i] = before + incl - v;
        __syncthreads();
        if (tid == blockDim.x - 1) *carry = before + incl;
        __syncthreads();
    }
    return *carry;
}

// Pass 1: occurrences grouped by bucket. A tile's occurrences are counted per
// bucket (shared counters), one reservation per non-empty bucket gives each run its
// place, a block scan of the counts orders the tile by bucket, and a second walk of
// the tile's literals (just read, so mostly cache hits) places every occurrence in
// shared memory at its bucket's position; the runs are then written out contiguously.
// A tile with more occurrences than shared memory holds (very long clauses) writes
// them to their runs directly instead. Tiles hold fill_tile clauses, sized from the
// mean clause length so that a tile's occurrences nearly fill the stage.
constexpr u32 OTB_FILL_THREADS = 512;
__global__ void __launch_bounds__(OTB_FILL_THREADS) ot_bucket_fill_k(OtbArgs a) {
    extern __shared__ u64 otb_fsm[];
    u64* sorted = otb_fsm;                                      // OTB_FILL_CAP
    u32* cnt = reinterpret_cast<u32*>(otb_fsm + OTB_FILL_CAP);  // nb: counts, then tile offsets
    u32* run = cnt + a.nb;                                      // nb: global start of the tile's run
    u32* cur = run + a.nb;                                      // nb: cursors
    __shared__ u32 warp_tot[OTB_FILL_THREADS / 32];
    __shared__ u32 carry, ntile;
    const u32 warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const u32 T = a.fill_tile;
    const u32 ntiles = (a.c.ncls + T - 1u) / T;
    for (u32 t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const u32 c0 = t * T, c1 = a.c.ncls - c0 < T ? a.c.ncls : c0 + T;
        for (u32 b = threadIdx.x; b < a.nb; b += blockDim.x) cnt[b] = 0;
        if (threadIdx.x == 0) ntile = 0;
        __syncthreads();
        for (u32 g = c0 + warp * 32u; g < c1; g += nw * 32u)
            warp_clause_literals(a.c, g, c1 - g < 32u ? c1 - g : 32u, [&](bool valid, u32 lit, u32) {
                const unsigned m = __ballot_sync(OTB_FULL, valid);
                if ((threadIdx.x & 31u) == 0 && m) atomicAdd(&ntile, (u32)__popc(m));
                if (valid) atomicAdd(&cnt[lit >> a.shift], 1u);
            });
        __syncthreads();
        const u32 n = ntile;
        for (u32 b = threadIdx.x; b < a.nb; b += blockDim.x) {
            const u32 k = cnt[b];
            run[b] = k ? atomicAdd(&a.cursor[b], k) : 0u;
        }
        if (n <= OTB_FILL_CAP) {
            otb_block_scan(cnt, a.nb, warp_tot, &carry);
            for (u32 b = threadIdx.x; b < a.nb; b += blockDim.x) cur[b] = cnt[b];
            __syncthreads();
            for (u32 g = c0 + warp * 32u; g < c1; g += nw * 32u)
                warp_clause_literals(a.c, g, c1 - g < 32u ? c1 - g : 32u, [&](bool valid, u32 lit, u32 cid) {
                    if (valid) sorted[atomicAdd(&cur[lit >> a.shift], 1u)] = ((u64)cid << 32) | lit;
                });
            __syncthreads();
            for (u32 i = threadIdx.x; i < n; i += blockDim.x) {
                const u64 x = sorted[i];
                const u32 b = (u32)x >> a.shift;
                a.tpair[run[b] + (i - cnt[b])] = x;
            }
        } else {
            for (u32 b = threadIdx.x; b < a.nb; b += blockDim.x) cur[b] = 0;
            __syncthreads();
            for (u32 g = c0 + warp * 32u; g < c1; g += nw * 32u)
                warp_clause_literals(a.c, g, c1 - g < 32u ? c1 - g : 32u, [&](bool valid, u32 lit, u32 cid) {
                    if (!valid) return;
                    const u32 b = lit >> a.shift;
                    a.tpair[run[b] + atomicAdd(&cur[b], 1u)] = ((u64)cid << 32) | lit;
                });
        }
        __syncthreads();
    }
}

// Pass 2: one block per bucket. Shared memory: 2^shift slot counters.
__global__ void __launch_bounds__(OTB_LIST_THREADS) ot_bucket_lists_k(OtbArgs a) {
    extern __shared__ u32 otb_cnt[];
    __shared__ u32 warp_tot[OTB_LIST_THREADS / 32];
    __shared__ u32 carry;
    const u32 b = blockIdx.x;
    const u32 l0 = b << a.shift;
    const u32 D = a.c.D;
    const u32 nl = D - l0 < (1u << a.shift) ? D - l0 : (1u << a.shift);
    const u32 p0 = a.base[b], p1 = a.base[b + 1];
    const u32 tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    for (u32 i = tid; i < nl; i += blockDim.x) otb_cnt[i] = 0;
    if (tid == 0) carry = 0;
    __syncthreads();
    // four occurrences per thread per step, their loads issued before the atomics; the
    // staged pairs are read twice and then dead (evicted first), the lists' lines are
    // filled by scattered stores and kept while they fill
    const u64 pf = l2_policy_first(), pl = l2_policy_last();
    const u32 step = 4u * blockDim.x;
    for (u32 k0 = p0 + tid; k0 < p1; k0 += step) {
        u64 x[4];
#pragma unroll
        for (u32 j = 0; j < 4; j++) x[j] = k0 + j * blockDim.x < p1 ? ldcg_hint64(&a.tpair[k0 + j * blockDim.x], pf) : 0ull;
#pragma unroll
        for (u32 j = 0; j < 4; j++)
            if (k0 + j * blockDim.x < p1) atomicAdd(&otb_cnt[(u32)x[j] - l0], 1u);
    }
    __syncthreads();
    // block scan of the slot counts, blockDim.x slots per step: list sizes and starts
    for (u32 i0 = 0; i0 < nl; i0 += blockDim.x) {
        const u32 i = i0 + tid;
        const u32 v = i < nl ? otb_cnt[i] : 0u;
        u32 incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u32 t = __shfl_up_sync(OTB_FULL, incl, o);
            if ((int)lane >= o) incl += t;
        }
        if (lane == 31) warp_tot[warp] = incl;
        __syncthreads();
        u32 before = carry;
        for (u32 w = 0; w < warp; w++) before += warp_tot[w];
        const u32 excl = before + incl - v;
        if (i < nl) {
            a.c.ot_size[l0 + i] = v;
            a.c.ot_off[l0 + i] = p0 + excl;
            otb_cnt[i] = excl;
        }
        __syncthreads();
        if (tid == blockDim.x - 1) carry = excl + v;
        __syncthreads();
    }
    for (u32 k0 = p0 + tid; k0 < p1; k0 += step) {
        u64 x[4];
#pragma unroll
        for (u32 j = 0; j < 4; j++) x[j] = k0 + j * blockDim.x < p1 ? ldcg_hint64(&a.tpair[k0 + j * blockDim.x], pf) : 0ull;
#pragma unroll
        for (u32 j = 0; j < 4; j++)
            if (k0 + j * blockDim.x < p1)
                st_hint(&a.c.ot_refs[p0 + atomicAdd(&otb_cnt[(u32)x[j] - l0], 1u)], (u32)(x[j] >> 32), pl);
    }
}

#endif  // SIGMA_CUDA

}  // namespace sigma
