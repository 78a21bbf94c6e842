// Device abstraction for the sigma_gb300 kernels.
//
// Every kernel is written as a per-item __host__ __device__ function plus a thin
// grid-stride __global__ wrapper. The CUDA build launches the wrappers; the
// serial emulation build (SIGMA_EMU, compiled by g++ for the CPU test suite only)
// calls the item functions in a loop, so kernel logic can be checked without a
// GPU. The product library is always the CUDA build.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__) && !defined(SIGMA_EMU)
#define SIGMA_CUDA 1
#include <cuda_runtime.h>
#define HD __host__ __device__ __forceinline__
#define DEV __device__ __forceinline__
#else
#define SIGMA_CUDA 0
#define HD inline
#define DEV inline
#define __align__(n) alignas(n)
#endif

namespace sigma {

typedef uint32_t u32;
typedef uint64_t u64;
typedef int64_t i64;

// ---------------------------------------------------------------- atomics
// Sequential emulation performs plain read-modify-writes.
HD u32 atom_add(u32* p, u32 v) {
#if defined(__CUDA_ARCH__)
    return atomicAdd(p, v);
#else
    u32 o = *p; *p = o + v; return o;
#endif
}
HD u64 atom_add64(u64* p, u64 v) {
#if defined(__CUDA_ARCH__)
    return (u64)atomicAdd((unsigned long long*)p, (unsigned long long)v);
#else
    u64 o = *p; *p = o + v; return o;
#endif
}
HD u32 atom_min(u32* p, u32 v) {
#if defined(__CUDA_ARCH__)
    return atomicMin(p, v);
#else
    u32 o = *p; if (v < o) *p = v; return o;
#endif
}
HD u64 atom_min64(u64* p, u64 v) {
#if defined(__CUDA_ARCH__)
    return (u64)atomicMin((unsigned long long*)p, (unsigned long long)v);
#else
    u64 o = *p; if (v < o) *p = v; return o;
#endif
}
HD u32 atom_max(u32* p, u32 v) {
#if defined(__CUDA_ARCH__)
    return atomicMax(p, v);
#else
    u32 o = *p; if (v > o) *p = v; return o;
#endif
}
HD u32 atom_cas(u32* p, u32 cmp, u32 v) {
#if defined(__CUDA_ARCH__)
    return atomicCAS(p, cmp, v);
#else
    u32 o = *p; if (o == cmp) *p = v; return o;
#endif
}
HD u64 atom_or64(u64* p, u64 v) {
#if defined(__CUDA_ARCH__)
    return (u64)atomicOr((unsigned long long*)p, (unsigned long long)v);
#else
    u64 o = *p; *p = o | v; return o;
#endif
}
HD u32 atom_or(u32* p, u32 v) {
#if defined(__CUDA_ARCH__)
    return atomicOr(p, v);
#else
    u32 o = *p; *p = o | v; return o;
#endif
}
HD u32 atom_exch(u32* p, u32 v) {
#if defined(__CUDA_ARCH__)
    return atomicExch(p, v);
#else
    u32 o = *p; *p = v; return o;
#endif
}
// Add to one counter from many threads: the active lanes of a warp combine their
// values first, so the counter sees one atomic per warp.
HD void warp_sum_add64(u64* p, u64 v) {
#if defined(__CUDA_ARCH__)
    const unsigned mask = __activemask();
    if (mask != 0xffffffffu) {  // partial warp (tail of a grid-stride loop): plain atomics
        atomicAdd((unsigned long long*)p, (unsigned long long)v);
        return;
    }
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd((unsigned long long*)p, (unsigned long long)v);
#else
    *p += v;
#endif
}

// Sum into one of kSpreadSlots words chosen by the block (the caller adds the
// slots up): a sum that every warp of a large launch feeds would otherwise queue
// all its atomics on one address.
constexpr u32 kSpreadSlots = 32;
HD void spread_sum_add64(u64* slots, u64 v) {
#if defined(__CUDA_ARCH__)
    warp_sum_add64(slots + (blockIdx.x & (kSpreadSlots - 1u)), v);
#else
    slots[0] += v;
#endif
}

// Maximum into one word from many threads: one atomic per full warp, and only
// when the warp's value exceeds what the word already holds (the word settles
// early, so most warps only read it).
HD void warp_max_atomic(u32* p, u32 v) {
#if defined(__CUDA_ARCH__)
    if (__activemask() != 0xffffffffu) {
        if (v > *(volatile u32*)p) atomicMax(p, v);
        return;
    }
    v = __reduce_max_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0 && v > *(volatile u32*)p) atomicMax(p, v);
#else
    if (v > *p) *p = v;
#endif
}

// Sets bit v of a zeroed bitmap when pred holds: the lanes of a warp that share a
// word combine their bits and one of them ORs the word.
HD void bitmap_set(u32* bits, u32 v, bool pred) {
#if defined(__CUDA_ARCH__)
    const unsigned mask = __activemask();
    const unsigned peers = __match_any_sync(mask, v >> 5);
    const u32 b = __reduce_or_sync(peers, pred ? 1u << (v & 31u) : 0u);
    if (b && (threadIdx.x & 31u) == (u32)(__ffs(peers) - 1)) atomicOr(&bits[v >> 5], b);
#else
    if (pred) bits[v >> 5] |= 1u << (v & 31u);
#endif
}

// Append to a list through one shared counter: the lanes of a warp that append
// reserve their slots with one atomic. Returns the slot (only meaningful when pred).
HD u32 warp_append(u32* counter, bool pred) {
#if defined(__CUDA_ARCH__)
    const unsigned mask = __activemask();
    const unsigned bal = __ballot_sync(mask, pred);
    if (!bal) return 0;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(bal) - 1;
    u32 base = 0;
    if (lane == leader) base = atomicAdd(counter, (u32)__popc(bal));
    base = __shfl_sync(mask, base, leader);
    return base + (u32)__popc(bal & ((1u << lane) - 1u));
#else
    if (!pred) return 0;
    const u32 o = *counter;
    *counter = o + 1;
    return o;
#endif
}

// ---------------------------------------------------------------- warp steps
// Warp-cooperative code is written as uniform steps whose per-lane parts are
// lambdas of the lane (or item) index. On the GPU every lane of the warp runs the
// same step; the serial emulation runs the step once, evaluating the lambda for each
// lane in turn, so the same source is checked on the CPU.
constexpr u32 kFull = 0xffffffffu;

HD u32 lane_id() {
#if defined(__CUDA_ARCH__)
    return threadIdx.x & 31u;
#else
    return 0;
#endif
}
HD void wsync() {
#if defined(__CUDA_ARCH__)
    __syncwarp();
#endif
}
// f(i) for i in [0, n), items strided over the lanes; ends with a warp barrier.
template <class F>
HD void wfor(u32 n, F f) {
#if defined(__CUDA_ARCH__)
    for (u32 i = threadIdx.x & 31u; i < n; i += 32) f(i);
    __syncwarp();
#else
    for (u32 i = 0; i < n; i++) f(i);
#endif
}
// Bit l set when p(l) holds, for lanes l < 32.
template <class P>
HD u32 wballot(P p) {
#if defined(__CUDA_ARCH__)
    return __ballot_sync(kFull, p(threadIdx.x & 31u));
#else
    u32 m = 0;
    for (u32 l = 0; l < 32; l++) if (p(l)) m |= 1u << l;
    return m;
#endif
}
// Sum of f(i) over i in [0, n).
template <class F>
HD u32 wsum(u32 n, F f) {
#if defined(__CUDA_ARCH__)
    u32 s = 0;
    for (u32 i = threadIdx.x & 31u; i < n; i += 32) s += f(i);
    return __reduce_add_sync(kFull, s);
#else
    u32 s = 0;
    for (u32 i = 0; i < n; i++) s += f(i);
    return s;
#endif
}
template <class F>
HD u64 wsum64(u32 n, F f) {
#if defined(__CUDA_ARCH__)
    u64 s = 0;
    for (u32 i = threadIdx.x & 31u; i < n; i += 32) s += f(i);
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(kFull, s, o);
    return s;
#else
    u64 s = 0;
    for (u32 i = 0; i < n; i++) s += f(i);
    return s;
#endif
}
// Smallest i in [0, n) with p(i), or NONE_IDX. p is evaluated on batches of 32 in
// order and stops at the first batch with a hit.
constexpr u32 NONE_IDX = 0xFFFFFFFFu;
template <class P>
HD u32 wfirst(u32 n, P p) {
    for (u32 base = 0; base < n; base += 32) {
        const u32 m = wballot([&](u32 l) { return base + l < n && p(base + l); });
#if defined(__CUDA_ARCH__)
        if (m) return base + (u32)(__ffs(m) - 1);
#else
        if (m) return base + (u32)__builtin_ctz(m);
#endif
    }
    return NONE_IDX;
}
// Smallest i in [0, n) with p(i) (NONE_IDX if none), and in kmin the minimum of
// key(i) over every such i (NONE_IDX if none), in one pass.
template <class P, class K>
HD u32 wfirst_min(u32 n, P p, K key, u32& kmin) {
#if defined(__CUDA_ARCH__)
    u32 first = NONE_IDX, m = NONE_IDX;
    for (u32 base = 0; base < n; base += 32) {
        const u32 i = base + (threadIdx.x & 31u);
        const bool ok = i < n && p(i);
        const u32 b = __ballot_sync(kFull, ok);
        if (first == NONE_IDX && b) first = base + (u32)(__ffs(b) - 1);
        const u32 k = ok ? key(i) : NONE_IDX;
        if (k < m) m = k;
    }
    kmin = __reduce_min_sync(kFull, m);
    return first;
#else
    u32 first = NONE_IDX, m = NONE_IDX;
    for (u32 i = 0; i < n; i++) {
        if (!p(i)) continue;
        if (first == NONE_IDX) first = i;
        const u32 k = key(i);
        if (k < m) m = k;
    }
    kmin = m;
    return first;
#endif
}
// Minimum of f(i) over i in [0, n) (f returns NONE_IDX for "no value").
template <class F>
HD u32 wmin(u32 n, F f) {
#if defined(__CUDA_ARCH__)
    u32 m = NONE_IDX;
    for (u32 i = threadIdx.x & 31u; i < n; i += 32) { const u32 x = f(i); if (x < m) m = x; }
    return __reduce_min_sync(kFull, m);
#else
    u32 m = NONE_IDX;
    for (u32 i = 0; i < n; i++) { const u32 x = f(i); if (x < m) m = x; }
    return m;
#endif
}
// Runs f once per warp (lane 0), then a warp barrier.
template <class F>
HD void wone(F f) {
#if defined(__CUDA_ARCH__)
    if ((threadIdx.x & 31u) == 0) f();
    __syncwarp();
#else
    f();
#endif
}
// Value of lane `src`'s v (uniform broadcast; the emulation's v is already uniform).
HD u32 wbcast(u32 v, u32 src) {
#if defined(__CUDA_ARCH__)
    return __shfl_sync(kFull, v, (int)src);
#else
    (void)src;
    return v;
#endif
}

// Largest f < n with start[f] <= key (start ascending, start[0] <= key): the
// segment holding item `key` of a list of segments given by their starts.
template <class T>
HD u32 upper_segment(const T* start, u32 n, T key) {
    u32 lo = 0, hi = n;  // answer in [lo, hi)
    while (hi - lo > 1) {
        const u32 mid = (lo + hi) >> 1;
        if (start[mid] <= key) lo = mid;
        else hi = mid;
    }
    return lo;
}

#if SIGMA_CUDA
// Work of the per-variable warp kernels: warps take elected variables from one counter
// in work order (longest lists first), kWarpChunkFar at a time while more than
// kWarpFarLeft variables a warp are left (millions of elected variables: fewer atomics
// on the counter), else kWarpChunkNear at a time (measured: larger chunks slow the
// AIG workload's 0.8M-variable phases, where a warp's share is about 80 variables).
constexpr u32 kWarpChunkFar = 16, kWarpChunkNear = 4, kWarpFarLeft = 128;
DEV u32 warp_chunk(u32 left) {
    const u32 warps = (gridDim.x * blockDim.x) >> 5;
    return (u64)left > (u64)warps * kWarpFarLeft ? kWarpChunkFar : kWarpChunkNear;
}
#endif

// Volatile load for values that other threads of the same launch may update.
HD u32 vload(const u32* p) { return *(const volatile u32*)p; }
HD u64 vload64(const u64* p) { return *(const volatile u64*)p; }
// Load through the read-only path, for data no thread writes during the launch.
template <class T>
HD T ldro(const T* p) {
#if defined(__CUDA_ARCH__)
    return __ldg(p);
#else
    return *p;
#endif
}

HD int popc32(u32 x) {
#if defined(__CUDA_ARCH__)
    return __popc(x);
#else
    return __builtin_popcount(x);
#endif
}

// Four words in one 16-byte load (usable in host and device code alike).
struct __align__(16) Q4 {
    u32 x, y, z, w;
};
// L2 eviction priorities for loads and stores (PTX createpolicy + .L2::cache_hint):
// streams read once (clause records, occurrence lists, staged pairs) go first, so
// the small arrays read again and again (independent-set words) and lines still
// being filled by scattered stores stay in L2. In the emulation build they are
// plain accesses.
#if SIGMA_CUDA
DEV u64 l2_policy_first() {
    u64 p = 0;
#if defined(__CUDA_ARCH__)
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
#endif
    return p;
}
DEV u64 l2_policy_last() {
    u64 p = 0;
#if defined(__CUDA_ARCH__)
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
#endif
    return p;
}
#endif
// read-only load (no thread writes it during the launch) with a policy
HD u32 ldro_hint(const u32* p, u64 pol) {
#if defined(__CUDA_ARCH__)
    u32 v;
    asm("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    return v;
#else
    (void)pol;
    return *p;
#endif
}
// load of a word other blocks write during the launch (at L2, past L1) with a policy
HD u32 ldcg_hint(const u32* p, u64 pol) {
#if defined(__CUDA_ARCH__)
    u32 v;
    asm volatile("ld.global.cg.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol) : "memory");
    return v;
#else
    (void)pol;
    return *(const volatile u32*)p;
#endif
}
HD u64 ldcg_hint64(const u64* p, u64 pol) {
#if defined(__CUDA_ARCH__)
    u64 v;
    asm volatile("ld.global.cg.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(v) : "l"(p), "l"(pol) : "memory");
    return v;
#else
    (void)pol;
    return *(const volatile u64*)p;
#endif
}
HD void st_hint(u32* p, u32 v, u64 pol) {
#if defined(__CUDA_ARCH__)
    asm volatile("st.global.L2::cache_hint.u32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(pol) : "memory");
#else
    (void)pol;
    *p = v;
#endif
}
HD Q4 ldro4(const Q4* p) {
#if defined(__CUDA_ARCH__)
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(p));
    Q4 q;
    q.x = v.x;
    q.y = v.y;
    q.z = v.z;
    q.w = v.w;
    return q;
#else
    return *p;
#endif
}
HD Q4 ldro4_hint(const Q4* p, u64 pol) {
#if defined(__CUDA_ARCH__)
    Q4 q;
    asm("ld.global.nc.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
        : "=r"(q.x), "=r"(q.y), "=r"(q.z), "=r"(q.w)
        : "l"(p), "l"(pol));
    return q;
#else
    (void)pol;
    return *p;
#endif
}

// Pair of words (usable in host and device code alike).
struct U2 {
    u32 x, y;
};
HD U2 mk_u2(u32 x, u32 y) { U2 r; r.x = x; r.y = y; return r; }

// Error word bits (sticky per context; read back by the host after a stage).
enum : u32 {
    ERR_UNSAT = 1u << 0,        // a stage derived the empty clause
    ERR_CAP_CLAUSES = 1u << 1,  // clause-slot capacity exceeded
    ERR_CAP_LITS = 1u << 2,     // literal-pool capacity exceeded
    ERR_CAP_WITNESS = 1u << 3,  // witness-stack capacity exceeded
    ERR_CAP_SCRATCH = 1u << 4,  // per-variable scratch exceeded
    ERR_ITER = 1u << 5,         // a bounded iteration gave up
    ERR_INTERNAL = 1u << 6,     // invariant violated (bug)
    ERR_INPUT = 1u << 7,        // invalid input formula
};

#if SIGMA_CUDA
// ---------------------------------------------------------------- grid barrier
constexpr u64 kBarrierNs = 2000000000ull;  // a barrier wait longer than 2 s is an error

DEV u64 global_ns() {
    u64 t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Barrier over all blocks of a cooperative launch. A block whose wait runs out
// records ERR_ITER and gets false (the launch then winds down). With snap_src, the
// last block to arrive copies *snap_src to *snap_dst before it releases the others:
// a counter that blocks advance between barriers, read at a moment when every block
// is inside the barrier, so every block reads the same value after it.
DEV bool grid_barrier(u32* bar, u32* err, const u32* snap_src = nullptr, u32* snap_dst = nullptr) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        const u32 gen = vload(&bar[1]);
        __threadfence();
        if (atomicAdd(&bar[0], 1u) == gridDim.x - 1) {
            if (snap_src) *(volatile u32*)snap_dst = vload(snap_src);
            atomicExch(&bar[0], 0u);
            __threadfence();
            atomicAdd(&bar[1], 1u);
        } else {
            const u64 t0 = global_ns();
            while (vload(&bar[1]) == gen) {
                if (global_ns() - t0 > kBarrierNs) {
                    atomicOr(err, ERR_ITER);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}
#endif


}  // namespace sigma
