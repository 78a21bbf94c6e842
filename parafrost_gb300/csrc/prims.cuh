// Device-wide primitives written for this library: exclusive scan and a stable
// LSD radix sort of (key, value) pairs. No CUB/Thrust: each is a few plain
// kernels (block reduce -> scan of block sums -> block scan; digit histogram ->
// digit-major scan -> stable warp-ranked scatter).
#pragma once

#include "device.cuh"

#include <algorithm>
#include <vector>

namespace sigma {

#if SIGMA_CUDA

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;  // per thread
constexpr int kScanTile = kScanThreads * kScanItems;

template <class T>
__device__ __forceinline__ T warp_incl_scan(T v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

template <class Tin, class T>
__global__ void scan_reduce_k(const Tin* in, size_t n, T* sums) {
    const size_t base = (size_t)blockIdx.x * kScanTile;
    T s = 0;
    for (int k = 0; k < kScanItems; k++) {
        const size_t i = base + (size_t)k * kScanThreads + threadIdx.x;
        if (i < n) s += (T)in[i];
    }
    // block reduce
    for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __shared__ T ws[kScanThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        T t = 0;
        for (int w = 0; w < kScanThreads / 32; w++) t += ws[w];
        sums[blockIdx.x] = t;
    }
}

// Single block: exclusive scan of the block sums in place; writes the grand total.
template <class T>
__global__ void scan_sums_k(T* sums, size_t nb, T* total) {
    __shared__ T carry_s;
    __shared__ T ws[kScanThreads / 32];
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    for (size_t base = 0; base < nb; base += kScanThreads) {
        const size_t i = base + threadIdx.x;
        const T v = i < nb ? sums[i] : T(0);
        const T incl = warp_incl_scan(v);
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if (lane == 31) ws[warp] = incl;
        __syncthreads();
        T wpre = 0, btot = 0;
        for (int w = 0; w < kScanThreads / 32; w++) {
            if (w < warp) wpre += ws[w];
            btot += ws[w];
        }
        const T carry = carry_s;
        if (i < nb) sums[i] = carry + wpre + incl - v;
        __syncthreads();
        if (threadIdx.x == 0) carry_s = carry + btot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total) *total = carry_s;
}

template <class Tin, class T>
__global__ void scan_down_k(const Tin* in, T* out, size_t n, const T* sums) {
    const size_t base = (size_t)blockIdx.x * kScanTile;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ T ws[kScanThreads / 32];
    __shared__ T carry_s;
    if (threadIdx.x == 0) carry_s = sums[blockIdx.x];
    __syncthreads();
    for (int k = 0; k < kScanItems; k++) {
        const size_t i = base + (size_t)k * kScanThreads + threadIdx.x;
        const T v = i < n ? (T)in[i] : T(0);
        const T incl = warp_incl_scan(v);
        if (lane == 31) ws[warp] = incl;
        __syncthreads();
        T wpre = 0, btot = 0;
        for (int w = 0; w < kScanThreads / 32; w++) {
            if (w < warp) wpre += ws[w];
            btot += ws[w];
        }
        const T carry = carry_s;
        if (i < n) out[i] = carry + wpre + incl - v;
        __syncthreads();
        if (threadIdx.x == 0) carry_s = carry + btot;
        __syncthreads();
    }
}

// out[i] = sum(in[0..i)), total (device pointer, may be null) = sum(in[0..n)).
// tmp needs scan_tmp_elems(n) elements of T.
inline size_t scan_tmp_elems(size_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

template <class Tin, class T>
void excl_scan(const Tin* in, T* out, size_t n, T* total, T* tmp, cudaStream_t s) {
    const size_t nb = (n + kScanTile - 1) / kScanTile;
    if (n == 0) {
        if (total) cudaMemsetAsync(total, 0, sizeof(T), s);
        return;
    }
    scan_reduce_k<Tin, T><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, tmp);
    scan_sums_k<T><<<1, kScanThreads, 0, s>>>(tmp, nb, total);
    scan_down_k<Tin, T><<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n, tmp);
}

// Single-pass exclusive scan (decoupled look-back): each tile takes its index from
// a counter in launch order, publishes its aggregate, adds the aggregates (or the
// first inclusive prefix) of the tiles before it, publishes its inclusive prefix
// and scans itself. Flags carry the scan's epoch, so nothing is cleared between
// scans; a tile index counter keeps running and base is where this scan's tiles
// start. A look-back wait that runs out records ERR_ITER in err.
struct Scan1State {
    u64* agg;       // per tile
    u64* incl;      // per tile
    u32* flag;      // per tile: epoch << 2 | 1 (aggregate) or | 2 (inclusive)
    u32* counter;   // tile index counter
    u32* err;
};

// A tile is kScan1Items consecutive items per thread: read once from memory in
// coalesced order into shared memory, scanned per thread in registers, combined
// across the block by one warp scan of the thread sums, and written back in
// coalesced order. Shared-memory positions are padded (one slot per 32) so the
// per-thread runs of consecutive items do not fall on one bank.
constexpr int kScan1Items = 16;
constexpr int kScan1Tile = kScanThreads * kScan1Items;
__device__ __forceinline__ int scan1_pad(int i) { return i + (i >> 5); }

template <class Tin, class T>
__global__ void __launch_bounds__(kScanThreads) scan1_k(const Tin* in, T* out, size_t n, T* total, Scan1State st,
                                                       u32 base, u32 epoch) {
    __shared__ T items[kScan1Tile + kScan1Tile / 32];
    __shared__ T ws[kScanThreads / 32];
    __shared__ u32 tile_s;
    __shared__ T carry_s;
    if (threadIdx.x == 0) tile_s = atomicAdd(st.counter, 1u) - base;
    __syncthreads();
    const u32 tile = tile_s;
    const size_t nb = (n + kScan1Tile - 1) / kScan1Tile;
    const size_t t0 = (size_t)tile * kScan1Tile;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kScan1Items; k++) {
        const int j = k * kScanThreads + threadIdx.x;
        const size_t i = t0 + (size_t)j;
        items[scan1_pad(j)] = i < n ? (T)in[i] : T(0);
    }
    __syncthreads();
    // this thread's run: items [threadIdx.x * kScan1Items, +kScan1Items)
    T run = 0;
    const int r0 = threadIdx.x * kScan1Items;
#pragma unroll
    for (int k = 0; k < kScan1Items; k++) run += items[scan1_pad(r0 + k)];
    const T incl = warp_incl_scan(run);
    if (lane == 31) ws[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        // block aggregate and per-warp offsets, then the look-back (as before, 32
        // tiles at a time: wait for their flags, add the aggregates after the
        // nearest inclusive prefix and stop there)
        T wv = lane < kScanThreads / 32 ? ws[lane] : T(0);
        const T winc = warp_incl_scan(wv);
        const T a = __shfl_sync(0xffffffffu, winc, kScanThreads / 32 - 1);
        if (lane < kScanThreads / 32) ws[lane] = winc - wv;
        T prefix = 0;
        if (lane == 0) {
            if (tile == 0) st.incl[0] = (u64)a;
            else st.agg[tile] = (u64)a;
            __threadfence();
            atomicExch(&st.flag[tile], (epoch << 2) | (tile == 0 ? 2u : 1u));
        }
        __syncwarp();
        bool late = false;
        for (long long top = (long long)tile - 1; top >= 0 && !late; top -= 32) {
            const long long p = top - lane;
            u32 f = (epoch << 2) | 1u;  // lanes past tile 0 add nothing
            u32 it = 0;
            if (p >= 0) {
                while (((f = *(volatile u32*)&st.flag[p]) >> 2) != epoch) {
                    if (++it > (1u << 24)) {
                        late = true;
                        break;
                    }
                    __nanosleep(32);
                }
            }
            late = __any_sync(0xffffffffu, late);
            if (late) break;
            __threadfence();
            const u32 incl_mask = __ballot_sync(0xffffffffu, p >= 0 && (f & 3u) == 2u);
            const int stop = incl_mask ? __ffs(incl_mask) - 1 : 32;
            T v = 0;
            if (p >= 0 && lane <= stop) {
                v = lane == stop ? (T)(*(volatile u64*)&st.incl[p]) : (T)(*(volatile u64*)&st.agg[p]);
            }
            for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            prefix += __shfl_sync(0xffffffffu, v, 0);
            if (incl_mask) break;
        }
        if (lane == 0) {
            if (late) atomicOr(st.err, ERR_ITER);
            if (tile != 0) {
                st.incl[tile] = (u64)(prefix + a);
                __threadfence();
                atomicExch(&st.flag[tile], (epoch << 2) | 2u);
            }
            if (tile + 1 == nb && total) *total = prefix + a;
            carry_s = prefix;
        }
    }
    __syncthreads();
    // exclusive prefixes of this thread's run, in place
    T acc = carry_s + ws[warp] + incl - run;
#pragma unroll
    for (int k = 0; k < kScan1Items; k++) {
        const int q = scan1_pad(r0 + k);
        const T v = items[q];
        items[q] = acc;
        acc += v;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kScan1Items; k++) {
        const int j = k * kScanThreads + threadIdx.x;
        const size_t i = t0 + (size_t)j;
        if (i < n) out[i] = items[scan1_pad(j)];
    }
}

inline size_t scan1_tiles(size_t n) { return (n + kScan1Tile - 1) / kScan1Tile; }

// ---------------------------------------------------------------- radix sort
constexpr int kRadixThreads = 256;
constexpr int kRadixChunks = 16;  // items per thread per tile
constexpr int kRadixTile = kRadixThreads * kRadixChunks;

__global__ void radix_hist_k(const u32* keys, size_t n, int shift, u32* hist, u32 nblocks) {
    __shared__ u32 h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const size_t base = (size_t)blockIdx.x * kRadixTile;
    for (int k = 0; k < kRadixChunks; k++) {
        const size_t i = base + (size_t)k * kRadixThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(size_t)d * nblocks + blockIdx.x] = h[d];
}

__global__ void radix_scatter_k(const u32* keys, const u32* vals, u32* okeys, u32* ovals, size_t n, int shift,
                                const u32* offs, u32 nblocks) {
    __shared__ u32 base_d[256];
    __shared__ u32 wcnt[kRadixThreads / 32][257];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < 256; d += blockDim.x) base_d[d] = offs[(size_t)d * nblocks + blockIdx.x];
    const size_t tbase = (size_t)blockIdx.x * kRadixTile;
    const u32 lt = (1u << lane) - 1u;
    for (int k = 0; k < kRadixChunks; k++) {
        for (int i = threadIdx.x; i < (kRadixThreads / 32) * 257; i += blockDim.x) (&wcnt[0][0])[i] = 0;
        __syncthreads();
        const size_t i = tbase + (size_t)k * kRadixThreads + threadIdx.x;
        const bool valid = i < n;
        const u32 key = valid ? keys[i] : 0u;
        const u32 d = valid ? ((key >> shift) & 255u) : 256u;
        const u32 peers = __match_any_sync(0xffffffffu, d);
        const u32 rank = __popc(peers & lt);
        if (rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            u32 pre = 0;
            for (int w = 0; w < warp; w++) pre += wcnt[w][d];
            const u32 pos = base_d[d] + pre + rank;
            if (pos < n) {
                okeys[pos] = key;
                ovals[pos] = vals[i];
            }
        }
        __syncthreads();
        if (threadIdx.x < 256) {
            u32 t = 0;
            for (int w = 0; w < kRadixThreads / 32; w++) t += wcnt[w][threadIdx.x];
            base_d[threadIdx.x] += t;
        }
        __syncthreads();
    }
}

inline size_t radix_hist_elems(size_t n) { return 256 * ((n + kRadixTile - 1) / kRadixTile) + 1; }

// Stable sort of (keys, vals) by the low `bits` bits of keys. Uses (k2, v2) as the
// ping-pong buffers; the result ends in (keys, vals). hist/hscan need
// radix_hist_elems(n) u32 each; stmp needs scan_tmp_elems(that) u32.
inline void radix_sort_pairs(u32* keys, u32* vals, u32* k2, u32* v2, size_t n, int bits, u32* hist, u32* hscan,
                             u32* stmp, cudaStream_t s) {
    if (n <= 1) return;
    const u32 nb = (u32)((n + kRadixTile - 1) / kRadixTile);
    u32 *ka = keys, *va = vals, *kb = k2, *vb = v2;
    int passes = 0;
    for (int shift = 0; shift < bits; shift += 8, passes++) {
        radix_hist_k<<<nb, kRadixThreads, 0, s>>>(ka, n, shift, hist, nb);
        excl_scan<u32, u32>(hist, hscan, (size_t)256 * nb, nullptr, stmp, s);
        radix_scatter_k<<<nb, kRadixThreads, 0, s>>>(ka, va, kb, vb, n, shift, hscan, nb);
        u32* t = ka; ka = kb; kb = t;
        t = va; va = vb; vb = t;
    }
    if (passes & 1) {
        cudaMemcpyAsync(keys, ka, n * sizeof(u32), cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(vals, va, n * sizeof(u32), cudaMemcpyDeviceToDevice, s);
    }
}

#else  // serial emulation

inline size_t scan_tmp_elems(size_t n) { return 1; }
inline size_t radix_hist_elems(size_t n) { return 1; }

template <class Tin, class T>
void excl_scan(const Tin* in, T* out, size_t n, T* total, T* /*tmp*/, void* /*stream*/) {
    T s = 0;
    for (size_t i = 0; i < n; i++) {
        const T v = (T)in[i];
        out[i] = s;
        s += v;
    }
    if (total) *total = s;
}

inline void radix_sort_pairs(u32* keys, u32* vals, u32*, u32*, size_t n, int bits, u32*, u32*, u32*, void*) {
    std::vector<size_t> idx(n);
    for (size_t i = 0; i < n; i++) idx[i] = i;
    const u32 mask = bits >= 32 ? 0xFFFFFFFFu : ((1u << bits) - 1u);
    std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return (keys[a] & mask) < (keys[b] & mask); });
    std::vector<u32> k(n), v(n);
    for (size_t i = 0; i < n; i++) { k[i] = keys[idx[i]]; v[i] = vals[idx[i]]; }
    std::copy(k.begin(), k.end(), keys);
    std::copy(v.begin(), v.end(), vals);
}

#endif

}  // namespace sigma
