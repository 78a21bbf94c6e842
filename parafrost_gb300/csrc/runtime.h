// Host-side runtime: device buffers, stream, launches, events. The CUDA build
// uses the CUDA runtime; the serial emulation build (SIGMA_EMU, CPU tests only)
// uses host memory and runs item functions in a loop.
#pragma once

#include "device.cuh"

#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace sigma {

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct OomError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

#if SIGMA_CUDA
typedef cudaStream_t Stream;
inline void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}
#else
typedef void* Stream;
#endif

// Device allocations made by the library in this process (every one goes through
// Runtime::alloc); read by pf_device_alloc_count.
inline std::atomic<unsigned long long>& device_alloc_count() {
    static std::atomic<unsigned long long> n{0};
    return n;
}

// Grid-stride launch of a functor f(i) for i in [0, n).
#if SIGMA_CUDA
template <class F>
__global__ void for_each_k(F f, u32 n) {
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += blockDim.x * gridDim.x) f(i);
}
// Dynamic scheduling: every warp takes the next 32 items from a shared counter until
// none are left, so long items do not leave most SMs idle at the end.
template <class F>
__global__ void for_each_dyn_k(F f, u32 n, u32* next) {
    const u32 lane = threadIdx.x & 31u;
    while (true) {
        u32 base = 0;
        if (lane == 0) base = atomicAdd(next, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const u32 i = base + lane;
        if (i < n) f(i);
        __syncwarp();
    }
}
template <class F>
__global__ void single_k(F f) {
    if (blockIdx.x == 0 && threadIdx.x == 0) f();
}
#endif

struct Runtime {
    Stream stream = nullptr;
    int sms = 152;
    size_t bytes_live = 0;
    size_t budget = 0;  // 0 = no limit
    unsigned launches = 0;
    unsigned syncs = 0;  // host waits for the device (synchronous reads, stream and event syncs)

    void init() {
#if SIGMA_CUDA
        int dev = 0;
        ck(cudaGetDevice(&dev), "cudaGetDevice");
        ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attr");
        ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream");
#endif
    }
    void destroy() {
#if SIGMA_CUDA
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
#endif
    }
    void* alloc(size_t bytes) {
        if (bytes == 0) bytes = 16;
        if (budget && bytes_live + bytes > budget) throw OomError("device memory budget exceeded");
        void* p = nullptr;
#if SIGMA_CUDA
        if (cudaMalloc(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            throw OomError("cudaMalloc failed");
        }
#else
        p = std::malloc(bytes);
        if (!p) throw OomError("malloc failed");
#endif
        device_alloc_count().fetch_add(1, std::memory_order_relaxed);
        bytes_live += bytes;
        return p;
    }
    void release(void* p, size_t bytes) {
        if (!p) return;
#if SIGMA_CUDA
        cudaFree(p);
#else
        std::free(p);
#endif
        bytes_live -= bytes ? bytes : 16;
    }
    void h2d(void* d, const void* h, size_t b) {
        if (!b) return;
#if SIGMA_CUDA
        ck(cudaMemcpyAsync(d, h, b, cudaMemcpyHostToDevice, stream), "h2d");
#else
        std::memcpy(d, h, b);
#endif
    }
    // queued on the stream; the caller synchronises before reading h
    void d2h_async(void* h, const void* d, size_t b) {
        if (!b) return;
#if SIGMA_CUDA
        ck(cudaMemcpyAsync(h, d, b, cudaMemcpyDeviceToHost, stream), "d2h");
#else
        std::memcpy(h, d, b);
#endif
    }
    void d2h(void* h, const void* d, size_t b) {
        if (!b) return;
        syncs++;
#if SIGMA_CUDA
        ck(cudaMemcpyAsync(h, d, b, cudaMemcpyDeviceToHost, stream), "d2h");
        ck(cudaStreamSynchronize(stream), "sync");
#else
        std::memcpy(h, d, b);
#endif
    }
    void d2d(void* d, const void* s, size_t b) {
        if (!b) return;
#if SIGMA_CUDA
        ck(cudaMemcpyAsync(d, s, b, cudaMemcpyDeviceToDevice, stream), "d2d");
#else
        std::memmove(d, s, b);
#endif
    }
    void zero(void* d, size_t b, int byte = 0) {
        if (!b) return;
#if SIGMA_CUDA
        ck(cudaMemsetAsync(d, byte, b, stream), "memset");
#else
        std::memset(d, byte, b);
#endif
    }
    void sync() {
        syncs++;
#if SIGMA_CUDA
        ck(cudaStreamSynchronize(stream), "sync");
#endif
    }
    u32 grid(u32 n, int per_sm = 8) const {
        u64 g = ((u64)n + 255) / 256;
        const u64 cap = (u64)sms * per_sm;
        if (g > cap) g = cap;
        return g ? (u32)g : 1u;
    }
    template <class F>
    void each(const F& f, u32 n) {
        if (!n) return;
        launches++;
#if SIGMA_CUDA
        for_each_k<F><<<grid(n), 256, 0, stream>>>(f, n);
        ck(cudaGetLastError(), "launch");
#else
        for (u32 i = 0; i < n; i++) f(i);
#endif
    }
    // f(i) for i in [0, n) with dynamic warp-chunk scheduling; `next` is a device
    // counter the call resets.
    template <class F>
    void each_dyn(const F& f, u32 n, u32* next) {
        if (!n) return;
        launches++;
#if SIGMA_CUDA
        ck(cudaMemsetAsync(next, 0, 4, stream), "memset");
        u32 g = (u32)sms * 8u;
        const u32 need = (n + 255u) / 256u;
        if (g > need) g = need;
        for_each_dyn_k<F><<<g, 256, 0, stream>>>(f, n, next);
        ck(cudaGetLastError(), "launch");
#else
        (void)next;
        for (u32 i = 0; i < n; i++) f(i);
#endif
    }
    template <class F>
    void one(const F& f) {
        launches++;
#if SIGMA_CUDA
        single_k<F><<<1, 32, 0, stream>>>(f);
        ck(cudaGetLastError(), "launch");
#else
        f();
#endif
    }
};

template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    Runtime* rt = nullptr;
    void reserve(Runtime& r, size_t count) {
        rt = &r;
        if (count <= n && p) return;
        free();
        rt = &r;
        p = (T*)r.alloc(count * sizeof(T));
        n = count;
    }
    // grow keeping the first `keep` elements
    void grow(Runtime& r, size_t count, size_t keep) {
        if (count <= n && p) return;
        T* q = (T*)r.alloc(count * sizeof(T));
        if (p && keep) r.d2d(q, p, keep * sizeof(T));
        if (p) r.release(p, n * sizeof(T));
        p = q;
        n = count;
        rt = &r;
    }
    void free() {
        if (p && rt) rt->release(p, n * sizeof(T));
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
};

// Device-time stage timer (CUDA events on the context stream; wall clock in emulation).
// Device time of one kernel over a round: an event pair around each launch, read
// once after the round has finished (no synchronisation per launch).
struct KernelClock {
#if SIGMA_CUDA
    std::vector<cudaEvent_t> ev;
#else
    std::chrono::steady_clock::time_point t0;
    double acc = 0;
#endif
    size_t used = 0;
    void start(Runtime& rt) {
#if SIGMA_CUDA
        while (used + 2 > ev.size()) {
            cudaEvent_t e;
            ck(cudaEventCreate(&e), "event");
            ev.push_back(e);
        }
        ck(cudaEventRecord(ev[used], rt.stream), "event");
#else
        (void)rt;
        t0 = std::chrono::steady_clock::now();
#endif
    }
    void stop(Runtime& rt) {
#if SIGMA_CUDA
        ck(cudaEventRecord(ev[used + 1], rt.stream), "event");
#else
        (void)rt;
        acc += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
#endif
        used += 2;
    }
    u32 launches() const { return (u32)(used / 2); }
    // Sum over the recorded launches; the stream must have finished them.
    double total_ms() const {
#if SIGMA_CUDA
        double t = 0;
        for (size_t i = 0; i + 1 < used; i += 2) {
            float ms = 0;
            ck(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]), "event time");
            t += ms;
        }
        return t;
#else
        return acc;
#endif
    }
    void reset() {
        used = 0;
#if !SIGMA_CUDA
        acc = 0;
#endif
    }
    void destroy() {
#if SIGMA_CUDA
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
        ev.clear();
#endif
        used = 0;
    }
};

struct StageTimer {
#if SIGMA_CUDA
    cudaEvent_t a = nullptr, b = nullptr;
#else
    std::chrono::steady_clock::time_point t0;
#endif
    void init() {
#if SIGMA_CUDA
        cudaEventCreate(&a);
        cudaEventCreate(&b);
#endif
    }
    void destroy() {
#if SIGMA_CUDA
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
        a = b = nullptr;
#endif
    }
    void start(Runtime& rt) {
#if SIGMA_CUDA
        cudaEventRecord(a, rt.stream);
#else
        (void)rt;
        t0 = std::chrono::steady_clock::now();
#endif
    }
    double stop(Runtime& rt) {
        rt.syncs++;
#if SIGMA_CUDA
        cudaEventRecord(b, rt.stream);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        return ms;
#else
        (void)rt;
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
#endif
    }
};

}  // namespace sigma
