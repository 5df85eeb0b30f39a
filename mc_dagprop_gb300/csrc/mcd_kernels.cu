// mcd_kernels.cu -- launch dispatch, statistics finish, earliest-tick tables and
// layout kernels.
//
// The propagation kernel itself (k_propagate, mcd_device.cuh) is instantiated in
// mcd_prop_sample.cu, mcd_prop_sample_gt.cu and mcd_prop_given.cu.
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <utility>

#include "mcd_device.cuh"
#include "mcd_internal.hpp"

namespace mcd {

// One warp per event.  Lane j holds bins 8j .. 8j+7 and their running count from
// a warp scan (exact integers), so finding the bin of a quantile is a ballot, not a
// 256-step loop.
constexpr int kBinsPerLane = kHistBins / 32;
static_assert(kHistBins == 32 * kBinsPerLane && kBinsPerLane == 8, "two 16-byte loads per lane");

// Quantile at probability p from the lane's bins: rank p*(n-1) as numpy's default
// ("linear") takes it, atoms exact, samples spread evenly inside a bin.
// below: the count before this lane's first bin, on-time atom included.
__device__ double warp_quantile(const uint32_t (&c)[kBinsPerLane], uint32_t below, uint32_t c_lo, uint32_t c_hi,
                                int64_t n, double p, double lo, double hi, double w) {
    const int lane = threadIdx.x & 31;
    const double k = p * (double)(n - 1);
    if (k < (double)c_lo) return lo;
    if (k >= (double)n - (double)c_hi) return hi;
    // the first bin whose cumulative count (on-time atom included) exceeds k
    uint32_t cum = below;
    int found = -1;
    uint32_t cum_before = 0;
#pragma unroll
    for (int j = 0; j < kBinsPerLane; ++j) {
        if (found < 0 && (double)(cum + c[j]) > k) {
            found = j;
            cum_before = cum;
        }
        cum += c[j];
    }
    const unsigned hit = __ballot_sync(0xFFFFFFFFu, found >= 0);
    if (!hit) return hi;
    const int src = __ffs(hit) - 1;
    const int j = __shfl_sync(0xFFFFFFFFu, found, src);
    const uint32_t cb = __shfl_sync(0xFFFFFFFFu, cum_before, src);
    uint32_t cj = 0;
#pragma unroll
    for (int t = 0; t < kBinsPerLane; ++t)
        if (t == j) cj = c[t];
    cj = __shfl_sync(0xFFFFFFFFu, cj, src);
    const int bin = src * kBinsPerLane + j;
    const double v = lo + ((double)bin + (k - (double)cb + 0.5) / (double)cj) * w;
    (void)lane;
    return v < hi ? v : hi;
}

__device__ __forceinline__ void finish_event_warp(const FArgs &f, int e) {
    const int lane = threadIdx.x & 31;
    const uint32_t *h = f.hist + (int64_t)e * kHistStride;
    const uint4 a = reinterpret_cast<const uint4 *>(h)[2 * lane];
    const uint4 b = reinterpret_cast<const uint4 *>(h)[2 * lane + 1];
    const uint32_t c[kBinsPerLane] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    const uint32_t c_lo = h[kBinLo], c_hi = h[kBinHi];
    uint32_t mine = 0;
#pragma unroll
    for (int j = 0; j < kBinsPerLane; ++j) mine += c[j];
    uint32_t incl = mine;  // inclusive scan over lanes (the counts sum to at most n <= 2^31)
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t o = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        if (lane >= d) incl += o;
    }
    const uint32_t below = c_lo + incl - mine;
    const double lo = f.earliest[e], hi = f.ub[e];
    const double p50 = warp_quantile(c, below, c_lo, c_hi, f.n, 0.50, lo, hi, f.bin_w);
    const double p90 = warp_quantile(c, below, c_lo, c_hi, f.n, 0.90, lo, hi, f.bin_w);
    const double p99 = warp_quantile(c, below, c_lo, c_hi, f.n, 0.99, lo, hi, f.bin_w);
    if (lane != 0) return;
    const double n = (double)f.n;
    if (f.mean) {
        double sum;
        if (f.stats_fixed) sum = ldexp((double)(long long)f.acc[e], -f.tick_q);
        else sum = __longlong_as_double((long long)f.acc[e]);
        f.mean[e] = lo + sum / n;
    }
    if (f.p50) f.p50[e] = p50;
    if (f.p90) f.p90[e] = p90;
    if (f.p99) f.p99[e] = p99;
    if (f.p_on_time) f.p_on_time[e] = (double)c_lo / n;
}

__global__ void __launch_bounds__(256) k_stats_finish(const FArgs f) {
    const int e = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (e < f.E) finish_event_warp(f, e);
}

// The finish of every DAG of a batch in one launch: blockIdx.y selects the DAG.
__global__ void __launch_bounds__(256) k_batch_finish(const FArgs *__restrict__ fs, int32_t n_dags) {
    const int e = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    for (int32_t d = (int32_t)blockIdx.y; d < n_dags; d += (int32_t)gridDim.y) {
        const FArgs &f = fs[d];
        if (e < f.E) finish_event_warp(f, e);
    }
}

// Self-test of the bounded stage wait: an mbarrier whose phase expects 16 bytes
// that no copy delivers, waited on by every thread with a short poll limit.  The
// wait must give up, latch ERR_STAGE_TIMEOUT and let the kernel return.
__global__ void k_wait_selftest(int32_t *err, uint32_t limit) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_expect_tx(&bar, 16);  // the arrival; the 16 bytes never come
    __syncthreads();
    if (!stage_wait(&bar, 0u, err, limit) && threadIdx.x == 0) atomicOr(err, 1 << 30);  // "returned"
}

// Every event's earliest in ticks of 2^-q seconds (KArgs::te) for one run.
__global__ void k_event_ticks(const double *__restrict__ earliest, int32_t E, int32_t q, long long *__restrict__ te) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x)
        te[e] = ticks_of(__double_as_longlong(earliest[e]), q);
}

// ---------------------------------------------------------------- layout change
// Sample-minor [rows][ld_in] -> sample-major [cols][ld_out] (cols = samples).
template <typename T>
__global__ void k_transpose(const T *__restrict__ in, int64_t ld_in, T *__restrict__ out, int64_t ld_out,
                            int64_t rows, int64_t cols) {
    __shared__ T tile[32][33];
    const int64_t r0 = (int64_t)blockIdx.x * 32, c0 = (int64_t)blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int64_t r = r0 + k, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[k][threadIdx.x] = in[r * ld_in + c];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int64_t c = c0 + k, r = r0 + threadIdx.x;
        if (c < cols && r < rows) out[c * ld_out + r] = tile[threadIdx.x][k];
    }
}

// ---------------------------------------------------------------- launchers
cudaError_t raise_smem_limit(const void *fn, size_t smem) {
    if (smem <= 48 * 1024) return cudaSuccess;
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, size_t> limit;  // (kernel, device) -> bytes set
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    size_t &cur = limit[{fn, dev}];
    if (smem <= cur) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) cur = smem;
    return e;
}

cudaError_t launch_prop_sample(const KArgs &a, bool win_smem, bool stats, bool positive, dim3 grid, dim3 block,
                               size_t smem, cudaStream_t st);
cudaError_t launch_prop_given(const KArgs &a, bool win_smem, bool stats, dim3 grid, dim3 block, size_t smem,
                              cudaStream_t st);

// One launch of the propagation kernel over a.n samples: one CTA per tile of 32.
// The shared-memory layout is fixed by the host compiler (KArgs::smem_*).
cudaError_t launch_propagate(const KArgs &a, bool given, bool win_smem, bool stats, cudaStream_t st) {
    if (a.n <= 0) return cudaSuccess;
    const dim3 grid((unsigned)((a.n + kTile - 1) / kTile));
    const dim3 block((unsigned)(a.n_warps * 32));
    const size_t smem = (size_t)a.smem_total;
    if (given) return launch_prop_given(a, win_smem, stats, grid, block, smem, st);
    return launch_prop_sample(a, win_smem, stats, a.positive != 0, grid, block, smem, st);
}

// ---------------------------------------------------------------- fixed scratch
// Device scratch for mcd_stats_device_noalloc: the per-event accumulators
// (8 bytes of sum, kHistStride 32-bit counters and 8 bytes of earliest ticks per
// event) of callers that cannot allocate device memory.  34 MiB, held by every
// GPU that loads this library until the process exits.  Host code must not use the symbol as an
// address; noalloc_scratch() below looks the device address up.
constexpr size_t kNoAllocScratchBytes = 34ull << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Unique id of the calling thread's current CUDA context (the driver's
// cuCtxGetCurrent and cuCtxGetId, found through the runtime so the library needs
// no link to the driver library; ids are never reused within a process), or 0
// when no context is current yet.
static unsigned long long current_context_id() {
    using CtxGetCurrent = int (*)(void **);
    using CtxGetId = int (*)(void *, unsigned long long *);
    static const std::pair<CtxGetCurrent, CtxGetId> fns = [] {
        void *a = nullptr, *b = nullptr;
        cudaDriverEntryPointQueryResult qa{}, qb{};
        const bool ok = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) ==
                            cudaSuccess &&
                        qa == cudaDriverEntryPointSuccess &&
                        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) ==
                            cudaSuccess &&
                        qb == cudaDriverEntryPointSuccess;
        return ok ? std::make_pair(reinterpret_cast<CtxGetCurrent>(a), reinterpret_cast<CtxGetId>(b))
                  : std::make_pair((CtxGetCurrent) nullptr, (CtxGetId) nullptr);
    }();
    void *ctx = nullptr;
    unsigned long long id = 0;
    if (!fns.first || fns.first(&ctx) != 0 || !ctx || fns.second(ctx, &id) != 0) return 0;
    return id;
}

// Device address of g_noalloc_scratch in the current device's context, looked up
// (cudaGetSymbolAddress, with that device current) once per device and context and
// cached under both: a device reset or another context made current on the same
// device loads the module anew, at another address, so a cache keyed by the device
// alone would hand out a stale pointer.  Without a context id (an older driver),
// every call looks the address up again.
cudaError_t noalloc_scratch(void **ptr, size_t *bytes) {
    static std::map<std::pair<int, unsigned long long>, void *> cached;
    static std::mutex mu;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    unsigned long long ctx = current_context_id();
    auto it = ctx ? cached.find({dev, ctx}) : cached.end();
    if (it == cached.end()) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // makes the device's primary context current if none was
        if (e != cudaSuccess) return e;
        ctx = current_context_id();
        if (ctx) cached[{dev, ctx}] = p;
        *ptr = p;
    } else {
        *ptr = it->second;
    }
    *bytes = kNoAllocScratchBytes;
    return cudaSuccess;
}

cudaError_t launch_batch_finish(const FArgs *fs, int32_t n_dags, int32_t max_events, cudaStream_t st) {
    if (n_dags <= 0 || max_events <= 0) return cudaSuccess;
    const unsigned gy = (unsigned)(n_dags < 65535 ? n_dags : 65535);  // grid y limit; the kernel strides
    k_batch_finish<<<dim3((unsigned)((max_events + 7) / 8), gy), 256, 0, st>>>(fs, n_dags);  // a warp per event
    return cudaGetLastError();
}

cudaError_t launch_wait_selftest(int32_t *err, uint32_t limit, cudaStream_t st) {
    k_wait_selftest<<<1, 64, 0, st>>>(err, limit);
    return cudaGetLastError();
}

cudaError_t launch_event_ticks(const double *earliest, int32_t E, int32_t q, long long *te, cudaStream_t st) {
    if (E <= 0) return cudaSuccess;
    const int blocks = (E + 255) / 256;
    k_event_ticks<<<blocks < 4096 ? blocks : 4096, 256, 0, st>>>(earliest, E, q, te);
    return cudaGetLastError();
}

cudaError_t launch_stats_finish(const FArgs &f, cudaStream_t st) {
    if (f.E <= 0) return cudaSuccess;
    k_stats_finish<<<(unsigned)((f.E + 7) / 8), 256, 0, st>>>(f);  // a warp per event
    return cudaGetLastError();
}

template <typename T>
static cudaError_t launch_transpose_t(const T *in, int64_t ld_in, T *out, int64_t ld_out, int64_t rows,
                                      int64_t cols, cudaStream_t st) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    const dim3 grid((unsigned)((rows + 31) / 32), (unsigned)((cols + 31) / 32));
    k_transpose<T><<<grid, dim3(32, 8), 0, st>>>(in, ld_in, out, ld_out, rows, cols);
    return cudaGetLastError();
}

cudaError_t launch_transpose_f64(const double *in, int64_t ld_in, double *out, int64_t ld_out, int64_t rows,
                                 int64_t cols, cudaStream_t st) {
    return launch_transpose_t(in, ld_in, out, ld_out, rows, cols, st);
}

cudaError_t launch_transpose_i32(const int32_t *in, int64_t ld_in, int32_t *out, int64_t ld_out, int64_t rows,
                                 int64_t cols, cudaStream_t st) {
    return launch_transpose_t(in, ld_in, out, ld_out, rows, cols, st);
}

}  // namespace mcd
