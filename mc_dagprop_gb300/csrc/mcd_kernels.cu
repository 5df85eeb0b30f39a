// mcd_kernels.cu -- sm_103a kernels of the Monte Carlo DAG-propagation path.
//
// k_propagate: one CTA owns a tile of 32 samples (one per lane) and walks the
// whole compiled DAG level by level; the warps of the CTA split each level's
// events and meet at a barrier between levels.  Realized times of events that
// later levels still read live in a shared-memory "window" (slot-major, one
// 256-byte row of 32 samples per live event), so predecessor reads never touch
// HBM; every output row is written once, coalesced (256 B per warp store).
//
// The propagation arithmetic is the reference's loop (_core.cpp:331-350): one
// IEEE FP64 add per edge, then std::min with the upper bound and `>=` against the
// running maximum.  FP64 compare/select runs at ~1.4 ops/clk/SM on this part
// (measured), so the comparisons run on 64-bit integer order keys instead, which
// order doubles exactly like the IEEE comparison operators (see order_key).
//
// Delays are drawn in the same kernel from Philox4x32-10 (Salmon, Moraes, Dror,
// Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11), keyed by the
// sample's 64-bit seed with (link, attempt) in the counter.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "mcd_internal.hpp"

namespace mcd {

// ---------------------------------------------------------------- Philox4x32-10
struct U4 {
    uint32_t x, y, z, w;
};

constexpr uint32_t kPhiloxM0 = 0xD2511F53u, kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u, kPhiloxW1 = 0xBB67AE85u;
constexpr uint32_t kStreamSalt = 0x6D636470u;  // counter word 3: separates this stream's use

__device__ __forceinline__ U4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                     uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = kPhiloxM0 * c0, hi0 = __umulhi(kPhiloxM0, c0);
        const uint32_t lo1 = kPhiloxM1 * c2, hi1 = __umulhi(kPhiloxM1, c2);
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += kPhiloxW0;
        k1 += kPhiloxW1;
    }
    return U4{c0, c1, c2, c3};
}

// Uniform in (0, 1]: (r + 1/2) / 2^32 rounded to float.
__device__ __forceinline__ float u01_open0(uint32_t r) {
    return fmaf(__uint2float_rn(r), 2.3283064365386963e-10f, 1.1641532182693481e-10f);
}

// ---------------------------------------------------------------- order keys
// Signed 64-bit key with key(a) < key(b) <=> a < b for non-NaN doubles, and
// key(-0) == key(+0) as the IEEE comparison has it.  NaN maps to INT64_MIN so
// that `ub < t` and `t >= latest` are both false for a NaN t, as in C++.
__device__ __forceinline__ long long order_key(long long b) {
    const long long mag = b & 0x7FFFFFFFFFFFFFFFll;
    const long long k = b < 0 ? -mag : mag;
    return mag > 0x7FF0000000000000ll ? (long long)0x8000000000000000ull : k;
}

// ---------------------------------------------------------------- samplers
// Each returns the link's duration (base + extra) for one sample.

// Exponential with mean lambda_, redrawn above max_scale (_core.cpp:83-89).  The
// redraw loop is replaced by the inverse CDF of the truncated law, which is the
// same distribution: X = -lambda_ * log(1 - c u), c = 1 - exp(-max_scale/lambda_).
__device__ __forceinline__ double draw_exponential(const DistParam &p, double base, uint32_t link, uint32_t k0,
                                                   uint32_t k1) {
    const U4 r = philox(link, 0u, 0u, kStreamSalt, k0, k1);
    const float w = u01_open0(r.x);                 // plays the role of 1 - u
    const float V = fmaf(p.f1, w, p.f2);            // 1 - c (1 - w), in (1-c, 1]
    float X = -p.f0 * logf(V);
    X = fminf(X, p.f3);
    return fma((double)X, base, base);
}

// Gamma(shape, scale) redrawn above max_scale (_core.cpp:98-104), by Marsaglia &
// Tsang (ACM TOMS 26(3), 2000) in FP32, normals from Box-Muller.  Shapes below 1
// draw Gamma(shape+1) times U^(1/shape).  Rejection loops are capped; a lane that
// hits the cap latches ERR_GAMMA_REJECTION and returns the truncation point.
__device__ __noinline__ double draw_gamma(const DistParam &p, double base, uint32_t link, uint32_t k0,
                                          uint32_t k1, int32_t *err) {
    const float d = p.f0, cc = p.f1;
    for (uint32_t attempt = 0; attempt < 4096u; ++attempt) {
        const U4 r = philox(link, attempt, 0u, kStreamSalt, k0, k1);
        const float rad = sqrtf(-2.0f * logf(u01_open0(r.x)));
        float sn, cs;
        sincospif(2.0f * (float)(r.y >> 8) * 5.9604644775390625e-08f, &sn, &cs);
        float X = -1.0f;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const float z = j == 0 ? rad * cs : rad * sn;
            const float t = fmaf(cc, z, 1.0f);
            if (X < 0.0f && t > 0.0f) {
                const float v = t * t * t;
                const float u = u01_open0(j == 0 ? r.z : r.w);
                const float z2 = z * z;
                if (u < 1.0f - 0.0331f * z2 * z2 || logf(u) < 0.5f * z2 + d * (1.0f - v + logf(v))) X = d * v;
            }
        }
        if (X < 0.0f) continue;
        if (p.boost) {
            const U4 r2 = philox(link, attempt, 1u, kStreamSalt, k0, k1);
            X *= exp2f(log2f(u01_open0(r2.x)) * p.f2);
        }
        X *= p.f3;
        if (X > p.f4) continue;
        return fma((double)X, base, base);
    }
    atomicOr(err, ERR_GAMMA_REJECTION);
    return fma((double)p.f4, base, base);
}

// Empirical tables (_core.cpp:110-141) by Walker/Vose alias sampling: one
// 32-bit word picks the bin, a second decides bin or alias.
__device__ __forceinline__ double draw_empirical(const DistParam &p, const AliasEntry *__restrict__ alias,
                                                 double base, bool relative, uint32_t link, uint32_t k0,
                                                 uint32_t k1) {
    const U4 r = philox(link, 0u, 0u, kStreamSalt, k0, k1);
    const uint32_t j = __umulhi(r.x, (uint32_t)p.tab_n);
    const AliasEntry *e = alias + p.tab_off + j;
    const double2 vv = __ldg(reinterpret_cast<const double2 *>(e));
    const uint32_t th = __ldg(&e->thresh);
    const double val = r.y < th ? vv.x : vv.y;
    return relative ? __dadd_rn(base, __dmul_rn(val, base)) : __dadd_rn(base, val);
}

__device__ __forceinline__ double link_duration(int32_t kd, double v, uint32_t link, uint32_t k0, uint32_t k1,
                                                const DistParam *__restrict__ dists,
                                                const AliasEntry *__restrict__ alias, int32_t *err) {
    const int kind = kd & KD_KIND_MASK;
    if (kind == K_FIXED) return v;
    const DistParam &p = dists[kd >> 8];
    switch (kind) {
        case K_EXP: return draw_exponential(p, v, link, k0, k1);
        case K_GAMMA: return draw_gamma(p, v, link, k0, k1, err);
        case K_EMP_ABS: return draw_empirical(p, alias, v, false, link, k0, k1);
        default: return draw_empirical(p, alias, v, true, link, k0, k1);
    }
}

// ---------------------------------------------------------------- statistics helpers
// x * 2^q truncated toward zero, from the bits of a finite double x with
// |x| * 2^q < 2^62 (the host picks q so that every realized time qualifies).
__device__ __forceinline__ long long to_ticks(long long b, int q) {
    const int e = (int)((b >> 52) & 0x7FF);
    const long long m = (b & 0xFFFFFFFFFFFFFll) | (e ? (1ll << 52) : 0ll);
    const int sh = (e ? e : 1) - 1075 + q;
    long long t;
    if (sh >= 0) t = m << sh;
    else t = sh > -63 ? (m >> -sh) : 0ll;
    return b < 0 ? -t : t;
}

// One event's realized values of the tile into the per-event accumulators:
// the tile's sum of (realized - earliest) with one 64-bit atomic, and the
// histogram with one atomic per distinct bin of the warp.
__device__ __forceinline__ void accumulate_stats(const KArgs &a, const EvRec &ev, long long lbits, bool active,
                                                 unsigned active_mask) {
    int bin;
    if (a.stats_fixed) {
        const long long te = to_ticks(ev.init_bits, a.tick_q);
        long long d = active ? to_ticks(lbits, a.tick_q) - te : 0ll;
        const unsigned long long du = (unsigned long long)(d > 0 ? d : 0ll);
        bin = (int)__umul64hi(du, a.bin_mul);
        bin = bin > kHistBins - 1 ? kHistBins - 1 : bin;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) d += __shfl_xor_sync(0xFFFFFFFFu, d, off);
        if ((threadIdx.x & 31) == 0 && d != 0) atomicAdd(&a.acc[ev.user], (unsigned long long)d);
    } else {
        const double dd = active ? __longlong_as_double(lbits) - __longlong_as_double(ev.init_bits) : 0.0;
        const double x = dd * a.hist_inv_w;
        bin = x >= (double)(kHistBins - 1) ? kHistBins - 1 : (x > 0.0 ? (int)x : 0);
        if (active && dd != 0.0) atomicAdd(reinterpret_cast<double *>(&a.acc[ev.user]), dd);
    }
    if (lbits == ev.init_bits) bin = kBinLo;
    else if (lbits == ev.ub_bits) bin = kBinHi;
    if (active) {
        const unsigned same = __match_any_sync(active_mask, bin);
        if ((threadIdx.x & 31) == __ffs(same) - 1)
            atomicAdd(&a.hist[(int64_t)ev.user * kHistStride + bin], (unsigned)__popc(same));
    }
}

// ---------------------------------------------------------------- propagation
// GIVEN: durations come from a.dur_in instead of the sampler.
// WIN_SMEM: predecessor values come from the shared-memory window; otherwise
// from the realized rows in global memory (the output, or scratch).
// STATS: instead of output rows, each event's realized values feed the
// per-event accumulators (mean, histogram); nothing per sample leaves the chip.
template <bool GIVEN, bool WIN_SMEM, bool STATS>
__global__ void __launch_bounds__(512) k_propagate(const KArgs a) {
    extern __shared__ double win[];  // [window_slots][kTile]
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int NW = a.n_warps;
    const int64_t s = (int64_t)blockIdx.x * kTile + lane;
    const bool active = s < a.n;
    const unsigned active_mask = __ballot_sync(0xFFFFFFFFu, active);
    uint64_t seed = 0;
    if (!GIVEN && active) seed = a.seeds ? (uint64_t)a.seeds[s] : (uint64_t)(a.seed0 + s);
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    double *rows = a.realized ? a.realized : a.scratch;  // global realized rows
    if (STATS && WIN_SMEM) rows = nullptr;

    for (int l = 0; l < a.n_levels; ++l) {
        const int ib = __ldg(&a.wk_off[l * NW + warp]);
        const int ie = __ldg(&a.wk_off[l * NW + warp + 1]);
        for (int i = ib; i < ie; ++i) {
            const EvRec ev = a.ev[i];
            long long lk = ev.init_key, lbits = ev.init_bits;
            int32_t cause = -1;
            for (int p = ev.pred_begin; p < ev.pred_end; ++p) {
                const PredRec pr = a.pred[p];
                double dur;
                if (GIVEN) {
                    dur = (active && pr.link >= 0) ? __ldg(&a.dur_in[(int64_t)pr.link * a.ld_in + s]) : 0.0;
                } else {
                    dur = link_duration(pr.kd, pr.v, (uint32_t)pr.link, k0, k1, a.dist, a.alias, a.err);
                    if (!STATS && (pr.kd & KD_WRITE) && a.durations && active)
                        a.durations[(int64_t)pr.link * a.ld + s] = dur;
                }
                double src;
                if (WIN_SMEM && pr.src_slot >= 0) {
                    src = win[pr.src_slot * kTile + lane];
                } else {
                    src = active ? rows[(int64_t)pr.src_user * a.ld + s] : 0.0;
                }
                const double t = src + dur;  // the one FP64 add of the edge (_core.cpp:341)
                long long tb = __double_as_longlong(t);
                long long tk = order_key(tb);
                if (ev.ub_key < tk) {  // t = std::min(t, ub)
                    tk = ev.ub_key;
                    tb = ev.ub_bits;
                }
                if (tk >= lk) {  // if (t >= latest) { latest = t; cause = src; }
                    lk = tk;
                    lbits = tb;
                    cause = pr.src_user;
                }
            }
            if (ev.ub_key < lk) lbits = ev.ub_bits;  // realized = std::min(latest, ub)
            const double real = __longlong_as_double(lbits);
            if (WIN_SMEM && ev.slot >= 0) win[ev.slot * kTile + lane] = real;
            if (STATS) accumulate_stats(a, ev, lbits, active, active_mask);
            if (active) {
                const int64_t o = (int64_t)ev.user * a.ld + s;
                if (rows) rows[o] = real;
                if (!STATS && a.cause) a.cause[o] = cause;
            }
        }
        __syncthreads();
    }
    // Aux pass: duration rows of fixed links and of links no precedence entry references.
    if (!STATS && !GIVEN && a.durations) {
        for (int i = warp; i < a.n_aux; i += NW) {
            const LinkRec lr = a.aux[i];
            const double dur = link_duration(lr.kd, lr.v, (uint32_t)lr.link, k0, k1, a.dist, a.alias, a.err);
            if (active) a.durations[(int64_t)lr.link * a.ld + s] = dur;
        }
    }
}

// Quantile at probability p of one event from its histogram: rank p*(n-1) as
// numpy's default ("linear") takes it, atoms exact, samples spread evenly
// inside a bin.
__device__ double hist_quantile(const uint32_t *h, int64_t n, double p, double lo, double hi, double w) {
    const double k = p * (double)(n - 1);
    const double c_lo = h[kBinLo], c_hi = h[kBinHi];
    if (k < c_lo) return lo;
    if (k >= (double)n - c_hi) return hi;
    double cum = c_lo;
    for (int b = 0; b < kHistBins; ++b) {
        const double c = h[b];
        if (c > 0.0 && k < cum + c) {
            const double v = lo + ((double)b + (k - cum + 0.5) / c) * w;
            return v < hi ? v : hi;
        }
        cum += c;
    }
    return hi;
}

__global__ void k_stats_finish(const FArgs f) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= f.E) return;
    const double lo = f.earliest[e], hi = f.ub[e];
    const double n = (double)f.n;
    if (f.mean) {
        double sum;
        if (f.stats_fixed) sum = ldexp((double)(long long)f.acc[e], -f.tick_q);
        else sum = __longlong_as_double((long long)f.acc[e]);
        f.mean[e] = lo + sum / n;
    }
    const uint32_t *h = f.hist + (int64_t)e * kHistStride;
    if (f.p50) f.p50[e] = hist_quantile(h, f.n, 0.50, lo, hi, f.bin_w);
    if (f.p90) f.p90[e] = hist_quantile(h, f.n, 0.90, lo, hi, f.bin_w);
    if (f.p99) f.p99[e] = hist_quantile(h, f.n, 0.99, lo, hi, f.bin_w);
    if (f.p_on_time) f.p_on_time[e] = (double)h[kBinLo] / n;
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
cudaError_t launch_propagate(const KArgs &a, bool given, bool win_smem, bool stats, cudaStream_t st) {
    if (a.n <= 0) return cudaSuccess;
    const dim3 grid((unsigned)((a.n + kTile - 1) / kTile));
    const dim3 block((unsigned)(a.n_warps * 32));
    const size_t smem = win_smem ? (size_t)a.window_slots * kTile * sizeof(double) : 0;
    void (*fn)(const KArgs);
    if (stats) {
        if (given) fn = win_smem ? k_propagate<true, true, true> : k_propagate<true, false, true>;
        else fn = win_smem ? k_propagate<false, true, true> : k_propagate<false, false, true>;
    } else {
        if (given) fn = win_smem ? k_propagate<true, true, false> : k_propagate<true, false, false>;
        else fn = win_smem ? k_propagate<false, true, false> : k_propagate<false, false, false>;
    }
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    fn<<<grid, block, smem, st>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- fixed scratch
// Device scratch for mcd_stats_device_noalloc: the per-event accumulators
// (8 bytes of sum + kHistStride 32-bit counters per event) of callers that
// cannot allocate device memory.  32 MiB, held by every GPU that loads this
// library until the process exits.  Host code must not use the symbol as an
// address; noalloc_scratch() below looks the device address up.
constexpr size_t kNoAllocScratchBytes = 32ull << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch on the current device, looked up once per
// device (cudaGetSymbolAddress, with that device current) and cached.
cudaError_t noalloc_scratch(void **ptr, size_t *bytes) {
    constexpr int kMaxDevices = 64;
    static void *cached[kMaxDevices] = {};
    static std::mutex mu;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (!cached[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        cached[dev] = p;
    }
    *ptr = cached[dev];
    *bytes = kNoAllocScratchBytes;
    return cudaSuccess;
}

cudaError_t launch_stats_finish(const FArgs &f, cudaStream_t st) {
    if (f.E <= 0) return cudaSuccess;
    k_stats_finish<<<(unsigned)((f.E + 255) / 256), 256, 0, st>>>(f);
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
