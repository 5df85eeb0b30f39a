// mcd_analytic.cu -- analytic PMF propagation on the GPU (the reference's
// src/mc_dagprop/analytic/, pure Python there), behind the mcd_analytic_* C ABI.
//
// A PMF is (first value, probabilities) on the context's step grid.  Events are
// processed level by level (longest path from a source), two launches a level:
// k_an_conv computes every convolution of the level, its outputs split into
// one-warp chunks of 8 dealt out costliest first across the warps (the FP64
// multiply-adds are the bulk of the work);
// k_an_fold then takes one event per CTA:
//   convolution along each incoming activity       _pmf.py:107-125
//   maximum over the predecessors, pairwise in      _pmf.py:127-148
//   precedence order, by cumulative products
//   mass correction after each operation            _pmf.py:82-105
//   clipping to the event's bounds under the        _propagator.py:150-265
//   underflow/overflow rules
// The reference accumulates convolutions and cumulative sums in np.longdouble;
// here they run in FP64 (fused multiply-adds, blocked scans), so results agree
// with the reference to rounding, not bit for bit.
//
// Working arrays (five of the event's grid bound) live in dynamic shared memory
// when they fit, else in a global scratch slice per event of the level.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <limits>
#include <string>
#include <vector>

#include "mcd_handle.hpp"

namespace mcd {
namespace {

constexpr int kAnThreads = 128;
// Outputs (and threads) per convolution chunk and CTA, and convolution CTAs per SM.
constexpr int kConvLanes = 4;                 // lanes per output
constexpr int kConvOuts = 32 / kConvLanes;    // outputs per chunk (one warp)
constexpr int kConvWarpsPerSm = 16;
constexpr int64_t kAnSmemBins = 4096;  // 5 arrays x 4096 doubles = 160 KB of shared memory

// Kernel-reported errors (the reference raises ValueError in each case).
enum : int32_t {
    AN_ERR_UNDER_TRUNC = 1,   // underflow mass but no lower-bound bin (_propagator.py:192-193)
    AN_ERR_OVER_TRUNC = 2,    // overflow mass but no upper-bound bin (:203-205)
    AN_ERR_EMPTY = 4,         // nothing left after clipping (:229-232)
    AN_ERR_BOUNDS = 8,        // lower bound above upper bound (:163-164)
    AN_ERR_GRID = 16,         // operands that do not fit their common grid (misaligned values)
    AN_ERR_CAPACITY = 32,     // internal: a support larger than planned
};

struct AnEv {
    int32_t pred_begin, pred_end;  // predecessor entries, precedence order
    int64_t lower, upper;          // event bounds (_propagator.py:150-156)
    int64_t pool_off;              // output probabilities
    int32_t cap;                   // output capacity (bins)
    int32_t gmax;                  // grid bound of the event's intermediate PMFs
    int64_t scratch_off;           // global scratch slice (5 x gmax doubles), -1: shared memory
};

struct AnOut {
    double first;
    double under, over;
    double mass;  // total probability of the event's PMF
    int32_t len;
    int32_t pad;
};

struct AnArgs {
    const AnEv *ev;
    const int32_t *pred_src;
    const int32_t *pred_pmf;
    const int64_t *pmf_off;
    const double *pmf_first;
    const double *pmf_probs;
    const double *pmf_mass;
    AnOut *out;
    double *pool;
    double *scratch;
    double *convbuf;          // the level's convolutions, conv_off[p] per predecessor entry
    const int64_t *conv_off;
    int32_t *err;
    int32_t step;
    int32_t urule, orule;
};

__device__ __forceinline__ bool close12(double a, double b) {  // np.isclose(a, b, rtol=1e-12, atol=1e-15)
    return fabs(a - b) <= 1e-15 + 1e-12 * fabs(b);
}
__device__ __forceinline__ bool close_default(double a, double b) {  // np.isclose defaults
    return fabs(a - b) <= 1e-8 + 1e-5 * fabs(b);
}
__device__ __forceinline__ double expected_mass(double m1, double m2) {  // _pmf.py:96-105
    return (close12(m1, 1.0) && close12(m2, 1.0)) ? 1.0 : m1 * m2;
}

constexpr int kAnWarps = kAnThreads / 32;

// Block-wide sums with one barrier each.  The FP64 pipe (2 lanes per clock per
// SM) and the chain of dependent phases bound this kernel, so a sum is a warp
// shuffle tree, one barrier, and every thread adding the few warp totals itself.
// Warps post their totals to one of two slot sets, alternately: a call never
// overwrites totals a slower thread may still be reading from the call before it
// (the barrier of the call in between separates them).  Every thread of the
// block must make the same sequence of calls.
struct BlockRed {
    double *slots;  // [2][2][kAnWarps]
    int parity;
    __device__ double2 sum2(double x, double y) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            x += __shfl_xor_sync(0xFFFFFFFFu, x, o);
            y += __shfl_xor_sync(0xFFFFFFFFu, y, o);
        }
        double *sl = slots + parity * 2 * kAnWarps;
        parity ^= 1;
        const int w = threadIdx.x >> 5;
        if ((threadIdx.x & 31) == 0) {
            sl[w] = x;
            sl[kAnWarps + w] = y;
        }
        __syncthreads();
        double tx = 0.0, ty = 0.0;
#pragma unroll
        for (int i = 0; i < kAnWarps; ++i) {
            tx += sl[i];
            ty += sl[kAnWarps + i];
        }
        return make_double2(tx, ty);
    }
    __device__ double sum(double x) { return sum2(x, 0.0).x; }
};

// The first index >= lo this thread owns under the strided mapping (index i
// belongs to thread i mod kAnThreads).  Every elementwise phase uses that
// mapping, so a phase that only touches its own elements needs no barrier.
__device__ __forceinline__ int64_t own_from(int64_t lo) {
    const int64_t r = ((int64_t)threadIdx.x - lo) % kAnThreads;
    return lo + (r < 0 ? r + kAnThreads : r);
}

// Inclusive prefix sums ox = cumsum(x[0, n)), oy = cumsum(y[0, n)), each thread
// scanning one contiguous chunk of both; two barriers.  x and y must be complete
// (a barrier after their last writes); the closing barrier lets callers read any
// element of ox and oy.
__device__ void block_scan2(const double *x, const double *y, double *ox, double *oy, int64_t n, BlockRed &r) {
    const int64_t chunk = (n + kAnThreads - 1) / kAnThreads;
    const int64_t a0 = (int64_t)threadIdx.x * chunk, a = a0 < n ? a0 : n, b = a + chunk < n ? a + chunk : n;
    double lx = 0.0, ly = 0.0;
    for (int64_t i = a; i < b; ++i) {
        lx += x[i];
        ly += y[i];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double ix = lx, iy = ly;  // inclusive within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double ux = __shfl_up_sync(0xFFFFFFFFu, ix, o), uy = __shfl_up_sync(0xFFFFFFFFu, iy, o);
        if (lane >= o) {
            ix += ux;
            iy += uy;
        }
    }
    double ex = __shfl_up_sync(0xFFFFFFFFu, ix, 1), ey = __shfl_up_sync(0xFFFFFFFFu, iy, 1);
    if (lane == 0) ex = ey = 0.0;
    double *sl = r.slots + r.parity * 2 * kAnWarps;
    r.parity ^= 1;
    if (lane == 31) {
        sl[w] = ix;
        sl[kAnWarps + w] = iy;
    }
    __syncthreads();
    double bx = 0.0, by = 0.0;
    for (int i = 0; i < w; ++i) {
        bx += sl[i];
        by += sl[kAnWarps + i];
    }
    double rx = bx + ex, ry = by + ey;
    for (int64_t i = a; i < b; ++i) {
        rx += x[i];
        ox[i] = rx;
        ry += y[i];
        oy[i] = ry;
    }
    __syncthreads();
}

__device__ __forceinline__ int64_t round_half_even(double x) { return (int64_t)rint(x); }

// Length of the convolution of a pred PMF of n entries with an activity PMF of m.
__device__ __forceinline__ int64_t conv_len(int64_t n, int64_t m) { return n == 1 ? m : (m == 1 ? n : n + m - 1); }

// One chunk of kConvOuts outputs of one convolution (predecessor entry c.x, chunk
// index c.y), computed by one warp: kConvLanes lanes per output split its terms
// and add their partial sums with shuffles.  A warp's FP64 multiply-adds issue at
// the SM sub-partition's FP64 rate (a warp instruction per 64 clocks), so chunks
// are kept small: the last chunks of a level then finish soon after the others.
// Operands are read through the L1 cache (every chunk of a convolution reads the
// same activity PMF and overlapping windows of the predecessor's).
__device__ void conv_chunk(const AnArgs &A, int2 c) {
    const int32_t s = A.pred_src[c.x], k = A.pred_pmf[c.x];
    const int64_t n = A.out[s].len, m = A.pmf_off[k + 1] - A.pmf_off[k];
    const int lane = threadIdx.x & 31, sub = lane % kConvLanes;
    const int64_t len = conv_len(n, m), j = (int64_t)c.y * kConvOuts + lane / kConvLanes;
    const double *p = A.pool + A.ev[s].pool_off, *q = A.pmf_probs + A.pmf_off[k];
    double *out = A.convbuf + A.conv_off[c.x];
    if (n == 1 || m == 1) {  // the reference's scaled copies (_pmf.py:111-116)
        if (j < len && sub == 0) out[j] = n == 1 ? __ldg(q + j) * __ldg(p) : __ldg(p + j) * __ldg(q);
        return;
    }
    double acc = 0.0;
    if (j < len) {
        const int64_t i0 = j - (m - 1) > 0 ? j - (m - 1) : 0, i1 = j < n - 1 ? j : n - 1;
        for (int64_t i = i0 + sub; i <= i1; i += kConvLanes) acc = fma(__ldg(p + i), __ldg(q + (j - i)), acc);
    }
#pragma unroll
    for (int o = 1; o < kConvLanes; o <<= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
    if (j < len && sub == 0) out[j] = acc;
}

// Every convolution of a level.  A level's chunks differ in cost (a chunk at a
// convolution's edge has few terms); the host lists them costliest first and each
// warp takes every gridDim.x-th, so the warps' loads come out nearly equal without
// a shared counter (one counter's atomics serialise at its L2 slice).
__global__ void __launch_bounds__(32) k_an_conv(const AnArgs A, const int2 *__restrict__ chunks, int32_t n_chunks) {
    for (int32_t ci = blockIdx.x; ci < n_chunks; ci += gridDim.x) conv_chunk(A, chunks[ci]);
}

__global__ void __launch_bounds__(kAnThreads) k_an_fold(const AnArgs A, const int32_t *__restrict__ level_ev) {
    extern __shared__ __align__(16) double sm[];
    __shared__ double slots[4 * kAnWarps];
    BlockRed red{slots, 0};
    const int32_t e = level_ev[blockIdx.x];
    const AnEv ev = A.ev[e];
    const int64_t G = ev.gmax;
    double *X = ev.scratch_off >= 0 ? A.scratch + ev.scratch_off : sm;  // current result
    double *Rp = X + G, *Cp = X + 2 * G, *cR = X + 3 * G, *cC = X + 4 * G;
    const double step = (double)A.step;
#define fail(code)                                     \
    do {                                               \
        if (threadIdx.x == 0) atomicOr(A.err, (code)); \
    } while (0)

    // ---- predecessor 0: R = pred0 (*) activity0, rescaled to its expected mass
    double fX;
    int64_t nX;
    double mR;
    {
        const int32_t s = A.pred_src[ev.pred_begin], k = A.pred_pmf[ev.pred_begin];
        const AnOut ps = A.out[s];
        const int64_t m = A.pmf_off[k + 1] - A.pmf_off[k];
        nX = conv_len(ps.len, m);
        fX = ps.first + A.pmf_first[k];
        if (nX > G) {
            fail(AN_ERR_CAPACITY);
            return;
        }
        const double *conv = A.convbuf + A.conv_off[ev.pred_begin];
        double part = 0.0;
        for (int64_t j = threadIdx.x; j < nX; j += kAnThreads) {
            const double v = conv[j];
            X[j] = v;
            part += v;
        }
        const double tot = red.sum(part);
        const double expct = expected_mass(ps.mass, A.pmf_mass[k]);
        mR = tot;
        if (tot > 0.0 && !close12(tot, expct)) {
            const double f = expct / tot;
            part = 0.0;
            for (int64_t j = threadIdx.x; j < nX; j += kAnThreads) part += (X[j] *= f);
            mR = red.sum(part);
        }
    }
    // ---- later predecessors: R = max(R, pred_k (*) activity_k)
    for (int32_t pi = ev.pred_begin + 1; pi < ev.pred_end; ++pi) {
        const int32_t s = A.pred_src[pi], k = A.pred_pmf[pi];
        const AnOut ps = A.out[s];
        const int64_t m = A.pmf_off[k + 1] - A.pmf_off[k];
        const int64_t nC = conv_len(ps.len, m);
        const double fC = ps.first + A.pmf_first[k];
        // common grid: np.arange(min start, max end + step, step) (_pmf.py:129-134)
        const double lo = fmin(fX, fC);
        const double hi = fmax(fX + step * (double)(nX - 1), fC + step * (double)(nC - 1));
        const int64_t n = (int64_t)ceil((hi + step - lo) / step);
        const int64_t oR = round_half_even((fX - lo) / step), oC = round_half_even((fC - lo) / step);
        if (n > G || oR + nX > n || oC + nC > n) {
            fail(n > G ? AN_ERR_CAPACITY : AN_ERR_GRID);
            return;
        }
        // both operands on the common grid; the convolution rescaled to its expected mass
        const double *conv = A.convbuf + A.conv_off[pi];
        double part = 0.0;
        for (int64_t i = threadIdx.x; i < n; i += kAnThreads) {
            Rp[i] = (i >= oR && i < oR + nX) ? X[i - oR] : 0.0;
            const double c = (i >= oC && i < oC + nC) ? conv[i - oC] : 0.0;
            Cp[i] = c;
            part += c;
        }
        const double totC = red.sum(part);
        const double expctC = expected_mass(ps.mass, A.pmf_mass[k]);
        double mC = totC;
        if (totC > 0.0 && !close12(totC, expctC)) {
            const double f = expctC / totC;
            part = 0.0;
            for (int64_t i = own_from(oC); i < oC + nC; i += kAnThreads) part += (Cp[i] *= f);
            mC = red.sum(part);
        }
        // max(R, C) by cumulative sums: P(max = x) = r(x) C(x) + c(x) R(x - 1); the
        // last sum's barrier completed Rp and Cp
        block_scan2(Rp, Cp, cR, cC, n, red);
        part = 0.0;
        for (int64_t i = threadIdx.x; i < n; i += kAnThreads) {
            const double v = fma(Rp[i], cC[i], Cp[i] * (i > 0 ? cR[i - 1] : 0.0));
            X[i] = v;
            part += v;
        }
        fX = lo;
        nX = n;
        const double tot = red.sum(part);
        const double expct = expected_mass(mR, mC);
        mR = tot;
        if (tot > 0.0 && !close12(tot, expct)) {
            const double f = expct / tot;
            part = 0.0;
            for (int64_t i = threadIdx.x; i < nX; i += kAnThreads) part += (X[i] *= f);
            mR = red.sum(part);
        }
    }

    // ---- clipping to [lower, upper] under the flow rules (_propagator.py:158-265);
    // from here on every thread touches only its own elements of X
    const double lower = (double)ev.lower, upper = (double)ev.upper;
    if (ev.lower > ev.upper) {
        fail(AN_ERR_BOUNDS);
        return;
    }
    int64_t ka = (int64_t)ceil((lower - fX) / step), kb = (int64_t)floor((upper - fX) / step) + 1;
    ka = ka < 0 ? 0 : (ka > nX ? nX : ka);
    kb = kb > nX ? nX : (kb < ka ? ka : kb);
    double u, o;
    {
        double pu = 0.0, po = 0.0;
        for (int64_t i = threadIdx.x; i < nX; i += kAnThreads) {
            if (i < ka) pu += X[i];
            else if (i >= kb) po += X[i];
        }
        const double2 uo = red.sum2(pu, po);
        u = uo.x;
        o = uo.y;
    }
    const bool own_ka = ka < nX && own_from(ka) == ka, own_last = kb > 0 && own_from(kb - 1) == kb - 1;
    // kept values: X[ka, kb) at fX + i * step, or one value `single_v` with mass `single_p`
    bool single = false;
    double single_v = 0.0, single_p = 0.0;
    int64_t nk = kb - ka;
    double red_u = 0.0, red_o = 0.0;
    if (A.urule == MCD_RULE_TRUNCATE && u > 0.0) {
        if (nk > 0 && close_default(fX + step * (double)ka, lower)) {
            if (own_ka) X[ka] += u;
        } else if (nk == 0) {
            single = true;
            single_v = lower;
            single_p = u;
        } else {
            fail(AN_ERR_UNDER_TRUNC);
            return;
        }
        u = 0.0;
    } else if (A.urule == MCD_RULE_REDISTRIBUTE && u > 0.0) {
        red_u = u;
        u = 0.0;
    }
    if (A.orule == MCD_RULE_TRUNCATE && o > 0.0) {
        const bool any = single || nk > 0;
        const double last = single ? single_v : fX + step * (double)(kb - 1);
        if (any && close_default(last, upper)) {
            if (single) single_p += o;
            else if (own_last) X[kb - 1] += o;
        } else if (!any) {
            single = true;
            single_v = upper;
            single_p = o;
        } else {
            fail(AN_ERR_OVER_TRUNC);
            return;
        }
        o = 0.0;
    } else if (A.orule == MCD_RULE_REDISTRIBUTE && o > 0.0) {
        red_o = o;
        o = 0.0;
    }
    auto kept_sum = [&]() {
        double part = 0.0;
        for (int64_t i = own_from(ka); i < kb; i += kAnThreads) part += X[i];
        return red.sum(part);
    };
    const double redist = red_u + red_o;
    if (redist > 0.0) {
        const double inside = single ? single_p : kept_sum();
        if (inside == 0.0) {
            single = true;
            single_v = lower;
            single_p = redist;
        } else if (single) {
            single_p = single_p + redist * (single_p / inside);
        } else {
            for (int64_t i = own_from(ka); i < kb; i += kAnThreads) X[i] = X[i] + redist * (X[i] / inside);
        }
    }
    if (!single && nk == 0) {
        fail(AN_ERR_EMPTY);
        return;
    }
    const double target = fmax(0.0, 1.0 - (u + o));
    double total;
    {
        const double s_in = single ? single_p : kept_sum();
        if (s_in > 0.0) {
            if (single) {
                single_p = (single_p / s_in) * target;
                total = single_p;
            } else {
                double part = 0.0;
                for (int64_t i = own_from(ka); i < kb; i += kAnThreads) part += (X[i] = (X[i] / s_in) * target);
                total = red.sum(part);
            }
        } else {
            if (target > 0.0) {
                single = true;
                single_v = lower;
                single_p = target;
            }
            total = single ? single_p : s_in;
        }
    }
    double mass = total;
    {
        const double all = total + u + o;
        if (!close12(all, 1.0)) {
            const double corr = all > 0.0 ? 1.0 / all : 1.0;
            if (single) {
                single_p *= corr;
                mass = single_p;
            } else {
                double part = 0.0;
                for (int64_t i = own_from(ka); i < kb; i += kAnThreads) part += (X[i] *= corr);
                mass = red.sum(part);
            }
        }
    }
    // ---- output
    const int64_t len = single ? 1 : nk;
    if (len > ev.cap) {
        fail(AN_ERR_CAPACITY);
        return;
    }
    double *dst = A.pool + ev.pool_off;
    if (single) {
        if (threadIdx.x == 0) dst[0] = single_p;
    } else {
        for (int64_t i = own_from(ka); i < kb; i += kAnThreads) dst[i - ka] = X[i];
    }
    if (threadIdx.x == 0) {
        AnOut r;
        r.first = single ? single_v : fX + step * (double)ka;
        r.under = u;
        r.over = o;
        r.mass = mass;
        r.len = (int32_t)len;
        r.pad = 0;
        A.out[e] = r;
    }
#undef fail
}

}  // namespace
}  // namespace mcd

using namespace mcd;

struct mcd_analytic {
    int device = 0;
    cudaStream_t stream = nullptr;
    int32_t E = 0;
    AnArgs args{};
    std::vector<int32_t> level_off;    // non-origin levels: events level_ev[level_off[l] .. level_off[l+1])
    std::vector<int32_t> level_smem;   // dynamic shared memory per fold launch (bytes)
    std::vector<int32_t> chunk_off;    // convolution chunks of each level: chunks[chunk_off[l] .. chunk_off[l+1])
    int32_t *d_level_ev = nullptr;
    int2 *d_chunks = nullptr;
    cudaGraphExec_t graph = nullptr;   // every level's two launches
    char *dmem = nullptr;
    int64_t bins = 0;                  // output pool size
    bool ran = false;
};

namespace {

int64_t py_round(double x) { return (int64_t)std::nearbyint(x); }  // half to even, as Python and numpy round

}  // namespace

extern "C" {

int mcd_analytic_create(const mcd_analytic_desc *d, mcd_analytic **out) {
    mcd_analytic *an = nullptr;
    const int rc = guarded([&] {
        if (!d || !out) throw McdError(MCD_ERR_INVALID, "null argument");
        *out = nullptr;
        const int32_t E = d->n_events, K = d->n_pmfs, T = d->n_targets;
        if (E < 0 || K < 0 || T < 0) throw McdError(MCD_ERR_INVALID, "negative array length");
        if (d->step <= 0) throw McdError(MCD_ERR_INVALID, "step_size must be positive");
        if (!(d->max_delay >= 0.0) && !std::isnan(d->max_delay))
            throw McdError(MCD_ERR_INVALID, "max_delay must be non-negative when provided");
        if (d->underflow_rule < 1 || d->underflow_rule > 3 || d->overflow_rule < 1 || d->overflow_rule > 3)
            throw McdError(MCD_ERR_INVALID, "unknown underflow/overflow rule");
        const int64_t P = T > 0 ? d->pred_off[T] : 0;
        if (d->pmf_off[0] != 0) throw McdError(MCD_ERR_INVALID, "pmf_off must start at 0");
        for (int32_t k = 0; k < K; ++k)
            if (d->pmf_off[k + 1] <= d->pmf_off[k]) throw McdError(MCD_ERR_INVALID, "PMF values cannot be empty");
        // predecessors by target, precedence order
        std::vector<int64_t> tstart((size_t)E, -1), tlen((size_t)E, 0);
        for (int32_t t = 0; t < T; ++t) {
            const int32_t tg = d->target[t];
            if (tg < 0 || tg >= E) throw McdError(MCD_ERR_INVALID, "target index out of range");
            if (tstart[tg] != -1) throw McdError(MCD_ERR_INVALID, "precedence_list names a target twice");
            tstart[tg] = d->pred_off[t];
            tlen[tg] = d->pred_off[t + 1] - d->pred_off[t];
            if (tlen[tg] < 0) throw McdError(MCD_ERR_INVALID, "pred_off must be non-decreasing");
            for (int64_t p = d->pred_off[t]; p < d->pred_off[t + 1]; ++p) {
                if (d->pred_src[p] < 0 || d->pred_src[p] >= E)
                    throw McdError(MCD_ERR_INVALID, "predecessor index out of range");
                if (d->pred_pmf[p] < 0 || d->pred_pmf[p] >= K)
                    throw McdError(MCD_ERR_INVALID, "missing activity for a predecessor entry");
            }
        }
        // Kahn order with levels (longest path from a source)
        std::vector<std::vector<int32_t>> adj((size_t)E);
        std::vector<int64_t> indeg(tlen);
        for (int32_t e = 0; e < E; ++e)
            for (int64_t k = 0; k < tlen[e]; ++k) adj[d->pred_src[tstart[e] + k]].push_back(e);
        std::vector<int32_t> level((size_t)E, 0), order;
        order.reserve((size_t)E);
        std::deque<int32_t> q;
        for (int32_t e = 0; e < E; ++e)
            if (indeg[e] == 0) q.push_back(e);
        while (!q.empty()) {
            const int32_t v = q.front();
            q.pop_front();
            order.push_back(v);
            for (int32_t w : adj[v]) {
                level[w] = std::max(level[w], level[v] + 1);
                if (--indeg[w] == 0) q.push_back(w);
            }
        }
        if ((int64_t)order.size() != E) throw McdError(MCD_ERR_RUNTIME, "Invalid DAG: cycle detected");

        // plan: bounds, value ranges of every event's PMF, grid bounds, pool offsets
        const double step = (double)d->step;
        std::vector<AnEv> ev((size_t)E);
        std::vector<double> vlo((size_t)E), vhi((size_t)E);  // value range of each event's PMF
        std::vector<double> pmf_mass((size_t)K), pmf_last((size_t)K);
        for (int32_t k = 0; k < K; ++k) {
            double s = 0.0;
            for (int64_t i = d->pmf_off[k]; i < d->pmf_off[k + 1]; ++i) s += d->pmf_probs[i];
            pmf_mass[k] = s;
            pmf_last[k] = d->pmf_first[k] + step * (double)(d->pmf_off[k + 1] - d->pmf_off[k] - 1);
        }
        std::vector<AnOut> init((size_t)E);
        int64_t pool = 0;
        for (int32_t e : order) {
            AnEv &r = ev[e];
            r.pred_begin = (int32_t)(tlen[e] > 0 ? tstart[e] : 0);
            r.pred_end = (int32_t)(tlen[e] > 0 ? tstart[e] + tlen[e] : 0);
            r.scratch_off = -1;
            if (tlen[e] == 0) {  // origin: a unit mass at the rounded earliest time (_propagator.py:105-111)
                const double v = (double)py_round(d->earliest[e] / step) * step;
                vlo[e] = vhi[e] = v;
                r.lower = r.upper = 0;
                r.cap = 1;
                r.gmax = 1;
                r.pool_off = pool;
                pool += 1;
                init[e] = AnOut{v, 0.0, 0.0, 1.0, 1, 0};
                continue;
            }
            const double lat = d->latest[e], ear = d->earliest[e];
            const double up = std::isnan(d->max_delay) ? lat : std::min(lat, ear + d->max_delay);
            r.lower = py_round(ear);
            r.upper = py_round(up);
            double glo = std::numeric_limits<double>::infinity(), ghi = -glo;
            for (int64_t p = tstart[e]; p < tstart[e] + tlen[e]; ++p) {
                const int32_t s = d->pred_src[p], k = d->pred_pmf[p];
                glo = std::min(glo, vlo[s] + d->pmf_first[k]);
                ghi = std::max(ghi, vhi[s] + pmf_last[k]);
            }
            const double span = std::floor((ghi - glo) / step) + 3.0;  // + grid rounding margin
            if (!(span < 2.0e9)) throw McdError(MCD_ERR_INVALID, "an event's PMF grid is too large");
            r.gmax = (int32_t)span;
            const double win = (double)(r.upper - r.lower);
            const double capd = win >= 0.0 ? std::floor(win / step) + 1.0 : 1.0;
            r.cap = (int32_t)std::max(1.0, std::min(capd, span));
            r.pool_off = pool;
            pool += r.cap;
            // the clipped PMF lies in [lower, upper] (a kept range or one bound value)
            vlo[e] = (double)r.lower;
            vhi[e] = (double)std::max(r.lower, r.upper);
            init[e] = AnOut{0.0, 0.0, 0.0, 0.0, 0, 0};
        }
        // levels of non-origin events, scratch per level
        int32_t n_levels = 0;
        for (int32_t e = 0; e < E; ++e)
            if (tlen[e] > 0) n_levels = std::max(n_levels, level[e]);
        std::vector<std::vector<int32_t>> by_level((size_t)n_levels + 1);
        for (int32_t e : order)
            if (tlen[e] > 0) by_level[level[e]].push_back(e);
        an = new mcd_analytic();
        an->E = E;
        std::vector<int32_t> level_ev;
        std::vector<int2> chunks;
        std::vector<int64_t> conv_off((size_t)std::max<int64_t>(P, 1), 0);
        an->level_off.push_back(0);
        an->chunk_off.push_back(0);
        int64_t scratch_max = 0, conv_max = 0;
        for (int32_t l = 1; l <= n_levels; ++l) {
            int64_t scratch = 0, smem_bins = 0, conv = 0;
            std::vector<std::pair<int64_t, int2>> level_chunks;  // (estimated multiply-adds, chunk)
            for (int32_t e : by_level[l]) {
                AnEv &r = ev[e];
                if (r.gmax <= kAnSmemBins) {
                    smem_bins = std::max<int64_t>(smem_bins, r.gmax);
                } else {
                    r.scratch_off = scratch;
                    scratch += 5 * (int64_t)r.gmax;
                }
                level_ev.push_back(e);
                for (int64_t p = tstart[e]; p < tstart[e] + tlen[e]; ++p) {  // each convolution's slot and chunks
                    const int64_t n = ev[d->pred_src[p]].cap, m = d->pmf_off[d->pred_pmf[p] + 1] - d->pmf_off[d->pred_pmf[p]];
                    const int64_t len = n == 1 ? m : (m == 1 ? n : n + m - 1);
                    conv_off[p] = conv;
                    conv += (len + 1) / 2 * 2;
                    for (int64_t c = 0; c * kConvOuts < len; ++c) {
                        const int64_t jm = c * kConvOuts + kConvOuts / 2;  // the chunk's middle output
                        const int64_t terms = (n == 1 || m == 1) ? 1
                                                                 : (std::min(jm, n - 1) - std::max<int64_t>(0, jm - (m - 1)) + 1);
                        level_chunks.emplace_back(std::max<int64_t>(terms, 1) * kConvOuts, make_int2((int)p, (int)c));
                    }
                }
            }
            std::stable_sort(level_chunks.begin(), level_chunks.end(),
                             [](const auto &x, const auto &y) { return x.first > y.first; });
            for (const auto &lc : level_chunks) chunks.push_back(lc.second);
            scratch_max = std::max(scratch_max, scratch);
            conv_max = std::max(conv_max, conv);
            an->level_off.push_back((int32_t)level_ev.size());
            an->chunk_off.push_back((int32_t)chunks.size());
            an->level_smem.push_back((int32_t)(5 * smem_bins * (int64_t)sizeof(double)));
        }
        an->bins = pool;
        // device layout: one allocation
        cuda_check(cudaGetDevice(&an->device), "cudaGetDevice");
        cuda_check(cudaStreamCreateWithFlags(&an->stream, cudaStreamNonBlocking), "stream create");
        const size_t s_ev = align_up((size_t)E * sizeof(AnEv), 256), s_pred = align_up((size_t)std::max<int64_t>(P, 1) * 4, 256),
                     s_poff = align_up((size_t)(K + 1) * 8, 256), s_pk = align_up((size_t)std::max(K, 1) * 8, 256),
                     s_probs = align_up((size_t)std::max<int64_t>(d->pmf_off[K], 1) * 8, 256),
                     s_out = align_up((size_t)std::max(E, 1) * sizeof(AnOut), 256),
                     s_pool = align_up((size_t)std::max<int64_t>(pool, 1) * 8, 256),
                     s_scr = align_up((size_t)std::max<int64_t>(scratch_max, 1) * 8, 256),
                     s_lev = align_up((size_t)std::max<size_t>(level_ev.size(), 1) * 4, 256), s_err = 256,
                     s_coff = align_up(conv_off.size() * 8, 256), s_conv = align_up((size_t)std::max<int64_t>(conv_max, 1) * 8, 256),
                     s_chunk = align_up(std::max<size_t>(chunks.size(), 1) * sizeof(int2), 256);
        const size_t total = s_ev + 2 * s_pred + s_poff + 2 * s_pk + s_probs + s_out + s_pool + s_scr + s_lev + s_err +
                             s_coff + s_conv + s_chunk;
        cuda_check(cudaMalloc(&an->dmem, total), "analytic allocation");
        char *p = an->dmem;
        auto put = [&](const void *src, size_t bytes, size_t slot) -> char * {
            char *at = p;
            if (bytes) cuda_check(cudaMemcpy(at, src, bytes, cudaMemcpyHostToDevice), "analytic upload");
            p += slot;
            return at;
        };
        std::vector<int32_t> psrc((size_t)P), ppmf((size_t)P);
        for (int64_t i = 0; i < P; ++i) {
            psrc[i] = d->pred_src[i];
            ppmf[i] = d->pred_pmf[i];
        }
        AnArgs &a = an->args;
        a.ev = reinterpret_cast<const AnEv *>(put(ev.data(), (size_t)E * sizeof(AnEv), s_ev));
        a.pred_src = reinterpret_cast<const int32_t *>(put(psrc.data(), (size_t)P * 4, s_pred));
        a.pred_pmf = reinterpret_cast<const int32_t *>(put(ppmf.data(), (size_t)P * 4, s_pred));
        a.pmf_off = reinterpret_cast<const int64_t *>(put(d->pmf_off, (size_t)(K + 1) * 8, s_poff));
        a.pmf_first = reinterpret_cast<const double *>(put(d->pmf_first, (size_t)K * 8, s_pk));
        a.pmf_mass = reinterpret_cast<const double *>(put(pmf_mass.data(), (size_t)K * 8, s_pk));
        a.pmf_probs = reinterpret_cast<const double *>(put(d->pmf_probs, (size_t)d->pmf_off[K] * 8, s_probs));
        a.out = reinterpret_cast<AnOut *>(put(init.data(), (size_t)E * sizeof(AnOut), s_out));
        a.pool = reinterpret_cast<double *>(p);
        {  // origins' unit masses
            std::vector<double> ones((size_t)std::max<int64_t>(pool, 1), 0.0);
            for (int32_t e = 0; e < E; ++e)
                if (tlen[e] == 0) ones[(size_t)ev[e].pool_off] = 1.0;
            cuda_check(cudaMemcpy(p, ones.data(), (size_t)pool * 8, cudaMemcpyHostToDevice), "analytic upload");
        }
        p += s_pool;
        a.scratch = reinterpret_cast<double *>(p);
        p += s_scr;
        an->d_level_ev = reinterpret_cast<int32_t *>(put(level_ev.data(), level_ev.size() * 4, s_lev));
        a.conv_off = reinterpret_cast<const int64_t *>(put(conv_off.data(), conv_off.size() * 8, s_coff));
        a.convbuf = reinterpret_cast<double *>(p);
        p += s_conv;
        an->d_chunks = reinterpret_cast<int2 *>(put(chunks.data(), chunks.size() * sizeof(int2), s_chunk));
        a.err = reinterpret_cast<int32_t *>(p);
        cuda_check(cudaMemset(a.err, 0, 4), "analytic error flag");
        a.step = d->step;
        a.urule = d->underflow_rule;
        a.orule = d->overflow_rule;
        cuda_check(cudaFuncSetAttribute(k_an_fold, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)(5 * kAnSmemBins * sizeof(double))),
                   "analytic shared memory");
        int sms = 0;
        cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, an->device), "device query");
        // every level's launches, captured once into a graph
        cuda_check(cudaStreamBeginCapture(an->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
        for (size_t l = 0; l + 1 < an->level_off.size(); ++l) {
            const int32_t nc = an->chunk_off[l + 1] - an->chunk_off[l], ne = an->level_off[l + 1] - an->level_off[l];
            if (nc > 0)
                k_an_conv<<<std::min(nc, sms * kConvWarpsPerSm), 32, 0, an->stream>>>(
                    an->args, an->d_chunks + an->chunk_off[l], nc);
            if (ne > 0)
                k_an_fold<<<ne, kAnThreads, an->level_smem[l], an->stream>>>(an->args, an->d_level_ev + an->level_off[l]);
        }
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(an->stream, &g);
        cuda_check(ce, "graph capture");
        const cudaError_t ie = cudaGraphInstantiate(&an->graph, g, 0);
        cudaGraphDestroy(g);
        cuda_check(ie, "graph instantiate");
        *out = an;
    });
    if (rc != MCD_OK && an) mcd_analytic_destroy(an);
    return rc;
}

void mcd_analytic_destroy(mcd_analytic *an) {
    if (!an) return;
    if (an->stream) cudaStreamSynchronize(an->stream);
    if (an->graph) cudaGraphExecDestroy(an->graph);
    if (an->stream) cudaStreamDestroy(an->stream);
    if (an->dmem) cudaFree(an->dmem);
    delete an;
}

int mcd_analytic_run(mcd_analytic *an) {
    return guarded([&] {
        if (!an) throw McdError(MCD_ERR_INVALID, "null handle");
        cuda_check(cudaSetDevice(an->device), "cudaSetDevice");
        cuda_check(cudaGraphLaunch(an->graph, an->stream), "analytic launch");
        cuda_check(cudaStreamSynchronize(an->stream), "analytic run");
        int32_t flags = 0;
        cuda_check(cudaMemcpy(&flags, an->args.err, 4, cudaMemcpyDeviceToHost), "analytic error flag");
        if (flags) {
            cuda_check(cudaMemset(an->args.err, 0, 4), "analytic error flag");
            if (flags & AN_ERR_BOUNDS) throw McdError(MCD_ERR_INVALID, "min_value must not exceed max_value");
            if (flags & AN_ERR_UNDER_TRUNC)
                throw McdError(MCD_ERR_INVALID, "Underflow mass cannot be truncated: no lower-bound bin present.");
            if (flags & AN_ERR_OVER_TRUNC)
                throw McdError(MCD_ERR_INVALID, "Overflow mass cannot be truncated: no upper-bound bin present.");
            if (flags & AN_ERR_EMPTY) throw McdError(MCD_ERR_INVALID, "PMF must not be empty after clipping");
            if (flags & AN_ERR_GRID)
                throw McdError(MCD_ERR_INVALID, "PMF values do not fit their common grid (values off the step grid)");
            throw McdError(MCD_ERR_RUNTIME, "analytic kernel: a PMF exceeded its planned support");
        }
        an->ran = true;
    });
}

int64_t mcd_analytic_bins(const mcd_analytic *an) { return an ? an->bins : 0; }

int mcd_analytic_fetch(const mcd_analytic *an, double *first, int64_t *offset, int64_t *length, double *probs,
                       double *underflow, double *overflow) {
    return guarded([&] {
        if (!an) throw McdError(MCD_ERR_INVALID, "null handle");
        if (!an->ran) throw McdError(MCD_ERR_INVALID, "run() has not completed");
        cuda_check(cudaSetDevice(an->device), "cudaSetDevice");
        std::vector<AnOut> o((size_t)an->E);
        std::vector<AnEv> ev((size_t)an->E);
        if (an->E) {
            cuda_check(cudaMemcpy(o.data(), an->args.out, o.size() * sizeof(AnOut), cudaMemcpyDeviceToHost),
                       "analytic fetch");
            cuda_check(cudaMemcpy(ev.data(), an->args.ev, ev.size() * sizeof(AnEv), cudaMemcpyDeviceToHost),
                       "analytic fetch");
        }
        if (probs && an->bins)
            cuda_check(cudaMemcpy(probs, an->args.pool, (size_t)an->bins * 8, cudaMemcpyDeviceToHost),
                       "analytic fetch");
        for (int32_t e = 0; e < an->E; ++e) {
            if (first) first[e] = o[e].first;
            if (offset) offset[e] = ev[e].pool_off;
            if (length) length[e] = o[e].len;
            if (underflow) underflow[e] = o[e].under;
            if (overflow) overflow[e] = o[e].over;
        }
    });
}

}  // extern "C"
