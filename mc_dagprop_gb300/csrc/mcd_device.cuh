// mcd_device.cuh -- device code of the Monte Carlo DAG-propagation path (sm_103a).
//
// k_propagate: one CTA owns a tile of 32 samples (one per lane) and walks the
// whole compiled DAG stage by stage (a stage is a level, or a slice of a wide
// level); the warps of the CTA split each stage's events and meet at a barrier
// between stages.  The records of the next stage are copied into shared memory
// by the TMA bulk-copy engine (cp.async.bulk + mbarrier, double-buffered) while
// the current one is processed, so no warp waits on L2 for DAG records.
// Realized times of events that later stages still read live in a shared-memory
// "window" (slot-major, one 256-byte row of 32 samples per live event), so
// predecessor reads never touch HBM; every output row is written once,
// coalesced (256 B per warp store).
//
// FP64 throughput on this part is about 2 lanes per clock per SM (a warp's FP64
// instruction holds the pipe ~16 SM clocks), against ~108 for 32-bit integer
// logic, so FP64 is spent only where bit-exactness needs it: the
// one IEEE add per edge of the reference's loop (_core.cpp:341).  Comparisons
// run on 64-bit integer order keys that order doubles like the IEEE operators;
// a sampled duration base * (1 + X) is one FP64 multiply by the double equal to
// the float 1 + X, that double built with integer operations.
//
// Delays come from Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11) in counter mode: the counter holds the
// sample's 64-bit seed, the link and the attempt.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "mcd_internal.hpp"

namespace mcd {

// Raises a kernel's dynamic shared-memory limit to at least `smem` bytes and
// never lowers it: kernels captured in graphs and launches from other threads
// keep the limit they were recorded with.
cudaError_t raise_smem_limit(const void *fn, size_t smem);

// ---------------------------------------------------------------- Philox4x32-10
// Counter mode under one fixed key: the 128-bit counter is (seed low, seed high,
// link, salt ^ attempt), so a draw depends only on (sample seed, link, attempt)
// and the ten round keys are compile-time constants (no key registers, no key
// schedule arithmetic in the loop).
struct U4 {
    uint32_t x, y, z, w;
};

constexpr uint32_t kPhiloxM0 = 0xD2511F53u, kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u, kPhiloxW1 = 0xBB67AE85u;
constexpr uint32_t kKey0 = 0x243F6A88u, kKey1 = 0x85A308D3u;  // fixed key (hex digits of pi)
constexpr uint32_t kStreamSalt = 0x6D636470u;               // counter word 3: separates this stream's use

__device__ __forceinline__ U4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)kPhiloxM0 * c0;  // one wide multiply: hi and lo words
        const uint64_t p1 = (uint64_t)kPhiloxM1 * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ (kKey0 + (uint32_t)r * kPhiloxW0);
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ (kKey1 + (uint32_t)r * kPhiloxW1);
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
    }
    return U4{c0, c1, c2, c3};
}

// The draw for (sample seed, link, attempt, sel): sel separates the calls one
// attempt may make.
__device__ __forceinline__ U4 draw_words(uint64_t seed, uint32_t link, uint32_t attempt, uint32_t sel) {
    return philox((uint32_t)seed, (uint32_t)(seed >> 32), link, kStreamSalt ^ ((attempt << 1) | sel));
}

// Uniform in (0, 1]: (r + 1/2) / 2^32 rounded to float.
__device__ __forceinline__ float u01_open0(uint32_t r) {
    return fmaf(__uint2float_rn(r), 2.3283064365386963e-10f, 1.1641532182693481e-10f);
}

// ---------------------------------------------------------------- order keys
// Signed 64-bit key with key(a) < key(b) <=> a < b for non-NaN doubles, and
// key(-0) == key(+0) as the IEEE comparison has it.  NaN maps to INT64_MIN so
// that `ub < t` and `t >= latest` are both false for a NaN t, as in C++.
// POSITIVE: every time of the DAG is a non-negative finite double (checked by
// the host), for which the bit pattern itself is the key.
template <bool POSITIVE>
__device__ __forceinline__ long long order_key(long long b) {
    if (POSITIVE) return b;
    const long long mag = b & 0x7FFFFFFFFFFFFFFFll;
    const long long k = b < 0 ? -mag : mag;
    return mag > 0x7FF0000000000000ll ? (long long)0x8000000000000000ull : k;
}

// ---------------------------------------------------------------- duration scaling
// The double equal to a finite float m >= 1, built with integer operations: a
// float-to-double conversion would occupy the FP64 pipe, which on this part
// issues about 2 lane-operations per clock per SM.
__device__ __forceinline__ double widen(float m) {
    const uint32_t b = __float_as_uint(m);
    const uint32_t hi = (((b >> 23) + 896u) << 20) | ((b >> 3) & 0x000FFFFFu);
    return __hiloint2double((int)hi, (int)(b << 29));
}

// A sampled duration base * (1 + X), 1 + X rounded to float and held below
// float overflow (reached only for means above ~1e37): one FP64 multiply.
__device__ __forceinline__ double scale_by(double base, float m) {
    return __dmul_rn(base, widen(fminf(m, 3.4028234663852886e38f)));
}

// ---------------------------------------------------------------- samplers
// Each returns the link's duration (base + extra) for one sample.

// Exponential with mean lambda_, redrawn above max_scale (_core.cpp:83-89).  The
// redraw loop is replaced by the inverse CDF of the truncated law, which is the
// same distribution: X = -lambda_ * log(1 - c u), c = 1 - exp(-max_scale/lambda_).
// r: the link's random word.  The duration is base * (1 + X), 1 + X in float.
__device__ __forceinline__ double draw_exponential(const DistParam &p, double base, uint32_t r, float &dfac) {
    const float w = u01_open0(r);         // plays the role of 1 - u
    const float V = fmaf(p.f1, w, p.f2);  // 1 - c (1 - w), in (1-c, 1]
    float X = -p.f0 * __logf(V);
    X = fmaxf(fminf(X, p.f3), 0.0f);
    dfac = 1.0f + X;
    return scale_by(base, dfac);
}

__device__ __forceinline__ uint32_t word_of(const U4 &g, int i) {
    return i == 0 ? g.x : i == 1 ? g.y : i == 2 ? g.z : g.w;
}

// Gamma(shape, scale) redrawn above max_scale (_core.cpp:98-104).  Shapes 1, 2
// and 3 are sums of that many exponentials (Erlang): X = -scale * log(U1 U2 U3).
// The first attempt takes its uniforms from words w.. of the block the event's
// links share (grp); redraws use blocks of the link's own, keyed by the attempt.
// Rejection loops are capped; a lane that hits the cap latches
// ERR_GAMMA_REJECTION and returns the truncation point.
static __device__ __forceinline__ double draw_erlang(const DistParam &p, double base, uint32_t link, uint64_t seed,
                                                  const U4 &grp, int w, int32_t *err, float *dfac) {
    float prod = u01_open0(word_of(grp, w));
    if (p.erlang > 1) prod *= u01_open0(word_of(grp, w + 1));
    if (p.erlang > 2) prod *= u01_open0(word_of(grp, w + 2));
    float X = fmaxf(-p.f3 * __logf(prod), 0.0f);
    for (uint32_t attempt = 1; X > p.f4; ++attempt) {
        if (attempt == 4096u) {
            atomicOr(err, ERR_GAMMA_REJECTION);
            X = p.f4;
            break;
        }
        const U4 r = draw_words(seed, link, attempt, 0u);
        prod = u01_open0(r.x);
        if (p.erlang > 1) prod *= u01_open0(r.y);
        if (p.erlang > 2) prod *= u01_open0(r.z);
        X = fmaxf(-p.f3 * __logf(prod), 0.0f);
    }
    *dfac = 1.0f + X;
    return scale_by(base, *dfac);
}

// Other shapes by Marsaglia & Tsang (ACM TOMS 26(3), 2000) in FP32, normals from
// Box-Muller; shapes below 1 draw Gamma(shape+1) times U^(1/shape).  The link
// owns its blocks.  Same rejection cap.
static __device__ __forceinline__ double draw_gamma(const DistParam &p, double base, uint32_t link, uint64_t seed,
                                                 int32_t *err, float *dfac) {
    const float d = p.f0, cc = p.f1;
    for (uint32_t attempt = 0; attempt < 4096u; ++attempt) {
        const U4 r = draw_words(seed, link, attempt, 0u);
        const float rad = __fsqrt_rn(-2.0f * __logf(u01_open0(r.x)));
        float sn, cs;
        __sincosf(6.2831853071795865f * ((float)(r.y >> 8) * 5.9604644775390625e-08f), &sn, &cs);
        float X = -1.0f;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const float z = j == 0 ? rad * cs : rad * sn;
            const float t = fmaf(cc, z, 1.0f);
            if (X < 0.0f && t > 0.0f) {
                const float v = t * t * t;
                const float u = u01_open0(j == 0 ? r.z : r.w);
                const float z2 = z * z;
                if (u < 1.0f - 0.0331f * z2 * z2 || __logf(u) < 0.5f * z2 + d * (1.0f - v + __logf(v))) X = d * v;
            }
        }
        if (X < 0.0f) continue;
        if (p.boost) {
            const U4 r2 = draw_words(seed, link, attempt, 1u);
            X *= exp2f(__log2f(u01_open0(r2.x)) * p.f2);
        }
        X *= p.f3;
        if (X > p.f4) continue;
        *dfac = 1.0f + X;
        return scale_by(base, *dfac);
    }
    atomicOr(err, ERR_GAMMA_REJECTION);
    *dfac = 1.0f + p.f4;
    return scale_by(base, *dfac);
}

// Empirical tables (_core.cpp:110-141) by Walker/Vose alias sampling.  One
// word r: the bin is the high half of r * n and the low half, uniform on a
// lattice of spacing n / 2^32, decides bin or alias (tables of at most
// kOneWordBins bins); two words (r, r2): r picks the bin, r2 decides.  The
// duration is the reference's -- base + value (absolute, :125, 328) or base +
// factor * base (relative, :140, 328) -- bit for bit, because the values are
// atoms and any last-bit difference would separate the two discrete
// distributions: read from the link's own table (vt, kLinkTableBins) or, for
// larger tables and links without one, evaluated here in FP64.
__device__ __forceinline__ double draw_empirical(const DistParam &p, const AliasEntry *alias, const AliasPick *picks,
                                                 const double *vt, double base, bool relative, uint32_t r,
                                                 uint32_t r2, bool two_word, float &dfac) {
    const uint32_t j = __umulhi(r, (uint32_t)p.tab_n);
    const uint32_t u = two_word ? r2 : r * (uint32_t)p.tab_n;
    if (vt) {
        const AliasPick pk = picks[p.tab_off + j];
        const int k = u < pk.thresh ? (int)j : pk.alias;
        dfac = relative ? 1.0f + (float)alias[p.tab_off + k].v_self : 1.0f;
        return vt[k];
    }
    const AliasEntry &e = alias[p.tab_off + j];
    const double val = u < e.thresh ? e.v_self : e.v_alias;
    dfac = relative ? 1.0f + (float)val : 1.0f;
    return relative ? __dadd_rn(base, __dmul_rn(val, base)) : __dadd_rn(base, val);
}

// A sampled link's duration.  TSMEM: the tables block is in shared memory;
// STAGED: the link's duration table (if any) is in the current stage's staging
// buffer.  Both are compile-time here so that every table read is a
// shared-memory load (or a global one) rather than a generic load.
template <bool STAGED, bool TSMEM>
__device__ __forceinline__ double sampled_duration(const KArgs &a, int32_t kd, double v, int32_t dvo, uint32_t block,
                                                   uint32_t link, uint64_t seed, U4 &grp, const unsigned char *smem,
                                                   int buf, float &dfac) {
    const DistParam *dists = TSMEM ? reinterpret_cast<const DistParam *>(smem + a.smem_tables_off) : a.dist;
    const DistParam &p = dists[kd >> 8];
    int32_t *err = a.err;
    const AliasEntry *alias = reinterpret_cast<const AliasEntry *>(dists + a.n_dist);
    const AliasPick *picks = reinterpret_cast<const AliasPick *>(alias + a.n_alias);
    const int kind = kd & KD_KIND_MASK;
    if (kind == K_GAMMA && !p.erlang) return draw_gamma(p, v, block, seed, err, &dfac);
    if (!(kd & KD_REUSE)) grp = draw_words(seed, block, 0u, 0u);
    const int wsel = (kd >> KD_WORD_SHIFT) & 3;
    if (kind == K_GAMMA) return draw_erlang(p, v, link, seed, grp, wsel, err, &dfac);
    const uint32_t r = word_of(grp, wsel);
    if (kind == K_EXP) return draw_exponential(p, v, r, dfac);
    const double *vt = nullptr;
    if (dvo >= 0)
        vt = STAGED ? reinterpret_cast<const double *>(smem + a.smem_stage_off + buf * a.stage_bytes + dvo)
                    : a.vals + (dvo ^ kVtGlobal);
    return draw_empirical(p, alias, picks, vt, v, kind == K_EMP_REL, r, grp.y, (kd & KD_TWO_WORD) != 0, dfac);
}

// The link's duration for one sample, and (dfac) its derivative with respect to
// the base duration: 1 + X for the multiplicative kinds, 1 for absolute tables,
// the host-computed value for fixed links.  block: the link's Philox block;
// grp: the words of the block the event's previous exponential or empirical
// reference drew, redrawn here unless KD_REUSE says they are this link's block.
// link: the link's index (the key of its own redraw blocks); dvo: the record's
// dvo (PredRec); buf: the staging buffer (0 or 1) that holds the link's
// duration table (STAGED; otherwise the table is in KArgs::vals).  Every table
// address is derived here from the kernel arguments, so that the propagation
// loop keeps no table pointers live.
// TS: where the tables block is -- kTablesGlobal, kTablesSmem (fixed for the
// kernel: one copy of the samplers, no branch per edge), or kTablesEither
// (KArgs::tables_in_smem decides per launch or per DAG).
enum : int { kTablesGlobal = 0, kTablesSmem = 1, kTablesEither = 2 };
template <bool STAGED, int TS>
__device__ __forceinline__ double link_duration(const KArgs &a, int32_t kd, double v, int32_t dvo, uint32_t block,
                                                uint32_t link, uint64_t seed, U4 &grp, const unsigned char *smem,
                                                int buf, float &dfac) {
    if ((kd & KD_KIND_MASK) == K_FIXED) {
        dfac = __int_as_float(dvo);
        return v;
    }
    if (TS == kTablesSmem || (TS == kTablesEither && a.tables_in_smem))
        return sampled_duration<STAGED, true>(a, kd, v, dvo, block, link, seed, grp, smem, buf, dfac);
    return sampled_duration<STAGED, false>(a, kd, v, dvo, block, link, seed, grp, smem, buf, dfac);
}

// ---------------------------------------------------------------- records
// Record reads as 16-byte vector loads (two for a predecessor; three for an event,
// two where the order keys go unused: the compiler drops the third).
__device__ __forceinline__ PredRec load_pred(const PredRec *p) {
    const int4 a = reinterpret_cast<const int4 *>(p)[0];
    const int4 b = reinterpret_cast<const int4 *>(p)[1];
    PredRec r;
    r.src_slot = a.x;
    r.src_user = a.y;
    r.link = a.z;
    r.kd = a.w;
    r.v = __hiloint2double(b.y, b.x);
    r.dvo = b.z;
    r.block = b.w;
    return r;
}

__device__ __forceinline__ EvRec load_ev(const EvRec *p) {
    const int4 a = reinterpret_cast<const int4 *>(p)[0];
    const int4 b = reinterpret_cast<const int4 *>(p)[1];
    const int4 c = reinterpret_cast<const int4 *>(p)[2];
    EvRec r;
    r.user = a.x;
    r.slot = a.y;
    r.pred_begin = a.z;
    r.pred_end = a.w;
    r.init_bits = (int64_t)(((uint64_t)(uint32_t)b.y << 32) | (uint32_t)b.x);
    r.ub_bits = (int64_t)(((uint64_t)(uint32_t)b.w << 32) | (uint32_t)b.z);
    r.init_key = (int64_t)(((uint64_t)(uint32_t)c.y << 32) | (uint32_t)c.x);
    r.ub_key = (int64_t)(((uint64_t)(uint32_t)c.w << 32) | (uint32_t)c.z);
    return r;
}

// ---------------------------------------------------------------- TMA staging
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Bulk copy global -> shared (16-byte aligned addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Issues the copies of one stage's event records, predecessor records and value
// region into a buffer.  A stage too large for the buffer (n_ev stored negated)
// copies nothing; its barrier phase still completes, so the buffers' phases
// stay in step.  A value region holds an even number of doubles (16-byte sizes
// and offsets).
__device__ __forceinline__ void stage_issue(const KArgs &a, int stage, char *buf, uint64_t *bar) {
    const int4 *meta = reinterpret_cast<const int4 *>(a.stage_meta + kStageMetaInts * stage);
    const int4 m = __ldg(meta);       // ev_first, n_ev, pred_first, n_pred
    const int4 mv = __ldg(meta + 1);  // val_first, n_val, byte offsets of predecessor records and values
    const bool staged = m.y >= 0;
    const uint32_t ev_bytes = staged ? (uint32_t)m.y * (uint32_t)sizeof(EvRec) : 0u;
    const uint32_t pr_bytes = staged ? (uint32_t)m.w * (uint32_t)sizeof(PredRec) : 0u;
    const uint32_t va_bytes = staged ? (uint32_t)mv.y * (uint32_t)sizeof(double) : 0u;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bar, ev_bytes + pr_bytes + va_bytes);
    if (ev_bytes) bulk_g2s(buf, a.ev + m.x, ev_bytes, bar);
    if (pr_bytes) bulk_g2s(buf + mv.z, a.pred + m.z, pr_bytes, bar);
    if (va_bytes) bulk_g2s(buf + mv.w, a.vals + mv.x, va_bytes, bar);
}

// Bounded wait for a stage buffer; false (and the error flag latched) if the copy
// did not land within `limit` polls.
__device__ __forceinline__ bool stage_wait(uint64_t *bar, uint32_t parity, int32_t *err,
                                           uint32_t limit = 1u << 24) {
    for (uint32_t it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    atomicOr(err, ERR_STAGE_TIMEOUT);
    return false;
}

// ---------------------------------------------------------------- statistics helpers
// Statistics tick count of a realized time (ticks_of).  POSITIVE: the time is
// non-negative and finite, and |x| * 2^q < 2^62 makes every shift of the
// mantissa m a right shift of m << 10 (below 2^63): one variable shift.
template <bool POSITIVE>
__device__ __forceinline__ long long tick_count(long long b, int q) {
    if (!POSITIVE) return ticks_of(b, q);
    const int e = (int)(b >> 52);
    const long long m = (b & 0xFFFFFFFFFFFFFll) | ((long long)(e != 0) << 52);
    const int r = 1085 - q - (e ? e : 1);
    return r < 64 ? (long long)((unsigned long long)(m << 10) >> r) : 0ll;
}

// Sum over the warp of non-negative 64-bit tick counts below 2^54: two 27-bit
// limbs summed with one redux.sync each (a limb's sum stays below 2^32), then
// recombined -- the exact sum.  The host's choice of tick keeps every per-sample
// count below 2^54 (and the sum over all samples below 2^63).
__device__ __forceinline__ long long warp_sum_ticks(long long d) {
    const unsigned long long u = (unsigned long long)d;
    const unsigned s0 = __reduce_add_sync(0xFFFFFFFFu, (unsigned)(u & 0x7FFFFFFu));
    const unsigned s1 = __reduce_add_sync(0xFFFFFFFFu, (unsigned)(u >> 27));
    return (long long)((unsigned long long)s0 + ((unsigned long long)s1 << 27));
}

// One event's realized values of the tile into the per-event accumulators:
// the tile's sum of (realized - earliest) with one 64-bit atomic, and the
// histogram with one atomic per lane (LANE_HIST and KArgs::hist_lane) or per
// distinct bin of the warp.  te: the event's earliest in ticks (KArgs::te),
// loaded when the event started.
template <bool POSITIVE, bool LANE_HIST>
__device__ __forceinline__ void accumulate_stats(const KArgs &a, const EvRec &ev, long long lbits, long long te,
                                                 bool active, unsigned active_mask) {
    int bin;
    if (a.stats_fixed) {
        // realized >= earliest and ticks are monotone: d >= 0
        const long long d = active ? tick_count<POSITIVE>(lbits, a.tick_q) - te : 0ll;
        bin = (int)__umul64hi((unsigned long long)d, a.bin_mul);
        bin = bin > kHistBins - 1 ? kHistBins - 1 : bin;
        const long long s = warp_sum_ticks(d);
        if ((threadIdx.x & 31) == 0 && s != 0) atomicAdd(&a.acc[ev.user], (unsigned long long)s);
    } else {
        const double dd = active ? __longlong_as_double(lbits) - __longlong_as_double(ev.init_bits) : 0.0;
        const double x = dd * a.hist_inv_w;
        bin = x >= (double)(kHistBins - 1) ? kHistBins - 1 : (x > 0.0 ? (int)x : 0);
        if (active && dd != 0.0) atomicAdd(reinterpret_cast<double *>(&a.acc[ev.user]), dd);
    }
    if (lbits == ev.init_bits) bin = kBinLo;
    else if (lbits == ev.ub_bits) bin = kBinHi;
    if (LANE_HIST && a.hist_lane) {
        if (active) atomicAdd(&a.hist[(int64_t)ev.user * kHistStride + bin], 1u);
    } else if (active) {
        const unsigned same = __match_any_sync(active_mask, bin);
        if ((threadIdx.x & 31) == __ffs(same) - 1)
            atomicAdd(&a.hist[(int64_t)ev.user * kHistStride + bin], (unsigned)__popc(same));
    }
}

// The tile's sum of (realized - earliest) ticks into a.acc (objective of the
// adjoint; the same integer accumulation as the statistics mean).
template <bool POSITIVE>
__device__ __forceinline__ void accumulate_sum(const KArgs &a, const EvRec &ev, long long lbits, long long te,
                                               bool active) {
    const long long s = warp_sum_ticks(active ? tick_count<POSITIVE>(lbits, a.tick_q) - te : 0ll);
    if ((threadIdx.x & 31) == 0 && s != 0) atomicAdd(&a.acc[ev.user], (unsigned long long)s);
}

// ---------------------------------------------------------------- stage bodies
// Offset of row `row` (>= 0) in rows of ld elements: one 32 x 32 -> 64-bit
// multiply (leading dimensions are below 2^32, checked by the host).
__device__ __forceinline__ uint64_t row_off(int32_t row, uint32_t ld) { return (uint64_t)(uint32_t)row * ld; }

// Element `row` (>= 0) of a column whose rows are ld_bytes apart: one 32 x 32-bit
// multiply-add onto the 64-bit column address (row pitches below 2^32 bytes: the
// host keeps leading dimensions below 2^29).
template <typename T>
__device__ __forceinline__ T *at_row(T *col, int32_t row, uint32_t ld_bytes) {
    return reinterpret_cast<T *>(reinterpret_cast<uintptr_t>(col) + (uint64_t)(uint32_t)row * ld_bytes);
}

// A tile's per-lane state: its sample, seed, and output columns.
struct TileCtx {
    int lane;
    int64_t s;                 // the lane's sample
    bool active;               // s < n
    unsigned active_mask;
    uint64_t seed;
    double *rcol;              // this lane's column of the global realized rows (window off chip, or
                               // output), or null
    uint32_t rows_ld8;         // their row pitch in bytes
    double *dcol;              // durations output column of this lane (null: none, or inactive)
    int32_t *ccol;             // cause_event output column of this lane (null: none, or inactive)
    uint32_t ld8, ld4;         // row pitches of the outputs in bytes (doubles, int32)
    const double *dincol;      // given durations: this lane's column (GIVEN)
    uint32_t ld_in8;
};

// Lane 0 takes the next event index of a stage from its shared-memory counter.
// (An increment with wrap-around at 2^31 - 1, which equals an add of one here: an
// add of a constant is compiled into a warp-aggregated atomic, several
// instructions per event for one active lane.)
__device__ __forceinline__ int take_next(uint32_t ctr) {
    int v;
    asm volatile("atom.shared.inc.u32 %0, [%1], 0x7FFFFFFF;" : "=r"(v) : "r"(ctr) : "memory");
    return v;
}

// One stage's work units, taken one at a time from the stage's counter: unit
// u < n_pair is the pair of events 2u and 2u + 1, run back to back so that the
// second continues the first's Philox block (grp); unit u >= n_pair is event
// u + n_pair alone (the compiler orders the pairs, then the single events,
// costliest first).  STAGED:
// sev/spred point into the staging buffer in shared memory; otherwise into
// global memory.  pred0: the stage's first predecessor record (the records'
// pred_begin/pred_end are global indices); ev0: its first event's compiled
// index; buf: the staging buffer (0 or 1) that holds the stage.
template <bool GIVEN, bool WIN_SMEM, bool STATS, bool POSITIVE, bool ADJ, bool STAGED, int TS, bool LANE_HIST>
__device__ __forceinline__ void stage_events(const KArgs &a, int buf, const EvRec *sev, const PredRec *spred, int pred0,
                                             int ev0, int n_ev, int n_pair, uint32_t ctr, const TileCtx &t,
                                             unsigned char *smem, U4 &grp) {
    double *win = reinterpret_cast<double *>(smem);
    const int lane = t.lane;
    // The warp's next event: the second of the current pair, or the first event of
    // the next unit, which lane 0 takes before this event's work, hiding the
    // atomic's latency (a warp holds at most one extra unit: the cheapest, by
    // order).  Units past the last map to events past n_ev.
    int i_next = 0;
    if (lane == 0) {
        const int u = take_next(ctr);
        i_next = u < n_pair ? 2 * u : u + n_pair;
    }
    i_next = __shfl_sync(0xFFFFFFFFu, i_next, 0);
    while (i_next < n_ev) {
        const int i = i_next;
        if (i < 2 * n_pair && !(i & 1)) {
            i_next = i + 1;
        } else if (lane == 0) {
            const int u = take_next(ctr);
            i_next = u < n_pair ? 2 * u : u + n_pair;
        }
        const EvRec ev = load_ev(sev + i);
        // the event's earliest in ticks, needed after its predecessors (the load's
        // latency hides behind them)
        const long long te =
            (STATS || (ADJ && (a.adj_flags & kAdjObjective))) && a.stats_fixed ? __ldg(a.te + ev.user) : 0ll;
        // POSITIVE: keys are the bits themselves (init_key == init_bits, ub_key == ub_bits),
        // so one 64-bit value carries both
        long long lk = POSITIVE ? ev.init_bits : ev.init_key, lbits = ev.init_bits;
        const long long ub_key = POSITIVE ? ev.ub_bits : ev.ub_key;
        int32_t cause = -1;
        uint32_t win_code = kAdjNone;  // ADJ: winner position | clamp flag
        float win_dfac = 0.0f;
        const int pb = ev.pred_begin - pred0, pe = ev.pred_end - pred0;
        // Given durations come from global memory, each an uncached DRAM read: the
        // reads of up to four entries are issued together, then the entries are
        // relaxed in order (one memory latency per four entries, not per entry).
        for (int p0 = pb; GIVEN && p0 < pe; p0 += 4) {
            double dg[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                dg[k] = 0.0;
                if (p0 + k < pe) {
                    const int32_t link = reinterpret_cast<const int4 *>(spred + p0 + k)->z;  // PredRec::link
                    if (t.active && link >= 0) dg[k] = __ldg(at_row(t.dincol, link, t.ld_in8));
                }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (p0 + k >= pe) continue;
                const PredRec pr = load_pred(spred + p0 + k);
                const double src = WIN_SMEM ? win[pr.src_slot * kTile + lane]
                                            : (t.active ? *at_row(t.rcol, pr.src_user, t.rows_ld8) : 0.0);
                const double tt = src + dg[k];  // the one FP64 add of the edge (_core.cpp:341)
                long long tb = __double_as_longlong(tt);
                long long tk = order_key<POSITIVE>(tb);
                const bool clamp = ub_key < tk;
                if (clamp) {  // t = std::min(t, ub)
                    tk = ub_key;
                    tb = ev.ub_bits;
                }
                if (tk >= lk) {  // if (t >= latest) { latest = t; cause = src; }
                    lk = tk;
                    lbits = POSITIVE ? tk : tb;
                    cause = pr.src_user;
                    if (ADJ) win_code = (uint32_t)(p0 + k - pb) | (clamp ? kAdjClamped : 0u);
                }
            }
        }
        for (int p = pb; !GIVEN && p < pe; ++p) {
            const PredRec pr = load_pred(spred + p);
            float dfac = 0.0f;
            const double dur = link_duration<STAGED, TS>(a, pr.kd, pr.v, pr.dvo, (uint32_t)pr.block,
                                                         (uint32_t)pr.link, t.seed, grp, smem, buf, dfac);
            if (!STATS && !ADJ && (pr.kd & KD_WRITE) && t.dcol) *at_row(t.dcol, pr.link, t.ld8) = dur;
            // with the window on chip every source has a slot (the compiler checks it)
            const double src = WIN_SMEM ? win[pr.src_slot * kTile + lane]
                                        : (t.active ? *at_row(t.rcol, pr.src_user, t.rows_ld8) : 0.0);
            const double tt = src + dur;  // the one FP64 add of the edge (_core.cpp:341)
            long long tb = __double_as_longlong(tt);
            long long tk = order_key<POSITIVE>(tb);
            const bool clamp = ub_key < tk;
            if (clamp) {  // t = std::min(t, ub)
                tk = ub_key;
                tb = ev.ub_bits;
            }
            if (tk >= lk) {  // if (t >= latest) { latest = t; cause = src; }
                lk = tk;
                lbits = POSITIVE ? tk : tb;
                cause = pr.src_user;
                if (ADJ) {
                    win_code = (uint32_t)(p - pb) | (clamp ? kAdjClamped : 0u);
                    win_dfac = dfac;
                }
            }
        }
        // realized = std::min(latest, ub): latest only exceeds ub when earliest does, which
        // non-negative max_delay rules out in POSITIVE mode
        if (!POSITIVE && ub_key < lk) lbits = ev.ub_bits;
        const double real = __longlong_as_double(lbits);
        if (WIN_SMEM && ev.slot >= 0) win[ev.slot * kTile + lane] = real;
        if (STATS) accumulate_stats<POSITIVE, LANE_HIST>(a, ev, lbits, te, t.active, t.active_mask);
        if (ADJ) {
            const bool delayed = lk > (POSITIVE ? ev.init_bits : ev.init_key);  // realized > earliest
            if (a.adj_flags & kAdjObjective) accumulate_sum<POSITIVE>(a, ev, lbits, te, t.active);
            if (t.active && a.adj_code) {  // rows by compiled index, from the block's first event
                const int64_t o = (int64_t)row_off(ev0 + i - a.code_base, (uint32_t)a.ld) + t.s;
                a.adj_code[o] = (uint16_t)(win_code | (delayed ? kAdjDelayed : 0u));
                a.adj_dfac[o] = win_dfac;
            }
        }
        if (t.active && t.rcol) *at_row(t.rcol, ev.user, t.rows_ld8) = real;
        if (!STATS && !ADJ && t.ccol) *at_row(t.ccol, ev.user, t.ld4) = cause;
        i_next = __shfl_sync(0xFFFFFFFFu, i_next, 0);
    }
}

// ---------------------------------------------------------------- propagation
// Walks the compiled DAG for one tile of 32 samples (the tile's sample s is
// tile * 32 + lane) with all warps of the CTA.
// GIVEN: durations come from a.dur_in instead of the sampler.
// WIN_SMEM: predecessor values come from the shared-memory window; otherwise
// from global realized rows: rows[event * rows_ld + rows_col].
// STATS: instead of output rows, each event's realized values feed the
// per-event accumulators (mean, histogram); nothing per sample leaves the chip.
// POSITIVE: all times non-negative and finite (host-checked): raw bits are keys.
// reuse: the CTA ran an earlier tile with these barriers (persistent kernels).
// Returns false when a staged copy never landed (then every thread returns false).
//
// Shared memory: [window: window_slots x 32 doubles][stage buffer 0][stage
// buffer 1][distribution params][alias entries][alias picks][2 mbarriers, 2
// stage counters]; a stage buffer holds [event records][predecessor
// records][value region]; `bars` is that layout's barrier region
// (kBarRegionBytes), or one fixed region for every tile of a persistent CTA (a
// barrier stays where it was initialised: only the same address is invalidated
// and initialised again between tiles).
// ADJ: the forward half of the adjoint: per event and sample, the winning
// predecessor's position, clamp and delay flags and d(duration)/d(base) go to
// a.adj_code / a.adj_dfac (when not null), and (realized - earliest) to the
// objective sum (kAdjObjective).  It runs stages [a.stage_begin, a.stage_end)
// only: with the window on chip it starts from the window a.win_in holds for
// this tile (when not null), and saves the window into a.win_ckpt as each of the
// a.blk_start stages begins -- the checkpoints a level-block recomputation
// starts from.
template <bool GIVEN, bool WIN_SMEM, bool STATS, bool POSITIVE, bool ADJ = false, int TS = kTablesEither,
          bool LANE_HIST = true>
__device__ __forceinline__ bool propagate_tile(const KArgs &a, int64_t tile, double *rows, int64_t rows_ld,
                                               bool rows_tile_local, unsigned char *smem, uint64_t *bars,
                                               bool reuse) {
    DistParam *s_dist = reinterpret_cast<DistParam *>(smem + a.smem_tables_off);

    TileCtx t;
    t.lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int NW = a.n_warps;
    t.s = tile * kTile + t.lane;
    t.active = t.s < a.n;
    t.active_mask = __ballot_sync(0xFFFFFFFFu, t.active);
    t.seed = 0;
    if (!GIVEN && t.active) t.seed = a.seeds ? (uint64_t)a.seeds[t.s] : (uint64_t)(a.seed0 + t.s);
    t.rcol = rows ? rows + (rows_tile_local ? (int64_t)t.lane : t.s) : nullptr;
    t.rows_ld8 = (uint32_t)rows_ld * 8u;
    t.ld8 = (uint32_t)a.ld * 8u;
    t.ld4 = (uint32_t)a.ld * 4u;
    t.dincol = GIVEN ? a.dur_in + t.s : nullptr;
    t.ld_in8 = (uint32_t)a.ld_in * 8u;
    t.dcol = (!STATS && !ADJ && !GIVEN && a.durations && t.active) ? a.durations + t.s : nullptr;
    t.ccol = (!STATS && !ADJ && a.cause && t.active) ? a.cause + t.s : nullptr;

    // distribution tables into shared memory; fresh barriers for this tile
    if (a.tables_in_smem) {  // the tables block, 8 bytes at a time (its size is a multiple of 8)
        const int n8 = (a.n_dist * (int)sizeof(DistParam) + a.n_alias * (int)(sizeof(AliasEntry) + sizeof(AliasPick))) / 8;
        for (int i = threadIdx.x; i < n8; i += blockDim.x)
            reinterpret_cast<uint2 *>(s_dist)[i] = reinterpret_cast<const uint2 *>(a.dist)[i];
    }
    // stages run: all, or (adjoint) one block of them
    const int s_begin = ADJ ? a.stage_begin : 0;
    const int s_end = ADJ ? a.stage_end : a.n_stages;
    const int win_n = a.window_slots * kTile;  // doubles of one tile's window
    if (ADJ && WIN_SMEM && a.win_in) {  // a block recomputed from its checkpoint
        const double *src = a.win_in + (int64_t)tile * win_n;
        double *win = reinterpret_cast<double *>(smem);
        for (int i = threadIdx.x; i < win_n; i += blockDim.x) win[i] = src[i];
    }
    int next_blk = 0;  // the next checkpoint to save (ADJ with a.win_ckpt)
    int *stage_ctr = reinterpret_cast<int *>(bars + 2);
    U4 grp{};  // the words of the Philox block the current event last drew (see KD_REUSE)
    if (threadIdx.x == 0) {
        if (reuse) {
            asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&bars[0])) : "memory");
            asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&bars[1])) : "memory");
        }
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        stage_ctr[0] = 0;
        stage_ctr[1] = 0;
    }
    // A persistent CTA's previous tile may have had another layout: its window
    // stores (generic proxy) can lie where this tile's staged copies (async
    // proxy) land, so every thread orders its stores before the copies.
    if (reuse) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    char *stage_buf0 = reinterpret_cast<char *>(smem + a.smem_stage_off);
    if (threadIdx.x == 0) {
        if (s_begin < s_end) stage_issue(a, s_begin, stage_buf0, &bars[0]);
        if (s_begin + 1 < s_end) stage_issue(a, s_begin + 1, stage_buf0 + a.stage_bytes, &bars[1]);
    }

    // a stage's metadata is loaded one stage ahead: its latency then hides behind
    // the previous stage's events instead of stalling every warp at the stage start
    const int4 *smeta = reinterpret_cast<const int4 *>(a.stage_meta);
    constexpr int kMetaVecs = kStageMetaInts / 4;
    int4 meta_next = make_int4(0, 0, 0, 0), mv_next = make_int4(0, 0, 0, 0);
    int pairs_next = 0;
    if (s_begin < s_end) {
        meta_next = __ldg(smeta + kMetaVecs * s_begin);
        mv_next = __ldg(smeta + kMetaVecs * s_begin + 1);
        pairs_next = __ldg(a.stage_meta + kStageMetaInts * s_begin + 8);
    }
    for (int l = s_begin; l < s_end; ++l) {
        const int4 meta = meta_next, mv = mv_next;
        const int n_pair = pairs_next;
        if (l + 1 < s_end) {
            meta_next = __ldg(smeta + kMetaVecs * (l + 1));
            mv_next = __ldg(smeta + kMetaVecs * (l + 1) + 1);
            pairs_next = __ldg(a.stage_meta + kStageMetaInts * (l + 1) + 8);
        }
        const int j = l - s_begin;  // stages run so far: buffer, barrier phase and counter
        const int b = j & 1;
        const bool ok = stage_wait(&bars[b], (uint32_t)((j >> 1) & 1), a.err);
        if (__syncthreads_or(!ok)) {  // a copy that never landed: drain, then leave together
            if (threadIdx.x == 0 && l + 1 < s_end)
                stage_wait(&bars[b ^ 1], (uint32_t)(((j + 1) >> 1) & 1), a.err);
            __syncthreads();
            return false;
        }
        if (ADJ && WIN_SMEM && a.win_ckpt && next_blk < a.n_blk && l == __ldg(a.blk_start + next_blk)) {
            // the window as this block starts (every earlier stage's stores are behind the barrier)
            double *dst = a.win_ckpt + ((int64_t)next_blk * gridDim.x + tile) * win_n;
            const double *win = reinterpret_cast<const double *>(smem);
            for (int i = threadIdx.x; i < win_n; i += blockDim.x) dst[i] = win[i];
            ++next_blk;
            __syncthreads();  // before this stage's events overwrite slots
        }
        if (threadIdx.x == 0) stage_ctr[(j + 1) & 1] = 0;  // last used by stage l - 1, before the barrier
        const uint32_t ctr = smem_u32(&stage_ctr[j & 1]);
        if (meta.y >= 0) {  // records in the staging buffer (shared memory)
            const unsigned char *buf = smem + a.smem_stage_off + b * a.stage_bytes;
            stage_events<GIVEN, WIN_SMEM, STATS, POSITIVE, ADJ, true, TS, LANE_HIST>(
                a, b, reinterpret_cast<const EvRec *>(buf), reinterpret_cast<const PredRec *>(buf + mv.z), meta.z,
                meta.x, meta.y, n_pair, ctr, t, smem, grp);
        } else {  // a stage whose records exceed the buffer is read from global memory
            stage_events<GIVEN, WIN_SMEM, STATS, POSITIVE, ADJ, false, TS, LANE_HIST>(
                a, b, a.ev + meta.x, a.pred + meta.z, meta.z, meta.x, -meta.y, n_pair, ctr, t, smem, grp);
        }
        __syncthreads();
        if (threadIdx.x == 0 && l + 2 < s_end)
            stage_issue(a, l + 2, stage_buf0 + b * a.stage_bytes, &bars[b]);
    }
    // Aux pass: duration rows of links no precedence entry references.
    if (!STATS && !ADJ && !GIVEN && a.durations) {
        for (int i = warp; i < a.n_aux; i += NW) {
            const LinkRec lr = a.aux[i];
            float dfac;
            U4 own;  // an unreferenced link owns its block
            const double dur =
                link_duration<false, TS>(a, lr.kd, lr.v, -1, (uint32_t)lr.link, (uint32_t)lr.link, t.seed, own, smem, 0, dfac);
            if (t.dcol) *at_row(t.dcol, lr.link, t.ld8) = dur;
        }
    }
    return true;
}

// One CTA per tile of 32 samples.  TS: the tables block's place (kTablesGlobal or
// kTablesSmem; the host launches the instantiation that matches the DAG).
template <bool GIVEN, bool WIN_SMEM, bool STATS, bool POSITIVE, int TS>
__global__ void __launch_bounds__(768, 1) k_propagate(const KArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    double *rows = a.realized ? a.realized : a.scratch;  // global realized rows
    if (STATS && WIN_SMEM) rows = nullptr;
    propagate_tile<GIVEN, WIN_SMEM, STATS, POSITIVE, false, TS>(a, (int64_t)blockIdx.x, rows, a.ld, false, smem,
                                                                reinterpret_cast<uint64_t *>(smem + a.smem_bar_off),
                                                                false);
}

}  // namespace mcd
