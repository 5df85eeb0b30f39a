// mcd_internal.hpp -- records shared by the host DAG compiler and the CUDA kernels.
//
// The compiled DAG is a level-ordered CSR: events are sorted by level (longest
// path from a source), each level is split into one contiguous chunk per warp,
// and every event's predecessors keep their precedence-list order (the tie rule
// of the reference's propagation loop, _core.cpp:338-347, depends on it).
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define MCD_HD __host__ __device__
#else
#define MCD_HD
#endif

namespace mcd {

// x * 2^q truncated toward zero, from the bits b of a finite double x with
// |x| * 2^q < 2^62: the statistics tick count of a time.  The host builds the
// per-run table of earliest ticks with this same definition the kernels use.
MCD_HD inline long long ticks_of(long long b, int q) {
    const int e = (int)((b >> 52) & 0x7FF);
    const long long m = (b & 0xFFFFFFFFFFFFFll) | (e ? (1ll << 52) : 0ll);
    const int sh = (e ? e : 1) - 1075 + q;
    long long t;
    if (sh >= 0) t = m << sh;
    else t = sh > -63 ? (m >> -sh) : 0ll;
    return b < 0 ? -t : t;
}

// Delay kinds as the kernels see them.  FIXED covers links whose duration does
// not vary between samples: unmapped types, gaps in the link index space and the
// constant distribution, whose `base + base*factor` the host evaluates once with
// the reference's two roundings (_core.cpp:75, 328).
enum Kind : int32_t { K_FIXED = 0, K_EXP = 1, K_GAMMA = 2, K_EMP_ABS = 3, K_EMP_REL = 4 };

// Packed kind word of a link reference:
//   kind | word << KD_WORD_SHIFT | KD_REUSE | KD_TWO_WORD | KD_WRITE | dist << 8.
// Random words: a link draws from the Philox block `block` of its PredRec.
// Links first referenced by the same work unit (one event, or a pair of events
// of one stage that one warp runs back to back) share blocks of four words:
// one-word links (exponential; empirical tables of at most kOneWordBins bins)
// take one word, gamma links of shape 1, 2 or 3 (sum of exponentials) take that
// many words for their first attempt; `word` is the first of them.  KD_REUSE
// marks a reference whose block the unit's previous reference of these kinds
// already drew (the words are still in registers).  Other gamma links and
// larger empirical tables (KD_TWO_WORD) own their block.  KD_WRITE marks the one
// reference of a link that stores its duration row; links no precedence entry
// references are stored by the aux-link pass.
constexpr int32_t KD_KIND_MASK = 0x07;
constexpr int KD_WORD_SHIFT = 3;  // bits 3-4
constexpr int32_t KD_REUSE = 0x20;
constexpr int32_t KD_TWO_WORD = 0x40;
constexpr int32_t KD_WRITE = 0x80;
constexpr int32_t kOneWordBins = 4096;  // one 32-bit word picks bin and alias (threshold lattice <= 2^-20)

// One event, in compiled (level) order.  48 bytes.
struct alignas(16) EvRec {
    int32_t user;        // event index as the caller numbers it (output row)
    int32_t slot;        // window slot holding this event's realized value, -1 if no consumer
    int32_t pred_begin;  // range in the PredRec array
    int32_t pred_end;
    int64_t init_bits;   // earliest (bits): the running max starts here (_core.cpp:336)
    int64_t ub_bits;     // earliest + max_delay (bits), evaluated on the host (_core.cpp:334)
    // (the keys last: with all times non-negative and finite the bits are the keys,
    // and the kernels skip this third 16-byte load)
    int64_t init_key;    // order key of earliest; INT64_MAX when earliest is NaN
    int64_t ub_key;      // order key of ub; INT64_MAX when ub is NaN (std::min then keeps t)
};

// One predecessor edge.  32 bytes.
struct alignas(16) PredRec {
    int32_t src_slot;  // window slot of the predecessor's realized value (-1: read its global row)
    int32_t src_user;  // predecessor event index (cause_event value, global row)
    int32_t link;      // link index: durations row and Philox counter; -1 for an index
                       // past the last link, which has duration 0 (see the compiler)
    int32_t kd;        // packed kind word (above)
    double v;          // FIXED: the duration; otherwise the base (minimal_duration)
    int32_t dvo;       // FIXED: bits of the float d(duration)/d(base) (1 + factor, 1, or 0
                       // for gaps); empirical kinds: where the link's duration table is
                       // (see kLinkTableBins), -1 without one
    int32_t block;     // Philox block of the link's random words (-1: fixed)
};

// Empirical links whose table has at most kLinkTableBins bins carry a duration
// table of their own: entry k is the reference's duration for bin k, evaluated
// once on the host with its two roundings (base + value, _core.cpp:125, 328;
// base + factor * base, :140, 328).  The tables of a stage's references follow
// its predecessor records (the stage's value region, staged with them), so a
// draw is a bin choice and one shared-memory read -- no FP64 arithmetic.
// PredRec::dvo locates the table: the byte offset of its first entry inside the
// staging buffer, or, for a stage read from global memory, kVtGlobal | the index
// of its first entry in KArgs::vals.
constexpr int32_t kLinkTableBins = 32;
constexpr int32_t kVtGlobal = 0x40000000;

// A link whose duration row the aux pass stores: a link no precedence entry
// references (its duration is still part of SimResult.durations).  16 bytes.
struct alignas(16) LinkRec {
    int32_t link;
    int32_t kd;
    double v;
};

// Per-distribution constants, single precision where the sampler works in FP32.
struct alignas(16) DistParam {
    int32_t kind;
    int32_t tab_off;   // empirical: first alias entry
    int32_t tab_n;     // empirical: number of bins
    int32_t boost;     // gamma: shape < 1 (Marsaglia-Tsang on shape+1, times U^(1/shape))
    float f0, f1, f2, f3, f4, f5;
    // exponential: f0 = lambda_ (mean), f1 = c = 1 - exp(-max_scale/lambda_), f2 = 1 - c,
    //              f3 = largest float <= max_scale
    // gamma:       f0 = d = shape' - 1/3, f1 = 1/sqrt(9 d), f2 = 1/shape, f3 = scale,
    //              f4 = largest float <= max_scale
    int32_t erlang;    // gamma: the shape when it is 1, 2 or 3 (sum of exponentials), else 0
    int32_t link_tab;  // empirical: tables of at most kLinkTableBins bins (per-link duration tables)
};

// Walker/Vose alias entry: bin j is kept when a 32-bit uniform is below
// `thresh`, otherwise its alias is taken.  The two candidate values are stored
// inline so a draw costs one gather.  32 bytes.
struct alignas(16) AliasEntry {
    double v_self;
    double v_alias;
    uint32_t thresh;
    uint32_t pad[3];
};

// The bin choice of the same table, 8 bytes per bin so that 32 lanes reading
// random bins of a table of up to 32 bins hit distinct shared-memory banks:
// bin j is kept when the uniform is below `thresh`, else bin `alias` is taken
// (alias == j when thresh is 0xFFFFFFFF).  Parallel to the AliasEntry array.
struct alignas(8) AliasPick {
    uint32_t thresh;
    int32_t alias;
};

// Adjoint forward record per (event, sample): the winning predecessor's position
// in the event's list (kAdjNone: no predecessor won, realized = earliest), and
// flags for "clamped at earliest + max_delay" and "realized > earliest".
constexpr uint32_t kAdjNone = 0x3FFFu;
constexpr uint32_t kAdjClamped = 0x4000u;
constexpr uint32_t kAdjDelayed = 0x8000u;
constexpr int32_t kAdjMaxPreds = 0x3FFF;     // events with more predecessors are rejected
constexpr int kAdjDfacShift = 20;            // link gradients accumulate cnt * dfac * 2^20

// Per-event statistics layout: 256 equal bins over [earliest, earliest +
// max_delay] plus two exact atoms -- realized == earliest (not delayed) and
// realized == earliest + max_delay (capped) -- padded to 260 counters.
constexpr int kHistBins = 256;
constexpr int kBinLo = 256;
constexpr int kBinHi = 257;
constexpr int kHistStride = 260;
// Histogram counters a single-DAG statistics launch updates, in bytes, up to which
// every lane adds its own count to its bin: the counters stay in L2, where one
// atomic per lane is cheaper than finding a warp's equal bins first (measured:
// the per-DAG statistics of the batching workload 1.41e11 -> 1.46e11
// sample-edges/s).  Above it, and in the batch and served kernels -- many DAGs'
// counters at once, where per-lane atomics measured slower -- a warp's equal
// bins are added once.
constexpr int64_t kHistLaneBytes = 48ll << 20;

// Ints of stage metadata per stage (three int4 loads).  A stage's first
// 2 * pairs events form pairs (events 2u and 2u + 1 are one work unit: one warp
// runs them back to back and they share Philox blocks); each later event is a
// unit of its own.
constexpr int kStageMetaInts = 12;

// Arguments of the propagation kernels.
struct KArgs {
    const EvRec *ev;
    const PredRec *pred;
    const LinkRec *aux;
    const DistParam *dist;    // tables block: DistParam[n_dist], AliasEntry[n_alias], AliasPick[n_alias]
    const int32_t *wk_off;    // [n_stages * n_warps + 1] event chunk per (stage, warp), compiled indices
    const int32_t *stage_meta;  // [n_stages][kStageMetaInts] {first event, events (negated: read from global),
                                //  first pred, preds, first value, values, byte offsets of the predecessor
                                //  records and of the value region inside a staging buffer, event pairs, 0, 0, 0}
    const double *vals;         // per-link duration tables, stage by stage (value regions)
    int32_t n_stages;
    int32_t n_warps;
    int32_t n_aux;
    int32_t window_slots;
    int32_t n_dist, n_alias;
    int32_t tables_in_smem;   // distribution tables copied into shared memory
    int32_t win_smem;         // window on chip (batch kernel dispatch)
    int32_t positive;         // every time non-negative and finite: raw bits order like doubles
    int32_t stage_bytes;      // one staging buffer
    int32_t smem_stage_off, smem_tables_off, smem_bar_off, smem_total;  // shared-memory layout (bytes)
    const int64_t *seeds;  // [n] per-sample seeds; null: sample s uses seed0 + s
    int64_t seed0;
    int64_t n;
    int64_t ld;            // leading dimension of the sample-minor outputs
    double *realized;      // [E][ld] or null (then `scratch` holds the rows the window spills)
    double *durations;     // [L][ld] or null
    int32_t *cause;        // [E][ld] or null
    const double *dur_in;  // given durations [L][ld_in] (propagation-only mode)
    int64_t ld_in;
    double *scratch;       // [E][ld] realized rows when the window is not on chip and realized is null
    int32_t *err;          // latched device error flags
    // statistics mode
    int32_t stats_fixed;          // 1: realized - earliest accumulated as exact integer ticks
    int32_t tick_q;               // tick = 2^-tick_q seconds
    unsigned long long bin_mul;   // bin = mulhi64(delta_ticks, bin_mul)
    double hist_inv_w;            // FP64 fallback: 256 / max_delay, 0 when not finite
    unsigned long long *acc;      // [E] sum of delta ticks (fixed) or FP64 sum bits (fallback)
    const long long *te;          // [E] ticks_of(earliest, tick_q), caller order (fixed ticks only)
    uint32_t *hist;               // [E][kHistStride]
    int32_t hist_lane;            // 1: every lane adds its own count (the counters stay in L2);
                                  // 0: a warp's equal bins are added once (kHistLaneBytes)
    // adjoint
    uint16_t *adj_code;           // [events of the block][ld] winner position and flags (forward), read
                                  // backward; row = compiled event index - code_base; null: not recorded
    float *adj_dfac;              // [events of the block][ld] d(duration)/d(base) of the winning link
    long long *grad_e;            // [E] sum over samples of the earliest-time derivative (counts)
    long long *grad_l;            // [L] sum over samples of cnt * dfac * 2^20 per link
    // adjoint by level blocks: the kernels run stages [stage_begin, stage_end)
    int32_t stage_begin, stage_end;
    int32_t code_base;            // compiled index of the event whose records are row 0 of adj_code
    int32_t adj_flags;            // kAdjObjective | kAdjCntLoad | kAdjCntSave
    const int32_t *blk_start;     // [n_blk] first stage of each block after the first (checkpoint pass)
    int32_t n_blk;
    double *win_ckpt;             // [n_blk][tiles][window_slots * 32]: the window as block k + 1 starts
    const double *win_in;         // [tiles][window_slots * 32]: the window to start from, or null
    uint32_t *cnt_ckpt;           // [tiles][window_slots * 32]: backward counts carried between blocks
    uint32_t *cnt_rows;           // [E][ld] backward counts by caller index (window not on chip)
};

// KArgs::adj_flags
constexpr int32_t kAdjObjective = 1;  // forward: add (realized - earliest) to the objective sum
constexpr int32_t kAdjCntLoad = 2;    // backward: start from the counts in cnt_ckpt (else zero)
constexpr int32_t kAdjCntSave = 4;    // backward: leave the counts in cnt_ckpt for the next block

// Arguments of the persistent batch kernel.
struct BatchArgs {
    const KArgs *dags;           // [n_dags] statistics-mode arguments, one per DAG
    const int32_t *items;        // [n_items][2] (dag, tile), longest first
    int32_t n_items;
    unsigned int *counter;       // work-queue head, zero before the launch
    double *scratch;             // per-CTA realized rows for DAGs whose window is not on chip
    int64_t scratch_stride;      // doubles per CTA (max events x 32)
    int32_t smem_bytes;          // dynamic shared memory of the launch (>= every DAG's layout)
};

// Arguments of the statistics finishing kernel.
struct FArgs {
    const unsigned long long *acc;
    const uint32_t *hist;
    const double *earliest;  // caller order
    const double *ub;        // earliest + max_delay, caller order
    int32_t E;
    int32_t stats_fixed;
    int32_t tick_q;
    double bin_w;            // seconds per bin
    int64_t n;               // samples accumulated
    double *mean, *p50, *p90, *p99, *p_on_time;  // [E] each, any may be null
};

// Device error flags.
enum : int32_t { ERR_GAMMA_REJECTION = 1, ERR_STAGE_TIMEOUT = 2, ERR_LAYOUT = 4 };

constexpr int kTile = 32;  // samples per tile: one per lane
// End of a CTA's shared memory: two mbarriers (8 bytes each), then the two
// stage work counters (int32 each), padded to 32 bytes.
constexpr int kBarRegionBytes = 32;

}  // namespace mcd
