/*
 * mc_dagprop_gb300.h -- C ABI of the GB300 Monte Carlo DAG-propagation engine.
 *
 * Plain C types only: pointers, sizes and opaque handles.  Every entry point
 * returns an int status (MCD_OK = 0); on failure mcd_last_error() gives the
 * message for the calling thread.  Nothing throws across this boundary.
 *
 * Each entry point replaces one piece of the reference's pybind11-bound C++
 * (paths inside the reference project, src/mc_dagprop/monte_carlo/_core.cpp):
 *
 *   mcd_generator_*           GenericDelayGenerator            _core.cpp:146-159, 519-542
 *   mcd_dag_create            Simulator::Simulator (DAG compile) _core.cpp:193-307
 *   mcd_dag_node_count        Simulator::node_count            _core.cpp:309
 *   mcd_dag_activity_count    Simulator::activity_count        _core.cpp:310
 *   mcd_run_many_host         Simulator::run_many / run        _core.cpp:312-361
 *   mcd_run_device            the same, device buffers, sample-minor layout
 *   mcd_propagate_*           the propagation loop alone       _core.cpp:331-350
 *   mcd_batch_*               many DAGs in one persistent launch (no reference counterpart)
 *   mcd_gradient_host/_plan   pathwise gradient of expected tardiness (no reference counterpart)
 *   mcd_server_*              continuous-batching request server (no reference counterpart)
 *   mcd_stats_*               per-event statistics (no reference counterpart; the
 *                             reference's users stack run_many results in numpy,
 *                             demo/monte_carlo.py:48-49)
 *   mcd_analytic_*            the analytic PMF propagator, src/mc_dagprop/analytic/
 *                             (pure Python in the reference)
 *   mcd_delay_histograms      per-type delay inspection, demo/inspection.py:11-29
 *
 * Layouts.  "Sample-major" (host entry points) is the reference's SimResult
 * layout: one contiguous row per sample, realized[s*E + e], durations[s*L + l],
 * cause_event[s*E + e].  "Sample-minor" (device entry points) is the GPU layout:
 * one row per event / link with samples contiguous, realized[e*ld + s],
 * durations[l*ld + s], cause_event[e*ld + s], n_samples <= ld < 2^29.
 *
 * Random numbers.  Each sample s is identified by a 64-bit seed; delays are drawn
 * from Philox4x32-10 keyed by that seed with the link index in the counter, so a
 * sample's delays do not depend on which batch, chunk or position it runs in.
 * Sampled delays therefore match the reference in distribution, not draw for
 * draw; given the same durations, propagation reproduces the reference bit for bit.
 */
#ifndef MC_DAGPROP_GB300_H
#define MC_DAGPROP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCD_ABI_VERSION 4

/* Status codes. */
#define MCD_OK 0
#define MCD_ERR_INVALID 1  /* bad argument: maps to ValueError / TypeError           */
#define MCD_ERR_RUNTIME 2  /* the reference's RuntimeError cases (cycle, reserved
                              type -1, negative max_delay, table length mismatch)   */
#define MCD_ERR_CUDA 3     /* CUDA runtime failure                                   */
#define MCD_ERR_NOMEM 4    /* device or host allocation failed                       */
#define MCD_ERR_DEVICE 5   /* a kernel reported an error (see message)              */

typedef struct mcd_generator mcd_generator; /* GenericDelayGenerator */
typedef struct mcd_dag mcd_dag;             /* compiled, device-resident Simulator */

/* Message of the last failing call on this thread ("" if none). */
const char *mcd_last_error(void);
int mcd_abi_version(void);

/* ---- GenericDelayGenerator (_core.cpp:146-159, bindings 519-542) ----
 * A later add_* for the same activity_type replaces the earlier one.
 * activity_type -1 is accepted here and rejected by mcd_dag_create, as in the
 * reference (_core.cpp:196-198).  Empirical tables with values/weights of
 * different lengths fail with MCD_ERR_RUNTIME (_core.cpp:119-120, 134-135). */
int mcd_generator_create(mcd_generator **out);
void mcd_generator_destroy(mcd_generator *gen);
int mcd_generator_set_seed(mcd_generator *gen, int64_t seed); /* stored; unused by runs, as in the reference */
int mcd_generator_add_constant(mcd_generator *gen, int32_t activity_type, double factor);
int mcd_generator_add_exponential(mcd_generator *gen, int32_t activity_type, double lambda_, double max_scale);
int mcd_generator_add_gamma(mcd_generator *gen, int32_t activity_type, double shape, double scale,
                            double max_scale);
int mcd_generator_add_empirical_absolute(mcd_generator *gen, int32_t activity_type, const double *values,
                                         int64_t n_values, const double *weights, int64_t n_weights);
int mcd_generator_add_empirical_relative(mcd_generator *gen, int32_t activity_type, const double *factors,
                                         int64_t n_factors, const double *weights, int64_t n_weights);

/* ---- DagContext, flattened (_core.cpp:52-62) ----
 * events:          earliest[n_events] (EventTimestamp.latest/actual are not read by the path)
 * activity map:    act_idx / act_duration / act_type [n_activities] (the (src,dst) key is not read)
 * precedence_list: target[n_targets], pred_offsets[n_targets+1],
 *                  pred_src / pred_act [pred_offsets[n_targets]] in list order */
typedef struct mcd_dag_desc {
    int32_t n_events;
    const double *earliest;
    int32_t n_activities;
    const int32_t *act_idx;
    const double *act_duration;
    const int32_t *act_type;
    int32_t n_targets;
    const int32_t *target;
    const int64_t *pred_offsets;
    const int32_t *pred_src;
    const int32_t *pred_act;
    double max_delay;
} mcd_dag_desc;

/* Compiled-DAG facts, for tests and tuning. */
typedef struct mcd_dag_info {
    int32_t n_events, n_links, n_levels, n_warps;
    int64_t n_preds;
    int32_t window_slots;      /* live event rows a sample tile keeps on chip */
    int32_t window_in_smem;    /* 1: window in shared memory, 0: re-read from global */
    int32_t n_orphan_links;    /* links sampled but not referenced by precedence_list */
    int32_t device;
    int64_t device_bytes;      /* resident compiled-DAG bytes */
    int32_t n_stages;          /* barrier-separated steps of the kernel (levels, wide ones split) */
    int32_t smem_bytes;        /* shared memory per CTA */
    int32_t positive;          /* 1: all times non-negative and finite (cheaper comparisons) */
    int32_t tables_in_smem;    /* 1: distribution tables held in shared memory */
    int32_t cache_hit;         /* 1: the compiled records are shared with an earlier live
                                  handle of identical inputs (compiled-DAG cache) */
    int32_t n_event_pairs;     /* pairs of events of one level that one warp runs back to
                                  back, sharing Philox blocks */
    int64_t block_draws;       /* Philox blocks one sample's propagation draws (first
                                  attempts; the rows of unreferenced links not counted) */
} mcd_dag_info;

/* Simulator::Simulator: validates, compiles to level-ordered CSR and uploads to
 * the current CUDA device.  The generator is copied; both inputs may be freed
 * afterwards.  Each handle owns its CUDA streams; a handle is not reentrant,
 * separate handles run concurrently.  A handle created from inputs identical to
 * those of a live handle on the same device (byte for byte: arrays, generator,
 * n_warps) shares that handle's compiled, read-only device records instead of
 * compiling again (the compiled-DAG cache; mcd_dag_options.no_cache opts out). */
int mcd_dag_create(const mcd_dag_desc *desc, const mcd_generator *gen, mcd_dag **out);
/* Compile options (the same call with explicit choices). */
#define MCD_WARPS_BATCH_CLASS (-1)
typedef struct mcd_dag_options {
    int32_t n_warps; /* warps per CTA, 1..24; 0 = chosen from the DAG's level width;
                        MCD_WARPS_BATCH_CLASS = chosen, then rounded up to 2, 4, 8, 12 or 24 */
    int32_t no_cache; /* 0: share the compiled records of a live handle created from
                         identical inputs (same arrays, generator, options and device);
                         1: compile a private copy */
    int32_t window;   /* where the propagation window lives (the realized times later
                         levels still read): MCD_WINDOW_AUTO in shared memory when it
                         fits, else global rows; MCD_WINDOW_GLOBAL always global rows */
} mcd_dag_options;
#define MCD_WINDOW_AUTO 0
#define MCD_WINDOW_GLOBAL 1
int mcd_dag_create_ex(const mcd_dag_desc *desc, const mcd_generator *gen, const mcd_dag_options *opts,
                      mcd_dag **out);
void mcd_dag_destroy(mcd_dag *dag);
/* Compiles on the host only (no CUDA call) and reports what mcd_dag_create
 * would build: validation errors are the same; device and device_bytes are -1. */
int mcd_dag_describe(const mcd_dag_desc *desc, const mcd_generator *gen, mcd_dag_info *info);
int32_t mcd_dag_node_count(const mcd_dag *dag);
int32_t mcd_dag_activity_count(const mcd_dag *dag);
int mcd_dag_get_info(const mcd_dag *dag, mcd_dag_info *info);
/* Random-number streams of the links ([activity_count] each): a sampled link's
 * draws come from Philox4x32-10 block block[l] (counter: sample seed, block,
 * attempt); word[l] in 0..3 is the first 32-bit word the link takes from it --
 * one word for exponential and small empirical links, 1-3 words for gamma of
 * shape 1-3, links first referenced by one event (or by a pair of events of one
 * level, run back to back) sharing blocks of four words --
 * and -1 when the link uses the whole block (other gamma shapes, large empirical
 * tables).  Gamma redraws above max_scale use blocks keyed by the link and the
 * attempt.  block[l] = -1 for links of fixed duration. */
int mcd_dag_link_streams(const mcd_dag *dag, int32_t *block, int32_t *word);
/* The handle's stream (a cudaStream_t), for callers that order their own work on it. */
void *mcd_dag_stream(const mcd_dag *dag);

/* ---- Host buffers, sample-major (reference SimResult layout) ----
 * run_many over n seeds: realized[n*E], durations[n*L], cause_event[n*E];
 * any output may be NULL.  Copies to and from the device happen inside; the call
 * returns when the outputs are in host memory.  Pinned host memory
 * (mcd_host_alloc) makes the copies run at full link speed. */
int mcd_run_many_host(mcd_dag *dag, const int64_t *seeds, int64_t n, double *realized, double *durations,
                      int32_t *cause_event);
/* Propagation alone, given durations[n*L] (for example the reference's own
 * SimResult.durations); bit-exact with the reference's loop. */
int mcd_propagate_host(mcd_dag *dag, const double *durations, int64_t n, double *realized,
                       int32_t *cause_event);

/* ---- Device buffers, sample-minor, asynchronous on `stream` (NULL = the handle's stream) ----
 * seeds[n] on the device; outputs realized[E*ld], durations[L*ld], cause_event[E*ld]
 * (any may be NULL).  Kernel errors are latched on the handle and reported by
 * mcd_dag_check(). */
int mcd_run_device(mcd_dag *dag, const int64_t *seeds, int64_t n, double *realized, double *durations,
                   int32_t *cause_event, int64_t ld, void *stream);
/* Propagation alone from device durations[L*ld_in] (sample-minor). */
int mcd_propagate_device(mcd_dag *dag, const double *durations, int64_t ld_in, int64_t n, double *realized,
                         int32_t *cause_event, int64_t ld, void *stream);
/* Synchronises the handle's stream and reports a latched kernel error, if any. */
int mcd_dag_check(mcd_dag *dag);
/* Self-test of the kernels' bounded waits (no reference counterpart): a kernel
 * waits on a barrier that nothing completes, with a short poll limit, on the
 * current device.  On return *timed_out is 1 when the wait gave up and latched its
 * error flag, *kernel_returned 1 when the kernel then ran to its end; the CUDA
 * context stays usable. */
int mcd_selftest_bounded_wait(int32_t *timed_out, int32_t *kernel_returned);

/* ---- Per-event statistics (the full sample matrix never leaves the chip) ----
 * For each event over n samples: mean of realized (FP64, accumulated exactly as
 * integer ticks of 2^-q s when all times are finite), p50/p90/p99 from a
 * 256-bin histogram over [earliest, earliest + max_delay] whose exact atoms --
 * realized == earliest ("on time") and realized == earliest + max_delay
 * ("capped") -- are counted apart, and the on-time fraction.
 * seeds[n] or, when seeds is NULL, seeds seed0 .. seed0+n-1.  Any output may be NULL.
 * hist: [n_events][MCD_HIST_STRIDE] counts: bins 0..255, then on-time, capped, 2 unused. */
#define MCD_HIST_BINS 256
#define MCD_HIST_STRIDE 260
typedef struct mcd_stats {
    double *mean, *p50, *p90, *p99, *p_on_time; /* [n_events] each */
    uint32_t *hist;                             /* [n_events][MCD_HIST_STRIDE] */
} mcd_stats;
/* Host outputs; returns when they are written. */
int mcd_stats_host(mcd_dag *dag, const int64_t *seeds, int64_t seed0, int64_t n, const mcd_stats *out);
/* Device outputs (and device seeds), asynchronous on `stream` (NULL = the handle's stream). */
int mcd_stats_device(mcd_dag *dag, const int64_t *seeds, int64_t seed0, int64_t n, const mcd_stats *out,
                     void *stream);
/* The same statistics without allocating device memory.  No counterpart in the
 * reference.  Some callers cannot call cudaMalloc: their GPU memory is owned by
 * another allocator (a framework's caching allocator that has reserved the
 * device), or an allocation would synchronise the device inside their
 * latency-critical loop.  This entry point keeps the per-event accumulators in a
 * fixed 34 MiB device array that the library holds on every GPU it is loaded on
 * until the process exits, so it supports DAGs of at most MCD_NOALLOC_MAX_EVENTS
 * events whose propagation window fits in shared memory (larger ones fail with
 * MCD_ERR_INVALID).  Inputs, outputs and the compiled DAG are the caller's, as in
 * mcd_stats_device (device pointers; asynchronous on `stream`, NULL = the
 * handle's stream).  The first call on a device (and in each CUDA context of it:
 * after a cudaDeviceReset, or with another context made current) looks the
 * array's device address up; make that first call before any stream capture.  All calls share the one
 * array, and each call clears it first: calls that overlap on the GPU (other
 * streams, other threads, other handles) race and corrupt each other's results. */
#define MCD_NOALLOC_MAX_EVENTS 32000
int mcd_stats_device_noalloc(mcd_dag *dag, const int64_t *seeds, int64_t seed0, int64_t n, const mcd_stats *out,
                             void *stream);
/* Width in seconds of one histogram bin for a run of n samples. */
int mcd_stats_bin_width(const mcd_dag *dag, int64_t n, double *out);

/* ---- Batches: many DAGs, each with its own samples, in one persistent launch ----
 * (no reference counterpart: the reference runs one DAG per run_many call).
 * DAG i runs samples with seeds seed0[i] .. seed0[i]+n_samples[i]-1 and produces
 * the same statistics as mcd_stats_* would for it alone.  All DAGs must share a
 * device and be compiled with the same n_warps (1..24, mcd_dag_create_ex); they
 * must outlive the batch.  A run is one CUDA graph (recorded on the first run,
 * replayed after): accumulator reset, the persistent kernel over (DAG, tile)
 * work items in longest-first order, the batched finish.  mcd_batch_run is
 * asynchronous on the batch's own stream; mcd_batch_sync waits and reports
 * kernel errors; mcd_batch_download copies DAG i's statistics to the host. */
typedef struct mcd_batch mcd_batch;
int mcd_batch_create(mcd_dag *const *dags, int32_t n_dags, const int64_t *seed0, const int64_t *n_samples,
                     mcd_batch **out);
void mcd_batch_destroy(mcd_batch *batch);
int mcd_batch_run(mcd_batch *batch);
int mcd_batch_sync(mcd_batch *batch);
int mcd_batch_download(mcd_batch *batch, int32_t i, const mcd_stats *host);
void *mcd_batch_stream(const mcd_batch *batch);
int64_t mcd_batch_items(const mcd_batch *batch);
int32_t mcd_batch_grid(const mcd_batch *batch);
/* CTAs of the persistent batch kernel one SM holds at n_warps warps per CTA and
 * smem_bytes of dynamic shared memory (the largest mcd_dag_info.smem_bytes of the
 * batch): DAGs with equal values share a launch without lowering each other's
 * occupancy.  (Every variant of the kernel runs at the same register count.) */
int mcd_batch_occupancy(int32_t n_warps, int64_t smem_bytes, int32_t *blocks_per_sm);

/* ---- Pathwise gradient (adjoint; no reference counterpart) ----
 * Objective J = mean over the n samples (seeds seed0 .. seed0+n-1) of
 * sum over events of (realized - earliest).  Writes J, dJ/d earliest [n_events]
 * and dJ/d base duration [activity_count] (per link index; Activity.minimal_duration
 * of the activity with that idx), any may be NULL.  The derivative follows each
 * sample's winning predecessor chain (the cause_event tie rule): slope 1 along
 * unclamped chains, d(duration)/d(base) at the winning link.  Needs finite times
 * and at most 16,383 predecessors per event.  Samples run in chunks; when the
 * winners of every event of a chunk (6 bytes per event and sample) do not fit the
 * memory budget (half the free device memory, at most 16 GiB), the levels are
 * split into blocks whose forward pass is recomputed from checkpoints of the
 * propagation window, block by block, last block first.  Every plan gives the
 * same bits. */
int mcd_gradient_host(mcd_dag *dag, int64_t seed0, int64_t n, double *objective, double *grad_earliest,
                      double *grad_base);
/* The plan the handle's last mcd_gradient_host call used: samples per chunk,
 * level blocks (1: every winner kept, no recomputation) and device bytes of its
 * per-chunk buffers; any may be NULL. */
int mcd_gradient_plan(const mcd_dag *dag, int64_t *samples_per_chunk, int64_t *level_blocks,
                      int64_t *buffer_bytes);

/* ---- Serving: continuous batching of statistics requests (no reference counterpart) ----
 * submit() copies a request (a DAG, its generator, seeds seed0 .. seed0+n-1) and
 * returns a ticket at once; host threads compile the DAGs and upload them while
 * their device memory fits memory_budget; a scheduler thread, whenever one of
 * n_streams slots is free, runs the uploaded requests of one class -- equal warps
 * per CTA and CTAs per SM, the class of the oldest waiting request -- as one
 * persistent batch.  A request's statistics equal those of the same request run
 * alone with mcd_stats_*.  Requests whose window does not fit in shared memory
 * run in batches of their own with per-CTA realized rows in global memory
 * (outside memory_budget: events x 32 samples x 8 B per CTA of such a batch, at
 * most one CTA per 32-sample tile).  wait() returns done = 1 and the statistics (and the latency
 * from submit to completion) when the request has finished, done = 0 when it is
 * still pending after wait_ms, or the request's error. */
typedef struct mcd_server mcd_server;
typedef struct mcd_server_options {
    int64_t memory_budget;    /* device bytes the admitted requests may hold */
    int32_t n_streams;        /* batches in flight at once, 1..16 */
    int32_t n_warps;          /* warps per CTA for every request, 1..24; 0 = per request
                                 (MCD_WARPS_BATCH_CLASS), batched by (warps, CTAs per SM) */
    int32_t max_batch;        /* requests per launch, 0 = no limit */
    int32_t compile_threads;  /* host threads compiling and uploading submitted DAGs */
} mcd_server_options;
typedef struct mcd_server_info {
    int64_t completed, batches, queued, running, bytes_in_use;
    double compile_seconds;   /* host compile time summed over requests */
    double upload_seconds;    /* allocation + upload time summed over requests */
    double launch_seconds;    /* scheduler time spent forming and launching batches */
    int64_t resident_hits;    /* requests whose DAG was already resident (no compile, no record upload) */
    int64_t resident_dags;    /* compiled DAGs resident now */
    int64_t resident_bytes;   /* their device bytes (part of bytes_in_use) */
    int64_t evicted;          /* resident DAGs evicted to make room */
} mcd_server_info;
int mcd_server_create(const mcd_server_options *opt, mcd_server **out);
void mcd_server_destroy(mcd_server *server);
int mcd_server_submit(mcd_server *server, const mcd_dag_desc *desc, const mcd_generator *gen, int64_t seed0,
                      int64_t n, int64_t *ticket);
int mcd_server_wait(mcd_server *server, int64_t ticket, double wait_ms, const mcd_stats *host, int32_t *done,
                    double *latency_ms);
int mcd_server_counters(mcd_server *server, mcd_server_info *info);

/* ---- Delay inspection ----
 * Per-class histograms of sampled delays, durations[l] - base[l] (absolute) and
 * (durations[l] - base[l]) / base[l] for base[l] != 0 (relative), over n samples:
 * the reference's demo/inspection.py:11-29 (which lists the delays of every
 * activity by type) without materialising the durations on the host.
 * link_class[l]: class of link l in 0..n_classes-1 (-1: skipped); link_base[l]: its
 * minimal duration.  ranges[c*4 .. c*4+3]: absolute lo, hi, relative lo, hi.
 * Bin of x: 0 below lo, 1 + floor((x - lo) * n_bins / (hi - lo)) inside, n_bins + 1
 * at or above hi.  counts[(c*2 + k)*(n_bins + 2) + bin] (k = 0 absolute, 1
 * relative); moments[c*6 + k*3 + {0, 1, 2}] = count, sum, sum of squares.
 * n_classes * 2 * (n_bins + 2) counters must fit 48 KB. */
int mcd_delay_histograms(mcd_dag *dag, const int64_t *seeds, int64_t n, const int32_t *link_class,
                         const double *link_base, int32_t n_classes, int32_t n_bins, const double *ranges,
                         uint64_t *counts, double *moments);

/* ---- Analytic PMF propagation ----
 * The reference's analytic engine (src/mc_dagprop/analytic/, pure Python there)
 * on the GPU: discrete PMFs on an integer step grid are propagated level by
 * level -- convolution along each incoming activity (_pmf.py:107-125), maximum
 * over predecessors by cumulative products (_pmf.py:127-148), clipping to the
 * event's bounds under the underflow/overflow rules (_propagator.py:150-265).
 * One CTA per event of a level; results stay on the device until fetched.
 *
 *   mcd_analytic_create   create_analytic_propagator (_propagator.py:48-72):
 *                         checks indices, orders the DAG, plans supports, uploads
 *   mcd_analytic_run      AnalyticPropagator.run (_propagator.py:89-148)
 *   mcd_analytic_fetch    the SimulatedEvent tuple (_context.py:29-40): per event
 *                         its PMF (first value, probabilities) and the underflow
 *                         and overflow masses
 *
 * Activity PMFs are probability arrays on the context's step grid: PMF k has
 * probabilities pmf_probs[pmf_off[k] .. pmf_off[k+1]) at values
 * pmf_first[k] + i * step.  The PMF of a predecessor entry is the one of its
 * (source, target) activity, pred_pmf[p]. */
#define MCD_RULE_TRUNCATE 1
#define MCD_RULE_REMOVE 2
#define MCD_RULE_REDISTRIBUTE 3
typedef struct mcd_analytic mcd_analytic;
typedef struct mcd_analytic_desc {
    int32_t n_events;
    const double *earliest;    /* [n_events] EventTimestamp.earliest */
    const double *latest;      /* [n_events] EventTimestamp.latest */
    int32_t n_pmfs;
    const int64_t *pmf_off;    /* [n_pmfs + 1] */
    const double *pmf_first;   /* [n_pmfs] */
    const double *pmf_probs;   /* [pmf_off[n_pmfs]] */
    int32_t n_targets;
    const int32_t *target;     /* [n_targets] */
    const int64_t *pred_off;   /* [n_targets + 1] */
    const int32_t *pred_src;   /* [pred_off[n_targets]] predecessor events, in order */
    const int32_t *pred_pmf;   /* [pred_off[n_targets]] activity PMF of each entry */
    int32_t step;              /* grid spacing, > 0 */
    double max_delay;          /* NaN: none */
    int32_t underflow_rule;    /* MCD_RULE_* */
    int32_t overflow_rule;
} mcd_analytic_desc;
int mcd_analytic_create(const mcd_analytic_desc *desc, mcd_analytic **out);
void mcd_analytic_destroy(mcd_analytic *an);
int mcd_analytic_run(mcd_analytic *an);
/* Total probability entries of the last run's results (the size of `probs` below). */
int64_t mcd_analytic_bins(const mcd_analytic *an);
/* Per event: first value, offset and length of its probabilities in `probs`,
 * underflow and overflow mass.  Any output may be NULL. */
int mcd_analytic_fetch(const mcd_analytic *an, double *first, int64_t *offset, int64_t *length, double *probs,
                       double *underflow, double *overflow);

/* ---- Pinned host memory ---- */
int mcd_host_alloc(size_t bytes, void **out);
void mcd_host_free(void *ptr);

#ifdef __cplusplus
}
#endif
#endif /* MC_DAGPROP_GB300_H */
