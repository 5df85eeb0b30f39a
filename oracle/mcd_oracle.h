/*
 * mcd_oracle.h -- CPU restatement of the reference Monte Carlo path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA path is compared
 * against, and the timed CPU baseline.  The product library never links it.
 *
 * It restates, in plain C, what the reference computes in
 * src/mc_dagprop/monte_carlo/_core.cpp:
 *   - Simulator::Simulator (_core.cpp:193-307): validation, dense activity array,
 *     Kahn FIFO topological order, predecessor CSR in precedence-list order;
 *   - Simulator::run (_core.cpp:312-353): reseed, per-link sampling in index
 *     order from one sequential stream, FP64 propagation with the max_delay clamp;
 *   - the five delay distributions (_core.cpp:71-141) with the arithmetic of
 *     libstdc++ <random> (GCC 13: generate_canonical, exponential_distribution,
 *     gamma_distribution with its normal_distribution, discrete_distribution);
 *   - the vendored Xoshiro256++ / SplitMix64 engine (_custom_rng.hpp:507-600).
 */
#ifndef MCD_ORACLE_H
#define MCD_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Distribution kinds (one per GenericDelayGenerator.add_* method). */
enum { ORC_CONSTANT = 0, ORC_EXPONENTIAL = 1, ORC_GAMMA = 2, ORC_EMP_ABS = 3, ORC_EMP_REL = 4 };

typedef struct {
    int32_t activity_type;
    int32_t kind;
    double p0, p1, p2;        /* constant: factor | exponential: lambda_, max_scale |
                                 gamma: shape, scale, max_scale */
    int64_t n_table;          /* empirical: number of (value, weight) pairs */
    const double *values;     /* empirical absolute values / relative factors */
    const double *weights;
} orc_dist_desc;

/* DagContext flattened to arrays (the activity map's key is not used by the path). */
typedef struct {
    int32_t n_events;
    const double *earliest;   /* [n_events] EventTimestamp.earliest */
    int32_t n_activities;     /* entries in the activity map */
    const int32_t *act_idx;   /* Activity.idx */
    const double *act_duration; /* Activity.minimal_duration */
    const int32_t *act_type;  /* Activity.activity_type */
    int32_t n_targets;        /* entries in precedence_list */
    const int32_t *target;    /* [n_targets] */
    const int64_t *pred_offsets; /* [n_targets+1] */
    const int32_t *pred_src;  /* predecessor event */
    const int32_t *pred_act;  /* link (activity index) */
    double max_delay;
} orc_dag_desc;

typedef struct orc_sim orc_sim;

/* Returns 0 on success; otherwise writes a message (the reference's RuntimeError
 * text where it has one) into err. */
int orc_sim_create(const orc_dag_desc *dag, const orc_dist_desc *dists, int32_t n_dists,
                   orc_sim **out, char *err, size_t errlen);
void orc_sim_destroy(orc_sim *sim);
int32_t orc_node_count(const orc_sim *sim);
int32_t orc_activity_count(const orc_sim *sim);

/* Sequential run_many on one simulator (distribution state carries across runs,
 * as in the reference).  Outputs are sample-major: realized[s*E+e],
 * durations[s*L+l], cause[s*E+e].  Any output may be NULL. */
int orc_run_many(orc_sim *sim, const int64_t *seeds, int64_t n,
                 double *realized, double *durations, int32_t *cause);

/* run_many over n_threads fresh copies of the simulator, each taking one
 * contiguous chunk of seeds (the reference's one-propagator-per-thread pattern). */
int orc_run_many_mt(const orc_sim *proto, const int64_t *seeds, int64_t n, int32_t n_threads,
                    double *realized, double *durations, int32_t *cause);

/* The propagation loop alone, given durations[s*L+l] (sample-major). */
int orc_propagate_given(const orc_sim *sim, const double *durations, int64_t n,
                        double *realized, int32_t *cause);

/* Kahn order computed by the compiler (for tests). */
int orc_eval_order(const orc_sim *sim, int32_t *order_out);

#ifdef __cplusplus
}
#endif
#endif
