/*
 * mcd_oracle.c -- CPU restatement of the reference Monte Carlo path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle for the CUDA path and the timed CPU
 * baseline.  Never linked into the product library.  Every function cites the
 * reference file:line it follows (paths inside the reference project).
 *
 * Third-party arithmetic restated here (absent from the reference tree):
 * libstdc++ <random> as shipped with GCC 13 -- generate_canonical<double,53>,
 * exponential_distribution, gamma_distribution (Marsaglia & Tsang 2000, with the
 * alpha<1 boost U^(1/alpha)), normal_distribution (Marsaglia polar method with one
 * cached value) and discrete_distribution (normalised cumulative table searched
 * with lower_bound).  Parity of this file is pinned bit-for-bit against the
 * reference compiled from source (oracle/build_ref.sh) by tests/test_oracle_pin.py.
 *
 * Build: gcc -O2 -ffp-contract=off -shared -fPIC (no FMA contraction, so the
 * operation sequence is the one written here).
 */
#include "mcd_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ---------------- Engine: SplitMix64 seeding + Xoshiro256++ ----------------
 * _custom_rng.hpp:530-536 (SplitMix64::operator()), :570-576 (seed: four
 * SplitMix64 outputs), :589-599 (Xoshiro256++ step).  Algorithms by Vigna and
 * Blackman & Vigna (prng.di.unimi.it). */
typedef struct { uint64_t s[4]; } xo256;

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static void xo_seed(xo256 *g, uint64_t seed) {
    uint64_t sm = seed;
    for (int i = 0; i < 4; ++i) {
        uint64_t z = (sm += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        g->s[i] = z ^ (z >> 31);
    }
}

static inline uint64_t xo_next(xo256 *g) {
    uint64_t *s = g->s;
    const uint64_t out = rotl64(s[0] + s[3], 23) + s[0];
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return out;
}

/* generate_canonical<double, 53> over a 64-bit engine: one draw, u / 2^64,
 * pulled below 1.0 when rounding reaches it. */
static inline double canonical(xo256 *g) {
    double r = (double)xo_next(g) / 18446744073709551616.0;
    if (r >= 1.0) r = nextafter(1.0, 0.0);
    return r;
}

/* ---------------- Distributions (_core.cpp:71-141) ---------------- */
typedef struct {
    int32_t type;
    int32_t kind;
    double factor;                 /* constant */
    double exp_rate, max_scale;    /* exponential: rate = 1/lambda_ (_core.cpp:81) */
    double g_alpha, g_beta, g_malpha, g_a1, g_a2; /* gamma parameters */
    int normal_saved_available;    /* gamma's normal_distribution cache */
    double normal_saved;
    int64_t n;                     /* empirical */
    double *values;                /* values / factors */
    double *cp;                    /* cumulative probabilities, empty when n < 2 */
} orc_dist;

/* normal_distribution<double>(0,1)::operator(): polar method, second value cached. */
static double dist_normal(orc_dist *d, xo256 *g) {
    double ret;
    if (d->normal_saved_available) {
        d->normal_saved_available = 0;
        ret = d->normal_saved;
    } else {
        double x, y, r2;
        do {
            x = 2.0 * canonical(g) - 1.0;
            y = 2.0 * canonical(g) - 1.0;
            r2 = x * x + y * y;
        } while (r2 > 1.0 || r2 == 0.0);
        const double mult = sqrt(-2 * log(r2) / r2);
        d->normal_saved = x * mult;
        d->normal_saved_available = 1;
        ret = y * mult;
    }
    return ret * 1.0 + 0.0; /* stddev 1, mean 0 */
}

/* gamma_distribution<double>(alpha, beta)::operator() (Marsaglia-Tsang). */
static double dist_gamma_raw(orc_dist *d, xo256 *g) {
    double u, v, n;
    const double a1 = d->g_a1;
    do {
        do {
            n = dist_normal(d, g);
            v = 1.0 + d->g_a2 * n;
        } while (v <= 0.0);
        v = v * v * v;
        u = canonical(g);
    } while (u > 1.0 - 0.0331 * n * n * n * n && log(u) > (0.5 * n * n + a1 * (1.0 - v + log(v))));
    if (d->g_alpha == d->g_malpha) return a1 * v * d->g_beta;
    do {
        u = canonical(g);
    } while (u == 0.0);
    return pow(u, 1.0 / d->g_alpha) * a1 * v * d->g_beta;
}

/* discrete_distribution<size_t>::operator(): no draw when the table has < 2 entries. */
static int64_t dist_discrete(const orc_dist *d, xo256 *g) {
    if (d->n < 2) return 0;
    const double p = canonical(g);
    int64_t lo = 0, hi = d->n; /* lower_bound: first cp[i] >= p */
    while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (d->cp[mid] < p) lo = mid + 1; else hi = mid;
    }
    return lo;
}

/* DistVar::sample(rng, d): the EXTRA delay, added to the base by the caller. */
static double dist_sample(orc_dist *d, xo256 *g, double dur) {
    switch (d->kind) {
    case ORC_CONSTANT:
        return dur * d->factor;                              /* _core.cpp:75 */
    case ORC_EXPONENTIAL: {                                  /* _core.cpp:83-89 */
        double x;
        do {
            x = -log(1.0 - canonical(g)) / d->exp_rate;
        } while (x > d->max_scale);
        return x * dur;
    }
    case ORC_GAMMA: {                                        /* _core.cpp:98-104 */
        double x;
        do {
            x = dist_gamma_raw(d, g);
        } while (x > d->max_scale);
        return x * dur;
    }
    case ORC_EMP_ABS:                                        /* _core.cpp:125 */
        return d->values[dist_discrete(d, g)];
    case ORC_EMP_REL:                                        /* _core.cpp:140 */
        return d->values[dist_discrete(d, g)] * dur;
    }
    return 0.0;
}

static int dist_init(orc_dist *d, const orc_dist_desc *s, char *err, size_t errlen) {
    memset(d, 0, sizeof(*d));
    d->type = s->activity_type;
    d->kind = s->kind;
    switch (s->kind) {
    case ORC_CONSTANT: d->factor = s->p0; break;
    case ORC_EXPONENTIAL: d->exp_rate = 1.0 / s->p0; d->max_scale = s->p1; break;
    case ORC_GAMMA:
        d->g_alpha = s->p0;
        d->g_beta = s->p1;
        d->max_scale = s->p2;
        d->g_malpha = d->g_alpha < 1.0 ? d->g_alpha + 1.0 : d->g_alpha;
        d->g_a1 = d->g_malpha - 1.0 / 3.0;
        d->g_a2 = 1.0 / sqrt(9.0 * d->g_a1);
        break;
    case ORC_EMP_ABS:
    case ORC_EMP_REL: {
        d->n = s->n_table;
        d->values = (double *)malloc(sizeof(double) * (size_t)(d->n > 0 ? d->n : 1));
        d->cp = (double *)malloc(sizeof(double) * (size_t)(d->n > 0 ? d->n : 1));
        if (!d->values || !d->cp) { snprintf(err, errlen, "out of memory"); return -1; }
        for (int64_t i = 0; i < d->n; ++i) d->values[i] = s->values[i];
        if (d->n >= 2) {
            double sum = 0.0;
            for (int64_t i = 0; i < d->n; ++i) sum += s->weights[i];
            double acc = 0.0;
            for (int64_t i = 0; i < d->n; ++i) {
                acc += s->weights[i] / sum;
                d->cp[i] = acc;
            }
            d->cp[d->n - 1] = 1.0;
        }
        break;
    }
    default: snprintf(err, errlen, "unknown distribution kind %d", s->kind); return -1;
    }
    return 0;
}

static void dist_copy(orc_dist *dst, const orc_dist *src) {
    *dst = *src;
    dst->normal_saved_available = 0;
    dst->normal_saved = 0.0;
    if (src->kind == ORC_EMP_ABS || src->kind == ORC_EMP_REL) {
        size_t nb = sizeof(double) * (size_t)(src->n > 0 ? src->n : 1);
        dst->values = (double *)malloc(nb);
        dst->cp = (double *)malloc(nb);
        memcpy(dst->values, src->values, nb);
        memcpy(dst->cp, src->cp, nb);
    }
}

/* ---------------- Compiled simulator (_core.cpp:161-307) ---------------- */
struct orc_sim {
    int32_t E, L;
    double *earliest;      /* [E] */
    double max_delay;
    int32_t n_dist;
    orc_dist *dists;
    double *base;          /* [L] Activity.duration per link (gaps: 0) */
    int32_t *link_dist;    /* [L] distribution index, -1 = no delay */
    int64_t *pred_off;     /* [E+1] CSR by event */
    int32_t *pred_src, *pred_edge;
    int32_t *order;        /* [E] Kahn FIFO order */
    /* scratch (_core.cpp:186-190) */
    double *dur, *real;
    int32_t *cause;
    xo256 rng;
};

void orc_sim_destroy(orc_sim *s) {
    if (!s) return;
    for (int32_t i = 0; i < s->n_dist; ++i) { free(s->dists[i].values); free(s->dists[i].cp); }
    free(s->dists); free(s->earliest); free(s->base); free(s->link_dist);
    free(s->pred_off); free(s->pred_src); free(s->pred_edge); free(s->order);
    free(s->dur); free(s->real); free(s->cause);
    free(s);
}

int orc_sim_create(const orc_dag_desc *dag, const orc_dist_desc *dists, int32_t n_dists,
                   orc_sim **out, char *err, size_t errlen) {
    *out = NULL;
    /* Distinct types, later add_* for the same type replacing the earlier one. */
    int32_t *keep = (int32_t *)calloc((size_t)(n_dists > 0 ? n_dists : 1), sizeof(int32_t));
    for (int32_t i = 0; i < n_dists; ++i) {
        keep[i] = 1;
        for (int32_t j = i + 1; j < n_dists; ++j)
            if (dists[j].activity_type == dists[i].activity_type) { keep[i] = 0; break; }
    }
    for (int32_t i = 0; i < n_dists; ++i)
        if (keep[i] && dists[i].activity_type == -1) {            /* _core.cpp:196-198 */
            snprintf(err, errlen, "Activity type -1 is reserved for no delay");
            free(keep);
            return -1;
        }
    if (dag->max_delay < 0.0) {                                    /* _core.cpp:199-201 */
        snprintf(err, errlen, "max_delay must be non-negative");
        free(keep);
        return -1;
    }
    orc_sim *s = (orc_sim *)calloc(1, sizeof(orc_sim));
    s->E = dag->n_events;
    s->max_delay = dag->max_delay;
    s->dists = (orc_dist *)calloc((size_t)(n_dists > 0 ? n_dists : 1), sizeof(orc_dist));
    for (int32_t i = 0; i < n_dists; ++i) {
        if (!keep[i]) continue;
        if (dist_init(&s->dists[s->n_dist], &dists[i], err, errlen) != 0) { free(keep); orc_sim_destroy(s); return -1; }
        s->n_dist++;
    }
    free(keep);

    /* Dense links, link_count = max idx + 1, gaps {idx -1, 0 s, type -1} (_core.cpp:213-229). */
    int32_t max_idx = -1;
    for (int32_t k = 0; k < dag->n_activities; ++k)
        if (dag->act_idx[k] > max_idx) max_idx = dag->act_idx[k];
    s->L = max_idx + 1;
    size_t L = (size_t)(s->L > 0 ? s->L : 1);
    s->base = (double *)calloc(L, sizeof(double));
    s->link_dist = (int32_t *)malloc(L * sizeof(int32_t));
    for (size_t l = 0; l < L; ++l) s->link_dist[l] = -1;
    for (int32_t k = 0; k < dag->n_activities; ++k) {
        int32_t l = dag->act_idx[k];
        if (l < 0) { snprintf(err, errlen, "activity idx must be non-negative"); orc_sim_destroy(s); return -1; }
        s->base[l] = dag->act_duration[k];
        s->link_dist[l] = -1;
        for (int32_t d = 0; d < s->n_dist; ++d)
            if (s->dists[d].type == dag->act_type[k]) { s->link_dist[l] = d; break; }
    }

    /* Adjacency, indegrees, Kahn FIFO (_core.cpp:235-264).  A later entry for the
     * same target replaces the predecessor list and indegree of the earlier one;
     * adjacency keeps every entry's edges, as in the reference. */
    const int32_t E = s->E;
    size_t Ez = (size_t)(E > 0 ? E : 1);
    int64_t *pb_start = (int64_t *)malloc(Ez * sizeof(int64_t));
    int64_t *pb_len = (int64_t *)calloc(Ez, sizeof(int64_t));
    int64_t *indeg = (int64_t *)calloc(Ez, sizeof(int64_t));
    int64_t *adj_cnt = (int64_t *)calloc(Ez + 1, sizeof(int64_t));
    for (int32_t t = 0; t < dag->n_targets; ++t) {
        int32_t tgt = dag->target[t];
        if (tgt < 0 || tgt >= E) { snprintf(err, errlen, "precedence target %d out of range", tgt); goto fail_kahn; }
        pb_start[tgt] = dag->pred_offsets[t];
        pb_len[tgt] = dag->pred_offsets[t + 1] - dag->pred_offsets[t];
        indeg[tgt] = pb_len[tgt];
        for (int64_t p = dag->pred_offsets[t]; p < dag->pred_offsets[t + 1]; ++p) {
            int32_t src = dag->pred_src[p];
            if (src < 0 || src >= E) { snprintf(err, errlen, "predecessor %d out of range", src); goto fail_kahn; }
            int32_t a = dag->pred_act[p];
            /* An index past the last link reads beyond the reference's duration
             * buffer (UB there; in practice it reads 0.0, and its chain test
             * test_simulator.py:175-199 relies on that): such an edge has duration 0. */
            if (a < 0) { snprintf(err, errlen, "activity index %d out of range", a); goto fail_kahn; }
            adj_cnt[src + 1]++;
        }
    }
    for (int32_t i = 0; i < E; ++i) adj_cnt[i + 1] += adj_cnt[i];
    {
        int64_t n_adj = adj_cnt[E];
        int32_t *adj = (int32_t *)malloc((size_t)(n_adj > 0 ? n_adj : 1) * sizeof(int32_t));
        int64_t *fill = (int64_t *)malloc(Ez * sizeof(int64_t));
        for (int32_t i = 0; i < E; ++i) fill[i] = adj_cnt[i];
        for (int32_t t = 0; t < dag->n_targets; ++t)
            for (int64_t p = dag->pred_offsets[t]; p < dag->pred_offsets[t + 1]; ++p)
                adj[fill[dag->pred_src[p]]++] = dag->target[t];
        free(fill);
        s->order = (int32_t *)malloc(Ez * sizeof(int32_t));
        int32_t *queue = (int32_t *)malloc((Ez + 1) * sizeof(int32_t));
        int64_t qh = 0, qt = 0, n_order = 0;
        for (int32_t i = 0; i < E; ++i) if (indeg[i] == 0) queue[qt++] = i;
        while (qh < qt) {
            int32_t nd = queue[qh++];
            s->order[n_order++] = nd;
            for (int64_t k = adj_cnt[nd]; k < adj_cnt[nd + 1]; ++k) {
                int32_t dst = adj[k];
                if (--indeg[dst] == 0) {
                    if (qt >= E) break; /* cannot happen for well-formed input */
                    queue[qt++] = dst;
                }
            }
        }
        free(queue);
        free(adj);
        if (n_order != E) {
            snprintf(err, errlen, "Invalid DAG: cycle detected in precedence list");
            goto fail_kahn;
        }
    }
    /* Predecessor CSR by event, list order kept (_core.cpp:267-285). */
    s->pred_off = (int64_t *)calloc(Ez + 1, sizeof(int64_t));
    for (int32_t i = 0; i < E; ++i) s->pred_off[i + 1] = s->pred_off[i] + pb_len[i];
    {
        int64_t P = s->pred_off[E];
        s->pred_src = (int32_t *)malloc((size_t)(P > 0 ? P : 1) * sizeof(int32_t));
        s->pred_edge = (int32_t *)malloc((size_t)(P > 0 ? P : 1) * sizeof(int32_t));
        for (int32_t i = 0; i < E; ++i)
            for (int64_t k = 0; k < pb_len[i]; ++k) {
                s->pred_src[s->pred_off[i] + k] = dag->pred_src[pb_start[i] + k];
                s->pred_edge[s->pred_off[i] + k] = dag->pred_act[pb_start[i] + k];
            }
    }
    free(pb_start); free(pb_len); free(indeg); free(adj_cnt);

    s->earliest = (double *)malloc(Ez * sizeof(double));
    for (int32_t i = 0; i < E; ++i) s->earliest[i] = dag->earliest[i];
    s->dur = (double *)malloc(L * sizeof(double));
    s->real = (double *)malloc(Ez * sizeof(double));
    s->cause = (int32_t *)malloc(Ez * sizeof(int32_t));
    for (int32_t l = 0; l < s->L; ++l) s->dur[l] = s->link_dist[l] < 0 ? s->base[l] : 0.0; /* :303-306 */
    xo_seed(&s->rng, 0);
    *out = s;
    return 0;
fail_kahn:
    free(pb_start); free(pb_len); free(indeg); free(adj_cnt);
    orc_sim_destroy(s);
    return -1;
}

int32_t orc_node_count(const orc_sim *s) { return s->E; }
int32_t orc_activity_count(const orc_sim *s) { return s->L; }

int orc_eval_order(const orc_sim *s, int32_t *o) {
    memcpy(o, s->order, sizeof(int32_t) * (size_t)s->E);
    return 0;
}

/* The propagation loop (_core.cpp:318-350) over one sample. */
static void propagate_one(const orc_sim *s, const double *dur, double *real, int32_t *cause) {
    for (int32_t i = 0; i < s->E; ++i) real[i] = s->earliest[i];
    for (int32_t k = 0; k < s->E; ++k) {
        const int32_t e = s->order[k];
        const double earliest = s->earliest[e];
        const double ub = earliest + s->max_delay;
        double latest = real[e];
        int32_t c = -1;
        for (int64_t p = s->pred_off[e]; p < s->pred_off[e + 1]; ++p) {
            const int32_t src = s->pred_src[p];
            const int32_t edge = s->pred_edge[p];
            double t = real[src] + (edge < s->L ? dur[edge] : 0.0);
            t = (ub < t) ? ub : t;                    /* std::min(t, ub) */
            if (t >= latest) { latest = t; c = src; }
        }
        real[e] = (ub < latest) ? ub : latest;        /* std::min(latest, ub) */
        cause[e] = c;
    }
}

/* Simulator::run (_core.cpp:312-353) for one seed. */
static void run_one(orc_sim *s, int64_t seed) {
    xo_seed(&s->rng, (uint64_t)seed);
    for (int32_t l = 0; l < s->L; ++l) {
        const int32_t d = s->link_dist[l];
        if (d < 0) continue;
        const double b = s->base[l];
        const double extra = dist_sample(&s->dists[d], &s->rng, b);
        s->dur[l] = b + extra;
    }
    propagate_one(s, s->dur, s->real, s->cause);
}

int orc_run_many(orc_sim *s, const int64_t *seeds, int64_t n, double *realized, double *durations,
                 int32_t *cause) {
    const size_t E = (size_t)s->E, L = (size_t)s->L;
    for (int64_t i = 0; i < n; ++i) {
        run_one(s, seeds[i]);
        if (realized) memcpy(realized + (size_t)i * E, s->real, E * sizeof(double));
        if (durations) memcpy(durations + (size_t)i * L, s->dur, L * sizeof(double));
        if (cause) memcpy(cause + (size_t)i * E, s->cause, E * sizeof(int32_t));
    }
    return 0;
}

static orc_sim *sim_clone(const orc_sim *p) {
    orc_sim *s = (orc_sim *)calloc(1, sizeof(orc_sim));
    *s = *p;
    const size_t E = (size_t)(p->E > 0 ? p->E : 1), L = (size_t)(p->L > 0 ? p->L : 1);
    const size_t P = (size_t)(p->pred_off[p->E] > 0 ? p->pred_off[p->E] : 1);
#define DUP(field, cnt) do { s->field = malloc(sizeof(*p->field) * (cnt)); memcpy(s->field, p->field, sizeof(*p->field) * (cnt)); } while (0)
    DUP(earliest, E); DUP(base, L); DUP(link_dist, L); DUP(pred_off, E + 1);
    DUP(pred_src, P); DUP(pred_edge, P); DUP(order, E); DUP(dur, L); DUP(real, E); DUP(cause, E);
#undef DUP
    s->dists = (orc_dist *)calloc((size_t)(p->n_dist > 0 ? p->n_dist : 1), sizeof(orc_dist));
    for (int32_t i = 0; i < p->n_dist; ++i) dist_copy(&s->dists[i], &p->dists[i]);
    return s;
}

typedef struct {
    const orc_sim *proto;
    const int64_t *seeds;
    int64_t lo, hi;
    double *realized, *durations;
    int32_t *cause;
} mt_job;

static void *mt_worker(void *arg) {
    mt_job *j = (mt_job *)arg;
    orc_sim *s = sim_clone(j->proto);
    const size_t E = (size_t)s->E, L = (size_t)s->L;
    orc_run_many(s, j->seeds + j->lo, j->hi - j->lo,
                 j->realized ? j->realized + (size_t)j->lo * E : NULL,
                 j->durations ? j->durations + (size_t)j->lo * L : NULL,
                 j->cause ? j->cause + (size_t)j->lo * E : NULL);
    orc_sim_destroy(s);
    return NULL;
}

int orc_run_many_mt(const orc_sim *proto, const int64_t *seeds, int64_t n, int32_t n_threads,
                    double *realized, double *durations, int32_t *cause) {
    if (n_threads < 1) n_threads = 1;
    if (n_threads > n) n_threads = (int32_t)(n > 0 ? n : 1);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)n_threads);
    mt_job *jobs = (mt_job *)malloc(sizeof(mt_job) * (size_t)n_threads);
    for (int32_t t = 0; t < n_threads; ++t) {
        jobs[t].proto = proto;
        jobs[t].seeds = seeds;
        jobs[t].lo = n * t / n_threads;
        jobs[t].hi = n * (t + 1) / n_threads;
        jobs[t].realized = realized;
        jobs[t].durations = durations;
        jobs[t].cause = cause;
        pthread_create(&th[t], NULL, mt_worker, &jobs[t]);
    }
    for (int32_t t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
    free(th);
    free(jobs);
    return 0;
}

int orc_propagate_given(const orc_sim *s, const double *durations, int64_t n, double *realized,
                        int32_t *cause) {
    const size_t E = (size_t)s->E, L = (size_t)s->L;
    double *real = (double *)malloc(sizeof(double) * (E > 0 ? E : 1));
    int32_t *c = (int32_t *)malloc(sizeof(int32_t) * (E > 0 ? E : 1));
    for (int64_t i = 0; i < n; ++i) {
        propagate_one(s, durations + (size_t)i * L, real, c);
        if (realized) memcpy(realized + (size_t)i * E, real, E * sizeof(double));
        if (cause) memcpy(cause + (size_t)i * E, c, E * sizeof(int32_t));
    }
    free(real);
    free(c);
    return 0;
}
