// mcd_host.hpp -- host-side types of the engine (generator, compiled DAG, errors).
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mc_dagprop_gb300.h"
#include "mcd_internal.hpp"

// Distribution kinds as the generator records them (one per add_* method).
enum : int32_t {
    MCD_KIND_CONSTANT = 0,
    MCD_KIND_EXPONENTIAL = 1,
    MCD_KIND_GAMMA = 2,
    MCD_KIND_EMP_ABS = 3,
    MCD_KIND_EMP_REL = 4,
};

struct DistSpec {
    int32_t type;
    int32_t kind;
    double p0, p1, p2;
    std::vector<double> values, weights;
};

// GenericDelayGenerator (_core.cpp:146-159): the add_* calls in order; the
// compiler keeps the last one per activity type.
struct mcd_generator {
    int64_t seed = 0;
    std::vector<DistSpec> dists;
};

namespace mcd {

struct McdError : std::runtime_error {
    int code;
    McdError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// Shared memory: the propagation window may take up to kMaxWindowBytes; each of
// the two record staging buffers up to kMaxStageBytes; the whole CTA kSmemMax.
constexpr size_t kMaxWindowBytes = 196 * 1024;
constexpr int32_t kMaxWarps = 24;       // single-DAG kernel: 768 threads per CTA
constexpr int32_t kMaxBatchWarps = 24;  // persistent batch kernel: 768 threads per CTA
// n_warps request: automatic, rounded up to 2, 4, 8, 12 or 24 warps -- block
// sizes whose CTAs fill an SM's 24 warps at the batch kernel's 80 registers
constexpr int32_t kBatchClassWarps = -1;
constexpr size_t kMaxStageBytes = 40 * 1024;
constexpr size_t kMinStageBytes = 4 * 1024;
constexpr size_t kMaxTableBytes = 16 * 1024;
constexpr size_t kSmemMax = 226 * 1024;  // 227 KB per CTA, less room for static shared data

// Output of compile_dag: everything the kernels need, host copies.
struct HostDag {
    int32_t E = 0, L = 0, n_levels = 0, n_warps = 1, window_slots = 0;
    bool win_smem = true;
    bool positive = false;        // all times non-negative and finite
    int64_t max_preds = 0;        // largest predecessor list
    bool tables_in_smem = true;
    int32_t n_stages = 0, stage_bytes = 0;
    int32_t smem_stage_off = 0, smem_tables_off = 0, smem_bar_off = 0, smem_total = 0;
    std::vector<int32_t> stage_meta;  // kStageMetaInts ints per stage (KArgs::stage_meta)
    std::vector<EvRec> ev;
    std::vector<PredRec> pred;
    std::vector<LinkRec> aux;  // links stored by the aux pass
    int32_t n_orphan = 0;      // sampled links no precedence entry references
    int32_t n_pairs = 0;       // event pairs over all stages (KArgs::stage_meta)
    int64_t block_draws = 0;   // Philox blocks a sample draws on first attempts
    std::vector<DistParam> dist;
    std::vector<AliasEntry> alias;
    std::vector<AliasPick> picks;  // parallel to alias
    std::vector<double> vals;      // per-link duration tables, stage by stage
    std::vector<int32_t> wk_off;
    std::vector<int32_t> link_kd;
    std::vector<double> link_v;
    std::vector<float> link_dv;    // FIXED links: d(duration)/d(base)
    std::vector<int32_t> link_block;  // Philox block of each link's random words (-1: fixed)
    std::vector<int8_t> link_word;    // word of a one-word link in its block; -1: the link owns the block
    std::vector<double> earliest;  // caller order
    std::vector<double> ub;        // earliest + max_delay, caller order
    double max_delay = 0.0;
    // statistics: all times finite -> exact integer-tick accumulation is possible
    bool times_finite = true;
    double max_abs_time = 0.0;  // max |earliest|, |ub|
    double max_span = 0.0;      // max (ub - earliest)
};

// Per-call parameters of the statistics mode (depend on the sample count).
struct StatsParams {
    int32_t fixed = 0;
    int32_t q = 0;
    unsigned long long bin_mul = 0;
    double inv_w = 0.0;
    double bin_w = 0.0;  // seconds per bin
};
StatsParams stats_params(const HostDag &h, int64_t n);

// The tables block as the kernels read it (KArgs::dist): DistParam[n_dist],
// AliasEntry[n_alias], AliasPick[n_alias], back to back.
size_t tables_bytes(const HostDag &h);
std::vector<unsigned char> tables_block(const HostDag &h);

// n_warps: warps per CTA the kernels will run with (0: chosen from the DAG's width);
// window: MCD_WINDOW_AUTO (shared memory when it fits) or MCD_WINDOW_GLOBAL.
void compile_dag(const mcd_dag_desc &d, const mcd_generator &g, HostDag &out, int32_t n_warps,
                 int32_t window = MCD_WINDOW_AUTO);

// The content key of a compiled DAG: everything compile_dag reads, serialized
// (the arrays, the generator, warps per CTA, device, the compiler's environment
// overrides); false where the arrays are too malformed to read safely.  Caches
// of compiled DAGs pick a bucket by hash_bytes and decide by full comparison.
bool image_key(const mcd_dag_desc &d, const mcd_generator &gen, int32_t n_warps, int device,
               std::vector<unsigned char> &k, int32_t window = MCD_WINDOW_AUTO);
uint64_t hash_bytes(const std::vector<unsigned char> &k);
int64_t order_key_host(int64_t bits);

}  // namespace mcd
