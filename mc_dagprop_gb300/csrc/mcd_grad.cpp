// mcd_grad.cpp -- pathwise gradient of the expected total tardiness (the adjoint).
// No counterpart in the reference; see mcd_adjoint.cu for the method.
//
// Memory.  The backward pass reads, for every event and sample, which
// predecessor won (6 bytes: position and flags, d(duration)/d(base)).  Samples run
// in chunks; within a chunk the records of every event are kept when they fit the
// memory budget ("full" plan).  Otherwise the stages are split into level blocks
// of about equal event counts: one forward pass over all stages saves the
// propagation window as each block starts (window on chip), then, from the last
// block to the first, the block's forward is recomputed from its checkpoint --
// the same Philox draws, so the same winners -- recording the block's events
// only, and the backward pass walks the block, carrying the counts of earlier
// events to the next block down.  With the window off chip the forward keeps
// every event's realized time in global rows, which serve as the checkpoint, and
// the backward's counts live in global rows too.  Gradients are integer sums, so
// every plan gives the same bits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <string>
#include <vector>

#include "mcd_handle.hpp"

namespace mcd {
cudaError_t launch_adjoint_forward(const KArgs &a, cudaStream_t st);
cudaError_t launch_adjoint_backward(const KArgs &a, cudaStream_t st);
cudaError_t launch_event_ticks(const double *earliest, int32_t E, int32_t q, long long *te, cudaStream_t st);
cudaError_t launch_adjoint_finish(const long long *grad_e, const long long *grad_l, const unsigned long long *acc,
                                  int32_t E, int32_t L, int64_t n, int32_t q, double *g_earliest, double *g_base,
                                  double *objective, cudaStream_t st);
}  // namespace mcd

using namespace mcd;

namespace {

// Samples per chunk and the level blocks (first stage of each, then n_stages).
struct AdjPlan {
    int64_t C = 32;
    std::vector<int32_t> blk;  // blk[k] .. blk[k+1]-1: the stages of block k
    int64_t eb_max = 0;        // events of the largest block
    size_t bytes = 0;          // device bytes of the per-chunk buffers
};

// Events of stage st (a stage read from global memory stores its count negated).
int64_t stage_events(const HostDag &h, int32_t st) {
    const int32_t n = h.stage_meta[(size_t)st * kStageMetaInts + 1];
    return n >= 0 ? n : -(int64_t)n;
}

// Blocks of at most `cap` events each, cut at stage boundaries (a stage larger
// than cap is a block of its own).
std::vector<int32_t> split_blocks(const HostDag &h, int64_t cap, int64_t *eb_max) {
    std::vector<int32_t> blk{0};
    int64_t cur = 0;
    *eb_max = 0;
    for (int32_t st = 0; st < h.n_stages; ++st) {
        const int64_t ne = stage_events(h, st);
        if (cur > 0 && cur + ne > cap) {
            blk.push_back(st);
            cur = 0;
        }
        cur += ne;
        *eb_max = std::max(*eb_max, cur);
    }
    blk.push_back(h.n_stages);
    return blk;
}

// Buffer bytes of a plan: records of the largest block, the window checkpoints
// and carried counts (window on chip) or the realized and count rows (off chip).
size_t plan_bytes(const HostDag &h, int64_t C, size_t n_blk, int64_t eb_max) {
    const size_t rec = (size_t)eb_max * (size_t)C * 6;
    if (!h.win_smem) return rec + (size_t)h.E * (size_t)C * 12;
    if (n_blk <= 1) return rec;
    const size_t win = (size_t)h.window_slots * (size_t)C;
    return rec + (n_blk - 1) * win * 8 + win * 4;
}

AdjPlan plan_adjoint(const HostDag &h, int64_t n, size_t budget) {
    AdjPlan p;
    // a forced block size (tests): MCD_ADJ_BLOCK_EVENTS events per block at most
    int64_t forced = 0;
    if (const char *s = std::getenv("MCD_ADJ_BLOCK_EVENTS")) forced = std::max<int64_t>(1, std::atoll(s));
    for (int64_t C = std::min<int64_t>((n + 31) / 32 * 32, 65536); C >= 32; C = C / 2 / 32 * 32) {
        std::vector<int32_t> best;
        int64_t best_eb = 0;
        size_t best_bytes = ~(size_t)0;
        if (forced) {
            best = split_blocks(h, forced, &best_eb);
            best_bytes = plan_bytes(h, C, best.size() - 1, best_eb);
        } else {
            for (int64_t nb = 1; nb <= std::max<int32_t>(h.n_stages, 1); nb = nb < 4 ? nb + 1 : nb + nb / 4) {
                int64_t eb = 0;
                std::vector<int32_t> blk = split_blocks(h, (h.E + nb - 1) / nb, &eb);
                const size_t b = plan_bytes(h, C, blk.size() - 1, eb);
                if (b < best_bytes) {
                    best_bytes = b;
                    best = std::move(blk);
                    best_eb = eb;
                }
                if (nb == 1 && b <= budget) break;  // every record fits: no recomputation
            }
        }
        if (best_bytes <= budget || C == 32) {
            p.C = C;
            p.blk = std::move(best);
            p.eb_max = best_eb;
            p.bytes = best_bytes;
            return p;
        }
    }
    return p;
}

}  // namespace

extern "C" int mcd_gradient_host(mcd_dag *g, int64_t seed0, int64_t n, double *objective, double *grad_earliest,
                                 double *grad_base) {
    return guarded([&] {
        if (!g) throw McdError(MCD_ERR_INVALID, "null handle");
        if (n <= 0 || n > (int64_t)1 << 31) throw McdError(MCD_ERR_INVALID, "need 0 < n <= 2^31 samples");
        const HostDag &h = g->h;
        if (h.max_preds > kAdjMaxPreds)
            throw McdError(MCD_ERR_INVALID, "the gradient supports at most 16383 predecessors per event");
        const StatsParams sp = stats_params(h, n);
        if (!sp.fixed) throw McdError(MCD_ERR_INVALID, "the gradient needs finite earliest times and max_delay");
        cuda_check(cudaSetDevice(g->device), "cudaSetDevice");
        cudaStream_t st = g->stream[0];
        const size_t E = (size_t)h.E, L = (size_t)std::max(h.L, 0);
        // the per-chunk buffers take at most half the free device memory, and 16 GiB
        // ($MCD_ADJ_BUDGET_MB overrides)
        size_t free_b = 0, total_b = 0;
        cuda_check(cudaMemGetInfo(&free_b, &total_b), "memory query");
        size_t budget = std::min<size_t>(free_b / 2, 16ull << 30);
        if (const char *s = std::getenv("MCD_ADJ_BUDGET_MB")) budget = (size_t)std::max(1ll, std::atoll(s)) << 20;
        const AdjPlan plan = plan_adjoint(h, n, budget);
        const int64_t C = plan.C;
        const size_t n_blk = plan.blk.size() - 1;
        const size_t tiles = (size_t)(C / 32);
        const size_t win_n = (size_t)h.window_slots * kTile;
        const bool blocks = n_blk > 1;
        const size_t s_code = align_up((size_t)plan.eb_max * (size_t)C * 2, 256),
                     s_dfac = align_up((size_t)plan.eb_max * (size_t)C * 4, 256), s_acc = align_up(E * 8, 256),
                     s_ge = align_up(E * 8, 256), s_gl = align_up(L * 8 + 8, 256),
                     s_out = align_up((E + L + 1) * 8, 256), s_te = align_up(E * 8, 256),
                     s_wck = (h.win_smem && blocks) ? align_up((n_blk - 1) * tiles * win_n * 8, 256) : 0,
                     s_cck = (h.win_smem && blocks) ? align_up(tiles * win_n * 4, 256) : 0,
                     s_rows = h.win_smem ? 0 : align_up(E * (size_t)C * 8, 256),
                     s_crow = h.win_smem ? 0 : align_up(E * (size_t)C * 4, 256),
                     s_blk = align_up(n_blk * 4 + 4, 256);
        ensure_ws(g, s_code + s_dfac + s_acc + s_ge + s_gl + s_out + s_te + s_wck + s_cck + s_rows + s_crow + s_blk);
        char *p = g->ws;
        auto take = [&p](size_t bytes) {
            char *q = p;
            p += bytes;
            return q;
        };
        auto *code = reinterpret_cast<uint16_t *>(take(s_code));
        auto *dfac = reinterpret_cast<float *>(take(s_dfac));
        char *zero_from = p;
        auto *acc = reinterpret_cast<unsigned long long *>(take(s_acc));
        auto *ge = reinterpret_cast<long long *>(take(s_ge));
        auto *gl = reinterpret_cast<long long *>(take(s_gl));
        cuda_check(cudaMemsetAsync(zero_from, 0, s_acc + s_ge + s_gl, st), "accumulator reset");
        auto *out = reinterpret_cast<double *>(take(s_out));
        auto *te = reinterpret_cast<long long *>(take(s_te));
        auto *wck = reinterpret_cast<double *>(take(s_wck));
        auto *cck = reinterpret_cast<uint32_t *>(take(s_cck));
        auto *rows = reinterpret_cast<double *>(take(s_rows));
        auto *crow = reinterpret_cast<uint32_t *>(take(s_crow));
        auto *d_blk = reinterpret_cast<int32_t *>(take(s_blk));
        if (blocks)  // the first stage of every block after the first
            cuda_check(cudaMemcpyAsync(d_blk, plan.blk.data() + 1, (n_blk - 1) * 4, cudaMemcpyHostToDevice, st),
                       "block table upload");
        cuda_check(launch_event_ticks(g->d_earliest, h.E, sp.q, te, st), "earliest ticks");
        for (int64_t off = 0; off < n; off += C) {
            KArgs a = base_args(g);
            a.seeds = nullptr;
            a.seed0 = seed0 + off;
            a.n = std::min(C, n - off);
            a.ld = C;
            a.stats_fixed = 1;
            a.tick_q = sp.q;
            a.acc = acc;
            a.te = te;
            a.grad_e = ge;
            a.grad_l = gl;
            a.adj_dfac = dfac;
            if (!h.win_smem) {
                a.scratch = rows;
                a.cnt_rows = crow;
                cuda_check(cudaMemsetAsync(crow, 0, s_crow, st), "count rows reset");
            }
            if (!blocks) {
                KArgs f = a;
                f.stage_begin = 0;
                f.stage_end = h.n_stages;
                f.adj_code = code;
                f.adj_flags = kAdjObjective;
                cuda_check(launch_adjoint_forward(f, st), "adjoint forward");
                f.adj_flags = 0;
                cuda_check(launch_adjoint_backward(f, st), "adjoint backward");
                continue;
            }
            // one forward over every stage: the objective and the blocks' checkpoints
            KArgs c = a;
            c.stage_begin = 0;
            c.stage_end = h.n_stages;
            c.adj_code = nullptr;
            c.adj_flags = kAdjObjective;
            c.blk_start = d_blk;
            c.n_blk = (int32_t)(n_blk - 1);
            c.win_ckpt = h.win_smem ? wck : nullptr;
            cuda_check(launch_adjoint_forward(c, st), "adjoint checkpoint forward");
            for (size_t k = n_blk; k-- > 0;) {  // last block first
                KArgs r = a;
                r.stage_begin = plan.blk[k];
                r.stage_end = plan.blk[k + 1];
                r.code_base = h.stage_meta[(size_t)plan.blk[k] * kStageMetaInts];  // compiled index of the block's first event
                r.adj_code = code;
                r.adj_flags = 0;
                r.win_in = (h.win_smem && k > 0) ? wck + (k - 1) * tiles * win_n : nullptr;
                cuda_check(launch_adjoint_forward(r, st), "adjoint block forward");
                r.adj_flags = (k + 1 < n_blk ? kAdjCntLoad : 0) | (k > 0 ? kAdjCntSave : 0);
                r.cnt_ckpt = cck;
                cuda_check(launch_adjoint_backward(r, st), "adjoint block backward");
            }
        }
        cuda_check(launch_adjoint_finish(ge, gl, acc, h.E, (int32_t)L, n, sp.q, out, out + E, out + E + L, st),
                   "adjoint finish");
        if (grad_earliest)
            cuda_check(cudaMemcpyAsync(grad_earliest, out, E * 8, cudaMemcpyDeviceToHost, st), "download");
        if (grad_base && L)
            cuda_check(cudaMemcpyAsync(grad_base, out + E, L * 8, cudaMemcpyDeviceToHost, st), "download");
        if (objective)
            cuda_check(cudaMemcpyAsync(objective, out + E + L, 8, cudaMemcpyDeviceToHost, st), "download");
        check_device_error(g);
        g->last_adj_plan[0] = (int64_t)C;
        g->last_adj_plan[1] = (int64_t)n_blk;
        g->last_adj_plan[2] = (int64_t)plan.bytes;
    });
}

extern "C" int mcd_gradient_plan(const mcd_dag *g, int64_t *samples_per_chunk, int64_t *level_blocks,
                                 int64_t *buffer_bytes) {
    return guarded([&] {
        if (!g) throw McdError(MCD_ERR_INVALID, "null handle");
        if (samples_per_chunk) *samples_per_chunk = g->last_adj_plan[0];
        if (level_blocks) *level_blocks = g->last_adj_plan[1];
        if (buffer_bytes) *buffer_bytes = g->last_adj_plan[2];
    });
}
