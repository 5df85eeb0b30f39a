// mcd_batch.cpp -- many DAGs, each with its own samples, in one persistent launch.
//
// The work is a queue of (DAG, 32-sample tile) items, most expensive DAG first
// (longest-processing-time order), consumed by a persistent grid of CTAs that
// fills every SM whatever the DAGs' sizes -- a plain per-DAG launch of a DAG
// with 1,000 samples keeps 32 CTAs busy and leaves the rest of the GPU idle.
// DAGs are grouped by kernel variant (window on chip or not, tables in shared
// memory or not, positive times or not); each group is one launch with its own
// queue.  Each run is one CUDA
// graph: reset the accumulators and the queue heads, the persistent statistics
// launches, the batched finish.  The graph is recorded on the first run and
// replayed afterwards.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>

#include "mcd_host.hpp"
#include "mcd_handle.hpp"

namespace mcd {
cudaError_t launch_batch_stats(const BatchArgs &b, bool win_smem, bool positive, bool tsmem, int n_warps, size_t smem,
                               int grid,
                               cudaStream_t st);
cudaError_t batch_blocks_per_sm(bool win_smem, bool positive, bool tsmem, int n_warps, size_t smem, int *out);
cudaError_t launch_batch_finish(const FArgs *fs, int32_t n_dags, int32_t max_events, cudaStream_t st);
}  // namespace mcd

using namespace mcd;

namespace {
// One persistent launch: the DAGs of one kernel variant.
struct Launch {
    bool win_smem = true, positive = true, tsmem = true;
    std::vector<int32_t> dags;
    size_t smem = 0;
    int grid = 1;
    BatchArgs args{};
};
}  // namespace

struct mcd_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<mcd_dag *> dags;
    std::vector<int64_t> n, ev_off;
    int n_warps = 1, grid = 1;
    int32_t max_E = 0;
    int64_t total_E = 0, n_items = 0;
    char *dmem = nullptr;
    size_t zero_bytes = 0;  // accumulators + queue heads, cleared every run
    double *out = nullptr;  // [5][total_E]: mean, p50, p90, p99, p_on_time
    uint32_t *hist = nullptr;
    FArgs *d_fargs = nullptr;
    std::vector<Launch> launches;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" {

int mcd_batch_create(mcd_dag *const *dags, int32_t n_dags, const int64_t *seed0, const int64_t *n_samples,
                     mcd_batch **out) {
    mcd_batch *B = nullptr;
    int rc = guarded([&] {
        if (!dags || !seed0 || !n_samples || !out || n_dags <= 0) throw McdError(MCD_ERR_INVALID, "bad arguments");
        *out = nullptr;
        B = new mcd_batch();
        B->device = dags[0]->device;
        B->n_warps = dags[0]->h.n_warps;
        if (B->n_warps > kMaxBatchWarps)
            throw McdError(MCD_ERR_INVALID, "DAGs of a batch must be compiled with n_warps <= 24");
        for (int32_t i = 0; i < n_dags; ++i) {
            const mcd_dag *g = dags[i];
            if (!g) throw McdError(MCD_ERR_INVALID, "null DAG handle");
            if (g->device != B->device) throw McdError(MCD_ERR_INVALID, "DAGs of a batch must share a device");
            if (g->h.n_warps != B->n_warps)
                throw McdError(MCD_ERR_INVALID, "DAGs of a batch must be compiled with the same n_warps");
            if (n_samples[i] <= 0 || n_samples[i] > (int64_t)1 << 31)
                throw McdError(MCD_ERR_INVALID, "each DAG needs 0 < n <= 2^31 samples");
            B->dags.push_back(const_cast<mcd_dag *>(g));
            B->n.push_back(n_samples[i]);
        }
        cuda_check(cudaSetDevice(B->device), "cudaSetDevice");
        cuda_check(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking), "stream create");
        // layout of the batch's device memory; launches by kernel variant
        B->ev_off.resize((size_t)n_dags + 1, 0);
        for (int32_t i = 0; i < n_dags; ++i) {
            const HostDag &h = B->dags[i]->h;
            B->max_E = std::max(B->max_E, h.E);
            B->ev_off[i + 1] = B->ev_off[i] + h.E;
            Launch *L = nullptr;
            for (Launch &x : B->launches)
                if (x.win_smem == h.win_smem && x.positive == h.positive && x.tsmem == h.tables_in_smem) L = &x;
            if (!L) {
                B->launches.emplace_back();
                L = &B->launches.back();
                L->win_smem = h.win_smem;
                L->positive = h.positive;
                L->tsmem = h.tables_in_smem;
            }
            L->dags.push_back(i);
            L->smem = std::max(L->smem, (size_t)h.smem_total);
        }
        B->total_E = B->ev_off[n_dags];
        int sms = 0;
        cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, B->device), "SM count");
        // items: within each launch, DAGs by cost per tile, most expensive first; every tile of a DAG
        auto cost = [&](int32_t i) { return (double)B->dags[i]->h.pred.size() + 2.0 * B->dags[i]->h.E; };
        std::vector<int32_t> items;
        std::vector<size_t> item_off;  // first item of each launch
        int32_t max_E_global = 0;
        int grid_global = 0;
        B->grid = 0;
        for (Launch &L : B->launches) {
            int per_sm = 0;
            cuda_check(batch_blocks_per_sm(L.win_smem, L.positive, L.tsmem, B->n_warps, L.smem, &per_sm),
                       "occupancy query");
            L.grid = std::max(1, per_sm) * std::max(1, sms);
            B->grid += L.grid;
            std::stable_sort(L.dags.begin(), L.dags.end(), [&](int32_t x, int32_t y) { return cost(x) > cost(y); });
            item_off.push_back(items.size() / 2);
            for (int32_t i : L.dags) {
                if (!L.win_smem) max_E_global = std::max(max_E_global, B->dags[i]->h.E);
                const int64_t tiles = (B->n[i] + kTile - 1) / kTile;
                for (int64_t t = 0; t < tiles; ++t) {
                    items.push_back(i);
                    items.push_back((int32_t)t);
                }
            }
            L.args.n_items = (int32_t)(items.size() / 2 - item_off.back());
            if (!L.win_smem) grid_global = std::max(grid_global, L.grid);  // launches run one after another
        }
        B->n_items = (int64_t)items.size() / 2;
        if (B->n_items > (int64_t)INT32_MAX) throw McdError(MCD_ERR_INVALID, "too many work items");
        const size_t E = (size_t)B->total_E;
        // one queue head per launch, 64 bytes apart (up to eight kernel variants)
        const size_t s_acc = align_up(E * 8, 256), s_hist = align_up(E * kHistStride * 4, 256),
                     s_ctr = align_up(B->launches.size() * 64, 256),
                     s_out = align_up(5 * E * 8, 256), s_te = align_up(E * 8, 256),
                     s_args = align_up((size_t)n_dags * sizeof(KArgs), 256),
                     s_fargs = align_up((size_t)n_dags * sizeof(FArgs), 256),
                     s_items = align_up(items.size() * 4, 256),
                     s_scr = align_up((size_t)grid_global * max_E_global * kTile * 8, 256);
        B->zero_bytes = s_acc + s_hist + s_ctr;
        cuda_check(cudaMalloc(&B->dmem, B->zero_bytes + s_out + s_te + s_args + s_fargs + s_items + s_scr),
                   "batch allocation");
        char *p = B->dmem;
        auto *acc = reinterpret_cast<unsigned long long *>(p);
        B->hist = reinterpret_cast<uint32_t *>(p + s_acc);
        auto *counter = reinterpret_cast<unsigned int *>(p + s_acc + s_hist);
        p += B->zero_bytes;
        B->out = reinterpret_cast<double *>(p);
        p += s_out;
        auto *d_te = reinterpret_cast<long long *>(p);
        p += s_te;
        auto *d_args = reinterpret_cast<KArgs *>(p);
        p += s_args;
        B->d_fargs = reinterpret_cast<FArgs *>(p);
        p += s_fargs;
        auto *d_items = reinterpret_cast<int32_t *>(p);
        p += s_items;
        double *scratch = s_scr ? reinterpret_cast<double *>(p) : nullptr;
        // per-DAG kernel and finish arguments
        std::vector<KArgs> ka((size_t)n_dags);
        std::vector<FArgs> fa((size_t)n_dags);
        std::vector<long long> te(E);  // every DAG's earliest in ticks of its statistics
        for (int32_t i = 0; i < n_dags; ++i) {
            mcd_dag *g = B->dags[i];
            const StatsParams sp = stats_params(g->h, B->n[i]);
            KArgs a = base_args(g);
            a.seeds = nullptr;
            a.seed0 = seed0[i];
            a.n = B->n[i];
            a.ld = 0;
            a.stats_fixed = sp.fixed;
            a.tick_q = sp.q;
            a.bin_mul = sp.bin_mul;
            a.hist_inv_w = sp.inv_w;
            a.acc = acc + B->ev_off[i];
            a.te = d_te + B->ev_off[i];
            a.hist = B->hist + (size_t)B->ev_off[i] * kHistStride;
            ka[i] = a;
            for (int32_t e = 0; e < g->h.E; ++e) {
                long long b;
                std::memcpy(&b, &g->h.earliest[(size_t)e], 8);
                te[(size_t)B->ev_off[i] + e] = sp.fixed ? ticks_of(b, sp.q) : 0ll;
            }
            FArgs f{};
            f.acc = a.acc;
            f.hist = a.hist;
            f.earliest = g->d_earliest;
            f.ub = g->d_ub;
            f.E = g->h.E;
            f.stats_fixed = sp.fixed;
            f.tick_q = sp.q;
            f.bin_w = sp.bin_w;
            f.n = B->n[i];
            for (int k = 0; k < 5; ++k) {
                double *o = B->out + (size_t)k * E + (size_t)B->ev_off[i];
                (k == 0 ? f.mean : k == 1 ? f.p50 : k == 2 ? f.p90 : k == 3 ? f.p99 : f.p_on_time) = o;
            }
            fa[i] = f;
        }
        cuda_check(cudaMemcpy(d_args, ka.data(), ka.size() * sizeof(KArgs), cudaMemcpyHostToDevice), "upload");
        cuda_check(cudaMemcpy(B->d_fargs, fa.data(), fa.size() * sizeof(FArgs), cudaMemcpyHostToDevice), "upload");
        cuda_check(cudaMemcpy(d_items, items.data(), items.size() * 4, cudaMemcpyHostToDevice), "upload");
        if (E) cuda_check(cudaMemcpy(d_te, te.data(), E * 8, cudaMemcpyHostToDevice), "upload");
        for (size_t k = 0; k < B->launches.size(); ++k) {
            Launch &L = B->launches[k];
            L.args.dags = d_args;
            L.args.items = d_items + 2 * item_off[k];
            L.args.counter = counter + 16 * k;  // one queue head per launch, 64 bytes apart
            L.args.scratch = L.win_smem ? nullptr : scratch;
            L.args.scratch_stride = L.win_smem ? 0 : (int64_t)max_E_global * kTile;
            L.args.smem_bytes = (int32_t)L.smem;
        }
        *out = B;
    });
    if (rc != MCD_OK && B) {
        std::string keep = mcd_last_error();
        mcd_batch_destroy(B);
        set_last_error(keep);
    }
    return rc;
}

void mcd_batch_destroy(mcd_batch *B) {
    if (!B) return;
    cudaSetDevice(B->device);
    if (B->stream) cudaStreamSynchronize(B->stream);
    if (B->exec) cudaGraphExecDestroy(B->exec);
    if (B->graph) cudaGraphDestroy(B->graph);
    if (B->stream) cudaStreamDestroy(B->stream);
    if (B->dmem) cudaFree(B->dmem);
    delete B;
}

int mcd_batch_run(mcd_batch *B) {
    return guarded([&] {
        if (!B) throw McdError(MCD_ERR_INVALID, "null batch");
        cuda_check(cudaSetDevice(B->device), "cudaSetDevice");
        if (!B->exec) {
            cuda_check(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
            cudaError_t e = cudaMemsetAsync(B->dmem, 0, B->zero_bytes, B->stream);
            for (const Launch &L : B->launches)
                if (e == cudaSuccess)
                    e = launch_batch_stats(L.args, L.win_smem, L.positive, L.tsmem, B->n_warps, L.smem, L.grid,
                                           B->stream);
            if (e == cudaSuccess)
                e = launch_batch_finish(B->d_fargs, (int32_t)B->dags.size(), B->max_E, B->stream);
            cudaGraph_t graph = nullptr;
            const cudaError_t e2 = cudaStreamEndCapture(B->stream, &graph);
            cuda_check(e, "batch capture");
            cuda_check(e2, "graph capture end");
            B->graph = graph;
            cuda_check(cudaGraphInstantiate(&B->exec, B->graph, 0), "graph instantiate");
        }
        cuda_check(cudaGraphLaunch(B->exec, B->stream), "graph launch");
    });
}

int mcd_batch_sync(mcd_batch *B) {
    return guarded([&] {
        if (!B) throw McdError(MCD_ERR_INVALID, "null batch");
        cuda_check(cudaSetDevice(B->device), "cudaSetDevice");
        cuda_check(cudaStreamSynchronize(B->stream), "batch sync");
        for (mcd_dag *g : B->dags) check_device_error(g);
    });
}

int mcd_batch_occupancy(int32_t n_warps, int64_t smem_bytes, int32_t *blocks_per_sm) {
    return guarded([&] {
        if (!blocks_per_sm || n_warps < 1 || n_warps > kMaxBatchWarps || smem_bytes < 0 ||
            smem_bytes > (int64_t)kSmemMax)
            throw McdError(MCD_ERR_INVALID, "bad arguments");
        int per_sm = 0;
        cuda_check(batch_blocks_per_sm(true, true, true, n_warps, (size_t)smem_bytes, &per_sm), "occupancy query");
        *blocks_per_sm = per_sm;
    });
}

void *mcd_batch_stream(const mcd_batch *B) { return B ? (void *)B->stream : nullptr; }
int64_t mcd_batch_items(const mcd_batch *B) { return B ? B->n_items : -1; }
int32_t mcd_batch_grid(const mcd_batch *B) { return B ? B->grid : -1; }

int mcd_batch_download(mcd_batch *B, int32_t i, const mcd_stats *host) {
    return guarded([&] {
        if (!B || !host || i < 0 || i >= (int32_t)B->dags.size()) throw McdError(MCD_ERR_INVALID, "bad arguments");
        cuda_check(cudaSetDevice(B->device), "cudaSetDevice");
        cuda_check(cudaStreamSynchronize(B->stream), "batch sync");
        const size_t E = (size_t)B->total_E, e0 = (size_t)B->ev_off[i], ne = (size_t)B->dags[i]->h.E;
        double *dst[5] = {host->mean, host->p50, host->p90, host->p99, host->p_on_time};
        for (int k = 0; k < 5; ++k)
            if (dst[k])
                cuda_check(cudaMemcpy(dst[k], B->out + k * E + e0, ne * 8, cudaMemcpyDeviceToHost), "download");
        if (host->hist)
            cuda_check(cudaMemcpy(host->hist, B->hist + e0 * kHistStride, ne * kHistStride * 4,
                                  cudaMemcpyDeviceToHost),
                       "download");
    });
}

}  // extern "C"
