// mcd_prop_sample.cu -- instantiations of k_propagate that draw their own delays,
// and the persistent batch kernel.  (Separate translation units keep the build
// parallel.)
#include "mcd_device.cuh"

namespace mcd {

// Persistent statistics kernel over a batch of DAGs: each CTA takes (DAG, tile)
// items from an atomic work queue (ordered longest first by the host) until the
// queue is empty.  No CTA waits on another: the queue head is a plain counter.
// One instantiation per (window on chip, positive times, tables in shared memory):
// every DAG of a launch shares all three, so only one propagation variant is
// inlined (fewer registers, one copy of the samplers).
// DAGs whose window is not on chip use per-CTA scratch rows (32 samples each).
// Each DAG has its own shared-memory layout; the barrier pair and the stage
// counters live outside all of them, in static shared memory, so they never
// move between items.
template <bool WIN_SMEM, bool POSITIVE, bool TSMEM>
__global__ void __launch_bounds__(768, 1) k_batch_stats(const BatchArgs b) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ KArgs s_args;
    __shared__ __align__(8) uint64_t s_bars[kBarRegionBytes / 8];
    __shared__ int s_item;
    bool reuse = false;
    for (;;) {
        if (threadIdx.x == 0) s_item = (int)atomicAdd(b.counter, 1u);
        __syncthreads();
        const int item = s_item;
        if (item >= b.n_items) return;
        const int2 it = __ldg(reinterpret_cast<const int2 *>(b.items) + item);
        if (threadIdx.x == 0) s_args = b.dags[it.x];
        __syncthreads();
        const KArgs &a = s_args;
        // a layout larger than the launch's shared memory, or of another variant: never touch it
        if (a.smem_total > b.smem_bytes || (a.win_smem != 0) != WIN_SMEM || (a.positive != 0) != POSITIVE ||
            (a.tables_in_smem != 0) != TSMEM || a.n_warps * 32 != (int)blockDim.x) {
            if (threadIdx.x == 0) atomicOr(a.err, ERR_LAYOUT);
            __syncthreads();
            continue;
        }
        double *rows = WIN_SMEM ? nullptr : b.scratch + (int64_t)blockIdx.x * b.scratch_stride;
        // (many DAGs' histogram counters at once: a warp's equal bins added once)
        const bool ok = propagate_tile<false, WIN_SMEM, true, POSITIVE, false, TSMEM ? kTablesSmem : kTablesGlobal,
                                       false>(
            a, it.y, rows, WIN_SMEM ? 0 : kTile, true, smem, s_bars, reuse);
        reuse = true;
        if (!ok) return;
        __syncthreads();  // s_args / s_item are rewritten by the next item
    }
}

static void (*batch_kernel(bool win_smem, bool positive, bool tsmem))(const BatchArgs) {
    if (tsmem) {
        if (win_smem) return positive ? k_batch_stats<true, true, true> : k_batch_stats<true, false, true>;
        return positive ? k_batch_stats<false, true, true> : k_batch_stats<false, false, true>;
    }
    if (win_smem) return positive ? k_batch_stats<true, true, false> : k_batch_stats<true, false, false>;
    return positive ? k_batch_stats<false, true, false> : k_batch_stats<false, false, false>;
}

cudaError_t launch_prop_sample_gt(const KArgs &a, bool win_smem, bool stats, bool positive, dim3 grid, dim3 block,
                                  size_t smem, cudaStream_t st);

// DAGs whose tables block sits in shared memory (all but those with very large
// empirical tables) run these; the others the kTablesGlobal instantiations of
// mcd_prop_sample_gt.cu.
cudaError_t launch_prop_sample(const KArgs &a, bool win_smem, bool stats, bool positive, dim3 grid, dim3 block,
                               size_t smem, cudaStream_t st) {
    if (!a.tables_in_smem) return launch_prop_sample_gt(a, win_smem, stats, positive, grid, block, smem, st);
    constexpr int S = kTablesSmem;
    void (*fn)(const KArgs);
    if (stats) {
        if (positive) fn = win_smem ? k_propagate<false, true, true, true, S> : k_propagate<false, false, true, true, S>;
        else fn = win_smem ? k_propagate<false, true, true, false, S> : k_propagate<false, false, true, false, S>;
    } else {
        if (positive) fn = win_smem ? k_propagate<false, true, false, true, S> : k_propagate<false, false, false, true, S>;
        else fn = win_smem ? k_propagate<false, true, false, false, S> : k_propagate<false, false, false, false, S>;
    }
    const cudaError_t e = raise_smem_limit((const void *)fn, smem);
    if (e != cudaSuccess) return e;
    fn<<<grid, block, smem, st>>>(a);
    return cudaGetLastError();
}

// Persistent batch launch: one CTA per SM slot, `blocks_per_sm` of them per SM.
cudaError_t launch_batch_stats(const BatchArgs &b, bool win_smem, bool positive, bool tsmem, int n_warps, size_t smem,
                               int grid, cudaStream_t st) {
    void (*fn)(const BatchArgs) = batch_kernel(win_smem, positive, tsmem);
    const cudaError_t e = raise_smem_limit((const void *)fn, smem);
    if (e != cudaSuccess) return e;
    fn<<<grid, n_warps * 32, smem, st>>>(b);
    return cudaGetLastError();
}

// CTAs of the batch kernel that fit on one SM at this block size and shared memory.
cudaError_t batch_blocks_per_sm(bool win_smem, bool positive, bool tsmem, int n_warps, size_t smem, int *out) {
    void (*fn)(const BatchArgs) = batch_kernel(win_smem, positive, tsmem);
    const cudaError_t e = raise_smem_limit((const void *)fn, smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, fn, n_warps * 32, smem);
}

}  // namespace mcd
