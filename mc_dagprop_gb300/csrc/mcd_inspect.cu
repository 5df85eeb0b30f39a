// mcd_inspect.cu -- per-type delay histograms of sampled durations, the GPU form of
// the reference's delay inspection (demo/inspection.py:11-29: durations - base per
// activity type, absolute and relative to the base).
//
// Samples run in chunks through the propagation kernel with only the durations
// output ([link][sample] rows in the handle's workspace); k_delay_hist then bins
// every (link, sample) duration of the chunk into per-class histograms held in
// shared memory and merged into device counters at the end of each CTA.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "mcd_handle.hpp"

namespace mcd {
cudaError_t launch_propagate(const KArgs &a, bool given, bool win_smem, bool stats, cudaStream_t st);

namespace {

// Bin of x in [lo, hi) with nb bins: 0 below lo, 1 + floor((x - lo) * nb / (hi - lo))
// inside, nb + 1 at or above hi.
__device__ __forceinline__ int delay_bin(double x, double lo, double hi, int nb) {
    if (!(x >= lo)) return 0;
    if (!(x < hi)) return nb + 1;
    const int b = (int)((x - lo) * (double)nb / (hi - lo));
    return 1 + (b < nb ? b : nb - 1);
}

// counts: [class][abs, rel][nb + 2]; moments: [class][abs, rel][count, sum, sum of squares].
__global__ void __launch_bounds__(256) k_delay_hist(const double *__restrict__ dur, int64_t ld, int64_t n, int32_t L,
                                                    const int32_t *__restrict__ cls, const double *__restrict__ base,
                                                    int32_t nc, int32_t nb, const double *__restrict__ ranges,
                                                    unsigned long long *counts, double *moments) {
    extern __shared__ __align__(16) unsigned char sm[];
    const int nh = nc * 2 * (nb + 2);
    double *smom = reinterpret_cast<double *>(sm);        // nc * 2 * 3
    unsigned *shist = reinterpret_cast<unsigned *>(smom + nc * 6);
    for (int i = threadIdx.x; i < nh; i += blockDim.x) shist[i] = 0u;
    for (int i = threadIdx.x; i < nc * 6; i += blockDim.x) smom[i] = 0.0;
    __syncthreads();
    const int64_t total = (int64_t)L * n;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int32_t l = (int32_t)(idx / n);
        const int64_t s = idx - (int64_t)l * n;
        const int32_t c = cls[l];
        if (c < 0) continue;
        const double b = base[l];
        const double delta = dur[(int64_t)l * ld + s] - b;  // demo/inspection.py:23-24
        const double *r = ranges + 4 * c;
        atomicAdd(&shist[(c * 2 + 0) * (nb + 2) + delay_bin(delta, r[0], r[1], nb)], 1u);
        atomicAdd(&smom[c * 6 + 0], 1.0);
        atomicAdd(&smom[c * 6 + 1], delta);
        atomicAdd(&smom[c * 6 + 2], delta * delta);
        if (b != 0.0) {  // relative delays of links with a non-zero base (:25-26)
            const double rel = delta / b;
            atomicAdd(&shist[(c * 2 + 1) * (nb + 2) + delay_bin(rel, r[2], r[3], nb)], 1u);
            atomicAdd(&smom[c * 6 + 3], 1.0);
            atomicAdd(&smom[c * 6 + 4], rel);
            atomicAdd(&smom[c * 6 + 5], rel * rel);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nh; i += blockDim.x)
        if (shist[i]) atomicAdd(&counts[i], (unsigned long long)shist[i]);
    for (int i = threadIdx.x; i < nc * 6; i += blockDim.x)
        if (smom[i] != 0.0) atomicAdd(&moments[i], smom[i]);
}

}  // namespace
}  // namespace mcd

using namespace mcd;

extern "C" {

int mcd_delay_histograms(mcd_dag *g, const int64_t *seeds, int64_t n, const int32_t *link_class,
                         const double *link_base, int32_t n_classes, int32_t n_bins, const double *ranges,
                         uint64_t *counts, double *moments) {
    return guarded([&] {
        if (!g || !link_class || !link_base || !ranges || !counts || !moments)
            throw McdError(MCD_ERR_INVALID, "null argument");
        if (n < 0) throw McdError(MCD_ERR_INVALID, "negative sample count");
        if (n > 0 && !seeds) throw McdError(MCD_ERR_INVALID, "null seeds");
        if (n_classes < 1 || n_bins < 1 || (size_t)n_classes * 2 * (n_bins + 2) * 4 + (size_t)n_classes * 48 > 48 * 1024)
            throw McdError(MCD_ERR_INVALID, "n_classes * 2 * (n_bins + 2) counters must fit 48 KB");
        const int32_t L = g->h.L, E = g->h.E;
        for (int32_t l = 0; l < L; ++l)
            if (link_class[l] < -1 || link_class[l] >= n_classes) throw McdError(MCD_ERR_INVALID, "link class out of range");
        for (int32_t c = 0; c < n_classes; ++c)
            if (!(ranges[4 * c] < ranges[4 * c + 1]) || !(ranges[4 * c + 2] < ranges[4 * c + 3]))
                throw McdError(MCD_ERR_INVALID, "each histogram range needs lo < hi");
        cuda_check(cudaSetDevice(g->device), "cudaSetDevice");
        cudaStream_t st = g->stream[0];
        const size_t nh = (size_t)n_classes * 2 * (n_bins + 2), nm = (size_t)n_classes * 6;
        // chunk: durations rows (and realized scratch rows when the window is off chip)
        const double per_sample = 8.0 * L + (g->h.win_smem ? 0.0 : 8.0 * E) + 8.0;
        int64_t C = std::max<int64_t>(32, std::min<int64_t>((n + 31) / 32 * 32, (int64_t)((double)(2ll << 30) / per_sample) / 32 * 32));
        const size_t o_cls = 0, o_base = align_up((size_t)L * 4, 256), o_rng = o_base + align_up((size_t)L * 8, 256),
                     o_cnt = o_rng + align_up((size_t)n_classes * 32, 256), o_mom = o_cnt + align_up(nh * 8, 256),
                     o_seed = o_mom + align_up(nm * 8, 256), o_dur = o_seed + align_up((size_t)C * 8, 256),
                     o_real = o_dur + align_up((size_t)L * C * 8, 256),
                     total = o_real + (g->h.win_smem ? 0 : align_up((size_t)E * C * 8, 256));
        ensure_ws(g, total);
        char *w = g->ws;
        cuda_check(cudaMemcpyAsync(w + o_cls, link_class, (size_t)L * 4, cudaMemcpyHostToDevice, st), "upload");
        cuda_check(cudaMemcpyAsync(w + o_base, link_base, (size_t)L * 8, cudaMemcpyHostToDevice, st), "upload");
        cuda_check(cudaMemcpyAsync(w + o_rng, ranges, (size_t)n_classes * 32, cudaMemcpyHostToDevice, st), "upload");
        cuda_check(cudaMemsetAsync(w + o_cnt, 0, nh * 8, st), "reset");
        cuda_check(cudaMemsetAsync(w + o_mom, 0, nm * 8, st), "reset");
        const size_t smem = nh * 4 + nm * 8;
        int sms = 0;
        cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g->device), "device query");
        for (int64_t off = 0; off < n; off += C) {
            const int64_t m = std::min(C, n - off);
            cuda_check(cudaMemcpyAsync(w + o_seed, seeds + off, (size_t)m * 8, cudaMemcpyHostToDevice, st), "seeds");
            KArgs a = base_args(g);
            a.seeds = reinterpret_cast<const int64_t *>(w + o_seed);
            a.n = m;
            a.ld = C;
            a.durations = reinterpret_cast<double *>(w + o_dur);
            if (!g->h.win_smem) a.scratch = reinterpret_cast<double *>(w + o_real);
            cuda_check(launch_propagate(a, false, g->h.win_smem, false, st), "propagate launch");
            const int64_t items = (int64_t)L * m;
            const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((items + 255) / 256, (int64_t)sms * 8));
            k_delay_hist<<<grid, 256, smem, st>>>(reinterpret_cast<const double *>(w + o_dur), C, m, L,
                                                  reinterpret_cast<const int32_t *>(w + o_cls),
                                                  reinterpret_cast<const double *>(w + o_base), n_classes, n_bins,
                                                  reinterpret_cast<const double *>(w + o_rng),
                                                  reinterpret_cast<unsigned long long *>(w + o_cnt),
                                                  reinterpret_cast<double *>(w + o_mom));
            cuda_check(cudaGetLastError(), "histogram launch");
        }
        cuda_check(cudaMemcpyAsync(counts, w + o_cnt, nh * 8, cudaMemcpyDeviceToHost, st), "download");
        cuda_check(cudaMemcpyAsync(moments, w + o_mom, nm * 8, cudaMemcpyDeviceToHost, st), "download");
        check_device_error(g);
    });
}

}  // extern "C"
