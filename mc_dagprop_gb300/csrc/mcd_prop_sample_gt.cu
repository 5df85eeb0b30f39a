// mcd_prop_sample_gt.cu -- instantiations of k_propagate that draw their own
// delays for DAGs whose distribution tables stay in global memory (a separate
// translation unit keeps the build parallel).
#include "mcd_device.cuh"

namespace mcd {

cudaError_t launch_prop_sample_gt(const KArgs &a, bool win_smem, bool stats, bool positive, dim3 grid, dim3 block,
                                  size_t smem, cudaStream_t st) {
    constexpr int G = kTablesGlobal;
    void (*fn)(const KArgs);
    if (stats) {
        if (positive) fn = win_smem ? k_propagate<false, true, true, true, G> : k_propagate<false, false, true, true, G>;
        else fn = win_smem ? k_propagate<false, true, true, false, G> : k_propagate<false, false, true, false, G>;
    } else {
        if (positive) fn = win_smem ? k_propagate<false, true, false, true, G> : k_propagate<false, false, false, true, G>;
        else fn = win_smem ? k_propagate<false, true, false, false, G> : k_propagate<false, false, false, false, G>;
    }
    const cudaError_t e = raise_smem_limit((const void *)fn, smem);
    if (e != cudaSuccess) return e;
    fn<<<grid, block, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace mcd
