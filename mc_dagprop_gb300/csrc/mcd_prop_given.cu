// mcd_prop_given.cu -- instantiations of k_propagate that read given durations.
#include "mcd_device.cuh"

namespace mcd {

cudaError_t launch_prop_given(const KArgs &a, bool win_smem, bool stats, dim3 grid, dim3 block, size_t smem,
                              cudaStream_t st) {
    void (*fn)(const KArgs);
    // (given durations: no sampler, so the tables' place does not matter)
    constexpr int E = kTablesEither;
    if (stats) fn = win_smem ? k_propagate<true, true, true, false, E> : k_propagate<true, false, true, false, E>;
    else fn = win_smem ? k_propagate<true, true, false, false, E> : k_propagate<true, false, false, false, E>;
    const cudaError_t e = raise_smem_limit((const void *)fn, smem);
    if (e != cudaSuccess) return e;
    fn<<<grid, block, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace mcd
