// mcd_grad.cpp -- pathwise gradient of the expected total tardiness (the adjoint).
// No counterpart in the reference; see mcd_adjoint.cu for the method.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "mcd_handle.hpp"

namespace mcd {
cudaError_t launch_adjoint(const KArgs &a, cudaStream_t st);
cudaError_t launch_event_ticks(const double *earliest, int32_t E, int32_t q, long long *te, cudaStream_t st);
cudaError_t launch_adjoint_finish(const long long *grad_e, const long long *grad_l, const unsigned long long *acc,
                                  int32_t E, int32_t L, int64_t n, int32_t q, double *g_earliest, double *g_base,
                                  double *objective, cudaStream_t st);
}  // namespace mcd

using namespace mcd;

extern "C" int mcd_gradient_host(mcd_dag *g, int64_t seed0, int64_t n, double *objective, double *grad_earliest,
                                 double *grad_base) {
    return guarded([&] {
        if (!g) throw McdError(MCD_ERR_INVALID, "null handle");
        if (n <= 0 || n > (int64_t)1 << 31) throw McdError(MCD_ERR_INVALID, "need 0 < n <= 2^31 samples");
        const HostDag &h = g->h;
        if (!h.win_smem)
            throw McdError(MCD_ERR_INVALID, "the gradient needs a DAG whose window fits in shared memory");
        if (h.max_preds > kAdjMaxPreds)
            throw McdError(MCD_ERR_INVALID, "the gradient supports at most 16383 predecessors per event");
        const StatsParams sp = stats_params(h, n);
        if (!sp.fixed) throw McdError(MCD_ERR_INVALID, "the gradient needs finite earliest times and max_delay");
        cuda_check(cudaSetDevice(g->device), "cudaSetDevice");
        cudaStream_t st = g->stream[0];
        const size_t E = (size_t)h.E, L = (size_t)std::max(h.L, 0);
        // samples per chunk: adjoint records (6 bytes per event and sample) within ~4 GiB
        int64_t C = (int64_t)((4ull << 30) / std::max<size_t>(6 * E, 1));
        C = std::max<int64_t>(32, std::min<int64_t>(C / 32 * 32, (n + 31) / 32 * 32));
        const size_t s_code = align_up(E * (size_t)C * 2, 256), s_dfac = align_up(E * (size_t)C * 4, 256),
                     s_acc = align_up(E * 8, 256), s_ge = align_up(E * 8, 256), s_gl = align_up(L * 8 + 8, 256),
                     s_out = align_up((E + L + 1) * 8, 256), s_te = align_up(E * 8, 256);
        ensure_ws(g, s_code + s_dfac + s_acc + s_ge + s_gl + s_out + s_te);
        char *p = g->ws;
        auto *code = reinterpret_cast<uint16_t *>(p);
        p += s_code;
        auto *dfac = reinterpret_cast<float *>(p);
        p += s_dfac;
        auto *acc = reinterpret_cast<unsigned long long *>(p);
        auto *ge = reinterpret_cast<long long *>(p + s_acc);
        auto *gl = reinterpret_cast<long long *>(p + s_acc + s_ge);
        cuda_check(cudaMemsetAsync(p, 0, s_acc + s_ge + s_gl, st), "accumulator reset");
        p += s_acc + s_ge + s_gl;
        auto *out = reinterpret_cast<double *>(p);
        auto *te = reinterpret_cast<long long *>(p + s_out);
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
            a.adj_code = code;
            a.adj_dfac = dfac;
            a.grad_e = ge;
            a.grad_l = gl;
            cuda_check(launch_adjoint(a, st), "adjoint launch");
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
    });
}
