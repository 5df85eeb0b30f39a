// mcd_handle.hpp -- the compiled-DAG handle and the helpers the C-ABI files share.
#pragma once

#include <cuda_runtime.h>

#include <new>
#include <string>

#include "mcd_host.hpp"

// A compiled, device-resident DAG: host copies of the records, one device
// allocation holding them, two streams, and a workspace for the host paths.
struct mcd_dag {
    int device = 0;
    cudaStream_t stream[2] = {nullptr, nullptr};
    mcd::HostDag h;
    char *dmem = nullptr;
    size_t dbytes = 0;
    mcd::EvRec *d_ev = nullptr;
    mcd::PredRec *d_pred = nullptr;
    mcd::LinkRec *d_aux = nullptr;
    mcd::DistParam *d_dist = nullptr;  // tables block: distributions, alias entries, alias picks
    double *d_vals = nullptr;
    int32_t *d_wk = nullptr;
    int32_t *d_stage_meta = nullptr;
    double *d_earliest = nullptr;  // caller order, for the statistics finish
    double *d_ub = nullptr;
    int32_t *d_err = nullptr;
    char *ws = nullptr;  // workspace
    size_t ws_bytes = 0;
};


namespace mcd {

extern thread_local std::string g_last_error;
void set_last_error(const std::string &msg);
void cuda_check(cudaError_t e, const char *what);
void ensure_ws(mcd_dag *g, size_t bytes);
KArgs base_args(const mcd_dag *g);
void check_device_error(mcd_dag *g);

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Runs f, turning exceptions into a status code and the thread's last error.
template <typename F>
int guarded(F &&f) {
    try {
        f();
        g_last_error.clear();
        return MCD_OK;
    } catch (const McdError &e) {
        g_last_error = e.what();
        return e.code;
    } catch (const std::bad_alloc &) {
        g_last_error = "host allocation failed";
        return MCD_ERR_NOMEM;
    } catch (const std::exception &e) {
        g_last_error = e.what();
        return MCD_ERR_RUNTIME;
    }
}

}  // namespace mcd
