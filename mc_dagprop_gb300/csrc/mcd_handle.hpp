// mcd_handle.hpp -- the compiled-DAG handle and the helpers the C-ABI files share.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <new>
#include <string>
#include <vector>

#include "mcd_host.hpp"

namespace mcd {
// The device image of a compiled DAG: the host copies of its records and one
// device allocation holding them.  Nothing writes it after the upload, so
// handles created from identical inputs on the same device share one image (the
// compiled-DAG cache keyed by the inputs' content, mcd_capi.cpp).
struct DagImage {
    int device = 0;
    HostDag h;
    char *dmem = nullptr;
    size_t dbytes = 0;
    EvRec *d_ev = nullptr;
    PredRec *d_pred = nullptr;
    LinkRec *d_aux = nullptr;
    DistParam *d_dist = nullptr;  // tables block: distributions, alias entries, alias picks
    double *d_vals = nullptr;
    int32_t *d_wk = nullptr;
    int32_t *d_stage_meta = nullptr;
    double *d_earliest = nullptr;  // caller order, for the statistics finish
    double *d_ub = nullptr;
    std::vector<unsigned char> key;  // the creation inputs, serialized (empty: not cached)
    DagImage() = default;
    DagImage(const DagImage &) = delete;
    DagImage &operator=(const DagImage &) = delete;
    ~DagImage();
};
}  // namespace mcd

// A handle: a device image (possibly shared), two streams, this handle's error
// flag, and a workspace for the host paths.  The image's device pointers are
// copied into the handle for the launch code.
struct mcd_dag {
    std::shared_ptr<const mcd::DagImage> img;
    const mcd::HostDag &h;
    int device = 0;
    bool cache_hit = false;  // the image came from the compiled-DAG cache
    cudaStream_t stream[2] = {nullptr, nullptr};
    size_t dbytes = 0;
    const mcd::EvRec *d_ev = nullptr;
    const mcd::PredRec *d_pred = nullptr;
    const mcd::LinkRec *d_aux = nullptr;
    const mcd::DistParam *d_dist = nullptr;
    const double *d_vals = nullptr;
    const int32_t *d_wk = nullptr;
    const int32_t *d_stage_meta = nullptr;
    const double *d_earliest = nullptr;
    const double *d_ub = nullptr;
    int32_t *d_err = nullptr;  // latched kernel errors of this handle's launches
    char *ws = nullptr;        // workspace
    size_t ws_bytes = 0;
    int64_t last_adj_plan[3] = {0, 0, 0};  // the last gradient's samples per chunk, level blocks, buffer bytes
    explicit mcd_dag(std::shared_ptr<const mcd::DagImage> image)
        : img(std::move(image)), h(img->h), device(img->device), dbytes(img->dbytes), d_ev(img->d_ev),
          d_pred(img->d_pred), d_aux(img->d_aux), d_dist(img->d_dist), d_vals(img->d_vals), d_wk(img->d_wk),
          d_stage_meta(img->d_stage_meta), d_earliest(img->d_earliest), d_ub(img->d_ub) {}
    mcd_dag(const mcd_dag &) = delete;
    mcd_dag &operator=(const mcd_dag &) = delete;
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
