// mcd_capi.cpp -- the extern "C" entry points of include/mc_dagprop_gb300.h.
//
// Owns the compiled, device-resident DAG images (one allocation each, shared by
// handles of identical inputs through a content-keyed cache), each handle's two
// CUDA streams and a workspace for the host-buffer entry points, which run in
// chunks: copy seeds in, run the fused kernel into sample-minor rows, transpose
// to the reference's sample-major SimResult layout, copy out -- a compute
// stream and a transfer stream, so the host link overlaps the sampling.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>

#include "mcd_handle.hpp"

namespace mcd {
cudaError_t launch_propagate(const KArgs &a, bool given, bool win_smem, bool stats, cudaStream_t st);
cudaError_t launch_stats_finish(const FArgs &f, cudaStream_t st);
cudaError_t launch_event_ticks(const double *earliest, int32_t E, int32_t q, long long *te, cudaStream_t st);
cudaError_t launch_wait_selftest(int32_t *err, uint32_t limit, cudaStream_t st);
cudaError_t noalloc_scratch(void **ptr, size_t *bytes);
cudaError_t launch_transpose_f64(const double *in, int64_t ld_in, double *out, int64_t ld_out, int64_t rows,
                                 int64_t cols, cudaStream_t st);
cudaError_t launch_transpose_i32(const int32_t *in, int64_t ld_in, int32_t *out, int64_t ld_out, int64_t rows,
                                 int64_t cols, cudaStream_t st);
}  // namespace mcd

using namespace mcd;

namespace mcd {

thread_local std::string g_last_error;

void set_last_error(const std::string &msg) { g_last_error = msg; }

void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        if (e == cudaErrorMemoryAllocation)
            throw McdError(MCD_ERR_NOMEM, std::string(what) + ": " + cudaGetErrorString(e));
        throw McdError(MCD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

void ensure_ws(mcd_dag *g, size_t bytes) {
    if (bytes <= g->ws_bytes) return;
    cuda_check(cudaStreamSynchronize(g->stream[0]), "stream sync");
    cuda_check(cudaStreamSynchronize(g->stream[1]), "stream sync");
    if (g->ws) cudaFree(g->ws);
    g->ws = nullptr;
    g->ws_bytes = 0;
    cuda_check(cudaMalloc(&g->ws, bytes), "workspace allocation");
    g->ws_bytes = bytes;
}

KArgs base_args(const mcd_dag *g) {
    KArgs a{};
    a.ev = g->d_ev;
    a.pred = g->d_pred;
    a.aux = g->d_aux;
    a.dist = g->d_dist;
    a.vals = g->d_vals;
    a.wk_off = g->d_wk;
    a.stage_meta = g->d_stage_meta;
    a.n_stages = g->h.n_stages;
    a.n_warps = g->h.n_warps;
    a.n_aux = (int32_t)g->h.aux.size();
    a.window_slots = g->h.window_slots;
    a.n_dist = (int32_t)g->h.dist.size();
    a.n_alias = (int32_t)g->h.alias.size();
    a.tables_in_smem = g->h.tables_in_smem ? 1 : 0;
    a.win_smem = g->h.win_smem ? 1 : 0;
    a.positive = g->h.positive ? 1 : 0;
    a.stage_bytes = g->h.stage_bytes;
    a.smem_stage_off = g->h.smem_stage_off;
    a.smem_tables_off = g->h.smem_tables_off;
    a.smem_bar_off = g->h.smem_bar_off;
    a.smem_total = g->h.smem_total;
    a.err = g->d_err;
    return a;
}

void check_device_error(mcd_dag *g) {
    cuda_check(cudaStreamSynchronize(g->stream[0]), "stream sync");
    cuda_check(cudaStreamSynchronize(g->stream[1]), "stream sync");
    int32_t flags = 0;
    cuda_check(cudaMemcpy(&flags, g->d_err, sizeof(flags), cudaMemcpyDeviceToHost), "error flag read");
    if (flags) {
        cuda_check(cudaMemset(g->d_err, 0, sizeof(int32_t)), "error flag reset");
        if (flags & ERR_GAMMA_REJECTION)
            throw McdError(MCD_ERR_DEVICE,
                           "gamma sampler: truncation at max_scale rejected 4096 consecutive attempts; "
                           "max_scale is too small for this shape/scale");
        if (flags & ERR_STAGE_TIMEOUT)
            throw McdError(MCD_ERR_DEVICE, "a staged record copy did not complete within the wait limit");
        if (flags & ERR_LAYOUT)
            throw McdError(MCD_ERR_DEVICE, "a DAG's shared-memory layout exceeds its launch's shared memory");
        throw McdError(MCD_ERR_DEVICE, "kernel reported error flags " + std::to_string(flags));
    }
}

}  // namespace mcd

DagImage::~DagImage() {
    if (!dmem) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(device);
    cudaFree(dmem);
    cudaSetDevice(prev);
}

namespace {

// Samples per chunk for the host-buffer entry points, a multiple of 32, and the
// number of chunk buffer sets: one when all n samples fit one chunk, else two,
// used alternately.  A chunk is one launch in which every 32-sample tile walks
// the whole DAG at one CTA per SM; half a wave of tiles leaves the other half of
// the SMs to the transfer of the previous chunk.  staged: some host buffer is
// pageable, so its rows go through a sample-major device copy as well.  Chunks
// stay within a workspace of a quarter of the device memory not otherwise in use
// (at most 32 GiB).
int64_t host_chunk(const mcd_dag *g, int64_t n, bool staged, int *sets) {
    const double per_sample = (staged ? 2.0 : 1.0) * (12.0 * g->h.E + 8.0 * g->h.L) + 8.0;
    size_t free_b = 0, total_b = 0;
    cuda_check(cudaMemGetInfo(&free_b, &total_b), "device memory query");
    int sms = 0;
    cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g->device), "device query");
    const int64_t half_wave = (int64_t)kTile * std::max(1, sms / 2);
    const double budget =
        std::min(std::max((double)(free_b + g->ws_bytes) / 4.0, (double)(1ll << 30)), (double)(32ll << 30));
    const int64_t n32 = std::max<int64_t>(32, (n + 31) / 32 * 32);
    if (n32 <= half_wave && (double)n32 * per_sample <= budget) {
        *sets = 1;
        return n32;
    }
    *sets = 2;
    const int64_t c = std::min<int64_t>(half_wave, (int64_t)(budget / (2.0 * std::max(per_sample, 1.0))));
    return std::max<int64_t>(32, c / 32 * 32);
}

// The two-stream chunk pipeline of the host-buffer entry points.  The handle's
// first stream computes chunk after chunk (uploads of given inputs, sampling and
// propagation into a buffer set); the second moves each computed chunk to the
// host (transposes, and copies for pageable buffers).  Chunk k's computation
// waits only until the transfer of chunk k - sets has released its buffer set,
// so after the first chunk the host link -- the bound -- does not wait for the
// sampler.
struct ChunkPipe {
    cudaStream_t compute, transfer;
    cudaEvent_t computed[2] = {}, moved[2] = {};
    int sets;
    ChunkPipe(mcd_dag *g, int sets_) : compute(g->stream[0]), transfer(g->stream[1]), sets(sets_) {
        for (int k = 0; k < 2; ++k) {
            cuda_check(cudaEventCreateWithFlags(&computed[k], cudaEventDisableTiming), "event create");
            cuda_check(cudaEventCreateWithFlags(&moved[k], cudaEventDisableTiming), "event create");
        }
    }
    ~ChunkPipe() {
        for (int k = 0; k < 2; ++k) {
            if (computed[k]) cudaEventDestroy(computed[k]);
            if (moved[k]) cudaEventDestroy(moved[k]);
        }
    }
    ChunkPipe(const ChunkPipe &) = delete;
    ChunkPipe &operator=(const ChunkPipe &) = delete;
    // before chunk idx's computation: its buffer set is free again
    void begin_compute(int64_t idx) {
        if (idx >= sets) cuda_check(cudaStreamWaitEvent(compute, moved[idx % sets], 0), "stream wait");
    }
    // after it: the transfer stream takes the chunk over
    void begin_transfer(int64_t idx) {
        cuda_check(cudaEventRecord(computed[idx % sets], compute), "event record");
        cuda_check(cudaStreamWaitEvent(transfer, computed[idx % sets], 0), "stream wait");
    }
    void end_transfer(int64_t idx) { cuda_check(cudaEventRecord(moved[idx % sets], transfer), "event record"); }
};

// The device-side address of a host buffer a kernel may access directly
// (pinned or registered memory, mapped under unified addressing), or null when
// the buffer must be copied (pageable memory).  Writing outputs straight from
// the transpose kernels saves the device staging copy and a copy-engine pass.
template <typename T>
T *device_view(T *host) {
    if (!host) return nullptr;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? static_cast<T *>(at.devicePointer) : nullptr;
}

struct ChunkBufs {
    int64_t *seeds;
    double *real_minor, *dur_minor;
    int32_t *cause_minor;
    double *real_major, *dur_major;
    int32_t *cause_major;
};

// Carves `sets` chunk buffer sets of C samples out of the workspace (a single
// set serves both slots); the sample-major rows only when staged.
void carve(mcd_dag *g, int64_t C, int sets, bool staged, ChunkBufs cb[2]) {
    const size_t E = (size_t)g->h.E, L = (size_t)g->h.L;
    const size_t sz_seed = align_up((size_t)C * 8, 256), sz_re = align_up(E * (size_t)C * 8, 256),
                 sz_du = align_up(L * (size_t)C * 8, 256), sz_ca = align_up(E * (size_t)C * 4, 256);
    const size_t per = sz_seed + (staged ? 2 : 1) * (sz_re + sz_du + sz_ca);
    ensure_ws(g, (size_t)sets * per);
    for (int k = 0; k < 2; ++k) {
        char *p = g->ws + (size_t)(k % sets) * per;
        cb[k].seeds = (int64_t *)p;
        p += sz_seed;
        cb[k].real_minor = (double *)p;
        p += sz_re;
        cb[k].dur_minor = (double *)p;
        p += sz_du;
        cb[k].cause_minor = (int32_t *)p;
        p += sz_ca;
        if (staged) {
            cb[k].real_major = (double *)p;
            p += sz_re;
            cb[k].dur_major = (double *)p;
            p += sz_du;
            cb[k].cause_major = (int32_t *)p;
        } else {
            cb[k].real_major = cb[k].dur_major = nullptr;
            cb[k].cause_major = nullptr;
        }
    }
}

// ---- the compiled-DAG cache
// Handles whose inputs (DAG arrays, generator, warps, device) are identical share
// one device image.  The key is the inputs serialized byte for byte, in the order
// the compiler reads them; a 64-bit hash picks the bucket and a full comparison
// decides, so two different inputs never share an image.  The cache holds weak
// references: an image lives as long as a handle uses it.

}  // namespace

namespace mcd {

void put_bytes(std::vector<unsigned char> &k, const void *p, size_t n) {
    if (!n) return;
    const size_t o = k.size();
    k.resize(o + n);
    std::memcpy(k.data() + o, p, n);
}
template <typename T>
void put(std::vector<unsigned char> &k, const T &v) {
    put_bytes(k, &v, sizeof(T));
}

// Serializes what compile_dag reads; false (no caching) where the arrays are not
// well-formed enough to read safely -- compile_dag then reports the error.
bool image_key(const mcd_dag_desc &d, const mcd_generator &gen, int32_t n_warps, int device,
               std::vector<unsigned char> &k, int32_t window) {
    if (d.n_events < 0 || d.n_activities < 0 || d.n_targets < 0) return false;
    if ((d.n_events && !d.earliest) ||
        (d.n_activities && (!d.act_idx || !d.act_duration || !d.act_type)) ||
        (d.n_targets && (!d.target || !d.pred_offsets)))
        return false;
    const size_t E = (size_t)d.n_events, A = (size_t)d.n_activities, T = (size_t)d.n_targets;
    int64_t P = 0;
    for (size_t t = 0; t < T; ++t) {
        const int64_t b = d.pred_offsets[t], e = d.pred_offsets[t + 1];
        if (b < 0 || e < b) return false;
        P += e - b;
    }
    if (P > 0 && (!d.pred_src || !d.pred_act)) return false;
    size_t gen_bytes = 0;
    for (const DistSpec &sp : gen.dists) gen_bytes += 48 + 8 * (sp.values.size() + sp.weights.size());
    k.clear();
    k.reserve(64 + E * 8 + A * 16 + T * 12 + (size_t)P * 8 + gen_bytes);
    put(k, (int32_t)0x4D434401);  // key format
    put(k, device);
    put(k, n_warps);
    put(k, window);
    for (const char *var : {"MCD_NO_SMEM_WINDOW", "MCD_WARPS"}) {  // compile_dag's environment overrides
        const char *v = std::getenv(var);
        put(k, (int64_t)(v ? (int64_t)std::strlen(v) : -1));
        if (v) put_bytes(k, v, std::strlen(v));
    }
    put(k, d.n_events);
    put_bytes(k, d.earliest, E * 8);
    put(k, d.n_activities);
    put_bytes(k, d.act_idx, A * 4);
    put_bytes(k, d.act_duration, A * 8);
    put_bytes(k, d.act_type, A * 4);
    put(k, d.n_targets);
    put_bytes(k, d.target, T * 4);
    if (T) put_bytes(k, d.pred_offsets, (T + 1) * 8);
    for (size_t t = 0; t < T; ++t) {
        const int64_t b = d.pred_offsets[t], e = d.pred_offsets[t + 1];
        put_bytes(k, d.pred_src + b, (size_t)(e - b) * 4);
        put_bytes(k, d.pred_act + b, (size_t)(e - b) * 4);
    }
    put(k, d.max_delay);
    put(k, gen.seed);
    put(k, (int64_t)gen.dists.size());
    for (const DistSpec &sp : gen.dists) {
        put(k, sp.type);
        put(k, sp.kind);
        put(k, sp.p0);
        put(k, sp.p1);
        put(k, sp.p2);
        put(k, (int64_t)sp.values.size());
        put_bytes(k, sp.values.data(), sp.values.size() * 8);
        put(k, (int64_t)sp.weights.size());
        put_bytes(k, sp.weights.data(), sp.weights.size() * 8);
    }
    return true;
}

// 64-bit multiply-xorshift hash over 8-byte words (the tail zero-padded).
uint64_t hash_bytes(const std::vector<unsigned char> &k) {
    uint64_t h = 0x9E3779B97F4A7C15ull ^ (uint64_t)k.size();
    const size_t nw = k.size() / 8;
    for (size_t i = 0; i < nw; ++i) {
        uint64_t w;
        std::memcpy(&w, k.data() + 8 * i, 8);
        h = (h ^ w) * 0xFF51AFD7ED558CCDull;
        h ^= h >> 32;
    }
    uint64_t tail = 0;
    std::memcpy(&tail, k.data() + 8 * nw, k.size() - 8 * nw);
    h = (h ^ tail) * 0xC4CEB9FE1A85EC53ull;
    return h ^ (h >> 29);
}

}  // namespace mcd

namespace {

std::mutex g_cache_mu;
std::unordered_multimap<uint64_t, std::weak_ptr<const DagImage>> g_cache;

std::shared_ptr<const DagImage> cache_find(uint64_t hash, const std::vector<unsigned char> &key) {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    auto range = g_cache.equal_range(hash);
    for (auto it = range.first; it != range.second; ++it)
        if (auto img = it->second.lock())
            if (img->key == key) return img;
    return nullptr;
}

void cache_insert(uint64_t hash, const std::shared_ptr<const DagImage> &img) {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    for (auto it = g_cache.begin(); it != g_cache.end();)  // drop the entries of freed images
        it = it->second.expired() ? g_cache.erase(it) : std::next(it);
    g_cache.emplace(hash, img);
}

// One device allocation holding the compiled records, uploaded from the host copies.
void upload_image(DagImage &im) {
    const HostDag &h = im.h;
    const size_t s_ev = align_up(h.ev.size() * sizeof(EvRec), 256),
                 s_pred = align_up(h.pred.size() * sizeof(PredRec), 256),
                 s_aux = align_up(h.aux.size() * sizeof(LinkRec), 256),
                 s_tables = align_up(tables_bytes(h), 256),
                 s_vals = align_up(h.vals.size() * sizeof(double), 256),
                 s_wk = align_up(h.wk_off.size() * sizeof(int32_t), 256),
                 s_meta = align_up(h.stage_meta.size() * sizeof(int32_t), 256),
                 s_times = align_up(h.earliest.size() * sizeof(double), 256);
    im.dbytes = s_ev + s_pred + s_aux + s_tables + s_vals + s_wk + s_meta + 2 * s_times;
    cuda_check(cudaMalloc(&im.dmem, std::max<size_t>(im.dbytes, 256)), "compiled DAG allocation");
    char *p = im.dmem;
    auto place = [&](auto *&dst, const auto &vec, size_t sz) {
        dst = reinterpret_cast<std::remove_reference_t<decltype(dst)>>(p);
        if (!vec.empty())
            cuda_check(cudaMemcpy(p, vec.data(), vec.size() * sizeof(vec[0]), cudaMemcpyHostToDevice),
                       "compiled DAG upload");
        p += sz;
    };
    place(im.d_ev, h.ev, s_ev);
    place(im.d_pred, h.pred, s_pred);
    place(im.d_aux, h.aux, s_aux);
    {
        const std::vector<unsigned char> tb = tables_block(h);
        place(im.d_dist, tb, s_tables);
    }
    place(im.d_vals, h.vals, s_vals);
    place(im.d_wk, h.wk_off, s_wk);
    place(im.d_stage_meta, h.stage_meta, s_meta);
    place(im.d_earliest, h.earliest, s_times);
    place(im.d_ub, h.ub, s_times);
}

// One output of a computed chunk to the host: sample-minor rows [rows][C] go to
// sample-major host rows [n][rows] from sample `off` on, transposed straight
// into pinned memory (dv: its device address) or, for a pageable buffer, into
// sample-major device rows and copied.
cudaError_t launch_transpose(const double *in, int64_t ld_in, double *out, int64_t ld_out, int64_t rows, int64_t cols,
                             cudaStream_t st) {
    return launch_transpose_f64(in, ld_in, out, ld_out, rows, cols, st);
}
cudaError_t launch_transpose(const int32_t *in, int64_t ld_in, int32_t *out, int64_t ld_out, int64_t rows,
                             int64_t cols, cudaStream_t st) {
    return launch_transpose_i32(in, ld_in, out, ld_out, rows, cols, st);
}
template <typename T>
void move_rows(const T *minor, int64_t C, T *dv, T *host, T *major, int64_t rows, int64_t off, int64_t m,
               cudaStream_t st, const char *what) {
    if (dv) {
        cuda_check(launch_transpose(minor, C, dv + off * rows, rows, rows, m, st), "transpose");
    } else if (host) {
        cuda_check(launch_transpose(minor, C, major, rows, rows, m, st), "transpose");
        cuda_check(cudaMemcpyAsync(host + off * rows, major, (size_t)(m * rows) * sizeof(T), cudaMemcpyDeviceToHost, st),
                   what);
    }
}

}  // namespace

extern "C" {

const char *mcd_last_error(void) { return mcd::g_last_error.c_str(); }
int mcd_abi_version(void) { return MCD_ABI_VERSION; }

int mcd_generator_create(mcd_generator **out) {
    return guarded([&] {
        if (!out) throw McdError(MCD_ERR_INVALID, "null output pointer");
        *out = new mcd_generator();
    });
}

void mcd_generator_destroy(mcd_generator *g) { delete g; }

int mcd_generator_set_seed(mcd_generator *g, int64_t seed) {
    return guarded([&] {
        if (!g) throw McdError(MCD_ERR_INVALID, "null generator");
        g->seed = seed;
    });
}

static int add_dist(mcd_generator *g, int32_t type, int32_t kind, double p0, double p1, double p2) {
    return guarded([&] {
        if (!g) throw McdError(MCD_ERR_INVALID, "null generator");
        g->dists.push_back(DistSpec{type, kind, p0, p1, p2, {}, {}});
    });
}

int mcd_generator_add_constant(mcd_generator *g, int32_t t, double factor) {
    return add_dist(g, t, MCD_KIND_CONSTANT, factor, 0.0, 0.0);
}
int mcd_generator_add_exponential(mcd_generator *g, int32_t t, double lambda_, double max_scale) {
    return add_dist(g, t, MCD_KIND_EXPONENTIAL, lambda_, max_scale, 0.0);
}
int mcd_generator_add_gamma(mcd_generator *g, int32_t t, double shape, double scale, double max_scale) {
    return add_dist(g, t, MCD_KIND_GAMMA, shape, scale, max_scale);
}

static int add_table(mcd_generator *g, int32_t t, int32_t kind, const double *v, int64_t nv, const double *w,
                     int64_t nw, const char *what) {
    return guarded([&] {
        if (!g) throw McdError(MCD_ERR_INVALID, "null generator");
        if (nv != nw)  // _core.cpp:119-120, 134-135
            throw McdError(MCD_ERR_RUNTIME, std::string(what) + " and weights must have same length");
        if (nv < 0 || (nv > 0 && (!v || !w))) throw McdError(MCD_ERR_INVALID, "bad table arguments");
        DistSpec s{t, kind, 0.0, 0.0, 0.0, std::vector<double>(v, v + nv), std::vector<double>(w, w + nw)};
        g->dists.push_back(std::move(s));
    });
}

int mcd_generator_add_empirical_absolute(mcd_generator *g, int32_t t, const double *values, int64_t nv,
                                         const double *weights, int64_t nw) {
    return add_table(g, t, MCD_KIND_EMP_ABS, values, nv, weights, nw, "EmpiricalAbsoluteDist: values");
}
int mcd_generator_add_empirical_relative(mcd_generator *g, int32_t t, const double *factors, int64_t nf,
                                         const double *weights, int64_t nw) {
    return add_table(g, t, MCD_KIND_EMP_REL, factors, nf, weights, nw, "EmpiricalRelativeDist: factors");
}

int mcd_dag_create(const mcd_dag_desc *desc, const mcd_generator *gen, mcd_dag **out) {
    return mcd_dag_create_ex(desc, gen, nullptr, out);
}

int mcd_dag_create_ex(const mcd_dag_desc *desc, const mcd_generator *gen, const mcd_dag_options *opts,
                      mcd_dag **out) {
    mcd_dag *g = nullptr;
    int rc = guarded([&] {
        if (!desc || !gen || !out) throw McdError(MCD_ERR_INVALID, "null argument");
        *out = nullptr;
        const int32_t nw = opts ? opts->n_warps : 0;
        if (nw < kBatchClassWarps || nw > kMaxWarps)
            throw McdError(MCD_ERR_INVALID, "n_warps must be -1 (batch class), 0 (automatic) or 1..24");
        const int32_t win = opts ? opts->window : MCD_WINDOW_AUTO;
        if (win != MCD_WINDOW_AUTO && win != MCD_WINDOW_GLOBAL)
            throw McdError(MCD_ERR_INVALID, "window must be MCD_WINDOW_AUTO (0) or MCD_WINDOW_GLOBAL (1)");
        const bool use_cache = !(opts && opts->no_cache);
        int dev = -1;
        if (cudaGetDevice(&dev) != cudaSuccess) {  // reported after validation, as before
            (void)cudaGetLastError();
            dev = -1;
        }
        std::vector<unsigned char> key;
        uint64_t hash = 0;
        std::shared_ptr<const DagImage> img;
        bool hit = false;
        if (use_cache && dev >= 0 && image_key(*desc, *gen, nw, dev, key, win)) {
            hash = hash_bytes(key);
            img = cache_find(hash, key);
            hit = img != nullptr;
        }
        if (!img) {
            auto fresh = std::make_shared<DagImage>();
            compile_dag(*desc, *gen, fresh->h, nw, win);
            cuda_check(cudaGetDevice(&fresh->device), "cudaGetDevice");
            upload_image(*fresh);
            if (!key.empty()) fresh->key = std::move(key);
            img = fresh;
            if (!img->key.empty()) cache_insert(hash, img);
        }
        g = new mcd_dag(img);
        g->cache_hit = hit;
        for (int k = 0; k < 2; ++k)
            cuda_check(cudaStreamCreateWithFlags(&g->stream[k], cudaStreamNonBlocking), "stream create");
        cuda_check(cudaMalloc(&g->d_err, 256), "error flag allocation");
        cuda_check(cudaMemset(g->d_err, 0, sizeof(int32_t)), "error flag init");
        *out = g;
    });
    if (rc != MCD_OK && g) {
        std::string keep = mcd::g_last_error;
        mcd_dag_destroy(g);
        mcd::g_last_error = keep;
    }
    return rc;
}

void mcd_dag_destroy(mcd_dag *g) {
    if (!g) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(g->device);
    for (int k = 0; k < 2; ++k)
        if (g->stream[k]) {
            cudaStreamSynchronize(g->stream[k]);
            cudaStreamDestroy(g->stream[k]);
        }
    if (g->ws) cudaFree(g->ws);
    if (g->d_err) cudaFree(g->d_err);
    cudaSetDevice(prev);
    delete g;  // the image goes with its last handle
}

int32_t mcd_dag_node_count(const mcd_dag *g) { return g ? g->h.E : -1; }
int32_t mcd_dag_activity_count(const mcd_dag *g) { return g ? g->h.L : -1; }
void *mcd_dag_stream(const mcd_dag *g) { return g ? (void *)g->stream[0] : nullptr; }

static void fill_info(const HostDag &h, mcd_dag_info *info) {
    info->n_events = h.E;
    info->n_links = h.L;
    info->n_levels = h.n_levels;
    info->n_warps = h.n_warps;
    info->n_preds = (int64_t)h.pred.size();
    info->window_slots = h.window_slots;
    info->window_in_smem = h.win_smem ? 1 : 0;
    info->n_orphan_links = h.n_orphan;
    info->n_stages = h.n_stages;
    info->smem_bytes = h.smem_total;
    info->positive = h.positive ? 1 : 0;
    info->tables_in_smem = h.tables_in_smem ? 1 : 0;
    info->n_event_pairs = h.n_pairs;
    info->block_draws = h.block_draws;
}

int mcd_dag_get_info(const mcd_dag *g, mcd_dag_info *info) {
    return guarded([&] {
        if (!g || !info) throw McdError(MCD_ERR_INVALID, "null argument");
        fill_info(g->h, info);
        info->device = g->device;
        info->device_bytes = (int64_t)g->dbytes;
        info->cache_hit = g->cache_hit ? 1 : 0;
    });
}

int mcd_dag_link_streams(const mcd_dag *g, int32_t *block, int32_t *word) {
    return guarded([&] {
        if (!g || !block || !word) throw McdError(MCD_ERR_INVALID, "null argument");
        for (int32_t l = 0; l < g->h.L; ++l) {
            block[l] = g->h.link_block[(size_t)l];
            word[l] = g->h.link_word[(size_t)l];
        }
    });
}

int mcd_dag_describe(const mcd_dag_desc *desc, const mcd_generator *gen, mcd_dag_info *info) {
    return guarded([&] {
        if (!desc || !gen || !info) throw McdError(MCD_ERR_INVALID, "null argument");
        HostDag h;
        compile_dag(*desc, *gen, h, 0);
        fill_info(h, info);
        info->device = -1;
        info->device_bytes = -1;
    });
}

int mcd_selftest_bounded_wait(int32_t *timed_out, int32_t *kernel_returned) {
    return guarded([&] {
        if (!timed_out || !kernel_returned) throw McdError(MCD_ERR_INVALID, "null argument");
        int32_t *d = nullptr;
        cudaStream_t st = nullptr;
        int32_t flags = 0;
        cudaError_t e = cudaMalloc(&d, sizeof(int32_t));
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, sizeof(int32_t), st);
        if (e == cudaSuccess) e = launch_wait_selftest(d, 1024u, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&flags, d, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (st) cudaStreamDestroy(st);
        if (d) cudaFree(d);
        cuda_check(e, "bounded-wait self-test");
        *timed_out = (flags & ERR_STAGE_TIMEOUT) ? 1 : 0;
        *kernel_returned = (flags >> 30) & 1;
    });
}

int mcd_dag_check(mcd_dag *g) {
    return guarded([&] {
        if (!g) throw McdError(MCD_ERR_INVALID, "null handle");
        cuda_check(cudaSetDevice(g->device), "cudaSetDevice");
        check_device_error(g);
    });
}

int mcd_run_device(mcd_dag *g, const int64_t *seeds, int64_t n, double *realized, double *durations,
                   int32_t *cause, int64_t ld, void *stream) {
    return guarded([&] {
        if (!g) throw McdError(MCD_ERR_INVALID, "null handle");
        if (n < 0 || ld < n || ld >= ((int64_t)1 << 29)) throw McdError(MCD_ERR_INVALID, "need 0 <= n <= ld < 2^29");
        if (n > 0 && !seeds) throw McdError(MCD_ERR_INVALID, "null seeds");
        cuda_check(cudaSetDevice(g->device), "cudaSetDevice");
        cudaStream_t st = stream ? (cudaStream_t)stream : g->stream[0];
        KArgs a = base_args(g);
        a.seeds = seeds;
        a.n = n;
        a.ld = ld;
        a.realized = realized;
        a.durations = durations;
        a.cause = cause;
        if (!g->h.win_smem && !realized) {
            ensure_ws(g, (size_t)g->h.E * (size_t)ld * 8);
            a.scratch = (double *)g->ws;
        }
        cuda_check(launch_propagate(a, false, g->h.win_smem, false, st), "propagate launch");
    });
}

int mcd_propagate_device(mcd_dag *g, const double *dur, int64_t ld_in, int64_t n, double *realized,
                         int32_t *cause, int64_t ld, void *stream) {
    return guarded([&] {
        if (!g) throw McdError(MCD_ERR_INVALID, "null handle");
        if (n < 0 || ld < n || ld_in < n || ld >= ((int64_t)1 << 29) || ld_in >= ((int64_t)1 << 29))
            throw McdError(MCD_ERR_INVALID, "need 0 <= n <= ld, ld_in < 2^29");
        if (n > 0 && g->h.L > 0 && !dur) throw McdError(MCD_ERR_INVALID, "null durations");
        cuda_check(cudaSetDevice(g->device), "cudaSetDevice");
        cudaStream_t st = stream ? (cudaStream_t)stream : g->stream[0];
        KArgs a = base_args(g);
        a.n = n;
        a.ld = ld;
        a.realized = realized;
        a.cause = cause;
        a.dur_in = dur;
        a.ld_in = ld_in;
        if (!g->h.win_smem && !realized) {
            ensure_ws(g, (size_t)g->h.E * (size_t)ld * 8);
            a.scratch = (double *)g->ws;
        }
        cuda_check(launch_propagate(a, true, g->h.win_smem, false, st), "propagate launch");
    });
}

int mcd_run_many_host(mcd_dag *g, const int64_t *seeds, int64_t n, double *realized, double *durations,
                      int32_t *cause) {
    return guarded([&] {
        if (!g) throw McdError(MCD_ERR_INVALID, "null handle");
        if (n < 0) throw McdError(MCD_ERR_INVALID, "negative sample count");
        if (n == 0) return;
        if (!seeds) throw McdError(MCD_ERR_INVALID, "null seeds");
        cuda_check(cudaSetDevice(g->device), "cudaSetDevice");
        const int64_t E = g->h.E, L = g->h.L;
        double *real_dv = device_view(realized), *dur_dv = device_view(durations);
        int32_t *cause_dv = device_view(cause);
        const bool staged = (realized && !real_dv) || (durations && !dur_dv) || (cause && !cause_dv);
        int sets = 1;
        const int64_t C = host_chunk(g, n, staged, &sets);
        ChunkBufs cb[2];
        carve(g, C, sets, staged, cb);
        ChunkPipe pipe(g, sets);
        int64_t idx = 0;
        for (int64_t off = 0; off < n; off += C, ++idx) {
            const ChunkBufs &b = cb[idx & 1];
            const int64_t m = std::min(C, n - off);
            pipe.begin_compute(idx);
            cuda_check(cudaMemcpyAsync(b.seeds, seeds + off, (size_t)m * 8, cudaMemcpyHostToDevice, pipe.compute),
                       "seed upload");
            KArgs a = base_args(g);
            a.seeds = b.seeds;
            a.n = m;
            a.ld = C;
            a.realized = b.real_minor;  // always: also the spill rows of a global window
            a.durations = durations ? b.dur_minor : nullptr;
            a.cause = cause ? b.cause_minor : nullptr;
            cuda_check(launch_propagate(a, false, g->h.win_smem, false, pipe.compute), "propagate launch");
            pipe.begin_transfer(idx);
            move_rows(b.real_minor, C, real_dv, realized, b.real_major, E, off, m, pipe.transfer, "realized download");
            move_rows(b.dur_minor, C, dur_dv, durations, b.dur_major, L, off, m, pipe.transfer, "durations download");
            move_rows(b.cause_minor, C, cause_dv, cause, b.cause_major, E, off, m, pipe.transfer, "cause download");
            pipe.end_transfer(idx);
        }
        check_device_error(g);
    });
}

int mcd_propagate_host(mcd_dag *g, const double *durations, int64_t n, double *realized, int32_t *cause) {
    return guarded([&] {
        if (!g) throw McdError(MCD_ERR_INVALID, "null handle");
        if (n < 0) throw McdError(MCD_ERR_INVALID, "negative sample count");
        if (n == 0) return;
        if (!durations && g->h.L > 0) throw McdError(MCD_ERR_INVALID, "null durations");
        cuda_check(cudaSetDevice(g->device), "cudaSetDevice");
        const int64_t E = g->h.E, L = g->h.L;
        const double *dur_dv = device_view(durations);
        double *real_dv = device_view(realized);
        int32_t *cause_dv = device_view(cause);
        const bool staged = (L > 0 && !dur_dv) || (realized && !real_dv) || (cause && !cause_dv);
        int sets = 1;
        const int64_t C = host_chunk(g, n, staged, &sets);
        ChunkBufs cb[2];
        carve(g, C, sets, staged, cb);
        ChunkPipe pipe(g, sets);
        int64_t idx = 0;
        for (int64_t off = 0; off < n; off += C, ++idx) {
            const ChunkBufs &b = cb[idx & 1];
            const int64_t m = std::min(C, n - off);
            pipe.begin_compute(idx);
            cudaStream_t cs = pipe.compute;
            if (L > 0 && dur_dv) {
                cuda_check(launch_transpose_f64(dur_dv + off * L, L, b.dur_minor, C, m, L, cs), "transpose");
            } else if (L > 0) {
                cuda_check(cudaMemcpyAsync(b.dur_major, durations + off * L, (size_t)(m * L) * 8,
                                           cudaMemcpyHostToDevice, cs),
                           "durations upload");
                cuda_check(launch_transpose_f64(b.dur_major, L, b.dur_minor, C, m, L, cs), "transpose");
            }
            KArgs a = base_args(g);
            a.n = m;
            a.ld = C;
            a.realized = b.real_minor;
            a.cause = cause ? b.cause_minor : nullptr;
            a.dur_in = b.dur_minor;
            a.ld_in = C;
            cuda_check(launch_propagate(a, true, g->h.win_smem, false, cs), "propagate launch");
            pipe.begin_transfer(idx);
            move_rows(b.real_minor, C, real_dv, realized, b.real_major, E, off, m, pipe.transfer, "realized download");
            move_rows(b.cause_minor, C, cause_dv, cause, b.cause_major, E, off, m, pipe.transfer, "cause download");
            pipe.end_transfer(idx);
        }
        check_device_error(g);
    });
}

// Statistics of n samples into device outputs, asynchronously on st.  The
// handle's workspace holds the per-event accumulators (and, when the window is
// not on chip, scratch realized rows for one chunk of samples at a time).
static void stats_device(mcd_dag *g, const int64_t *seeds, int64_t seed0, int64_t n, const mcd_stats *out,
                         cudaStream_t st) {
    const HostDag &h = g->h;
    const size_t E = (size_t)h.E;
    const StatsParams sp = stats_params(h, n);
    int64_t C = n;
    size_t scratch_bytes = 0;
    if (!h.win_smem) {
        C = std::max<int64_t>(32, std::min<int64_t>(n, (int64_t)((512ull << 20) / std::max<size_t>(E * 8, 1)) / 32 * 32));
        scratch_bytes = align_up(E * (size_t)C * 8, 256);
    }
    const size_t acc_bytes = align_up(E * 8, 256), hist_bytes = align_up(E * kHistStride * 4, 256),
                 te_bytes = align_up(E * 8, 256);
    ensure_ws(g, acc_bytes + hist_bytes + te_bytes + scratch_bytes);
    auto *acc = reinterpret_cast<unsigned long long *>(g->ws);
    auto *hist = reinterpret_cast<uint32_t *>(g->ws + acc_bytes);
    auto *te = reinterpret_cast<long long *>(g->ws + acc_bytes + hist_bytes);
    double *scratch =
        scratch_bytes ? reinterpret_cast<double *>(g->ws + acc_bytes + hist_bytes + te_bytes) : nullptr;
    cuda_check(cudaMemsetAsync(g->ws, 0, acc_bytes + hist_bytes, st), "accumulator reset");
    if (sp.fixed) cuda_check(launch_event_ticks(g->d_earliest, h.E, sp.q, te, st), "earliest ticks");
    for (int64_t off = 0; off < n; off += C) {
        const int64_t m = std::min(C, n - off);
        KArgs a = base_args(g);
        a.seeds = seeds ? seeds + off : nullptr;
        a.seed0 = seed0 + off;
        a.n = m;
        a.ld = C;
        a.scratch = scratch;
        a.stats_fixed = sp.fixed;
        a.tick_q = sp.q;
        a.bin_mul = sp.bin_mul;
        a.hist_inv_w = sp.inv_w;
        a.acc = acc;
        a.te = te;
        a.hist = hist;
        a.hist_lane = (int64_t)h.E * kHistStride * 4 <= kHistLaneBytes ? 1 : 0;
        cuda_check(launch_propagate(a, false, h.win_smem, true, st), "statistics launch");
    }
    FArgs f{};
    f.acc = acc;
    f.hist = hist;
    f.earliest = g->d_earliest;
    f.ub = g->d_ub;
    f.E = h.E;
    f.stats_fixed = sp.fixed;
    f.tick_q = sp.q;
    f.bin_w = sp.bin_w;
    f.n = n;
    f.mean = out->mean;
    f.p50 = out->p50;
    f.p90 = out->p90;
    f.p99 = out->p99;
    f.p_on_time = out->p_on_time;
    cuda_check(launch_stats_finish(f, st), "statistics finish");
    if (out->hist)
        cuda_check(cudaMemcpyAsync(out->hist, hist, E * kHistStride * 4, cudaMemcpyDeviceToDevice, st),
                   "histogram copy");
}

int mcd_stats_device(mcd_dag *g, const int64_t *seeds, int64_t seed0, int64_t n, const mcd_stats *out,
                     void *stream) {
    return guarded([&] {
        if (!g || !out) throw McdError(MCD_ERR_INVALID, "null argument");
        if (n <= 0 || n > (int64_t)1 << 31) throw McdError(MCD_ERR_INVALID, "need 0 < n <= 2^31 samples");
        cuda_check(cudaSetDevice(g->device), "cudaSetDevice");
        stats_device(g, seeds, seed0, n, out, stream ? (cudaStream_t)stream : g->stream[0]);
    });
}

int mcd_stats_host(mcd_dag *g, const int64_t *seeds, int64_t seed0, int64_t n, const mcd_stats *out) {
    return guarded([&] {
        if (!g || !out) throw McdError(MCD_ERR_INVALID, "null argument");
        if (n <= 0 || n > (int64_t)1 << 31) throw McdError(MCD_ERR_INVALID, "need 0 < n <= 2^31 samples");
        cuda_check(cudaSetDevice(g->device), "cudaSetDevice");
        cudaStream_t st = g->stream[0];
        const size_t E = (size_t)g->h.E;
        // device copies of the seeds and the outputs live after every region
        // stats_device carves (accumulators, histograms, earliest ticks, and the
        // chunk scratch when the window is off chip), so none of them aliases
        const size_t acc_bytes = align_up(E * 8, 256), hist_bytes = align_up(E * kHistStride * 4, 256),
                     te_bytes = align_up(E * 8, 256);
        const size_t seeds_bytes = seeds ? align_up((size_t)n * 8, 256) : 0;
        const size_t out_bytes = align_up(E * 8, 256);
        const size_t hist_out = out->hist ? hist_bytes : 0;
        // reserve: [accumulators | hist | ticks | scratch] ... [outputs (5 x E doubles) | hist copy | seeds]
        const size_t head = 5 * out_bytes + hist_out + seeds_bytes;
        size_t scratch_bytes = 0;
        if (!g->h.win_smem) {
            const int64_t C = std::max<int64_t>(32, std::min<int64_t>(n, (int64_t)((512ull << 20) / std::max<size_t>(E * 8, 1)) / 32 * 32));
            scratch_bytes = align_up(E * (size_t)C * 8, 256);
        }
        ensure_ws(g, acc_bytes + hist_bytes + te_bytes + scratch_bytes + head);
        // stats_device carves its regions from the start of the workspace, so the
        // staging area goes at the end
        char *tail = g->ws + g->ws_bytes - head;
        double *o[5];
        for (int k = 0; k < 5; ++k) o[k] = reinterpret_cast<double *>(tail + k * out_bytes);
        uint32_t *dh = out->hist ? reinterpret_cast<uint32_t *>(tail + 5 * out_bytes) : nullptr;
        int64_t *ds = seeds ? reinterpret_cast<int64_t *>(tail + 5 * out_bytes + hist_out) : nullptr;
        if (seeds) cuda_check(cudaMemcpyAsync(ds, seeds, (size_t)n * 8, cudaMemcpyHostToDevice, st), "seed upload");
        mcd_stats dev{out->mean ? o[0] : nullptr, out->p50 ? o[1] : nullptr, out->p90 ? o[2] : nullptr,
                      out->p99 ? o[3] : nullptr, out->p_on_time ? o[4] : nullptr, dh};
        stats_device(g, ds, seed0, n, &dev, st);
        double *host_out[5] = {out->mean, out->p50, out->p90, out->p99, out->p_on_time};
        for (int k = 0; k < 5; ++k)
            if (host_out[k])
                cuda_check(cudaMemcpyAsync(host_out[k], o[k], E * 8, cudaMemcpyDeviceToHost, st), "stats download");
        if (out->hist)
            cuda_check(cudaMemcpyAsync(out->hist, dh, E * kHistStride * 4, cudaMemcpyDeviceToHost, st),
                       "histogram download");
        check_device_error(g);
    });
}

// Statistics without any device allocation: the per-event accumulators live in
// the library's fixed 34 MiB device array instead of the handle's workspace.
// For callers that cannot allocate (their device memory belongs to another
// allocator, or a cudaMalloc would stall their latency-critical loop).  The
// first call on a device looks the array's address up; calls share the array,
// so calls that overlap on the GPU race.
int mcd_stats_device_noalloc(mcd_dag *g, const int64_t *seeds, int64_t seed0, int64_t n, const mcd_stats *out,
                             void *stream) {
    return guarded([&] {
        if (!g || !out) throw McdError(MCD_ERR_INVALID, "null argument");
        if (n <= 0 || n > (int64_t)1 << 31) throw McdError(MCD_ERR_INVALID, "need 0 < n <= 2^31 samples");
        const HostDag &h = g->h;
        if (!h.win_smem)
            throw McdError(MCD_ERR_INVALID,
                           "mcd_stats_device_noalloc needs a DAG whose window fits in shared memory");
        cuda_check(cudaSetDevice(g->device), "cudaSetDevice");
        void *base = nullptr;
        size_t cap = 0;
        cuda_check(noalloc_scratch(&base, &cap), "fixed scratch lookup");
        const size_t E = (size_t)h.E;
        const size_t acc_bytes = align_up(E * 8, 256), hist_bytes = align_up(E * kHistStride * 4, 256),
                     te_bytes = align_up(E * 8, 256);
        if (h.E > MCD_NOALLOC_MAX_EVENTS || acc_bytes + hist_bytes + te_bytes > cap)
            throw McdError(MCD_ERR_INVALID, "mcd_stats_device_noalloc supports at most " +
                                                std::to_string(MCD_NOALLOC_MAX_EVENTS) + " events; this DAG has " +
                                                std::to_string(h.E));
        cudaStream_t st = stream ? (cudaStream_t)stream : g->stream[0];
        auto *acc = reinterpret_cast<unsigned long long *>(base);
        auto *hist = reinterpret_cast<uint32_t *>(static_cast<char *>(base) + acc_bytes);
        auto *te = reinterpret_cast<long long *>(static_cast<char *>(base) + acc_bytes + hist_bytes);
        // the array keeps the previous call's counts: start from zero
        cuda_check(cudaMemsetAsync(base, 0, acc_bytes + hist_bytes, st), "fixed scratch reset");
        const StatsParams sp = stats_params(h, n);
        if (sp.fixed) cuda_check(launch_event_ticks(g->d_earliest, h.E, sp.q, te, st), "earliest ticks");
        KArgs a = base_args(g);
        a.seeds = seeds;
        a.seed0 = seed0;
        a.n = n;
        a.ld = n;
        a.stats_fixed = sp.fixed;
        a.tick_q = sp.q;
        a.bin_mul = sp.bin_mul;
        a.hist_inv_w = sp.inv_w;
        a.acc = acc;
        a.te = te;
        a.hist = hist;
        a.hist_lane = (int64_t)h.E * kHistStride * 4 <= kHistLaneBytes ? 1 : 0;
        cuda_check(launch_propagate(a, false, true, true, st), "statistics launch");
        FArgs f{};
        f.acc = acc;
        f.hist = hist;
        f.earliest = g->d_earliest;
        f.ub = g->d_ub;
        f.E = h.E;
        f.stats_fixed = sp.fixed;
        f.tick_q = sp.q;
        f.bin_w = sp.bin_w;
        f.n = n;
        f.mean = out->mean;
        f.p50 = out->p50;
        f.p90 = out->p90;
        f.p99 = out->p99;
        f.p_on_time = out->p_on_time;
        cuda_check(launch_stats_finish(f, st), "statistics finish");
        if (out->hist)
            cuda_check(cudaMemcpyAsync(out->hist, hist, E * kHistStride * 4, cudaMemcpyDeviceToDevice, st),
                       "histogram copy");
    });
}

int mcd_stats_bin_width(const mcd_dag *g, int64_t n, double *out) {
    return guarded([&] {
        if (!g || !out) throw McdError(MCD_ERR_INVALID, "null argument");
        *out = stats_params(g->h, n).bin_w;
    });
}

int mcd_host_alloc(size_t bytes, void **out) {
    return guarded([&] {
        if (!out) throw McdError(MCD_ERR_INVALID, "null output pointer");
        *out = nullptr;
        cuda_check(cudaHostAlloc(out, std::max<size_t>(bytes, 1), cudaHostAllocDefault), "pinned allocation");
    });
}

void mcd_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"
