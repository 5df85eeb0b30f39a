// mcd_server.cpp -- continuous-batching request server (no reference counterpart).
//
// Requests are (DAG, generator, seed0, n samples) asking for per-event
// statistics.  submit() copies the inputs and returns a ticket at once.
//   - A pool of host threads compiles the DAGs (mcd_compile.cpp) with warps per
//     CTA from each DAG's width (rounded to 2, 4, 8, 12 or 24), waits until the
//     request's device blocks fit the memory budget, takes them from the
//     stream-ordered allocator and uploads on its own stream: uploads run in
//     parallel, off the scheduler.
//   - Compiled DAGs stay resident on the device after their requests finish,
//     keyed by their content (the DAG's arrays, the generator, warps per CTA):
//     a request for a DAG already resident skips the compile and the upload of
//     its records and only gets accumulators of its own.  Resident DAGs no
//     request uses are evicted, least recently used first, when the budget
//     needs room.  (Draws need no per-request generator state on the device:
//     Philox is keyed by the sample's seed, the link and the attempt.)
//   - Requests are batched by class: equal warps per CTA, equal CTAs per SM for
//     their shared-memory layout (so no request lowers another's occupancy) and
//     the same kernel variant (window in shared memory or in per-CTA scratch
//     rows, positive times or not, tables in shared memory or not).
//   - One scheduler thread, whenever one of its stream slots is free, launches
//     the uploaded requests of the class of the oldest waiting request as one
//     batch (the persistent k_batch_stats over (request, tile) items, then the
//     batched finish and the copy of the statistics to pinned host memory);
//     batches on different slots overlap on the GPU.  It polls the slots'
//     events, completes tickets and returns memory.
// A request's statistics are the same alone and in any mix: every request has
// its own accumulators and the accumulation is exact integer arithmetic.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "mcd_handle.hpp"

namespace mcd {
cudaError_t launch_batch_stats(const BatchArgs &b, bool win_smem, bool positive, bool tsmem, int n_warps, size_t smem,
                               int grid,
                               cudaStream_t st);
cudaError_t batch_blocks_per_sm(bool win_smem, bool positive, bool tsmem, int n_warps, size_t smem, int *out);
cudaError_t launch_batch_finish(const FArgs *fs, int32_t n_dags, int32_t max_events, cudaStream_t st);
}  // namespace mcd

using namespace mcd;
using Clock = std::chrono::steady_clock;

namespace {

enum State : int { Q_COMPILE = 0, Q_READY = 1, Q_RUNNING = 2, Q_DONE = 3, Q_FAILED = 4 };

// Offsets inside a resident DAG's device block: its compiled records.
struct ImgLayout {
    size_t ev, pred, aux, tables, vals, wk, meta, earliest, ub, total;
};

ImgLayout img_layout_of(const HostDag &h) {
    ImgLayout L{};
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o += align_up(std::max<size_t>(bytes, 1), 256);
        return at;
    };
    L.ev = take(h.ev.size() * sizeof(EvRec));
    L.pred = take(h.pred.size() * sizeof(PredRec));
    L.aux = take(h.aux.size() * sizeof(LinkRec));
    L.tables = take(tables_bytes(h));
    L.vals = take(h.vals.size() * sizeof(double));
    L.wk = take(h.wk_off.size() * 4);
    L.meta = take(h.stage_meta.size() * 4);
    L.earliest = take((size_t)h.E * 8);
    L.ub = take((size_t)h.E * 8);
    L.total = o;
    return L;
}

// Offsets inside a request's own device block: the earliest times in the
// request's ticks, then the error flag and the accumulators (zeroed at upload),
// then the statistics.
struct RqLayout {
    size_t te, err, acc, hist, out, total;
};

RqLayout rq_layout_of(int32_t E) {
    RqLayout L{};
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o += align_up(std::max<size_t>(bytes, 1), 256);
        return at;
    };
    L.te = take((size_t)E * 8);
    L.err = take(4);
    L.acc = take((size_t)E * 8);
    L.hist = take((size_t)E * kHistStride * 4);
    L.out = take((size_t)E * 5 * 8);
    L.total = o;
    return L;
}

// A compiled DAG, shared by the requests for it: host records from its compile
// on, device records from its upload until it is evicted (the host records stay,
// so a request that waited while it was evicted uploads them again).
struct Resident {
    std::vector<unsigned char> key;  // empty: not shared (malformed arrays)
    uint64_t hash = 0;
    HostDag h;
    int32_t n_dist = 0, n_alias = 0, n_aux = 0;  // record counts for the kernel arguments
    ImgLayout lay{};
    char *dimg = nullptr;
    size_t bytes = 0;
    int32_t per_sm = 1;              // batch class: (h.n_warps, per_sm)
    double tile_cost = 0;            // work per 32-sample tile, for longest-first ordering
    int refs = 0;                    // admitted requests holding it (until their batch completes)
    bool compiled = false;           // h, lay, bytes, per_sm valid
    bool uploading = false;          // an admitted request's thread is uploading the records
    bool on_device = false;          // dimg holds the records
    bool failed = false;
    std::string error;
    uint64_t last_use = 0;
};

struct Request {
    int64_t ticket = 0;
    // inputs (copied at submit, dropped after compile)
    std::vector<double> earliest, act_duration;
    std::vector<int32_t> act_idx, act_type, target, pred_src, pred_act;
    std::vector<int64_t> pred_offsets;
    double max_delay = 0.0;
    mcd_generator gen;
    int64_t seed0 = 0, n = 0;
    // the compiled DAG (shared) and this request's own device block
    std::shared_ptr<Resident> res;
    RqLayout lay{};
    size_t bytes = 0;       // own device block
    int32_t E = 0;
    std::string error;
    // device (uploaded until the batch completes)
    char *dblock = nullptr;
    KArgs ka{};
    FArgs fa{};
    // results
    std::vector<double> out;  // 5 x E: mean, p50, p90, p99, p_on_time
    std::atomic<int> state{Q_COMPILE};
    Clock::time_point t_submit, t_done;
};

// Buffers grow geometrically and are never released while the server runs:
// cudaFree and cudaFreeHost synchronise the whole device, which would stall the
// scheduler behind every batch in flight.  Device metadata is stream-ordered;
// outgrown pinned buffers are retired and freed with the server.
struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    bool busy = false;
    std::vector<Request *> batch;
    char *meta_dev = nullptr;   // KArgs[], FArgs[], items, queue head
    char *meta_pinned = nullptr;
    size_t meta_bytes = 0;
    double *scratch = nullptr;  // per-CTA realized rows of a batch whose windows are off chip
    size_t scratch_bytes = 0;
    double *pinned = nullptr;   // statistics of the batch, host side
    size_t pinned_elems = 0;
    std::vector<void *> retired;  // outgrown pinned buffers
};

}  // namespace

struct mcd_server {
    mcd_server_options opt{};
    int device = 0, sms = 1;
    cudaMemPool_t pool = nullptr;
    std::mutex mu;
    std::condition_variable cv_compile, cv_sched, cv_done, cv_budget;
    std::deque<Request *> to_compile, ready;
    std::unordered_map<int64_t, std::unique_ptr<Request>> all;
    std::vector<Slot> slots;
    std::vector<std::thread> compilers;
    std::thread scheduler;
    std::atomic<bool> stop{false};
    int64_t next_ticket = 1;
    int64_t bytes_in_use = 0;
    int64_t completed = 0, launched_batches = 0, running = 0, pending = 0;
    double compile_s = 0.0, upload_s = 0.0, launch_s = 0.0;
    // resident compiled DAGs by content hash; their bytes count in bytes_in_use
    std::unordered_multimap<uint64_t, std::shared_ptr<Resident>> residents;
    std::condition_variable cv_resident;
    uint64_t use_clock = 0;
    int64_t resident_hits = 0, resident_bytes = 0, evicted = 0;
    char *zeros = nullptr;  // pinned zero bytes: accumulators are cleared by the copy engines
    std::string fatal;      // a CUDA failure of the scheduler: every later call reports it
};

namespace {
constexpr size_t kZeroBytes = 8u << 20;
}  // namespace

namespace {

double seconds_since(Clock::time_point t0) { return std::chrono::duration<double>(Clock::now() - t0).count(); }

// Kernel and finish arguments of an uploaded request.
void request_args(Request *r) {
    const HostDag &h = r->res->h;
    const ImgLayout &I = r->res->lay;
    const RqLayout &L = r->lay;
    const char *g = r->res->dimg;
    char *b = r->dblock;
    const StatsParams sp = stats_params(h, r->n);
    KArgs &a = r->ka;
    a = KArgs{};
    a.ev = reinterpret_cast<const EvRec *>(g + I.ev);
    a.pred = reinterpret_cast<const PredRec *>(g + I.pred);
    a.aux = reinterpret_cast<const LinkRec *>(g + I.aux);
    a.dist = reinterpret_cast<const DistParam *>(g + I.tables);
    a.vals = reinterpret_cast<const double *>(g + I.vals);
    a.wk_off = reinterpret_cast<const int32_t *>(g + I.wk);
    a.stage_meta = reinterpret_cast<const int32_t *>(g + I.meta);
    a.n_stages = h.n_stages;
    a.n_warps = h.n_warps;
    a.n_aux = r->res->n_aux;  // the host records themselves are gone after the upload
    a.window_slots = h.window_slots;
    a.n_dist = r->res->n_dist;
    a.n_alias = r->res->n_alias;
    a.tables_in_smem = h.tables_in_smem ? 1 : 0;
    a.win_smem = h.win_smem ? 1 : 0;
    a.positive = h.positive ? 1 : 0;
    a.stage_bytes = h.stage_bytes;
    a.smem_stage_off = h.smem_stage_off;
    a.smem_tables_off = h.smem_tables_off;
    a.smem_bar_off = h.smem_bar_off;
    a.smem_total = h.smem_total;
    a.err = reinterpret_cast<int32_t *>(b + L.err);
    a.seeds = nullptr;
    a.seed0 = r->seed0;
    a.n = r->n;
    a.stats_fixed = sp.fixed;
    a.tick_q = sp.q;
    a.bin_mul = sp.bin_mul;
    a.hist_inv_w = sp.inv_w;
    a.acc = reinterpret_cast<unsigned long long *>(b + L.acc);
    a.te = reinterpret_cast<const long long *>(b + L.te);
    a.hist = reinterpret_cast<uint32_t *>(b + L.hist);
    FArgs &f = r->fa;
    f = FArgs{};
    f.acc = a.acc;
    f.hist = a.hist;
    f.earliest = reinterpret_cast<const double *>(g + I.earliest);
    f.ub = reinterpret_cast<const double *>(g + I.ub);
    f.E = h.E;
    f.stats_fixed = sp.fixed;
    f.tick_q = sp.q;
    f.bin_w = sp.bin_w;
    f.n = r->n;
    double *o = reinterpret_cast<double *>(b + L.out);
    f.mean = o;
    f.p50 = o + h.E;
    f.p90 = o + 2 * (size_t)h.E;
    f.p99 = o + 3 * (size_t)h.E;
    f.p_on_time = o + 4 * (size_t)h.E;
}

// A compile thread's pinned staging buffer: records are gathered there and
// uploaded in one DMA copy (a copy from pageable memory is staged by the CUDA
// driver on the calling thread and serialises with other threads' CUDA calls).
struct Staging {
    char *p = nullptr;
    size_t bytes = 0;
    std::vector<void *> retired;  // outgrown buffers, freed when the thread ends
    ~Staging() {
        if (p) cudaFreeHost(p);
        for (void *q : retired) cudaFreeHost(q);
    }
};

// Grows a compile thread's pinned staging buffer to at least `bytes`.
void stage_reserve(Staging &stage, size_t bytes) {
    if (bytes <= stage.bytes) return;
    const size_t want = std::max(bytes, stage.bytes * 2);
    if (stage.p) stage.retired.push_back(stage.p);
    stage.p = nullptr;
    stage.bytes = 0;
    cuda_check(cudaHostAlloc(reinterpret_cast<void **>(&stage.p), want, cudaHostAllocDefault), "staging");
    stage.bytes = want;
}

// Uploads a compiled DAG's records into its resident block; returns when the
// copy has landed.  Only copies: a kernel would queue behind the persistent
// batch launches that hold every SM, while the copy engines are free.
void upload_image(Resident *res, cudaStream_t st, Staging &stage) {
    const HostDag &h = res->h;
    const ImgLayout &L = res->lay;
    stage_reserve(stage, L.total);
    auto put = [&](size_t off, const void *src, size_t bytes) {
        if (bytes) std::memcpy(stage.p + off, src, bytes);
    };
    put(L.ev, h.ev.data(), h.ev.size() * sizeof(EvRec));
    put(L.pred, h.pred.data(), h.pred.size() * sizeof(PredRec));
    put(L.aux, h.aux.data(), h.aux.size() * sizeof(LinkRec));
    {
        const std::vector<unsigned char> tb = tables_block(h);
        put(L.tables, tb.data(), tb.size());
    }
    put(L.vals, h.vals.data(), h.vals.size() * sizeof(double));
    put(L.wk, h.wk_off.data(), h.wk_off.size() * 4);
    put(L.meta, h.stage_meta.data(), h.stage_meta.size() * 4);
    put(L.earliest, h.earliest.data(), (size_t)h.E * 8);
    put(L.ub, h.ub.data(), (size_t)h.E * 8);
    cuda_check(cudaMallocAsync(reinterpret_cast<void **>(&res->dimg), res->bytes, st), "resident allocation");
    cuda_check(cudaMemcpyAsync(res->dimg, stage.p, L.total, cudaMemcpyHostToDevice, st), "resident upload");
    cuda_check(cudaStreamSynchronize(st), "resident upload sync");  // the staging buffer is reused next
}

// Uploads a request's own block: the earliest times in the request's ticks,
// then zeros over the error flag and the accumulators.
void upload_request(const mcd_server *S, Request *r, cudaStream_t st, Staging &stage) {
    const HostDag &h = r->res->h;
    const RqLayout &L = r->lay;
    stage_reserve(stage, L.err);
    const StatsParams sp = stats_params(h, r->n);
    auto *te = reinterpret_cast<long long *>(stage.p + L.te);
    for (int32_t e = 0; e < h.E; ++e) {
        long long b;
        std::memcpy(&b, &h.earliest[(size_t)e], 8);
        te[e] = sp.fixed ? ticks_of(b, sp.q) : 0ll;
    }
    cuda_check(cudaMallocAsync(reinterpret_cast<void **>(&r->dblock), r->bytes, st), "request allocation");
    char *b = r->dblock;
    cuda_check(cudaMemcpyAsync(b, stage.p, L.err, cudaMemcpyHostToDevice, st), "request upload");
    for (size_t off = L.err; off < L.out; off += kZeroBytes)  // flags + accumulators
        cuda_check(cudaMemcpyAsync(b + off, S->zeros, std::min(kZeroBytes, L.out - off), cudaMemcpyHostToDevice, st),
                   "request reset");
    cuda_check(cudaStreamSynchronize(st), "request upload sync");  // the staging buffer is reused next
}

// Waits (caller holds the lock) until `bytes` more fit the budget, evicting
// device records of DAGs no admitted request holds (other than `keep`), least
// recently used first.  False when the server stops.  Every byte of the budget
// is held by an admitted request (which runs and returns it) or by evictable
// records, so a request that fits the budget alone is admitted eventually.
bool admit(mcd_server *S, std::unique_lock<std::mutex> &lk, size_t bytes, cudaStream_t st, const Resident *keep) {
    for (;;) {
        if (S->stop) return false;
        if (S->bytes_in_use + (int64_t)bytes <= S->opt.memory_budget) {
            S->bytes_in_use += (int64_t)bytes;
            return true;
        }
        auto lru = S->residents.end();
        for (auto it = S->residents.begin(); it != S->residents.end(); ++it) {
            const Resident *c = it->second.get();
            if (c != keep && c->on_device && !c->uploading && c->refs == 0 &&
                (lru == S->residents.end() || c->last_use < lru->second->last_use))
                lru = it;
        }
        if (lru == S->residents.end()) {  // nothing to evict: wait for running requests to finish
            S->cv_budget.wait(lk);
            continue;
        }
        std::shared_ptr<Resident> victim = lru->second;
        S->residents.erase(lru);
        cudaFreeAsync(victim->dimg, st);  // no batch uses it (refs == 0)
        victim->dimg = nullptr;
        victim->on_device = false;
        S->bytes_in_use -= (int64_t)victim->bytes;
        S->resident_bytes -= (int64_t)victim->bytes;
        S->evicted += 1;
    }
}

// A DAG whose compile or upload failed (caller holds the lock): unlisted, and
// every request waiting for it wakes to the error.
void fail_resident(mcd_server *S, const std::shared_ptr<Resident> &R) {
    R->failed = true;
    auto range = S->residents.equal_range(R->hash);
    for (auto it = range.first; it != range.second; ++it)
        if (it->second == R) {
            S->residents.erase(it);
            break;
        }
    S->cv_resident.notify_all();
}

// Drops a request's hold on its resident DAG (caller holds the lock).
void release_resident(mcd_server *S, Request *r) {
    if (!r->res) return;
    r->res->refs -= 1;
    r->res->last_use = ++S->use_clock;
    S->cv_budget.notify_all();
}

template <typename T>
void drop(std::vector<T> &v) {
    std::vector<T>().swap(v);
}

void compile_loop(mcd_server *S) {
    cudaStream_t st = nullptr;
    Staging stage;
    if (cudaSetDevice(S->device) != cudaSuccess || cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->fatal.empty()) S->fatal = "compile thread: no CUDA stream";
        S->cv_done.notify_all();
        return;
    }
    for (;;) {
        Request *r = nullptr;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_compile.wait(lk, [&] { return S->stop || !S->to_compile.empty(); });
            if (S->stop) break;
            r = S->to_compile.front();
            S->to_compile.pop_front();
        }
        bool holds_budget = false;
        try {
            const Clock::time_point t0 = Clock::now();
            mcd_dag_desc d{};
            d.n_events = (int32_t)r->earliest.size();
            d.earliest = r->earliest.data();
            d.n_activities = (int32_t)r->act_idx.size();
            d.act_idx = r->act_idx.data();
            d.act_duration = r->act_duration.data();
            d.act_type = r->act_type.data();
            d.n_targets = (int32_t)r->target.size();
            d.target = r->target.data();
            d.pred_offsets = r->pred_offsets.data();
            d.pred_src = r->pred_src.data();
            d.pred_act = r->pred_act.data();
            d.max_delay = r->max_delay;
            const int32_t warps = S->opt.n_warps > 0 ? S->opt.n_warps : kBatchClassWarps;
            // The compiled DAG of this content (shared with other requests), or a new
            // one this thread compiles.  No reference is taken yet: a request that
            // waits for memory holds neither budget nor a resident DAG, so the
            // requests holding memory are always ones that will run and return it.
            std::vector<unsigned char> key;
            const bool keyed = image_key(d, r->gen, warps, S->device, key);
            const uint64_t hash = keyed ? hash_bytes(key) : 0;
            std::shared_ptr<Resident> R;
            bool mine = false;
            {
                std::unique_lock<std::mutex> lk(S->mu);
                if (keyed) {
                    auto range = S->residents.equal_range(hash);
                    for (auto it = range.first; it != range.second; ++it)
                        if (!it->second->failed && it->second->key == key) {
                            R = it->second;
                            break;
                        }
                }
                if (!R) {
                    R = std::make_shared<Resident>();
                    R->hash = hash;
                    R->key = std::move(key);
                    S->residents.emplace(hash, R);  // found by later requests (an empty key matches none)
                    mine = true;
                }
            }
            if (mine) {
                try {
                    compile_dag(d, r->gen, R->h, warps);
                    R->lay = img_layout_of(R->h);
                    R->bytes = R->lay.total;
                    if ((int64_t)(R->bytes + rq_layout_of(R->h.E).total) > S->opt.memory_budget)
                        throw McdError(MCD_ERR_INVALID, "request needs more device memory than the server's budget");
                    int per_sm = 0;
                    cuda_check(batch_blocks_per_sm(R->h.win_smem, R->h.positive, R->h.tables_in_smem,
                                                   R->h.n_warps, (size_t)R->h.smem_total, &per_sm),
                               "occupancy query");
                    R->per_sm = std::max(1, per_sm);
                    R->tile_cost = (double)R->h.pred.size() + 2.0 * R->h.E;
                    R->n_dist = (int32_t)R->h.dist.size();
                    R->n_alias = (int32_t)R->h.alias.size();
                    R->n_aux = (int32_t)R->h.aux.size();
                    std::lock_guard<std::mutex> lk(S->mu);
                    S->compile_s += seconds_since(t0);
                    R->compiled = true;
                    S->cv_resident.notify_all();
                } catch (const std::exception &e) {
                    std::lock_guard<std::mutex> lk(S->mu);
                    R->error = e.what();
                    fail_resident(S, R);
                    throw;
                }
            } else {  // another request's thread compiles or compiled it
                std::unique_lock<std::mutex> lk(S->mu);
                S->cv_resident.wait(lk, [&] { return S->stop || R->compiled || R->failed; });
                if (R->failed) throw McdError(MCD_ERR_INVALID, R->error);
                if (!R->compiled) break;  // the server stops
                S->resident_hits += 1;
            }
            drop(r->earliest);
            drop(r->act_duration);
            drop(r->act_idx);
            drop(r->act_type);
            drop(r->target);
            drop(r->pred_src);
            drop(r->pred_act);
            drop(r->pred_offsets);
            // this request's own block, and the DAG's records when they are not on the
            // device (never uploaded, or evicted while this request waited): admitted
            // together, and only then is the DAG referenced
            r->E = R->h.E;
            r->lay = rq_layout_of(r->E);
            r->bytes = r->lay.total;
            bool upload_dag = false;
            {
                std::unique_lock<std::mutex> lk(S->mu);
                for (;;) {
                    if (R->failed) throw McdError(MCD_ERR_INVALID, R->error);
                    const size_t need = r->bytes + (R->on_device || R->uploading ? 0 : R->bytes);
                    if (!admit(S, lk, need, st, R.get())) break;
                    const bool there = R->on_device || R->uploading;
                    if (R->failed || (!there && need == r->bytes)) {
                        // it failed, or was evicted, while this request waited: give the room back
                        S->bytes_in_use -= (int64_t)need;
                        S->cv_budget.notify_all();
                        continue;
                    }
                    if (there && need > r->bytes) {  // another request uploaded it meanwhile
                        S->bytes_in_use -= (int64_t)(need - r->bytes);
                        S->cv_budget.notify_all();
                    } else if (!there) {  // this thread uploads the records
                        R->uploading = true;
                        upload_dag = true;
                        S->resident_bytes += (int64_t)R->bytes;
                        bool listed = false;
                        auto range = S->residents.equal_range(R->hash);
                        for (auto it = range.first; it != range.second && !listed; ++it) listed = it->second == R;
                        if (!listed) S->residents.emplace(R->hash, R);
                    }
                    R->refs += 1;
                    r->res = R;
                    holds_budget = true;
                    break;
                }
                if (!holds_budget) break;  // the server stops
            }
            if (upload_dag) {
                try {
                    const Clock::time_point t1 = Clock::now();
                    upload_image(R.get(), st, stage);
                    std::lock_guard<std::mutex> lk(S->mu);
                    S->upload_s += seconds_since(t1);
                    R->uploading = false;
                    R->on_device = true;
                    S->cv_resident.notify_all();
                } catch (const std::exception &e) {
                    std::lock_guard<std::mutex> lk(S->mu);
                    R->uploading = false;
                    S->resident_bytes -= (int64_t)R->bytes;
                    S->bytes_in_use -= (int64_t)R->bytes;
                    if (R->dimg) {
                        cudaFreeAsync(R->dimg, st);
                        R->dimg = nullptr;
                    }
                    R->error = e.what();
                    fail_resident(S, R);
                    throw;
                }
            } else {  // another request's thread uploads it, or it is there
                std::unique_lock<std::mutex> lk(S->mu);
                S->cv_resident.wait(lk, [&] { return S->stop || R->on_device || R->failed; });
                if (R->failed) throw McdError(MCD_ERR_INVALID, R->error);
                if (!R->on_device) throw McdError(MCD_ERR_RUNTIME, "server stopped");
            }
            const Clock::time_point t1 = Clock::now();
            upload_request(S, r, st, stage);
            request_args(r);
            std::lock_guard<std::mutex> lk(S->mu);
            S->upload_s += seconds_since(t1);
            r->state = Q_READY;
            S->ready.push_back(r);
        } catch (const std::exception &e) {
            if (r->dblock) {
                cudaFreeAsync(r->dblock, st);
                cudaStreamSynchronize(st);
                r->dblock = nullptr;
            }
            std::lock_guard<std::mutex> lk(S->mu);
            if (holds_budget) {
                S->bytes_in_use -= (int64_t)r->bytes;
                S->cv_budget.notify_all();
            }
            release_resident(S, r);
            r->error = e.what();
            r->state = Q_FAILED;
            r->t_done = Clock::now();
            S->pending -= 1;
            S->cv_done.notify_all();
        }
        S->cv_sched.notify_one();
    }
    cudaStreamDestroy(st);
}

// Launches one batch of uploaded requests of one class on a free slot
// (scheduler thread; the lock is not held).
void launch_batch(mcd_server *S, Slot &slot, std::vector<Request *> &batch) {
    const Clock::time_point t0 = Clock::now();
    cudaStream_t st = slot.stream;
    const size_t nb = batch.size();
    // longest first: requests by cost per tile, descending
    std::vector<int32_t> order(nb);
    for (size_t i = 0; i < nb; ++i) order[i] = (int32_t)i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t x, int32_t y) { return batch[x]->res->tile_cost > batch[y]->res->tile_cost; });
    size_t smem = 0, out_elems = 0, n_items = 0;
    int32_t max_E = 0;
    for (Request *r : batch) {
        smem = std::max(smem, (size_t)r->res->h.smem_total);
        max_E = std::max(max_E, r->E);
        out_elems += (size_t)r->E * 5;
        n_items += (size_t)((r->n + kTile - 1) / kTile);
    }
    const size_t s_ka = align_up(nb * sizeof(KArgs), 256), s_fa = align_up(nb * sizeof(FArgs), 256),
                 s_items = align_up(n_items * 8, 256), s_ctr = 256;
    const size_t need = s_ka + s_fa + s_items + s_ctr;
    if (need > slot.meta_bytes) {  // the slot is idle: its stream has nothing in flight
        const size_t bytes = std::max(need * 2, slot.meta_bytes * 2);
        if (slot.meta_dev) cuda_check(cudaFreeAsync(slot.meta_dev, st), "slot metadata free");
        if (slot.meta_pinned) slot.retired.push_back(slot.meta_pinned);
        slot.meta_dev = nullptr;
        slot.meta_pinned = nullptr;
        slot.meta_bytes = 0;
        cuda_check(cudaMallocAsync(reinterpret_cast<void **>(&slot.meta_dev), bytes, st), "slot metadata");
        cuda_check(cudaHostAlloc(reinterpret_cast<void **>(&slot.meta_pinned), bytes, cudaHostAllocDefault),
                   "slot metadata");
        slot.meta_bytes = bytes;
    }
    if (out_elems > slot.pinned_elems) {
        const size_t elems = std::max(out_elems * 2, slot.pinned_elems * 2);
        if (slot.pinned) slot.retired.push_back(slot.pinned);
        slot.pinned = nullptr;
        slot.pinned_elems = 0;
        cuda_check(cudaHostAlloc(reinterpret_cast<void **>(&slot.pinned), elems * 8, cudaHostAllocDefault),
                   "pinned results");
        slot.pinned_elems = elems;
    }
    // metadata straight into pinned memory, one upload
    char *mh = slot.meta_pinned;
    auto *ka = reinterpret_cast<KArgs *>(mh);
    auto *fa = reinterpret_cast<FArgs *>(mh + s_ka);
    auto *items = reinterpret_cast<int32_t *>(mh + s_ka + s_fa);
    for (size_t i = 0; i < nb; ++i) {
        ka[i] = batch[i]->ka;
        fa[i] = batch[i]->fa;
    }
    size_t k = 0;
    for (int32_t i : order) {
        const int64_t tiles = (batch[i]->n + kTile - 1) / kTile;
        for (int64_t t = 0; t < tiles; ++t) {
            items[k++] = i;
            items[k++] = (int32_t)t;
        }
    }
    std::memset(mh + s_ka + s_fa + s_items, 0, s_ctr);  // queue head
    cuda_check(cudaMemcpyAsync(slot.meta_dev, mh, need, cudaMemcpyHostToDevice, st), "batch upload");
    BatchArgs ba{};
    ba.dags = reinterpret_cast<const KArgs *>(slot.meta_dev);
    ba.items = reinterpret_cast<const int32_t *>(slot.meta_dev + s_ka + s_fa);
    ba.n_items = (int32_t)n_items;
    ba.counter = reinterpret_cast<unsigned int *>(slot.meta_dev + s_ka + s_fa + s_items);
    ba.smem_bytes = (int32_t)smem;
    const HostDag &h0 = batch[0]->res->h;
    const int32_t nw = h0.n_warps;
    int grid = batch[0]->res->per_sm * S->sms;  // the class's CTAs per SM, on every SM
    ba.scratch = nullptr;
    ba.scratch_stride = 0;
    if (!h0.win_smem) {  // windows off chip: realized rows of 32 samples per CTA, at most one CTA per item
        grid = (int)std::min<size_t>((size_t)grid, n_items);
        ba.scratch_stride = (int64_t)max_E * kTile;
        const size_t bytes = (size_t)grid * (size_t)ba.scratch_stride * sizeof(double);
        if (bytes > slot.scratch_bytes) {  // the slot is idle: nothing in flight uses the old rows
            if (slot.scratch) cuda_check(cudaFreeAsync(slot.scratch, st), "slot scratch free");
            slot.scratch = nullptr;
            slot.scratch_bytes = 0;
            cuda_check(cudaMallocAsync(reinterpret_cast<void **>(&slot.scratch), bytes, st), "slot scratch");
            slot.scratch_bytes = bytes;
        }
        ba.scratch = slot.scratch;
    }
    cuda_check(launch_batch_stats(ba, h0.win_smem, h0.positive, h0.tables_in_smem, nw, smem, grid, st),
               "batch launch");
    cuda_check(launch_batch_finish(reinterpret_cast<const FArgs *>(slot.meta_dev + s_ka), (int32_t)nb, max_E, st),
               "batch finish");
    size_t pos = 0;
    for (Request *r : batch) {
        const size_t e5 = (size_t)r->E * 5;
        cuda_check(cudaMemcpyAsync(slot.pinned + pos, r->dblock + r->lay.out, e5 * 8, cudaMemcpyDeviceToHost, st),
                   "results download");
        cuda_check(cudaFreeAsync(r->dblock, st), "request free");
        pos += e5;
    }
    cuda_check(cudaEventRecord(slot.done, st), "event record");
    slot.batch = batch;
    slot.busy = true;
    std::lock_guard<std::mutex> lk(S->mu);
    S->launch_s += seconds_since(t0);
}

void complete_slot(mcd_server *S, Slot &slot) {
    size_t pos = 0;
    std::vector<Request *> done = slot.batch;
    for (Request *r : done) {
        const size_t e5 = (size_t)r->E * 5;
        r->out.assign(slot.pinned + pos, slot.pinned + pos + e5);
        pos += e5;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    for (Request *r : done) {
        r->dblock = nullptr;
        r->t_done = Clock::now();
        r->state = Q_DONE;
        S->bytes_in_use -= (int64_t)r->bytes;
        S->completed += 1;
        S->running -= 1;
        release_resident(S, r);
    }
    slot.batch.clear();
    slot.busy = false;
    S->cv_budget.notify_all();
    S->cv_done.notify_all();
}

// The uploaded requests of the oldest waiting request's class, oldest first
// (caller holds the lock).
std::vector<Request *> take_class(mcd_server *S) {
    std::vector<Request *> batch;
    if (S->ready.empty()) return batch;
    const Request *first = S->ready.front();
    const HostDag &h0 = first->res->h;
    const int32_t nw = h0.n_warps, per_sm = first->res->per_sm;
    const bool positive = h0.positive, tsmem = h0.tables_in_smem, win_smem = h0.win_smem;
    std::deque<Request *> rest;
    for (Request *r : S->ready) {
        const HostDag &h = r->res->h;
        if (h.n_warps == nw && r->res->per_sm == per_sm && h.positive == positive && h.tables_in_smem == tsmem &&
            h.win_smem == win_smem &&
            (S->opt.max_batch <= 0 || (int32_t)batch.size() < S->opt.max_batch))
            batch.push_back(r);
        else
            rest.push_back(r);
    }
    S->ready.swap(rest);
    for (Request *r : batch) {
        r->state = Q_RUNNING;
        S->running += 1;
        S->pending -= 1;
    }
    return batch;
}

void schedule_loop(mcd_server *S) {
    cudaSetDevice(S->device);
    while (!S->stop) {
        try {
            bool progressed = false;
            for (Slot &slot : S->slots) {
                if (!slot.busy) continue;
                const cudaError_t q = cudaEventQuery(slot.done);
                if (q == cudaSuccess) {
                    complete_slot(S, slot);
                    progressed = true;
                } else if (q != cudaErrorNotReady) {  // a failed batch: stop and report, never poll forever
                    cuda_check(q, "batch completion");
                }
            }
            for (Slot &slot : S->slots) {
                if (slot.busy) continue;
                std::vector<Request *> batch;
                {
                    std::lock_guard<std::mutex> lk(S->mu);
                    batch = take_class(S);
                }
                if (batch.empty()) break;
                launch_batch(S, slot, batch);
                {
                    std::lock_guard<std::mutex> lk(S->mu);
                    S->launched_batches += 1;
                }
                progressed = true;
            }
            if (!progressed) {
                std::unique_lock<std::mutex> lk(S->mu);
                S->cv_sched.wait_for(lk, std::chrono::microseconds(50));
            }
        } catch (const std::exception &e) {
            std::lock_guard<std::mutex> lk(S->mu);
            S->fatal = e.what();
            S->stop = true;
            S->cv_done.notify_all();
            S->cv_budget.notify_all();
            S->cv_compile.notify_all();
            S->cv_resident.notify_all();
            return;
        }
    }
}

}  // namespace

extern "C" {

int mcd_server_create(const mcd_server_options *opt, mcd_server **out) {
    return guarded([&] {
        if (!opt || !out) throw McdError(MCD_ERR_INVALID, "null argument");
        if (opt->memory_budget <= 0 || opt->n_streams < 1 || opt->n_streams > 16 || opt->n_warps < 0 ||
            opt->n_warps > kMaxBatchWarps || opt->compile_threads < 1 || opt->compile_threads > 256)
            throw McdError(MCD_ERR_INVALID, "bad server options");
        auto S = std::make_unique<mcd_server>();
        S->opt = *opt;
        cuda_check(cudaGetDevice(&S->device), "cudaGetDevice");
        cuda_check(cudaDeviceGetAttribute(&S->sms, cudaDevAttrMultiProcessorCount, S->device), "SM count");
        cuda_check(cudaDeviceGetDefaultMemPool(&S->pool, S->device), "memory pool");
        uint64_t keep = (uint64_t)opt->memory_budget;  // freed blocks stay in the pool for reuse
        cuda_check(cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep), "pool threshold");
        cuda_check(cudaHostAlloc(reinterpret_cast<void **>(&S->zeros), kZeroBytes, cudaHostAllocDefault),
                   "pinned zeros");
        std::memset(S->zeros, 0, kZeroBytes);
        S->slots.resize((size_t)opt->n_streams);
        for (Slot &s : S->slots) {
            cuda_check(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking), "stream create");
            cuda_check(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming), "event create");
        }
        mcd_server *raw = S.get();
        for (int i = 0; i < opt->compile_threads; ++i) S->compilers.emplace_back(compile_loop, raw);
        S->scheduler = std::thread(schedule_loop, raw);
        *out = S.release();
    });
}

void mcd_server_destroy(mcd_server *S) {
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_compile.notify_all();
    S->cv_sched.notify_all();
    S->cv_budget.notify_all();
    S->cv_resident.notify_all();
    if (S->scheduler.joinable()) S->scheduler.join();
    for (std::thread &t : S->compilers)
        if (t.joinable()) t.join();
    cudaSetDevice(S->device);
    for (Slot &s : S->slots) {
        if (s.stream) cudaStreamSynchronize(s.stream);
        if (s.meta_dev) cudaFree(s.meta_dev);
        if (s.scratch) cudaFree(s.scratch);
        if (s.meta_pinned) cudaFreeHost(s.meta_pinned);
        if (s.pinned) cudaFreeHost(s.pinned);
        for (void *p : s.retired) cudaFreeHost(p);
        if (s.done) cudaEventDestroy(s.done);
        if (s.stream) cudaStreamDestroy(s.stream);
    }
    for (auto &kv : S->all)  // uploaded requests that never ran
        if (kv.second->dblock && kv.second->state != Q_RUNNING) cudaFree(kv.second->dblock);
    for (auto &kv : S->residents)
        if (kv.second->dimg) cudaFree(kv.second->dimg);
    if (S->zeros) cudaFreeHost(S->zeros);
    delete S;
}

int mcd_server_submit(mcd_server *S, const mcd_dag_desc *d, const mcd_generator *gen, int64_t seed0, int64_t n,
                      int64_t *ticket) {
    return guarded([&] {
        if (!S || !d || !gen || !ticket) throw McdError(MCD_ERR_INVALID, "null argument");
        if (n <= 0 || n > (int64_t)1 << 31) throw McdError(MCD_ERR_INVALID, "need 0 < n <= 2^31 samples");
        if (d->n_events < 0 || d->n_activities < 0 || d->n_targets < 0)
            throw McdError(MCD_ERR_INVALID, "negative array length in DAG description");
        auto r = std::make_unique<Request>();
        r->earliest.assign(d->earliest, d->earliest + d->n_events);
        r->act_idx.assign(d->act_idx, d->act_idx + d->n_activities);
        r->act_duration.assign(d->act_duration, d->act_duration + d->n_activities);
        r->act_type.assign(d->act_type, d->act_type + d->n_activities);
        r->target.assign(d->target, d->target + d->n_targets);
        r->pred_offsets.assign(d->pred_offsets, d->pred_offsets + d->n_targets + 1);
        const int64_t P = d->n_targets > 0 ? d->pred_offsets[d->n_targets] : 0;
        r->pred_src.assign(d->pred_src, d->pred_src + P);
        r->pred_act.assign(d->pred_act, d->pred_act + P);
        r->max_delay = d->max_delay;
        r->gen = *gen;
        r->seed0 = seed0;
        r->n = n;
        r->t_submit = Clock::now();
        std::lock_guard<std::mutex> lk(S->mu);
        if (!S->fatal.empty()) throw McdError(MCD_ERR_CUDA, "server stopped: " + S->fatal);
        r->ticket = S->next_ticket++;
        *ticket = r->ticket;
        S->to_compile.push_back(r.get());
        S->all[r->ticket] = std::move(r);
        S->pending += 1;
        S->cv_compile.notify_one();
    });
}

// Copies the statistics of a finished request and forgets it.  status: 1 done,
// 0 still pending (wait_ms elapsed); an error status for a failed request.
int mcd_server_wait(mcd_server *S, int64_t ticket, double wait_ms, const mcd_stats *host, int32_t *done,
                    double *latency_ms) {
    return guarded([&] {
        if (!S || !done) throw McdError(MCD_ERR_INVALID, "null argument");
        std::unique_lock<std::mutex> lk(S->mu);
        auto it = S->all.find(ticket);
        if (it == S->all.end()) throw McdError(MCD_ERR_INVALID, "unknown ticket");
        Request *r = it->second.get();
        auto finished = [&] { return r->state == Q_DONE || r->state == Q_FAILED || !S->fatal.empty(); };
        if (!finished()) {
            if (wait_ms > 0)
                S->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(wait_ms), finished);
        }
        if (!S->fatal.empty() && r->state != Q_DONE) throw McdError(MCD_ERR_CUDA, "server stopped: " + S->fatal);
        if (r->state == Q_FAILED) {
            const std::string msg = r->error;
            S->all.erase(it);
            throw McdError(MCD_ERR_INVALID, msg);
        }
        if (r->state != Q_DONE) {
            *done = 0;
            return;
        }
        *done = 1;
        const size_t E = (size_t)r->E;
        double *dst[5] = {host ? host->mean : nullptr, host ? host->p50 : nullptr, host ? host->p90 : nullptr,
                          host ? host->p99 : nullptr, host ? host->p_on_time : nullptr};
        for (int k = 0; k < 5; ++k)
            if (dst[k]) std::memcpy(dst[k], r->out.data() + k * E, E * 8);
        if (latency_ms)
            *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
        S->all.erase(it);
    });
}

int mcd_server_counters(mcd_server *S, mcd_server_info *info) {
    return guarded([&] {
        if (!S || !info) throw McdError(MCD_ERR_INVALID, "null argument");
        std::lock_guard<std::mutex> lk(S->mu);
        info->completed = S->completed;
        info->batches = S->launched_batches;
        info->queued = S->pending;
        info->bytes_in_use = S->bytes_in_use;
        info->running = S->running;
        info->compile_seconds = S->compile_s;
        info->upload_seconds = S->upload_s;
        info->launch_seconds = S->launch_s;
        info->resident_hits = S->resident_hits;
        int64_t on_device = 0;
        for (const auto &kv : S->residents) on_device += kv.second->on_device ? 1 : 0;
        info->resident_dags = on_device;
        info->resident_bytes = S->resident_bytes;
        info->evicted = S->evicted;
    });
}

}  // extern "C"
