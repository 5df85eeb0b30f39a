// mcd_core_pybind.cpp -- the Python module `mc_dagprop_gb300._core`.
//
// Same classes, constructor arguments, properties, reprs and error types as the
// reference's pybind11 module (src/mc_dagprop/monte_carlo/_core.cpp:366-552, stub
// _core.pyi:8-101), so code written against `mc_dagprop` runs unchanged.  All
// work goes through the C ABI of include/mc_dagprop_gb300.h; nothing here touches
// CUDA directly.  The data classes are turned into frozen, slotted dataclasses
// the way the reference does it (_core.cpp:445-488).
//
// Additions beyond the reference surface (array in, array out):
//   MonteCarloPropagator.from_arrays(...)   flat-array DagContext, no Python objects per event
//   MonteCarloPropagator.run_many_arrays    (S,E)/(S,L)/(S,E) numpy arrays instead of S SimResults
//   MonteCarloPropagator.propagate          propagation alone from given durations
//   MonteCarloPropagator.info               compiled-DAG facts
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <unistd.h>

#include <cstdint>
#include <cstdlib>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../include/mc_dagprop_gb300.h"

namespace py = pybind11;

// Own namespace: the reference's module binds C++ types of the same names, and
// pybind11 identifies bound types by their C++ type name across modules.
namespace mcd_py {

using EventIndex = int;
using ActivityIndex = int;
using ActivityType = int;
using Preds = std::vector<std::pair<EventIndex, ActivityIndex>>;

struct PairHash {
    size_t operator()(const std::pair<int, int> &p) const noexcept {
        return std::hash<int>{}(p.first) * 1000003u ^ std::hash<int>{}(p.second);
    }
};

struct EventTimestamp {
    double earliest, latest, actual;
};
struct Event {
    std::string event_id;
    EventTimestamp ts;
};
struct Activity {
    ActivityIndex idx;
    double duration;
    ActivityType activity_type;
};
using ActivityMap = std::unordered_map<std::pair<EventIndex, EventIndex>, Activity, PairHash>;

struct DagContext {
    std::vector<Event> events;
    ActivityMap activity_map;
    std::vector<std::pair<EventIndex, Preds>> precedence_list;
    double max_delay;
    DagContext(std::vector<Event> ev, ActivityMap am, std::vector<std::pair<EventIndex, Preds>> pl, double md)
        : events(std::move(ev)), activity_map(std::move(am)), precedence_list(std::move(pl)), max_delay(md) {}
};

static void raise_status(int rc) {
    if (rc == MCD_OK) return;
    const std::string msg = mcd_last_error();
    if (rc == MCD_ERR_INVALID) throw py::value_error(msg);
    throw std::runtime_error(msg);  // -> RuntimeError, as the reference's C++ exceptions
}

// ---- GenericDelayGenerator: a value type (copied into each propagator).
struct Generator {
    std::shared_ptr<mcd_generator> g;
    Generator() {
        mcd_generator *p = nullptr;
        raise_status(mcd_generator_create(&p));
        g.reset(p, mcd_generator_destroy);
    }
    Generator(const Generator &o) : Generator() { replay_from(o); }
    Generator &operator=(const Generator &o) {
        if (this != &o) {
            Generator fresh(o);
            g = fresh.g;
            calls = fresh.calls;
        }
        return *this;
    }
    // The add_* calls so far, replayed on copies.
    struct Call {
        int kind;
        int type;
        double a, b, c;
        std::vector<double> v, w;
    };
    std::vector<Call> calls;
    int64_t seed = 0;
    void replay_from(const Generator &o) {
        for (const Call &c : o.calls) apply(c);
        seed = o.seed;
        raise_status(mcd_generator_set_seed(g.get(), seed));
    }
    void apply(const Call &c) {
        int rc = MCD_OK;
        switch (c.kind) {
            case 0: rc = mcd_generator_add_constant(g.get(), c.type, c.a); break;
            case 1: rc = mcd_generator_add_exponential(g.get(), c.type, c.a, c.b); break;
            case 2: rc = mcd_generator_add_gamma(g.get(), c.type, c.a, c.b, c.c); break;
            case 3:
                rc = mcd_generator_add_empirical_absolute(g.get(), c.type, c.v.data(), (int64_t)c.v.size(),
                                                          c.w.data(), (int64_t)c.w.size());
                break;
            default:
                rc = mcd_generator_add_empirical_relative(g.get(), c.type, c.v.data(), (int64_t)c.v.size(),
                                                          c.w.data(), (int64_t)c.w.size());
        }
        raise_status(rc);
        calls.push_back(c);
    }
};

// ---- Host memory for results: page-locked blocks, recycled.
// The device writes results into page-locked host memory at the link's full
// rate, but pinning memory is slow (about as slow as the copy it speeds up), so
// blocks are kept when their arrays die and handed to the next call that fits.
// The pool holds at most an eighth of the machine's memory and 64 GiB
// ($MCD_PINNED_POOL_MB overrides; 0 turns it off); past that, results go to
// ordinary (pageable) memory, copied through the device.  The pool lives until
// the process exits.
class PinnedPool {
   public:
    static PinnedPool &get() {
        static PinnedPool *p = new PinnedPool();  // never destroyed: outlives the CUDA context's teardown
        return *p;
    }
    // A block of at least `bytes`, or null (pool full or disabled).
    void *acquire(size_t bytes) {
        if (bytes == 0) return nullptr;
        std::lock_guard<std::mutex> lk(mu_);
        auto it = free_.lower_bound(bytes);
        if (it != free_.end() && it->first <= bytes + bytes / 4) {  // a free block that fits without much waste
            void *p = it->second;
            free_.erase(it);
            return p;
        }
        while (held_ + bytes > cap_ && !free_.empty()) {  // make room: return the largest free blocks
            auto big = std::prev(free_.end());
            mcd_host_free(big->second);
            held_ -= big->first;
            size_.erase(big->second);
            free_.erase(big);
        }
        if (held_ + bytes > cap_) return nullptr;
        void *p = nullptr;
        if (mcd_host_alloc(bytes, &p) != MCD_OK || !p) return nullptr;
        held_ += bytes;
        size_[p] = bytes;
        return p;
    }
    void release(void *p) {
        if (!p) return;
        std::lock_guard<std::mutex> lk(mu_);
        auto it = size_.find(p);
        if (it != size_.end()) free_.emplace(it->second, p);
    }

   private:
    PinnedPool() {
        const long pages = sysconf(_SC_PHYS_PAGES), page = sysconf(_SC_PAGE_SIZE);
        cap_ = pages > 0 && page > 0 ? std::min<size_t>((size_t)pages * (size_t)page / 8, 64ull << 30) : 0;
        if (const char *e = std::getenv("MCD_PINNED_POOL_MB")) cap_ = (size_t)std::max(0ll, std::atoll(e)) << 20;
    }
    std::mutex mu_;
    std::multimap<size_t, void *> free_;
    std::unordered_map<void *, size_t> size_;
    size_t held_ = 0, cap_ = 0;
};

// One result buffer: a pooled page-locked block, else pageable memory.
struct HostBuf {
    void *p = nullptr;
    bool pinned = false;
    HostBuf() = default;
    explicit HostBuf(size_t bytes) {
        p = PinnedPool::get().acquire(bytes);
        pinned = p != nullptr;
        if (!p && bytes) {
            p = std::malloc(bytes);
            if (!p) throw std::bad_alloc();
        }
    }
    HostBuf(const HostBuf &) = delete;
    HostBuf &operator=(const HostBuf &) = delete;
    ~HostBuf() {
        if (pinned) PinnedPool::get().release(p);
        else std::free(p);
    }
};

// A numpy array of `shape` over a new HostBuf, which returns to the pool when
// the array dies.
template <typename T>
py::array_t<T> host_array(std::vector<py::ssize_t> shape) {
    size_t n = 1;
    for (py::ssize_t d : shape) n *= (size_t)d;
    auto *buf = new HostBuf(n * sizeof(T));
    py::capsule owner(buf, [](void *b) { delete static_cast<HostBuf *>(b); });
    return py::array_t<T>(shape, static_cast<T *>(buf->p), owner);
}

// ---- SimResult: one sample of a result block, exposed as zero-copy numpy views.
struct SimBlock {
    int64_t E = 0, L = 0;
    std::unique_ptr<HostBuf> realized, durations, cause;
};
struct SimResult {
    std::shared_ptr<SimBlock> blk;
    int64_t i = 0;
    double *realized() const { return static_cast<double *>(blk->realized->p) + i * blk->E; }
    double *durations() const {
        return blk->durations ? static_cast<double *>(blk->durations->p) + i * blk->L : nullptr;
    }
    int32_t *cause() const { return static_cast<int32_t *>(blk->cause->p) + i * blk->E; }
};

// ---- MonteCarloPropagator
struct FlatDag {
    std::vector<double> earliest, act_duration;
    std::vector<int32_t> act_idx, act_type, target, pred_src, pred_act;
    std::vector<int64_t> pred_offsets{0};
    double max_delay = 0.0;
    mcd_dag_desc desc() const {
        mcd_dag_desc d{};
        d.n_events = (int32_t)earliest.size();
        d.earliest = earliest.data();
        d.n_activities = (int32_t)act_idx.size();
        d.act_idx = act_idx.data();
        d.act_duration = act_duration.data();
        d.act_type = act_type.data();
        d.n_targets = (int32_t)target.size();
        d.target = target.data();
        d.pred_offsets = pred_offsets.data();
        d.pred_src = pred_src.data();
        d.pred_act = pred_act.data();
        d.max_delay = max_delay;
        return d;
    }
};

class Propagator {
   public:
    Propagator(const FlatDag &f, const Generator &gen, int n_warps = 0, int window = MCD_WINDOW_AUTO) {
        mcd_dag *p = nullptr;
        const mcd_dag_desc d = f.desc();
        const mcd_dag_options opts{n_warps, 0, window};
        int rc;
        {
            py::gil_scoped_release release;
            rc = mcd_dag_create_ex(&d, gen.g.get(), &opts, &p);
        }
        raise_status(rc);
        dag_.reset(p, mcd_dag_destroy);
        E_ = mcd_dag_node_count(p);
        L_ = mcd_dag_activity_count(p);
    }
    static FlatDag flatten(const DagContext &c) {
        FlatDag f;
        f.max_delay = c.max_delay;
        f.earliest.reserve(c.events.size());
        for (const Event &e : c.events) f.earliest.push_back(e.ts.earliest);
        for (const auto &kv : c.activity_map) {
            f.act_idx.push_back(kv.second.idx);
            f.act_duration.push_back(kv.second.duration);
            f.act_type.push_back(kv.second.activity_type);
        }
        for (const auto &t : c.precedence_list) {
            f.target.push_back(t.first);
            for (const auto &pr : t.second) {
                f.pred_src.push_back(pr.first);
                f.pred_act.push_back(pr.second);
            }
            f.pred_offsets.push_back((int64_t)f.pred_src.size());
        }
        return f;
    }
    int node_count() const { return (int)E_; }
    int activity_count() const { return (int)L_; }

    std::shared_ptr<SimBlock> run_block(const std::vector<int64_t> &seeds, bool want_dur = true) {
        auto blk = std::make_shared<SimBlock>();
        const int64_t n = (int64_t)seeds.size();
        blk->E = E_;
        blk->L = L_;
        blk->realized.reset(new HostBuf((size_t)(n * E_) * sizeof(double)));
        if (want_dur) blk->durations.reset(new HostBuf((size_t)(n * L_) * sizeof(double)));
        blk->cause.reset(new HostBuf((size_t)(n * E_) * sizeof(int32_t)));
        int rc;
        {
            py::gil_scoped_release release;
            rc = mcd_run_many_host(dag_.get(), seeds.data(), n, static_cast<double *>(blk->realized->p),
                                   want_dur ? static_cast<double *>(blk->durations->p) : nullptr,
                                   static_cast<int32_t *>(blk->cause->p));
        }
        raise_status(rc);
        return blk;
    }
    SimResult run(int seed) {
        SimResult r;
        r.blk = run_block({(int64_t)seed});
        r.i = 0;
        return r;
    }
    std::vector<SimResult> run_many(const std::vector<int> &seeds) {
        std::vector<int64_t> s(seeds.begin(), seeds.end());
        auto blk = run_block(s);
        std::vector<SimResult> out(seeds.size());
        for (size_t i = 0; i < seeds.size(); ++i) out[i] = SimResult{blk, (int64_t)i};
        return out;
    }
    py::tuple run_many_arrays(py::array_t<int64_t, py::array::c_style | py::array::forcecast> seeds,
                              bool durations) {
        const int64_t n = (int64_t)seeds.size();
        py::array_t<double> real = host_array<double>({n, E_});
        py::array_t<int32_t> cause = host_array<int32_t>({n, E_});
        py::object dur = py::none();
        double *dp = nullptr;
        if (durations) {
            py::array_t<double> d = host_array<double>({n, L_});
            dp = d.mutable_data();
            dur = d;
        }
        const int64_t *sp = seeds.data();
        double *rp = real.mutable_data();
        int32_t *cp = cause.mutable_data();
        int rc;
        {
            py::gil_scoped_release release;
            rc = mcd_run_many_host(dag_.get(), sp, n, rp, dp, cp);
        }
        raise_status(rc);
        return py::make_tuple(real, dur, cause);
    }
    py::tuple propagate(py::array_t<double, py::array::c_style | py::array::forcecast> durations) {
        if (durations.ndim() != 2 || durations.shape(1) != L_)
            throw py::value_error("durations must have shape (n_samples, activity_count())");
        const int64_t n = durations.shape(0);
        py::array_t<double> real = host_array<double>({n, E_});
        py::array_t<int32_t> cause = host_array<int32_t>({n, E_});
        const double *dp = durations.data();
        double *rp = real.mutable_data();
        int32_t *cp = cause.mutable_data();
        int rc;
        {
            py::gil_scoped_release release;
            rc = mcd_propagate_host(dag_.get(), dp, n, rp, cp);
        }
        raise_status(rc);
        return py::make_tuple(real, cause);
    }
    py::dict run_stats(py::object seeds, int64_t n, int64_t seed0, bool hist) {
        std::vector<int64_t> sv;
        if (!seeds.is_none()) {
            auto a = py::array_t<int64_t, py::array::c_style | py::array::forcecast>::ensure(seeds);
            if (!a || a.ndim() != 1) throw py::value_error("seeds must be a 1-D integer array");
            sv.assign(a.data(), a.data() + a.size());
            n = (int64_t)sv.size();
        }
        if (n <= 0) throw py::value_error("need seeds or n > 0");
        py::array_t<double> mean(E_), p50(E_), p90(E_), p99(E_), pot(E_);
        py::object h = py::none();
        uint32_t *hp = nullptr;
        if (hist) {
            py::array_t<uint32_t> ha({E_, (int64_t)MCD_HIST_STRIDE});
            hp = ha.mutable_data();
            h = ha;
        }
        mcd_stats st{mean.mutable_data(), p50.mutable_data(), p90.mutable_data(), p99.mutable_data(),
                     pot.mutable_data(), hp};
        int rc;
        {
            py::gil_scoped_release release;
            rc = mcd_stats_host(dag_.get(), sv.empty() ? nullptr : sv.data(), seed0, n, &st);
        }
        raise_status(rc);
        double bw = 0.0;
        raise_status(mcd_stats_bin_width(dag_.get(), n, &bw));
        py::dict d;
        d["mean"] = mean;
        d["p50"] = p50;
        d["p90"] = p90;
        d["p99"] = p99;
        d["p_on_time"] = pot;
        d["hist"] = h;
        d["bin_width"] = bw;
        d["n"] = n;
        return d;
    }
    py::dict gradient(int64_t n, int64_t seed0) {
        py::array_t<double> ge(E_), gb(L_);
        double obj = 0.0;
        double *gp = ge.mutable_data(), *bp = gb.mutable_data();
        int rc;
        {
            py::gil_scoped_release release;
            rc = mcd_gradient_host(dag_.get(), seed0, n, &obj, gp, bp);
        }
        raise_status(rc);
        int64_t plan[3] = {0, 0, 0};
        raise_status(mcd_gradient_plan(dag_.get(), &plan[0], &plan[1], &plan[2]));
        py::dict d;
        d["objective"] = obj;
        d["grad_earliest"] = ge;
        d["grad_base"] = gb;
        d["samples_per_chunk"] = plan[0];
        d["level_blocks"] = plan[1];
        d["buffer_bytes"] = plan[2];
        return d;
    }
    py::tuple link_streams() const {
        const int32_t L = mcd_dag_activity_count(dag_.get());
        py::array_t<int32_t> block(L), word(L);
        raise_status(mcd_dag_link_streams(dag_.get(), block.mutable_data(), word.mutable_data()));
        return py::make_tuple(block, word);
    }
    py::dict info() const {
        mcd_dag_info i{};
        raise_status(mcd_dag_get_info(dag_.get(), &i));
        py::dict d;
        d["n_events"] = i.n_events;
        d["n_links"] = i.n_links;
        d["n_levels"] = i.n_levels;
        d["n_warps"] = i.n_warps;
        d["n_preds"] = i.n_preds;
        d["window_slots"] = i.window_slots;
        d["window_in_smem"] = (bool)i.window_in_smem;
        d["n_orphan_links"] = i.n_orphan_links;
        d["device"] = i.device;
        d["device_bytes"] = i.device_bytes;
        d["n_stages"] = i.n_stages;
        d["smem_bytes"] = i.smem_bytes;
        d["positive"] = (bool)i.positive;
        d["tables_in_smem"] = (bool)i.tables_in_smem;
        d["cache_hit"] = (bool)i.cache_hit;
        d["n_event_pairs"] = i.n_event_pairs;
        d["block_draws"] = i.block_draws;
        return d;
    }
    mcd_dag *handle() const { return dag_.get(); }

   private:
    std::shared_ptr<mcd_dag> dag_;
    int64_t E_ = 0, L_ = 0;
};

template <typename T>
static std::vector<T> to_vec(py::handle h) {
    auto a = py::array_t<T, py::array::c_style | py::array::forcecast>::ensure(h);
    if (!a) throw py::type_error("expected an array-like argument");
    if (a.ndim() != 1) throw py::value_error("expected a 1-D array");
    return std::vector<T>(a.data(), a.data() + a.size());
}

// Many propagators, each with its own samples, in one persistent launch.
class Batch {
   public:
    Batch(const std::vector<Propagator *> &props, const std::vector<int64_t> &seed0, const std::vector<int64_t> &n)
        : props_(props) {
        if (props.empty() || seed0.size() != props.size() || n.size() != props.size())
            throw py::value_error("need one seed0 and one sample count per propagator");
        std::vector<mcd_dag *> h;
        for (Propagator *p : props) {
            if (!p) throw py::value_error("null propagator");
            h.push_back(p->handle());
            keep_.push_back(py::cast(p));
        }
        mcd_batch *b = nullptr;
        raise_status(mcd_batch_create(h.data(), (int32_t)h.size(), seed0.data(), n.data(), &b));
        b_.reset(b, mcd_batch_destroy);
    }
    void run(bool wait) {
        int rc;
        {
            py::gil_scoped_release release;
            rc = mcd_batch_run(b_.get());
            if (rc == MCD_OK && wait) rc = mcd_batch_sync(b_.get());
        }
        raise_status(rc);
    }
    void sync() {
        int rc;
        {
            py::gil_scoped_release release;
            rc = mcd_batch_sync(b_.get());
        }
        raise_status(rc);
    }
    py::dict stats(int i, bool hist) {
        if (i < 0 || i >= (int)props_.size()) throw py::index_error("batch index out of range");
        const int64_t E = props_[i]->node_count();
        py::array_t<double> mean(E), p50(E), p90(E), p99(E), pot(E);
        py::object h = py::none();
        uint32_t *hp = nullptr;
        if (hist) {
            py::array_t<uint32_t> ha({E, (int64_t)MCD_HIST_STRIDE});
            hp = ha.mutable_data();
            h = ha;
        }
        mcd_stats st{mean.mutable_data(), p50.mutable_data(), p90.mutable_data(), p99.mutable_data(),
                     pot.mutable_data(), hp};
        raise_status(mcd_batch_download(b_.get(), i, &st));
        py::dict d;
        d["mean"] = mean;
        d["p50"] = p50;
        d["p90"] = p90;
        d["p99"] = p99;
        d["p_on_time"] = pot;
        d["hist"] = h;
        return d;
    }
    int64_t items() const { return mcd_batch_items(b_.get()); }
    int grid() const { return mcd_batch_grid(b_.get()); }
    uintptr_t stream() const { return (uintptr_t)mcd_batch_stream(b_.get()); }

   private:
    std::vector<Propagator *> props_;
    std::vector<py::object> keep_;  // the propagators outlive the batch
    std::shared_ptr<mcd_batch> b_;
};

// The continuous-batching server: submit requests, wait for their statistics.
class Server {
   public:
    Server(int64_t budget, int n_streams, int n_warps, int max_batch, int compile_threads) {
        mcd_server_options o{budget, n_streams, n_warps, max_batch, compile_threads};
        mcd_server *p = nullptr;
        raise_status(mcd_server_create(&o, &p));
        s_.reset(p, mcd_server_destroy);
    }
    int64_t submit(py::handle earliest, py::handle act_idx, py::handle act_duration, py::handle act_type,
                   py::handle target, py::handle pred_offsets, py::handle pred_src, py::handle pred_act,
                   double max_delay, const Generator &g, int64_t seed0, int64_t n) {
        FlatDag f;
        f.earliest = to_vec<double>(earliest);
        f.act_idx = to_vec<int32_t>(act_idx);
        f.act_duration = to_vec<double>(act_duration);
        f.act_type = to_vec<int32_t>(act_type);
        f.target = to_vec<int32_t>(target);
        f.pred_offsets = to_vec<int64_t>(pred_offsets);
        f.pred_src = to_vec<int32_t>(pred_src);
        f.pred_act = to_vec<int32_t>(pred_act);
        f.max_delay = max_delay;
        if (f.act_duration.size() != f.act_idx.size() || f.act_type.size() != f.act_idx.size() ||
            f.pred_offsets.size() != f.target.size() + 1 || f.pred_offsets.front() != 0 ||
            f.pred_offsets.back() != (int64_t)f.pred_src.size() || f.pred_src.size() != f.pred_act.size())
            throw py::value_error("inconsistent DAG arrays");
        const mcd_dag_desc d = f.desc();
        int64_t t = 0;
        int rc;
        {
            py::gil_scoped_release release;
            rc = mcd_server_submit(s_.get(), &d, g.g.get(), seed0, n, &t);
        }
        raise_status(rc);
        std::lock_guard<std::mutex> lk(mu_);
        sizes_[t] = (int64_t)f.earliest.size();
        return t;
    }
    py::object wait(int64_t ticket, double timeout_ms) {
        int64_t E;
        {
            std::lock_guard<std::mutex> lk(mu_);
            auto it = sizes_.find(ticket);
            if (it == sizes_.end()) throw py::value_error("unknown ticket");
            E = it->second;
        }
        py::array_t<double> mean(E), p50(E), p90(E), p99(E), pot(E);
        mcd_stats st{mean.mutable_data(), p50.mutable_data(), p90.mutable_data(), p99.mutable_data(),
                     pot.mutable_data(), nullptr};
        int32_t done = 0;
        double lat = 0.0;
        int rc;
        {
            py::gil_scoped_release release;
            rc = mcd_server_wait(s_.get(), ticket, timeout_ms, &st, &done, &lat);
        }
        if (rc != MCD_OK || done) {
            std::lock_guard<std::mutex> lk(mu_);
            sizes_.erase(ticket);
        }
        if (rc != MCD_OK) throw std::runtime_error(mcd_last_error());
        if (!done) return py::none();
        py::dict d;
        d["mean"] = mean;
        d["p50"] = p50;
        d["p90"] = p90;
        d["p99"] = p99;
        d["p_on_time"] = pot;
        d["latency_ms"] = lat;
        return std::move(d);
    }
    py::dict counters() {
        mcd_server_info i{};
        raise_status(mcd_server_counters(s_.get(), &i));
        py::dict d;
        d["completed"] = i.completed;
        d["batches"] = i.batches;
        d["queued"] = i.queued;
        d["running"] = i.running;
        d["bytes_in_use"] = i.bytes_in_use;
        d["compile_seconds"] = i.compile_seconds;
        d["upload_seconds"] = i.upload_seconds;
        d["launch_seconds"] = i.launch_seconds;
        d["resident_hits"] = i.resident_hits;
        d["resident_dags"] = i.resident_dags;
        d["resident_bytes"] = i.resident_bytes;
        d["evicted"] = i.evicted;
        return d;
    }

   private:
    std::shared_ptr<mcd_server> s_;
    std::mutex mu_;
    std::unordered_map<int64_t, int64_t> sizes_;
};

}  // namespace mcd_py

PYBIND11_MODULE(_core, m) {
    using namespace mcd_py;
    m.doc() = "GB300 Monte Carlo DAG-propagation engine (drop-in for mc_dagprop.monte_carlo._core)";

    py::class_<EventTimestamp> ts_cls(m, "EventTimestamp");
    ts_cls
        .def(py::init<double, double, double>(), py::arg("earliest"), py::arg("latest"), py::arg("actual"),
             "Create an event timestamp (earliest, latest, actual).")
        .def_readwrite("earliest", &EventTimestamp::earliest, "Earliest bound")
        .def_readwrite("latest", &EventTimestamp::latest, "Latest bound")
        .def_readwrite("actual", &EventTimestamp::actual, "Scheduled time")
        .def("__repr__", [](const EventTimestamp &t) {
            return py::str("EventTimestamp(earliest={}, latest={}, actual={})").format(t.earliest, t.latest, t.actual);
        });

    py::class_<Event> ev_cls(m, "Event");
    ev_cls
        .def(py::init<std::string, EventTimestamp>(), py::arg("event_id"), py::arg("timestamp"),
             "An event node with its ID and timestamp")
        .def_readwrite("event_id", &Event::event_id, "Node identifier")
        .def_readwrite("timestamp", &Event::ts, "Event timing info")
        .def("__repr__", [](const Event &e) {
            return py::str("Event(event_id={}, timestamp={})").format(py::repr(py::cast(e.event_id)),
                                                                       py::repr(py::cast(e.ts)));
        });

    py::class_<Activity> act_cls(m, "Activity");
    act_cls
        .def(py::init<ActivityIndex, double, ActivityType>(), py::arg("idx"), py::arg("minimal_duration"),
             py::arg("activity_type"), "An activity (edge) with index, base duration and type")
        .def_readwrite("idx", &Activity::idx, "Index of the activity")
        .def_readwrite("minimal_duration", &Activity::duration, "Base duration")
        .def_readwrite("activity_type", &Activity::activity_type, "Type ID for delay dist.")
        .def("__repr__", [](const Activity &a) {
            return py::str("Activity(idx={}, minimal_duration={}, activity_type={})")
                .format(a.idx, a.duration, a.activity_type);
        });

    py::class_<DagContext> ctx_cls(m, "DagContext");
    ctx_cls
        .def(py::init<std::vector<Event>, ActivityMap, std::vector<std::pair<EventIndex, Preds>>, double>(),
             py::arg("events"), py::arg("activities"), py::arg("precedence_list"), py::arg("max_delay"),
             "Wraps a DAG: events, activity_map, precedence_list, max_delay")
        .def_readwrite("events", &DagContext::events)
        .def_readwrite("activities", &DagContext::activity_map)
        .def_readwrite("precedence_list", &DagContext::precedence_list)
        .def_readwrite("max_delay", &DagContext::max_delay)
        .def("__repr__", [](const DagContext &c) {
            return py::str("DagContext(events={}, activities={}, precedence_list={}, max_delay={})")
                .format(py::repr(py::cast(c.events)), py::repr(py::cast(c.activity_map)),
                        py::repr(py::cast(c.precedence_list)), c.max_delay);
        });

    // Frozen, slotted dataclasses over the bound classes, as the reference does.
    {
        py::dict opts;
        opts["frozen"] = true;
        opts["slots"] = true;
        opts["init"] = false;
        py::object dataclass = py::module_::import("dataclasses").attr("dataclass")(**opts);
        py::module_ types = py::module_::import("mc_dagprop_gb300.types");
        py::object Second = types.attr("Second");
        py::dict a1;
        a1["earliest"] = Second;
        a1["latest"] = Second;
        a1["actual"] = Second;
        ts_cls.attr("__annotations__") = a1;
        dataclass(ts_cls);
        py::dict a2;
        a2["event_id"] = types.attr("EventId");
        a2["timestamp"] = ts_cls;
        ev_cls.attr("__annotations__") = a2;
        dataclass(ev_cls);
        py::dict a3;
        a3["idx"] = types.attr("ActivityIndex");
        a3["minimal_duration"] = Second;
        a3["activity_type"] = types.attr("ActivityType");
        act_cls.attr("__annotations__") = a3;
        dataclass(act_cls);
        py::module_ typing = py::module_::import("typing");
        py::dict a4;
        a4["events"] = typing.attr("Sequence");
        a4["activities"] = typing.attr("Mapping");
        a4["precedence_list"] = typing.attr("Sequence");
        a4["max_delay"] = Second;
        ctx_cls.attr("__annotations__") = a4;
        dataclass(ctx_cls);
    }

    py::class_<SimResult>(m, "SimResult", py::buffer_protocol())
        .def_buffer([](SimResult &r) -> py::buffer_info {
            return py::buffer_info(r.realized(), sizeof(double), py::format_descriptor<double>::format(), 1,
                                   {r.blk->E}, {(py::ssize_t)sizeof(double)});
        })
        .def_property_readonly(
            "realized", [](const SimResult &r) { return py::array(r.blk->E, r.realized(), py::cast(r)); },
            "Final event times as a NumPy array")
        .def_property_readonly(
            "durations", [](const SimResult &r) { return py::array(r.blk->L, r.durations(), py::cast(r)); },
            "Per-link durations (incl. extra) as a NumPy array")
        .def_property_readonly(
            "cause_event", [](const SimResult &r) { return py::array(r.blk->E, r.cause(), py::cast(r)); },
            "Index of predecessor causing each event as a NumPy array");

    py::class_<Generator>(m, "GenericDelayGenerator")
        .def(py::init<>(), "Create a new delay-generator")
        .def(
            "set_seed",
            [](Generator &g, int s) {
                g.seed = s;
                raise_status(mcd_generator_set_seed(g.g.get(), s));
            },
            py::arg("seed"), "Set RNG seed for reproducibility")
        .def(
            "add_constant", [](Generator &g, ActivityType t, double f) { g.apply({0, t, f, 0.0, 0.0, {}, {}}); },
            py::arg("activity_type"), py::arg("factor"), "Constant: delay = factor * duration")
        .def(
            "add_exponential",
            [](Generator &g, ActivityType t, double lam, double mx) { g.apply({1, t, lam, mx, 0.0, {}, {}}); },
            py::arg("activity_type"), py::arg("lambda_"), py::arg("max_scale"),
            "Exponential(lambda) truncated at max_scale")
        .def(
            "add_gamma",
            [](Generator &g, ActivityType t, double k, double s, double mx) { g.apply({2, t, k, s, mx, {}, {}}); },
            py::arg("activity_type"), py::arg("shape"), py::arg("scale"),
            py::arg("max_scale") = std::numeric_limits<double>::infinity(), "Gamma(shape,scale) truncated at max_scale")
        .def(
            "add_empirical_absolute",
            [](Generator &g, ActivityType t, std::vector<double> values, std::vector<double> weights) {
                g.apply({3, t, 0.0, 0.0, 0.0, std::move(values), std::move(weights)});
            },
            py::arg("activity_type"), py::arg("values"), py::arg("weights"),
            "Empirical absolute: draw one of your provided values, weighted by weights.")
        .def(
            "add_empirical_relative",
            [](Generator &g, ActivityType t, std::vector<double> factors, std::vector<double> weights) {
                g.apply({4, t, 0.0, 0.0, 0.0, std::move(factors), std::move(weights)});
            },
            py::arg("activity_type"), py::arg("factors"), py::arg("weights"),
            "Empirical relative: draw a factor in [0,inf), then multiply by the activity duration.");

    py::class_<Propagator>(m, "MonteCarloPropagator")
        .def(py::init([](const DagContext &c, const Generator &g) { return new Propagator(Propagator::flatten(c), g); }),
             py::arg("context"), py::arg("generator"), "Construct simulator with context and delay-generator")
        .def_static(
            "from_arrays",
            [](py::handle earliest, py::handle act_idx, py::handle act_duration, py::handle act_type,
               py::handle target, py::handle pred_offsets, py::handle pred_src, py::handle pred_act,
               double max_delay, const Generator &g, int n_warps, const std::string &window) {
                FlatDag f;
                f.earliest = to_vec<double>(earliest);
                f.act_idx = to_vec<int32_t>(act_idx);
                f.act_duration = to_vec<double>(act_duration);
                f.act_type = to_vec<int32_t>(act_type);
                f.target = to_vec<int32_t>(target);
                f.pred_offsets = to_vec<int64_t>(pred_offsets);
                f.pred_src = to_vec<int32_t>(pred_src);
                f.pred_act = to_vec<int32_t>(pred_act);
                f.max_delay = max_delay;
                if (f.act_duration.size() != f.act_idx.size() || f.act_type.size() != f.act_idx.size())
                    throw py::value_error("activity arrays must have equal length");
                if (f.pred_offsets.size() != f.target.size() + 1 || f.pred_offsets.front() != 0 ||
                    f.pred_offsets.back() != (int64_t)f.pred_src.size() || f.pred_src.size() != f.pred_act.size())
                    throw py::value_error("inconsistent precedence arrays");
                if (window != "auto" && window != "global")
                    throw py::value_error("window must be 'auto' or 'global'");
                return new Propagator(f, g, n_warps, window == "global" ? MCD_WINDOW_GLOBAL : MCD_WINDOW_AUTO);
            },
            py::arg("earliest"), py::arg("act_idx"), py::arg("act_duration"), py::arg("act_type"), py::arg("target"),
            py::arg("pred_offsets"), py::arg("pred_src"), py::arg("pred_act"), py::arg("max_delay"),
            py::arg("generator"), py::arg("n_warps") = 0, py::arg("window") = "auto",
            "Construct from a DagContext in flat-array form (n_warps: warps per CTA, 0 = automatic; window: "
            "'auto' keeps the propagation window in shared memory when it fits, 'global' in global rows)")
        .def("node_count", &Propagator::node_count, "Number of events")
        .def("activity_count", &Propagator::activity_count, "Number of links")
        .def("run", &Propagator::run, py::arg("seed"), "Run single sim")
        .def("run_many", &Propagator::run_many, py::arg("seeds"), "Run batch sims")
        .def("run_many_arrays", &Propagator::run_many_arrays, py::arg("seeds"), py::arg("durations") = true,
             "Batch run returning (realized (S,E), durations (S,L) or None, cause_event (S,E)) arrays")
        .def("propagate", &Propagator::propagate, py::arg("durations"),
             "Propagation alone from given durations (S,L): returns (realized, cause_event)")
        .def("run_stats", &Propagator::run_stats, py::arg("seeds") = py::none(), py::arg("n") = 0,
             py::arg("seed0") = 0, py::arg("hist") = false,
             "Per-event statistics over samples (seeds, or seed0..seed0+n-1) computed on the GPU: "
             "dict of mean, p50, p90, p99, p_on_time (and the raw histogram when hist=True)")
        .def("gradient", &Propagator::gradient, py::arg("n"), py::arg("seed0") = 0,
             "Pathwise gradient of J = mean_s sum_e (realized - earliest) over seeds seed0..seed0+n-1: "
             "dict of objective, grad_earliest (per event), grad_base (per link index), and the plan used "
             "(samples_per_chunk, level_blocks: 1 = every winner kept, more = level blocks recomputed from "
             "checkpoints; buffer_bytes)")
        .def("info", &Propagator::info, "Compiled-DAG facts")
        .def("link_streams", &Propagator::link_streams,
             "(block, word) per link: the Philox block of its draws and its first word (-1: whole block)")
        .def("_handle", [](const Propagator &p) { return (uintptr_t)p.handle(); });

    py::class_<Batch>(m, "Batch")
        .def(py::init<const std::vector<Propagator *> &, const std::vector<int64_t> &,
                      const std::vector<int64_t> &>(),
             py::arg("propagators"), py::arg("seed0"), py::arg("n_samples"),
             "Many propagators (compiled with the same n_warps), each with its own samples "
             "(seeds seed0[i]..seed0[i]+n_samples[i]-1), run as one persistent launch")
        .def("run", &Batch::run, py::arg("wait") = true, "Run the batch (one CUDA graph launch)")
        .def("sync", &Batch::sync, "Wait for the last run and report kernel errors")
        .def("stats", &Batch::stats, py::arg("i"), py::arg("hist") = false, "Statistics of propagator i")
        .def_property_readonly("items", &Batch::items, "Work items (DAG, 32-sample tile)")
        .def_property_readonly("grid", &Batch::grid, "CTAs of the persistent launch")
        .def_static(
            "occupancy",
            [](int32_t n_warps, int64_t smem_bytes) {
                int32_t per_sm = 0;
                raise_status(mcd_batch_occupancy(n_warps, smem_bytes, &per_sm));
                return per_sm;
            },
            py::arg("n_warps"), py::arg("smem_bytes"),
            "CTAs per SM of the batch kernel at this block size and shared memory")
        .def_property_readonly("stream", &Batch::stream, "The batch's CUDA stream");

    py::class_<Server>(m, "Server")
        .def(py::init<int64_t, int, int, int, int>(), py::arg("memory_budget") = (int64_t)64 << 30,
             py::arg("n_streams") = 4, py::arg("n_warps") = 0, py::arg("max_batch") = 0,
             py::arg("compile_threads") = 8,
             "Continuous-batching statistics server on the current GPU (n_warps 0: per request, "
             "batched by warps per CTA and CTAs per SM)")
        .def("submit", &Server::submit, py::arg("earliest"), py::arg("act_idx"), py::arg("act_duration"),
             py::arg("act_type"), py::arg("target"), py::arg("pred_offsets"), py::arg("pred_src"),
             py::arg("pred_act"), py::arg("max_delay"), py::arg("generator"), py::arg("seed0"), py::arg("n"),
             "Submit a request (flat DAG, generator, seeds seed0..seed0+n-1); returns a ticket")
        .def("wait", &Server::wait, py::arg("ticket"), py::arg("timeout_ms") = 0.0,
             "Statistics of a finished request (dict with latency_ms), None while pending")
        .def("counters", &Server::counters,
             "completed, batches, queued, running, bytes_in_use, and compile/upload/launch seconds");
}
