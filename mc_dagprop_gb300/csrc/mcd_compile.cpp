// mcd_compile.cpp -- host DAG compiler: DagContext + GenericDelayGenerator ->
// level-ordered CSR records for the kernels.
//
// Mirrors Simulator::Simulator (src/mc_dagprop/monte_carlo/_core.cpp:193-307):
//   - the same three RuntimeError cases with the same messages
//     (reserved type -1 :196-198, negative max_delay :199-201, cycle :262-264);
//   - dense link array of max idx + 1 entries, gaps of duration 0 with no delay,
//     unmapped types with no delay (:213-229);
//   - predecessors of each event kept in precedence-list order (:267-285).
// Where the reference has undefined behaviour (indices out of range, a target
// listed twice, empty tables, parameters for which its rejection loops never
// end) this compiler rejects the input with MCD_ERR_INVALID instead.
//
// Compiled with -ffp-contract=off: `base + base*factor` and `earliest +
// max_delay` must round exactly as the reference's two separate operations.
#include "mcd_host.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <limits>
#include <string>
#include <unordered_map>

namespace mcd {

int64_t order_key_host(int64_t b) {
    const int64_t mag = b & 0x7FFFFFFFFFFFFFFFll;
    const int64_t k = b < 0 ? -mag : mag;
    return mag > 0x7FF0000000000000ll ? std::numeric_limits<int64_t>::min() : k;
}

static int64_t bits_of(double x) {
    int64_t b;
    std::memcpy(&b, &x, sizeof(b));
    return b;
}

static int32_t float_bits(float x) {
    int32_t b;
    std::memcpy(&b, &x, sizeof(b));
    return b;
}

// Largest float not above x (x may be +inf).
static float float_at_or_below(double x) {
    float f = (float)x;
    if ((double)f > x) f = std::nextafter(f, -std::numeric_limits<float>::infinity());
    return f;
}

static uint32_t keep_threshold(double prob) {
    if (!(prob < 1.0)) return 0xFFFFFFFFu;
    if (!(prob > 0.0)) return 0u;
    const double t = std::floor(prob * 4294967296.0);
    return t >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t;
}

// Walker/Vose alias table over weights w (validated: finite, >= 0, sum > 0).
static void build_alias(const std::vector<double> &values, const std::vector<double> &w,
                        std::vector<AliasEntry> &out, std::vector<AliasPick> &picks) {
    const size_t n = w.size();
    double sum = 0.0;
    for (double x : w) sum += x;
    std::vector<double> q(n);
    for (size_t i = 0; i < n; ++i) q[i] = w[i] / sum * (double)n;
    std::vector<int64_t> small, large;
    for (size_t i = 0; i < n; ++i) (q[i] < 1.0 ? small : large).push_back((int64_t)i);
    std::vector<double> prob(n, 1.0);
    std::vector<int64_t> alias(n);
    for (size_t i = 0; i < n; ++i) alias[i] = (int64_t)i;
    while (!small.empty() && !large.empty()) {
        const int64_t s = small.back();
        small.pop_back();
        const int64_t l = large.back();
        large.pop_back();
        prob[s] = q[s];
        alias[s] = l;
        q[l] = (q[l] + q[s]) - 1.0;
        (q[l] < 1.0 ? small : large).push_back(l);
    }
    // Leftovers (rounding) keep their own bin.
    for (size_t i = 0; i < n; ++i) {
        AliasEntry e{};
        e.v_self = values[i];
        e.thresh = keep_threshold(prob[i]);
        e.v_alias = e.thresh == 0xFFFFFFFFu ? values[i] : values[(size_t)alias[i]];
        out.push_back(e);
        picks.push_back(AliasPick{e.thresh, e.thresh == 0xFFFFFFFFu ? (int32_t)i : (int32_t)alias[i]});
    }
}

static void check_table(const DistSpec &d) {
    if (d.values.empty()) throw McdError(MCD_ERR_INVALID, "empirical distribution needs at least one value");
    double sum = 0.0;
    for (double x : d.weights) {
        if (!(x >= 0.0) || !std::isfinite(x))
            throw McdError(MCD_ERR_INVALID, "empirical weights must be finite and non-negative");
        sum += x;
    }
    if (!(sum > 0.0)) throw McdError(MCD_ERR_INVALID, "empirical weights must not all be zero");
}

// The invariants every kernel access relies on, checked on the compiled DAG:
// shared-memory regions in order, aligned and within the budget; staged
// records within their buffer; warp chunks covering each stage; work units
// within their stage; every source in an earlier stage; window slots reused only
// after the stage of the last read of the previous tenant; and every KD_REUSE
// reference naming the block its work unit drew last.  A violation is a
// compiler defect and fails the compile rather than a launch.
static void verify_layout(const HostDag &H) {
    auto fail = [](const char *what) {
        throw McdError(MCD_ERR_RUNTIME, std::string("internal layout check failed: ") + what);
    };
    const int64_t E = H.E, P = (int64_t)H.pred.size(), NW = H.n_warps, NS = H.n_stages;
    if ((int64_t)H.ev.size() != E) fail("event records");
    if ((int64_t)H.stage_meta.size() != NS * kStageMetaInts || (int64_t)H.wk_off.size() != NS * NW + 1)
        fail("stage tables");
    if (H.picks.size() != H.alias.size()) fail("alias picks");
    // shared memory: [window][stage buffer 0][stage buffer 1][tables][2 mbarriers, 2 stage counters]
    const int64_t win = H.win_smem ? (int64_t)H.window_slots * kTile * (int64_t)sizeof(double) : 0;
    const int64_t tables = H.tables_in_smem ? (int64_t)(H.dist.size() * sizeof(DistParam) +
                                                        H.alias.size() * (sizeof(AliasEntry) + sizeof(AliasPick)))
                                            : 0;
    if (H.smem_stage_off < win || H.smem_stage_off % 16) fail("stage buffer offset");
    if (H.stage_bytes % 16) fail("stage buffer size");
    if (H.smem_tables_off < (int64_t)H.smem_stage_off + 2 * (int64_t)H.stage_bytes || H.smem_tables_off % 16)
        fail("table offset");
    if (H.smem_bar_off % 8 || H.smem_bar_off < H.smem_tables_off + tables) fail("barrier offset");
    if (H.smem_total < (int64_t)H.smem_bar_off + kBarRegionBytes || H.smem_total > (int64_t)kSmemMax)
        fail("shared memory total");
    // records
    std::vector<int32_t> stage_of((size_t)E, -1);  // by caller index
    std::vector<char> seen((size_t)E, 0);
    int64_t ev_next = 0, pred_next = 0, val_next = 0;
    for (int64_t st = 0; st < NS; ++st) {
        const int32_t *m = &H.stage_meta[(size_t)st * kStageMetaInts];
        const int64_t first = m[0], nev = m[1] >= 0 ? m[1] : -(int64_t)m[1], pfirst = m[2], npred = m[3];
        const int64_t vfirst = m[4], nval = m[5];
        if (first != ev_next || nev <= 0 || first + nev > E || pfirst != pred_next) fail("stage ranges");
        if (m[8] < 0 || 2 * (int64_t)m[8] > nev || m[9] || m[10] || m[11]) fail("event pairs");
        if (vfirst != val_next || nval < 0 || nval % 2 || vfirst + nval > (int64_t)H.vals.size())
            fail("value region");
        const int64_t pboff = m[6], vboff = m[7];
        if (m[1] >= 0 && (pboff % 16 || vboff % 16 || nev * (int64_t)sizeof(EvRec) > pboff ||
                          pboff + npred * (int64_t)sizeof(PredRec) > vboff ||
                          vboff + nval * (int64_t)sizeof(double) > H.stage_bytes))
            fail("staged records exceed the buffer");
        val_next = vfirst + nval;
        if (H.wk_off[(size_t)(st * NW)] != first) fail("warp chunk start");
        for (int64_t w = 0; w < NW; ++w)
            if (H.wk_off[(size_t)(st * NW + w + 1)] < H.wk_off[(size_t)(st * NW + w)]) fail("warp chunk order");
        if (H.wk_off[(size_t)((st + 1) * NW)] != first + nev) fail("warp chunk end");
        int64_t pos = pfirst;
        for (int64_t i = first; i < first + nev; ++i) {
            const EvRec &r = H.ev[(size_t)i];
            if (r.user < 0 || r.user >= E || seen[(size_t)r.user]) fail("event permutation");
            seen[(size_t)r.user] = 1;
            stage_of[(size_t)r.user] = (int32_t)st;
            if (r.pred_begin != pos || r.pred_end < r.pred_begin || r.pred_end > pfirst + npred) fail("pred ranges");
            pos = r.pred_end;
        }
        if (pos != pfirst + npred) fail("stage pred count");
        ev_next = first + nev;
        pred_next = pfirst + npred;
    }
    if (ev_next != E || pred_next != P || val_next != (int64_t)H.vals.size()) fail("stage coverage");
    // sources and window slots, in execution order
    std::vector<int32_t> slot_of((size_t)E, -1), tenant((size_t)std::max(H.window_slots, 1), -1),
        last_read((size_t)std::max(H.window_slots, 1), -1);
    for (int64_t i = 0; i < E; ++i) slot_of[(size_t)H.ev[(size_t)i].user] = H.ev[(size_t)i].slot;
    for (int64_t st = 0, i = 0; st < NS; ++st) {
        const int64_t end = H.wk_off[(size_t)((st + 1) * NW)];
        const int32_t *sm = &H.stage_meta[(size_t)st * kStageMetaInts];
        int64_t drawn = -1;  // the block whose words the unit's registers hold (-1: none yet)
        for (; i < end; ++i) {
            const EvRec &r = H.ev[(size_t)i];
            const int64_t local = i - sm[0];
            if (!(local < 2 * (int64_t)sm[8] && (local & 1))) drawn = -1;  // a unit starts
            for (int64_t k = r.pred_begin; k < r.pred_end; ++k) {
                const PredRec &p = H.pred[(size_t)k];
                if (p.src_user < 0 || p.src_user >= E || stage_of[(size_t)p.src_user] >= st) fail("source order");
                if (p.link < -1 || p.link >= H.L) fail("link index");
                const int kind = p.kd & KD_KIND_MASK;
                if (kind < K_FIXED || kind > K_EMP_REL) fail("delay kind");
                if (kind != K_FIXED && (p.link < 0 || p.block < 0 || p.block >= H.L ||
                                        p.block != H.link_block[(size_t)p.link]))
                    fail("Philox block");
                if (kind != K_FIXED) {
                    const int64_t di = (int64_t)(p.kd >> 8);
                    if (di < 0 || di >= (int64_t)H.dist.size()) fail("distribution index");
                    const DistParam &dp = H.dist[(size_t)di];
                    if (!(kind == K_GAMMA && !dp.erlang)) {  // draws into the unit's registers
                        if ((p.kd & KD_REUSE) && p.block != drawn) fail("Philox block reuse");
                        drawn = p.block;
                    } else if (p.kd & (KD_REUSE | KD_TWO_WORD)) {
                        fail("Philox block reuse");
                    }
                    const bool emp = kind == K_EMP_ABS || kind == K_EMP_REL;
                    if (emp &&
                        (dp.tab_n <= 0 || dp.tab_off < 0 || (int64_t)dp.tab_off + dp.tab_n > (int64_t)H.alias.size()))
                        fail("alias table range");
                    if (emp && dp.link_tab) {
                        const int32_t *m = sm;
                        int64_t first;  // the table's first entry in the stage's value region
                        if (m[1] >= 0) {
                            if (p.dvo < 0 || (p.dvo & kVtGlobal) || (p.dvo - m[7]) % (int32_t)sizeof(double))
                                fail("link table offset");
                            first = (p.dvo - m[7]) / (int32_t)sizeof(double);
                        } else {
                            if (p.dvo < 0 || !(p.dvo & kVtGlobal)) fail("link table index");
                            first = (int64_t)(p.dvo ^ kVtGlobal) - m[4];
                        }
                        if (dp.tab_n > kLinkTableBins || first < 0 || first + dp.tab_n > m[5])
                            fail("link table range");
                        for (int32_t k = 0; k < dp.tab_n; ++k) {
                            const AliasPick &pk = H.picks[(size_t)(dp.tab_off + k)];
                            if (pk.alias < 0 || pk.alias >= dp.tab_n) fail("alias pick");
                        }
                    } else if (p.dvo != -1) {
                        fail("link table without a table");
                    }
                }
                if (!H.win_smem) {
                    if (p.src_slot != -1) fail("window slot without a window");
                    continue;
                }
                if (p.src_slot < 0 || p.src_slot >= H.window_slots || p.src_slot != slot_of[(size_t)p.src_user] ||
                    tenant[(size_t)p.src_slot] != p.src_user)
                    fail("window slot of a source");
                last_read[(size_t)p.src_slot] = std::max(last_read[(size_t)p.src_slot], (int32_t)st);
            }
            if (r.slot >= 0) {
                if (!H.win_smem || r.slot >= H.window_slots || last_read[(size_t)r.slot] >= st)
                    fail("window slot reuse");
                tenant[(size_t)r.slot] = r.user;
            } else if (r.slot != -1) {
                fail("window slot");
            }
        }
    }
}

void compile_dag(const mcd_dag_desc &d, const mcd_generator &g, HostDag &H, int32_t n_warps, int32_t window) {
    // ---- 1) distributions: the last add_* per type wins (dist_map_[t] = ..., _core.cpp:154-158)
    std::unordered_map<int32_t, size_t> type_spec;
    for (size_t i = 0; i < g.dists.size(); ++i) type_spec[g.dists[i].type] = i;
    if (type_spec.count(-1)) throw McdError(MCD_ERR_RUNTIME, "Activity type -1 is reserved for no delay");
    if (d.max_delay < 0.0) throw McdError(MCD_ERR_RUNTIME, "max_delay must be non-negative");
    if (d.n_events < 0 || d.n_activities < 0 || d.n_targets < 0)
        throw McdError(MCD_ERR_INVALID, "negative array length in DAG description");

    // Per-type compiled form: constant and degenerate laws become FIXED.
    struct TypeForm {
        int32_t kind;    // K_FIXED when duration = f(base) without randomness
        int32_t dist;    // index into H.dist
        int32_t fixed;   // 0: none, 1: base*(1+factor) style constant, 2: emp single value
        double factor;   // constant factor / single empirical value
        bool relative;
    };
    std::unordered_map<int32_t, TypeForm> form;
    H.dist.clear();
    H.alias.clear();
    H.picks.clear();
    std::unordered_map<int32_t, std::vector<double>> dist_values;  // empirical dists: values by bin
    for (const auto &kv : type_spec) {
        const DistSpec &s = g.dists[kv.second];
        TypeForm f{K_FIXED, -1, 0, 0.0, false};
        switch (s.kind) {
            case MCD_KIND_CONSTANT:
                f.fixed = 1;
                f.factor = s.p0;
                break;
            case MCD_KIND_EXPONENTIAL: {
                const double lam = s.p0;
                double ms = s.p1;
                if (std::isnan(lam) || lam < 0.0 || std::isinf(lam))
                    throw McdError(MCD_ERR_INVALID, "exponential lambda_ must be finite and non-negative");
                if (std::isnan(ms)) ms = INFINITY;  // x > NaN is never true: no truncation
                if (ms < 0.0) throw McdError(MCD_ERR_INVALID, "exponential max_scale must be non-negative");
                if (lam == 0.0) {  // rate 1/0: every draw is 0
                    f.fixed = 1;
                    f.factor = 0.0;
                    break;
                }
                DistParam p{};
                p.kind = K_EXP;
                const double ratio = ms / lam;
                const double c = std::isinf(ratio) ? 1.0 : -std::expm1(-ratio);
                const double omc = std::isinf(ratio) ? 0.0 : std::exp(-ratio);
                p.f0 = (float)lam;
                p.f1 = (float)c;
                p.f2 = (float)omc;
                p.f3 = float_at_or_below(ms);
                f.kind = K_EXP;
                f.dist = (int32_t)H.dist.size();
                H.dist.push_back(p);
                break;
            }
            case MCD_KIND_GAMMA: {
                const double k = s.p0, theta = s.p1;
                double ms = s.p2;
                if (!(k > 0.0) || std::isinf(k))
                    throw McdError(MCD_ERR_INVALID, "gamma shape must be finite and positive");
                if (!(theta >= 0.0) || std::isinf(theta))
                    throw McdError(MCD_ERR_INVALID, "gamma scale must be finite and non-negative");
                if (std::isnan(ms)) ms = INFINITY;
                if (theta == 0.0) {
                    f.fixed = 1;
                    f.factor = 0.0;
                    break;
                }
                if (!(ms > 0.0))
                    throw McdError(MCD_ERR_INVALID, "gamma max_scale must be positive (no draw would be accepted)");
                DistParam p{};
                p.kind = K_GAMMA;
                const double kk = k < 1.0 ? k + 1.0 : k;
                const double dd = kk - 1.0 / 3.0;
                p.boost = k < 1.0 ? 1 : 0;
                p.erlang = (k == 1.0 || k == 2.0 || k == 3.0) ? (int32_t)k : 0;
                p.f0 = (float)dd;
                p.f1 = (float)(1.0 / std::sqrt(9.0 * dd));
                p.f2 = (float)(1.0 / k);
                p.f3 = (float)theta;
                p.f4 = float_at_or_below(ms);
                f.kind = K_GAMMA;
                f.dist = (int32_t)H.dist.size();
                H.dist.push_back(p);
                break;
            }
            case MCD_KIND_EMP_ABS:
            case MCD_KIND_EMP_REL: {
                check_table(s);
                f.relative = s.kind == MCD_KIND_EMP_REL;
                if (s.values.size() == 1) {  // the reference draws nothing for one entry
                    f.fixed = 2;
                    f.factor = s.values[0];
                    break;
                }
                DistParam p{};
                p.kind = f.relative ? K_EMP_REL : K_EMP_ABS;
                p.tab_off = (int32_t)H.alias.size();
                p.tab_n = (int32_t)s.values.size();
                p.link_tab = p.tab_n <= kLinkTableBins ? 1 : 0;
                build_alias(s.values, s.weights, H.alias, H.picks);
                f.kind = p.kind;
                f.dist = (int32_t)H.dist.size();
                dist_values[f.dist] = s.values;
                H.dist.push_back(p);
                break;
            }
            default: throw McdError(MCD_ERR_INVALID, "unknown distribution kind");
        }
        form[kv.first] = f;
    }

    // ---- 2) dense links (_core.cpp:213-229)
    int32_t max_idx = -1;
    for (int32_t k = 0; k < d.n_activities; ++k) {
        if (d.act_idx[k] < 0) throw McdError(MCD_ERR_INVALID, "Activity.idx must be non-negative");
        max_idx = std::max(max_idx, d.act_idx[k]);
    }
    const int32_t L = max_idx + 1;
    H.L = L;
    H.link_kd.assign((size_t)L, K_FIXED);
    H.link_v.assign((size_t)L, 0.0);  // gaps: duration 0, no delay
    H.link_dv.assign((size_t)L, 0.0f);
    for (int32_t k = 0; k < d.n_activities; ++k) {
        const int32_t l = d.act_idx[k];
        const double base = d.act_duration[k];
        auto it = form.find(d.act_type[k]);
        if (it == form.end()) {
            H.link_kd[l] = K_FIXED;
            H.link_v[l] = base;
            H.link_dv[l] = 1.0f;
            continue;
        }
        const TypeForm &f = it->second;
        if (f.kind == K_FIXED) {
            double extra;
            if (f.fixed == 1) extra = base * f.factor;            // _core.cpp:75
            else extra = f.relative ? f.factor * base : f.factor;  // _core.cpp:125, 140
            H.link_kd[l] = K_FIXED;
            H.link_v[l] = base + extra;                           // _core.cpp:328
            H.link_dv[l] = (float)(f.fixed == 1 ? 1.0 + f.factor : (f.relative ? 1.0 + f.factor : 1.0));
        } else {
            H.link_kd[l] = f.kind | (f.dist << 8);
            H.link_v[l] = base;
        }
    }

    // ---- 3) precedence list, predecessors by target
    const int32_t E = d.n_events;
    H.E = E;
    std::vector<int64_t> tstart((size_t)E, -1), tlen((size_t)E, 0);
    for (int32_t t = 0; t < d.n_targets; ++t) {
        const int32_t tgt = d.target[t];
        if (tgt < 0 || tgt >= E) throw McdError(MCD_ERR_INVALID, "precedence_list target out of range");
        if (tstart[tgt] != -1)
            throw McdError(MCD_ERR_INVALID, "precedence_list names target " + std::to_string(tgt) + " twice");
        const int64_t b = d.pred_offsets[t], e = d.pred_offsets[t + 1];
        if (e < b) throw McdError(MCD_ERR_INVALID, "pred_offsets must be non-decreasing");
        tstart[tgt] = b;
        tlen[tgt] = e - b;
        for (int64_t p = b; p < e; ++p) {
            if (d.pred_src[p] < 0 || d.pred_src[p] >= E)
                throw McdError(MCD_ERR_INVALID, "predecessor event index out of range");
            if (d.pred_act[p] < 0) throw McdError(MCD_ERR_INVALID, "predecessor activity index is negative");
        }
    }
    if (d.n_targets > 0 && d.pred_offsets[d.n_targets] > (int64_t)std::numeric_limits<int32_t>::max())
        throw McdError(MCD_ERR_INVALID, "too many predecessor entries");

    // ---- 4) Kahn order (_core.cpp:235-264), with levels = longest path from a source
    std::vector<int64_t> adj_off((size_t)E + 1, 0);
    for (int32_t e = 0; e < E; ++e)
        for (int64_t k = 0; k < tlen[e]; ++k) adj_off[(size_t)d.pred_src[tstart[e] + k] + 1]++;
    for (int32_t e = 0; e < E; ++e) adj_off[e + 1] += adj_off[e];
    std::vector<int32_t> adj((size_t)adj_off[E]);
    {
        std::vector<int64_t> fill(adj_off.begin(), adj_off.end() - 1);
        for (int32_t e = 0; e < E; ++e)
            for (int64_t k = 0; k < tlen[e]; ++k) adj[(size_t)fill[(size_t)d.pred_src[tstart[e] + k]]++] = e;
    }
    std::vector<int64_t> indeg(tlen);
    std::vector<int32_t> level((size_t)E, 0);
    std::vector<int32_t> queue;
    queue.reserve((size_t)E);
    for (int32_t e = 0; e < E; ++e)
        if (indeg[e] == 0) queue.push_back(e);
    for (size_t qh = 0; qh < queue.size(); ++qh) {
        const int32_t nd = queue[qh];
        for (int64_t k = adj_off[nd]; k < adj_off[nd + 1]; ++k) {
            const int32_t c = adj[(size_t)k];
            level[c] = std::max(level[c], level[nd] + 1);
            if (--indeg[c] == 0) queue.push_back(c);
        }
    }
    if ((int64_t)queue.size() != (int64_t)E)
        throw McdError(MCD_ERR_RUNTIME, "Invalid DAG: cycle detected in precedence list");
    int32_t n_levels = 0;
    for (int32_t e = 0; e < E; ++e) n_levels = std::max(n_levels, level[e] + 1);
    H.n_levels = n_levels;

    H.max_preds = 0;
    for (int32_t e = 0; e < E; ++e) H.max_preds = std::max<int64_t>(H.max_preds, tlen[e]);

    // ---- 5) last level at which each event is read
    std::vector<int32_t> last_use((size_t)E, -1);
    for (int32_t e = 0; e < E; ++e)
        for (int64_t k = 0; k < tlen[e]; ++k) {
            const int32_t s = d.pred_src[tstart[e] + k];
            last_use[s] = std::max(last_use[s], level[e]);
        }

    // ---- 6) events by level (stable in caller order)
    std::vector<int32_t> lvl_off((size_t)n_levels + 1, 0);
    for (int32_t e = 0; e < E; ++e) lvl_off[(size_t)level[e] + 1]++;
    for (int32_t l = 0; l < n_levels; ++l) lvl_off[l + 1] += lvl_off[l];
    std::vector<int32_t> by_level((size_t)E);
    {
        std::vector<int32_t> fill(lvl_off.begin(), lvl_off.end() - 1);
        for (int32_t e = 0; e < E; ++e) by_level[(size_t)fill[(size_t)level[e]]++] = e;
    }

    // ---- 7) window slots: linear scan over levels, a slot is free again after
    // the last level that reads its event
    std::vector<int32_t> slot((size_t)E, -1);
    {
        std::vector<int32_t> free_slots;
        std::vector<std::vector<int32_t>> release((size_t)n_levels + 1);
        int32_t n_slots = 0;
        for (int32_t l = 0; l < n_levels; ++l) {
            for (int32_t s : release[l]) free_slots.push_back(s);
            for (int32_t i = lvl_off[l]; i < lvl_off[l + 1]; ++i) {
                const int32_t e = by_level[i];
                if (last_use[e] < 0) continue;
                int32_t s;
                if (!free_slots.empty()) {
                    s = free_slots.back();
                    free_slots.pop_back();
                } else {
                    s = n_slots++;
                }
                slot[e] = s;
                release[(size_t)last_use[e] + 1].push_back(s);
            }
        }
        H.window_slots = n_slots;
    }

    // ---- 8) warps per CTA; work cost of an event for balancing the warps
    int32_t nw = 1;
    if (n_levels > 0) {
        const double avg_width = (double)E / (double)n_levels;
        nw = (int32_t)std::ceil(avg_width / 6.0);
    }
    if (const char *env = std::getenv("MCD_WARPS")) nw = std::atoi(env);
    if (n_warps > 0) nw = n_warps;
    if (n_warps == kBatchClassWarps) nw = nw <= 2 ? 2 : nw <= 4 ? 4 : nw <= 8 ? 8 : nw <= 12 ? 12 : 24;
    nw = std::max(1, std::min(kMaxWarps, nw));
    H.n_warps = nw;
    // relative cost of an edge by delay kind (kernel time per edge, fixed = 1)
    // and of an event's own work
    auto kind_cost = [&](int32_t l) -> double {
        if (l >= L) return 1.0;
        switch (H.link_kd[l] & KD_KIND_MASK) {
            case K_FIXED: return 1.0;
            case K_EXP: return 2.4;
            case K_GAMMA: return 3.5;
            default: return 2.0;
        }
    };
    std::vector<double> cost((size_t)E, 1.0);
    for (int32_t e = 0; e < E; ++e)
        for (int64_t k = 0; k < tlen[e]; ++k) cost[e] += kind_cost(d.pred_act[tstart[e] + k]);

    // Within a level, costliest events first: warps take a stage's events one at
    // a time from a shared counter, so this is longest-processing-time order.
    for (int32_t l = 0; l < n_levels; ++l)
        std::stable_sort(by_level.begin() + lvl_off[l], by_level.begin() + lvl_off[l + 1],
                         [&](int32_t x, int32_t y) { return cost[x] > cost[y]; });

    // per-link duration tables: bins of an empirical link's own table (kLinkTableBins), 0 without
    auto table_bins = [&](int32_t l) -> int32_t {
        if (l < 0 || l >= L) return 0;
        const int kind = H.link_kd[l] & KD_KIND_MASK;
        if (kind != K_EMP_ABS && kind != K_EMP_REL) return 0;
        const DistParam &dp = H.dist[(size_t)(H.link_kd[l] >> 8)];
        return dp.link_tab ? dp.tab_n : 0;
    };
    auto one_word = [&](int32_t l) {
        const int kind = H.link_kd[l] & KD_KIND_MASK;
        return kind == K_EXP || ((kind == K_EMP_ABS || kind == K_EMP_REL) &&
                                 H.dist[(size_t)(H.link_kd[l] >> 8)].tab_n <= kOneWordBins);
    };
    auto link_words = [&](int32_t l) -> int32_t {  // words of a shared block the link's first draw takes
        if (one_word(l)) return 1;
        if ((H.link_kd[l] & KD_KIND_MASK) == K_GAMMA) return H.dist[(size_t)(H.link_kd[l] >> 8)].erlang;
        return 0;
    };
    // Words an event's draws take from shared blocks, when all of them do (-1:
    // some reference draws a block of its own).  Two events of a level whose words
    // add up to at most four draw one block between them when one warp runs them
    // back to back (step 8b pairs such events).
    std::vector<int32_t> ev_words((size_t)E, 0);
    for (int32_t e = 0; e < E; ++e)
        for (int64_t k = 0; k < tlen[e] && ev_words[e] >= 0; ++k) {
            const int32_t l = d.pred_act[tstart[e] + k];
            if (l >= L || (H.link_kd[l] & KD_KIND_MASK) == K_FIXED) continue;
            const int32_t w = link_words(l);
            ev_words[e] = w > 0 ? ev_words[e] + w : -1;
        }
    std::vector<int64_t> ev_vals((size_t)E, 0);  // value-region entries of an event's references
    for (int32_t e = 0; e < E; ++e)
        for (int64_t k = 0; k < tlen[e]; ++k) ev_vals[e] += table_bins(d.pred_act[tstart[e] + k]);
    auto ev_bytes = [&](int32_t e) {  // an event's records and value region in a staging buffer
        return sizeof(EvRec) + (size_t)tlen[e] * sizeof(PredRec) + (size_t)ev_vals[e] * sizeof(double);
    };

    // ---- 8b) work units, level by level: pairs of events drawing 1-3 words each,
    // at most four together (3 + 1, 2 + 2, 2 + 1, 1 + 1; each class costliest
    // first), then the other events.  A level lists its pairs (costliest first)
    // before its single events (in cost order).  The units depend on the levels
    // and the delay kinds only -- not on warps per CTA, the window's place or the
    // staging budget -- so a sample's draws are the same under every layout.  Only
    // events of at most kMinStageBytes / 4 of records pair up, so a pair always
    // fits the smallest staging buffer.
    std::vector<char> pair_first((size_t)E, 0);
    {
        std::vector<int32_t> by_w[4], seq;
        std::vector<std::pair<int32_t, int32_t>> pairs;
        std::vector<char> paired((size_t)E, 0);
        for (int32_t l = 0; l < n_levels; ++l) {
            for (auto &v : by_w) v.clear();
            for (int32_t k = lvl_off[l]; k < lvl_off[l + 1]; ++k) {
                const int32_t e = by_level[k];
                if (ev_words[e] >= 1 && ev_words[e] <= 3 && ev_bytes(e) <= kMinStageBytes / 4)
                    by_w[ev_words[e]].push_back(e);
            }
            size_t at[4] = {0, 0, 0, 0};
            pairs.clear();
            auto pair_up = [&](int wa, int wb) {
                while (at[wa] < by_w[wa].size() && at[wb] + (wa == wb ? 1 : 0) < by_w[wb].size()) {
                    const int32_t ea = by_w[wa][at[wa]++];
                    pairs.emplace_back(ea, by_w[wb][at[wb]++]);
                }
            };
            pair_up(3, 1);
            pair_up(2, 2);
            pair_up(2, 1);
            pair_up(1, 1);
            if (pairs.empty()) continue;
            std::stable_sort(pairs.begin(), pairs.end(), [&](const auto &x, const auto &y) {
                return cost[x.first] + cost[x.second] > cost[y.first] + cost[y.second];
            });
            seq.clear();
            for (const auto &pr : pairs) {
                seq.push_back(pr.first);
                seq.push_back(pr.second);
                paired[(size_t)pr.first] = paired[(size_t)pr.second] = 1;
                pair_first[(size_t)pr.first] = 1;
            }
            for (int32_t k = lvl_off[l]; k < lvl_off[l + 1]; ++k)
                if (!paired[(size_t)by_level[k]]) seq.push_back(by_level[k]);
            std::copy(seq.begin(), seq.end(), by_level.begin() + lvl_off[l]);
        }
    }

    // ---- 9) shared-memory budget: window rows, two record staging buffers
    // (each stage's event and predecessor records and value region), distribution tables
    const size_t table_bytes =
        H.dist.size() * sizeof(DistParam) + H.alias.size() * (sizeof(AliasEntry) + sizeof(AliasPick));
    H.tables_in_smem = table_bytes <= kMaxTableBytes;
    const size_t fixed_bytes = (H.tables_in_smem ? table_bytes : 0) + 3 * 128;
    const size_t win_bytes = (size_t)H.window_slots * kTile * sizeof(double);
    H.win_smem = win_bytes <= kMaxWindowBytes && win_bytes + fixed_bytes + 2 * kMinStageBytes <= kSmemMax &&
                 window != MCD_WINDOW_GLOBAL && std::getenv("MCD_NO_SMEM_WINDOW") == nullptr;
    const size_t avail = kSmemMax - fixed_bytes - (H.win_smem ? win_bytes : 0);
    size_t budget = std::min(kMaxStageBytes, avail / 2 > 256 ? avail / 2 - 256 : avail / 2);  // room for padding

    // ---- 10) stages (a level, or a slice of a wide level that fits a buffer)
    // and per-(stage, warp) chunks balanced by cost
    std::vector<int32_t> order;
    std::vector<int32_t> meta;  // ev_first, n_ev (negated: unstaged), n_pred, n_val (even), offsets, pairs
    std::vector<int32_t> wk;
    for (;;) {
        order.clear();
        meta.clear();
        wk.clear();
        size_t max_bytes = 0;
        for (int32_t l = 0; l < n_levels; ++l) {
            int32_t i = lvl_off[l];
            while (i < lvl_off[l + 1]) {
                // one stage: events i .. j-1 of this level (a pair is never split)
                int32_t j = i;
                size_t bytes = 0, nev = 0, npred = 0, nval = 0;
                while (j < lvl_off[l + 1]) {
                    const int32_t cnt = pair_first[by_level[j]] ? 2 : 1;
                    size_t add = 0;
                    for (int32_t k = j; k < j + cnt; ++k) add += ev_bytes(by_level[k]);
                    if (j > i && bytes + add > budget) break;
                    bytes += add;
                    for (int32_t k = j; k < j + cnt; ++k) {
                        nev += 1;
                        npred += (size_t)tlen[by_level[k]];
                        nval += (size_t)ev_vals[by_level[k]];
                    }
                    j += cnt;
                }
                nval = (nval + 1) / 2 * 2;  // 16-byte copies
                if (nval > (size_t)std::numeric_limits<int32_t>::max() / 2)
                    throw McdError(MCD_ERR_INVALID, "too many per-link table entries in one level");
                const bool staged = bytes <= budget;
                if (staged) max_bytes = std::max(max_bytes, nev * sizeof(EvRec) + npred * sizeof(PredRec) +
                                                               nval * sizeof(double));
                int32_t n_pairs = 0;
                for (int32_t k = i; k < j; ++k) n_pairs += pair_first[by_level[k]];
                double total = 0.0;
                for (int32_t k = i; k < j; ++k) total += cost[by_level[k]];
                const int32_t first = (int32_t)order.size();
                double acc = 0.0;
                int32_t w = 0;
                wk.push_back(first);
                for (int32_t k = i; k < j; ++k) {
                    const int32_t e = by_level[k];
                    const double c = cost[e];
                    while (w + 1 < nw && acc + 0.5 * c > total * (double)(w + 1) / (double)nw) {
                        ++w;
                        wk.push_back((int32_t)order.size());
                    }
                    order.push_back(e);
                    acc += c;
                }
                while (w + 1 < nw) {
                    ++w;
                    wk.push_back((int32_t)order.size());
                }
                meta.push_back(first);
                meta.push_back(staged ? (int32_t)nev : -(int32_t)nev);
                meta.push_back((int32_t)npred);
                meta.push_back((int32_t)nval);
                meta.push_back((int32_t)(nev * sizeof(EvRec)));  // 48-byte records: 16-byte aligned offsets
                meta.push_back((int32_t)(nev * sizeof(EvRec) + npred * sizeof(PredRec)));
                meta.push_back(n_pairs);
                i = j;
            }
        }
        wk.push_back((int32_t)order.size());
        H.stage_bytes = (int32_t)((max_bytes + 127) / 128 * 128);
        if (2 * (size_t)H.stage_bytes <= avail || budget <= kMinStageBytes) break;
        budget = std::max(kMinStageBytes, budget * 3 / 4);
    }
    constexpr size_t kMetaPerStage = 7;
    H.n_stages = (int32_t)(meta.size() / kMetaPerStage);
    H.wk_off = wk;
    // stage_meta with predecessor and value offsets (records and value regions
    // are laid out in compiled order)
    H.stage_meta.assign((size_t)H.n_stages * kStageMetaInts, 0);
    {
        int64_t pos = 0, vpos = 0;
        for (int32_t st = 0; st < H.n_stages; ++st) {
            int32_t *m = &H.stage_meta[(size_t)st * kStageMetaInts];
            const int32_t *q = &meta[(size_t)st * kMetaPerStage];
            m[0] = q[0];
            m[1] = q[1];
            m[2] = (int32_t)pos;
            m[3] = q[2];
            if (vpos + q[3] >= (int64_t)kVtGlobal)  // table indices must stay below the flag bit
                throw McdError(MCD_ERR_INVALID, "too many per-link table entries");
            m[4] = (int32_t)vpos;
            m[5] = q[3];
            m[6] = q[4];
            m[7] = q[5];
            m[8] = q[6];
            pos += q[2];
            vpos += q[3];
        }
    }
    // layout: [window][stage buffer 0][stage buffer 1][tables][2 mbarriers, 2 stage counters]
    {
        size_t off = H.win_smem ? win_bytes : 0;
        off = (off + 127) / 128 * 128;
        H.smem_stage_off = (int32_t)off;
        off += 2 * (size_t)H.stage_bytes;
        off = (off + 127) / 128 * 128;
        H.smem_tables_off = (int32_t)off;
        if (H.tables_in_smem) off += table_bytes;
        off = (off + 15) / 16 * 16;
        H.smem_bar_off = (int32_t)off;
        off += kBarRegionBytes;
        H.smem_total = (int32_t)off;
        if (off > kSmemMax) throw McdError(MCD_ERR_INVALID, "compiled DAG does not fit the shared-memory budget");
    }

    // ---- 9) records in compiled order
    H.ev.resize((size_t)E);
    H.pred.clear();
    H.pred.reserve((size_t)(d.n_targets > 0 ? d.pred_offsets[d.n_targets] : 0));
    std::vector<char> referenced((size_t)L, 0), written((size_t)L, 0);
    // Philox blocks (see KD_REUSE): links drawing from a shared block group per
    // work unit, up to four words a block; the rest own one
    H.link_block.assign((size_t)L, -1);
    H.link_word.assign((size_t)L, -1);
    H.earliest.assign(d.earliest, d.earliest + E);
    H.ub.resize((size_t)E);
    H.max_delay = d.max_delay;
    H.times_finite = std::isfinite(d.max_delay);
    H.max_abs_time = 0.0;
    H.max_span = 0.0;
    for (int32_t e = 0; e < E; ++e) {
        H.ub[e] = d.earliest[e] + d.max_delay;
        if (!std::isfinite(d.earliest[e]) || !std::isfinite(H.ub[e])) H.times_finite = false;
        H.max_abs_time = std::max(H.max_abs_time, std::max(std::fabs(d.earliest[e]), std::fabs(H.ub[e])));
        H.max_span = std::max(H.max_span, H.ub[e] - d.earliest[e]);
    }
    H.vals.clear();
    int32_t st_cur = -1;
    int64_t st_end = 0, vbase = 0;
    auto close_stage = [&]() {  // pad the stage's value region to its recorded (even) size
        if (st_cur < 0) return;
        const int32_t *m = &H.stage_meta[(size_t)st_cur * kStageMetaInts];
        if ((int64_t)H.vals.size() - vbase > m[5]) throw McdError(MCD_ERR_RUNTIME, "value region overflow");
        while ((int64_t)H.vals.size() < vbase + m[5]) H.vals.push_back(0.0);
    };
    int32_t group = -1, group_n = 0;  // the work unit's open Philox block of one-word links
    int32_t last_block = -1;          // block its last non-gamma random reference drew (in registers)
    for (int32_t i = 0; i < E; ++i) {
        const int32_t e = order[i];
        while (i >= st_end) {  // the first event of the next stage
            close_stage();
            ++st_cur;
            const int32_t *m = &H.stage_meta[(size_t)st_cur * kStageMetaInts];
            st_end = (int64_t)m[0] + (m[1] >= 0 ? m[1] : -(int64_t)m[1]);
            vbase = (int64_t)H.vals.size();
            if (vbase != m[4]) throw McdError(MCD_ERR_RUNTIME, "value region offset");
        }
        {  // the second event of a pair continues its unit's block; any other event starts a unit
            const int32_t *m = &H.stage_meta[(size_t)st_cur * kStageMetaInts];
            const int64_t local = (int64_t)i - m[0];
            if (!(local < 2 * (int64_t)m[8] && (local & 1))) {
                group = -1;
                group_n = 0;
                last_block = -1;
            }
        }
        EvRec r{};
        r.user = e;
        r.slot = H.win_smem ? slot[e] : -1;
        r.pred_begin = (int32_t)H.pred.size();
        const double earliest = d.earliest[e];
        const double ub = earliest + d.max_delay;  // _core.cpp:334
        r.init_bits = bits_of(earliest);
        r.init_key = std::isnan(earliest) ? std::numeric_limits<int64_t>::max() : order_key_host(r.init_bits);
        r.ub_bits = bits_of(ub);
        r.ub_key = std::isnan(ub) ? std::numeric_limits<int64_t>::max() : order_key_host(r.ub_bits);
        for (int64_t k = 0; k < tlen[e]; ++k) {
            const int32_t src = d.pred_src[tstart[e] + k];
            const int32_t l = d.pred_act[tstart[e] + k];
            PredRec p{};
            p.src_slot = H.win_smem ? slot[src] : -1;
            p.src_user = src;
            if (l >= L) {
                // Past the last link the reference reads beyond its duration
                // buffer (_core.cpp:340-341, undefined); in practice it reads 0.0
                // and its own chain test (test_simulator.py:175-199) relies on
                // that, so such an edge has duration 0 here.
                p.link = -1;
                p.kd = K_FIXED;
                p.v = 0.0;
                p.dvo = float_bits(0.0f);
            } else {
                p.link = l;
                p.kd = H.link_kd[l];
                p.v = H.link_v[l];
                p.dvo = float_bits(H.link_dv[l]);
                p.block = -1;
                if ((H.link_kd[l] & KD_KIND_MASK) != K_FIXED) {
                    const int32_t nw = link_words(l);
                    if (H.link_block[l] < 0) {  // first reference: the link's block and first word
                        if (nw > 0) {
                            if (group < 0 || group_n + nw > 4) {
                                group = l;
                                group_n = 0;
                            }
                            H.link_block[l] = group;
                            H.link_word[l] = (int8_t)group_n;
                            group_n += nw;
                        } else {
                            H.link_block[l] = l;
                        }
                    }
                    p.block = H.link_block[l];
                    const bool mt_gamma = (H.link_kd[l] & KD_KIND_MASK) == K_GAMMA && nw == 0;
                    if (!mt_gamma) {  // draws into the shared registers
                        if (nw > 0) p.kd |= (int32_t)H.link_word[l] << KD_WORD_SHIFT;
                        else p.kd |= KD_TWO_WORD;
                        if (p.block == last_block) p.kd |= KD_REUSE;
                        last_block = p.block;
                    }
                }
                if ((H.link_kd[l] & KD_KIND_MASK) != K_FIXED) p.dvo = -1;
                if (const int32_t nb = table_bins(l)) {  // the link's duration table, bin by bin
                    const int32_t di = H.link_kd[l] >> 8;
                    const bool rel = (H.link_kd[l] & KD_KIND_MASK) == K_EMP_REL;
                    const double base = H.link_v[l];
                    const int32_t *sm = &H.stage_meta[(size_t)st_cur * kStageMetaInts];
                    const int64_t local = (int64_t)H.vals.size() - vbase;
                    if (sm[1] >= 0) p.dvo = (int32_t)(sm[7] + local * (int64_t)sizeof(double));  // staged: byte offset
                    else p.dvo = kVtGlobal | (int32_t)(vbase + local);                           // index in vals
                    const std::vector<double> &vv = dist_values[di];
                    for (int32_t k = 0; k < nb; ++k)
                        H.vals.push_back(rel ? base + vv[(size_t)k] * base : base + vv[(size_t)k]);  // _core.cpp:140, 328
                }
                if (!written[l]) {  // the first reference stores the link's duration row
                    p.kd |= KD_WRITE;
                    written[l] = 1;
                }
                referenced[l] = 1;
            }
            H.pred.push_back(p);
        }
        r.pred_end = (int32_t)H.pred.size();
        H.ev[i] = r;
    }
    close_stage();
    // ---- 12) positive mode: every earliest, bound and duration is a non-negative
    // finite double, so t = src + dur never is NaN or negative and the raw bit
    // patterns order like the values
    {
        auto nonneg = [](double x) { return std::isfinite(x) && !std::signbit(x); };
        bool pos = nonneg(d.max_delay);
        for (int32_t e = 0; pos && e < E; ++e) pos = nonneg(d.earliest[e]) && nonneg(H.ub[e]);
        for (int32_t l = 0; pos && l < L; ++l) pos = nonneg(H.link_v[l]) && H.link_v[l] < 1e300;
        for (const AliasEntry &ae : H.alias) pos = pos && nonneg(ae.v_self) && nonneg(ae.v_alias) && ae.v_self < 1e300;
        for (double x : H.vals) pos = pos && nonneg(x);
        H.positive = pos;
    }
    H.aux.clear();
    H.n_orphan = 0;
    for (int32_t l = 0; l < L; ++l) {
        if (!referenced[l]) ++H.n_orphan;
        if (written[l]) continue;
        // an unreferenced random link owns its block (word 0)
        int32_t kd = H.link_kd[l];
        if ((kd & KD_KIND_MASK) != K_FIXED) {
            H.link_block[l] = l;
            if (link_words(l) > 0) H.link_word[l] = 0;
            else if ((kd & KD_KIND_MASK) != K_GAMMA) kd |= KD_TWO_WORD;
        }
        H.aux.push_back(LinkRec{l, kd, H.link_v[l]});
    }
    // what the work units save: Philox blocks a sample's propagation draws
    H.n_pairs = 0;
    for (int32_t st = 0; st < H.n_stages; ++st) H.n_pairs += H.stage_meta[(size_t)st * kStageMetaInts + 8];
    H.block_draws = 0;
    for (const PredRec &p : H.pred)
        if ((p.kd & KD_KIND_MASK) != K_FIXED && !(p.kd & KD_REUSE)) ++H.block_draws;
    verify_layout(H);
}

size_t tables_bytes(const HostDag &h) {
    return h.dist.size() * sizeof(DistParam) + h.alias.size() * (sizeof(AliasEntry) + sizeof(AliasPick));
}

std::vector<unsigned char> tables_block(const HostDag &h) {
    std::vector<unsigned char> b(tables_bytes(h));
    size_t o = 0;
    auto put = [&](const void *src, size_t n) {
        if (n) std::memcpy(b.data() + o, src, n);
        o += n;
    };
    put(h.dist.data(), h.dist.size() * sizeof(DistParam));
    put(h.alias.data(), h.alias.size() * sizeof(AliasEntry));
    put(h.picks.data(), h.picks.size() * sizeof(AliasPick));
    return b;
}

// Ticks of 2^-q seconds: every |time| * 2^q must stay below 2^62, one sample's
// (realized - earliest) * 2^q below 2^53 (the kernels sum a warp's counts in two
// 27-bit limbs), and the sum over n samples below 2^63.
StatsParams stats_params(const HostDag &h, int64_t n) {
    StatsParams p;
    const double span = std::max(h.max_span, 0.0);
    if (h.times_finite) {
        const int lg_abs = (int)std::ceil(std::log2(std::max(h.max_abs_time, 1.0) * 1.001));
        const int lg_span = (int)std::ceil(std::log2(std::max(span, 1e-300) * 1.001 + 1e-300));
        const int lg_n = (int)std::ceil(std::log2((double)std::max<int64_t>(n, 2)));
        int q = std::min(61 - lg_abs, 62 - lg_n - std::max(lg_span, -1000));
        q = std::min(q, 53 - std::max(lg_span, -1000));
        q = std::min(q, 1000);
        if (q >= -60) {
            p.fixed = 1;
            p.q = q;
            const long double dt = std::ceil((long double)span * std::ldexp(1.0L, q)) + 1.0L;  // span in ticks
            if (dt <= (long double)kHistBins) {
                p.bin_mul = ~0ull;  // spans under 256 ticks: the tick count is the bin
                p.bin_w = 1.0 / std::ldexp(1.0, q);
            } else {
                const long double mul = std::ldexp((long double)kHistBins, 64) / dt;
                p.bin_mul = mul >= 18446744073709551615.0L ? ~0ull : (unsigned long long)mul;
                p.bin_w = (double)(dt / kHistBins / std::ldexp(1.0L, q));
            }
            return p;
        }
    }
    p.fixed = 0;
    if (std::isfinite(span) && span > 0.0) {
        p.inv_w = (double)kHistBins / span;
        p.bin_w = span / kHistBins;
    }
    return p;
}

}  // namespace mcd
