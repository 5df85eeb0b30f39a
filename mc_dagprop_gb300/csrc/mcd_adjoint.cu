// mcd_adjoint.cu -- pathwise gradient of the expected total tardiness
//   J = mean over samples of sum over events of (realized - earliest)
// with respect to every event's earliest time and every link's base duration.
//
// Forward (k_propagate<..., ADJ>, mcd_device.cuh) records for each event and
// sample which predecessor won the maximum, whether the bound clamped it, and
// d(duration)/d(base) of that link.  Along the winning chain realized times add
// up with slope 1, so for one sample
//   dJ/d realized_e * S = cnt_e = [realized_e > earliest_e] + sum of cnt_c over
//                         events c whose unclamped winning predecessor is e,
// an integer.  The backward kernel walks the stages in reverse, keeping cnt of
// the events still to be visited in a shared-memory window (the forward
// window's slots: an event's live range is the same in both directions), and
// accumulates exactly, as integers:
//   grad_earliest_e * S = sum_s (cnt_e [no predecessor won, or clamped] - [delayed])
//   grad_base_l * S     = sum_s cnt_e * d(duration_l)/d(base_l)   (l the winning link)
// the second in fixed point (2^-20).
#include "mcd_device.cuh"

namespace mcd {

// One CTA per tile of 32 samples; warps take each stage's events one at a time
// from the stage's counter, stages from a.stage_end - 1 down to a.stage_begin
// (the whole DAG, or one level block of a recomputation).  Counts of events still
// to be visited: with the window on chip, the forward window's slots in shared
// memory -- [counts: window_slots x 32 uint32][stage buffer 0][stage buffer
// 1][tables][2 mbarriers], the forward layout, whose window rows are twice the
// size the counts need -- started from and left in a.cnt_ckpt between blocks
// (kAdjCntLoad / kAdjCntSave); otherwise one uint32 per event and sample in
// a.cnt_rows (global, by caller index).  Records: row (compiled index -
// a.code_base) of a.adj_code / a.adj_dfac.
template <bool WIN_SMEM>
__global__ void __launch_bounds__(768) k_adjoint(const KArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    uint32_t *cnt = reinterpret_cast<uint32_t *>(smem);
    char *stage_buf0 = reinterpret_cast<char *>(smem + a.smem_stage_off);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + a.smem_bar_off);
    const int lane = threadIdx.x & 31;
    const int64_t s = (int64_t)blockIdx.x * kTile + lane;
    const bool active = s < a.n;
    const int cnt_n = a.window_slots * kTile;
    if (WIN_SMEM) {
        const uint32_t *in = (a.adj_flags & kAdjCntLoad) ? a.cnt_ckpt + (int64_t)blockIdx.x * cnt_n : nullptr;
        for (int i = threadIdx.x; i < cnt_n; i += blockDim.x) cnt[i] = in ? in[i] : 0u;
    }
    int *stage_ctr = reinterpret_cast<int *>(bars + 2);
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        stage_ctr[0] = 0;
        stage_ctr[1] = 0;
    }
    __syncthreads();
    const int NS = a.stage_end - a.stage_begin;
    if (threadIdx.x == 0) {
        if (NS > 0) stage_issue(a, a.stage_end - 1, stage_buf0, &bars[0]);
        if (NS > 1) stage_issue(a, a.stage_end - 2, stage_buf0 + a.stage_bytes, &bars[1]);
    }
    for (int j = 0; j < NS; ++j) {  // j-th stage from the end of the range
        const int l = a.stage_end - 1 - j;
        const int b = j & 1;
        const char *buf = stage_buf0 + b * a.stage_bytes;
        const bool ok = stage_wait(&bars[b], (uint32_t)((j >> 1) & 1), a.err);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0 && j + 1 < NS) stage_wait(&bars[b ^ 1], (uint32_t)(((j + 1) >> 1) & 1), a.err);
            __syncthreads();
            return;
        }
        const int4 meta = __ldg(reinterpret_cast<const int4 *>(a.stage_meta + kStageMetaInts * l));
        const int pred_boff = __ldg(a.stage_meta + kStageMetaInts * l + 6);
        const EvRec *sev = meta.y >= 0 ? reinterpret_cast<const EvRec *>(buf) : a.ev + meta.x;
        const PredRec *spred = meta.y >= 0 ? reinterpret_cast<const PredRec *>(buf + pred_boff)
                                           : a.pred + meta.z;
        const int n_ev = meta.y >= 0 ? meta.y : -meta.y;
        if (threadIdx.x == 0) stage_ctr[(j + 1) & 1] = 0;  // last used by stage j - 1, before the barrier
        const uint32_t ctr = smem_u32(&stage_ctr[j & 1]);
        // events one at a time from the stage's counter, the next taken ahead
        int i_next = 0;
        if (lane == 0) i_next = take_next(ctr);
        i_next = __shfl_sync(0xFFFFFFFFu, i_next, 0);
        while (i_next < n_ev) {
            const int i = i_next;
            if (lane == 0) i_next = take_next(ctr);
            const EvRec ev = load_ev(sev + i);
            const int64_t o = (int64_t)row_off(meta.x + i - a.code_base, (uint32_t)a.ld) + s;
            const uint32_t code = active ? (uint32_t)a.adj_code[o] : kAdjNone;
            const float dfac = active ? a.adj_dfac[o] : 0.0f;
            const uint32_t k = code & kAdjNone;
            const bool clamped = (code & kAdjClamped) != 0u;
            const bool delayed = (code & kAdjDelayed) != 0u;
            uint32_t c = delayed ? 1u : 0u;
            if (WIN_SMEM) {
                if (ev.slot >= 0) {  // read and clear: the slot's next tenant starts from zero
                    c += cnt[ev.slot * kTile + lane];
                    cnt[ev.slot * kTile + lane] = 0u;
                }
            } else if (active) {
                c += a.cnt_rows[(int64_t)row_off(ev.user, (uint32_t)a.ld) + s];
            }
            if (!active) c = 0u;
            // this lane's share of d J / d earliest, >= -1: summed over the warp as ge + 1
            const long long ge = ((k == kAdjNone || clamped) ? (long long)c : 0ll) - (delayed ? 1ll : 0ll);
            const long long ge_sum = warp_sum_ticks(ge + 1) - 32;
            if (lane == 0 && ge_sum != 0)
                atomicAdd(reinterpret_cast<unsigned long long *>(&a.grad_e[ev.user]), (unsigned long long)ge_sum);
            const bool wins = k != kAdjNone && !clamped && c != 0u;
            const unsigned wmask = __ballot_sync(0xFFFFFFFFu, wins);
            if (wins) {
                const PredRec pr = load_pred(spred + (ev.pred_begin - meta.z + (int)k));
                if (WIN_SMEM) {
                    if (pr.src_slot >= 0) atomicAdd(&cnt[pr.src_slot * kTile + lane], c);
                } else {
                    atomicAdd(&a.cnt_rows[(int64_t)row_off(pr.src_user, (uint32_t)a.ld) + s], c);
                }
                // lanes whose winner is the same predecessor add their link terms in one atomic
                const long long gl = (pr.link >= 0 && dfac != 0.0f)
                                         ? __float2ll_rn((float)c * dfac * (float)(1 << kAdjDfacShift))
                                         : 0ll;
                const unsigned grp = __match_any_sync(wmask, k);
                long long sum = 0;
                for (unsigned mm = grp; mm; mm &= mm - 1) sum += __shfl_sync(grp, gl, __ffs(mm) - 1);
                if (lane == __ffs(grp) - 1 && pr.link >= 0 && sum != 0)
                    atomicAdd(reinterpret_cast<unsigned long long *>(&a.grad_l[pr.link]), (unsigned long long)sum);
            }
            i_next = __shfl_sync(0xFFFFFFFFu, i_next, 0);
        }
        __syncthreads();
        if (threadIdx.x == 0 && j + 2 < NS) stage_issue(a, l - 2, stage_buf0 + b * a.stage_bytes, &bars[b]);
    }
    if (WIN_SMEM && (a.adj_flags & kAdjCntSave)) {  // counts of earlier events, for the next block down
        uint32_t *out = a.cnt_ckpt + (int64_t)blockIdx.x * cnt_n;
        for (int i = threadIdx.x; i < cnt_n; i += blockDim.x) out[i] = cnt[i];
    }
}

// Forward half: the propagation kernel in its adjoint form.  With the window
// off chip, predecessors come from (and realized times go to) the global rows
// a.scratch[E][ld], which hold every event's time: a level block's recomputation
// needs no other checkpoint.
template <bool WIN_SMEM, bool POSITIVE, int TS>
__global__ void __launch_bounds__(768) k_adjoint_forward(const KArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    propagate_tile<false, WIN_SMEM, false, POSITIVE, true, TS>(a, (int64_t)blockIdx.x, WIN_SMEM ? nullptr : a.scratch,
                                                               a.ld, false, smem,
                                                               reinterpret_cast<uint64_t *>(smem + a.smem_bar_off),
                                                               false);
}

// grad_earliest[e] = grad_e[e] / n, grad_base[l] = grad_l[l] 2^-20 / n, and the
// objective sum_e acc[e] 2^-q / n (one thread).
__global__ void k_adjoint_finish(const long long *grad_e, const long long *grad_l, const unsigned long long *acc,
                                 int32_t E, int32_t L, int64_t n, int32_t q, double *g_earliest, double *g_base,
                                 double *objective) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double dn = (double)n;
    if (i < E && g_earliest) g_earliest[i] = (double)grad_e[i] / dn;
    if (i < L && g_base) g_base[i] = ldexp((double)grad_l[i], -kAdjDfacShift) / dn;
    if (objective && blockIdx.x == gridDim.x - 1) {  // the objective: one block, a fixed summation order
        __shared__ double part[256];
        double t = 0.0;
        for (int e = threadIdx.x; e < E; e += blockDim.x) t += ldexp((double)(long long)acc[e], -q);
        part[threadIdx.x] = t;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) *objective = part[0] / dn;
    }
}

template <bool WIN_SMEM>
static void (*forward_kernel(const KArgs &a))(const KArgs) {
    if (a.tables_in_smem)
        return a.positive ? k_adjoint_forward<WIN_SMEM, true, kTablesSmem> : k_adjoint_forward<WIN_SMEM, false, kTablesSmem>;
    return a.positive ? k_adjoint_forward<WIN_SMEM, true, kTablesGlobal> : k_adjoint_forward<WIN_SMEM, false, kTablesGlobal>;
}

// The forward half over stages [a.stage_begin, a.stage_end).
cudaError_t launch_adjoint_forward(const KArgs &a, cudaStream_t st) {
    if (a.n <= 0) return cudaSuccess;
    const dim3 grid((unsigned)((a.n + kTile - 1) / kTile)), block((unsigned)(a.n_warps * 32));
    const size_t smem = (size_t)a.smem_total;
    void (*fwd)(const KArgs) = a.win_smem ? forward_kernel<true>(a) : forward_kernel<false>(a);
    cudaError_t e = raise_smem_limit((const void *)fwd, smem);
    if (e != cudaSuccess) return e;
    fwd<<<grid, block, smem, st>>>(a);
    return cudaGetLastError();
}

// The backward half over stages [a.stage_begin, a.stage_end), last stage first.
cudaError_t launch_adjoint_backward(const KArgs &a, cudaStream_t st) {
    if (a.n <= 0) return cudaSuccess;
    const dim3 grid((unsigned)((a.n + kTile - 1) / kTile)), block((unsigned)(a.n_warps * 32));
    const size_t smem = (size_t)a.smem_total;
    void (*bwd)(const KArgs) = a.win_smem ? k_adjoint<true> : k_adjoint<false>;
    cudaError_t e = raise_smem_limit((const void *)bwd, smem);
    if (e != cudaSuccess) return e;
    bwd<<<grid, block, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_finish(const long long *grad_e, const long long *grad_l, const unsigned long long *acc,
                                  int32_t E, int32_t L, int64_t n, int32_t q, double *g_earliest, double *g_base,
                                  double *objective, cudaStream_t st) {
    const int m = E > L ? E : L;
    k_adjoint_finish<<<(unsigned)((m + 255) / 256 + 1), 256, 0, st>>>(grad_e, grad_l, acc, E, L, n, q, g_earliest,
                                                                       g_base, objective);
    return cudaGetLastError();
}

}  // namespace mcd
