"""GPU parity at the sizes the benchmark configurations state.

1. The 1,000-event configuration over all 10,000 seeds (0..9999): the CUDA
   propagation of the oracle's durations reproduces the oracle's realized and
   cause_event bit for bit, and -- when this host's libm reproduces the
   reference's durations (digests in golden/config0_hashes_ref.npz, made by the
   reference itself) -- the reference's own rows as well.
2. The benchmark's exact single-large-DAG workload (200,000 events, 499,128
   links, 1,434 levels, window on chip): bit-exact through the given-durations
   path (host and device entry points) and through the sampled path
   (GPU durations -> the oracle's propagation), on 70 and 96 samples.
3. Sampled runs at 10^6 samples per event against the oracle's run_many on the
   1,000-event DAG and on a five-kind DAG of the same shape: two-sample KS at
   alpha = 0.01 and means within 3 standard errors per event, each with a
   one-sided binomial test on the number of events that reject (the events are
   tested on shared samples, so the count is a global check, not independent
   trials); and the fused statistics path's p50/p90/p99 against the oracle's
   empirical quantiles within one histogram bin plus 5 sampling standard errors.

Reference: src/mc_dagprop/monte_carlo/_core.cpp:312-361 (run / run_many).
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np
import pytest

import mc_dagprop_gb300 as m
import oracle
from mc_dagprop_gb300 import replicas
from mc_dagprop_gb300 import workloads as W
from mcd_testlib import MCD_OK, block_digests, last_error, lib, propagator_from_flat

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
GOLDEN_HASHES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "config0_hashes_ref.npz")


def _bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.int64)


def _assert_bits_equal(a, b, what):
    bad = np.argwhere(_bits(a) != _bits(b))
    assert len(bad) == 0, f"{what}: {len(bad)} mismatches, first {bad[:3].tolist()}"


@pytest.mark.parametrize("window", ["smem", "global"])
def test_config0_all_10000_seeds_bitexact(cuda, window, monkeypatch):
    if window == "global":
        monkeypatch.setenv("MCD_NO_SMEM_WINDOW", "1")
    flat, gen = W.config0()
    z = np.load(GOLDEN_HASHES)
    seeds = z["seeds"]
    assert len(seeds) == 10_000 and seeds[0] == 0 and seeds[-1] == 9999
    real_o, dur_o, cause_o = oracle.OracleSim(flat, gen).run_many(seeds, threads=THREADS)
    prop = propagator_from_flat(m, flat, gen)
    assert prop.info()["window_in_smem"] == (window == "smem")
    real, cause = prop.propagate(dur_o)
    _assert_bits_equal(real, real_o, "realized")
    assert np.array_equal(cause, cause_o)
    blk = int(z["block"])
    if np.array_equal(block_digests(dur_o, blk), z["durations"]):
        # this host's durations are the reference's: the GPU rows are the reference's rows
        assert np.array_equal(block_digests(real, blk), z["realized"])
        assert np.array_equal(block_digests(cause, blk), z["cause"])
    else:  # another libm rounds log differently in the last place: the oracle chain above stands
        assert not np.array_equal(block_digests(dur_o, blk), z["durations"])


@pytest.fixture(scope="module")
def bench_dag():
    """The benchmark's single-large-DAG workload, exactly as bench.py builds it."""
    flat, gen = W.config1(seed=1, n_layers=2000, width=100)
    prop = propagator_from_flat(m, flat, gen)
    info = prop.info()
    assert (info["n_events"], info["n_links"], info["n_levels"]) == (200_000, 499_128, 1434)
    assert info["window_in_smem"] and info["n_warps"] == 24
    return flat, gen, prop, oracle.OracleSim(flat, gen)


def test_bench_dag_given_durations_host_and_device(cuda, bench_dag):
    import torch

    flat, gen, prop, sim = bench_dag
    seeds = np.arange(96, dtype=np.int64) + 5_000_000
    real_o, dur_o, cause_o = sim.run_many(seeds, threads=THREADS)
    real, cause = prop.propagate(dur_o)  # host entry point (sample-major)
    _assert_bits_equal(real, real_o, "realized (host path)")
    assert np.array_equal(cause, cause_o)
    # device entry point, sample-minor rows with a padded leading dimension
    E, L, n, ld = prop.node_count(), prop.activity_count(), len(seeds), 128
    dur_d = torch.zeros((L, ld), dtype=torch.float64, device=cuda)
    dur_d[:, :n] = torch.from_numpy(np.ascontiguousarray(dur_o.T)).to(cuda)
    real_d = torch.full((E, ld), -7.0, dtype=torch.float64, device=cuda)
    cause_d = torch.full((E, ld), -7, dtype=torch.int32, device=cuda)
    torch.cuda.synchronize()  # the C ABI runs on the handle's own stream
    h = C.c_void_p(prop._handle())
    assert lib().mcd_propagate_device(h, dur_d.data_ptr(), ld, n, real_d.data_ptr(), cause_d.data_ptr(), ld,
                                      None) == MCD_OK, last_error()
    assert lib().mcd_dag_check(h) == MCD_OK, last_error()
    _assert_bits_equal(real_d[:, :n].T.cpu().numpy(), real_o, "realized (device path)")
    assert np.array_equal(cause_d[:, :n].T.cpu().numpy(), cause_o)
    assert (real_d[:, n:] == -7.0).all() and (cause_d[:, n:] == -7).all()


@pytest.mark.parametrize("n", [70, 96])
def test_bench_dag_sampled_is_oracle_propagation(cuda, bench_dag, n):
    """The sampled path exactly as the benchmark launches it (device entry point,
    sample-minor rows, the benchmark's seeds): realized and cause_event are the
    oracle's propagation of the GPU's own durations."""
    import torch

    flat, gen, prop, sim = bench_dag
    E, L, ld = prop.node_count(), prop.activity_count(), 128
    seeds = replicas.seed_range(0, 1, 19_456)[-n:]  # the last samples of the benchmark's step
    seeds_d = torch.from_numpy(np.ascontiguousarray(seeds, np.int64)).to(cuda)
    real_d = torch.empty((E, ld), dtype=torch.float64, device=cuda)
    dur_d = torch.empty((L, ld), dtype=torch.float64, device=cuda)
    cause_d = torch.empty((E, ld), dtype=torch.int32, device=cuda)
    torch.cuda.synchronize()  # the C ABI runs on the handle's own stream
    h = C.c_void_p(prop._handle())
    assert lib().mcd_run_device(h, seeds_d.data_ptr(), n, real_d.data_ptr(), dur_d.data_ptr(), cause_d.data_ptr(),
                                ld, None) == MCD_OK, last_error()
    assert lib().mcd_dag_check(h) == MCD_OK, last_error()
    dur = np.ascontiguousarray(dur_d[:, :n].T.cpu().numpy())
    real_o, cause_o = sim.propagate_given(dur)
    _assert_bits_equal(real_d[:, :n].T.cpu().numpy(), real_o, "realized")
    assert np.array_equal(cause_d[:, :n].T.cpu().numpy(), cause_o)
    # and the host entry point returns the same samples
    r2, d2, c2 = prop.run_many_arrays(np.ascontiguousarray(seeds, np.int64))
    _assert_bits_equal(d2, dur, "durations (host path)")
    _assert_bits_equal(r2, real_o, "realized (host path)")
    assert np.array_equal(c2, cause_o)


# ---------------------------------------------------------------- 10^6 samples

N_SAMPLES = 1_000_000


def _five_kind_config0_shape():
    flat = W.layered_dag(31, 50, 20, 3, [1, 2, 3, 4, 5], 1800.0)
    return flat, W.gen_five_types(np.random.default_rng(31))


def _oracle_realized_on_device(flat, gen, n, cuda, chunk=100_000):
    """The oracle's realized times for seeds 0..n-1 as an (E, n) device tensor."""
    import torch

    sim = oracle.OracleSim(flat, gen)
    out = torch.empty((sim.node_count(), n), dtype=torch.float64, device=cuda)
    for off in range(0, n, chunk):
        k = min(chunk, n - off)
        real, _, _ = sim.run_many(np.arange(off, off + k), threads=THREADS, want=("realized",))
        out[:, off:off + k] = torch.from_numpy(real).to(cuda).T
    return out


def _gpu_realized(prop, n, seed_offset, cuda):
    import torch

    E = prop.node_count()
    seeds = torch.arange(seed_offset, seed_offset + n, dtype=torch.int64, device=cuda)
    real = torch.empty((E, n), dtype=torch.float64, device=cuda)
    torch.cuda.synchronize()  # the seeds come from torch's stream; the C ABI runs on the handle's
    h = C.c_void_p(prop._handle())
    assert lib().mcd_run_device(h, seeds.data_ptr(), n, real.data_ptr(), None, None, n, None) == MCD_OK, \
        last_error()
    assert lib().mcd_dag_check(h) == MCD_OK, last_error()
    return real


def _ks_statistics(a, b, chunk=32):
    """Two-sample KS statistic per row of two row-sorted device tensors: the
    largest gap between the two right-continuous empirical CDFs, taken at every
    sample point of both rows (ties and atoms included)."""
    import torch

    n, mm = a.shape[1], b.shape[1]
    D = torch.empty(a.shape[0], dtype=torch.float64, device=a.device)
    for i in range(0, a.shape[0], chunk):
        aa, bb = a[i:i + chunk].contiguous(), b[i:i + chunk].contiguous()
        d1 = (torch.searchsorted(aa, aa, right=True).double() / n
              - torch.searchsorted(bb, aa, right=True).double() / mm).abs().amax(dim=1)
        d2 = (torch.searchsorted(aa, bb, right=True).double() / n
              - torch.searchsorted(bb, bb, right=True).double() / mm).abs().amax(dim=1)
        D[i:i + chunk] = torch.maximum(d1, d2)
    return D


@pytest.mark.parametrize("cfg", ["config0", "five_kinds"])
def test_distributions_at_1e6_samples_match_oracle(cuda, cfg):
    import torch
    from scipy import special, stats

    flat, gen = W.config0() if cfg == "config0" else _five_kind_config0_shape()
    prop = propagator_from_flat(m, flat, gen)
    g = _gpu_realized(prop, N_SAMPLES, 10**12, cuda)  # independent of the oracle's stream by construction
    o = _oracle_realized_on_device(flat, gen, N_SAMPLES, cuda)
    degenerate = ((g.amin(1) == g.amax(1)) & (o.amin(1) == o.amax(1))).cpu().numpy()
    # events that never move (no predecessors) must agree exactly
    assert torch.equal(g[torch.from_numpy(degenerate).to(cuda), 0], o[torch.from_numpy(degenerate).to(cuda), 0])
    live = ~degenerate
    n_live = int(live.sum())
    assert n_live >= 100  # events whose time varies between samples (the rest are fixed by their fixed-delay paths)

    # means within 3 standard errors
    mg, mo = g.mean(1), o.mean(1)
    se = torch.sqrt(g.var(1) / N_SAMPLES + o.var(1) / N_SAMPLES)
    z = ((mg - mo).abs() / se.clamp_min(1e-300)).cpu().numpy()[live]
    mean_out = int((z > 3.0).sum())

    # two-sample KS at alpha = 0.01 (asymptotic Kolmogorov law, exact enough at 10^6)
    gs, _ = torch.sort(g, dim=1)
    del g
    os_, _ = torch.sort(o, dim=1)
    del o
    D = _ks_statistics(gs, os_).cpu().numpy()
    lam = D * math.sqrt(N_SAMPLES * N_SAMPLES / (2.0 * N_SAMPLES))
    pvals = special.kolmogorov(lam)[live]
    ks_reject = int((pvals < 0.01).sum())

    # global checks on the counts (one-sided: too many rejections)
    p_ks = stats.binomtest(ks_reject, n_live, 0.01, alternative="greater").pvalue
    p_mean = stats.binomtest(mean_out, n_live, 0.0027, alternative="greater").pvalue
    msg = (f"{cfg}: {ks_reject}/{n_live} KS rejections (binomial p {p_ks:.3g}), {mean_out} means beyond 3 SE "
           f"(binomial p {p_mean:.3g}), max D {D[live].max():.4g}, min KS p {pvals.min():.3g}")
    print(msg)
    assert p_ks > 1e-3, msg
    assert p_mean > 1e-3, msg

    # the fused statistics path's quantiles against the oracle's empirical CDF
    st = prop.run_stats(n=N_SAMPLES, seed0=10**12)
    w = float(st["bin_width"])
    for key, p in (("p50", 0.5), ("p90", 0.9), ("p99", 0.99)):
        q = torch.from_numpy(np.ascontiguousarray(st[key])).to(cuda)[:, None]
        eps = 5.0 * math.sqrt(2.0 * p * (1.0 - p) / N_SAMPLES) + 2.0 / N_SAMPLES
        # fraction of the oracle's samples <= q + w, and < q - w
        upper = torch.searchsorted(os_, (q + w).contiguous(), right=True).double().squeeze(1) / N_SAMPLES
        lower = torch.searchsorted(os_, (q - w).contiguous(), right=False).double().squeeze(1) / N_SAMPLES
        ok = ((upper >= p - eps) & (lower <= p + eps)).cpu().numpy()
        assert ok.all(), (key, np.flatnonzero(~ok)[:5].tolist())
