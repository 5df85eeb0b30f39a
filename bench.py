"""Benchmark of the plain Monte Carlo path: run_many over one large DAG.

Workload (one "step"): the single-large-DAG configuration -- 200,000 events in
2,000 layers of 100, ~500,000 links, five activity types, max_delay 3,600 s --
for one chunk of `--samples` samples (default 19,456 = 4 waves of 152 SMs x 32
samples) with full outputs (realized, durations, cause_event) resident in HBM.
The configuration's 65,536-sample chunks would need 419 GB of outputs, more
than HBM holds, so a step is the largest chunk that keeps all outputs resident
with room to spare (125 GB).  A step is one launch of the fused
sampler+propagation kernel; its outputs are far larger than L2, so no flush is
needed between steps.

Printed (one JSON line, rank 0):
  value      sample-edges/s with inputs resident in HBM (device-timed, CUDA events
             on the launching stream, max over ranks)
  e2e        the same metric through the C ABI with pinned HOST buffers
             (mcd_run_many_host: seeds in, realized/durations/cause_event out, sample-major)
  roofline   algorithmic bytes of the kernel / its event-timed duration vs measured HBM peak
  cpu_baseline  the oracle (C restatement of the reference) on all host cores
  clocks     nvidia-smi samples taken during the timed region

    python bench.py [--gpus N] [--steps K] [--warmup W] [--samples S] [--impl reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "single large DAG: 200,000 events (2,000 layers x 100), 1-4 preds from the previous 1-5 layers, " \
           "5 activity types, max_delay 3600 s; one chunk of samples per step, full outputs"
METRIC = "sample-edges/s"


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, path):
        self.path = path
        self.proc = None

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self, device_index=0):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9 or parts[0] != str(device_index):
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def build_dag(n_layers=2000, width=100):
    from mc_dagprop_gb300 import workloads as W

    return W.config1(seed=1, n_layers=n_layers, width=width)


def make_propagator(flat, gen):
    import mc_dagprop_gb300 as m
    from mc_dagprop_gb300 import workloads as W

    return m.MonteCarloPropagator.from_arrays(
        flat["earliest"], flat["act_idx"], flat["act_duration"], flat["act_type"], flat["target"],
        flat["pred_offsets"], flat["pred_src"], flat["pred_act"], flat["max_delay"], W.to_generator(m, gen))


def _capi():
    lib = C.CDLL(os.path.join(ROOT, "mc_dagprop_gb300", "_lib", "libmcdagprop_gb300.so"))
    P, I64 = C.c_void_p, C.c_int64
    lib.mcd_run_device.argtypes = [P, P, I64, P, P, P, I64, P]
    lib.mcd_run_many_host.argtypes = [P, P, I64, P, P, P]
    lib.mcd_dag_check.argtypes = [P]
    lib.mcd_host_alloc.argtypes = [C.c_size_t, C.POINTER(P)]
    lib.mcd_host_free.argtypes = [P]
    lib.mcd_last_error.restype = C.c_char_p
    return lib


def cpu_baseline(flat, gen, seconds=10.0, kind="port"):
    """The reference's algorithm on all host cores: one simulator per thread,
    contiguous seed chunks (the reference's multithreading pattern), full outputs
    into a reused buffer; repeated until `seconds` have passed."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    threads = os.cpu_count() or 1
    sim = oracle.OracleSim(flat, gen)
    per_call = 8 * threads
    L = sim.activity_count()
    done = 0
    t0 = time.perf_counter()
    while True:
        seeds = np.arange(done, done + per_call, dtype=np.int64)
        sim.run_many(seeds, threads=threads)
        done += per_call
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": done * L / dt, "unit": METRIC, "cores": threads, "kind": kind,
            "sample": f"{done} samples of the same DAG ({done * L:.3g} sample-edges) in {dt:.1f} s, "
                      f"calls of {per_call} samples, full outputs"}


def run_reference_arm(args):
    rank, world, _ = _dist_env()
    if rank != 0:
        return 0
    flat, gen = build_dag()
    per_step_seconds = float(os.environ.get("MCD_REF_STEP_SECONDS", "5"))
    for _ in range(args.warmup):
        cpu_baseline(flat, gen, seconds=min(1.0, per_step_seconds))
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline(flat, gen, seconds=per_step_seconds))
    dt = time.perf_counter() - t0
    v = float(np.mean([x["value"] for x in vals]))
    cb = dict(vals[-1])
    cb["value"] = v
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "events": len(flat["earliest"]), "links": int(flat["act_idx"].max()) + 1,
                   "implementation": "C restatement of the reference's run_many (oracle/mcd_oracle.c), "
                                     "one simulator per host thread"},
        "cpu_baseline": cb,
        "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))
    return 0


class _Stats(C.Structure):
    _fields_ = [("mean", C.c_void_p), ("p50", C.c_void_p), ("p90", C.c_void_p), ("p99", C.c_void_p),
                ("p_on_time", C.c_void_p), ("hist", C.c_void_p)]


def run_batched(args):
    """Batching workload: 512 DAGs (events log-uniform 100-50,000, layer width
    20-200, two delay kinds), each with its own sample count (log-uniform
    1,000-100,000) and seed range; per-event mean and p50/p90/p99 from 256-bin
    histograms.  The batched form (one persistent launch per step, CUDA graph,
    warps per CTA from the autotuner) against the plain form (one
    mcd_stats_device call per DAG, the same statistics) on the same GPU."""
    import torch

    from mc_dagprop_gb300 import batching
    from mc_dagprop_gb300 import workloads as W

    t0 = time.perf_counter()
    dags = W.config2(n_dags=args.dags)
    gen_s = time.perf_counter() - t0
    flats = [d[0] for d in dags]
    gens = [d[1] for d in dags]
    ns = [int(d[2]) for d in dags]
    seed0 = [int(d[3]) for d in dags]
    units = sum(int(f["act_idx"].max() + 1) * n for f, n in zip(flats, ns))
    t0 = time.perf_counter()
    nw = batching.tune_warps(flats, gens, ns, use_cache=False)
    tune_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    props = [batching.compile_dag(f, g, nw) for f, g in zip(flats, gens)]
    compile_s = time.perf_counter() - t0
    lib = _capi()
    lib.mcd_stats_device.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.POINTER(_Stats), C.c_void_p]
    dev = torch.device("cuda", 0)
    outs = []
    for p in props:
        t = torch.empty((5, p.node_count()), dtype=torch.float64, device=dev)
        outs.append((t, _Stats(*(t[k].data_ptr() for k in range(5)), None)))
    stream = torch.cuda.Stream(device=dev)

    def plain_run():
        for i, (p, (t, st)) in enumerate(zip(props, outs)):
            if lib.mcd_stats_device(C.c_void_p(p._handle()), None, seed0[i], ns[i], C.byref(st),
                                    C.c_void_p(stream.cuda_stream)) != 0:
                raise RuntimeError(lib.mcd_last_error().decode())

    def timed(fn, st, reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(st)
        for _ in range(reps):
            fn()
        b.record(st)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    plain_run()  # workspaces allocated here
    torch.cuda.synchronize()
    plain_ms = timed(plain_run, stream, args.steps)
    batch = __import__("mc_dagprop_gb300").Batch(props, seed0, ns)
    bstream = torch.cuda.ExternalStream(batch.stream, device=dev)
    for _ in range(max(1, args.warmup)):
        batch.run(wait=True)
    batch_ms = timed(lambda: batch.run(wait=False), bstream, args.steps)
    batch.sync()
    # the batch's statistics equal the plain path's, DAG by DAG
    mism = 0
    for i in range(0, len(props), max(1, len(props) // 16)):
        got = batch.stats(i)
        ref = outs[i][0].cpu().numpy()
        mism += int(not np.array_equal(got["mean"], ref[0]) or not np.array_equal(got["p99"], ref[3]))
    print(json.dumps({
        "metric": "sample-edges/s (batched statistics)", "value": units / (batch_ms * 1e-3), "unit": METRIC,
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": batch_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "512 DAGs, events log-uniform 100-50,000 (width 20-200), samples log-uniform "
                               "1,000-100,000, own seed ranges; per-event mean, p50/p90/p99 (256-bin histograms)",
                   "dags": len(props), "events_total": int(sum(len(f["earliest"]) for f in flats)),
                   "sample_edges_per_step": units, "n_warps": nw, "work_items": batch.items, "grid": batch.grid},
        "plain": {"value": units / (plain_ms * 1e-3), "ms_per_step": plain_ms,
                  "path": "one mcd_stats_device call per DAG on one stream"},
        "batched_over_plain": plain_ms / batch_ms, "check_mismatches": mism,
        "host_seconds": {"generate": gen_s, "autotune": tune_s, "compile_512": compile_s},
    }))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--samples", type=int, default=19456)
    ap.add_argument("--e2e-samples", type=int, default=512)
    ap.add_argument("--layers", type=int, default=2000)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--workload", default="single", choices=["single", "batched"])
    ap.add_argument("--dags", type=int, default=512)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.workload == "batched":
        return run_batched(args)

    import torch

    rank, world, local = _dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    flat, gen = build_dag(n_layers=args.layers)
    prop = make_propagator(flat, gen)
    info = prop.info()
    E, L = prop.node_count(), prop.activity_count()
    S = args.samples
    lib = _capi()
    h = C.c_void_p(prop._handle())
    dev = torch.device("cuda", local)
    # per-rank disjoint seed ranges (weak scaling: every rank runs its own samples)
    seeds = torch.arange(rank * S, (rank + 1) * S, dtype=torch.int64, device=dev)
    ld = S
    real = torch.empty((E, ld), dtype=torch.float64, device=dev)
    durs = torch.empty((L, ld), dtype=torch.float64, device=dev)
    cause = torch.empty((E, ld), dtype=torch.int32, device=dev)
    # Launch on the handle's own stream and time with events recorded on that
    # same stream (torch's default stream handle is 0, which the C ABI reads as
    # "the handle's stream", so wrap the handle's stream explicitly).
    lib.mcd_dag_stream.argtypes = [C.c_void_p]
    lib.mcd_dag_stream.restype = C.c_void_p
    stream = torch.cuda.ExternalStream(lib.mcd_dag_stream(h), device=dev)

    def step():
        rc = lib.mcd_run_device(h, seeds.data_ptr(), S, real.data_ptr(), durs.data_ptr(), cause.data_ptr(), ld,
                                C.c_void_p(stream.cuda_stream))
        if rc != 0:
            raise RuntimeError(lib.mcd_last_error().decode())

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    if lib.mcd_dag_check(h) != 0:
        raise RuntimeError(lib.mcd_last_error().decode())

    clocks = Clocks(os.path.join(ROOT, "gpurun_out", f"clocks_rank{rank}.csv")
                    if os.path.isdir(os.path.join(ROOT, "gpurun_out")) else f"/tmp/mcd_clocks_{rank}.csv")
    if rank == 0:
        clocks.start()
        time.sleep(0.4)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for a, b in evs:
        a.record(stream)
        step()
        b.record(stream)
    t_end.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ck = clocks.stop(local) if rank == 0 else None
    if lib.mcd_dag_check(h) != 0:
        raise RuntimeError(lib.mcd_last_error().decode())
    total_ms = t_start.elapsed_time(t_end)
    kernel_ms = [a.elapsed_time(b) for a, b in evs]
    if dist:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    units_per_step = S * L
    value = units_per_step * world * args.steps / (total_ms * 1e-3)

    # roofline of the dominant kernel (the only launch of a step)
    out_bytes = S * (8 * L + 8 * E + 4 * E)
    alg_bytes = out_bytes + info["device_bytes"]
    avg_kernel_s = float(np.mean(kernel_ms)) * 1e-3
    achieved = alg_bytes / avg_kernel_s / 1e9
    peak, peak_kind = _peaks()
    traffic = None
    tf = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tf):  # one ncu capture of a smaller case, scaled by samples x links
        with open(tf) as f:
            traffic = json.load(f)["dram_bytes_per_sample_edge"] * S * L

    # e2e through the C ABI with pinned host buffers
    e2e = None
    if rank == 0:
        n2 = args.e2e_samples
        bufs = []
        for nbytes in (n2 * 8, n2 * E * 8, n2 * L * 8, n2 * E * 4):
            p = C.c_void_p()
            if lib.mcd_host_alloc(nbytes, C.byref(p)) != 0:
                raise RuntimeError(lib.mcd_last_error().decode())
            bufs.append(p)
        sv = np.frombuffer((C.c_int64 * n2).from_address(bufs[0].value), dtype=np.int64)
        sv[:] = np.arange(10**9, 10**9 + n2)

        def e2e_step():
            rc = lib.mcd_run_many_host(h, bufs[0], n2, bufs[1], bufs[2], bufs[3])
            if rc != 0:
                raise RuntimeError(lib.mcd_last_error().decode())

        e2e_step()
        reps = 3
        t0 = time.perf_counter()
        for _ in range(reps):
            e2e_step()
        dt = (time.perf_counter() - t0) / reps
        e2e = {"value": n2 * L / dt, "unit": METRIC, "h2d_bytes_per_step": n2 * 8,
               "d2h_bytes_per_step": n2 * (8 * E + 8 * L + 4 * E), "samples_per_step": n2,
               "ms_per_step": dt * 1e3, "path": "mcd_run_many_host, pinned host buffers, sample-major outputs"}
        for p in bufs:
            lib.mcd_host_free(p)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(flat, gen, seconds=float(os.environ.get("MCD_CPU_SECONDS", "10")))

    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "events": E, "links": L, "preds": info["n_preds"],
                       "levels": info["n_levels"], "samples_per_step": S, "samples_total": S * args.steps * world,
                       "outputs": "realized (E,S) f64 + durations (L,S) f64 + cause_event (E,S) i32, sample-minor",
                       "l2": f"outputs {out_bytes / 1e9:.1f} GB per step >> 129 MB L2, no flush needed; "
                             f"compiled DAG ({info['device_bytes'] / 1e6:.1f} MB) stays L2-resident by design",
                       "window_slots": info["window_slots"], "window_in_smem": info["window_in_smem"],
                       "warps_per_cta": info["n_warps"], "parallelism": f"replicas x{world}, disjoint seeds"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "kernel": "k_propagate<false,true> (fused Philox sampler + FP64 propagation)",
                         "kernel_ms": float(np.mean(kernel_ms))},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": args.steps, "clocks": ck,
        }))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
