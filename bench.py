"""Benchmark: NEE path-contributions/s of the 3D temporal-correlation workload.

Workload (one step = one render): the 3D correlation scene -- slab
[-100,100]^2 x [0,20], sigs=[0,0.5], siga=[0,0.01], HG g=0.9, 64 point
illuminations at z=-5 and 64 point views at z=25 on jittered 8x8 lattices,
Brownian D=[0,1e-3], 8 lags -- with 2^22 paths (4 waves of 2^20), seeded
synthetic inputs.  One contribution is one (path, scattering vertex,
illumination, view, lag) term of the estimator.

value : contributions / device time of the render (CUDA events on the
        library's stream; scene tables resident in HBM).
e2e   : the same metric through the public C-ABI call a MATLAB-style user
        makes -- scene creation (host -> device upload of the config tables),
        render, read-back of u and iter, scene destruction -- timed on the host.
--impl reference: the reference has no CPU implementation and its CUDA
        sources do not exist on the GPU host, so the reference arm times the
        CPU FP64 restatement of its estimator (oracle/) on all host threads.

Multi-GPU (torchrun): independent replicas with disjoint seeds ("replicas
only": the paths are i.i.d., there is no exchange step); value is the sum of
contributions over ranks divided by the max time over ranks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "NEE path-contributions/s at <=1e-5 err vs FP64 (vs plain FP32); p50/p99 latency"
UNIT = "contributions/s"
WORKLOAD = "correlation_3d"   # the headline; --workload speckle_2d measures the 2D far-field speckle field
WORKLOADS = ("correlation_3d", "speckle_2d")


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl"
        try:
            import torch
            if not torch.cuda.is_available():
                backend = "gloo"
            else:
                torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
        return dist, rank, ws
    return None, 0, 1


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _sum_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def _workload(seed: int, paths_log2: int):
    from temporalspecklescode_gb300 import workloads as wl
    waves = max(1, 1 << max(0, paths_log2 - 20))
    batch = (1 << paths_log2) // waves
    if WORKLOAD == "speckle_2d":   # 16 x 16 far-field field speckle, one tick
        return wl.speckle_2d(batch_size=batch, full_iteration=waves, seed=seed)
    cfg, dims = wl.correlation_3d(batch_size=batch, full_iteration=waves, seed=seed)
    return cfg, dims


def cpu_baseline(sample_paths: int, threads: int):
    """Time the CPU oracle (FP64 restatement, OpenMP) on a bounded sample."""
    from temporalspecklescode_gb300 import config as cf
    from tests.oracle_lib import Oracle
    cfg, dims = _workload(0, 20)
    cfg["simulation"]["batchSize"] = sample_paths
    cfg["simulation"]["fullIteration"] = 1
    pc = cf.prepare(cfg, dims)
    oracle = Oracle()
    t0 = time.perf_counter()
    _, _, st = oracle.render(pc, 0, threads=threads)
    dt = time.perf_counter() - t0
    return st["contributions"] / dt, st, dt


def run_reference(args, dist, rank, ws):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    sample = args.ref_sample
    times = []
    contrib = 0
    for i in range(args.warmup + args.steps):
        v, st, dt = cpu_baseline(sample, threads)
        if i >= args.warmup:
            times.append(dt)
            contrib = st["contributions"]
    ms = 1000 * statistics.mean(times)
    value = contrib / (ms / 1000)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "paths_per_step": sample, "note": "CPU FP64 restatement of the reference estimator"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{sample} paths of the {WORKLOAD} workload per step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# DRAM bytes (read + write) per path of each kernel class from one ncu capture
# of this workload at 2^16 paths (profiles/kernels_correlation_3d_2p16.md);
# every class streams per-path rows, so a launch's traffic scales with the
# paths it processes.
NCU_DRAM_BYTES_PER_PATH = {
    "nee": (8354816 + 156937728 + 14934272 + 75123456) / 65536,   # illum_kernel + view_kernel
    "walk": (242688 + 176896 + 18749184 + 1536) / 65536,          # walk_kernel<slots> + compact_kernel
    "gemm": (269205504 + 3310592) / 65536,                         # gemm_tc_kernel (real rows)
    "ss": (68522752 + 932352) / 65536,                             # ss_fast_kernel
}


def _kernel_rooflines(scene, mean, verts_per_step, chunks, peaks):
    """Per kernel class: time per step, algorithmic bytes or flops per launch,
    achieved rate and the fraction of the measured peak."""
    m = scene.meta
    P = m["P"] * m["waves"]
    Nl, Nv, Nt = m["Nl"], m["Nv"], m["Nt"]
    hbm, tc = peaks["hbm_gbs"], peaks["bf16_tflops"]
    out = {}

    def add(key, name, ms, bound, amount, note):
        per_launch = amount / chunks
        traffic = NCU_DRAM_BYTES_PER_PATH[key] * P / chunks if WORKLOAD == "correlation_3d" else None
        if bound == "hbm":
            ach = amount / (ms / 1000) / 1e9
            out[key] = {"kernel": name, "ms": ms, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                        "frac": ach / hbm, "peak_name": "hbm_gbs", "algorithmic_per_launch": per_launch,
                        "traffic": traffic, "note": note}
        else:
            ach = amount / (ms / 1000) / 1e12
            out[key] = {"kernel": name, "ms": ms, "bound": "tensor", "achieved": ach, "peak": tc, "unit": "TFLOP/s",
                        "frac": ach / tc, "peak_name": "bf16_tflops", "algorithmic_per_launch": per_launch,
                        "traffic": traffic, "note": note}

    # NEE vectors (illum_kernel + view_kernel): rows written once (a_ms all ticks,
    # tick-invariant single-scattering rows at tick 0, s_ms), P_l, the vertices read.
    # The correlation sampler's rows are real here: 4 bytes per (tick, element).
    rb = 4.0 if m["correlation"] else 8.0
    nee_bytes = P * (rb * Nt * Nl + 8.0 * (Nl + Nv) + rb * Nt * Nv + 4 * Nl + 13 + 12) + 16.0 * verts_per_step
    add("nee", "illum_kernel + view_kernel (NEE vectors)", mean["ms_nee"], "hbm", nee_bytes,
        "FP32-issue bound: DRAM traffic equals the row bytes")
    # random walk: one pass into per-path slots + compaction; vertices written once, counts / misses / offsets
    add("walk", "walk_kernel (single-pass random walk) + compaction", mean["ms_walk"], "hbm", 16.0 * verts_per_step + 20.0 * P,
        "FP32-issue bound (IEEE-rounded decision path)")
    # multiple-scattering contraction: HBM-bound at this shape (M = N = 128 per tick
    # pair, 2 Nl Nv Nt flops per path against rb Nt (Nl + Nv) bytes read)
    add("gemm", "gemm_tc_kernel (multiple-scattering contraction, 3xTF32)", mean["ms_contract_ms"], "hbm",
        rb * Nt * (Nl + Nv) * P, "reads the a_ms and s_ms rows once; tensor pipe 23 % active (ncu)")
    # single-scattering contraction: tick-0 rows read (tick-invariant form)
    add("ss", "ss_fast_kernel (single-scattering contraction)", mean["ms_contract_ss"], "hbm", P * 8.0 * (Nl + Nv),
        "FP32/SFU-issue bound: one exp and one rsqrt per (path, l, v)")
    return out


def run_gpu(args, dist, rank, ws):
    import numpy as np
    from temporalspecklescode_gb300 import api, config as cf
    api.load_library()
    precision = cf.PRECISION_FP32 if args.precision == "fp32" else cf.PRECISION_SPLIT
    cfg, dims = _workload(seed=1000 * rank, paths_log2=args.paths_log2)
    scene = api.Scene(cfg, dims, precision)
    lat = []
    dev_ms = []
    parts = {"ms_trace": [], "ms_contract_ms": [], "ms_contract_ss": [], "ms_walk": [], "ms_nee": []}
    chunks = 1
    verts = 0
    contrib = 0
    launches = 0
    for i in range(args.warmup):
        scene.render(seed=i)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    _barrier(dist)
    clocks.start()
    t0 = time.perf_counter()
    for i in range(args.steps):
        ts = time.perf_counter()
        u, it = scene.render(seed=100 + i)
        lat.append(1000 * (time.perf_counter() - ts))
        tm = scene.timing()
        dev_ms.append(tm["ms_total"])
        for k in parts:
            parts[k].append(tm[k])
        launches += tm["launches"]
        chunks = tm["chunks"]
        st = scene.stats()
        contrib += st["contributions"]
        verts += st["vertices"]
    wall = time.perf_counter() - t0
    _barrier(dist)
    clk = clocks.stop()
    dev_total_s = sum(dev_ms) / 1000.0
    dev_total_s = _max_over_ranks(dist, dev_total_s)
    contrib_all = _sum_over_ranks(dist, float(contrib))
    value = contrib_all / dev_total_s

    # end to end through the C-ABI: create (upload) + render + read back + destroy
    e2e_t = []
    h2d = 0
    # one untimed call first: the first scene created next to the resident one
    # grows the stream-ordered memory pool
    with api.Scene(cfg, dims, precision) as s2:
        s2.render(seed=199)
    for i in range(max(1, min(3, args.steps))):
        ts = time.perf_counter()
        with api.Scene(cfg, dims, precision) as s2:
            u2, it2 = s2.render(seed=200 + i)
        e2e_t.append(time.perf_counter() - ts)
    pc = scene.prepared
    for a in pc._keep:
        h2d += a.nbytes
    d2h = u.size * 16 + it.size * 8
    e2e_s = _max_over_ranks(dist, statistics.mean(e2e_t))
    e2e_value = _sum_over_ranks(dist, float(contrib / args.steps)) / e2e_s

    peaks, pk_kind = _peaks()
    m = scene.meta
    P = m["P"] * m["waves"]
    Nl, Nv, Nt = m["Nl"], m["Nv"], m["Nt"]
    mean = {k: statistics.mean(v) for k, v in parts.items()}
    kernels = _kernel_rooflines(scene, mean, verts / args.steps, chunks, peaks)
    dom = max(kernels, key=lambda k: kernels[k]["ms"])
    d = kernels[dom]
    roof = {"kernel": d["kernel"], "bound": d["bound"], "achieved": d["achieved"], "peak": d["peak"], "unit": d["unit"],
            "frac": d["frac"], "traffic": d["traffic"], "peak_source": pk_kind + " (" + d["peak_name"] + ")",
            "algorithmic_per_launch": d["algorithmic_per_launch"], "launches_per_step": chunks}
    if dom == "ss" and m["correlation"]:
        # ss_fast_kernel is bound by FP32 issue, not by HBM: the algorithmic FP32 lane
        # operations per (path, l, v) element are 6 (q^2) + 5 (pdf) + 1 (decay
        # argument) per 8-tick chunk and 2 per tick (one product for the tick's decay
        # power, one accumulation) less one per chunk, plus 2 MUFU (rsqrt, ex2).  The
        # kernel issues 3 more products per chunk (a depth-3 product tree instead of
        # a serial chain, for latency); those are not counted as work.
        # Peak: the nominal FP32 lane rate, SMs x 128 lanes x the SM clock sampled
        # during the timed region (a nominal figure, not a measured one).
        import torch
        tchunks = (Nt + 7) // 8
        ops = float(P) * Nl * Nv * (11 * tchunks + 2 * Nt)
        sm_mhz = (clk or {}).get("sm_mhz") or 2070.0
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        lane_peak = sms * 128 * sm_mhz * 1e6 / 1e12
        ach = ops / (mean["ms_contract_ss"] / 1000) / 1e12
        roof["issue"] = {"unit": "FP32 lane-Tops/s", "achieved": ach, "peak": lane_peak, "frac": ach / lane_peak,
                         "ops_per_element": 11 * tchunks + 2 * Nt, "mufu_per_element": 2 * tchunks,
                         "peak_source": f"nominal: {sms} SMs x 128 FP32 lanes x {sm_mhz:.0f} MHz (sampled SM clock)"}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, st, dt = cpu_baseline(args.cpu_sample, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{args.cpu_sample} paths of the {WORKLOAD} workload (oracle, FP64, OpenMP), {dt:.1f} s"}

    lat_sorted = sorted(lat)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(dev_ms), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64 (split: FP64 path length and phase, 3xTF32 tensor-core contraction)" if precision == 0 else "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "paths_per_step": P, "Nl": Nl, "Nv": Nv, "Nt": Nt, "dims": dims,
                   "precision": args.precision, "parallelism": f"replicas{ws}",
                   "l2": "per-step working set (per-path rows) larger than L2"},
        "latency_ms": {"p50": lat_sorted[len(lat) // 2], "p99": lat_sorted[min(len(lat) - 1, int(math.ceil(0.99 * len(lat))) - 1)]},
        "phases_ms": mean,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": 1000 * e2e_s},
        "gpu_launches": int(launches),
        "roofline": roof,
        "kernels": {k: {kk: vv for kk, vv in v.items() if kk not in ("peak_name",)} for k, v in kernels.items()},
        "cpu_baseline": cpu,
        "clocks": clk,
        "wall_s": wall,
    }
    scene.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


def _serving_media(seed: int):
    """Eight seeded scenes of the serving mix: correlation slabs, 2D speckle,
    transmission-matrix grids and tracking frames of mixed sizes."""
    import random
    from temporalspecklescode_gb300 import workloads as wl
    rng = random.Random(seed)
    media = []
    for k in range(8):
        kind = k % 4
        paths_log2 = rng.randint(16, 20)
        waves = max(1, 1 << max(0, paths_log2 - 18))
        batch = (1 << paths_log2) // waves
        if kind == 0:
            media.append(wl.correlation_3d(batch_size=batch, full_iteration=waves, n_side=rng.choice([4, 6, 8]),
                                           n_lags=rng.randint(1, 8), seed=k))
        elif kind == 1:
            media.append(wl.speckle_2d(batch_size=batch, full_iteration=waves, n_dirs=rng.choice([16, 32, 64, 128]), seed=k))
        elif kind == 2:
            media.append(wl.transmission_matrix_3d(batch_size=batch // 16, full_iteration=waves, n_dirs=rng.choice([16, 32, 64]),
                                                   grid=(16, 16, 8), seed=k))
        else:
            media.append(wl.tracking_2d(batch_size=batch // 16, full_iteration=waves, n_dirs=rng.choice([16, 32]),
                                        frames=rng.randint(2, 8), seed=k))
    return media


def run_serve(args):
    """Serving mix: a Poisson stream of render requests over eight device-
    resident scenes, through the server (continuous batching) and one by one."""
    import random
    from temporalspecklescode_gb300 import api
    api.load_library()
    media = _serving_media(5)
    scenes = [api.Scene(cfg, dims) for cfg, dims in media]
    rng = random.Random(5)
    n_req = args.serve_requests
    picks = [rng.randrange(len(scenes)) for _ in range(n_req)]
    for s in scenes:          # warm-up: every kernel variant once
        s.render(seed=1)
    # one by one (sstmc_render), back to back
    t0 = time.perf_counter()
    contrib = 0
    for i, k in enumerate(picks):
        scenes[k].render(seed=100 + i)
        contrib += scenes[k].stats()["contributions"]
    one_s = time.perf_counter() - t0
    one_rate = contrib / one_s
    # served: Poisson arrivals at the one-by-one request rate x load
    mean_gap = one_s / n_req / args.serve_load
    with api.Server(slots=4) as srv:
        reqs = []
        t_next = time.perf_counter()
        for i, k in enumerate(picks):
            t_next += rng.expovariate(1.0 / mean_gap)
            delay = t_next - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            reqs.append(srv.submit(scenes[k], 100 + i))
        for r in reqs:
            r.result()
        st = srv.stats()
    for s in scenes:
        s.close()
    line = {
        "metric": "served NEE path-contributions/s (Poisson request mix over 8 resident scenes); p50/p99 latency",
        "value": st["contributions_per_s"], "unit": UNIT, "n_gpus": 1, "higher_is_better": True,
        "latency_ms": {"p50": st["p50_ms"], "p99": st["p99_ms"]}, "requests": n_req, "completed": st["completed"],
        "one_by_one": {"value": one_rate, "unit": UNIT, "seconds": one_s},
        "config": {"workload": "serving_mix", "media": len(scenes), "slots": 4, "load": args.serve_load,
                   "paths_per_request": "2^16 - 2^20", "seed": 5},
        "data": "synthetic",
    }
    print(json.dumps(line), flush=True)


def main():
    global WORKLOAD
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="split", choices=["split", "fp32"])
    ap.add_argument("--paths-log2", type=int, default=22)
    ap.add_argument("--cpu-sample", type=int, default=1 << 15)
    ap.add_argument("--ref-sample", type=int, default=1 << 14)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default=WORKLOAD, choices=WORKLOADS,
                    help="correlation_3d (the headline) or speckle_2d (2D far-field field speckle)")
    ap.add_argument("--serve", action="store_true", help="measure the serving mix instead of the headline workload")
    ap.add_argument("--serve-requests", type=int, default=48)
    ap.add_argument("--serve-load", type=float, default=2.0, help="arrival rate / one-by-one completion rate")
    args = ap.parse_args()
    WORKLOAD = args.workload
    if args.serve:
        run_serve(args)
        return
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    dist, rank, ws = _dist()
    if args.impl == "reference":
        run_reference(args, dist, rank, ws)
    else:
        run_gpu(args, dist, rank, ws)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
