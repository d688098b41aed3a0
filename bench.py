"""Benchmark: NEE path-contributions/s of the path tracer on one workload.

Workloads (one step = one render of seeded synthetic inputs; one contribution
is one (path, scattering vertex, illumination, view, tick) term of the
estimator):
  correlation_3d (default, the headline): slab [-100,100]^2 x [0,20],
      sigs=[0,0.5], siga=[0,0.01], HG g=0.9, 64 point illuminations at z=-5
      and 64 point views at z=25 on jittered 8x8 lattices, Brownian
      D=[0,1e-3], 8 lags; 2^22 paths (4 waves of 2^20).
  speckle_2d: 2D single-bin box [-50,50]^2, sigs=[0,1], HG g=0.8, 16 x 16
      far-field directions over [-pi/6, pi/6]; 65,536 paths.
  transmission_matrix_3d: 64x64x32 grid over [-64,64]^2 x [0,64] of iid
      materials {1..4}, HG g=0.85, 1024 x 1024 far-field directions on
      20-degree cones; 2^24 paths.
  tracking_2d_pairs: 256^2 grid with a disc (sigs=4) whose scatterers drift
      by (0.5, 0) per frame, HG g=0.7, 128 x 128 far field, correlations of
      all 32 x 32 frame pairs from the 32 lags t2 - t1 >= 0 (conjugates for the rest); 2^23 paths.

value : contributions / device time of the render (CUDA events on the
        library's stream; scene tables resident in HBM).
e2e   : the same metric through the public C-ABI call a MATLAB-style user
        makes -- scene creation (host -> device upload of the config tables),
        render, read-back of u and iter, scene destruction -- timed on the host.
plain_fp32 : the plain FP32 form (FP32 phases, SIMT contraction) on the same
        workload; rel_err_vs_fp64: both forms against the FP64 oracle on a
        path subset of the workload.
--impl reference: the reference has no CPU implementation, so the reference
        arm times the CPU FP64 restatement of its estimator (oracle/) on all
        host threads.
--impl reference-gpu: the reference's own CUDA path (its headers staged by
        oracle/stage_reference.sh, built by oracle/refharness.mk) on the
        workload's scene at a reduced batch.

Multi-GPU (torchrun): replicas with disjoint seeds ("replicas only": the
paths are i.i.d.); the one exchange step sums the ranks' accumulators and
iteration counts after each render (all_reduce, its time part of the step);
value is the sum of contributions over ranks divided by the max time over
ranks.
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
WORKLOAD = "correlation_3d"   # the headline (3D temporal correlation, 64 x 64 x 8, 2^22 paths)

# Per workload: default path count, CPU oracle sample sizes (about 10-30 s of
# host work on 16 cores) and the path subset of the error measurement against
# the FP64 oracle.
WORKLOADS = {
    # 3D temporal correlation: point sources on jittered 8x8 lattices, 8 lags
    "correlation_3d": {"paths_log2": 22, "cpu_sample": 1 << 15, "ref_sample": 1 << 14, "err_paths": 1 << 14},
    # 2D far-field speckle field: 16 x 16, one tick, 65,536 paths
    "speckle_2d": {"paths_log2": 16, "cpu_sample": 1 << 16, "ref_sample": 1 << 15, "err_paths": 1 << 14},
    # 3D transmission matrix: 1024 x 1024 far field, 64x64x32 grid of 4 materials, 2^24 paths
    "transmission_matrix_3d": {"paths_log2": 24, "cpu_sample": 1 << 11, "ref_sample": 1 << 10, "err_paths": 1 << 8},
    # 2D tracking: 128 x 128 far field, 256^2 grid with a drifting disc, all 32 x 32 frame pairs (32 lags)
    "tracking_2d_pairs": {"paths_log2": 23, "cpu_sample": 1 << 6, "ref_sample": 1 << 5, "err_paths": 1 << 3},
    # 3D focused Gaussian beams: 64 x 64 beams on a confocal grid in a four-material vMF slab
    "confocal_3d": {"paths_log2": 14, "cpu_sample": 1 << 14, "ref_sample": 1 << 12, "err_paths": 1 << 11},
}

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


def _merge_over_ranks(dist, u, it):
    """The replicas' one exchange step: the sum of every rank's accumulator u
    (complex, Nl x Nv x Nt x renderings) and iteration counts, so the merged
    render is the render of all ranks' paths (normalise by the summed iter)."""
    import numpy as np
    if dist is None:
        return u, it
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.from_numpy(np.ascontiguousarray(np.stack([u.real, u.imag]))).to(dev)
    n = torch.from_numpy(np.ascontiguousarray(it, dtype=np.float64)).to(dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    t = t.cpu().numpy()
    return t[0] + 1j * t[1], n.cpu().numpy()


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


def _workload(seed: int, paths_log2: int, workload: str | None = None):
    """The workload's scene with 2^paths_log2 paths (waves of at most 2^20)."""
    from temporalspecklescode_gb300 import workloads as wl
    workload = workload or WORKLOAD
    waves = max(1, 1 << max(0, paths_log2 - 20))
    batch = (1 << paths_log2) // waves
    if workload == "speckle_2d":
        return wl.speckle_2d(batch_size=batch, full_iteration=waves, seed=seed)
    if workload == "transmission_matrix_3d":
        return wl.transmission_matrix_3d(batch_size=batch, full_iteration=waves, seed=seed)
    if workload == "tracking_2d_pairs":
        return wl.tracking_2d_pairs(batch_size=batch, full_iteration=waves, seed=seed)
    if workload == "confocal_3d":
        return wl.confocal_3d(batch_size=batch, full_iteration=waves, seed=seed)
    return wl.correlation_3d(batch_size=batch, full_iteration=waves, seed=seed)


def _sample_workload(paths: int, seed: int = 0):
    cfg, dims = _workload(seed, 20)
    cfg["simulation"]["batchSize"] = paths
    cfg["simulation"]["fullIteration"] = 1
    return cfg, dims


def cpu_baseline(sample_paths: int, threads: int):
    """Time the CPU oracle (FP64 restatement, OpenMP) on a bounded sample."""
    from temporalspecklescode_gb300 import config as cf
    from tests.oracle_lib import Oracle
    cfg, dims = _sample_workload(sample_paths)
    pc = cf.prepare(cfg, dims)
    oracle = Oracle()
    t0 = time.perf_counter()
    _, _, st = oracle.render(pc, 0, threads=threads)
    dt = time.perf_counter() - t0
    return st["contributions"] / dt, st, dt


def error_vs_oracle(paths: int, threads: int):
    """Relative Frobenius error of the split-precision and plain FP32 renders
    against the FP64 oracle on the same seeded paths (a subset of the
    workload: its scene with `paths` paths)."""
    import numpy as np
    from temporalspecklescode_gb300 import api, config as cf
    from tests.oracle_lib import Oracle
    cfg, dims = _sample_workload(paths, seed=0)
    uo, ito, _ = Oracle().render(cf.prepare(cfg, dims), 7, threads=threads)
    out = {"paths": paths}
    for name, prec in (("split", cf.PRECISION_SPLIT), ("plain_fp32", cf.PRECISION_FP32)):
        with api.Scene(cfg, dims, prec) as s:
            u, it = s.render(seed=7)
        if it[0] != ito:
            raise RuntimeError(f"error subset: iteration count {it[0]} differs from the oracle's {ito}")
        out[name] = float(np.linalg.norm(u[..., 0] - uo) / np.linalg.norm(uo))
    return out


def run_reference(args, dist, rank, ws):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    sample = args.ref_sample or WORKLOADS[WORKLOAD]["ref_sample"]
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


def run_reference_gpu(args):
    """The reference's own CUDA path (oracle/refharness.cu over the staged
    reference headers) on the workload's scene with a reduced batch (the
    reference materialises P x P permutation matrices and P x Nl x Nv x Nt
    products): device time per trace from its harness, contributions per
    trace estimated by this build's render of the same scene (the same path
    distribution; the reference reports no vertex counts)."""
    from temporalspecklescode_gb300 import api
    from tests import refharness_lib as ref
    if not ref.available():
        print(json.dumps({"impl": "reference-gpu", "unavailable": "the reference headers are not staged (oracle/stage_reference.sh)"}))
        return
    batch = args.ref_gpu_batch
    cfg, dims = _workload(0, 20)
    cfg["simulation"]["batchSize"] = batch
    cfg["simulation"]["fullIteration"] = args.ref_gpu_waves
    R = args.warmup + args.steps
    _, it_ref, ms = ref.render(cfg, dims, R, seed=0)
    ms = ms[args.warmup:]
    api.load_library()
    contrib = []
    with api.Scene(cfg, dims) as s:
        for sd in range(3):
            s.render(seed=100 + sd)
            contrib.append(s.stats()["contributions"])
    c = statistics.mean(contrib)
    mms = statistics.mean(ms)
    line = {"impl": "reference-gpu", "metric": METRIC, "value": c / (mms / 1000), "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": mms, "higher_is_better": True,
            "dtype": "f64 (the reference's PRECISION DOUBLE)", "data": "synthetic",
            "config": {"workload": WORKLOAD, "paths_per_step": batch * args.ref_gpu_waves, "batch": batch,
                       "note": "contributions per trace estimated from this build's render of the same scene"}}
    print(json.dumps(line), flush=True)


# DRAM bytes (read + write) per path of each kernel class from one ncu capture
# of the workload at a small path count; every class streams per-path rows,
# so a launch's traffic scales with the paths it processes.
NCU_DRAM_BYTES_PER_PATH = {
    "correlation_3d": {   # 2^16 paths
        "nee": (8354816 + 156937728 + 14934272 + 75123456) / 65536,   # illum_kernel + view_kernel
        "walk": (242688 + 176896 + 18749184 + 1536) / 65536,          # walk_kernel<slots> + compact_kernel
        "gemm": (269205504 + 3310592) / 65536,                         # gemm_tc_kernel (real rows)
        "ss": (68522752 + 932352) / 65536,                             # ss_fast_kernel
    },
}

KERNEL_NAMES = {
    "correlation_3d": {"nee": "illum_kernel + view_kernel (NEE vectors)", "ss": "ss_fast_kernel (single-scattering contraction)"},
    "speckle_2d": {"nee": "trace_kernel (illumination side) + view_kernel (NEE vectors)",
                   "ss": "gemm_tc_kernel x materials (far x far single scattering, weight tables)"},
    "transmission_matrix_3d": {"nee": "trace_kernel (illumination side) + view_kernel (NEE vectors)",
                               "ss": "gemm_tc_kernel x materials (far x far single scattering, weight tables)"},
    "tracking_2d_pairs": {"nee": "trace_kernel (fused NEE vectors, drifting scatterers)",
                          "ss": "gemm_tc_kernel x materials (far x far single scattering, weight tables)"},
    "confocal_3d": {"nee": "gauss_trace_kernel (beam NEE vectors, FP64 amplitudes)",
                    "ss": "gauss_ss_kernel (beam x beam single scattering, FP64 amplitudes)"},
}


def _kernel_rooflines(scene, mean, verts_per_step, dda_per_step, chunks, peaks, rows_real):
    """Per kernel class: time per step, algorithmic bytes or flops per launch,
    achieved rate and the fraction of the measured peak."""
    m = scene.meta
    P = m["P"] * m["waves"]
    Nl, Nv, Nt = m["Nl"], m["Nv"], m["Nt"]
    hbm, tc = peaks["hbm_gbs"], peaks["bf16_tflops"]
    ridge = tc * 1e12 / (hbm * 1e9)   # flop per byte where the two measured roofs meet
    ncu = NCU_DRAM_BYTES_PER_PATH.get(WORKLOAD, {})
    names = KERNEL_NAMES.get(WORKLOAD, KERNEL_NAMES["correlation_3d"])
    out = {}

    def add(key, name, ms, bound, amount, note, extra=None):
        per_launch = amount / chunks
        traffic = ncu[key] * P / chunks if key in ncu else None
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
        if extra:
            out[key].update(extra)

    # NEE vectors: rows written once (a_ms all ticks, single-scattering rows, s_ms),
    # P_l, the vertices read.  Real rows (correlation, static, u1 = u2): 4 bytes per
    # (tick, element); complex: 8.
    rb = 4.0 if rows_real else 8.0
    ss_ticks = 1 if rows_real else Nt
    nee_bytes = P * (rb * Nt * Nl + 8.0 * ss_ticks * (Nl + Nv) + rb * Nt * Nv + 4 * Nl + 13 + 12) + 16.0 * verts_per_step
    add("nee", names["nee"], mean["ms_nee"], "hbm", nee_bytes,
        "FP32 / voxel-step issue bound: DRAM traffic equals the row bytes",
        {"voxel_steps_per_s": dda_per_step / (mean["ms_nee"] / 1000) if mean["ms_nee"] > 0 else None})
    # random walk: one pass into per-path slots + compaction; vertices written once, counts / misses / offsets
    add("walk", "walk_kernel (single-pass random walk) + compaction", mean["ms_walk"], "hbm", 16.0 * verts_per_step + 20.0 * P,
        "FP32-issue bound (IEEE-rounded decision path)")
    # multiple-scattering contraction: useful flops 8 Nl Nv Nt per path for complex rows
    # (a complex MAC), 2 Nl Nv Nt for real rows; bytes: the a_ms and s_ms rows read once.
    # The binding roof is the one its arithmetic intensity reaches first.
    gflops = (2.0 if rows_real else 8.0) * Nl * Nv * Nt * P
    gbytes = rb * Nt * (Nl + Nv) * P
    gbound = "tensor" if gflops / gbytes >= ridge else "hbm"
    other = ({"achieved_tflops": gflops / (mean["ms_contract_ms"] / 1000) / 1e12} if gbound == "hbm"
             else {"achieved_gbs": gbytes / (mean["ms_contract_ms"] / 1000) / 1e9})
    other["useful_flops_per_launch"] = gflops / chunks
    other["flop_per_byte"] = gflops / gbytes
    add("gemm", "gemm_tc_kernel (multiple-scattering contraction, tcgen05 3xTF32)", mean["ms_contract_ms"], gbound,
        gflops if gbound == "tensor" else gbytes,
        "useful flops (not the 3 TF32 passes) against the measured dense bf16 peak" if gbound == "tensor"
        else "reads the a_ms and s_ms rows once", other)
    if WORKLOAD == "correlation_3d":
        # single-scattering contraction: tick-0 rows read (tick-invariant form)
        add("ss", names["ss"], mean["ms_contract_ss"], "hbm", P * 8.0 * (Nl + Nv),
            "FP32/SFU-issue bound: one exp and one rsqrt per (path, l, v)")
    elif WORKLOAD == "confocal_3d":
        # beam x beam single scattering: the rows of every tick read once, V written;
        # the FP64 amplitude per (path, l, v) bounds it, not the bytes
        add("ss", names["ss"], mean["ms_contract_ss"], "hbm", P * 8.0 * Nt * (Nl + Nv) + 16.0 * Nl * Nv * Nt,
            "FP64-issue bound: one beam x lobe x beam amplitude per (path, l, v)")
    else:
        # far x far: one GEMM per material over its paths, weights per (l, v, t, material)
        sflops = 8.0 * Nl * Nv * Nt * P
        sbytes = 8.0 * Nt * (Nl + Nv) * P
        sbound = "tensor" if sflops / sbytes >= ridge else "hbm"
        add("ss", names["ss"], mean["ms_contract_ss"], sbound, sflops if sbound == "tensor" else sbytes,
            "per-material GEMMs over the paths of that first-vertex material", {"useful_flops_per_launch": sflops / chunks})
    return out


def _render_series(scene, seeds, dist=None):
    """Render each seed; device time, statistics and (over replicas) the time
    of merging the ranks' accumulators per render."""
    res = []
    for sd in seeds:
        ts = time.perf_counter()
        u, it = scene.render(seed=sd)
        host_ms = 1000 * (time.perf_counter() - ts)
        tm, st = scene.timing(), scene.stats()
        tm["ms_merge"] = 0.0
        if dist is not None:
            tq = time.perf_counter()
            _merge_over_ranks(dist, u, it)
            tm["ms_merge"] = 1000 * (time.perf_counter() - tq)
        res.append((host_ms, tm, st))
    return res


def side_workload(name: str, paths_log2: int, renders: int = 2):
    """A second workload measured in the same run at a stated path count: its
    contributions/s (CUDA-event device time), phases and the contraction's
    useful tensor throughput; the headline line carries it beside its own."""
    global WORKLOAD
    from temporalspecklescode_gb300 import api
    saved, WORKLOAD = WORKLOAD, name
    try:
        cfg, dims = _workload(0, paths_log2)
        with api.Scene(cfg, dims) as s:
            s.render(seed=1)
            series = _render_series(s, [50 + i for i in range(renders)])
            m = s.meta
    finally:
        WORKLOAD = saved
    ms = statistics.mean([tm["ms_total"] for _, tm, _ in series])
    contrib = statistics.mean([st["contributions"] for _, _, st in series])
    dda = statistics.mean([st["dda_steps"] for _, _, st in series])
    phases = {k: statistics.mean([tm[k] for _, tm, _ in series]) for k in ("ms_walk", "ms_nee", "ms_contract_ms", "ms_contract_ss")}
    P = m["P"] * m["waves"]
    flops = 8.0 * m["Nl"] * m["Nv"] * m["Nt"] * P   # complex MACs of one contraction over every path's rows
    peaks, _ = _peaks()
    out = {"workload": name, "paths": P, "value": contrib / (ms / 1000), "unit": UNIT, "ms_per_render": ms,
           "renders": renders, "phases_ms": phases, "voxel_steps_per_s": dda / (phases["ms_nee"] / 1000)}
    for key, label in (("ms_contract_ms", "gemm_multiple"), ("ms_contract_ss", "gemm_single")):
        t = phases[key] / 1000
        if t > 0:
            out[label] = {"useful_tflops": flops / t / 1e12, "frac_of_bf16_peak": flops / t / 1e12 / peaks["bf16_tflops"]}
    return out


def run_gpu(args, dist, rank, ws):
    from temporalspecklescode_gb300 import api, config as cf
    api.load_library()
    spec = WORKLOADS[WORKLOAD]
    paths_log2 = args.paths_log2 or spec["paths_log2"]
    precision = cf.PRECISION_FP32 if args.precision == "fp32" else cf.PRECISION_SPLIT
    cfg, dims = _workload(seed=1000 * rank, paths_log2=paths_log2)
    scene = api.Scene(cfg, dims, precision)
    wavefront = scene.autotune(args.autotune) if args.autotune else None
    lat = []
    dev_ms = []
    parts = {"ms_trace": [], "ms_contract_ms": [], "ms_contract_ss": [], "ms_walk": [], "ms_nee": []}
    chunks = 1
    verts = 0
    dda = 0
    contrib = 0
    launches = 0
    for i in range(args.warmup):
        scene.render(seed=i)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    _barrier(dist)
    clocks.start()
    t0 = time.perf_counter()
    for host_ms, tm, st in _render_series(scene, [100 + i for i in range(args.steps)], dist):
        lat.append(host_ms)
        dev_ms.append(tm["ms_total"] + tm["ms_merge"])   # replicas: the accumulator merge is part of the step
        for k in parts:
            parts[k].append(tm[k])
        launches += tm["launches"]
        chunks = tm["chunks"]
        contrib += st["contributions"]
        verts += st["vertices"]
        dda += st["dda_steps"]
    wall = time.perf_counter() - t0
    _barrier(dist)
    clk = clocks.stop()
    dev_total_s = sum(dev_ms) / 1000.0
    dev_total_s = _max_over_ranks(dist, dev_total_s)
    contrib_all = _sum_over_ranks(dist, float(contrib))
    value = contrib_all / dev_total_s
    rows_real = bool(scene.meta["correlation"]) and WORKLOAD == "correlation_3d" and precision == cf.PRECISION_SPLIT
    heavy = statistics.mean(dev_ms) > 2000.0   # renders of seconds: fewer repeats in the side measurements

    # end to end through the C-ABI: create (upload) + render + read back + destroy
    e2e_t = []
    h2d = 0
    # one untimed call first: the first scene created next to the resident one
    # grows the stream-ordered memory pool
    with api.Scene(cfg, dims, precision) as s2:
        u, it = s2.render(seed=199)
    for i in range(1 if heavy else max(1, min(3, args.steps))):
        ts = time.perf_counter()
        with api.Scene(cfg, dims, precision) as s2:
            u, it = s2.render(seed=200 + i)
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
    kernels = _kernel_rooflines(scene, mean, verts / args.steps, dda / args.steps, chunks, peaks, rows_real)
    dom = max(kernels, key=lambda k: kernels[k]["ms"])
    d = kernels[dom]
    roof = {"kernel": d["kernel"], "bound": d["bound"], "achieved": d["achieved"], "peak": d["peak"], "unit": d["unit"],
            "frac": d["frac"], "traffic": d["traffic"], "peak_source": pk_kind + " (" + d["peak_name"] + ")",
            "algorithmic_per_launch": d["algorithmic_per_launch"], "launches_per_step": chunks}
    if dom == "ss" and WORKLOAD == "correlation_3d":
        # ss_fast_kernel is bound by FP32 issue, not by HBM.  FP32 lane operations
        # per (path, l, v) element and 8-tick chunk, an FMA
        # counted once: 3 (q^2 as 2 - 2 in . out) + 1 (the pdf's base) + 1 (row
        # product) + 1 (decay argument) + 1 (first tick's exponent with the pdf's
        # power) + 1 (first term) + 2 (squared and fourth decay powers) + 11 (the
        # 8 tick terms: 3 products, 4 adds, 4 FMAs) = 21, plus 3 MUFU (lg2, 2 ex2).
        # Peak: the nominal FP32 lane rate, SMs x 128 lanes x the SM clock sampled
        # during the timed region (a nominal figure, not a measured one).
        import torch
        tchunks = (Nt + 7) // 8
        ops = float(P) * Nl * Nv * 21 * tchunks
        sm_mhz = (clk or {}).get("sm_mhz") or 2070.0
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        lane_peak = sms * 128 * sm_mhz * 1e6 / 1e12
        ach = ops / (mean["ms_contract_ss"] / 1000) / 1e12
        roof["issue"] = {"unit": "FP32 lane-Tops/s", "achieved": ach, "peak": lane_peak, "frac": ach / lane_peak,
                         "ops_per_element": 21 * tchunks, "mufu_per_element": 3 * tchunks,
                         "peak_source": f"nominal: {sms} SMs x 128 FP32 lanes x {sm_mhz:.0f} MHz (sampled SM clock)"}

    # the plain FP32 form (FP32 phases, uncompensated SIMT contraction) on the same
    # workload and paths, for the split / plain ratio
    plain = None
    if precision == cf.PRECISION_SPLIT and not args.no_plain:
        with api.Scene(cfg, dims, cf.PRECISION_FP32) as s3:
            s3.render(seed=0)
            series = _render_series(s3, [100 + i for i in range(1 if heavy else 3)])
        pms = statistics.mean([tm["ms_total"] for _, tm, _ in series])
        pval = statistics.mean([st["contributions"] for _, _, st in series]) / (pms / 1000)
        plain = {"value": pval, "unit": UNIT, "ms_per_step": pms, "renders": len(series),
                 "split_over_plain": value / pval if ws == 1 else None}

    side = None
    if rank == 0 and ws == 1 and args.side_paths_log2 > 0 and WORKLOAD == "correlation_3d":
        side = side_workload("transmission_matrix_3d", args.side_paths_log2)

    cpu = None
    err = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sample = args.cpu_sample or spec["cpu_sample"]
        v, st, dt = cpu_baseline(sample, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{sample} paths of the {WORKLOAD} workload (oracle, FP64, OpenMP), {dt:.1f} s"}
        err = error_vs_oracle(spec["err_paths"], threads)

    lat_sorted = sorted(lat)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(dev_ms), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": ("f32 (split: path length and phase reduction in float-float FP32 in the view kernel and FP64 in the "
                  "general kernel, 3xTF32 tensor-core contraction with FP32 accumulation, FP64 output)")
                 if precision == cf.PRECISION_SPLIT else "f32 (plain: FP32 phases, FP32 SIMT contraction)",
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
        "plain_fp32": plain,
        "other_workloads": [side] if side else [],
        "rel_err_vs_fp64": err,
        "cpu_baseline": cpu,
        "clocks": clk,
        "wall_s": wall,
    }
    if wavefront:
        line["config"]["wavefront"] = f"{wavefront} paths per chunk (sstmc_scene_autotune over a {args.autotune}-path sample)"
    if WORKLOAD == "tracking_2d_pairs":
        line["config"]["frame_pairs"] = "32 x 32 frame pairs from the 32 lags t2 - t1 >= 0, conjugates for t2 < t1 (workloads.frame_pairs)"
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
    for s in scenes:          # wavefront per medium, then warm-up: every kernel variant once
        if args.autotune:
            s.autotune(args.autotune)
        s.render(seed=1)
    # one by one (sstmc_render), back to back; each request's own render time
    t0 = time.perf_counter()
    contrib = 0
    solo = []
    for i, k in enumerate(picks):
        ts = time.perf_counter()
        scenes[k].render(seed=100 + i)
        solo.append(time.perf_counter() - ts)
        contrib += scenes[k].stats()["contributions"]
    one_s = time.perf_counter() - t0
    one_rate = contrib / one_s
    # served: Poisson arrivals at the one-by-one request rate x load
    mean_gap = one_s / n_req / args.serve_load
    with api.Server(slots=4) as srv:
        reqs = []
        submitted = []
        done = [None] * n_req

        def poll():
            # completion times by polling every 0.2 ms, also between arrivals
            # (latency = completion - submission)
            for i, r in enumerate(reqs):
                if done[i] is None and r.done():
                    done[i] = time.perf_counter()
            time.sleep(2e-4)

        t_next = time.perf_counter()
        for i, k in enumerate(picks):
            t_next += rng.expovariate(1.0 / mean_gap)
            while time.perf_counter() < t_next:
                poll()
            reqs.append(srv.submit(scenes[k], 100 + i))
            submitted.append(time.perf_counter())
        while any(d is None for d in done):
            poll()
        for r in reqs:
            r.result()
        st = srv.stats()
    # slowdown: a request's latency over its own render time alone (1 = no
    # queueing or sharing cost; the mix's long renders make the raw latency
    # percentiles a property of the request sizes, the slowdown one of the server)
    slow = sorted((d - t) / max(so, 1e-9) for d, t, so in zip(done, submitted, solo))
    pct = lambda v, q: v[min(len(v) - 1, int(math.ceil(q * len(v))) - 1)]
    for s in scenes:
        s.close()
    line = {
        "metric": "served NEE path-contributions/s (Poisson request mix over 8 resident scenes); p50/p99 latency",
        "value": st["contributions_per_s"], "unit": UNIT, "n_gpus": 1, "higher_is_better": True,
        "latency_ms": {"p50": st["p50_ms"], "p99": st["p99_ms"]}, "requests": n_req, "completed": st["completed"],
        "slowdown": {"p50": pct(slow, 0.50), "p99": pct(slow, 0.99),
                     "what": "latency / the request's own render time alone"},
        "solo_ms": {"p50": 1000 * sorted(solo)[len(solo) // 2], "max": 1000 * max(solo)},
        "one_by_one": {"value": one_rate, "unit": UNIT, "seconds": one_s},
        "config": {"workload": "serving_mix", "media": len(scenes), "slots": 4, "load": args.serve_load,
                   "paths_per_request": "2^16 - 2^20", "seed": 5,
                   "wavefront": f"autotuned per medium over {args.autotune} paths" if args.autotune else "default"},
        "data": "synthetic",
    }
    print(json.dumps(line), flush=True)


def main():
    global WORKLOAD
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference", "reference-gpu"],
                    help="reference: the CPU FP64 oracle; reference-gpu: the reference's own CUDA path (staged headers)")
    ap.add_argument("--ref-gpu-batch", type=int, default=512, help="reference-gpu: batchSize per wave")
    ap.add_argument("--ref-gpu-waves", type=int, default=4, help="reference-gpu: fullIteration")
    ap.add_argument("--precision", default="split", choices=["split", "fp32"])
    ap.add_argument("--paths-log2", type=int, default=0, help="paths per render (log2); 0: the workload's own")
    ap.add_argument("--cpu-sample", type=int, default=0, help="paths of the CPU oracle sample; 0: the workload's own")
    ap.add_argument("--ref-sample", type=int, default=0, help="paths per reference-arm step; 0: the workload's own")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU oracle sample and the error subset")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP32 comparison render")
    ap.add_argument("--workload", default=WORKLOAD, choices=sorted(WORKLOADS),
                    help="correlation_3d (the headline), speckle_2d, transmission_matrix_3d or tracking_2d_pairs")
    ap.add_argument("--side-paths-log2", type=int, default=18,
                    help="headline run: also measure the 1024 x 1024 transmission matrix at this many paths (0: off)")
    ap.add_argument("--autotune", type=int, default=0,
                    help="choose the wavefront (paths per chunk) by timing this many paths per candidate first (0: off)")
    ap.add_argument("--serve", action="store_true", help="measure the serving mix instead of the headline workload")
    ap.add_argument("--serve-requests", type=int, default=48)
    ap.add_argument("--serve-load", type=float, default=2.0, help="arrival rate / one-by-one completion rate")
    args = ap.parse_args()
    WORKLOAD = args.workload
    if args.serve:
        run_serve(args)
        return
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    if args.impl == "reference-gpu":
        run_reference_gpu(args)
        return
    dist, rank, ws = _dist()
    if args.impl == "reference":
        run_reference(args, dist, rank, ws)
    else:
        run_gpu(args, dist, rank, ws)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
