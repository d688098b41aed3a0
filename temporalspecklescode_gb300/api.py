"""Python host API over the C-ABI (include/sstmc.h).

``sstmc2D(config)`` / ``sstmc3D(config)`` return ``(u, iter)`` like the
reference's MEX functions (README.md:355-373, MatlabInterface.cu:1565-1825):
``u`` complex, shape (Nl, Nv, Nt, renderingsNum); ``iter`` shape
(renderingsNum,), with ``iter[r] = batchSize * fullIteration + missed first
vertices``.  Normalise a field by ``sqrt(iter)`` and a correlation by ``iter``.

The CUDA library must be built (``__graft_entry__.build()``); there is no CPU
fallback: a missing library raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Any, Dict, Optional, Tuple

import numpy as np

from . import _build
from . import config as cf

_LIB: Optional[C.CDLL] = None


class SstmcError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        super().__init__(f"sstmc error {code}: {what}")


def load_library() -> C.CDLL:
    """Load the in-tree CUDA library; raise if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.lib_path()
    if not os.path.exists(path):
        raise ImportError(f"{path} not found: build the CUDA library first (__graft_entry__.build())")
    lib = C.CDLL(path)
    i32, u32, u64, vp = C.c_int32, C.c_uint32, C.c_uint64, C.c_void_p
    dp = C.POINTER(C.c_double)
    lib.sstmc_config_init.argtypes = [C.POINTER(cf.SstmcConfig)]
    lib.sstmc_config_init.restype = None
    lib.sstmc_scene_create.argtypes = [C.POINTER(cf.SstmcConfig), C.POINTER(vp)]
    lib.sstmc_scene_create.restype = i32
    lib.sstmc_scene_shape.argtypes = [vp, C.POINTER(u32), C.POINTER(u32), C.POINTER(u32)]
    lib.sstmc_scene_shape.restype = i32
    lib.sstmc_render.argtypes = [vp, u64, dp, dp]
    lib.sstmc_render.restype = i32
    lib.sstmc_scene_autotune.argtypes = [vp, u32, C.POINTER(u64)]
    lib.sstmc_scene_autotune.restype = i32
    lib.sstmc_render_static.argtypes = [vp, u64, dp, dp]
    lib.sstmc_render_static.restype = i32
    lib.sstmc_last_stats.argtypes = [vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)]
    lib.sstmc_last_stats.restype = i32
    lib.sstmc_last_timing.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(u64)]
    lib.sstmc_last_timing.restype = i32
    lib.sstmc_scene_destroy.argtypes = [vp]
    lib.sstmc_scene_destroy.restype = i32
    lib.sstmc_error_string.argtypes = [i32]
    lib.sstmc_error_string.restype = C.c_char_p
    lib.sstmc_last_error_text.argtypes = []
    lib.sstmc_last_error_text.restype = C.c_char_p
    lib.sstmc_trace_paths.argtypes = [vp, u64, u32, u32, C.POINTER(cf.PathTrace)]
    lib.sstmc_trace_paths.restype = i32
    lib.sstmc_server_create.argtypes = [i32, u64, u32, C.POINTER(vp)]
    lib.sstmc_server_create.restype = i32
    lib.sstmc_server_destroy.argtypes = [vp]
    lib.sstmc_server_destroy.restype = i32
    lib.sstmc_submit.argtypes = [vp, vp, u64, dp, dp, C.POINTER(u64)]
    lib.sstmc_submit.restype = i32
    lib.sstmc_poll.argtypes = [vp, u64, C.POINTER(i32), C.POINTER(i32)]
    lib.sstmc_poll.restype = i32
    lib.sstmc_wait.argtypes = [vp, u64, C.c_double, C.POINTER(i32)]
    lib.sstmc_wait.restype = i32
    lib.sstmc_cancel.argtypes = [vp, u64]
    lib.sstmc_cancel.restype = i32
    lib.sstmc_server_stats.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(u64)]
    lib.sstmc_server_stats.restype = i32
    _declare_objects(lib)
    _LIB = lib
    return lib


def _declare_objects(lib: C.CDLL) -> None:
    """Signatures of the object-model entry points (sstmc_simulation_* ..
    sstmc_tracer_*), the reference's plugin setters."""
    i32, u32, u64, vp, d = C.c_int32, C.c_uint32, C.c_uint64, C.c_void_p, C.c_double
    dp, up = C.POINTER(C.c_double), C.POINTER(C.c_uint32)
    sig = {
        "sstmc_simulation_create": [u32, u32, d, i32, i32, C.POINTER(vp)],
        "sstmc_simulation_destroy": [vp],
        "sstmc_scattering_create": [C.POINTER(vp)],
        "sstmc_scattering_set_isotropic": [vp, u32],
        "sstmc_scattering_set_henyey_greenstein": [vp, d, u32],
        "sstmc_scattering_set_tabular": [vp, dp, u32, u32],
        "sstmc_scattering_set_von_mises_fisher": [vp, dp, dp, dp, u32, u32],
        "sstmc_scattering_destroy": [vp],
        "sstmc_medium_create_heterogeneous": [up, dp, u32, dp, u32, dp, u32, C.POINTER(vp)],
        "sstmc_medium_create_homogeneous": [u32, dp, dp, d, C.POINTER(vp)],
        "sstmc_medium_set_material": [vp, d, d, u32],
        "sstmc_medium_destroy": [vp],
        "sstmc_source_create_point": [vp, i32, dp, u32, i32, C.POINTER(vp)],
        "sstmc_source_create_far_field": [vp, i32, dp, u32, C.POINTER(vp)],
        "sstmc_source_create_gaussian_beam": [vp, i32, dp, dp, u32, C.c_double, C.POINTER(vp)],
        "sstmc_source_size": [vp, up],
        "sstmc_source_destroy": [vp],
        "sstmc_sampler_create_temporal": [vp, vp, vp, vp, vp, dp, u32, i32, i32, C.POINTER(vp)],
        "sstmc_sampler_create_correlation": [vp, vp, vp, vp, vp, vp, vp, dp, u32, C.POINTER(vp)],
        "sstmc_sampler_set_material": [vp, d, dp, u32],
        "sstmc_sampler_shape": [vp, up, up, up],
        "sstmc_sampler_is_correlation": [vp, C.POINTER(i32)],
        "sstmc_sampler_config": [vp, u32, u64, i32, C.POINTER(cf.SstmcConfig)],
        "sstmc_sampler_destroy": [vp],
        "sstmc_tracer_create_nee": [vp, u32, u64, i32, C.POINTER(vp)],
        "sstmc_tracer_trace": [vp, dp],
        "sstmc_tracer_update_seed": [vp, u64],
        "sstmc_tracer_zero_contribution_paths": [vp, C.POINTER(u64)],
        "sstmc_tracer_photons_budget": [vp, C.POINTER(u64)],
        "sstmc_tracer_is_cbs": [vp, C.POINTER(i32)],
        "sstmc_tracer_destroy": [vp],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = i32
    lib.sstmc_tracer_scene.argtypes = [vp]
    lib.sstmc_tracer_scene.restype = vp


def error_string(code: int) -> str:
    return load_library().sstmc_error_string(code).decode()


def _check(code: int, extra: str = "") -> None:
    if code != 0:
        msg = error_string(code)
        raise SstmcError(code, msg + (f" ({extra})" if extra else ""))


class Scene:
    """A device-resident scene (the objects mexFunction builds, MatlabInterface.cu:1677-1700)."""

    def __init__(self, config: Dict[str, Any], dims: int, precision: int = cf.PRECISION_SPLIT):
        self.lib = load_library()
        self.prepared = cf.prepare(config, dims, precision)
        self.meta = self.prepared.meta
        h = C.c_void_p()
        code = self.lib.sstmc_scene_create(self.prepared.ptr(), C.byref(h))
        if code != 0:
            detail = self.lib.sstmc_last_error_text().decode()
            raise SstmcError(code, error_string(code) + (f": {detail}" if detail else ""))
        self.handle = h
        nl, nv, nt = C.c_uint32(), C.c_uint32(), C.c_uint32()
        _check(self.lib.sstmc_scene_shape(h, C.byref(nl), C.byref(nv), C.byref(nt)))
        self.Nl, self.Nv, self.Nt = nl.value, nv.value, nt.value
        self.renders = self.meta["R"]

    def render(self, seed: Optional[int] = None) -> Tuple[np.ndarray, np.ndarray]:
        return self._render(self.lib.sstmc_render, seed)

    def autotune(self, sample_paths: int = 1 << 18) -> int:
        """Time the scene's first `sample_paths` paths at each candidate wavefront
        (paths per chunk of kernel launches) and keep the fastest for later
        renders (sstmc_scene_autotune); returns the chosen paths per chunk."""
        n = C.c_uint64()
        _check(self.lib.sstmc_scene_autotune(self.handle, C.c_uint32(sample_paths), C.byref(n)))
        return n.value

    def render_static(self, seed: Optional[int] = None) -> Tuple[np.ndarray, np.ndarray]:
        """``render`` with no device memory allocation: every device buffer is in
        the library's 64 MiB per-device static scratch (sstmc_render_static)."""
        return self._render(self.lib.sstmc_render_static, seed)

    def _render(self, fn, seed: Optional[int]) -> Tuple[np.ndarray, np.ndarray]:
        seed = self.prepared.struct.seed if seed is None else int(seed)
        n = self.Nl * self.Nv * self.Nt
        u = np.zeros(2 * n * self.renders, dtype=np.float64)
        it = np.zeros(self.renders, dtype=np.float64)
        code = fn(self.handle, C.c_uint64(seed), u.ctypes.data_as(C.POINTER(C.c_double)),
                  it.ctypes.data_as(C.POINTER(C.c_double)))
        if code != 0:
            detail = self.lib.sstmc_last_error_text().decode()
            raise SstmcError(code, error_string(code) + (f": {detail}" if detail else ""))
        uc = (u[0::2] + 1j * u[1::2]).reshape(self.renders, self.Nt, self.Nv, self.Nl)
        return np.transpose(uc, (3, 2, 1, 0)), it

    def stats(self) -> Dict[str, int]:
        v = [C.c_uint64() for _ in range(4)]
        _check(self.lib.sstmc_last_stats(self.handle, *[C.byref(x) for x in v]))
        return {"contributions": v[0].value, "dda_steps": v[1].value, "vertices": v[2].value, "paths": v[3].value}

    def timing(self) -> Dict[str, float]:
        ms = (C.c_double * 6)()
        n = (C.c_uint64 * 2)()
        _check(self.lib.sstmc_last_timing(self.handle, ms, n))
        return {"ms_total": ms[0], "ms_trace": ms[1], "ms_contract_ms": ms[2], "ms_contract_ss": ms[3],
                "ms_walk": ms[4], "ms_nee": ms[5], "launches": n[0], "chunks": n[1]}

    def trace_paths(self, seed: int, first_path: int, paths: int) -> Dict[str, np.ndarray]:
        """Per-path quantities of paths [first_path, first_path + paths) (parity tests)."""
        out, tr = _alloc_trace(paths, self.Nl, self.Nv, self.Nt)
        _check(self.lib.sstmc_trace_paths(self.handle, C.c_uint64(seed), C.c_uint32(first_path), C.c_uint32(paths), C.byref(tr)))
        return out

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.sstmc_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Request:
    """A submitted render: its host output buffers stay alive with this object."""

    def __init__(self, server: "Server", scene: Scene, seed: int):
        self.server, self.scene, self.seed = server, scene, seed
        n = scene.Nl * scene.Nv * scene.Nt
        self._u = np.zeros(2 * n * scene.renders, dtype=np.float64)
        self._it = np.zeros(scene.renders, dtype=np.float64)
        t = C.c_uint64()
        _check(server.lib.sstmc_submit(server.handle, scene.handle, C.c_uint64(seed),
                                       self._u.ctypes.data_as(C.POINTER(C.c_double)),
                                       self._it.ctypes.data_as(C.POINTER(C.c_double)), C.byref(t)))
        self.ticket = t.value

    def done(self) -> bool:
        d, st = C.c_int32(), C.c_int32()
        _check(self.server.lib.sstmc_poll(self.server.handle, C.c_uint64(self.ticket), C.byref(d), C.byref(st)))
        return bool(d.value)

    def wait(self, timeout: float = 600.0) -> int:
        """Status of the finished render; raises SstmcError(SSTMC_TIMEOUT) if still open."""
        st = C.c_int32()
        _check(self.server.lib.sstmc_wait(self.server.handle, C.c_uint64(self.ticket), C.c_double(timeout), C.byref(st)))
        return st.value

    def cancel(self) -> None:
        _check(self.server.lib.sstmc_cancel(self.server.handle, C.c_uint64(self.ticket)))

    def result(self, timeout: float = 600.0) -> Tuple[np.ndarray, np.ndarray]:
        _check(self.wait(timeout))
        s = self.scene
        uc = (self._u[0::2] + 1j * self._u[1::2]).reshape(s.renders, s.Nt, s.Nv, s.Nl)
        return np.transpose(uc, (3, 2, 1, 0)), self._it.copy()


class Server:
    """Continuous batching of renders over resident scenes (sstmc_server_*)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0, slots: int = 4):
        self.lib = load_library()
        h = C.c_void_p()
        _check(self.lib.sstmc_server_create(C.c_int32(device), C.c_uint64(hbm_budget_bytes), C.c_uint32(slots), C.byref(h)))
        self.handle = h

    def submit(self, scene: Scene, seed: int) -> Request:
        return Request(self, scene, seed)

    def stats(self) -> Dict[str, float]:
        p50, p99, cps, n = C.c_double(), C.c_double(), C.c_double(), C.c_uint64()
        _check(self.lib.sstmc_server_stats(self.handle, C.byref(p50), C.byref(p99), C.byref(cps), C.byref(n)))
        return {"p50_ms": p50.value, "p99_ms": p99.value, "contributions_per_s": cps.value, "completed": n.value}

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.sstmc_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _alloc_trace(paths: int, Nl: int, Nv: int, Nt: int):
    out = {
        "misses": np.zeros(paths, np.int32), "vertices": np.zeros(paths, np.int32),
        "vertex_hash": np.zeros(paths, np.uint32), "dda_steps": np.zeros(paths, np.uint32),
        "x1": np.zeros((paths, 3), np.float32), "m1": np.zeros(paths, np.int32),
        "a_ms": np.zeros((paths, Nt, Nl, 2)), "s_ms": np.zeros((paths, Nt, Nv, 2)),
        "a_ss": np.zeros((paths, Nt, Nl, 2)), "b_ss": np.zeros((paths, Nt, Nv, 2)),
    }
    tr = cf.PathTrace()
    tr.misses = out["misses"].ctypes.data_as(C.POINTER(C.c_int32))
    tr.vertices = out["vertices"].ctypes.data_as(C.POINTER(C.c_int32))
    tr.vertex_hash = out["vertex_hash"].ctypes.data_as(C.POINTER(C.c_uint32))
    tr.dda_steps = out["dda_steps"].ctypes.data_as(C.POINTER(C.c_uint32))
    tr.x1 = out["x1"].ctypes.data_as(C.POINTER(C.c_float))
    tr.m1 = out["m1"].ctypes.data_as(C.POINTER(C.c_int32))
    for k in ("a_ms", "s_ms", "a_ss", "b_ss"):
        setattr(tr, k, out[k].ctypes.data_as(C.POINTER(C.c_double)))
    return out, tr


def wavelengths(config: Dict[str, Any]) -> np.ndarray:
    """config.simulation.lambda as a vector (default [1])."""
    sim = config.get("simulation", {}) or {}
    return np.atleast_1d(np.asarray(sim.get("lambda", 1.0), dtype=np.float64)).ravel()


def _run(config: Dict[str, Any], dims: int, precision: int):
    lam = wavelengths(config)
    if lam.size <= 1:
        with Scene(config, dims, precision) as s:
            return s.render()
    # Several wavelengths (MatlabInterface.cu:1512-1545).  The reference traces
    # the paths once for all wavelengths but returns an Nl x Nv x Nt x R array
    # (MatlabInterface.cu:1731-1738) for device buffers of Nl x Nv x Nw x Nt, so
    # Nw > 1 overruns its output.  Here every wavelength renders the same paths
    # (they are keyed by seed and path id, not by the wavelength) and u has the
    # device layout's wavelength axis: (Nl, Nv, Nw, Nt, R).
    us, it = [], None
    for w in lam:
        c = dict(config)
        c["simulation"] = dict(config.get("simulation", {}) or {})
        c["simulation"]["lambda"] = float(w)
        with Scene(c, dims, precision) as s:
            u, it = s.render()
        us.append(u)
    return np.stack(us, axis=2), it


def sstmc2D(config: Dict[str, Any], precision: int = cf.PRECISION_SPLIT):
    """[u, iter] = sstmc2D(config); u is (Nl, Nv, Nt, R), or (Nl, Nv, Nw, Nt, R)
    for a vector of wavelengths."""
    return _run(config, 2, precision)


def sstmc3D(config: Dict[str, Any], precision: int = cf.PRECISION_SPLIT):
    """[u, iter] = sstmc3D(config); u is (Nl, Nv, Nt, R), or (Nl, Nv, Nw, Nt, R)
    for a vector of wavelengths."""
    return _run(config, 3, precision)
