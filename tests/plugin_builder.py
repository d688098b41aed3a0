"""Build a scene object by object through the C-ABI's plugin setters
(sstmc_simulation_* .. sstmc_tracer_*), in the order mexFunction builds the
reference's objects (MatlabInterface.cu:1677-1700), from the same MATLAB-style
config dict that config.prepare turns into one sstmc_config."""
from __future__ import annotations

import ctypes as C

import numpy as np

from temporalspecklescode_gb300 import config as cf

CONNECTION = {"illumination": 0, "view": 1, "illumination2": 2, "view2": 3}


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class ObjectScene:
    """Simulation, Scattering, Medium, Sources and Sampler handles of one
    config; `tracer()` creates the NextEventEstimation tracer (device scene)."""

    def __init__(self, lib, config: dict, dims: int, precision: int = cf.PRECISION_SPLIT):
        self.lib = lib
        self.keep = []
        self.handles = []   # (destroy function, handle) in creation order
        L = lib
        sim = config["simulation"]
        self.full_iteration = int(sim.get("fullIteration", 1))
        self.seed = int(sim.get("seed", 0))
        self.is_cbs = 1 if config["tracer"].get("isCBS", False) else 0
        self.sim = self._make(L.sstmc_simulation_create, L.sstmc_simulation_destroy, C.c_uint32(dims),
                              C.c_uint32(int(sim.get("batchSize", 1024))), C.c_double(float(np.ravel(sim.get("lambda", 1.0))[0])),
                              C.c_int32(int(sim.get("deviceNumber", 0))), C.c_int32(precision))
        # scattering, one setter per material
        sc = config["scattering"]
        types = [sc["type"]] if isinstance(sc["type"], str) else list(sc["type"])
        amps = cf._amplitude_cells(sc.get("amplitudeFunction", [0.0] * len(types)), types)
        self.scattering = self._make(L.sstmc_scattering_create, L.sstmc_scattering_destroy)
        for m, t in enumerate(types):
            if t == "Isotropic":
                self._ok(L.sstmc_scattering_set_isotropic(self.scattering, m))
            elif t in ("HG", "HenyeyGreenstein"):
                self._ok(L.sstmc_scattering_set_henyey_greenstein(self.scattering, float(np.ravel(amps[m])[0]), m))
            elif t == "Tabular":
                f = np.ascontiguousarray(np.asarray(amps[m], dtype=np.complex128).ravel().view(np.float64))
                self.keep.append(f)
                self._ok(L.sstmc_scattering_set_tabular(self.scattering, _dp(f), f.size // 2, m))
            elif t in ("vMF", "VonMisesFisher"):
                mu, c, al = (np.ascontiguousarray(np.asarray(amps[m][k], dtype=np.float64).ravel())
                             for k in ("mixtureMu", "mixtureC", "mixtureAlpha"))
                self.keep += [mu, c, al]
                self._ok(L.sstmc_scattering_set_von_mises_fisher(self.scattering, _dp(mu), _dp(c), _dp(al), mu.size, m))
            else:
                raise ValueError(t)
        mat_num = len(types) if len(types) > 1 else 2
        # medium
        med = config["medium"]
        if med["type"] == "Heterogeneous":
            axes = [np.ascontiguousarray(np.asarray(med[k], dtype=np.float64).ravel()) for k in ("xAxis", "yAxis", "zAxis")[:dims]]
            shape = tuple(a.size - 1 for a in axes)
            grid = np.ascontiguousarray(np.reshape(np.asarray(med["materialGrid"]), shape, order="F").ravel(order="F").astype(np.uint32))
            self.keep += axes + [grid]
            z = _dp(axes[2]) if dims == 3 else None
            nz = axes[2].size if dims == 3 else 0
            self.medium = self._make(L.sstmc_medium_create_heterogeneous, L.sstmc_medium_destroy,
                                     grid.ctypes.data_as(C.POINTER(C.c_uint32)), _dp(axes[0]), axes[0].size,
                                     _dp(axes[1]), axes[1].size, z, nz)
            sigs = np.ravel(med["sigs"]).astype(float)
            siga = np.ravel(med["siga"]).astype(float) if med.get("siga") is not None else np.zeros(mat_num)
            for m in range(mat_num):
                self._ok(L.sstmc_medium_set_material(self.medium, float(sigs[m]), float(siga[m]), m))
        else:
            bmin = np.array([np.ravel(med["boxMin"][k])[0] if k in med["boxMin"] else 0.0 for k in "xyz"], dtype=np.float64)
            bmax = np.array([np.ravel(med["boxMax"][k])[0] if k in med["boxMax"] else 0.0 for k in "xyz"], dtype=np.float64)
            self.keep += [bmin, bmax]
            self.medium = self._make(L.sstmc_medium_create_homogeneous, L.sstmc_medium_destroy, dims, _dp(bmin), _dp(bmax),
                                     float(np.ravel(med["sigs"])[0]))
        # sources
        self.src = {}
        for role in ("illumination", "view", "illumination2", "view2"):
            blk = config.get(role)
            if blk is None:
                continue
            key = {"FarField": "direction", "GaussianBeam": "focalPoint"}.get(blk["type"], "location")
            vec = lambda d: np.ascontiguousarray(np.stack([np.ravel(d["x"]), np.ravel(d["y"]),
                                                           np.ravel(d["z"]) if dims == 3 else np.zeros(np.ravel(d["x"]).size)],
                                                          axis=1).astype(np.float64).reshape(-1))
            xyz = vec(blk[key])
            self.keep.append(xyz)
            if blk["type"] == "GaussianBeam":
                fd = vec(blk["focalDirection"])
                self.keep.append(fd)
                self.src[role] = self._make(L.sstmc_source_create_gaussian_beam, L.sstmc_source_destroy, self.sim,
                                            CONNECTION[role], _dp(xyz), _dp(fd), xyz.size // 3,
                                            float(np.ravel(blk["aperture"])[0]))
            elif blk["type"] == "FarField":
                self.src[role] = self._make(L.sstmc_source_create_far_field, L.sstmc_source_destroy, self.sim,
                                            CONNECTION[role], _dp(xyz), xyz.size // 3)
            else:
                self.src[role] = self._make(L.sstmc_source_create_point, L.sstmc_source_destroy, self.sim, CONNECTION[role],
                                            _dp(xyz), xyz.size // 3, 1 if blk.get("isAreaSource", False) else 0)
        # sampler
        smp = config["sampler"]
        t = np.ascontiguousarray(np.ravel(smp["t"]).astype(np.float64))
        self.keep.append(t)
        if smp["type"] == "TemporalSampler":
            self.sampler = self._make(L.sstmc_sampler_create_temporal, L.sstmc_sampler_destroy, self.sim, self.medium,
                                      self.scattering, self.src["illumination"], self.src["view"], _dp(t), t.size,
                                      1 if smp.get("isTemporalAmplitude", True) else 0,
                                      1 if smp.get("isForcedInsideBin", False) else 0)
        else:
            self.sampler = self._make(L.sstmc_sampler_create_correlation, L.sstmc_sampler_destroy, self.sim, self.medium,
                                      self.scattering, self.src["illumination"], self.src["illumination2"],
                                      self.src["view"], self.src["view2"], _dp(t), t.size)
        D = np.ravel(smp["D"]).astype(float)
        U = smp["U"]
        for m in range(mat_num):
            u = np.array([np.ravel(U["x"])[m], np.ravel(U["y"])[m], np.ravel(U["z"])[m] if dims == 3 else 0.0], dtype=np.float64)
            self.keep.append(u)
            self._ok(L.sstmc_sampler_set_material(self.sampler, float(D[m]), _dp(u), m))

    def _ok(self, code):
        if code != 0:
            raise RuntimeError(f"sstmc error {code}: {self.lib.sstmc_last_error_text().decode()}")

    def _make(self, create, destroy, *args):
        h = C.c_void_p()
        self._ok(create(*args, C.byref(h)))
        self.handles.append((destroy, h))
        return h

    def config(self) -> cf.SstmcConfig:
        c = cf.SstmcConfig()
        self._ok(self.lib.sstmc_sampler_config(self.sampler, self.full_iteration, self.seed, self.is_cbs, C.byref(c)))
        return c

    def tracer(self):
        return self._make(self.lib.sstmc_tracer_create_nee, self.lib.sstmc_tracer_destroy, self.sampler,
                          self.full_iteration, C.c_uint64(self.seed), self.is_cbs)

    def close(self):
        for destroy, h in reversed(self.handles):
            destroy(h)
        self.handles = []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
