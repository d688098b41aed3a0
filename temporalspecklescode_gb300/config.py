"""MATLAB-style config dict -> ``sstmc_config`` (the C-ABI struct of include/sstmc.h).

The dict mirrors the struct that the reference's MEX functions take,
``[u, iter] = sstmc2D(config)`` / ``sstmc3D(config)`` (README.md:74-373,
MatlabInterface.cu:712-1672):

    config['simulation']   batchSize, fullIteration, renderingsNum, lambda, seed, deviceNumber
    config['scattering']   type (list of 'Isotropic' / 'HG' / 'HenyeyGreenstein' / 'Tabular' / 'vMF' /
                           'VonMisesFisher'), amplitudeFunction (list: g for HG, a complex vector for
                           Tabular, a dict with mixtureMu / mixtureC / mixtureAlpha for vMF)
    config['medium']       type 'Heterogeneous' (xAxis, yAxis, zAxis, materialGrid, sigs, siga)
                           or 'Homogeneous' (boxMin, boxMax, sigs)
    config['illumination'] / ['view'] / ['illumination2'] / ['view2']
                           type 'FarField' (direction.x/y/z) or 'PointSource' (location.x/y/z, isAreaSource)
    config['sampler']      type 'TemporalSampler' / 'TemporalCorrelationSampler', t, D, U.x/y/z,
                           isTemporalAmplitude, isForcedInsideBin
    config['tracer']       type 'nee', isCBS

``materialGrid`` is indexed (x, y[, z]) like the MATLAB array and is flattened
x-fastest (MATLAB column order, HeterogeneousMedium.cuh:260-267).
"""
from __future__ import annotations

import ctypes as C
from typing import Any, Dict

import numpy as np

# Error codes (Simulation.cuh:111-162 numeric values; >= 100 new)
NO_ERROR = 0
DEVICE_ERROR = 1
ALLOCATION_ERROR = 2
KERNEL_ERROR = 3
CUBLAS_ERROR = 4
NOT_SUPPORTED = 5
MISC_ERROR = 6
INVALID_CONFIG = 100
TIMEOUT = 101
CANCELLED = 102
INVALID_HANDLE = 103
PATH_LIMIT = 104

SCATTERING_ISOTROPIC = 1
SCATTERING_TABULAR = 2
SCATTERING_HG = 3
SCATTERING_VMF = 4
MEDIUM_HETEROGENEOUS = 0
MEDIUM_HOMOGENEOUS = 1
SOURCE_NONE = 0
SOURCE_POINT = 1
SOURCE_FARFIELD = 2
SOURCE_GAUSSIANBEAM = 3
SAMPLER_TEMPORAL = 0
SAMPLER_CORRELATION = 1
PRECISION_SPLIT = 0
PRECISION_FP32 = 1

_dp = C.POINTER(C.c_double)


class SourceCfg(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("count", C.c_uint32),
        ("xyz", _dp),
        ("is_area_source", C.c_int32),
        ("focal_direction", _dp),
        ("aperture", C.c_double),
    ]


class SstmcConfig(C.Structure):
    _fields_ = [
        ("dims", C.c_uint32),
        ("batch_size", C.c_uint32),
        ("full_iteration", C.c_uint32),
        ("renderings_num", C.c_uint32),
        ("lam", C.c_double),
        ("seed", C.c_uint64),
        ("device_number", C.c_int32),
        ("scattering_num", C.c_uint32),
        ("scattering_type", C.POINTER(C.c_int32)),
        ("scattering_g", _dp),
        ("medium_type", C.c_int32),
        ("x_axis", _dp), ("x_axis_size", C.c_uint32),
        ("y_axis", _dp), ("y_axis_size", C.c_uint32),
        ("z_axis", _dp), ("z_axis_size", C.c_uint32),
        ("material_grid", C.POINTER(C.c_uint32)),
        ("sigs", _dp),
        ("siga", _dp),
        ("box_min", C.c_double * 3),
        ("box_max", C.c_double * 3),
        ("homogeneous_sigs", C.c_double),
        ("illumination", SourceCfg),
        ("view", SourceCfg),
        ("illumination2", SourceCfg),
        ("view2", SourceCfg),
        ("sampler_type", C.c_int32),
        ("t", _dp), ("t_num", C.c_uint32),
        ("D", _dp),
        ("U", _dp),
        ("is_temporal_amplitude", C.c_int32),
        ("is_forced_inside_bin", C.c_int32),
        ("is_cbs", C.c_int32),
        ("precision", C.c_int32),
        ("tabular_n", C.POINTER(C.c_uint32)),
        ("tabular_f", C.POINTER(C.c_double)),
        ("vmf_n", C.POINTER(C.c_uint32)),
        ("vmf_mu", C.POINTER(C.c_double)),
        ("vmf_c", C.POINTER(C.c_double)),
        ("vmf_alpha", C.POINTER(C.c_double)),
    ]


class PathTrace(C.Structure):
    _fields_ = [
        ("misses", C.POINTER(C.c_int32)),
        ("vertices", C.POINTER(C.c_int32)),
        ("vertex_hash", C.POINTER(C.c_uint32)),
        ("dda_steps", C.POINTER(C.c_uint32)),
        ("x1", C.POINTER(C.c_float)),
        ("m1", C.POINTER(C.c_int32)),
        ("a_ms", _dp),
        ("s_ms", _dp),
        ("a_ss", _dp),
        ("b_ss", _dp),
    ]


class ConfigError(ValueError):
    """Raised for configs the MEX layer would reject (MatlabInterface.cu mexErrMsgIdAndTxt)."""


def _arr(x, dtype=np.float64) -> np.ndarray:
    a = np.ascontiguousarray(np.atleast_1d(np.asarray(x, dtype=dtype)).ravel())
    return a


def _vec3(d: Dict[str, Any], n_expected: int | None, dims: int, name: str) -> np.ndarray:
    xs = _arr(d["x"])
    ys = _arr(d["y"])
    zs = _arr(d.get("z", np.zeros_like(xs))) if dims == 3 else np.zeros_like(xs)
    if dims == 3 and "z" not in d:
        raise ConfigError(f"{name} must have field z")
    if not (len(xs) == len(ys) == len(zs)):
        raise ConfigError(f"{name} x, y, z must have the same number of elements")
    if len(xs) == 0:   # the MEX layer's array readers require at least one element
        raise ConfigError(f"{name} must have at least one element")
    if n_expected is not None and len(xs) != n_expected:
        raise ConfigError(f"{name} must have {n_expected} elements")
    return np.ascontiguousarray(np.stack([xs, ys, zs], axis=1).reshape(-1))


class PreparedConfig:
    """An ``SstmcConfig`` plus the numpy arrays its pointers refer to."""

    def __init__(self, struct: SstmcConfig, keep: list, meta: Dict[str, Any]):
        self.struct = struct
        self._keep = keep
        self.meta = meta

    def ptr(self):
        return C.byref(self.struct)


def _source(cfg: Dict[str, Any], name: str, dims: int, keep: list, required: bool) -> SourceCfg:
    s = SourceCfg()
    block = cfg.get(name)
    if block is None:
        if required:
            raise ConfigError(f"config must have field {name}")
        s.type = SOURCE_NONE
        return s
    ty = block.get("type")
    if ty == "FarField":
        xyz = _vec3(block["direction"], None, dims, f"{name}.direction")
        s.type = SOURCE_FARFIELD
    elif ty == "PointSource":
        xyz = _vec3(block["location"], None, dims, f"{name}.location")
        s.type = SOURCE_POINT
        s.is_area_source = 1 if block.get("isAreaSource", False) else 0
    elif ty == "GaussianBeam":
        # focalPoint, focalDirection (one per focal point) and a scalar aperture
        # (MatlabInterface.cu:1161-1200)
        if "focalPoint" not in block or "focalDirection" not in block or "aperture" not in block:
            raise ConfigError(f"{name}: GaussianBeam needs focalPoint, focalDirection and aperture")
        xyz = _vec3(block["focalPoint"], None, dims, f"{name}.focalPoint")
        fd = _vec3(block["focalDirection"], len(xyz) // 3, dims, f"{name}.focalDirection")
        ap = _arr(block["aperture"])
        if ap.size != 1:
            raise ConfigError(f"{name}.aperture must be a scalar")
        keep.append(fd)
        s.type = SOURCE_GAUSSIANBEAM
        s.focal_direction = fd.ctypes.data_as(_dp)
        s.aperture = float(ap[0])
    else:
        raise ConfigError(f"Unsupported source type {ty!r}. Available {name} types are PointSource, FarField and GaussianBeam.")
    keep.append(xyz)
    s.count = len(xyz) // 3
    s.xyz = xyz.ctypes.data_as(_dp)
    return s


def _amplitude_cells(raw: Any, types: list) -> list:
    """scattering.amplitudeFunction as one entry per material: a scalar g (HG),
    a vector of complex values (Tabular) or anything (Isotropic).  MATLAB passes
    a cell array; a .mat reader gives a list, and a one-material cell may arrive
    as the bare value."""
    if isinstance(raw, (list, tuple)):
        cells = list(raw)
    elif isinstance(raw, np.ndarray) and raw.dtype == object:
        cells = list(raw.ravel())
    elif len(types) == 1:
        cells = [raw]
    else:
        cells = list(np.atleast_1d(np.asarray(raw)).ravel())
    if len(cells) < len(types):
        cells += [0.0] * (len(types) - len(cells))
    return cells


def prepare(config: Dict[str, Any], dims: int, precision: int = PRECISION_SPLIT) -> PreparedConfig:
    """Convert a MATLAB-style config dict into the C-ABI struct."""
    if dims not in (2, 3):
        raise ConfigError("dims must be 2 or 3")
    keep: list = []
    c = SstmcConfig()
    c.dims = dims
    sim = config.get("simulation", {}) or {}
    c.batch_size = int(sim.get("batchSize", 1024))
    c.full_iteration = int(sim.get("fullIteration", 1))
    c.renderings_num = int(sim.get("renderingsNum", 1))
    if c.batch_size <= 0 or c.full_iteration <= 0 or c.renderings_num <= 0:
        raise ConfigError("batchSize, fullIteration and renderingsNum must be positive")
    lam = _arr(sim.get("lambda", 1.0))
    if lam.size != 1:
        raise ConfigError("a scene has one wavelength; sstmc2D / sstmc3D render a lambda vector one wavelength at a time")
    c.lam = float(lam[0])
    c.seed = int(abs(sim.get("seed", 0)))
    c.device_number = int(sim.get("deviceNumber", 0))

    sc = config.get("scattering")
    if sc is None:
        raise ConfigError("config must have field scattering")
    types = sc["type"]
    if isinstance(types, str):
        types = [types]
    else:   # a list, or a MATLAB cell array read from a .mat file (object array)
        types = [str(t) for t in np.atleast_1d(np.asarray(types, dtype=object))]
    amps = _amplitude_cells(sc.get("amplitudeFunction", [0.0] * len(types)), types)
    st = np.zeros(len(types), dtype=np.int32)
    sg = np.zeros(len(types), dtype=np.float64)
    tn = np.zeros(len(types), dtype=np.uint32)
    vn = np.zeros(len(types), dtype=np.uint32)
    tabs = []
    vmfs = []
    for i, t in enumerate(types):
        if t == "Isotropic":
            st[i] = SCATTERING_ISOTROPIC
        elif t in ("HG", "HenyeyGreenstein"):
            st[i] = SCATTERING_HG
            sg[i] = float(np.asarray(amps[i]).ravel()[0])
        elif t == "Tabular":
            st[i] = SCATTERING_TABULAR
            f = np.asarray(amps[i], dtype=np.complex128).ravel()
            if f.size < 2 or not np.all(np.isfinite(f)):
                raise ConfigError(f"scattering.amplitudeFunction of tabular material {i} must be >= 2 finite values")
            tn[i] = f.size
            tabs.append(f)
        elif t in ("vMF", "VonMisesFisher"):
            # a struct with mixtureMu, mixtureC, mixtureAlpha (MatlabInterface.cu:827-868)
            st[i] = SCATTERING_VMF
            cell = amps[i]
            if not isinstance(cell, dict) or not all(k in cell for k in ("mixtureMu", "mixtureC", "mixtureAlpha")):
                raise ConfigError(f"scattering.amplitudeFunction of vMF material {i} must be a struct with "
                                  "mixtureMu, mixtureC and mixtureAlpha")
            mu, cc, al = (np.asarray(cell[k], dtype=np.float64).ravel() for k in ("mixtureMu", "mixtureC", "mixtureAlpha"))
            if mu.size < 1 or cc.size != mu.size or al.size != mu.size:
                raise ConfigError(f"vMF material {i}: mixtureMu, mixtureC and mixtureAlpha must have the same length >= 1")
            if not (np.all(np.isfinite(mu)) and np.all(np.isfinite(cc)) and np.all(np.isfinite(al))
                    and np.all(al >= 0) and np.any(al > 0)):
                raise ConfigError(f"vMF material {i}: finite values and mixtureAlpha >= 0 (not all 0) required")
            vn[i] = mu.size
            vmfs.append((mu, cc, al))
        else:
            raise ConfigError(f"Unsupported scattering type in material {i}: {t}")
    keep += [st, sg]
    if tabs:
        tf = np.ascontiguousarray(np.concatenate(tabs).view(np.float64))   # (re, im) pairs
        keep += [tn, tf]
        c.tabular_n = tn.ctypes.data_as(C.POINTER(C.c_uint32))
        c.tabular_f = tf.ctypes.data_as(_dp)
    if vmfs:
        vmu, vc, val = (np.ascontiguousarray(np.concatenate([v[j] for v in vmfs])) for j in range(3))
        keep += [vn, vmu, vc, val]
        c.vmf_n = vn.ctypes.data_as(C.POINTER(C.c_uint32))
        c.vmf_mu = vmu.ctypes.data_as(_dp)
        c.vmf_c = vc.ctypes.data_as(_dp)
        c.vmf_alpha = val.ctypes.data_as(_dp)
    c.scattering_num = len(types)
    c.scattering_type = st.ctypes.data_as(C.POINTER(C.c_int32))
    c.scattering_g = sg.ctypes.data_as(_dp)
    mat_num = len(types) if len(types) > 1 else 2

    med = config.get("medium")
    if med is None:
        raise ConfigError("config must have field medium")
    if med.get("type") == "Heterogeneous":
        c.medium_type = MEDIUM_HETEROGENEOUS
        axes = []
        for key in ("xAxis", "yAxis", "zAxis")[:dims]:
            a = _arr(med[key])
            if a.size < 2:
                raise ConfigError(f"medium.{key} must have at least 2 elements")
            axes.append(a)
        keep += axes
        c.x_axis, c.x_axis_size = axes[0].ctypes.data_as(_dp), axes[0].size
        c.y_axis, c.y_axis_size = axes[1].ctypes.data_as(_dp), axes[1].size
        if dims == 3:
            c.z_axis, c.z_axis_size = axes[2].ctypes.data_as(_dp), axes[2].size
        shape = tuple(a.size - 1 for a in axes)
        grid = np.asarray(med["materialGrid"])
        if grid.size != int(np.prod(shape)):
            raise ConfigError(f"medium.materialGrid must have {int(np.prod(shape))} elements")
        grid = np.ascontiguousarray(np.reshape(grid, shape, order="F").ravel(order="F").astype(np.uint32))
        keep.append(grid)
        c.material_grid = grid.ctypes.data_as(C.POINTER(C.c_uint32))
        sigs = _arr(med["sigs"])
        if sigs.size != mat_num:
            raise ConfigError(f"medium.sigs must have {mat_num} elements")
        keep.append(sigs)
        c.sigs = sigs.ctypes.data_as(_dp)
        if "siga" in med and med["siga"] is not None:
            siga = _arr(med["siga"])
            if siga.size != mat_num:
                raise ConfigError(f"medium.siga must have {mat_num} elements")
            keep.append(siga)
            c.siga = siga.ctypes.data_as(_dp)
    elif med.get("type") == "Homogeneous":
        c.medium_type = MEDIUM_HOMOGENEOUS
        bmin = _vec3(med["boxMin"], 1, dims, "medium.boxMin")
        bmax = _vec3(med["boxMax"], 1, dims, "medium.boxMax")
        for i in range(3):
            c.box_min[i] = bmin[i]
            c.box_max[i] = bmax[i]
        c.homogeneous_sigs = float(np.asarray(med["sigs"]).ravel()[0])
    else:
        raise ConfigError("Unsupported medium type. Available medium types are Homogeneous and Heterogeneous")

    c.illumination = _source(config, "illumination", dims, keep, True)
    c.view = _source(config, "view", dims, keep, True)
    c.illumination2 = _source(config, "illumination2", dims, keep, False)
    c.view2 = _source(config, "view2", dims, keep, False)

    smp = config.get("sampler")
    if smp is None:
        raise ConfigError("config must have field sampler")
    if smp["type"] == "TemporalSampler":
        c.sampler_type = SAMPLER_TEMPORAL
    elif smp["type"] == "TemporalCorrelationSampler":
        c.sampler_type = SAMPLER_CORRELATION
    else:
        raise ConfigError("Unsupported sapmler type. Available sampler types are TemporalSampler and TemporalCorrelationSampler")
    t = _arr(smp["t"])
    if t.size == 0:
        raise ConfigError("sampler.t must have at least one element")
    D = _arr(smp["D"])
    if D.size != mat_num:
        raise ConfigError(f"sampler.D must have {mat_num} elements")
    if np.any(D < 0):
        raise ConfigError("D values in temporal sampler must be non-negative")
    U = _vec3(smp["U"], mat_num, dims, "sampler.U")
    keep += [t, D, U]
    c.t, c.t_num = t.ctypes.data_as(_dp), t.size
    c.D = D.ctypes.data_as(_dp)
    c.U = U.ctypes.data_as(_dp)
    c.is_temporal_amplitude = 1 if smp.get("isTemporalAmplitude", True) else 0
    c.is_forced_inside_bin = 1 if smp.get("isForcedInsideBin", False) else 0

    tr = config.get("tracer")
    if tr is None:
        raise ConfigError("Input must have field named tracer.")
    if tr.get("type") != "nee":
        raise ConfigError(f"Unsupported tracer type. Type entered: {tr.get('type')}. Available tracer type is nee")
    c.is_cbs = 1 if tr.get("isCBS", False) else 0
    c.precision = int(precision)

    nl = c.illumination.count
    nv = c.view.count
    meta = dict(Nl=nl, Nv=nv, Nt=int(t.size), R=c.renderings_num, P=c.batch_size,
                waves=c.full_iteration, dims=dims, correlation=c.sampler_type == SAMPLER_CORRELATION)
    return PreparedConfig(c, keep, meta)
