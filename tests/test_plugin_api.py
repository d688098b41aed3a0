"""The reference's object model through the C-ABI (sstmc_simulation_* ..
sstmc_tracer_*) and the C++ header over it (include/sstmc.hpp).

CPU: a scene built object by object -- Simulation, Scattering and its
per-material setters, Medium + setMaterial, the sources with their connection
types, the sampler + setMaterial (MatlabInterface.cu:1677-1700) -- describes
the same sstmc_config as the MATLAB-style config dict does, field by field;
the setters refuse what the MEX layer refuses; the C++ header compiles.
GPU: the NextEventEstimation tracer of such a build renders what sstmc_render
renders for the config (the same paths: iteration counts and vertex counts
exact, fields to FP64 accumulation order), and a C++ program written against
the header does too.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from temporalspecklescode_gb300 import config as cf
from temporalspecklescode_gb300 import workloads as wl
from tests import scenes
from tests.plugin_builder import ObjectScene

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SCENES = scenes.small_scenes()
NAMES = ["speckle_2d", "correlation_3d", "transmission_matrix_3d", "field_point_3d", "corr_far_2d_drift",
         "homogeneous_3d", "tabular_corr_2d", "vmf_corr_3d", "forced_bin_3d", "reciprocal_far_3d_cbs", "gauss_3d_moving"]


@pytest.fixture(scope="module")
def lib():
    from temporalspecklescode_gb300 import _build, api
    if not os.path.exists(_build.lib_path()):
        _build.build_library()
    return api.load_library()


def _arrays(c: cf.SstmcConfig):
    """Every value a config describes, with its arrays read through their lengths."""
    dims = c.dims
    mat_num = c.scattering_num if c.scattering_num > 1 else 2
    out = {k: getattr(c, k) for k in ("dims", "batch_size", "full_iteration", "lam", "seed", "device_number",
                                      "scattering_num", "medium_type", "sampler_type", "t_num", "is_temporal_amplitude",
                                      "is_forced_inside_bin", "is_cbs", "precision", "homogeneous_sigs")}
    rd = lambda p, n: np.ctypeslib.as_array(p, shape=(n,)).copy() if n and p else np.zeros(0)
    out["scattering_type"] = rd(c.scattering_type, c.scattering_num)
    out["scattering_g"] = rd(c.scattering_g, c.scattering_num)
    out["box"] = np.array(list(c.box_min) + list(c.box_max))
    if c.medium_type == cf.MEDIUM_HETEROGENEOUS:
        out["x"] = rd(c.x_axis, c.x_axis_size)
        out["y"] = rd(c.y_axis, c.y_axis_size)
        out["z"] = rd(c.z_axis, c.z_axis_size) if dims == 3 else np.zeros(0)
        cells = (c.x_axis_size - 1) * (c.y_axis_size - 1) * ((c.z_axis_size - 1) if dims == 3 else 1)
        out["grid"] = rd(c.material_grid, cells)
        out["sigs"] = rd(c.sigs, mat_num)
        out["siga"] = rd(c.siga, mat_num) if c.siga else np.zeros(mat_num)   # absent siga reads as zeros
    for role in ("illumination", "view", "illumination2", "view2"):
        s = getattr(c, role)
        out[role] = (s.type, s.count, s.is_area_source, tuple(rd(s.xyz, 3 * s.count)) if s.type else ())
        if s.type == cf.SOURCE_GAUSSIANBEAM:
            out[role] += (tuple(rd(s.focal_direction, 3 * s.count)), s.aperture)
    out["t"] = rd(c.t, c.t_num)
    out["D"] = rd(c.D, mat_num)
    out["U"] = rd(c.U, 3 * mat_num)
    if c.tabular_n:
        n = rd(c.tabular_n, c.scattering_num)
        out["tabular_n"] = n
        out["tabular_f"] = rd(c.tabular_f, 2 * int(n.sum()))
    if c.vmf_n:
        n = rd(c.vmf_n, c.scattering_num)
        out["vmf_n"] = n
        for k in ("vmf_mu", "vmf_c", "vmf_alpha"):
            out[k] = rd(getattr(c, k), int(n.sum()))
    return out


def _same(a, b):
    assert a.keys() == b.keys(), set(a) ^ set(b)
    for k in a:
        if isinstance(a[k], np.ndarray):
            assert np.array_equal(a[k], b[k]), k
        else:
            assert a[k] == b[k], (k, a[k], b[k])


@pytest.mark.parametrize("name", NAMES)
def test_object_build_describes_the_config(name, lib):
    cfg, dims = SCENES[name]
    pc = cf.prepare(cfg, dims)
    with ObjectScene(lib, cfg, dims) as obj:
        got = _arrays(obj.config())
    _same(got, _arrays(pc.struct))


def test_sampler_queries(lib):
    cfg, dims = SCENES["corr_far_2d_drift"]
    with ObjectScene(lib, cfg, dims) as obj:
        nl, nv, nt = C.c_uint32(), C.c_uint32(), C.c_uint32()
        assert lib.sstmc_sampler_shape(obj.sampler, C.byref(nl), C.byref(nv), C.byref(nt)) == 0
        m = cf.prepare(cfg, dims).meta
        assert (nl.value, nv.value, nt.value) == (m["Nl"], m["Nv"], m["Nt"])
        corr = C.c_int32()
        assert lib.sstmc_sampler_is_correlation(obj.sampler, C.byref(corr)) == 0 and corr.value == 1
        n = C.c_uint32()
        assert lib.sstmc_source_size(obj.src["view2"], C.byref(n)) == 0 and n.value == len(np.ravel(cfg["view2"]["direction"]["x"]))


def test_setters_refuse_what_the_mex_layer_refuses(lib):
    vp = C.c_void_p
    sim, sc, med, il, vw, smp = vp(), vp(), vp(), vp(), vp(), vp()
    assert lib.sstmc_simulation_create(4, 64, 1.0, 0, 0, C.byref(sim)) == cf.INVALID_CONFIG      # dims
    assert lib.sstmc_simulation_create(3, 0, 1.0, 0, 0, C.byref(sim)) == cf.INVALID_CONFIG       # batch
    assert lib.sstmc_simulation_create(3, 64, 1.0, 0, 0, C.byref(sim)) == 0
    assert lib.sstmc_scattering_create(C.byref(sc)) == 0
    assert lib.sstmc_scattering_set_henyey_greenstein(sc, 1.0, 1) == cf.INVALID_CONFIG           # |g| < 1
    assert lib.sstmc_scattering_set_isotropic(sc, 10) == cf.INVALID_CONFIG                       # MATERIAL_NUM
    assert lib.sstmc_scattering_set_henyey_greenstein(sc, 0.5, 0) == 0
    x = np.array([-1.0, 1.0]); g = np.ones(1, dtype=np.uint32)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    assert lib.sstmc_medium_create_heterogeneous(g.ctypes.data_as(C.POINTER(C.c_uint32)), dp(x), 2, dp(x), 2, dp(x), 2,
                                                 C.byref(med)) == 0
    assert lib.sstmc_medium_set_material(med, -1.0, 0.0, 1) == cf.INVALID_CONFIG                 # sigs >= 0
    for m in (0, 1):
        assert lib.sstmc_medium_set_material(med, 1.0, 0.0, m) == 0
    p = np.array([0.0, 0.0, -2.0])
    assert lib.sstmc_source_create_point(sim, 5, dp(p), 1, 0, C.byref(il)) == cf.INVALID_CONFIG  # connection type
    assert lib.sstmc_source_create_point(sim, 0, dp(p), 1, 0, C.byref(il)) == 0
    assert lib.sstmc_source_create_point(sim, 0, dp(p), 1, 0, C.byref(vw)) == 0                  # an illumination ...
    t = np.zeros(1)
    assert lib.sstmc_sampler_create_temporal(sim, med, sc, il, vw, dp(t), 1, 1, 0, C.byref(smp)) == cf.INVALID_CONFIG  # ... as view
    assert lib.sstmc_source_destroy(vw) == 0
    assert lib.sstmc_source_create_point(sim, 1, dp(p), 1, 0, C.byref(vw)) == 0
    assert lib.sstmc_sampler_create_temporal(sim, med, sc, il, vw, dp(t), 0, 1, 0, C.byref(smp)) == cf.INVALID_CONFIG  # t empty
    assert lib.sstmc_sampler_create_temporal(sim, med, sc, il, vw, dp(t), 1, 1, 0, C.byref(smp)) == 0
    u = np.zeros(3)
    assert lib.sstmc_sampler_set_material(smp, -1e-3, dp(u), 1) == cf.INVALID_CONFIG             # D >= 0
    assert "non-negative" in lib.sstmc_last_error_text().decode()
    for h, f in ((smp, lib.sstmc_sampler_destroy), (vw, lib.sstmc_source_destroy), (il, lib.sstmc_source_destroy),
                 (med, lib.sstmc_medium_destroy), (sc, lib.sstmc_scattering_destroy), (sim, lib.sstmc_simulation_destroy)):
        assert f(h) == 0


def test_cpp_header_compiles():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    r = subprocess.run([gxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), "-fsyntax-only",
                        os.path.join(ROOT, "tests", "cpp", "object_by_object.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def _tracer_render(lib, cfg, dims, seed):
    with ObjectScene(lib, cfg, dims) as obj:
        tr = obj.tracer()
        m = cf.prepare(cfg, dims).meta
        v = np.zeros(2 * m["Nl"] * m["Nv"] * m["Nt"])
        assert lib.sstmc_tracer_update_seed(tr, seed) == 0
        assert lib.sstmc_tracer_trace(tr, v.ctypes.data_as(C.POINTER(C.c_double))) == 0, lib.sstmc_last_error_text()
        z, b, cbs = C.c_uint64(), C.c_uint64(), C.c_int32()
        lib.sstmc_tracer_zero_contribution_paths(tr, C.byref(z))
        lib.sstmc_tracer_photons_budget(tr, C.byref(b))
        lib.sstmc_tracer_is_cbs(tr, C.byref(cbs))
    u = (v[0::2] + 1j * v[1::2]).reshape(m["Nt"], m["Nv"], m["Nl"]).transpose(2, 1, 0)
    return u, m["P"] * m["waves"] + z.value, b.value, cbs.value


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_tracer_renders_the_config(name, lib):
    from temporalspecklescode_gb300 import api
    cfg, dims = SCENES[name]
    u, it, budget, cbs = _tracer_render(lib, cfg, dims, 41)
    with api.Scene(cfg, dims) as s:
        ur, itr = s.render(seed=41)
        st = s.stats()
    assert it == itr[0]
    assert budget == st["vertices"]
    assert cbs == (1 if cfg["tracer"].get("isCBS", False) else 0)
    assert np.linalg.norm(u - ur[..., 0]) <= 1e-12 * np.linalg.norm(ur)


def _cpp_scene():
    """The scene tests/cpp/object_by_object.cpp builds, as a config dict."""
    grid = np.zeros((4, 3, 2), dtype=np.uint32)
    for k in range(2):
        for j in range(3):
            for i in range(4):
                grid[i, j, k] = 1 + (i + j + k) % 2
    cfg = {
        "simulation": {"batchSize": 64, "fullIteration": 2, "renderingsNum": 2, "lambda": 0.75, "seed": 5},
        "scattering": {"type": ["Isotropic", "HG", "HG"], "amplitudeFunction": [0.0, 0.5, 0.7]},
        "medium": {"type": "Heterogeneous", "xAxis": [-8.0, -4.0, 0.0, 4.0, 8.0], "yAxis": [-6.0, -2.0, 2.0, 6.0],
                   "zAxis": [0.0, 2.0, 4.0], "materialGrid": grid, "sigs": [0.0, 0.5, 1.0], "siga": [0.0, 0.01, 0.02]},
        "illumination": {"type": "PointSource", "location": {"x": [-3.0, 0.0, 2.5], "y": [1.0, 0.0, -1.5], "z": [-1.0, -1.0, -1.0]}},
        "view": {"type": "FarField", "direction": {"x": [0.6, 0.0], "y": [0.0, 0.6], "z": [0.8, 0.8]}},
        "sampler": {"type": "TemporalSampler", "t": [0.0, 1.0, 2.5], "D": [0.0, 2e-3, 5e-3],
                    "U": {"x": [0.0, 0.01, 0.0], "y": [0.0, 0.0, 0.02], "z": [0.0, 0.0, 0.0]}},
        "tracer": {"type": "nee"},
    }
    return cfg, 3


@pytest.mark.gpu
def test_cpp_program_renders_the_config(lib, tmp_path):
    """A C++ program against include/sstmc.hpp, linked to the library, renders
    two renderings with updateSeed between them; the same config through
    sstmc_render (renderingsNum = 2, seed, seed + 1) gives the same result."""
    from temporalspecklescode_gb300 import _build, api
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "object_by_object")
    libdir = os.path.dirname(_build.lib_path())
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "object_by_object.cpp"), "-L", libdir, "-lsstmc_gb300",
                        f"-Wl,-rpath,{libdir}", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = str(tmp_path / "u.bin")
    r = subprocess.run([exe, out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stderr)
    vals = np.fromfile(out, dtype=np.float64)
    cfg, dims = _cpp_scene()
    with api.Scene(cfg, dims) as s:
        ur, itr = s.render(seed=5)
        st_last = s.stats()
    n = 2 * 3 * 2 * 3
    assert vals.size == 2 * (n + 2)
    for rr in range(2):
        blk = vals[rr * (n + 2):(rr + 1) * (n + 2)]
        u = (blk[0:n:2] + 1j * blk[1:n:2]).reshape(3, 2, 3).transpose(2, 1, 0)
        assert blk[n] == itr[rr]
        assert np.linalg.norm(u - ur[..., rr]) <= 1e-12 * np.linalg.norm(ur[..., rr])
    assert vals[-1] == st_last["vertices"]
