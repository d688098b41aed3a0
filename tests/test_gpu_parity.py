"""GPU parity: the CUDA path (through the C-ABI) against the CPU oracle on the
same seeded Philox paths.

Bit-exact: first-vertex misses, vertex counts, the hash of every vertex
position and material, and the number of voxel steps of all NEE rays.
Floating point: every per-path NEE row and the rendered field / correlation
within a relative Frobenius error of 1e-5 of the FP64 oracle (split-precision
form).
"""
import numpy as np
import pytest

from temporalspecklescode_gb300 import config as cf
from tests.scenes import small_scenes

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
SCENES = small_scenes()


def rel_fro(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope="module")
def api():
    from temporalspecklescode_gb300 import api as A
    A.load_library()
    return A


@pytest.mark.parametrize("name", sorted(SCENES))
def test_trace_rows_bit_exact(name, api, oracle):
    cfg, dims = SCENES[name]
    n = 64
    with api.Scene(cfg, dims) as s:
        g = s.trace_paths(seed=123, first_path=5, paths=n)
        pc = cf.prepare(cfg, dims)
        o = oracle.trace_paths(pc, 123, 5, n)
    for k in ("misses", "vertices", "vertex_hash", "dda_steps", "m1"):
        assert np.array_equal(g[k], o[k]), (name, k, np.nonzero(g[k] != o[k])[0][:5])
    assert np.array_equal(g["x1"], o["x1"])
    for k in ("a_ms", "s_ms", "a_ss", "b_ss"):
        err = rel_fro(g[k], o[k])
        assert err <= REL_TOL, (name, k, err)


@pytest.mark.parametrize("name", sorted(SCENES))
def test_render_matches_oracle(name, api, oracle):
    cfg, dims = SCENES[name]
    with api.Scene(cfg, dims) as s:
        u, it = s.render(seed=77)
        st = s.stats()
    pc = cf.prepare(cfg, dims)
    uo, ito, sto = oracle.render(pc, 77)
    assert it[0] == ito
    assert st["vertices"] == sto["vertices"] and st["paths"] == sto["paths"]
    assert st["dda_steps"] == sto["dda_steps"]
    assert st["contributions"] == sto["contributions"]
    err = rel_fro(u[..., 0], uo)
    assert err <= REL_TOL, (name, err)


@pytest.mark.parametrize("name", ["speckle_2d", "correlation_3d"])
def test_plain_fp32_form_runs(name, api, oracle):
    """The plain FP32 form (FP32 phase, uncompensated FP32 contraction) traces
    the same paths; its error against FP64 is reported by the benchmark."""
    cfg, dims = SCENES[name]
    with api.Scene(cfg, dims, precision=cf.PRECISION_FP32) as s:
        u, it = s.render(seed=77)
    pc = cf.prepare(cfg, dims)
    uo, ito, _ = oracle.render(pc, 77)
    assert it[0] == ito
    assert rel_fro(u[..., 0], uo) < 1e-2


def test_renderings_and_seed_increment(api, oracle):
    """renderingsNum > 1 renders seed, seed + 1, ... (MatlabInterface.cu:1783-1801)."""
    cfg, dims = SCENES["speckle_2d"]
    cfg = dict(cfg)
    cfg["simulation"] = dict(cfg["simulation"], renderingsNum=3)
    with api.Scene(cfg, dims) as s:
        u, it = s.render(seed=40)
    assert u.shape[-1] == 3
    pc = cf.prepare(cfg, dims)
    for r in range(3):
        uo, ito, _ = oracle.render(pc, 40 + r)
        assert it[r] == ito
        assert rel_fro(u[..., r], uo) <= REL_TOL


def test_chunking_is_invisible(api, oracle, monkeypatch):
    """A render split into device chunks gives the same paths."""
    monkeypatch.setenv("SSTMC_CHUNK_BYTES", "200000")
    cfg, dims = SCENES["correlation_3d"]
    with api.Scene(cfg, dims) as s:
        u, it = s.render(seed=9)
    pc = cf.prepare(cfg, dims)
    uo, ito, _ = oracle.render(pc, 9)
    assert it[0] == ito
    assert rel_fro(u[..., 0], uo) <= REL_TOL


@pytest.mark.parametrize("name", ["correlation_64x64", "speckle_2d", "transmission_matrix_3d", "corr_far_2d_drift"])
def test_tensor_core_contraction_matches_simt(name, api, monkeypatch):
    """The tcgen05 3xTF32 contraction (default) against the compensated SIMT
    contraction on the same rows.  Both carry FP32-level rounding (~1e-7 per
    product, amplified by the cancellation of the random-phase sum), so they
    agree within 2e-6, inside the 1e-5 budget against the FP64 oracle."""
    from temporalspecklescode_gb300 import workloads as wl
    if name == "correlation_64x64":
        cfg, dims = wl.correlation_3d(batch_size=4096, full_iteration=2, n_side=8, n_lags=8)
    else:
        cfg, dims = SCENES[name]
    with api.Scene(cfg, dims) as s:
        u_tc, it_tc = s.render(seed=21)
        monkeypatch.setenv("SSTMC_CONTRACTION", "simt")
        u_simt, it_simt = s.render(seed=21)
    assert np.array_equal(it_tc, it_simt)
    err = rel_fro(u_tc, u_simt)
    assert err <= 2e-6, (name, err)


def test_tensor_core_contraction_large_k_against_oracle(api, oracle):
    """64 x 64 x 8 correlation over 16384 paths (K per CTA in the thousands,
    many 128-path accumulation windows) against the FP64 oracle."""
    from temporalspecklescode_gb300 import workloads as wl
    cfg, dims = wl.correlation_3d(batch_size=8192, full_iteration=2, n_side=8, n_lags=8)
    with api.Scene(cfg, dims) as s:
        u, it = s.render(seed=4)
    uo, ito, _ = oracle.render(cf.prepare(cfg, dims), 4)
    assert it[0] == ito
    assert rel_fro(u[..., 0], uo) <= REL_TOL


@pytest.mark.parametrize("name", ["correlation_64x64", "speckle_2d", "correlation_3d", "transmission_matrix_3d", "mcx_3d",
                                  "homogeneous_3d", "point_2d_iso_field", "point_2d_iso_corr",
                                  "correlation_wide", "correlation_wide_irregular"])
def test_view_kernel_matches_fused_kernel(name, api, monkeypatch):
    """The view-side kernel (default for static scenes) against the view loop
    of the fused trace kernel: identical voxel-step counts and per-path view
    rows within FP32 rounding."""
    from temporalspecklescode_gb300 import workloads as wl
    if name == "correlation_64x64":
        cfg, dims = wl.correlation_3d(batch_size=512, full_iteration=1, n_side=8, n_lags=8)
    else:
        cfg, dims = SCENES[name]
    with api.Scene(cfg, dims) as s:
        a = s.trace_paths(seed=8, first_path=3, paths=256)
        monkeypatch.setenv("SSTMC_VIEW_KERNEL", "fused")
        b = s.trace_paths(seed=8, first_path=3, paths=256)
    for k in ("misses", "vertices", "vertex_hash", "dda_steps"):
        assert np.array_equal(a[k], b[k]), (name, k)
    for k in ("a_ms", "s_ms", "a_ss", "b_ss"):
        err = rel_fro(a[k], b[k])
        assert err <= 2e-6, (name, k, err)


@pytest.mark.parametrize("name", ["reciprocal_far_3d_cbs", "reciprocal_point_2d_cbs",
                                  "reciprocal_far_3d_corr_cbs", "reciprocal_point_2d_corr_cbs",
                                  "reciprocal_far_3d_vmf_cbs"])
def test_cbs_reciprocity(name, api):
    """Field CBS on the GPU: with the views the reversed illuminations the field
    is symmetric in (l, v) (the reversed-path rows are the direct rows with the
    sources' roles exchanged); FP32 rows, so to 1e-5."""
    from tests.test_oracle_pins import _sym_err
    cfg, dims = SCENES[name]
    with api.Scene(cfg, dims) as s:
        u, _ = s.render(seed=21)
    assert _sym_err(u[..., 0]) < 1e-5


def test_wavelength_vector_renders_each_wavelength(api):
    """sstmc2D with a lambda vector: u gains a wavelength axis (Nl, Nv, Nw, Nt, R)
    and each wavelength's slice is the single-wavelength render of the same paths."""
    from tests.scenes import point_2d_iso
    cfg, dims = point_2d_iso(False)
    lams = [0.5, 0.65]
    multi = dict(cfg)
    multi["simulation"] = dict(cfg["simulation"], **{"lambda": lams})
    u, it = api.sstmc2D(multi)
    assert u.shape[2] == 2
    for w, lam in enumerate(lams):
        one = dict(cfg)
        one["simulation"] = dict(cfg["simulation"], **{"lambda": lam})
        uw, itw = api.sstmc2D(one)
        assert np.array_equal(it, itw)
        assert rel_fro(u[:, :, w], uw) <= 1e-12
    assert rel_fro(u[:, :, 0], u[:, :, 1]) > 1e-3   # the phases differ


@pytest.mark.parametrize("make", ["static", "correlation"])
def test_forced_inside_bin_neutral_cases(api, make):
    """isForcedInsideBin changes nothing, bit for bit, where the reference's
    option has no effect: every material static (all ticks on the sampled
    point), or the correlation sampler (which has no such option)."""
    from tests import scenes
    cfg, dims = scenes.field_point_3d(moving=False) if make == "static" else scenes.corr_far_2d_drift()
    forced = dict(cfg, sampler=dict(cfg["sampler"], isForcedInsideBin=True))
    with api.Scene(cfg, dims) as s:
        u0, _ = s.render(seed=31)
    with api.Scene(forced, dims) as s:
        u1, _ = s.render(seed=31)
    assert np.array_equal(u0, u1)


def test_vmf_scatters_isotropically_in_2d(api):
    """A 2D vMF material scatters isotropically, as in the reference: the render
    equals the one with an Isotropic material, bit for bit."""
    from tests.scenes import vmf_2d
    out = []
    for vmf in (True, False):
        with api.Scene(*vmf_2d(vmf)) as s:
            out.append(s.render(seed=8)[0])
    assert np.array_equal(out[0], out[1])


def test_walk_overflow_pool_grows(api, oracle):
    """Paths of hundreds of vertices exhaust the walk's default overflow pool:
    the first render grows the pool and walks the chunk again, the second
    (same seed) keeps every path in the grown pool from the start.  Both
    renders are identical and match the oracle."""
    from tests.scenes import very_long_paths_2d
    cfg, dims = very_long_paths_2d()
    with api.Scene(cfg, dims) as s:
        u1, it1 = s.render(seed=31)
        st1 = s.stats()
        u2, it2 = s.render(seed=31)
        st2 = s.stats()
    assert np.array_equal(u1, u2) and np.array_equal(it1, it2)
    # far past the 64-vertex slots: the default pool (paths / 16 + 64 blocks) runs dry
    assert st1["vertices"] == st2["vertices"] and st1["vertices"] > 100 * st1["paths"]
    uo, ito, sto = oracle.render(cf.prepare(cfg, dims), 31)
    assert it1[0] == ito and st1["vertices"] == sto["vertices"]
    assert rel_fro(u1[..., 0], uo) <= REL_TOL


def test_autotuned_wavefront_keeps_the_render(api, oracle):
    """sstmc_scene_autotune picks the wavefront (paths per chunk) from timed
    samples; a render at the chosen wavefront traces the same paths (integer
    statistics exact) and stays within the tolerance of the FP64 oracle."""
    from temporalspecklescode_gb300 import workloads as wl
    cfg, dims = wl.correlation_3d(batch_size=8192, full_iteration=2, n_side=4, n_lags=4)
    with api.Scene(cfg, dims) as s:
        chunk = s.autotune(sample_paths=16384)
        assert 4096 <= chunk <= 16384 and chunk & (chunk - 1) == 0
        u, it = s.render(seed=6)
        st = s.stats()
    uo, ito, sto = oracle.render(cf.prepare(cfg, dims), 6)
    assert it[0] == ito and st["vertices"] == sto["vertices"] and st["dda_steps"] == sto["dda_steps"]
    assert rel_fro(u[..., 0], uo) <= REL_TOL
