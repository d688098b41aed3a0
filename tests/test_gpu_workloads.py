"""GPU parity at the full shapes of the benchmark workloads, on path subsets
the FP64 oracle finishes in seconds.

* transmission_matrix_3d: 1024 x 1024 far-field directions on 20-degree
  cones, a 64x64x32 grid of four iid materials; its far-field x far-field
  single-scattering GEMMs run per material.
* tracking_2d_pairs: 128 x 128 far-field directions on a 256^2 grid whose
  disc drifts, the correlation sampler over the 32 lags of 32 frames, and
  the frame-pair correlations filled from them.

Integers (iteration counts, vertices, voxel steps, contributions) exact,
fields within a relative Frobenius error of 1e-5.
"""
import numpy as np
import pytest

from temporalspecklescode_gb300 import config as cf
from temporalspecklescode_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


def rel_fro(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope="module")
def api():
    from temporalspecklescode_gb300 import api as A
    A.load_library()
    return A


def _render_vs_oracle(api, oracle, cfg, dims, seed):
    with api.Scene(cfg, dims) as s:
        u, it = s.render(seed=seed)
        st = s.stats()
    uo, ito, sto = oracle.render(cf.prepare(cfg, dims), seed)
    assert it[0] == ito
    for k in ("vertices", "paths", "dda_steps", "contributions"):
        assert st[k] == sto[k], (k, st[k], sto[k])
    return u[..., 0], uo


def test_transmission_matrix_full_shape(api, oracle):
    cfg, dims = wl.transmission_matrix_3d(batch_size=256, full_iteration=1, seed=3)
    u, uo = _render_vs_oracle(api, oracle, cfg, dims, 11)
    assert u.shape == (1024, 1024, 1)
    assert rel_fro(u, uo) <= REL_TOL


def test_transmission_matrix_rows_full_shape(api, oracle):
    cfg, dims = wl.transmission_matrix_3d(batch_size=256, full_iteration=1, seed=3)
    with api.Scene(cfg, dims) as s:
        g = s.trace_paths(seed=5, first_path=17, paths=16)
    o = oracle.trace_paths(cf.prepare(cfg, dims), 5, 17, 16)
    for k in ("misses", "vertices", "vertex_hash", "dda_steps", "m1"):
        assert np.array_equal(g[k], o[k]), k
    for k in ("a_ms", "s_ms", "a_ss", "b_ss"):
        assert rel_fro(g[k], o[k]) <= REL_TOL, k


def test_tracking_pairs_full_shape(api, oracle):
    cfg, dims = wl.tracking_2d_pairs(batch_size=8, full_iteration=1, seed=2)
    u, uo = _render_vs_oracle(api, oracle, cfg, dims, 13)
    assert u.shape == (128, 128, 32)
    assert rel_fro(u, uo) <= REL_TOL
    C = wl.frame_pairs(u[..., None], 32)[..., 0]
    Co = wl.frame_pairs(uo[..., None], 32)[..., 0]
    assert C.shape == (128, 128, 32, 32)
    assert rel_fro(C, Co) <= REL_TOL


def test_frame_pairs_equal_per_pair_ticks(api):
    """Rendering the F non-negative lags and filling the F x F frame pairs
    from them (conjugates for t2 < t1) gives the render whose ticks are every
    pair's own lag t2 - t1, negative lags included (the same paths; the two
    renders differ only in how the contraction splits its FP32 windows)."""
    F = 4
    cfg, dims = wl.tracking_2d_pairs(batch_size=64, full_iteration=2, n_dirs=8, frames=F, seed=4)
    with api.Scene(cfg, dims) as s:
        u, it = s.render(seed=3)
    pairs = np.array([t2 - t1 for t1 in range(F) for t2 in range(F)], dtype=float)
    cfg2 = dict(cfg, sampler=dict(cfg["sampler"], t=pairs))
    with api.Scene(cfg2, dims) as s:
        u2, it2 = s.render(seed=3)
    assert np.array_equal(it, it2)
    C = wl.frame_pairs(u, F)[..., 0]
    C2 = u2[..., 0].reshape(8, 8, F, F)
    assert rel_fro(C, C2) <= 1e-6


def test_long_path_segments_match_oracle(api, oracle):
    """Correlation sampler with drifting scatterers and paths of hundreds to
    thousands of vertices: the general kernel sums such paths in segments of
    256 vertices on separate warps (each starting from the momentum-transfer
    sum of the vertices before it); the render matches the oracle, which walks
    every path in one piece."""
    cfg, dims = wl.tracking_2d_pairs(batch_size=96, full_iteration=1, n_dirs=8, frames=4, seed=6)
    with api.Scene(cfg, dims) as s:
        g = s.trace_paths(seed=21, first_path=0, paths=96)
        assert g["vertices"].max() > 2 * 256 + 1   # several segments on the longest path
        u, it = s.render(seed=21)
        st = s.stats()
    pc = cf.prepare(cfg, dims)
    o = oracle.trace_paths(pc, 21, 0, 96)
    for k in ("vertices", "vertex_hash", "dda_steps"):
        assert np.array_equal(g[k], o[k]), k
    assert rel_fro(g["s_ms"], o["s_ms"]) <= REL_TOL
    uo, ito, sto = oracle.render(pc, 21)
    assert it[0] == ito and st["dda_steps"] == sto["dda_steps"]
    assert rel_fro(u[..., 0], uo) <= REL_TOL


def test_long_path_segments_field_sampler_match_oracle(api, oracle):
    """The field sampler with drifting scatterers and paths of thousands of
    vertices: each 256-vertex segment replays the per-tick positions and
    path-length sums of the vertices before it (the same FP64 additions in the
    same order), so its path phases are the path's own; rows and render match
    the oracle."""
    cfg, dims = wl.tracking_2d(batch_size=48, full_iteration=1, n_dirs=8, frames=4, seed=6)
    with api.Scene(cfg, dims) as s:
        g = s.trace_paths(seed=23, first_path=0, paths=48)
        assert g["vertices"].max() > 2 * 256 + 1
        u, it = s.render(seed=23)
    pc = cf.prepare(cfg, dims)
    o = oracle.trace_paths(pc, 23, 0, 48)
    for k in ("vertices", "vertex_hash", "dda_steps"):
        assert np.array_equal(g[k], o[k]), k
    assert rel_fro(g["s_ms"], o["s_ms"]) <= REL_TOL
    uo, ito, _ = oracle.render(pc, 23)
    assert it[0] == ito
    assert rel_fro(u[..., 0], uo) <= REL_TOL


def test_confocal_shape_matches_oracle(api, oracle):
    """The focused-beam workload at its full 64 x 64 beam shape on a path
    subset: integers bit-exact, rows and render within the tolerance."""
    cfg, dims = wl.confocal_3d(batch_size=128, full_iteration=1)
    with api.Scene(cfg, dims) as s:
        g = s.trace_paths(seed=9, first_path=0, paths=128)
        u, it = s.render(seed=9)
    pc = cf.prepare(cfg, dims)
    o = oracle.trace_paths(pc, 9, 0, 128)
    for k in ("vertices", "vertex_hash", "dda_steps", "misses"):
        assert np.array_equal(g[k], o[k]), k
    for k in ("a_ms", "s_ms", "a_ss", "b_ss"):
        assert rel_fro(g[k], o[k]) <= REL_TOL, k
    uo, ito, _ = oracle.render(pc, 9)
    assert it[0] == ito
    assert rel_fro(u[..., 0], uo) <= REL_TOL
