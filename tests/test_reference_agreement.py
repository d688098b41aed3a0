"""Agreement of the estimator with the reference's own CUDA path (the
reference's objects and kernels run without MATLAB by oracle/refharness.cu).

The reference draws its random numbers from cuRAND XORWOW and this build from
Philox, so the two renders are independent samples of the same estimator:
they must agree in distribution.  Per scene, both sides render R independent
renderings (seeds s, s + 1, ...); per output entry the means are compared in
units of their combined standard error (from the spread over renderings):

* the global mean over all entries agrees within 3 standard errors;
* the per-entry z-scores have mean square below 3 (about 1 when the two
  estimators agree; a systematic error in a term shows up as a large value);
* the missed first vertices agree within 3 standard errors of a binomial.

Field renders are compared through their intensity |u|^2 / iter (the field's
mean is zero: every path carries a uniform random phase), correlation renders
through u / iter.  Skipped when the reference's headers are not staged
(oracle/stage_reference.sh).
"""
import numpy as np
import pytest

from temporalspecklescode_gb300 import workloads as wl
from tests import refharness_lib as ref
from tests import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    if not ref.available():
        pytest.skip("the reference's headers are not staged (sh oracle/stage_reference.sh <reference checkout>)")
    from temporalspecklescode_gb300 import api as A
    A.load_library()
    return A


def _scenes():
    far3d, _ = wl.transmission_matrix_3d(batch_size=1024, full_iteration=2, n_dirs=12, grid=(16, 16, 8), seed=0)
    return {
        # 2D far-field speckle: the 16 x 16 geometry of the speckle workload
        "speckle_2d": (wl.speckle_2d(batch_size=1024, full_iteration=2)[0], 2, "field"),
        # 3D temporal correlation: the correlation workload's geometry on 4 x 4 lattices
        "correlation_3d": (wl.correlation_3d(batch_size=1024, full_iteration=2, n_side=4, n_lags=8)[0], 3, "correlation"),
        # 3D heterogeneous far field: four iid materials on a 16x16x8 grid, 12 x 12 directions
        "transmission_3d": (far3d, 3, "field"),
        # 3D focused Gaussian beams in a two-material vMF slab (two lobes per material)
        "gauss_3d": (scenes.gauss_beams_3d(batch_size=1024, full_iteration=16, n_l=4, n_v=6, equal_lobes=True)[0], 3, "field"),
        # 2D focused Gaussian beams (point-source sampling, Bessel-I0 amplitudes)
        "gauss_2d": (scenes.gauss_beams_2d(batch_size=1024, full_iteration=8)[0], 2, "field"),
        # 2D correlation with coherent backscattering and drifting scatterers (U != 0)
        "corr_drift_cbs_2d": (scenes.with_cbs(scenes.corr_far_2d_drift(batch_size=1024, full_iteration=4))[0], 2,
                              "correlation"),
    }


SCENES = _scenes()


def _estimates(u, it, kind):
    """Per rendering the estimated quantity: |u|^2 / iter (field) or u / iter."""
    if kind == "field":
        return np.abs(u) ** 2 / it[None, None, None, :]
    return u / it[None, None, None, :]


def _mean_se(x):
    R = x.shape[-1]
    return x.mean(axis=-1), x.std(axis=-1, ddof=1) / np.sqrt(R)


@pytest.mark.parametrize("name", sorted(SCENES))
def test_estimator_agrees_with_reference(name, api):
    cfg, dims, kind = SCENES[name]
    R = 24
    u_ref, it_ref, ms_ref = ref.render(cfg, dims, R, seed=1000)
    c = dict(cfg, simulation=dict(cfg["simulation"], renderingsNum=R))
    with api.Scene(c, dims) as s:
        u, it = s.render(seed=5000)
    e_ref = _estimates(u_ref, it_ref, kind)
    e = _estimates(u, it, kind)
    parts = [(np.real, "re")] + ([(np.imag, "im")] if kind == "correlation" else [])
    for f, label in parts:
        m_ref, se_ref = _mean_se(f(e_ref))
        m, se = _mean_se(f(e))
        # global mean over all entries, its standard error from the per-rendering means
        g_ref = f(e_ref).reshape(-1, R).mean(axis=0)
        g = f(e).reshape(-1, R).mean(axis=0)
        gz = (g_ref.mean() - g.mean()) / np.sqrt(g_ref.var(ddof=1) / R + g.var(ddof=1) / R)
        den = np.sqrt(se_ref ** 2 + se ** 2)
        ok = den > 1e-12 * max(np.abs(m_ref).max(), 1e-300)
        z = (m_ref - m)[ok] / den[ok]
        print(f"{name} {label}: global mean reference {g_ref.mean():.6g} this build {g.mean():.6g} z {gz:+.2f}; "
              f"per-entry mean z^2 {np.mean(z ** 2):.2f} over {z.size} entries; reference trace {np.mean(ms_ref):.1f} ms")
        assert abs(gz) < 3.0, (name, label, g_ref.mean(), g.mean(), gz)
        assert np.mean(z ** 2) < 3.0, (name, label, np.mean(z ** 2), np.abs(z).max())
    # missed first vertices: iter - batch * fullIteration, a binomial count per attempt
    n = cfg["simulation"]["batchSize"] * cfg["simulation"]["fullIteration"]
    miss_ref, miss = (it_ref - n).sum(), (it - n).sum()
    p = (miss_ref + miss) / (2 * R * n + miss_ref + miss)
    sd = np.sqrt(max(p * (1 - p), 1e-12) * 2 * R * n)
    assert abs(miss_ref - miss) <= 3.0 * sd + 3.0, (name, miss_ref, miss)
