"""Host-side config handling (temporalspecklescode_gb300/config.py): the
MATLAB config struct as a dict -> the C-ABI struct, with the validation the
MEX layer performs (MatlabInterface.cu:712-1457).  CPU only."""
import numpy as np
import pytest

from temporalspecklescode_gb300 import config as cf
from temporalspecklescode_gb300 import workloads as wl
from tests import scenes


def _speckle():
    cfg, dims = wl.speckle_2d(batch_size=8, full_iteration=1, n_dirs=3)
    return cfg, dims


def test_prepare_fills_the_struct():
    cfg, dims = scenes.field_point_3d()
    pc = cf.prepare(cfg, dims)
    s = pc.struct
    assert s.dims == 3 and s.batch_size == 64 and s.full_iteration == 2
    assert s.scattering_num == 3 and s.illumination.count == 6 and s.view.count == 5
    assert s.sampler_type == cf.SAMPLER_TEMPORAL and s.t_num == 5
    # materialGrid flattened x fastest (MATLAB column order)
    grid = np.asarray(cfg["medium"]["materialGrid"])
    flat = np.ctypeslib.as_array(s.material_grid, (grid.size,))
    assert np.array_equal(flat, grid.ravel(order="F"))


def test_gaussian_beam_config_fields():
    """focalPoint, focalDirection and aperture (MatlabInterface.cu:1161-1200)
    reach the source block; a missing field or a direction count that differs
    from the focal points' is refused."""
    cfg, dims = _speckle()
    cfg["illumination"] = {"type": "GaussianBeam", "focalPoint": {"x": [0.0, 1.0], "y": [0.0, 2.0]},
                           "focalDirection": {"x": [0.0, 0.6], "y": [1.0, 0.8]}, "aperture": 0.4}
    pc = cf.prepare(cfg, dims)
    s = pc.struct.illumination
    assert s.type == cf.SOURCE_GAUSSIANBEAM and s.count == 2 and s.aperture == 0.4
    assert [s.xyz[i] for i in range(6)] == [0.0, 0.0, 0.0, 1.0, 2.0, 0.0]
    assert [s.focal_direction[i] for i in range(6)] == [0.0, 1.0, 0.0, 0.6, 0.8, 0.0]
    bad = dict(cfg["illumination"], focalDirection={"x": [0.0], "y": [1.0]})
    with pytest.raises(cf.ConfigError, match="focalDirection"):
        cf.prepare(dict(cfg, illumination=bad), dims)
    with pytest.raises(cf.ConfigError, match="aperture"):
        cf.prepare(dict(cfg, illumination={k: v for k, v in cfg["illumination"].items() if k != "aperture"}), dims)


@pytest.mark.parametrize("edit,match", [
    (lambda c: c["simulation"].update(batchSize=0), "positive"),
    (lambda c: c["simulation"].update(**{"lambda": [0.5, 0.7]}), "one wavelength"),
    (lambda c: c.pop("scattering"), "scattering"),
    (lambda c: c["scattering"].update(type=["HG", "Mie"]), "Unsupported scattering type"),
    (lambda c: c["medium"].update(sigs=[0.0, 1.0, 2.0]), "sigs"),
    (lambda c: c["sampler"].update(D=[0.0, -1.0]), "non-negative"),
    (lambda c: c["sampler"].update(type="Spectral"), "sampler"),
    (lambda c: c["tracer"].update(type="pathTracer"), "tracer"),
    (lambda c: c["view"].update(type="Pencil"), "Unsupported source type"),
])
def test_config_errors(edit, match):
    cfg, dims = _speckle()
    edit(cfg)
    with pytest.raises(cf.ConfigError, match=match):
        cf.prepare(cfg, dims)


def test_tabular_and_vmf_tables_are_concatenated_in_material_order():
    amp = np.exp(1j * np.linspace(0, 1, 5)) * np.linspace(1, 2, 5)
    cfg, dims = scenes.field_point_3d()
    cfg["scattering"] = {"type": ["Tabular", "vMF", "Tabular"],
                         "amplitudeFunction": [amp, scenes.vmf_mixture([0.0, 2.0], [0.5, 0.5]), amp[:3]]}
    pc = cf.prepare(cfg, dims)
    s = pc.struct
    tn = np.ctypeslib.as_array(s.tabular_n, (3,))
    assert list(tn) == [5, 0, 3]
    tf = np.ctypeslib.as_array(s.tabular_f, (2 * 8,)).view(np.complex128)
    assert np.array_equal(tf, np.concatenate([amp, amp[:3]]))
    vn = np.ctypeslib.as_array(s.vmf_n, (3,))
    assert list(vn) == [0, 2, 0]
    assert list(np.ctypeslib.as_array(s.vmf_mu, (2,))) == [0.0, 2.0]


def test_forced_inside_bin_and_cbs_flags():
    cfg, dims = scenes.forced_bin_2d()
    assert cf.prepare(cfg, dims).struct.is_forced_inside_bin == 1
    cfg2 = dict(cfg, sampler=dict(cfg["sampler"], isForcedInsideBin=False), tracer={"type": "nee", "isCBS": True})
    s = cf.prepare(cfg2, dims).struct
    assert s.is_forced_inside_bin == 0 and s.is_cbs == 1


def test_homogeneous_medium_maps_to_a_box():
    cfg, dims = _speckle()
    cfg["medium"] = {"type": "Homogeneous", "boxMin": {"x": -3.0, "y": -2.0}, "boxMax": {"x": 3.0, "y": 2.0}, "sigs": 0.8}
    s = cf.prepare(cfg, dims).struct
    assert s.medium_type == cf.MEDIUM_HOMOGENEOUS
    assert list(s.box_min)[:2] == [-3.0, -2.0] and list(s.box_max)[:2] == [3.0, 2.0]


@pytest.mark.parametrize("edit", [
    lambda c: c.update(view={"type": "FarField", "direction": {"x": [], "y": []}}),
    lambda c: c.update(illumination={"type": "PointSource", "location": {"x": [], "y": []}}),
    lambda c: c["sampler"].update(t=[]),
])
def test_empty_inputs_are_refused(edit):
    """Empty source lists and tick lists are refused by the host mirror (the
    MEX layer's readers require one element), and by the C-ABI's own
    validation when a caller fills the struct directly (checked here on the
    oracle, which validates like the library)."""
    cfg, dims = _speckle()
    edit(cfg)
    with pytest.raises(cf.ConfigError, match="at least one element"):
        cf.prepare(cfg, dims)


def test_c_abi_refuses_empty_sources(oracle):
    cfg, dims = _speckle()
    pc = cf.prepare(cfg, dims)
    pc.struct.view.count = 0
    with pytest.raises(RuntimeError, match="100"):
        oracle.render(pc, 0)


def test_frame_pairs_indexing():
    """frame_pairs maps the lags 0 .. F-1 onto the F x F pairs by t2 - t1, and
    the pairs with t2 < t1 onto the conjugate of lag t1 - t2."""
    from temporalspecklescode_gb300 import workloads as wl
    F = 5
    lags = wl.frame_lags(F)
    assert lags.tolist() == list(range(F))
    u = np.broadcast_to((lags + 1j * (lags + 10))[None, None, :, None], (2, 3, F, 1))
    C = wl.frame_pairs(u, F)
    assert C.shape == (2, 3, F, F, 1)
    for t1 in range(F):
        for t2 in range(F):
            d = abs(t2 - t1)
            assert C[1, 2, t1, t2, 0] == (d + 1j * (d + 10) if t2 >= t1 else d - 1j * (d + 10))


def test_frame_pairs_oracle_equals_per_pair_ticks(oracle):
    """On the oracle (FP64, every tick evaluated on its own), the render over
    the non-negative lags, filled onto the frame pairs by conjugation, equals
    the render whose ticks are every pair's own lag t2 - t1 (negative lags
    included): the estimator is conjugate-symmetric in the lag path by path."""
    from temporalspecklescode_gb300 import config as cf
    from temporalspecklescode_gb300 import workloads as wl
    F = 3
    cfg, dims = wl.tracking_2d_pairs(batch_size=6, full_iteration=1, n_dirs=4, frames=F, seed=4)
    u, it, _ = oracle.render(cf.prepare(cfg, dims), 3)
    pairs = np.array([t2 - t1 for t1 in range(F) for t2 in range(F)], dtype=float)
    cfg2 = dict(cfg, sampler=dict(cfg["sampler"], t=pairs))
    u2, it2, _ = oracle.render(cf.prepare(cfg2, dims), 3)
    assert it == it2
    C = wl.frame_pairs(u[..., None], F)[..., 0]
    assert np.allclose(C, u2.reshape(4, 4, F, F), rtol=0, atol=1e-12 * np.abs(u2).max())
