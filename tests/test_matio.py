"""MATLAB .mat I/O of the sstmc2D / sstmc3D mirror: a config written as a
MATLAB struct and read back renders identically (oracle, CPU), the outputs
are written as the MEX call returns them, and a lambda vector is split into
wavelengths."""
import numpy as np
import pytest

pytest.importorskip("scipy")

from temporalspecklescode_gb300 import api, config as cf, matio
from tests import scenes


@pytest.mark.parametrize("name", ["field_point_3d", "corr_far_2d_drift", "point_2d_iso_field", "speckle_2d_cbs"])
def test_config_round_trip_renders_identically(tmp_path, oracle, name):
    cfg, dims = scenes.small_scenes()[name]
    path = str(tmp_path / "cfg.mat")
    matio.save_config(path, cfg)
    back = matio.load_config(path)
    u0, it0, st0 = oracle.render(cf.prepare(cfg, dims), 5)
    u1, it1, st1 = oracle.render(cf.prepare(back, dims), 5)
    assert it0 == it1 and st0 == st1
    assert np.array_equal(u0, u1)


def test_result_file(tmp_path):
    from scipy.io import loadmat
    u = (np.arange(24.0) + 1j * np.arange(24.0)[::-1]).reshape(2, 3, 4, 1)
    path = str(tmp_path / "out.mat")
    matio.save_result(path, u, np.array([128.0]))
    m = loadmat(path)
    assert m["u"].shape == (2, 3, 4, 1) and np.array_equal(m["u"], u)
    assert m["iter"].shape == (1, 1) and m["iter"][0, 0] == 128.0


def test_wavelength_vector():
    cfg, _ = scenes.point_2d_iso(False)
    assert np.array_equal(api.wavelengths(cfg), [0.5])
    cfg = dict(cfg)
    cfg["simulation"] = dict(cfg["simulation"], **{"lambda": np.array([0.5, 0.6, 0.7])})
    assert np.array_equal(api.wavelengths(cfg), [0.5, 0.6, 0.7])
    with pytest.raises(cf.ConfigError):
        cf.prepare(cfg, 2)   # one scene has one wavelength; the mirror splits the vector


def test_vmf_struct_cells_round_trip(tmp_path):
    """vMF materials are struct cells (mixtureMu / mixtureC / mixtureAlpha) inside
    the amplitudeFunction cell array; a .mat round trip keeps every component."""
    from tests.scenes import small_scenes
    cfg, dims = small_scenes()["vmf_field_3d"]
    p = str(tmp_path / "vmf.mat")
    matio.save_config(p, cfg)
    back = matio.load_config(p)
    a, b = cf.prepare(cfg, dims), cf.prepare(back, dims)
    n = int(np.ctypeslib.as_array(a.struct.vmf_n, (3,)).sum())
    assert n == int(np.ctypeslib.as_array(b.struct.vmf_n, (3,)).sum())
    for f in ("vmf_mu", "vmf_c", "vmf_alpha"):
        assert np.array_equal(np.ctypeslib.as_array(getattr(a.struct, f), (n,)),
                              np.ctypeslib.as_array(getattr(b.struct, f), (n,)))
