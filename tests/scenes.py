"""Scaled-down scenes for the parity tests: every sampler x source x medium
combination the path supports, at sizes the oracle finishes in seconds."""
from __future__ import annotations

import json
import os

import numpy as np

from temporalspecklescode_gb300 import workloads as wl

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def mcx_fixture():
    with open(os.path.join(GOLDEN, "mcx_validation.json")) as f:
        return json.load(f)


def mudiff_fixture():
    import numpy as _np
    return dict(_np.load(os.path.join(GOLDEN, "mudiff_cbs.npz")))


def mudiff_scene(cbs: bool, correlation: bool = True, batch_size=4000, full_iteration=25):
    """The scene of examples/mudiffCBSValidation2D.m from its fixture: a 2D
    square of mean free path MFP with a tabular amplitude function, one
    far-field illumination along +y, views at the fixture's angles; the
    correlation sampler at t = 0 (an intensity) or the field sampler."""
    fx = mudiff_fixture()
    deg = fx["degList"]
    view = {"type": "FarField", "direction": {"x": np.sin(deg), "y": np.cos(deg)}}
    ill = {"type": "FarField", "direction": {"x": [0.0], "y": [1.0]}}
    amp = fx["ampFunc"]
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 1.0, "seed": 0},
        "scattering": {"type": ["Tabular", "Tabular"], "amplitudeFunction": [amp, amp]},
        "medium": {"type": "Heterogeneous", "xAxis": fx["x"], "yAxis": fx["y"], "materialGrid": np.ones((1, 1), dtype=np.uint32),
                   "sigs": [0.0, 1.0 / float(fx["MFP"])], "siga": [0.0, 0.0]},
        "illumination": ill, "view": view,
        "sampler": {"type": "TemporalCorrelationSampler" if correlation else "TemporalSampler", "t": [0.0],
                    "D": [0.0, 0.0], "U": {"x": [0.0, 0.0], "y": [0.0, 0.0]}},
        "tracer": {"type": "nee", "isCBS": cbs},
    }
    if correlation:
        cfg["illumination2"] = ill
        cfg["view2"] = view
    return cfg, 2


def field_point_3d(moving: bool = True, area: bool = False, batch_size=64, full_iteration=2):
    """3D field sampler with point sources, Brownian + drift motion (ticks around their mean)."""
    rng = np.random.default_rng(7)
    ill = {"type": "PointSource", "location": {"x": rng.uniform(-8, 8, 6), "y": rng.uniform(-8, 8, 6), "z": np.full(6, -2.0)},
           "isAreaSource": area}
    view = {"type": "PointSource", "location": {"x": rng.uniform(-8, 8, 5), "y": rng.uniform(-8, 8, 5), "z": np.full(5, 12.0)}}
    grid = rng.integers(1, 3, size=(4, 3, 5)).astype(np.uint32)
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 0.7, "seed": 3},
        "scattering": {"type": ["HG", "HG", "Isotropic"], "amplitudeFunction": [0.5, 0.6, 0.0]},
        "medium": {"type": "Heterogeneous", "xAxis": np.linspace(-10, 10, 5), "yAxis": [-10.0, -2.0, 3.0, 10.0],
                   "zAxis": np.linspace(0, 10, 6), "materialGrid": grid, "sigs": [0.0, 0.6, 1.1], "siga": [0.0, 0.02, 0.05]},
        "illumination": ill, "view": view,
        "sampler": {"type": "TemporalSampler", "t": [0.0, 1.0, 2.5, -1.5, 4.0],
                    "D": [0.0, 2e-3 if moving else 0.0, 5e-3 if moving else 0.0],
                    "U": {"x": [0.0, 0.01 if moving else 0.0, 0.0], "y": [0.0, 0.0, 0.02 if moving else 0.0], "z": [0.0, 0.0, 0.0]}},
        "tracer": {"type": "nee"},
    }
    return cfg, 3


def corr_far_2d_drift(batch_size=64, full_iteration=2):
    """2D correlation sampler, far-field, different u1/u2 view sets, drift U != 0."""
    d = wl._farfield_fan(6)
    d2 = wl._farfield_fan(5, 0.4)
    grid = np.array([[1, 2], [2, 1], [1, 1]], dtype=np.uint32)
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 1.0, "seed": 5},
        "scattering": {"type": ["HG", "HG", "HG"], "amplitudeFunction": [0.3, 0.3, 0.85]},
        "medium": {"type": "Heterogeneous", "xAxis": [-6.0, -1.0, 2.0, 6.0], "yAxis": [-5.0, 0.5, 5.0],
                   "materialGrid": grid, "sigs": [0.0, 0.8, 1.5], "siga": [0.0, 0.01, 0.0]},
        "illumination": {"type": "FarField", "direction": d}, "view": {"type": "FarField", "direction": d2},
        "illumination2": {"type": "FarField", "direction": {"x": d["x"] * 0.98 + 0.02, "y": d["y"]}},
        "view2": {"type": "FarField", "direction": d2},
        "sampler": {"type": "TemporalCorrelationSampler", "t": [0.5, 1.0, 3.0],
                    "D": [0.0, 1e-3, 4e-3], "U": {"x": [0.0, 0.05, 0.0], "y": [0.0, 0.0, -0.03]}},
        "tracer": {"type": "nee"},
    }
    return cfg, 2


def point_2d_iso(correlation: bool, batch_size=64, full_iteration=2):
    """2D point sources, isotropic scattering, single bin (scalar single-scattering amplitude)."""
    ill = {"type": "PointSource", "location": {"x": [-3.0, 0.0, 2.5], "y": [-7.0, -7.0, -7.0]}}
    view = {"type": "PointSource", "location": {"x": [-2.0, 1.0, 3.0, 4.0], "y": [7.0, 7.0, 7.0, 7.0]}}
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 0.5, "seed": 11},
        "scattering": {"type": ["Isotropic"], "amplitudeFunction": [0.0]},
        "medium": {"type": "Heterogeneous", "xAxis": [-5.0, 5.0], "yAxis": [-5.0, 5.0],
                   "materialGrid": np.ones((1, 1), np.uint32), "sigs": [0.0, 0.7], "siga": [0.0, 0.05]},
        "illumination": ill, "view": view,
        "sampler": {"type": "TemporalCorrelationSampler" if correlation else "TemporalSampler", "t": [0.0, 2.0],
                    "D": [0.0, 1e-2], "U": {"x": [0.0, 0.0], "y": [0.0, 0.0]}},
        "tracer": {"type": "nee"},
    }
    if correlation:
        cfg["illumination2"] = ill
        cfg["view2"] = view
    return cfg, 2


def homogeneous_3d(batch_size=64, full_iteration=1):
    d = {"x": [0.0, 0.1, -0.2], "y": [0.0, 0.05, 0.1], "z": [1.0, 0.99, 0.97]}
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 1.0, "seed": 2},
        "scattering": {"type": ["HG"], "amplitudeFunction": [0.7]},
        "medium": {"type": "Homogeneous", "boxMin": {"x": [-5.0], "y": [-5.0], "z": [0.0]},
                   "boxMax": {"x": [5.0], "y": [5.0], "z": [4.0]}, "sigs": 1.0},
        "illumination": {"type": "FarField", "direction": d}, "view": {"type": "FarField", "direction": d},
        "sampler": {"type": "TemporalSampler", "t": [0.0], "D": [0.0, 0.0],
                    "U": {"x": [0.0, 0.0], "y": [0.0, 0.0], "z": [0.0, 0.0]}},
        "tracer": {"type": "nee"},
    }
    return cfg, 3


def long_paths_3d(batch_size=64, full_iteration=2):
    """Point sources inside an optically thick homogeneous cube (optical
    radius 20, no absorption): nearly every path runs past 64 vertices, so
    the walk's overflow blocks are used and the default overflow pool runs dry
    (sstmc_render walks the chunk again with a grown pool; the fixed-scratch
    sstmc_render_static replays the listed paths in the write pass)."""
    ill = {"type": "PointSource", "location": {"x": [0.0, 0.5], "y": [0.0, -0.5], "z": [5.0, 5.0]}}
    view = {"type": "PointSource", "location": {"x": [0.0, 2.0, -1.0], "y": [0.0, 0.0, 1.0], "z": [12.0, 12.0, 12.0]}}
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 1.0, "seed": 9},
        "scattering": {"type": ["HG"], "amplitudeFunction": [0.4]},
        "medium": {"type": "Homogeneous", "boxMin": {"x": [-5.0], "y": [-5.0], "z": [0.0]},
                   "boxMax": {"x": [5.0], "y": [5.0], "z": [10.0]}, "sigs": 4.0},
        "illumination": ill, "view": view, "illumination2": ill, "view2": view,
        "sampler": {"type": "TemporalCorrelationSampler", "t": [0.5, 2.0],
                    "D": [0.0, 1e-3], "U": {"x": [0.0, 0.0], "y": [0.0, 0.0], "z": [0.0, 0.0]}},
        "tracer": {"type": "nee"},
    }
    return cfg, 3


def with_cbs(scene):
    """The same scene with coherent backscattering (tracer.isCBS)."""
    cfg, dims = scene
    cfg = dict(cfg)
    cfg["tracer"] = {"type": "nee", "isCBS": True}
    return cfg, dims


def reciprocal_far_3d(cbs: bool = True, batch_size=64, full_iteration=2):
    """Far-field field scene whose views are the illuminations reversed
    (d_v = -d_l, same order), HG scattering in a two-material grid: with CBS
    the rendered field is symmetric, u[l=k][v=j] == u[l=j][v=k]."""
    d = {"x": [0.0, 0.25, -0.2, 0.1], "y": [0.0, 0.1, 0.15, -0.3], "z": [1.0, 0.96, 0.97, 0.95]}
    n = np.sqrt(np.array(d["x"]) ** 2 + np.array(d["y"]) ** 2 + np.array(d["z"]) ** 2)
    dl = {k: np.array(v) / n for k, v in d.items()}
    dv = {k: -v for k, v in dl.items()}
    grid = np.array([[[1, 2], [2, 1]], [[2, 2], [1, 1]]], dtype=np.uint32)
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 0.8, "seed": 4},
        "scattering": {"type": ["HG", "HG", "HG"], "amplitudeFunction": [0.0, 0.6, 0.3]},
        "medium": {"type": "Heterogeneous", "xAxis": [-4.0, 0.5, 4.0], "yAxis": [-4.0, -1.0, 4.0], "zAxis": [0.0, 1.5, 3.0],
                   "materialGrid": grid, "sigs": [0.0, 1.2, 0.8], "siga": [0.0, 0.02, 0.05]},
        "illumination": {"type": "FarField", "direction": dl}, "view": {"type": "FarField", "direction": dv},
        "sampler": {"type": "TemporalSampler", "t": [0.0, 1.0], "D": [0.0, 0.0, 0.0],
                    "U": {"x": [0.0, 0.0, 0.0], "y": [0.0, 0.0, 0.0], "z": [0.0, 0.0, 0.0]}},
        "tracer": {"type": "nee", "isCBS": cbs},
    }
    return cfg, 3


def reciprocal_point_2d(cbs: bool = True, batch_size=64, full_iteration=2):
    """2D point sources with the views at the illumination positions, HG
    scattering and moving scatterers (temporal amplitude): with CBS the field
    is symmetric in (l, v)."""
    pts = {"x": [-3.0, 0.5, 2.5], "y": [-6.5, -6.5, -6.0]}
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 0.6, "seed": 8},
        "scattering": {"type": ["HG", "HG"], "amplitudeFunction": [0.5, 0.5]},
        "medium": {"type": "Heterogeneous", "xAxis": [-5.0, 5.0], "yAxis": [-5.0, 5.0],
                   "materialGrid": np.ones((1, 1), np.uint32), "sigs": [0.0, 0.9], "siga": [0.0, 0.03]},
        "illumination": {"type": "PointSource", "location": pts}, "view": {"type": "PointSource", "location": pts},
        "sampler": {"type": "TemporalSampler", "t": [0.0, 1.5, -1.0],
                    "D": [0.0, 3e-3], "U": {"x": [0.0, 0.02], "y": [0.0, 0.0]}},
        "tracer": {"type": "nee", "isCBS": cbs},
    }
    return cfg, 2


def hg_table(g: float, n: int, dims: int, phase: float = 0.4) -> np.ndarray:
    """A tabular amplitude: sqrt of the HG pdf on n equal angle steps over
    0..pi (3D) or 0..2pi (2D), with a phase ramp exp(i phase theta) so that
    the amplitudes are complex."""
    th = np.linspace(0.0, np.pi if dims == 3 else 2.0 * np.pi, n)
    c = np.cos(th)
    dn = 1.0 + g * g - 2.0 * g * c
    pdf = (1.0 - g * g) / dn ** (1.5 if dims == 3 else 1.0)
    return np.sqrt(pdf) * np.exp(1j * phase * th)


def reciprocal_corr(make, cbs: bool = True):
    """The correlation-sampler version of a reciprocal scene: u2 sources equal
    to u1, Brownian D only (static scatterers, no drift)."""
    cfg, dims = make(cbs=cbs)
    cfg = dict(cfg)
    cfg["illumination2"] = cfg["illumination"]
    cfg["view2"] = cfg["view"]
    nm = len(np.atleast_1d(cfg["medium"]["sigs"]))
    zeros = [0.0] * nm
    U = {"x": zeros, "y": zeros} if dims == 2 else {"x": zeros, "y": zeros, "z": zeros}
    cfg["sampler"] = {"type": "TemporalCorrelationSampler", "t": [0.5, 1.5, 3.0],
                      "D": [0.0] + [2e-3 * (i + 1) for i in range(nm - 1)], "U": U}
    return cfg, dims


def tabular_field_3d(batch_size=64, full_iteration=2):
    """3D field sampler, point sources, a tabular material next to an HG one,
    moving scatterers (per-tick positions)."""
    cfg, dims = field_point_3d(batch_size=batch_size, full_iteration=full_iteration)
    cfg = dict(cfg)
    cfg["scattering"] = {"type": ["Tabular", "HG", "Tabular"],
                         "amplitudeFunction": [hg_table(0.7, 181, 3), 0.6, hg_table(0.2, 91, 3, phase=-0.8)]}
    return cfg, dims


def tabular_corr_2d(sym: bool = True, batch_size=64, full_iteration=2):
    """2D correlation sampler with a tabular material (far-field sources);
    sym=False gives u2 different illuminations and drift, so the u1 and u2
    amplitudes differ (complex products)."""
    cfg, dims = corr_far_2d_drift(batch_size=batch_size, full_iteration=full_iteration)
    cfg = dict(cfg)
    cfg["scattering"] = {"type": ["Tabular", "HG", "Tabular"],
                         "amplitudeFunction": [hg_table(0.85, 361, 2), 0.3, hg_table(0.5, 200, 2, phase=1.1)]}
    if sym:
        cfg["illumination2"] = cfg["illumination"]
        cfg["view2"] = cfg["view"]
        cfg["sampler"] = dict(cfg["sampler"], U={"x": [0.0, 0.0, 0.0], "y": [0.0, 0.0, 0.0]})
    return cfg, dims


def correlation_wide(geometric: bool = True, batch_size=24, full_iteration=2):
    """The bench geometry at 100 x 100 sources and 12 lags: two tick chunks in
    the single-scattering and view kernels (the second starts at tick 8), two
    view passes, the 8-element-per-lane illumination variant; geometric=False
    gives irregular lags (no tick chain)."""
    cfg, dims = wl.correlation_3d(batch_size=batch_size, full_iteration=full_iteration, n_side=10, n_lags=12, dt=0.7)
    cfg = dict(cfg)
    if not geometric:
        cfg["sampler"] = dict(cfg["sampler"], t=np.array([0.3, 0.9, 1.0, 2.2, 3.1, 3.3, 4.8, 5.0, 6.5, 7.7, 8.1, 9.9]))
    return cfg, dims


def forced_bin_3d(batch_size=64, full_iteration=2):
    """3D field sampler with isForcedInsideBin: the point-source scene with
    motion large enough (Brownian D and drift U against 4-5 unit cells) that
    about half of the ticks leave their vertex's cell."""
    cfg, dims = field_point_3d(batch_size=batch_size, full_iteration=full_iteration)
    cfg["sampler"]["D"] = [0.0, 0.08, 0.2]
    cfg["sampler"]["U"] = {"x": [0.0, 0.6, 0.0], "y": [0.0, 0.0, -0.4], "z": [0.0, 0.2, 0.0]}
    cfg["sampler"]["isForcedInsideBin"] = True
    return cfg, dims


def forced_bin_2d(batch_size=64, full_iteration=2):
    """2D field sampler with isForcedInsideBin, far-field sources, a 4 x 3 grid,
    one static material next to a moving one, ticks on both sides of zero."""
    d = wl._farfield_fan(6)
    d2 = wl._farfield_fan(5, 0.3)
    grid = np.array([[1, 2, 1], [2, 2, 1], [1, 2, 2], [2, 1, 1]], dtype=np.uint32)
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 0.9, "seed": 11},
        "scattering": {"type": ["HG", "HG", "HG"], "amplitudeFunction": [0.3, 0.7, 0.5]},
        "medium": {"type": "Heterogeneous", "xAxis": [-6.0, -3.0, 0.0, 2.5, 6.0], "yAxis": [-5.0, -1.0, 2.0, 5.0],
                   "materialGrid": grid, "sigs": [0.0, 0.7, 1.2], "siga": [0.0, 0.02, 0.0]},
        "illumination": {"type": "FarField", "direction": d}, "view": {"type": "FarField", "direction": d2},
        "sampler": {"type": "TemporalSampler", "t": [-2.0, -1.0, 0.0, 1.0, 2.0, 3.5],
                    "D": [0.0, 0.0, 0.15], "U": {"x": [0.0, 0.0, 0.5], "y": [0.0, 0.0, -0.3]},
                    "isForcedInsideBin": True},
        "tracer": {"type": "nee"},
    }
    return cfg, 2


def vmf_mixture(mus, alphas, iso_amp=0.28209479177387814):
    """A vMF-mixture amplitude cell: lobes e^{mu (c - 1)} scaled to the 3D
    isotropic amplitude (mixtureC = log(iso_amp) - mu)."""
    mus = np.asarray(mus, dtype=np.float64)
    return {"mixtureMu": mus, "mixtureC": np.log(iso_amp) - mus, "mixtureAlpha": np.asarray(alphas, dtype=np.float64)}


VMF_FORWARD = ([0.0, 3.5, 22.0], [0.35, 0.45, 0.2])
VMF_TWO_SIDED = ([0.0, 6.0, -0.8], [0.3, 0.5, 0.4])   # a backward lobe: negative-kappa pairs


def with_vmf(scene, lobes=(VMF_FORWARD, VMF_TWO_SIDED)):
    """The scene with material 0 an isotropic-like vMF (mu = 0) and materials
    1, 2 (when present) the given vMF mixtures; further materials keep theirs."""
    cfg, dims = scene
    cfg = dict(cfg)
    sc = cfg["scattering"]
    types = list(sc["type"]) if not isinstance(sc["type"], str) else [sc["type"]]
    amps = list(sc.get("amplitudeFunction", [0.0] * len(types)))
    types[0], amps[0] = "vMF", vmf_mixture([0.0], [1.0])
    for i, (mu, al) in enumerate(lobes):
        if 1 + i < len(types):
            types[1 + i], amps[1 + i] = "vMF", vmf_mixture(mu, al)
    cfg["scattering"] = {"type": types, "amplitudeFunction": amps}
    return cfg, dims


def reciprocal_far_3d_vmf(cbs: bool = True, batch_size=64, full_iteration=2):
    """The reciprocal far-field scene with vMF mixtures: a vMF amplitude depends on
    the scattering cosine only, so with CBS the field is symmetric in (l, v)."""
    return with_vmf(reciprocal_far_3d(cbs=cbs, batch_size=batch_size, full_iteration=full_iteration))


def vmf_iso_mixed_3d(correlation: bool, batch_size=64, full_iteration=2):
    """Every material isotropic with vMF mixtures among them (all |mu| <= 1e-4,
    one mixture not normalised to the isotropic amplitude), point illuminations
    and far-field views: point sources take the isotropic amplitude, far-field
    ones the mixture's (PointSource.cuh:347-399, FarField.cuh:546-599)."""
    cfg, dims = field_point_3d(moving=not correlation, batch_size=batch_size, full_iteration=full_iteration)
    cfg = dict(cfg)
    cfg["scattering"] = {"type": ["vMF", "Isotropic", "vMF"],
                         "amplitudeFunction": [vmf_mixture([0.0], [1.0]), 0.0, vmf_mixture([0.0, 5e-5], [1.0, 0.8])]}
    th = np.linspace(-0.3, 0.3, 4)
    cfg["view"] = {"type": "FarField", "direction": {"x": np.sin(th), "y": 0.1 * np.sin(th), "z": np.cos(th)}}
    if correlation:
        cfg["illumination2"], cfg["view2"] = cfg["illumination"], cfg["view"]
        cfg["sampler"] = {"type": "TemporalCorrelationSampler", "t": [0.5, 1.0, 2.0], "D": [0.0, 2e-3, 5e-3],
                          "U": {"x": [0.0, 0.0, 0.0], "y": [0.0, 0.0, 0.0], "z": [0.0, 0.0, 0.0]}}
    return cfg, dims


def vmf_corr_3d(batch_size=96, full_iteration=2):
    """The bench geometry (correlation sampler, point sources, one cell) with a
    forward-peaked vMF mixture."""
    cfg, dims = wl.correlation_3d(batch_size=batch_size, full_iteration=full_iteration, n_side=4, n_lags=4)
    cfg = dict(cfg)
    cfg["scattering"] = {"type": ["vMF", "vMF"],
                         "amplitudeFunction": [vmf_mixture([0.0], [1.0]), vmf_mixture(*VMF_FORWARD)]}
    return cfg, dims


def vmf_corr_drift_3d(batch_size=64, full_iteration=2):
    """Correlation sampler, 3D, vMF mixtures, drift U != 0 and u2 illuminations
    shifted from u1: the complex route (u1 amplitude x conj(u2 amplitude))."""
    cfg, dims = vmf_corr_3d(batch_size=batch_size, full_iteration=full_iteration)
    cfg = dict(cfg)
    ill = cfg["illumination"]
    loc = {k: np.asarray(v, dtype=np.float64) for k, v in ill["location"].items()}
    cfg["illumination2"] = {"type": "PointSource", "location": {"x": loc["x"] + 3.0, "y": loc["y"], "z": loc["z"]}}
    cfg["scattering"] = {"type": ["vMF", "vMF"],
                         "amplitudeFunction": [vmf_mixture([0.0], [1.0]), vmf_mixture(*VMF_TWO_SIDED)]}
    cfg["sampler"] = dict(cfg["sampler"], U={"x": [0.0, 0.4], "y": [0.0, -0.2], "z": [0.0, 0.1]})
    return cfg, dims


def vmf_2d(vmf: bool = True, batch_size=64, full_iteration=2):
    """2D far-field field scene with a vMF material next to an HG one: the
    reference scatters a 2D vMF material isotropically."""
    d = wl._farfield_fan(6)
    d2 = wl._farfield_fan(5, 0.3)
    grid = np.array([[1, 2], [2, 1], [1, 1]], dtype=np.uint32)
    first = ("vMF", vmf_mixture(*VMF_TWO_SIDED)) if vmf else ("Isotropic", 0.0)
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 0.8, "seed": 13},
        "scattering": {"type": [first[0], first[0], "HG"], "amplitudeFunction": [first[1], first[1], 0.6]},
        "medium": {"type": "Heterogeneous", "xAxis": [-6.0, -1.0, 2.0, 6.0], "yAxis": [-5.0, 0.5, 5.0],
                   "materialGrid": grid, "sigs": [0.0, 0.8, 1.5], "siga": [0.0, 0.01, 0.0]},
        "illumination": {"type": "FarField", "direction": d}, "view": {"type": "FarField", "direction": d2},
        "sampler": {"type": "TemporalSampler", "t": [0.0, 1.0], "D": [0.0, 1e-3, 0.0], "U": {"x": [0.0, 0.0, 0.0], "y": [0.0, 0.0, 0.0]}},
        "tracer": {"type": "nee"},
    }
    return cfg, 2


def one_path(correlation: bool):
    """One path per wave, one illumination, one view, one tick."""
    if correlation:
        return wl.correlation_3d(batch_size=1, full_iteration=3, n_side=1, n_lags=1)
    cfg, dims = wl.speckle_2d(batch_size=1, full_iteration=3, n_dirs=2)
    cfg = dict(cfg)
    cfg["illumination"] = {"type": "FarField", "direction": {"x": [0.2], "y": [0.98]}}
    cfg["view"] = {"type": "FarField", "direction": {"x": [-0.1], "y": [0.995]}}
    return cfg, dims


def ragged_corr_3d(batch_size=40, full_iteration=2):
    """The bench geometry with element and tick counts off every tile width:
    33 illuminations, 65 views, 17 lags."""
    cfg, dims = wl.correlation_3d(batch_size=batch_size, full_iteration=full_iteration, n_side=9, n_lags=17)
    cfg = dict(cfg)
    def cut(src, n):
        loc = src["location"]
        return {"type": "PointSource", "location": {k: np.asarray(v)[:n] for k, v in loc.items()}}
    ill, view = cut(cfg["illumination"], 33), cut(cfg["view"], 65)
    cfg.update(illumination=ill, illumination2=ill, view=view, view2=view)
    return cfg, dims


def mostly_misses_3d(batch_size=32, full_iteration=2):
    """A point illumination 30 units from a small, thin box: about 99 % of the
    first-vertex attempts miss, and every miss counts into iter."""
    ill = {"type": "PointSource", "location": {"x": [0.0, 1.0], "y": [0.0, -1.0], "z": [-30.0, -30.0]}}
    view = {"type": "PointSource", "location": {"x": [0.0, 3.0, -2.0], "y": [0.0, 1.0, 2.0], "z": [12.0, 12.0, 12.0]}}
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 1.0, "seed": 9},
        "scattering": {"type": ["HG", "HG"], "amplitudeFunction": [0.5, 0.5]},
        "medium": {"type": "Heterogeneous", "xAxis": [-5.0, 5.0], "yAxis": [-5.0, 5.0], "zAxis": [0.0, 5.0],
                   "materialGrid": np.ones((1, 1, 1), dtype=np.uint32), "sigs": [0.0, 0.3], "siga": [0.0, 0.0]},
        "illumination": ill, "view": view,
        "sampler": {"type": "TemporalSampler", "t": [0.0], "D": [0.0, 0.0], "U": {"x": [0.0, 0.0], "y": [0.0, 0.0], "z": [0.0, 0.0]}},
        "tracer": {"type": "nee"},
    }
    return cfg, 3


def absorbing_2d(batch_size=64, full_iteration=2):
    """Albedo 0.09: most paths end after their first vertex."""
    cfg, dims = wl.speckle_2d(batch_size=batch_size, full_iteration=full_iteration, n_dirs=5)
    cfg = dict(cfg)
    cfg["medium"] = dict(cfg["medium"], sigs=[0.0, 0.3], siga=[0.0, 3.0])
    return cfg, dims


def ten_materials_2d(batch_size=64, full_iteration=2):
    """All ten materials: a 5 x 4 grid of materials 1..9, HG of several g and
    isotropic cells, Brownian motion in some, far-field sources."""
    rng = np.random.default_rng(21)
    grid = rng.integers(1, 10, size=(5, 4)).astype(np.uint32)
    grid.ravel()[:9] = np.arange(1, 10)
    types = ["HG", "HG", "Isotropic", "HG", "HG", "Isotropic", "HG", "HG", "Isotropic", "HG"]
    amps = [0.0, 0.5, 0.0, -0.3, 0.9, 0.0, 0.1, 0.7, 0.0, 0.2]
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 0.9, "seed": 17},
        "scattering": {"type": types, "amplitudeFunction": amps},
        "medium": {"type": "Heterogeneous", "xAxis": np.linspace(-6, 6, 6), "yAxis": np.linspace(-5, 5, 5),
                   "materialGrid": grid, "sigs": [0.0] + list(np.round(rng.uniform(0.3, 1.6, 9), 3)),
                   "siga": [0.0] + list(np.round(rng.uniform(0.0, 0.1, 9), 3))},
        "illumination": {"type": "FarField", "direction": wl._farfield_fan(4)},
        "view": {"type": "FarField", "direction": wl._farfield_fan(3, 0.4)},
        "sampler": {"type": "TemporalSampler", "t": [0.0, 1.5, 3.0],
                    "D": [0.0, 0.0, 2e-3, 0.0, 1e-3, 0.0, 0.0, 4e-3, 0.0, 0.0],
                    "U": {"x": [0.0] * 10, "y": [0.0] * 10}},
        "tracer": {"type": "nee"},
    }
    return cfg, 2


def very_long_paths_2d(batch_size=256, full_iteration=2):
    """Optically thick, nearly non-absorbing 2D medium: paths of hundreds of
    vertices, far past the walk's 64-vertex slots and its default overflow pool."""
    cfg, dims = wl.speckle_2d(batch_size=batch_size, full_iteration=full_iteration, n_dirs=3)
    cfg = dict(cfg)
    cfg["medium"] = dict(cfg["medium"], sigs=[0.0, 4.0], siga=[0.0, 0.002])
    cfg["scattering"] = {"type": ["HG", "HG"], "amplitudeFunction": [0.3, 0.3]}
    return cfg, dims


def far_phases_3d(point: bool, batch_size=64, full_iteration=2):
    """Field sampler with the medium far from the origin and a short wavelength:
    phases of ~1e5 cycles per NEE vector (far-field d.x / lambda or point-source
    |v - x| / lambda) and long path phases, which FP32 alone cannot resolve."""
    rng = np.random.default_rng(23)
    off = np.array([4000.0, -2500.0, 3000.0])
    grid = rng.integers(1, 3, size=(3, 3, 2)).astype(np.uint32)
    if point:
        ill = {"type": "PointSource", "location": {"x": off[0] + rng.uniform(-6, 6, 5), "y": off[1] + rng.uniform(-6, 6, 5),
                                                     "z": np.full(5, off[2] - 3.0)}}
        view = {"type": "PointSource", "location": {"x": off[0] + rng.uniform(-6, 6, 4), "y": off[1] + rng.uniform(-6, 6, 4),
                                                      "z": np.full(4, off[2] + 12.0)}}
    else:
        ill = {"type": "FarField", "direction": {"x": [0.0, 0.2, -0.15], "y": [0.0, 0.1, 0.2], "z": [1.0, 0.97, 0.96]}}
        view = {"type": "FarField", "direction": {"x": [0.05, -0.2, 0.1, 0.3], "y": [0.0, 0.1, -0.25, 0.05], "z": [1.0, 0.95, 0.96, 0.93]}}
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 0.05, "seed": 29},
        "scattering": {"type": ["HG", "HG", "HG"], "amplitudeFunction": [0.4, 0.6, 0.2]},
        "medium": {"type": "Heterogeneous", "xAxis": off[0] + np.linspace(-8, 8, 4), "yAxis": off[1] + np.linspace(-8, 8, 4),
                   "zAxis": off[2] + np.linspace(0, 9, 3), "materialGrid": grid, "sigs": [0.0, 0.6, 1.0], "siga": [0.0, 0.02, 0.01]},
        "illumination": ill, "view": view,
        "sampler": {"type": "TemporalSampler", "t": [0.0], "D": [0.0, 0.0, 0.0], "U": {"x": [0.0] * 3, "y": [0.0] * 3, "z": [0.0] * 3}},
        "tracer": {"type": "nee"},
    }
    return cfg, 3


def gauss_beams_3d(moving: bool = False, iso: bool = False, tilted: bool = False, back: bool = False,
                   n_l: int = 3, n_v: int = 4, batch_size=64, full_iteration=2, equal_lobes: bool = False,
                   fan: bool = False):
    """Focused Gaussian beams (3D field sampler): vMF materials, illumination and
    view beams focused inside a two-material slab (a three-lobe and a two-lobe
    mixture), optionally drifting and diffusing scatterers over three ticks,
    every lobe isotropic, tilted illumination beams, or views looking back
    along -z (backscattering).  equal_lobes: two-lobe mixtures everywhere.
    fan: view beams fanned out in x, each with its own direction."""
    lobes = [([0.0], [1.0]), ([0.0], [1.0]), ([0.0], [1.0])] if iso else \
        [([0.0], [1.0]), ([0.0, 4.0, 15.0], [0.3, 0.5, 0.2]), ([0.0, 2.5], [0.6, 0.4])]
    if equal_lobes:
        lobes = [([0.0, 1.0], [0.5, 0.5]), ([0.0, 4.0], [0.5, 0.5]), ([0.0, 2.5], [0.6, 0.4])]
    cells = [vmf_mixture(m, a) for m, a in lobes]
    xl = np.linspace(-1.5, 1.5, n_l)
    xv = np.linspace(-2.0, 2.0, n_v)
    dl = np.array([0.3, 0.0, 1.0]) / np.hypot(0.3, 1.0) if tilted else np.array([0.0, 0.0, 1.0])
    dv = np.array([0.0, 0.0, -1.0 if back else 1.0])
    t = [0.0, 0.5, 1.0] if moving else [0.0]
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 0.8},
        "scattering": {"type": ["vMF"] * 3, "amplitudeFunction": cells},
        "medium": {"type": "Heterogeneous", "xAxis": [-12.0, 0.0, 12.0], "yAxis": [-12.0, 12.0], "zAxis": [0.0, 4.0, 10.0],
                   "materialGrid": np.array([1, 2, 2, 1]).reshape(2, 1, 2, order="F"), "sigs": [0.0, 0.25, 0.15],
                   "siga": [0.0, 0.01, 0.0]},
        "illumination": {"type": "GaussianBeam",
                         "focalPoint": {"x": xl, "y": 0.2 * xl, "z": np.full(n_l, 3.0)},
                         "focalDirection": {"x": np.full(n_l, dl[0]), "y": np.full(n_l, dl[1]), "z": np.full(n_l, dl[2])},
                         "aperture": 0.4},
        "view": {"type": "GaussianBeam",
                 "focalPoint": {"x": xv, "y": np.zeros(n_v), "z": np.full(n_v, 5.0)},
                 "focalDirection": {"x": np.linspace(-0.3, 0.3, n_v) if fan else np.zeros(n_v), "y": np.zeros(n_v),
                                    "z": np.full(n_v, dv[2])},
                 "aperture": 0.5},
        "sampler": {"type": "TemporalSampler", "t": t, "D": [0.0, 0.02 if moving else 0.0, 0.0],
                    "U": {"x": [0.0, 0.3 if moving else 0.0, 0.0], "y": [0.0, 0.0, 0.0], "z": [0.0, 0.0, 0.0]}},
        "tracer": {"type": "nee"},
    }
    return cfg, 3


def gauss_beams_2d(moving: bool = False, n_l: int = 3, n_v: int = 4, batch_size=64, full_iteration=2):
    """Focused Gaussian beams in 2D (field sampler): beams act as point sources
    at their focal points, with the Bessel-I0 amplitudes of the vMF lobes (the
    walk scatters vMF materials isotropically in 2D)."""
    cells = [vmf_mixture([0.0], [1.0]), vmf_mixture([0.0, 3.0], [0.5, 0.5]), vmf_mixture([0.0, 1.5, 6.0], [0.4, 0.4, 0.2])]
    xl = np.linspace(-1.5, 1.5, n_l)
    xv = np.linspace(-2.0, 2.0, n_v)
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 0.8},
        "scattering": {"type": ["vMF"] * 3, "amplitudeFunction": cells},
        "medium": {"type": "Heterogeneous", "xAxis": [-12.0, 0.0, 12.0], "yAxis": [0.0, 4.0, 10.0],
                   "materialGrid": np.array([[1, 2], [2, 1]], dtype=np.uint32), "sigs": [0.0, 0.25, 0.15],
                   "siga": [0.0, 0.01, 0.0]},
        "illumination": {"type": "GaussianBeam", "focalPoint": {"x": xl, "y": np.full(n_l, 3.0)},
                         "focalDirection": {"x": np.zeros(n_l), "y": np.ones(n_l)}, "aperture": 0.4},
        "view": {"type": "GaussianBeam", "focalPoint": {"x": xv, "y": np.full(n_v, 5.0)},
                 "focalDirection": {"x": np.full(n_v, 0.28), "y": np.full(n_v, 0.96)}, "aperture": 0.5},
        "sampler": {"type": "TemporalSampler", "t": [0.0, 0.5, 1.0] if moving else [0.0],
                    "D": [0.0, 0.02 if moving else 0.0, 0.0],
                    "U": {"x": [0.0, 0.3 if moving else 0.0, 0.0], "y": [0.0, 0.0, 0.0]}},
        "tracer": {"type": "nee"},
    }
    return cfg, 2


def small_scenes():
    """name -> (config, dims)"""
    return {
        "speckle_2d": wl.speckle_2d(batch_size=96, full_iteration=2),
        "correlation_3d": wl.correlation_3d(batch_size=96, full_iteration=2, n_side=4, n_lags=4),
        "transmission_matrix_3d": wl.transmission_matrix_3d(batch_size=32, full_iteration=2, n_dirs=24, grid=(16, 16, 8)),
        "tracking_2d": wl.tracking_2d(batch_size=16, full_iteration=2, n_dirs=8, frames=4),
        "mcx_3d": wl.mcx_validation_3d(mcx_fixture(), batch_size=48, full_iteration=1),
        "field_point_3d": field_point_3d(),
        "field_point_3d_area": field_point_3d(moving=False, area=True),
        "corr_far_2d_drift": corr_far_2d_drift(),
        "point_2d_iso_field": point_2d_iso(False),
        "point_2d_iso_corr": point_2d_iso(True),
        "homogeneous_3d": homogeneous_3d(),
        "long_paths_3d": long_paths_3d(),
        "field_point_3d_cbs": with_cbs(field_point_3d()),
        "point_2d_iso_field_cbs": with_cbs(point_2d_iso(False)),
        "speckle_2d_cbs": with_cbs(wl.speckle_2d(batch_size=48, full_iteration=2, n_dirs=6)),
        "reciprocal_far_3d_cbs": reciprocal_far_3d(),
        "reciprocal_point_2d_cbs": reciprocal_point_2d(),
        "reciprocal_far_3d_corr_cbs": reciprocal_corr(reciprocal_far_3d),
        "reciprocal_point_2d_corr_cbs": reciprocal_corr(reciprocal_point_2d),
        "correlation_wide": correlation_wide(),
        "correlation_wide_irregular": correlation_wide(geometric=False),
        "tabular_field_3d": tabular_field_3d(),
        "tabular_corr_2d": tabular_corr_2d(),
        "tabular_corr_2d_drift": tabular_corr_2d(sym=False),
        "tabular_field_3d_cbs": with_cbs(tabular_field_3d()),
        "forced_bin_3d": forced_bin_3d(),
        "forced_bin_2d": forced_bin_2d(),
        "forced_bin_2d_cbs": with_cbs(forced_bin_2d()),
        "vmf_field_3d": with_vmf(field_point_3d()),
        "vmf_transmission_3d": with_vmf(wl.transmission_matrix_3d(batch_size=32, full_iteration=2, n_dirs=12, grid=(8, 8, 4))),
        "vmf_corr_3d": vmf_corr_3d(),
        "vmf_field_3d_cbs": with_cbs(with_vmf(field_point_3d())),
        "vmf_2d": vmf_2d(),
        "vmf_corr_drift_3d": vmf_corr_drift_3d(),
        "edge_very_long_paths_2d": very_long_paths_2d(),
        "tabular_corr_2d_cbs": with_cbs(tabular_corr_2d()),
        "vmf_corr_3d_cbs": with_cbs(vmf_corr_3d()),
        "mudiff_corr_cbs": mudiff_scene(cbs=True, batch_size=96, full_iteration=2),
        "edge_far_phases_far_3d": far_phases_3d(False),
        "edge_far_phases_point_3d": far_phases_3d(True),
        "reciprocal_far_3d_vmf_cbs": reciprocal_far_3d_vmf(),
        "edge_one_path_corr_3d": one_path(True),
        "edge_one_path_field_2d": one_path(False),
        "corr_far_2d_drift_cbs": with_cbs(corr_far_2d_drift()),
        "vmf_iso_point_far_field_3d": vmf_iso_mixed_3d(False),
        "vmf_iso_point_far_corr_3d": vmf_iso_mixed_3d(True),
        "vmf_corr_drift_3d_cbs": with_cbs(vmf_corr_drift_3d()),
        "gauss_2d": gauss_beams_2d(),
        "gauss_2d_moving": gauss_beams_2d(moving=True),
        "gauss_3d": gauss_beams_3d(),
        "gauss_3d_moving": gauss_beams_3d(moving=True),
        "gauss_3d_iso": gauss_beams_3d(iso=True),
        "gauss_3d_tilted_back": gauss_beams_3d(tilted=True, back=True),
        "gauss_3d_fan": gauss_beams_3d(fan=True),
        "gauss_3d_fan_moving": gauss_beams_3d(fan=True, moving=True),
        "edge_ragged_corr_3d": ragged_corr_3d(),
        "edge_mostly_misses_3d": mostly_misses_3d(),
        "edge_absorbing_2d": absorbing_2d(),
        "edge_ten_materials_2d": ten_materials_2d(),
    }
