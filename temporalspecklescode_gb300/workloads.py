"""Seeded synthetic scenes of the benchmark configurations.

Each function returns ``(config, dims)`` with ``config`` a MATLAB-style dict
(see :mod:`config`).  The reference publishes no benchmark scenes; these are
the synthetic stand-ins with the stated shapes and value distributions.
Random draws use ``numpy.random.default_rng(seed)``.
"""
from __future__ import annotations

import math

import numpy as np


def _farfield_fan(n: int, half_angle: float = math.pi / 6):
    th = -half_angle + np.arange(n) * (2 * half_angle) / (n - 1)
    return {"x": np.sin(th), "y": np.cos(th)}


def speckle_2d(batch_size: int = 1024, full_iteration: int = 64, n_dirs: int = 16, seed: int = 0):
    """2D plain method: single-bin box [-50,50]^2, sigs=[0,1], HG g=0.8,
    16 far-field illuminations and views over [-pi/6, pi/6] about +y, t=[0]."""
    d = _farfield_fan(n_dirs)
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "renderingsNum": 1,
                       "lambda": 1.0, "seed": seed},
        "scattering": {"type": ["HG", "HG"], "amplitudeFunction": [0.8, 0.8]},
        "medium": {"type": "Heterogeneous", "xAxis": [-50.0, 50.0], "yAxis": [-50.0, 50.0],
                   "materialGrid": np.ones((1, 1), dtype=np.uint32), "sigs": [0.0, 1.0], "siga": [0.0, 0.0]},
        "illumination": {"type": "FarField", "direction": d},
        "view": {"type": "FarField", "direction": d},
        "sampler": {"type": "TemporalSampler", "t": [0.0], "D": [0.0, 0.0], "U": {"x": [0.0, 0.0], "y": [0.0, 0.0]}},
        "tracer": {"type": "nee"},
    }
    return cfg, 2


def _jittered_lattice(n_side: int, half: float, rng: np.random.Generator):
    cell = 2 * half / n_side
    c = -half + cell * (np.arange(n_side) + 0.5)
    X, Y = np.meshgrid(c, c, indexing="ij")
    X = X.ravel() + rng.uniform(-cell / 4, cell / 4, X.size)
    Y = Y.ravel() + rng.uniform(-cell / 4, cell / 4, Y.size)
    return X, Y


def correlation_3d(batch_size: int = 1 << 20, full_iteration: int = 4, n_side: int = 8, n_lags: int = 8,
                   dt: float = 1.0, seed: int = 0, lattice_seed: int = 2):
    """3D temporal correlation: slab x,y in [-100,100], z in [0,20], sigs=[0,0.5],
    siga=[0,0.01], HG g=0.9; 64 point illuminations on a jittered 8x8 lattice in
    z=-5 and 64 point views in z=25; Brownian D=[0,1e-3], U=0; 8 lags k*dt."""
    rng = np.random.default_rng(lattice_seed)
    ix, iy = _jittered_lattice(n_side, 100.0, rng)
    vx, vy = _jittered_lattice(n_side, 100.0, rng)
    ill = {"type": "PointSource", "location": {"x": ix, "y": iy, "z": np.full(ix.size, -5.0)}}
    view = {"type": "PointSource", "location": {"x": vx, "y": vy, "z": np.full(vx.size, 25.0)}}
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "renderingsNum": 1,
                       "lambda": 1.0, "seed": seed},
        "scattering": {"type": ["HG", "HG"], "amplitudeFunction": [0.9, 0.9]},
        "medium": {"type": "Heterogeneous", "xAxis": [-100.0, 100.0], "yAxis": [-100.0, 100.0], "zAxis": [0.0, 20.0],
                   "materialGrid": np.ones((1, 1, 1), dtype=np.uint32), "sigs": [0.0, 0.5], "siga": [0.0, 0.01]},
        "illumination": ill,
        "view": view,
        "illumination2": ill,
        "view2": view,
        "sampler": {"type": "TemporalCorrelationSampler", "t": dt * np.arange(1, n_lags + 1),
                    "D": [0.0, 1e-3], "U": {"x": [0.0, 0.0], "y": [0.0, 0.0], "z": [0.0, 0.0]}},
        "tracer": {"type": "nee"},
    }
    return cfg, 3


def _cone_dirs(n: int, half_angle_deg: float, rng: np.random.Generator):
    ca = math.cos(math.radians(half_angle_deg))
    ct = rng.uniform(ca, 1.0, n)
    ph = rng.uniform(0.0, 2 * math.pi, n)
    st = np.sqrt(1 - ct * ct)
    return {"x": st * np.cos(ph), "y": st * np.sin(ph), "z": ct}


def transmission_matrix_3d(batch_size: int = 1 << 18, full_iteration: int = 64, n_dirs: int = 1024,
                           grid=(64, 64, 32), seed: int = 0):
    """3D heterogeneous transmission matrix: 64x64x32 voxels over [-64,64]^2 x [0,64],
    materials iid uniform {1..4} (seed 1), sigs=[0,.5,1,2,4], siga=[0,.01,.01,.02,.05],
    HG g=0.85; 1024 far-field illuminations and views on a 20-degree cone about +z
    (seeds 3, 4)."""
    nx, ny, nz = grid
    grid_rng = np.random.default_rng(1)
    mg = grid_rng.integers(1, 5, size=(nx, ny, nz)).astype(np.uint32)
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "renderingsNum": 1,
                       "lambda": 1.0, "seed": seed},
        "scattering": {"type": ["HG"] * 5, "amplitudeFunction": [0.85] * 5},
        "medium": {"type": "Heterogeneous", "xAxis": np.linspace(-64, 64, nx + 1), "yAxis": np.linspace(-64, 64, ny + 1),
                   "zAxis": np.linspace(0, 64, nz + 1), "materialGrid": mg,
                   "sigs": [0.0, 0.5, 1.0, 2.0, 4.0], "siga": [0.0, 0.01, 0.01, 0.02, 0.05]},
        "illumination": {"type": "FarField", "direction": _cone_dirs(n_dirs, 20.0, np.random.default_rng(3))},
        "view": {"type": "FarField", "direction": _cone_dirs(n_dirs, 20.0, np.random.default_rng(4))},
        "sampler": {"type": "TemporalSampler", "t": [0.0], "D": [0.0] * 5,
                    "U": {"x": [0.0] * 5, "y": [0.0] * 5, "z": [0.0] * 5}},
        "tracer": {"type": "nee"},
    }
    return cfg, 3


def tracking_2d(batch_size: int = 1 << 17, full_iteration: int = 64, n_dirs: int = 128, frames: int = 32,
                seed: int = 0):
    """2D spatio-temporal tracking in the form the reference can express: a static
    256x256 grid over [-128,128]^2 whose disc (radius 16, material 2, sigs=4)
    scatterers translate by (0.5, 0) per frame (sampler U of material 2), over
    32 frames t=0..31; background sigs=1, siga=0, HG g=0.7; 128 far-field
    illuminations and views over [-pi/6, pi/6] about +y."""
    n = 256
    c = -128 + (np.arange(n) + 0.5)
    X, Y = np.meshgrid(c, c, indexing="ij")
    mg = np.where(X * X + Y * Y <= 16 * 16, 2, 1).astype(np.uint32)
    d = _farfield_fan(n_dirs)
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "renderingsNum": 1,
                       "lambda": 1.0, "seed": seed},
        "scattering": {"type": ["HG"] * 3, "amplitudeFunction": [0.7] * 3},
        "medium": {"type": "Heterogeneous", "xAxis": np.linspace(-128, 128, n + 1), "yAxis": np.linspace(-128, 128, n + 1),
                   "materialGrid": mg, "sigs": [0.0, 1.0, 4.0], "siga": [0.0, 0.0, 0.0]},
        "illumination": {"type": "FarField", "direction": d},
        "view": {"type": "FarField", "direction": d},
        "sampler": {"type": "TemporalSampler", "t": np.arange(frames, dtype=float), "D": [0.0, 0.0, 0.0],
                    "U": {"x": [0.0, 0.0, 0.5], "y": [0.0, 0.0, 0.0]}},
        "tracer": {"type": "nee"},
    }
    return cfg, 2


def frame_lags(frames: int) -> np.ndarray:
    """The non-negative lags t2 - t1 of the frame pairs (t1, t2) of `frames`
    frames 0 .. frames-1: 0 .. frames-1 (the negative ones follow by
    conjugation, `frame_pairs`)."""
    return np.arange(frames, dtype=float)


def tracking_2d_pairs(batch_size: int = 1 << 17, full_iteration: int = 64, n_dirs: int = 128, frames: int = 32,
                      seed: int = 0):
    """2D spatio-temporal tracking as frame-pair correlations, in the form the
    reference expresses tracking (examples/trackingLinearMotion.m:61-76,
    examples/spatioTemporalCorrelation2D.m:62-84): the correlation sampler
    with illumination2 = illumination and view2 = view, the disc material's
    scatterers drifting by U = (0.5, 0) per frame.

    The medium is the static 256x256 grid of `tracking_2d` (background sigs=1,
    disc of radius 16 with sigs=4, siga=0, HG g=0.7) with 128 far-field
    illuminations and views over [-pi/6, pi/6] about +y.  The correlation
    sampler's estimator for a frame pair (t1, t2) depends on the pair only
    through t2 - t1 (the u1 and u2 paths take the sampled positions displaced
    by -U (t2 - t1) / 2 and +U (t2 - t1) / 2; the grid itself does not move),
    and with identical u1 / u2 sources a negative lag gives, path by path, the
    conjugate of the positive one (the two displacements trade places and every
    u1 x conj(u2) product turns into its conjugate; Brownian terms depend on
    |t2 - t1|).  So the ticks are the `frames` lags 0 .. frames-1
    (`frame_lags`) and `frame_pairs` fills the frames x frames pairs."""
    n = 256
    c = -128 + (np.arange(n) + 0.5)
    X, Y = np.meshgrid(c, c, indexing="ij")
    mg = np.where(X * X + Y * Y <= 16 * 16, 2, 1).astype(np.uint32)
    d = _farfield_fan(n_dirs)
    src = {"type": "FarField", "direction": d}
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "renderingsNum": 1,
                       "lambda": 1.0, "seed": seed},
        "scattering": {"type": ["HG"] * 3, "amplitudeFunction": [0.7] * 3},
        "medium": {"type": "Heterogeneous", "xAxis": np.linspace(-128, 128, n + 1), "yAxis": np.linspace(-128, 128, n + 1),
                   "materialGrid": mg, "sigs": [0.0, 1.0, 4.0], "siga": [0.0, 0.0, 0.0]},
        "illumination": src, "view": src, "illumination2": src, "view2": src,
        "sampler": {"type": "TemporalCorrelationSampler", "t": frame_lags(frames), "D": [0.0, 0.0, 0.0],
                    "U": {"x": [0.0, 0.0, 0.5], "y": [0.0, 0.0, 0.0]}},
        "tracer": {"type": "nee"},
    }
    return cfg, 2


def frame_pairs(u: np.ndarray, frames: int) -> np.ndarray:
    """Correlations of every frame pair from a render over `frame_lags(frames)`
    with identical u1 / u2 sources: C[..., t1, t2] = u[..., t2 - t1] for
    t2 >= t1 and conj(u[..., t1 - t2]) for t2 < t1, for u of shape
    (Nl, Nv, frames, ...) (the tick axis third, as sstmc2D returns it).
    Returns shape (Nl, Nv, frames, frames, ...)."""
    if u.shape[2] != frames:
        raise ValueError(f"u has {u.shape[2]} ticks, expected the {frames} lags of {frames} frames")
    t = np.arange(frames)
    lag = t[None, :] - t[:, None]   # [t1, t2] -> t2 - t1
    C = u[:, :, np.abs(lag)]
    neg = (lag < 0).reshape((1, 1, frames, frames) + (1,) * (u.ndim - 3))
    return np.where(neg, np.conj(C), C)


def _vmf_cell(mus, alphas, amp=0.28209479177387814):
    """vMF-mixture amplitude cell: lobes alpha_k e^{mu_k (c - 1)} scaled to the
    3D isotropic amplitude (mixtureC = log(amp) - mu)."""
    mus = np.asarray(mus, dtype=np.float64)
    return {"mixtureMu": mus, "mixtureC": np.log(amp) - mus, "mixtureAlpha": np.asarray(alphas, dtype=np.float64)}


def confocal_3d(batch_size: int = 1 << 14, full_iteration: int = 1, n_x: int = 8, n_z: int = 8, shifts=(0.0,),
                seed: int = 0):
    """Focused Gaussian beams (3D field sampler): a 200 x 200 x 20 slab of four
    vMF materials (two layers, two halves in x, three forward-peaked lobes
    each), illumination beams along +z focused on an n_x x n_z grid of the
    x-z plane (x in [-8, 8], z in [2, 18]) and view beams focused on the same
    grid shifted along x by each of `shifts`; aperture 0.4, lambda 1.  The
    shape of a confocal scan: Nl = n_x n_z, Nv = Nl x len(shifts)."""
    rng = np.random.default_rng(seed)
    lobes = [([0.0, 1.0, 3.0], [0.5, 0.3, 0.2])] + [
        ([0.0, float(a), float(b)], [0.2, 0.5, 0.3]) for a, b in zip(rng.uniform(2, 6, 4), rng.uniform(10, 40, 4))]
    X, Z = np.meshgrid(np.linspace(-8, 8, n_x), np.linspace(2, 18, n_z), indexing="ij")
    xl, zl = X.ravel(), Z.ravel()
    xv = np.concatenate([xl + s for s in shifts])
    zv = np.tile(zl, len(shifts))
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "lambda": 1.0},
        "scattering": {"type": ["vMF"] * 5, "amplitudeFunction": [_vmf_cell(m, a) for m, a in lobes]},
        "medium": {"type": "Heterogeneous", "xAxis": [-100.0, 0.0, 100.0], "yAxis": [-100.0, 100.0],
                   "zAxis": [0.0, 10.0, 20.0], "materialGrid": np.array([1, 2, 3, 4]).reshape(2, 1, 2, order="F"),
                   "sigs": [0.0, 0.2, 0.1, 0.25, 0.05], "siga": [0.0, 0.0, 0.0, 0.0, 0.0]},
        "illumination": {"type": "GaussianBeam", "focalPoint": {"x": xl, "y": np.zeros_like(xl), "z": zl},
                         "focalDirection": {"x": np.zeros_like(xl), "y": np.zeros_like(xl), "z": np.ones_like(xl)},
                         "aperture": 0.4},
        "view": {"type": "GaussianBeam", "focalPoint": {"x": xv, "y": np.zeros_like(xv), "z": zv},
                 "focalDirection": {"x": np.zeros_like(xv), "y": np.zeros_like(xv), "z": np.ones_like(xv)},
                 "aperture": 0.4},
        "sampler": {"type": "TemporalSampler", "t": [0.0], "D": [0.0] * 5,
                    "U": {"x": [0.0] * 5, "y": [0.0] * 5, "z": [0.0] * 5}},
        "tracer": {"type": "nee"},
    }
    return cfg, 3


WORKLOADS = {
    "speckle_2d": speckle_2d,
    "confocal_3d": confocal_3d,
    "correlation_3d": correlation_3d,
    "transmission_matrix_3d": transmission_matrix_3d,
    "tracking_2d": tracking_2d,
    "tracking_2d_pairs": tracking_2d_pairs,
}


def _lattice_axis(lo: float, hi: float, h: float, R: float) -> np.ndarray:
    """Edges lo:h/2:hi (hi appended if missing), every second edge moved to the
    previous edge + R, as examples/mcxValidation3D.m:32-54 builds them."""
    n = int(np.floor((hi - lo) / (h / 2) + 1e-9)) + 1
    ax = lo + (h / 2) * np.arange(n)
    if ax[-1] != hi:
        ax = np.append(ax, hi)
    ax[1::2] = ax[0:-1:2][: ax[1::2].size] + R
    return ax


def mcx_validation_3d(fx: dict, batch_size: int = 10000, full_iteration: int = 10, seed: int = 0):
    """The MCX validation scene of examples/mcxValidation3D.m (units: cm, s):
    a 1 cm cube of static scatterers with a lattice of dynamic R x R rods
    (Brownian D), isotropic scattering, point source and point view on the
    z = 0 face viSep apart, lambda = 500 nm, correlation sampler."""
    dims_ = fx["dims"]
    h, R = fx["h"], fx["R"]
    xa = _lattice_axis(-dims_[0] / 2, dims_[0] / 2, h, R)
    za = _lattice_axis(0.0, dims_[2], h, R)
    ya = np.array([-dims_[1] / 2, dims_[1] / 2])
    mg = np.ones((xa.size - 1, 1, za.size - 1), dtype=np.uint32)
    mg[0::2, :, 0::2] = 2
    s = 1.0 / fx["MFP"]
    src = {"type": "PointSource", "location": {"x": [-fx["viSep"] / 2], "y": [0.0], "z": [0.0]}}
    view = {"type": "PointSource", "location": {"x": [fx["viSep"] / 2], "y": [0.0], "z": [0.0]}}
    cfg = {
        "simulation": {"batchSize": batch_size, "fullIteration": full_iteration, "renderingsNum": 1,
                       "lambda": 500e-9 * 100, "seed": seed},
        "scattering": {"type": ["HG"] * 3, "amplitudeFunction": [0.0, 0.0, 0.0]},
        "medium": {"type": "Heterogeneous", "xAxis": xa, "yAxis": ya, "zAxis": za, "materialGrid": mg,
                   "sigs": [0.0, s, s], "siga": [0.0, 0.0, 0.0]},
        "illumination": src, "view": view, "illumination2": src, "view2": view,
        "sampler": {"type": "TemporalCorrelationSampler", "t": np.asarray(fx["t"]), "D": [0.0, 0.0, fx["D"]],
                    "U": {"x": [0.0] * 3, "y": [0.0] * 3, "z": [0.0] * 3}},
        "tracer": {"type": "nee"},
    }
    return cfg, 3
