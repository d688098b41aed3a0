"""Pins of the CPU oracle before it is trusted as the parity checker.

* Philox4x32-10 against the published Random123 known-answer vectors.
* The portable FP32 log / sin(pi x) / cos(pi x) of the decision path against
  libm (accuracy) -- the GPU restates the same operations bit for bit.
* Henyey-Greenstein pdf normalisation in 2D and 3D (Scattering.cuh:500-572)
  and |amplitude|^2 == pdf; the HG sampler against the pdf (chi^2).
* Voxel traversal against brute-force fine marching and analytic box exits.
* The reference's own validation fixture: the MCX temporal correlation curve
  of examples/mcxValidation3D.m (tests/golden/mcx_validation.json).
"""
import math

import numpy as np
import pytest

from temporalspecklescode_gb300 import config as cf
from temporalspecklescode_gb300 import workloads as wl
from tests.scenes import mcx_fixture


def test_philox_known_answers(oracle):
    assert oracle.philox([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert oracle.philox([0xffffffff] * 4, [0xffffffff] * 2) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert oracle.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_portable_log_accuracy(oracle):
    xs = np.concatenate([(np.arange(1, 2 ** 16 + 1) * 2.0 ** -16), np.float32(2.0 ** -24) * np.arange(1, 2000)])
    xs = xs.astype(np.float32)
    got = np.array([oracle.logf(float(x)) for x in xs[::7]], dtype=np.float64)
    ref = np.log(xs[::7].astype(np.float64))
    err = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30)
    # a few ulp relative, absolute 1e-7 near x = 1
    assert np.all((err < 4e-7) | (np.abs(got - ref) < 2e-7))


def test_portable_sincospi_accuracy(oracle):
    xs = np.linspace(0.0, 2.0, 40001, dtype=np.float32)
    s = np.zeros(xs.size)
    c = np.zeros(xs.size)
    for i, x in enumerate(xs):
        s[i], c[i] = oracle.sincospif(float(x))
    xd = xs.astype(np.float64)
    assert np.max(np.abs(s - np.sin(np.pi * xd))) < 3e-7
    assert np.max(np.abs(c - np.cos(np.pi * xd))) < 3e-7


@pytest.mark.parametrize("dims,g", [(2, 0.8), (3, 0.9), (2, 0.0), (3, -0.4)])
def test_hg_normalisation(oracle, dims, g):
    cfg, _ = wl.speckle_2d() if dims == 2 else wl.correlation_3d(n_side=2, n_lags=1)
    cfg["scattering"] = {"type": ["HG", "HG"], "amplitudeFunction": [g, g]}
    pc = cf.prepare(cfg, dims)
    if dims == 2:
        th = np.linspace(-np.pi, np.pi, 200001)
        vals = np.array([oracle.phase(pc, 1, math.cos(t)) for t in th[::10]])
        integral = np.trapezoid(vals[:, 1], th[::10])
    else:
        mu = np.linspace(-1, 1, 200001)
        vals = np.array([oracle.phase(pc, 1, m) for m in mu[::10]])
        integral = 2 * np.pi * np.trapezoid(vals[:, 1], mu[::10])
    assert abs(integral - 1.0) < 2e-3
    assert np.allclose(vals[:, 0] ** 2, vals[:, 1], rtol=1e-12)


@pytest.mark.parametrize("dims,g", [(2, 0.8), (3, 0.9), (3, 0.0005), (2, -0.5)])
def test_hg_sampler_matches_pdf(oracle, dims, g):
    cfg, _ = wl.speckle_2d() if dims == 2 else wl.correlation_3d(n_side=2, n_lags=1)
    cfg["scattering"] = {"type": ["HG", "HG"], "amplitudeFunction": [g, g]}
    pc = cf.prepare(cfg, dims)
    n = 200000
    c = oracle.sample_cos(pc, 1, 5, n).astype(np.float64)
    edges = np.linspace(-1, 1, 41)
    hist, _ = np.histogram(c, edges)
    if abs(g) < 0.001:
        # |g| < 0.001: uniform cosine (Scattering.cuh:1049-1052)
        p = np.full(40, 1 / 40)
    elif dims == 3:
        cdf = lambda m: (1 - g * g) / (2 * g) * (1 / np.sqrt(1 + g * g - 2 * g * m) - 1 / (1 + g))
        p = np.diff(cdf(edges))
    else:
        # 2D: the angle is wrapped Cauchy; integrate the pdf over theta for each cos bin
        th = np.linspace(0, np.pi, 400001)
        pdf = (1 - g * g) / (2 * np.pi * (1 + g * g - 2 * g * np.cos(th))) * 2
        cth = np.cos(th)
        p = np.array([np.trapezoid(np.where((cth >= a) & (cth < b), pdf, 0.0), th) for a, b in zip(edges[:-1], edges[1:])])
        p = p / p.sum()
    exp = p * n
    chi2 = np.sum((hist - exp) ** 2 / np.maximum(exp, 1e-9))
    assert chi2 < 90, chi2  # 39 dof; p < 1e-5 above ~90


def test_dda_against_fine_marching(oracle):
    cfg, dims = wl.transmission_matrix_3d(grid=(16, 16, 8))
    pc = cf.prepare(cfg, dims)
    med = cfg["medium"]
    ax = [np.asarray(med[k], dtype=np.float32).astype(np.float64) for k in ("xAxis", "yAxis", "zAxis")]
    grid = np.asarray(med["materialGrid"])
    sigs = np.asarray(med["sigs"]) + np.asarray(med["siga"])
    sigt = (np.asarray(med["sigs"], np.float32) + np.asarray(med["siga"], np.float32)).astype(np.float64)
    rng = np.random.default_rng(3)
    for _ in range(40):
        o = np.array([rng.uniform(-60, 60), rng.uniform(-60, 60), rng.uniform(1, 63)], dtype=np.float32)
        d = rng.normal(size=3)
        d = (d / np.linalg.norm(d)).astype(np.float32)
        steps, t32, t64 = oracle.dda(pc, o, d)
        # brute force: march in tiny steps
        od, dd = o.astype(np.float64), d.astype(np.float64)
        bmin = np.array([a[0] for a in ax]); bmax = np.array([a[-1] for a in ax])
        with np.errstate(divide="ignore"):
            tx = np.where(dd > 0, (bmax - od) / dd, np.where(dd < 0, (bmin - od) / dd, np.inf))
        tend = tx.min()
        ts = np.linspace(0, tend, 200001)
        mid = 0.5 * (ts[1:] + ts[:-1])
        pts = od[None, :] + mid[:, None] * dd[None, :]
        idx = [np.clip(np.searchsorted(a, pts[:, i], side="right") - 1, 0, a.size - 2) for i, a in enumerate(ax)]
        tau = np.sum(sigt[grid[idx[0], idx[1], idx[2]]] * np.diff(ts))
        assert abs(t64 - tau) < 2e-3 * max(1.0, tau), (t64, tau)
        assert abs(t32 - t64) < 1e-4 * max(1.0, tau)
        # each step enters a new voxel: at least the number of distinct voxels visited
        assert steps >= len({(a, b, c) for a, b, c in zip(*idx)}) - 2
    del sigs


def test_single_cell_exit_is_analytic(oracle):
    cfg, dims = wl.speckle_2d()
    pc = cf.prepare(cfg, dims)
    d = np.float32([0.6, 0.8]).astype(np.float64)
    steps, t32, t64 = oracle.dda(pc, (10.0, -20.0, 0.0), (float(d[0]), float(d[1]), 0.0))
    assert steps == 1
    assert abs(t64 - min((50 - 10) / d[0], (50 + 20) / d[1])) < 1e-9


def test_oracle_reproduces_mcx_validation_curve(oracle):
    """The reference validates its correlation sampler against MCX
    (examples/mcxValidation3D.m).  With 1.6e5 paths the oracle reproduces the
    decay of the MCX curve over all 51 lags within 3% and its level within 12%
    (the reference itself uses 1e7 paths for this plot)."""
    fx = mcx_fixture()
    cfg, dims = wl.mcx_validation_3d(fx, batch_size=40000, full_iteration=4)
    pc = cf.prepare(cfg, dims)
    u, it, st = oracle.render(pc, seed=1)
    c = np.abs(u[0, 0, :]) / it
    mcx = np.asarray(fx["mcx_res"])
    shape = (c / c[0]) / (mcx / mcx[0])
    assert np.max(np.abs(shape - 1)) < 0.03, shape
    assert abs(c[0] / mcx[0] - 1) < 0.12, c[0] / mcx[0]


def _sym_err(u):
    """Relative asymmetry of u[l][v] over the first min(Nl, Nv) elements (all ticks)."""
    n = min(u.shape[0], u.shape[1])
    a = u[:n, :n]
    d = a - np.transpose(a, (1, 0, 2))
    return np.linalg.norm(d) / np.linalg.norm(a)


@pytest.mark.parametrize("make,corr", [("reciprocal_far_3d", False), ("reciprocal_point_2d", False),
                                       ("reciprocal_far_3d_vmf", False),
                                       ("reciprocal_far_3d", True), ("reciprocal_point_2d", True)])
def test_cbs_reciprocity(oracle, make, corr):
    """Field CBS (NextEventEstimation.cuh:1212-1235, :1385-1391): with the views
    the reversed illuminations, each path's reversed-path product for (l=k, v=j)
    is its direct product for (l=j, v=k), so the rendered field is symmetric in
    (l, v); without CBS it is not."""
    from tests import scenes
    res = {}
    for cbs in (False, True):
        if corr:   # the correlation sampler's four cross terms (NextEventEstimation.cuh:1237-1378)
            cfg, dims = scenes.reciprocal_corr(getattr(scenes, make), cbs=cbs)
        else:
            cfg, dims = getattr(scenes, make)(cbs=cbs)
        pc = cf.prepare(cfg, dims)
        u, it, st = oracle.render(pc, 21)
        res[cbs] = u[..., 0] if u.ndim == 4 else u
    assert _sym_err(res[True]) < 1e-12
    assert _sym_err(res[False]) > 1e-3


def test_cbs_correlation_drift_reduces_to_static(oracle):
    """Correlation CBS with drifting scatterers evaluates its vectors per tick at
    the displaced positions.  At tick 0 the displacement is zero, so a render
    of t = [0] equals the same scene with U = 0; with a drift of 1e-7 the
    renders over several ticks agree with U = 0 to the displacement's order."""
    from tests.scenes import with_cbs, corr_far_2d_drift
    cfg, dims = with_cbs(corr_far_2d_drift())
    static = dict(cfg, sampler=dict(cfg["sampler"], U={"x": [0.0] * 3, "y": [0.0] * 3}))
    t0 = lambda c: dict(c, sampler=dict(c["sampler"], t=[0.0]))
    u, it, _ = oracle.render(cf.prepare(t0(cfg), dims), 1)
    us, its, _ = oracle.render(cf.prepare(t0(static), dims), 1)
    assert it == its and np.array_equal(u, us)
    tiny = dict(cfg, sampler=dict(cfg["sampler"], U={"x": [0.0, 1e-7, 0.0], "y": [0.0, 0.0, -1e-7]}))
    u, it, _ = oracle.render(cf.prepare(tiny, dims), 1)
    us, its, _ = oracle.render(cf.prepare(static, dims), 1)
    assert it == its
    assert np.abs(u - us).max() <= 1e-4 * np.abs(us).max()


def _tabular_cfg(dims, table, g_other=0.5):
    cfg, _ = wl.speckle_2d() if dims == 2 else wl.correlation_3d(n_side=2, n_lags=1)
    cfg = dict(cfg)
    cfg["scattering"] = {"type": ["Tabular", "HG"], "amplitudeFunction": [table, g_other]}
    return cf.prepare(cfg, dims)


@pytest.mark.parametrize("dims,g", [(2, 0.8), (3, 0.9), (3, 0.3)])
def test_tabular_normalised_like_hg(oracle, dims, g):
    """A table of sqrt(HG pdf) (Scattering.cuh:272-384): after the cross-section
    normalisation the tabular amplitude and (2D) pdf match HG's at the nodes,
    to the table's angular resolution."""
    from tests.scenes import hg_table
    n = 4001
    pc = _tabular_cfg(dims, np.abs(hg_table(g, n, dims)), g)
    th = np.linspace(0.05, 0.95, 7) * np.pi
    for t in th:
        a_tab = oracle.amplitude(pc, 0, math.cos(t))
        a_hg, pdf_hg = oracle.phase(pc, 1, math.cos(t))
        assert abs(a_tab.imag) < 1e-15
        assert abs(a_tab.real / a_hg - 1.0) < 2e-3
        _, pdf_tab = oracle.phase(pc, 0, math.cos(t))
        if dims == 2:   # the 3D evaluation pdf carries sin(theta), as the reference's table
            assert abs(pdf_tab / pdf_hg - 1.0) < 4e-3
        else:
            assert abs(pdf_tab / (pdf_hg * math.sin(t)) - 1.0) < 4e-3


def test_tabular_lookup_is_nearest_entry(oracle):
    """The amplitude is the table entry nearest the angle (round half to even),
    scaled by one real normalisation: the complex phase of each entry is kept."""
    n = 37
    f = (1.0 + np.arange(n)) * np.exp(1j * 0.1 * np.arange(n) ** 1.3)
    pc = _tabular_cfg(3, f)
    step = np.pi / (n - 1)
    ratios = []
    for i in range(n):
        for off in (-0.3, 0.0, 0.3):
            th = min(max(i * step + off * step, 0.0), np.pi)
            a = oracle.amplitude(pc, 0, math.cos(th))
            ratios.append(a / f[i])
    ratios = np.array(ratios)
    assert np.allclose(ratios.imag, 0.0, atol=1e-12)
    assert np.allclose(ratios.real, ratios.real[0], rtol=1e-12)


@pytest.mark.parametrize("dims,g", [(2, 0.7), (3, 0.8)])
def test_tabular_sampler_matches_table(oracle, dims, g):
    """Inverse-cdf sampling of a tabular material (Scattering.cuh:1030-1037):
    the mean scattering cosine of an HG-shaped table is g."""
    from tests.scenes import hg_table
    pc = _tabular_cfg(dims, hg_table(g, 2001, dims))
    c = np.asarray(oracle.sample_cos(pc, 0, 3, 200000), dtype=np.float64)
    assert abs(c.mean() - g) < 0.01


def _cell(ax, v):
    """Cell index as Simulation.cuh:325-367 returns it (n-1 at or past the last edge)."""
    return max(int(np.searchsorted(np.asarray(ax, dtype=np.float32), np.float32(v), side="right")) - 1, 0)


@pytest.mark.parametrize("make", ["forced_bin_3d", "forced_bin_2d"])
def test_forced_inside_bin_restatement(oracle, make):
    """isForcedInsideBin (TemporalSampler.cuh:439-534, 1637-1698), restated
    independently here: the drawn tick r sits on the sampled point, the tick
    chain is the plain one shifted by x - xt[r], and the weights are 1 exactly on
    the ticks between the last tick <= r and the first tick > r that leave the
    sampled point's grid cell (or the box)."""
    from tests import scenes
    cfg, dims = getattr(scenes, make)()
    plain = dict(cfg, sampler=dict(cfg["sampler"], isForcedInsideBin=False))
    pf, pp = cf.prepare(cfg, dims), cf.prepare(plain, dims)
    med = cfg["medium"]
    axes = [med["xAxis"], med["yAxis"]] + ([med["zAxis"]] if dims == 3 else [])
    lo = np.array([a[0] for a in axes], dtype=np.float32)
    hi = np.array([a[-1] for a in axes], dtype=np.float32)
    rng = np.random.default_rng(4)
    zeros = ones = 0
    for pid in range(300):
        x = np.float32(rng.uniform(lo, hi))
        b = int(rng.integers(1, 6))
        xf, w, r = oracle.tick_positions(pf, 9, pid, b, x, 2)
        xp, wp, rp = oracle.tick_positions(pp, 9, pid, b, x, 2)
        assert rp == -1 and np.all(wp == 1.0)
        assert 0 <= r < len(w)
        shift = (x - xp[r, :dims]).astype(np.float32)
        assert np.array_equal(xf[:, :dims], (xp[:, :dims] + shift).astype(np.float32))
        same = [bool(np.all(p[:dims] >= lo) and np.all(p[:dims] <= hi))
                and all(_cell(axes[a], p[a]) == _cell(axes[a], x[a]) for a in range(dims)) for p in xf]
        neg = max([t for t in range(len(w)) if t <= r and not same[t]], default=-1)
        pos = min([t for t in range(len(w)) if t > r and not same[t]], default=len(w))
        want = np.array([1.0 if neg < t < pos else 0.0 for t in range(len(w))], dtype=np.float32)
        assert np.array_equal(w, want)
        zeros += int((w == 0).sum()); ones += int((w == 1).sum())
    assert zeros > 0.2 * (zeros + ones) and ones > 0.2 * (zeros + ones)


def test_forced_inside_bin_without_motion_changes_nothing(oracle):
    """With every material static all ticks sit on the sampled point: forcing
    the drawn tick there moves nothing and no tick leaves the cell."""
    from tests import scenes
    cfg, dims = scenes.field_point_3d(moving=False)
    forced = dict(cfg, sampler=dict(cfg["sampler"], isForcedInsideBin=True))
    u0 = oracle.render(cf.prepare(cfg, dims), 2)[0]
    u1 = oracle.render(cf.prepare(forced, dims), 2)[0]
    assert np.array_equal(u0, u1)


def test_forced_inside_bin_ignored_by_correlation_sampler(oracle):
    """The correlation sampler has no isForcedInsideBin (MatlabInterface.cu:1245-1282):
    the field is accepted and changes nothing."""
    from tests import scenes
    cfg, dims = scenes.corr_far_2d_drift()
    forced = dict(cfg, sampler=dict(cfg["sampler"], isForcedInsideBin=True))
    u0 = oracle.render(cf.prepare(cfg, dims), 2)[0]
    u1 = oracle.render(cf.prepare(forced, dims), 2)[0]
    assert np.array_equal(u0, u1)


def test_forced_inside_bin_weights_the_render(oracle):
    """With motion the forced render differs from the plain one, and zeroed
    ticks lower the summed intensity."""
    from tests import scenes
    cfg, dims = scenes.forced_bin_2d()
    plain = dict(cfg, sampler=dict(cfg["sampler"], isForcedInsideBin=False))
    uf = oracle.render(cf.prepare(cfg, dims), 2)[0]
    up = oracle.render(cf.prepare(plain, dims), 2)[0]
    assert not np.allclose(uf, up)
    assert np.abs(uf).sum() < np.abs(up).sum()


def _vmf_cfg(mus, alphas, cs=None):
    """3D scene with material 1 a vMF mixture (material 0 a mu = 0 lobe)."""
    from tests.scenes import vmf_mixture
    cfg, _ = wl.correlation_3d(n_side=2, n_lags=1)
    cell = vmf_mixture(mus, alphas)
    if cs is not None:
        cell["mixtureC"] = np.asarray(cs, dtype=np.float64)
    cfg["scattering"] = {"type": ["vMF", "vMF"], "amplitudeFunction": [vmf_mixture([0.0], [1.0]), cell]}
    return cf.prepare(cfg, 3)


@pytest.mark.parametrize("mus,alphas", [([0.0, 3.5, 22.0], [0.35, 0.45, 0.2]), ([1.0], [1.0]), ([0.5, 80.0], [0.9, 0.1])])
def test_vmf_pdf_and_amplitude(oracle, mus, alphas):
    """vMF mixture (Scattering.cuh:636-774, 933-1012), restated independently:
    the amplitude is sum_k alpha_k exp(mu_k c + C_k), the pdf integrates to 1
    over the sphere (all kappa >= 0) and is |amplitude|^2 over its integral."""
    pc = _vmf_cfg(mus, alphas)
    mu, al = np.asarray(mus), np.asarray(alphas)
    C = np.log(0.28209479177387814) - mu
    c = np.linspace(-1.0, 1.0, 40001)
    vals = np.array([oracle.phase(pc, 1, float(x)) for x in c[::4]])
    cs = c[::4]
    amp_want = (al[None, :] * np.exp(mu[None, :] * cs[:, None] + C[None, :])).sum(axis=1)
    assert np.allclose(vals[:, 0], amp_want, rtol=1e-12)
    assert abs(2 * np.pi * np.trapezoid(vals[:, 1], cs) - 1.0) < 1e-4
    a2 = vals[:, 0] ** 2
    assert np.allclose(vals[:, 1], a2 / (2 * np.pi * np.trapezoid(a2, cs)), rtol=2e-4)


def test_vmf_negative_kappa_takes_isotropic_normalisation(oracle):
    """A pair with kappa < 1e-12 (here mu = -0.8 with itself) takes the isotropic
    log normalisation -log(4 pi) (SpecialFunctions.cuh:187-203), so its pdf
    integrates to sinh(|kappa|) / |kappa| rather than 1, as in the reference."""
    pc = _vmf_cfg([-0.8], [1.0])
    c = np.linspace(-1.0, 1.0, 20001)
    pdf = np.array([oracle.phase(pc, 1, float(x))[1] for x in c])
    k = 1.6
    assert abs(2 * np.pi * np.trapezoid(pdf, c) - np.sinh(k) / k) < 1e-6


@pytest.mark.parametrize("mus,alphas", [([0.0, 3.5, 22.0], [0.35, 0.45, 0.2]), ([0.5, 80.0], [0.9, 0.1])])
def test_vmf_sampler_matches_pdf(oracle, mus, alphas):
    """The walk samples a lobe pair by its weight and the lobe's cosine by the
    exact inverse cdf: the cosines follow the pdf (chi^2 on 40 equal-mass bins)."""
    pc = _vmf_cfg(mus, alphas)
    n = 200000
    x = oracle.sample_cos(pc, 1, 7, n).astype(np.float64)
    assert np.all(np.abs(x) <= 1.0)
    c = np.linspace(-1.0, 1.0, 400001)
    pdf = np.array([oracle.phase(pc, 1, float(v))[1] for v in c[::20]])
    cdf = np.concatenate([[0.0], np.cumsum(0.5 * (pdf[1:] + pdf[:-1]) * np.diff(c[::20]))]) * 2 * np.pi
    edges = np.interp(np.linspace(0, 1, 41), cdf / cdf[-1], c[::20])
    hist, _ = np.histogram(x, edges)
    chi2 = np.sum((hist - n / 40) ** 2 / (n / 40))
    assert chi2 < 90, chi2


def test_vmf_scatters_isotropically_in_2d(oracle):
    """In 2D the reference's vMF amplitude, pdf and sampler are the isotropic
    ones (Scattering.cuh:899-905, 960-970, 1093-1100): the render equals the one
    with an Isotropic material, bit for bit."""
    from tests.scenes import vmf_2d
    a = oracle.render(cf.prepare(*vmf_2d(True)), 3)[0]
    b = oracle.render(cf.prepare(*vmf_2d(False)), 3)[0]
    assert np.array_equal(a, b)


def test_vmf_all_isotropic_amplitude_split(oracle):
    """Every material isotropic with a vMF among them (all |mu| <= 1e-4): a point
    source's three-point amplitude is the isotropic one, a far-field source's
    the mixture's (here twice the isotropic amplitude: two unit-weight lobes),
    and the single-scattering amplitude follows the illumination's type
    (PointSource.cuh:347-399, FarField.cuh:546-599)."""
    from tests.scenes import vmf_iso_mixed_3d, vmf_mixture
    cfg, dims = vmf_iso_mixed_3d(False)
    cells = cfg["scattering"]["amplitudeFunction"]
    cfg["scattering"] = {"type": cfg["scattering"]["type"],
                         "amplitudeFunction": [cells[0], 0.0, vmf_mixture([0.0, 5e-5], [1.0, 1.0])]}
    pc = cf.prepare(cfg, dims)
    iso = 0.282094791773878143
    assert abs(oracle.amplitude(pc, 2, 0.3) - iso * (1.0 + np.exp(5e-5 * (0.3 - 1.0)))) < 1e-12
    u, it, _ = oracle.render(pc, 1)
    assert np.all(np.isfinite(u)) and np.abs(u).max() > 0


def test_vmf_config_validation():
    """vMF cells need mixtureMu, mixtureC and mixtureAlpha of one length
    (MatlabInterface.cu:827-868) and non-negative, not all zero, weights."""
    from tests.scenes import field_point_3d
    cfg, dims = field_point_3d()
    bad = [{"mixtureMu": [1.0, 2.0], "mixtureC": [0.0], "mixtureAlpha": [1.0, 1.0]},
           {"mixtureMu": [1.0], "mixtureC": [0.0]},
           {"mixtureMu": [1.0], "mixtureC": [0.0], "mixtureAlpha": [-1.0]},
           {"mixtureMu": [1.0], "mixtureC": [0.0], "mixtureAlpha": [0.0]}, 0.5]
    for cell in bad:
        c = dict(cfg, scattering={"type": ["HG", "vMF", "HG"], "amplitudeFunction": [0.1, cell, 0.2]})
        with pytest.raises(cf.ConfigError):
            cf.prepare(c, dims)


@pytest.mark.parametrize("make", ["mostly_misses_3d", "absorbing_2d"])
def test_iter_counts_every_missed_attempt(oracle, make):
    """iter = batchSize x fullIteration + the first-vertex attempts that missed
    (MatlabInterface.cu:1796): the render's iter equals the paths plus the
    per-path miss counts of the same paths, and a scene that mostly misses has
    iter far above its path count."""
    from tests import scenes
    cfg, dims = getattr(scenes, make)()
    pc = cf.prepare(cfg, dims)
    u, it, st = oracle.render(pc, 5)
    n = cfg["simulation"]["batchSize"] * cfg["simulation"]["fullIteration"]
    tr = oracle.trace_paths(pc, 5, 0, n)
    assert it == n + int(np.sum(tr["misses"]))
    assert st["paths"] == n
    if make == "mostly_misses_3d":
        assert it > 50 * n


def test_oracle_reproduces_mudiff_curve_outside_the_cbs_cone(oracle):
    """The reference's own tabular-scattering validation (examples/
    mudiffCBSValidation2D.m against the mudiff solver, examples/data/
    mudiffCBS.mat via tests/golden/make_mudiff_fixture.py): the correlation
    sampler at t = 0 without CBS reproduces the solver's angular intensity
    over all 721 angles outside the coherent-backscattering cone (about 2 %
    per angle at 1e5 paths), and falls short inside it, where the solver
    includes the cone."""
    from tests.scenes import mudiff_fixture, mudiff_scene
    fx = mudiff_fixture()
    cfg, dims = mudiff_scene(cbs=False)
    u, it, st = oracle.render(cf.prepare(cfg, dims), 0)
    ratio = np.abs(u.ravel()) / it / fx["mudiffRes"]
    ang = np.degrees(fx["degList"])
    out = np.abs(ang - 180.0) > 3.0
    assert abs(ratio[out].mean() - 1.0) < 0.03, ratio[out].mean()
    smooth = np.convolve(ratio[out], np.ones(11) / 11, mode="valid")
    assert np.max(np.abs(smooth - 1.0)) < 0.06
    assert ratio[np.argmin(np.abs(ang - 180.0))] < 0.8   # the solver's curve has the CBS peak there


def test_oracle_reproduces_mudiff_cbs_cone(oracle):
    """The same validation with coherent backscattering (tracer.isCBS, the
    correlation sampler's C2-C4 cross terms with the tabular amplitudes): the
    solver's curve is reproduced inside the backscattering cone too, where
    the estimator without CBS falls a third short."""
    from tests.scenes import mudiff_fixture, mudiff_scene
    fx = mudiff_fixture()
    cfg, dims = mudiff_scene(cbs=True, batch_size=2000, full_iteration=25)
    u, it, st = oracle.render(cf.prepare(cfg, dims), 0)
    ratio = np.abs(u.ravel()) / it / fx["mudiffRes"]
    ang = np.degrees(fx["degList"])
    cone = np.abs(ang - 180.0) <= 2.0
    assert np.all(np.abs(ratio[cone] - 1.0) < 0.08), ratio[cone]
    assert abs(ratio[~cone].mean() - 1.0) < 0.03
    assert np.abs(u.imag).max() <= 1e-9 * np.abs(u.real).max()   # u1 == u2, t = 0: real


def test_oracle_field_cbs_reproduces_mudiff(oracle):
    """The field half of examples/mudiffCBSValidation2D.m: the speckle
    intensity |u|^2 / iter averaged over renderings (200 renderings of 500
    paths here) follows the mudiff solver away from backscattering with and
    without CBS, and only with CBS (the reversed-path rows Gv0 / GlSum)
    inside the cone.  Both runs walk the same paths, so the cone's gain is
    the CBS term alone."""
    from tests.scenes import mudiff_fixture, mudiff_scene
    fx = mudiff_fixture()
    ang = np.degrees(fx["degList"])
    cone = np.abs(ang - 180.0) <= 2.0
    out = np.abs(ang - 180.0) > 3.0
    res = {}
    for cbs in (False, True):
        cfg, dims = mudiff_scene(cbs=cbs, correlation=False, batch_size=500, full_iteration=1)
        pc = cf.prepare(cfg, dims)
        acc = np.zeros(ang.size)
        for r in range(200):
            u, it, st = oracle.render(pc, 1000 + r)
            acc += np.abs(u.ravel()) ** 2 / it
        res[cbs] = acc / 200 / fx["mudiffRes"]
    for cbs in (False, True):
        assert abs(res[cbs][out].mean() - 1.0) < 0.03
    assert abs(res[True][cone].mean() - 1.0) < 0.06
    assert res[True][cone].mean() - res[False][cone].mean() > 0.06


def _wood_vmf_cosines(kappa, n, rng):
    """Wood's rejection sampler for the vMF cosine on the sphere (Wood 1994,
    m = 3), the method of the reference's random_vMF_cosine
    (VectorType.cuh:169-203), written from the published algorithm."""
    b = -kappa + np.hypot(kappa, 1.0)
    x0 = (1.0 - b) / (1.0 + b)
    c = kappa * x0 + 2.0 * np.log(1.0 - x0 * x0)
    out = np.empty(0)
    while out.size < n:
        z = rng.uniform(size=2 * n)
        u = rng.uniform(size=2 * n)
        w = (1.0 - (1.0 + b) * z) / (1.0 - (1.0 - b) * z)
        keep = kappa * w + 2.0 * np.log(1.0 - x0 * w) - c >= np.log(u)
        out = np.concatenate([out, w[keep]])
    return out[:n]


@pytest.mark.parametrize("kappa", [0.5, 5.0, 60.0])
def test_vmf_inverse_cdf_matches_wood_sampler(oracle, kappa):
    """The walk draws a vMF lobe's cosine by the exact inverse cdf
    w = 1 + log(v + (1 - v) e^{-2 kappa}) / kappa; the reference runs Wood's
    rejection loop.  Both sample exp(kappa w) on [-1, 1]: a two-sample
    Kolmogorov-Smirnov test does not tell them apart."""
    stats = pytest.importorskip("scipy.stats")
    pc = _vmf_cfg([kappa / 2.0], [1.0])   # one lobe: its pair has kappa = mu + mu
    ours = np.asarray(oracle.sample_cos(pc, 1, 11, 100000), dtype=np.float64)
    wood = _wood_vmf_cosines(kappa, 100000, np.random.default_rng(5))
    assert stats.ks_2samp(ours, wood).pvalue > 1e-3
