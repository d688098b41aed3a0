"""The oracle's Gaussian-beam sources (3D, GaussianBeam.cuh) on the CPU.

Pins, none of which reads the oracle's own code path twice:
* the source terms (the second-direction density, f of both roles, fs)
  against a second, numpy restatement of GaussianBeam.cuh's formulas written
  here;
* the first-vertex sampler against P_l: the sampled points' axial histogram
  against the distance-bin pdf recovered from P_l on the beam axis, the bin
  pdf's normalisation to B - 1 (the reference's (B - 1) / sum scaling), and
  the transverse offsets' r^2 / 2 w^2(dz) against Exp(1);
* the second-direction sampler against its density (a chi-square over
  direction cells, the density integrated over the sphere to 1 when no lobe
  pair has kappa < 1e-4; the reference's log C = 1 / (4 pi) for such pairs
  makes the density integrate above 1, also checked);
* the 2D beams' complex Bessel I0 against scipy where the reference's
  algorithm holds;
* the refusals (mixed source types, the correlation sampler, CBS, a non-vMF
  material, a focal point outside the medium, no mean view direction).
"""
import numpy as np
import pytest

from temporalspecklescode_gb300 import config as cf
from tests import scenes

B = 1000   # distance bins per beam and lobe (zSamplesNum)


def _prep(cfg):
    return cf.prepare(cfg, 3)


# ---------------- a numpy restatement of the beam terms ----------------

def _vmf_log_norm(x):
    if x < 1e-12:
        return -np.log(4 * np.pi)
    if x < 5.0:
        return np.log(x) - np.log(4 * np.pi * np.sinh(x))
    return np.log(x) - np.log(2 * np.pi) - x


def _lobes(cell):
    mu = np.asarray(cell["mixtureMu"], float)
    return mu, np.asarray(cell["mixtureC"], float) + np.log(np.asarray(cell["mixtureAlpha"], float))


def _two_sinh(z, c):
    r = 0j
    if (c + z).real > -10:
        r += np.exp(c + z)
    if (c - z).real > -10:
        r -= np.exp(c - z)
    return r


class NumpyBeams:
    """GaussianBeam.cuh's terms for one scene, from the config dict."""

    def __init__(self, cfg):
        self.cfg = cfg
        f32 = lambda v: np.asarray(v, dtype=np.float32).astype(np.float64)
        il, vw = cfg["illumination"], cfg["view"]
        self.fl = np.stack([f32(il["focalPoint"][k]) for k in "xyz"], 1)
        self.dl = np.stack([f32(il["focalDirection"][k]) for k in "xyz"], 1)
        self.fv = np.stack([f32(vw["focalPoint"][k]) for k in "xyz"], 1)
        self.dv = np.stack([f32(vw["focalDirection"][k]) for k in "xyz"], 1)
        self.gal, self.gav = 1 / il["aperture"] ** 2, 1 / vw["aperture"] ** 2
        self.nl, self.nv = _vmf_log_norm(self.gal), _vmf_log_norm(self.gav)
        self.k = 2 * np.pi / cfg["simulation"]["lambda"]
        self.cells = [_lobes(c) for c in cfg["scattering"]["amplitudeFunction"]]
        mv = self.dv.mean(0)
        self.mv = mv / np.linalg.norm(mv)
        med = cfg["medium"]
        self.ax = [f32(med[k]) for k in ("xAxis", "yAxis", "zAxis")]
        self.grid = np.asarray(med["materialGrid"]).ravel(order="F")
        self.sigs = np.asarray(med["sigs"], float)

    def material(self, x):
        c = [min(max(np.searchsorted(a, v, side="right") - 1, 0), a.size - 2) for a, v in zip(self.ax, x)]
        nx, ny = self.ax[0].size - 1, self.ax[1].size - 1
        return int(self.grid[c[0] + c[1] * nx + c[2] * nx * ny])

    def f(self, beam, view, pa, pb, m):
        """threePointFunction (GaussianBeam.cuh:818-892)."""
        f0, d, ga, an = (self.fv[beam], self.dv[beam], self.gav, self.nv) if view else (self.fl[beam], self.dl[beam], self.gal, self.nl)
        w0 = (pa - pb) if view else (pb - pa)
        w0 = w0 / np.linalg.norm(w0)
        k = -self.k if view else self.k
        T = ga * d + 1j * k * (pa - f0)
        mu, cc = self.cells[m]
        acc = 0j
        for g, c in zip(mu, cc):
            lnu = an + np.log(2 * np.pi) + c
            s = np.sqrt(np.sum((g * w0 + T) ** 2))
            acc += 2 * np.exp(lnu) if (abs(s.real) < 1e-4 and abs(s.imag) < 1e-4) else _two_sinh(s, lnu) / s
        return acc

    def fs(self, l, v, x, m):
        """threePointFunctionSingle (GaussianBeam.cuh:894-999)."""
        aT = self.gal * self.dl[l] + 1j * self.k * (x - self.fl[l])
        bT = self.gav * self.dv[v] + 1j * self.k * (self.fv[v] - x)
        tc = self.nl + self.nv + 2 * np.log(2 * np.pi)
        mu, cc = self.cells[m]
        acc = 0j
        for g, c0 in zip(mu, cc):
            lnu = tc + c0
            c = 0j
            if abs(g) < 1e-6:
                C, s = np.sqrt(np.sum(aT ** 2)), np.sqrt(np.sum(bT ** 2))
            else:
                g0 = g / np.sqrt(np.sum((g * self.dv[v] + aT) ** 2))
                s = np.sqrt(np.sum((g0 * aT + bT) ** 2))
                w = (g0 * aT).real
                ra = 1 / np.linalg.norm(w)
                C = np.sqrt(np.sum((g * ra * w + aT) ** 2))
                c = -ra * g0 * np.sum(aT * w)
            sb = abs(s.real) > 1e-4 or abs(s.imag) > 1e-4
            cb = abs(C.real) > 1e-4 or abs(C.imag) > 1e-4
            if sb and cb:
                acc += _two_sinh(C + s, c + lnu) / (C * s)
            elif not sb and not cb:
                acc += 4 * np.exp(c + lnu)
            elif not sb:
                acc += 2 * _two_sinh(C, c + lnu) / C
            else:
                acc += 2 * _two_sinh(s, lnu) / s
        return acc

    def pairs(self, l, x1):
        """computeCdfBuffer (GaussianBeam.cuh:489-621): mean directions, log C, weights."""
        fm = self.material(self.fl[l])
        mu, cc = self.cells[fm]
        T = self.gal * self.dl[l] + 1j * self.k * (x1 - self.fl[l])
        lc, lv = [], []
        for g, c in zip(mu, cc):
            if abs(g) < 1e-9:
                C = np.sqrt(np.sum(T ** 2))
                lc.append(C.real - np.log(abs(C)) + c)
                lv.append(np.zeros(3))
            else:
                g0 = g / np.sqrt(np.sum((g * self.mv + T) ** 2))
                cv = (g0 * T).real
                w = cv / np.linalg.norm(cv)
                C = np.sqrt(np.sum((g * w + T) ** 2))
                lc.append(C.real - np.log(abs(C)) + c - w @ cv)
                lv.append(cv)
        M = len(mu)
        conv, logC, wt = [], [], []
        for j in range(M * M):
            i1, i2 = j % M, j // M
            cv = lv[i1] + lv[i2]
            kap = np.linalg.norm(cv)
            lC = 1 / (4 * np.pi) if kap < 1e-4 else _vmf_log_norm(kap)
            conv.append(cv); logC.append(lC); wt.append(np.exp(lc[i1] + lc[i2] - lC - 2 * self.gal))
        wt = np.asarray(wt) / np.sum(wt)
        return np.asarray(conv), np.asarray(logC), wt

    def pw(self, l, x1, o):
        conv, logC, wt = self.pairs(l, x1)
        return float(np.sum(wt * np.exp(conv @ o + logC)))


def _points(rng, n):
    return np.stack([rng.uniform(-9, 9, n), rng.uniform(-9, 9, n), rng.uniform(0.2, 9.8, n)], 1).astype(np.float32)


@pytest.mark.parametrize("variant", [{}, {"tilted": True, "back": True}])
def test_terms_match_numpy_restatement(oracle, variant):
    cfg, _ = scenes.gauss_beams_3d(**variant)
    pc = _prep(cfg)
    nb = NumpyBeams(cfg)
    rng = np.random.default_rng(3)
    x1s, x2s = _points(rng, 24), _points(rng, 24)
    for i in range(24):
        x1, x2 = x1s[i], x2s[i]
        m1 = nb.material(x1.astype(np.float64))
        l, v = i % len(nb.fl), i % len(nb.fv)
        t = oracle.gauss_terms(pc, l, v, x1, m1, x2)
        a, b = x1.astype(np.float64), x2.astype(np.float64)
        o = (b - a) / np.linalg.norm(b - a)
        for got, want in ((t["f_illum"], nb.f(l, False, a, b, m1)), (t["f_view"], nb.f(v, True, a, b, m1)),
                          (t["fs"], nb.fs(l, v, a, m1)), (t["pw"], nb.pw(l, a, o))):
            assert abs(got - want) <= 1e-9 * max(abs(want), 1e-300), (i, got, want)


def test_first_vertex_sampler_matches_pfirst(oracle):
    """One beam along z focused in a one-lobe (mu = 0) material: the sampled
    points follow P_l's axial bin pdf and the transverse Gaussian w^2(dz)."""
    cfg, _ = scenes.gauss_beams_3d(iso=True, n_l=1)
    pc = _prep(cfg)
    nb = NumpyBeams(cfg)
    n = 200_000
    xyz, mat, beam, _ = oracle.gauss_sample(pc, 11, n)
    f, d = nb.fl[0], nb.dl[0]
    z0, z1 = nb.ax[2][0], nb.ax[2][-1]
    dt = (z1 - z0) / B
    # the bin pdf on the axis: P = pdf_b / (2 pi w^2) / (sigs Lz) for the single lobe
    ga, k = nb.gal, nb.k
    zc = z0 + (np.arange(B) + 0.5) * dt
    pdf = np.empty(B)
    for b, z in enumerate(zc):
        x = np.array([f[0], f[1], z], dtype=np.float32)
        m = nb.material(x.astype(np.float64))
        P = oracle.gauss_terms(pc, 0, 0, x, m, x + np.float32(1.0))["P"]
        w2 = ga / k ** 2 + (z - f[2]) ** 2 / ga
        pdf[b] = P * 2 * np.pi * w2 * nb.sigs[m] * (z1 - z0)
    assert abs(pdf.sum() - (B - 1)) < 1e-6 * B
    # axial histogram in 40 groups of 25 bins against the pdf
    zs = xyz[:, 2].astype(np.float64)
    groups = np.clip(((zs - z0) / dt).astype(int), 0, B - 1) // 25
    obs = np.bincount(groups, minlength=B // 25)
    exp = n * pdf.reshape(-1, 25).sum(1) / (B - 1)
    keep = exp > 5
    chi2 = np.sum((obs[keep] - exp[keep]) ** 2 / exp[keep])
    assert chi2 < keep.sum() + 6 * np.sqrt(2 * keep.sum()), chi2
    # transverse offsets: r^2 / (2 w^2(dz)) ~ Exp(1)
    r2 = (xyz[:, 0] - f[0]) ** 2 + (xyz[:, 1] - f[1]) ** 2
    w2 = ga / k ** 2 + (zs - f[2]) ** 2 / ga
    e = np.sort(r2 / (2 * w2))
    ks = np.max(np.abs((np.arange(1, n + 1) / n) - (1 - np.exp(-e))))
    assert ks < 1.7 / np.sqrt(n), ks


def _sphere_grid(nth=240, nph=480):
    ct = np.cos((np.arange(nth) + 0.5) * np.pi / nth)
    ph = (np.arange(nph) + 0.5) * 2 * np.pi / nph
    st = np.sqrt(1 - ct ** 2)
    o = np.stack([np.outer(st, np.cos(ph)), np.outer(st, np.sin(ph)), np.outer(ct, np.ones(nph))], -1).reshape(-1, 3)
    dw = np.outer(np.sin((np.arange(nth) + 0.5) * np.pi / nth) * np.pi / nth, np.full(nph, 2 * np.pi / nph)).ravel()
    return o, dw


def test_second_direction_density_normalisation():
    """Without isotropic lobes the second-direction density integrates to 1 over
    the sphere; with them the reference's log C = 1 / (4 pi) below kappa = 1e-4
    lifts the (iso, iso) pair's mass to 4 pi e^(1 / (4 pi)) times its weight."""
    o, dw = _sphere_grid()
    cfg, _ = scenes.gauss_beams_3d()
    nb = NumpyBeams(cfg)
    x1 = np.array([0.5, 0.3, 3.5])
    for l in range(len(nb.fl)):
        conv, logC, wt = nb.pairs(l, x1)
        dens = (wt[None, :] * np.exp(o @ conv.T + logC[None, :])).sum(1)
        iso = np.linalg.norm(conv, axis=1) < 1e-4
        want = wt[~iso].sum() + wt[iso].sum() * 4 * np.pi * np.exp(1 / (4 * np.pi))
        assert abs(dens @ dw - want) < 2e-4 * want
    # no isotropic lobe: a proper density
    cfg2 = _no_iso(cfg)
    nb2 = NumpyBeams(cfg2)
    conv, logC, wt = nb2.pairs(0, x1)
    assert abs((wt[None, :] * np.exp(o @ conv.T + logC[None, :])).sum(1) @ dw - 1.0) < 2e-4


def _no_iso(cfg):
    cells = [scenes.vmf_mixture([0.0], [1.0]), scenes.vmf_mixture([1.5, 4.0, 15.0], [0.3, 0.5, 0.2]),
             scenes.vmf_mixture([2.5, 0.8], [0.6, 0.4])]
    return dict(cfg, scattering={"type": ["vMF"] * 3, "amplitudeFunction": cells})


def test_second_direction_sampler_matches_density(oracle):
    """Directions drawn for a beam at fixed first vertices against the density
    p_l(x1 -> x1 + o): a chi-square over 12 x 16 cells of (cos theta, phi)."""
    cfg, _ = scenes.gauss_beams_3d(n_l=2)
    cfg = _no_iso(cfg)
    pc = _prep(cfg)
    nb = NumpyBeams(cfg)
    o, dw = _sphere_grid(240, 480)
    ct_edges, ph_edges = np.linspace(-1, 1, 13), np.linspace(-np.pi, np.pi, 17)
    n = 120_000
    for l, x1 in ((0, np.array([-1.4, -0.3, 3.2], np.float32)), (1, np.array([2.0, 0.5, 6.0], np.float32))):
        _, _, _, dirs = oracle.gauss_sample(pc, 5 + l, n, x1=x1, beam=l)
        conv, logC, wt = nb.pairs(l, x1.astype(np.float64))
        dens = (wt[None, :] * np.exp(o @ conv.T + logC[None, :])).sum(1) * dw
        exp = np.histogram2d(o[:, 2], np.arctan2(o[:, 1], o[:, 0]), bins=(ct_edges, ph_edges), weights=dens)[0].ravel()
        obs = np.histogram2d(dirs[:, 2], np.arctan2(dirs[:, 1], dirs[:, 0]), bins=(ct_edges, ph_edges))[0].ravel()
        exp *= n / exp.sum()
        keep = exp > 5
        chi2 = np.sum((obs[keep] - exp[keep]) ** 2 / exp[keep])
        assert chi2 < keep.sum() + 6 * np.sqrt(2 * keep.sum()), (l, chi2, keep.sum())


def test_bessel_i0_restatement(oracle):
    """The 2D beams' I0 (the reference's besseli algorithm): the power series
    below |z| = 5 to 1e-13 of scipy's iv(0, z); the asymptotic modulus-phase
    form of J0(iz) where it holds (|arg z| <= pi/4) to its truncation error,
    2e-4 at |z| = 7 falling to 1e-13 at |z| = 120.
    Near the imaginary axis that form leaves its domain: there the reference's
    values (restated here as they are) differ from I0 at the 10 % level."""
    sp = pytest.importorskip("scipy.special")
    for r in (0.3, 1.0, 2.5, 4.9):
        for th in np.linspace(-np.pi, np.pi, 25):
            z = r * np.exp(1j * th)
            assert abs(oracle.bessel_i0(complex(z)) - sp.iv(0, z)) <= 1e-13 * abs(sp.iv(0, z))
    for r, tol in ((7.0, 2e-4), (10.0, 3e-6), (30.0, 1e-11), (120.0, 1e-13)):
        for th in np.linspace(-np.pi / 4, np.pi / 4, 9):
            z = r * np.exp(1j * th)
            assert abs(oracle.bessel_i0(complex(z)) - sp.iv(0, z)) <= tol * abs(sp.iv(0, z))
    z = 1.0 + 10.0j
    assert abs(oracle.bessel_i0(z) - sp.iv(0, z)) > 0.1 * abs(sp.iv(0, z))
    assert oracle.bessel_i0(0j) == 1.0


@pytest.mark.parametrize("edit", [
    "mixed", "correlation", "cbs", "hg", "focal_outside", "no_mean_view"])
def test_refusals(oracle, edit):
    cfg, dims = scenes.gauss_beams_3d()
    if edit == "mixed":
        cfg = dict(cfg, view={"type": "FarField", "direction": {"x": [0.0], "y": [0.0], "z": [1.0]}})
    elif edit == "correlation":
        cfg = dict(cfg, sampler=dict(cfg["sampler"], type="TemporalCorrelationSampler"),
                   illumination2=cfg["illumination"], view2=cfg["view"])
    elif edit == "cbs":
        cfg = dict(cfg, tracer={"type": "nee", "isCBS": True})
    elif edit == "hg":
        cfg = dict(cfg, scattering={"type": ["vMF", "HG", "vMF"],
                                    "amplitudeFunction": [cfg["scattering"]["amplitudeFunction"][0], 0.5,
                                                          cfg["scattering"]["amplitudeFunction"][2]]})
    elif edit == "focal_outside":
        il = dict(cfg["illumination"], focalPoint=dict(cfg["illumination"]["focalPoint"], z=np.full(3, -1.0)))
        cfg = dict(cfg, illumination=il)
    elif edit == "no_mean_view":
        vw = dict(cfg["view"], focalDirection={"x": [0.0] * 4, "y": [0.0] * 4, "z": [1.0, -1.0, 1.0, -1.0]})
        cfg = dict(cfg, view=vw)
    with pytest.raises(RuntimeError, match=r"\b5\b"):
        oracle.render(cf.prepare(cfg, dims), 1)


def test_render_is_finite_and_counts_misses(oracle):
    """Beam scenes render finite fields; tilted beams place some first vertices
    outside the box, which count as missed paths (iter > batch x fullIteration)."""
    for variant in ({}, {"moving": True}, {"iso": True}, {"tilted": True, "back": True}, "2d"):
        cfg, dims = scenes.gauss_beams_2d() if variant == "2d" else scenes.gauss_beams_3d(**variant)
        u, it, _ = oracle.render(cf.prepare(cfg, dims), 2)
        variant = {} if variant == "2d" else variant
        assert np.all(np.isfinite(u)) and np.abs(u).max() > 0
        n = cfg["simulation"]["batchSize"] * cfg["simulation"]["fullIteration"]
        assert it >= n
        if variant.get("tilted"):
            assert it > n
