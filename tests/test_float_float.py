"""The float-float phase arithmetic of the NEE vectors (csrc/nee.cuh:
two_prod, two_sum, dot_ff, dist_ff, scale_ff, add_ff, frac_ff), restated in
numpy float32 (IEEE round-to-nearest; the FMA error term a*b - round(a*b)
is exact in float64 for float32 a, b), checked against float64 phases: the
phase modulo 1 stays within 2e-7 cycles at phases of up to 1e6 cycles,
where a plain FP32 phase is off by tenths of a cycle.  The GPU parity scenes
`edge_far_phases_*` check the CUDA code itself against the FP64 oracle."""
import numpy as np

f32 = np.float32


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def two_prod(a, b):
    p = f32(a * b)
    return p, f32(np.float64(a) * np.float64(b) - np.float64(p))


def dot_ff(a, b):
    p0, p1, p2 = two_prod(a[0], b[0]), two_prod(a[1], b[1]), two_prod(a[2], b[2])
    s1 = two_sum(p0[0], p1[0])
    s2 = two_sum(s1[0], p2[0])
    return s2[0], f32(f32(f32(s1[1] + s2[1]) + f32(p0[1] + p1[1])) + p2[1])


def scale_ff(x, ih, il):
    p = two_prod(x[0], ih)
    return p[0], f32(p[1] + f32(f32(x[0] * il) + f32(x[1] * ih)))


def dist_ff(v, x):
    d = [two_sum(v[i], f32(-x[i])) for i in range(3)]
    q = [two_prod(d[i][0], d[i][0]) for i in range(3)]
    s1 = two_sum(q[0][0], q[1][0])
    s2 = two_sum(s1[0], q[2][0])
    cross = f32(2.0 * f32(f32(f32(d[0][0] * d[0][1]) + f32(d[1][0] * d[1][1])) + f32(d[2][0] * d[2][1])))
    sl = f32(f32(f32(s1[1] + s2[1]) + f32(f32(q[0][1] + q[1][1]) + q[2][1])) + cross)
    r0 = f32(np.sqrt(s2[0]))
    r2 = two_prod(r0, r0)
    res = f32(f32(f32(s2[0] - r2[0]) - r2[1]) + sl)
    return r0, f32(res / f32(2.0 * r0))


def frac_ff(ph_h, ph_l, t):
    k = f32(np.rint(t[0]))
    f = f32(f32(ph_h + f32(t[0] - k)) + f32(ph_l + t[1]))
    return f32(f - np.rint(f))


def _wrap(x):
    return (x + 0.5) % 1.0 - 0.5


def test_far_field_phase_modulo_one():
    rng = np.random.default_rng(1)
    lam = 0.01
    ih = f32(1.0 / lam)
    il = f32(1.0 / lam - np.float64(ih))
    worst = worst32 = 0.0
    for _ in range(4000):
        o = rng.normal(size=3)
        o = (o / np.linalg.norm(o)).astype(np.float32)
        x = rng.uniform(-1e4, 1e4, 3).astype(np.float32)
        want = _wrap(np.dot(o.astype(np.float64), x.astype(np.float64)) / lam)
        got = frac_ff(f32(0), f32(0), scale_ff(dot_ff(o, x), ih, il))
        worst = max(worst, abs(_wrap(np.float64(got) - want)))
        plain = f32(f32(o[0] * x[0] + o[1] * x[1] + o[2] * x[2]) * f32(1.0 / lam))
        worst32 = max(worst32, abs(_wrap(np.float64(plain - np.rint(plain)) - want)))
    assert worst < 2e-7, worst
    assert worst32 > 1e-2   # plain FP32 cannot resolve these phases


def test_point_phase_modulo_one():
    rng = np.random.default_rng(2)
    lam = 0.02
    ih = f32(1.0 / lam)
    il = f32(1.0 / lam - np.float64(ih))
    worst = 0.0
    for _ in range(4000):
        x = rng.uniform(-5e3, 5e3, 3).astype(np.float32)
        v = (x + rng.uniform(-2e3, 2e3, 3)).astype(np.float32)
        ph = np.float64(rng.uniform(-0.5, 0.5))
        ph_h = f32(ph)
        ph_l = f32(ph - np.float64(ph_h))
        want = _wrap(np.linalg.norm(v.astype(np.float64) - x.astype(np.float64)) / lam + ph)
        got = frac_ff(ph_h, ph_l, scale_ff(dist_ff(v, x), ih, il))
        worst = max(worst, abs(_wrap(np.float64(got) - want)))
    assert worst < 2e-7, worst
