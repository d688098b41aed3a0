"""ctypes wrapper of the CPU oracle (oracle/) for the tests.

The oracle is test infrastructure: it is only ever the checker.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from temporalspecklescode_gb300 import config as cf

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "_build", "libsstmc_oracle.so")


def build() -> str:
    r = subprocess.run(["make", "-C", os.path.join(ROOT, "oracle")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)
    return LIB


class Oracle:
    def __init__(self):
        build()
        self.lib = C.CDLL(LIB)
        L = self.lib
        dp = C.POINTER(C.c_double)
        L.oracle_render.argtypes = [C.POINTER(cf.SstmcConfig), C.c_uint64, C.c_uint32, C.c_uint32, C.c_int32, dp, dp,
                                    C.POINTER(C.c_uint64)]
        L.oracle_render.restype = C.c_int32
        L.oracle_trace_paths.argtypes = [C.POINTER(cf.SstmcConfig), C.c_uint64, C.c_uint32, C.c_uint32, C.POINTER(cf.PathTrace)]
        L.oracle_trace_paths.restype = C.c_int32
        L.oracle_dda.argtypes = [C.POINTER(cf.SstmcConfig), C.POINTER(C.c_float), C.POINTER(C.c_float), dp, dp]
        L.oracle_dda.restype = C.c_int32
        L.oracle_phase.argtypes = [C.POINTER(cf.SstmcConfig), C.c_int32, C.c_double, dp, dp]
        L.oracle_phase.restype = C.c_int32
        L.oracle_amplitude.argtypes = [C.POINTER(cf.SstmcConfig), C.c_int32, C.c_double, dp, dp]
        L.oracle_amplitude.restype = C.c_int32
        L.oracle_sample_cos.argtypes = [C.POINTER(cf.SstmcConfig), C.c_int32, C.c_uint64, C.c_uint32, C.POINTER(C.c_float)]
        L.oracle_sample_cos.restype = C.c_int32
        L.oracle_logf.argtypes = [C.c_float]
        L.oracle_logf.restype = C.c_float
        L.oracle_sincospif.argtypes = [C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.oracle_tick_positions.argtypes = [C.POINTER(cf.SstmcConfig), C.c_uint64, C.c_uint32, C.c_uint32,
                                            C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_float),
                                            C.POINTER(C.c_float), C.POINTER(C.c_int32)]
        L.oracle_philox.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        fp = C.POINTER(C.c_float)
        ip = C.POINTER(C.c_int32)
        L.oracle_gauss_terms.argtypes = [C.POINTER(cf.SstmcConfig), C.c_int32, C.c_int32, fp, C.c_int32, fp, dp]
        L.oracle_gauss_terms.restype = C.c_int32
        L.oracle_gauss_sample.argtypes = [C.POINTER(cf.SstmcConfig), C.c_uint64, C.c_uint32, fp, C.c_int32, fp, ip, ip, fp]
        L.oracle_gauss_sample.restype = C.c_int32
        L.oracle_bessel_i0.argtypes = [C.c_double, C.c_double, dp, dp]
        L.oracle_bessel_i0.restype = None

    def render(self, pc: cf.PreparedConfig, seed: int, first_wave: int = 0, waves: int | None = None, threads: int = 0):
        m = pc.meta
        waves = m["waves"] if waves is None else waves
        n = m["Nl"] * m["Nv"] * m["Nt"]
        u = np.zeros(2 * n)
        it = np.zeros(1)
        st = np.zeros(4, dtype=np.uint64)
        e = self.lib.oracle_render(pc.ptr(), C.c_uint64(seed), C.c_uint32(first_wave), C.c_uint32(waves), C.c_int32(threads),
                                   u.ctypes.data_as(C.POINTER(C.c_double)), it.ctypes.data_as(C.POINTER(C.c_double)),
                                   st.ctypes.data_as(C.POINTER(C.c_uint64)))
        if e != 0:
            raise RuntimeError(f"oracle_render error {e}")
        uc = (u[0::2] + 1j * u[1::2]).reshape(m["Nt"], m["Nv"], m["Nl"]).transpose(2, 1, 0)
        stats = {"contributions": int(st[0]), "dda_steps": int(st[1]), "vertices": int(st[2]), "paths": int(st[3])}
        return uc, float(it[0]), stats

    def trace_paths(self, pc: cf.PreparedConfig, seed: int, first: int, paths: int):
        from temporalspecklescode_gb300.api import _alloc_trace
        m = pc.meta
        out, tr = _alloc_trace(paths, m["Nl"], m["Nv"], m["Nt"])
        e = self.lib.oracle_trace_paths(pc.ptr(), C.c_uint64(seed), C.c_uint32(first), C.c_uint32(paths), C.byref(tr))
        if e != 0:
            raise RuntimeError(f"oracle_trace_paths error {e}")
        return out

    def dda(self, pc: cf.PreparedConfig, o, d):
        of = (C.c_float * 3)(*o)
        df = (C.c_float * 3)(*d)
        t32, t64 = C.c_double(), C.c_double()
        steps = self.lib.oracle_dda(pc.ptr(), of, df, C.byref(t32), C.byref(t64))
        return steps, t32.value, t64.value

    def phase(self, pc: cf.PreparedConfig, m: int, c: float):
        a, p = C.c_double(), C.c_double()
        e = self.lib.oracle_phase(pc.ptr(), m, c, C.byref(a), C.byref(p))
        assert e == 0
        return a.value, p.value

    def amplitude(self, pc: cf.PreparedConfig, m: int, c: float) -> complex:
        re, im = C.c_double(), C.c_double()
        e = self.lib.oracle_amplitude(pc.ptr(), m, c, C.byref(re), C.byref(im))
        if e != 0:
            raise RuntimeError(f"oracle_amplitude error {e}")
        return complex(re.value, im.value)

    def sample_cos(self, pc: cf.PreparedConfig, m: int, seed: int, n: int):
        out = np.zeros(n, dtype=np.float32)
        e = self.lib.oracle_sample_cos(pc.ptr(), m, C.c_uint64(seed), C.c_uint32(n), out.ctypes.data_as(C.POINTER(C.c_float)))
        assert e == 0
        return out

    def tick_positions(self, pc: cf.PreparedConfig, seed: int, pid: int, b: int, x, m: int):
        """Field sampler: (xt [Nt, 3], weights [Nt], forced tick or -1) of one vertex."""
        nt = int(pc.struct.t_num)
        xt = np.zeros((nt, 3), dtype=np.float32)
        w = np.zeros(nt, dtype=np.float32)
        r = C.c_int32()
        xx = np.asarray(list(x) + [0.0] * (3 - len(x)), dtype=np.float32)
        fp = C.POINTER(C.c_float)
        e = self.lib.oracle_tick_positions(pc.ptr(), C.c_uint64(seed), C.c_uint32(pid), C.c_uint32(b),
                                           xx.ctypes.data_as(fp), m, xt.ctypes.data_as(fp), w.ctypes.data_as(fp), C.byref(r))
        assert e == 0, e
        return xt, w, r.value

    def logf(self, x: float) -> float:
        return self.lib.oracle_logf(x)

    def sincospif(self, x: float):
        s, c = C.c_float(), C.c_float()
        self.lib.oracle_sincospif(x, C.byref(s), C.byref(c))
        return s.value, c.value

    def philox(self, ctr, key):
        k = (C.c_uint32 * 2)(*key)
        c = (C.c_uint32 * 4)(*ctr)
        o = (C.c_uint32 * 4)()
        self.lib.oracle_philox(k, c, o)
        return [int(x) for x in o]

    def gauss_terms(self, pc: cf.PreparedConfig, l: int, v: int, x1, m1: int, x2) -> dict:
        """Gaussian-beam source terms at x1 (material m1) with the path on to x2."""
        a = np.ascontiguousarray(x1, dtype=np.float32)
        b = np.ascontiguousarray(x2, dtype=np.float32)
        out = np.zeros(10)
        e = self.lib.oracle_gauss_terms(pc.ptr(), l, v, a.ctypes.data_as(C.POINTER(C.c_float)), m1,
                                        b.ctypes.data_as(C.POINTER(C.c_float)), out.ctypes.data_as(C.POINTER(C.c_double)))
        if e:
            raise RuntimeError(f"oracle_gauss_terms failed: {e}")
        return {"P": out[0], "pw": out[1], "f_illum": complex(out[2], out[3]), "f_view": complex(out[4], out[5]),
                "fs": complex(out[6], out[7]), "g_illum": out[8], "g_view": out[9]}

    def gauss_sample(self, pc: cf.PreparedConfig, seed: int, n: int, x1=None, beam: int = 0):
        """n beam-sampled first vertices, their materials, beams and second
        directions; with x1 given, n second directions drawn at x1 for `beam`."""
        fix = None if x1 is None else np.ascontiguousarray(x1, dtype=np.float32)
        xyz = np.zeros((n, 3), dtype=np.float32)
        d = np.zeros((n, 3), dtype=np.float32)
        mat = np.zeros(n, dtype=np.int32)
        b = np.zeros(n, dtype=np.int32)
        fp = C.POINTER(C.c_float)
        ip = C.POINTER(C.c_int32)
        e = self.lib.oracle_gauss_sample(pc.ptr(), seed, n, None if fix is None else fix.ctypes.data_as(fp), beam,
                                         xyz.ctypes.data_as(fp), mat.ctypes.data_as(ip), b.ctypes.data_as(ip),
                                         d.ctypes.data_as(fp))
        if e:
            raise RuntimeError(f"oracle_gauss_sample failed: {e}")
        return xyz, mat, b, d

    def bessel_i0(self, z: complex) -> complex:
        re, im = C.c_double(), C.c_double()
        self.lib.oracle_bessel_i0(z.real, z.imag, C.byref(re), C.byref(im))
        return complex(re.value, im.value)
