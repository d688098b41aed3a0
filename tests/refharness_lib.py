"""Run the reference's own CUDA path (oracle/refharness.cu, built against the
reference headers staged by oracle/stage_reference.sh) on a config dict.

Test infrastructure: the reference is only ever the checker.  The harness
binaries are built on first use where a GPU runs them (make -C oracle -f
refharness.mk); without the staged headers the callers skip.
"""
from __future__ import annotations

import os
import subprocess
import tempfile

import numpy as np

from temporalspecklescode_gb300 import config as cf

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ODIR = os.path.join(ROOT, "oracle")
STAGED = os.path.join(ODIR, "_ref", "src", "Simulation.cuh")


def available() -> bool:
    return os.path.exists(STAGED)


def build() -> None:
    r = subprocess.run(["make", "-C", ODIR, "-f", "refharness.mk"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout[-4000:] + r.stderr[-4000:])


def _tokens(pc: cf.PreparedConfig, renderings: int, seed: int) -> str:
    c = pc.struct
    dims = c.dims
    mat_num = c.scattering_num if c.scattering_num > 1 else 2
    rd = lambda p, n: np.ctypeslib.as_array(p, shape=(n,)).copy()
    out = [f"batch {c.batch_size}", f"full_iteration {c.full_iteration}", f"renderings {renderings}", f"seed {seed}",
           f"lambda {c.lam!r}"]
    kinds = rd(c.scattering_type, c.scattering_num)
    g = rd(c.scattering_g, c.scattering_num)
    cells = []
    vpos = 0
    for k, x in zip(kinds, g):
        if k == cf.SCATTERING_VMF:
            n = int(c.vmf_n[len(cells)])
            mu, cc, al = (rd(p, vpos + n)[vpos:] for p in (c.vmf_mu, c.vmf_c, c.vmf_alpha))
            vpos += n
            cells.append(f"4 {n} " + " ".join(repr(float(v)) for v in np.concatenate([mu, cc, al])))
        elif k in (cf.SCATTERING_ISOTROPIC, cf.SCATTERING_HG):
            cells.append(f"{int(k)} {float(x)!r}")
        else:
            raise ValueError("the harness builds isotropic, Henyey-Greenstein and vMF materials only")
    if c.scattering_num == 1:   # one cell is material 1 as well (MatlabInterface.cu:750-760)
        cells = cells * 2
    out.append(f"scattering {mat_num} " + " ".join(cells))
    if c.medium_type != cf.MEDIUM_HETEROGENEOUS:
        raise ValueError("the harness builds heterogeneous media only")
    axes = [rd(c.x_axis, c.x_axis_size), rd(c.y_axis, c.y_axis_size)] + ([rd(c.z_axis, c.z_axis_size)] if dims == 3 else [])
    for a, ax in enumerate(axes):
        out.append(f"axis {a} {ax.size} " + " ".join(repr(float(v)) for v in ax))
    cells = int(np.prod([ax.size - 1 for ax in axes]))
    grid = rd(c.material_grid, cells)
    out.append(f"grid {cells} " + " ".join(str(int(v)) for v in grid))
    sigs = rd(c.sigs, mat_num)
    siga = rd(c.siga, mat_num) if c.siga else np.zeros(mat_num)
    out.append(f"materials {mat_num} " + " ".join(f"{float(s)!r} {float(a)!r}" for s, a in zip(sigs, siga)))
    for role, s in enumerate((c.illumination, c.view, c.illumination2, c.view2)):
        if s.type == cf.SOURCE_NONE:
            continue
        if s.is_area_source:
            raise ValueError("the harness builds point sources without isAreaSource")
        xyz = rd(s.xyz, 3 * s.count)
        line = f"source {role} {s.type} {s.count} " + " ".join(repr(float(v)) for v in xyz)
        if s.type == cf.SOURCE_GAUSSIANBEAM:
            line += " " + " ".join(repr(float(v)) for v in rd(s.focal_direction, 3 * s.count)) + f" {float(s.aperture)!r}"
        out.append(line)
    out.append(f"sampler {c.sampler_type}")
    t = rd(c.t, c.t_num)
    out.append(f"ticks {t.size} " + " ".join(repr(float(v)) for v in t))
    D = rd(c.D, mat_num)
    U = rd(c.U, 3 * mat_num)
    out.append(f"motion {mat_num} " + " ".join(f"{float(D[m])!r} {float(U[3 * m])!r} {float(U[3 * m + 1])!r} {float(U[3 * m + 2])!r}"
                                               for m in range(mat_num)))
    if c.is_cbs:
        out.append("cbs 1")
    out.append("end")
    return "\n".join(out) + "\n"


def render(config: dict, dims: int, renderings: int, seed: int, timeout: float = 1800.0):
    """(u of shape (Nl, Nv, Nt, renderings), iter per rendering, trace ms per rendering)."""
    pc = cf.prepare(config, dims)
    exe = os.path.join(ODIR, "_ref", f"refharness{dims}d")
    if not os.path.exists(exe):
        build()
    with tempfile.TemporaryDirectory() as td:
        scene = os.path.join(td, "scene.txt")
        res = os.path.join(td, "u.bin")
        with open(scene, "w") as f:
            f.write(_tokens(pc, renderings, seed))
        r = subprocess.run([exe, scene, res], capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"reference harness failed ({r.returncode}): {r.stderr[-2000:]}")
        vals = np.fromfile(res, dtype=np.float64)
    Nl, Nv, Nt, R = (int(v) for v in vals[:4])
    n = Nl * Nv * Nt
    blk = vals[4:].reshape(R, 2 * n + 2)
    u = (blk[:, 0:2 * n:2] + 1j * blk[:, 1:2 * n:2]).reshape(R, Nt, Nv, Nl).transpose(3, 2, 1, 0)
    return u, blk[:, 2 * n], blk[:, 2 * n + 1]
