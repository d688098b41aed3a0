"""MATLAB .mat files for the sstmc2D / sstmc3D mirror.

The reference is called from MATLAB as ``[u, iter] = sstmc2D(config)`` with a
struct ``config`` (README.md:74-373; MatlabInterface.cu:1565-1825 reads it).
``load_config`` reads such a struct from a .mat file into the dict that
``api.sstmc2D`` / ``api.sstmc3D`` take (same field names; numeric fields keep
MATLAB's index order, so materialGrid stays x-fastest); ``save_result``
writes ``u`` and ``iter`` the way the MEX call returns them; ``run_mat`` does
both around one render.
"""
from __future__ import annotations

from typing import Any, Dict, Tuple

import numpy as np


def _to_py(x: Any) -> Any:
    """A value read by scipy.io.loadmat (struct_as_record=False, squeeze_me=True)
    as plain Python: structs -> dicts, cell arrays -> lists, 0-d -> scalars."""
    from scipy.io.matlab import mat_struct
    if isinstance(x, mat_struct):
        return {k: _to_py(getattr(x, k)) for k in x._fieldnames}
    if isinstance(x, np.ndarray):
        if x.dtype == object:
            return [_to_py(e) for e in x.ravel(order="F")]
        if x.dtype.kind in "US":   # a char matrix: rows padded with blanks
            return str(x.item()).rstrip() if x.ndim == 0 else [str(e).rstrip() for e in x.ravel(order="F")]
        if x.ndim == 0:
            return x.item()
        return x
    if isinstance(x, np.generic):
        return x.item()
    return x


def load_config(path: str, name: str = "config") -> Dict[str, Any]:
    """The struct variable ``name`` of a .mat file as a config dict."""
    from scipy.io import loadmat
    m = loadmat(path, struct_as_record=False, squeeze_me=True)
    if name not in m:
        raise KeyError(f"{path} has no variable {name!r}")
    cfg = _to_py(m[name])
    if not isinstance(cfg, dict):
        raise TypeError(f"{name!r} in {path} is not a struct")
    return cfg


def _to_mat(x: Any) -> Any:
    """Python config values as savemat writes MATLAB ones: lists of strings as
    cell arrays (MATLAB's {'HG', 'Isotropic'}), nested dicts as structs."""
    if isinstance(x, dict):
        return {k: _to_mat(v) for k, v in x.items()}
    if isinstance(x, (list, tuple)) and x and all(isinstance(e, str) for e in x):
        cell = np.empty(len(x), dtype=object)
        cell[:] = list(x)
        return cell
    return x


def save_config(path: str, config: Dict[str, Any], name: str = "config") -> None:
    """Write a config dict as a MATLAB struct (the inverse of load_config)."""
    from scipy.io import savemat
    savemat(path, {name: _to_mat(config)})


def save_result(path: str, u: np.ndarray, iterations: np.ndarray) -> None:
    """Write the render's outputs as the MEX call returns them: u complex
    (Nl x Nv x Nt x renderingsNum, or with a wavelength axis), iter 1 x R."""
    from scipy.io import savemat
    savemat(path, {"u": np.asarray(u), "iter": np.atleast_2d(np.asarray(iterations, dtype=np.float64))})


def run_mat(config_path: str, out_path: str, dims: int, name: str = "config") -> Tuple[np.ndarray, np.ndarray]:
    """Load ``name`` from config_path, render it with sstmc2D / sstmc3D and
    write u and iter to out_path."""
    from . import api
    cfg = load_config(config_path, name)
    u, it = (api.sstmc2D if dims == 2 else api.sstmc3D)(cfg)
    save_result(out_path, u, it)
    return u, it
