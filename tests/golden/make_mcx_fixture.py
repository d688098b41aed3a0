"""Generate tests/golden/mcx_validation.json from the reference's validation data.

Reads examples/data/mcxValidationData.mat of chabner/temporalSpecklesCode (the
external MCX solver curve that examples/mcxValidation3D.m compares the
reference's correlation sampler against) and writes the scene scalars, the
time lags and the MCX correlation curve.  Run once in a checkout where the
reference is available:

    python tests/golden/make_mcx_fixture.py /path/to/temporalSpecklesCode
"""
import json
import os
import sys

import scipy.io as sio


def main(ref_root: str) -> None:
    d = sio.loadmat(os.path.join(ref_root, "examples", "data", "mcxValidationData.mat"))
    out = {
        "source": "examples/data/mcxValidationData.mat (scene of examples/mcxValidation3D.m)",
        "D": float(d["D"].ravel()[0]),
        "MFP": float(d["MFP"].ravel()[0]),
        "R": float(d["R"].ravel()[0]),
        "h": float(d["h"].ravel()[0]),
        "viSep": float(d["viSep"].ravel()[0]),
        "dims": [float(v) for v in d["dims"].ravel()],
        "t": [float(v) for v in d["t"].ravel()],
        "mcx_res": [float(v) for v in d["mcx_res"].ravel()],
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mcx_validation.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(__file__)} <root of the reference checkout>")
    main(sys.argv[1])
