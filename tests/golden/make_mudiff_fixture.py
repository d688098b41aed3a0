"""Generate tests/golden/mudiff_cbs.npz from the reference's validation data.

Reads examples/data/mudiffCBS.mat of chabner/temporalSpecklesCode: the scene
of examples/mudiffCBSValidation2D.m (a 2D square medium of mean free path
MFP, a tabular amplitude function, one far-field illumination along +y and
views at the listed angles) and the external mudiff solver's angular
intensity, which that script compares the reference's correlation and field
samplers against.  Run once in a checkout where the reference is available:

    python tests/golden/make_mudiff_fixture.py /path/to/temporalSpecklesCode
"""
import os
import sys

import numpy as np
import scipy.io as sio


def main(ref_root: str) -> None:
    d = sio.loadmat(os.path.join(ref_root, "examples", "data", "mudiffCBS.mat"))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mudiff_cbs.npz")
    np.savez_compressed(path,
                        MFP=np.float64(d["MFP"].ravel()[0]),
                        x=d["x"].ravel().astype(np.float64),
                        y=d["y"].ravel().astype(np.float64),
                        ampFunc=d["ampFunc"].ravel().astype(np.complex128),
                        degList=d["degList"].ravel().astype(np.float64),
                        mudiffRes=d["mudiffRes"].ravel().astype(np.float64))
    print("wrote", path)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(__file__)} <root of the reference checkout>")
    main(sys.argv[1])
