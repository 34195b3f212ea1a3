"""Writes tests/golden/fpinputf32rad512.npz: an exact, compact copy of the
reference's only shipped dataset, ``futhark/data/fpinputf32rad512``.

That file holds the five arguments of forwardprojection.main
(futhark/forwardprojection.fut:71-75) in Futhark's text value format: 805
angles in [pi/4, 3pi/4), rhozero -362, deltarho 1, 725 detectors and a
512 x 512 image whose pixels take 10 grey levels.  The copy stores the angles
as float32, the image as uint8 codes into its float32 grey levels (so it
decodes to the identical float32 array), and the SHA-256 of the source file.
The GPU tests run the drop-in programs on it and compare with the oracle;
nothing at run time needs the reference's tree.

Run from the repository root:
    python tests/golden/make_fpinput512.py [path to fpinputf32rad512]
(default path: the reference checkout at /root/reference).
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from synkrotomo_gb300 import fbench, fvalues  # noqa: E402

DEFAULT_SRC = "/root/reference/futhark/data/fpinputf32rad512"
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fpinputf32rad512.npz")


def main(src: str = DEFAULT_SRC) -> str:
    raw = open(src, "rb").read()
    angles, rhozero, deltarho, numrhos, image = fbench.parse_args_for("forwardprojection", fvalues.read_values(raw))
    levels, codes = np.unique(image, return_inverse=True)
    assert levels.size <= 256
    codes = codes.astype(np.uint8)
    assert np.array_equal(levels[codes].astype(np.float32), image)
    np.savez_compressed(OUT, angles=angles.astype(np.float32), rhozero=np.float32(rhozero),
                        deltarho=np.float32(deltarho), numrhos=np.int32(numrhos),
                        levels=levels.astype(np.float32), codes=codes,
                        source_sha256=np.array(hashlib.sha256(raw).hexdigest()))
    return OUT


if __name__ == "__main__":
    print(main(*sys.argv[1:]))
