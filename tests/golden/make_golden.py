"""Regenerates the golden fixtures in this folder from the reference checkout.

Run where the reference sources are present, with the checkout's root as
the one argument (`python make_golden.py <reference checkout>`); the tests
read only the committed fixtures.  Writes:

  stalled_frame110.npz, stalled_frame112.npz
      The frozen 48x24x24 pressure systems that the reference ships under
      packages/fluxflow/sandbox/stalled-system/data/frame-11{0,2}/ (raw
      little-endian float32, i-fastest; see R/export_system.mjs:105-126),
      repacked losslessly with their meta.json.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ["b", "pressure", "dirichletMask", "ventMask", "weightU", "weightV", "weightW"]


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <reference checkout>")
    base = os.path.join(sys.argv[1], "packages/fluxflow/sandbox/stalled-system/data")
    for frame in ("frame-110", "frame-112"):
        d = os.path.join(base, frame)
        meta = json.load(open(os.path.join(d, "meta.json")))
        arrays = {n: np.fromfile(os.path.join(d, n + ".bin"), dtype="<f4") for n in NAMES}
        out = os.path.join(HERE, "stalled_" + frame.replace("-", "") + ".npz")
        np.savez_compressed(out, meta=json.dumps(meta), **arrays)
        print("wrote", out, os.path.getsize(out))


if __name__ == "__main__":
    sys.exit(main())
