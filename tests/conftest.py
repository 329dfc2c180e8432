import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


def load_stalled(frame):
    """A frozen 48x24x24 system shipped by the reference
    (sandbox/stalled-system/data/frame-11x), as float64 arrays."""
    z = np.load(os.path.join(GOLDEN, f"stalled_frame{frame}.npz"))
    meta = json.loads(str(z["meta"]))
    arr = {k: z[k].astype(np.float64) for k in z.files if k != "meta"}
    return meta, arr


def oracle_pressure(O, shape, h, b, mask, weights, vent=None, levels=3, tol=1e-11, max_iter=400):
    """The FP64 oracle's pressure for A p = b, converged far below any
    solver tolerance (relative residual `tol`), as the reference solution
    that GPU pressures and velocities are compared with."""
    nz = shape[2] if len(shape) > 2 else 1
    w = tuple(weights[:2]) + ((weights[2],) if nz > 1 and len(weights) > 2 and weights[2] is not None else (None,))
    mg = O.Multigrid(shape, h, mask, vent, w, levels=levels, coarse_direct=True)
    x, r, _ = O.pcg_solve(shape, h, b, None, mask, w, mg, "multigrid", tol=tol, max_iter=max_iter)
    assert r["converged"], r
    return x


@pytest.fixture(scope="session")
def libff():
    """libff.so, built in-tree if needed.  GPU tests only."""
    from tsl_array_n_gb300 import build, _lib
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def gpu(libff):
    from tsl_array_n_gb300 import tsl_array_n
    return tsl_array_n.init(0)
