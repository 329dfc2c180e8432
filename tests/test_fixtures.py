"""Fixture I/O in the reference's on-disk formats (export_system.mjs,
export_system2.mjs): the reference's own frozen 3D systems survive a write
and read unchanged, and what the 2D writer produces is what
cpu_reference.mjs reads (its cross-check of the operator against the
solver's reported residual holds on the written files)."""
import json
import os

import numpy as np
import pytest


def raw_stalled(frame):
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", f"stalled_frame{frame}.npz"))
    return json.loads(str(z["meta"])), {k: z[k] for k in z.files if k != "meta"}


@pytest.mark.parametrize("frame", [110, 112])
def test_system3_round_trip_of_reference_fixture(tmp_path, frame):
    from tsl_array_n_gb300 import fixtures
    meta, arrays = raw_stalled(frame)
    d = str(tmp_path / f"frame-{frame}")
    fixtures.write_system3_arrays(d, meta["resolution"], arrays, meta["gridSpacing"], meta["source"], meta["frame"],
                                  meta["diagnostics"], meta["multigrid"], meta["tolerance"], meta["maxIterations"])
    m2, a2 = fixtures.read_system3(d)
    assert m2 == meta   # every key of the reference's meta.json, same values
    for n in fixtures.SYSTEM3_ARRAYS:
        assert a2[n].dtype == np.dtype("<f4") and np.array_equal(a2[n], arrays[n]), n
        assert os.path.getsize(os.path.join(d, n + ".bin")) == 4 * arrays[n].size


def test_system3_absent_weights_and_size_check(tmp_path):
    from tsl_array_n_gb300 import fixtures
    res = (4, 3, 2)
    n = 24
    a = {"b": np.arange(n, dtype=np.float32), "pressure": np.zeros(n), "dirichletMask": np.zeros(n),
         "ventMask": np.zeros(n), "weightU": None, "weightV": None, "weightW": None}
    fixtures.write_system3_arrays(str(tmp_path), res, a)
    m, r = fixtures.read_system3(str(tmp_path))
    assert r["weightU"] is None and m["dataSizeU"] == [5, 3, 2] and np.array_equal(r["b"], a["b"])
    a["b"] = np.zeros(5)
    with pytest.raises(ValueError):
        fixtures.write_system3_arrays(str(tmp_path), res, a)


def test_system2_is_what_cpu_reference_reads(tmp_path, oracle):
    """A 2D system with pinned cells, solved here in double by the oracle's
    restatement of cpu_reference.mjs's CG, written in the export_system2
    format and read back the way cpu_reference.mjs:35-48 reads it."""
    from tsl_array_n_gb300 import fixtures
    nx, ny, h = 24, 16, (0.5, 0.25)
    rng = np.random.default_rng(2)
    pinned = np.zeros((ny, nx), bool)
    pinned[:, -2:] = True
    pinned = pinned.ravel()
    b = rng.standard_normal(nx * ny)
    b[pinned] = 0.0
    it, rel, x = oracle.cpuref_cg((nx, ny), h, b, pinned)
    assert rel < 1e-6
    resid = float(np.linalg.norm(b - oracle.cpuref_apply((nx, ny), h, x.astype(np.float32), pinned)))
    fixtures.write_system2_arrays(str(tmp_path), (nx, ny), h, b, np.zeros(nx * ny), x,
                                  pinned.astype(np.float32), gpu={"converged": True, "iterations": it,
                                                                  "residual": resid, "stoppedBy": "none"})
    meta = json.load(open(tmp_path / "meta.json"))
    NX, NY = meta["shape"]
    rd = lambda n: np.fromfile(tmp_path / f"{n}.bin", dtype="<f4").astype(np.float64)
    bb, mask, after = rd("b"), rd("dirichletMask") > 0.5, rd("pressureAfter")
    assert (NX, NY) == (nx, ny) and meta["pinned"] == int(pinned.sum()) and meta["cells"] == nx * ny
    assert np.isclose(meta["bNorm"], np.linalg.norm(b.astype(np.float32)))
    # cpu_reference.mjs's cross-check 2: ||b - A pressureAfter|| against the reported residual
    ratio = np.linalg.norm(bb - oracle.cpuref_apply((NX, NY), meta["gridSpacing"], after, mask)) / \
        meta["gpu"]["residual"]
    assert 0.5 < ratio < 2


@pytest.mark.gpu
def test_system3_solve_write_read(gpu, tmp_path, oracle):
    """Rebuild the reference's frame-110 system from its fixture, solve it,
    write what the solver holds and read it back: the same b, the same
    Dirichlet mask (vent cells plus the cells the weights enclose), and a
    pressure that solves the fixture's operator."""
    from tsl_array_n_gb300 import fixtures
    meta, arrays = raw_stalled(110)
    s, b, meta, a = fixtures.solver_from_system3((meta, arrays), multigrid={"numberOfLevels": 4},
                                                 tolerance=1e-5, max_iterations=200)
    d = s.solve(b)
    assert d["converged"] and not d["rejected"], d
    out = str(tmp_path / "sys")
    fixtures.write_system3(out, s, source="solver_from_system3", frame=110)
    m2, a2 = fixtures.read_system3(out)
    assert np.array_equal(a2["b"], arrays["b"])
    assert np.array_equal(a2["dirichletMask"] > 0.5, arrays["dirichletMask"] > 0.5)
    assert np.array_equal(a2["ventMask"] > 0.5, arrays["ventMask"] > 0.5)
    for n in ("weightU", "weightV", "weightW"):
        assert np.array_equal(a2[n], arrays[n])
    assert m2["diagnostics"]["converged"] and m2["multigrid"]["numberOfLevels"] == 4
    mask = arrays["dirichletMask"] > 0.5
    w = (arrays["weightU"], arrays["weightV"], arrays["weightW"])
    ap = oracle.laplacian(tuple(meta["resolution"]), meta["gridSpacing"], a2["pressure"].astype(np.float64), mask, w)
    b64 = arrays["b"].astype(np.float64)
    # the pressure on disk is FP32: its residual evaluated in double carries
    # that rounding (|A dp| ~ 1e-7 |A| |p|), well under 1e-3 of |b|
    assert np.linalg.norm(b64 - ap) / np.linalg.norm(b64) < 1e-3


@pytest.mark.gpu
def test_system2_export_passes_cpu_reference_cross_check(gpu, tmp_path, oracle):
    """A 2D solve (nz = 1) exported in the export_system2 format: the
    operator cpu_reference.mjs rebuilds from the files reproduces the
    residual the solver reported for its own answer (its cross-check 2).
    The tolerance is loose so that the residual at the stop is far above
    the FP32 rounding of the pressure written to disk."""
    from tsl_array_n_gb300 import fixtures, fluxflow as ff
    from tsl_array_n_gb300.tsl_array_n import Field
    nx, ny, h = 64, 48, (1.0, 1.0)
    pinned = np.zeros((ny, nx), bool)
    pinned[:, -3:] = True
    pinned = pinned.ravel()
    s = ff.create_grid_pressure_solver2((nx, ny), h, dirichlet=(pinned, np.zeros(nx * ny)),
                                        multigrid={"numberOfLevels": 3}, tolerance=1e-3)
    rng = np.random.default_rng(4)
    b = rng.standard_normal(nx * ny).astype(np.float32)
    b[pinned] = 0.0
    d = s.solve(Field("float", (nx, ny, 1)).from_array(b))
    assert d["converged"], d
    fixtures.write_system2(str(tmp_path), s, np.zeros(nx * ny, np.float32), url="solve", frame=0)
    meta = json.load(open(tmp_path / "meta.json"))
    NX, NY = meta["shape"]
    rd = lambda n: np.fromfile(tmp_path / f"{n}.bin", dtype="<f4").astype(np.float64)
    bb, mask, after = rd("b"), rd("dirichletMask") > 0.5, rd("pressureAfter")
    assert np.array_equal(mask, pinned) and meta["pinned"] == int(pinned.sum())
    ratio = np.linalg.norm(bb - oracle.cpuref_apply((NX, NY), meta["gridSpacing"], after, mask)) / \
        meta["gpu"]["residual"]
    assert 0.5 < ratio < 2, ratio
