"""Pressure systems on disk in the reference's two fixture formats.

Both formats are a directory of raw little-endian float32 arrays in
i-fastest order, one ``<name>.bin`` per array, plus ``meta.json``:

* 3D, the ``stalled-system`` format (export_system.mjs:77-126, read by
  sandbox/stalled-system/main.js): ``b``, ``pressure``, ``dirichletMask``,
  ``ventMask`` and, when a collider is present, ``weightU/V/W``; meta holds
  ``source, frame, resolution, gridSpacing, dataSizeU/V/W, diagnostics,
  multigrid, tolerance, maxIterations``.
* 2D (export_system2.mjs:83-144, read by cpu_reference.mjs:35-48): ``b``,
  ``dirichletMask``, ``pressureBefore``, ``pressureAfter``; the mask is
  written even when no cell is pinned (all zeros), since
  cpu_reference.mjs:44 reads it unconditionally; meta holds ``url, frame, shape,
  gridSpacing, hasWeights, settings, gpu {converged, iterations, residual,
  stoppedBy}, bNorm, pinned, cells``.

Masks are stored as 0/1 floats, as the reference's float mask fields are.
``write_*`` take a solver that has run ``project`` or ``solve``;
``write_*_arrays`` take host arrays; ``read_*`` return ``(meta, arrays)``
with absent arrays as None; ``solver_from_system3`` rebuilds the operator
from a 3D fixture the way the stalled-system sandbox does (collider
weights, the vent cells pinned to 0; enclosed cells follow from the
weights).
"""
import json
import os

import numpy as np

from .fluxflow import PRECONDITIONERS

SYSTEM3_ARRAYS = ("b", "pressure", "dirichletMask", "ventMask", "weightU", "weightV", "weightW")
SYSTEM2_ARRAYS = ("b", "dirichletMask", "pressureBefore", "pressureAfter")


def _write_bin(path, values):
    np.ascontiguousarray(values, dtype="<f4").ravel().tofile(path)


def _read_dir(path, names):
    meta = json.load(open(os.path.join(path, "meta.json")))
    arrays = {}
    for n in names:
        f = os.path.join(path, n + ".bin")
        arrays[n] = np.fromfile(f, dtype="<f4") if os.path.exists(f) else None
    return meta, arrays


def _face_sizes(res):
    nx, ny, nz = res
    return [nx + 1, ny, nz], [nx, ny + 1, nz], [nx, ny, nz + 1]


def _mg_options(desc):
    return {"numberOfLevels": int(desc.mg_levels), "numberOfSmoothingIterationsDown": int(desc.mg_down),
            "numberOfSmoothingIterationsUp": int(desc.mg_up),
            "numberOfCoarsestIterations": int(desc.mg_coarsest), "numberOfFinalIterations": int(desc.mg_final),
            "sorFactor": float(desc.mg_sor), "coarsenDirichletMask": bool(desc.mg_coarsen_mask),
            "coarsenFaceWeights": bool(desc.mg_coarsen_weights),
            "coarseSolve": "direct" if desc.mg_coarse_mode == 1 else "sweeps"}


# ------------------------------------------------------------------ 3D ----
def write_system3_arrays(path, resolution, arrays, grid_spacing=(1.0, 1.0, 1.0), source="", frame=0,
                         diagnostics=None, multigrid=None, tolerance=None, max_iterations=None):
    """Write a stalled-system directory from host arrays (``arrays`` maps
    the names in SYSTEM3_ARRAYS to arrays or None)."""
    res = [int(n) for n in resolution]
    cells = res[0] * res[1] * res[2]
    su, sv, sw = _face_sizes(res)
    sizes = {"b": cells, "pressure": cells, "dirichletMask": cells, "ventMask": cells,
             "weightU": int(np.prod(su)), "weightV": int(np.prod(sv)), "weightW": int(np.prod(sw))}
    os.makedirs(path, exist_ok=True)
    for n in SYSTEM3_ARRAYS:
        v = arrays.get(n)
        f = os.path.join(path, n + ".bin")
        if v is None:
            if os.path.exists(f):
                os.remove(f)
            continue
        v = np.asarray(v)
        if v.size != sizes[n]:
            raise ValueError(f"write_system3: {n} has {v.size} values, expected {sizes[n]}")
        _write_bin(f, v)
    meta = {"source": source, "frame": frame, "resolution": res, "gridSpacing": [float(h) for h in grid_spacing],
            "dataSizeU": su, "dataSizeV": sv, "dataSizeW": sw, "diagnostics": dict(diagnostics or {}),
            "multigrid": dict(multigrid or {}), "tolerance": tolerance, "maxIterations": max_iterations}
    with open(os.path.join(path, "meta.json"), "w") as fh:
        fh.write(json.dumps(meta, indent="\t") + "\n")
    return meta


def write_system3(path, solver, collider_weights=None, source="", frame=0):
    """The system ``solver`` (a GridPressureSolver3) built and solved last:
    its b, pressure, Dirichlet and vent masks, and the collider face
    weights it was given (``collider_weights``, a {u, v, w} dict of Fields,
    or the ones set on the solver)."""
    cw = collider_weights if collider_weights is not None else solver._keep.get("cw")
    arrays = {"b": solver.b.to_array(), "pressure": solver.pressure.to_array(),
              "dirichletMask": solver.dirichlet_mask.to_array().astype(np.float32),
              "ventMask": solver.vent_mask.to_array().astype(np.float32),
              "weightU": cw["u"].to_array() if cw else None, "weightV": cw["v"].to_array() if cw else None,
              "weightW": cw["w"].to_array() if cw else None}
    d = solver.desc
    return write_system3_arrays(path, solver.resolution, arrays, solver.grid_spacing, source, frame,
                                diagnostics=solver.diagnostics, multigrid=_mg_options(d),
                                tolerance=float(d.tolerance), max_iterations=int(d.max_iterations) or None)


def read_system3(path):
    return _read_dir(path, SYSTEM3_ARRAYS)


def solver_from_system3(path_or_loaded, **options):
    """A GridPressureSolver3 over a 3D fixture's operator: its collider
    weights, the vent cells Dirichlet at 0 (enclosed cells are pinned by the
    solver from the weights, as grid_pressure_solver3.js:171-206 does).
    ``options`` go to create_grid_pressure_solver3 (multigrid defaults to
    the fixture's own).  Returns (solver, b Field, meta, arrays)."""
    from . import fluxflow as ff
    from .tsl_array_n import Field
    meta, a = read_system3(path_or_loaded) if isinstance(path_or_loaded, str) else path_or_loaded
    res = tuple(meta["resolution"])
    cw = None
    if a.get("weightU") is not None:
        cw = {"u": Field("float", tuple(meta["dataSizeU"])).from_array(a["weightU"]),
              "v": Field("float", tuple(meta["dataSizeV"])).from_array(a["weightV"]),
              "w": Field("float", tuple(meta["dataSizeW"])).from_array(a["weightW"])}
    vent = (a["ventMask"] > 0.5) if a.get("ventMask") is not None else np.zeros(int(np.prod(res)), bool)
    opts = {"multigrid": {k: v for k, v in (meta.get("multigrid") or {}).items() if isinstance(v, (int, float, str))}}
    if meta.get("tolerance") is not None:
        opts["tolerance"] = meta["tolerance"]
    if meta.get("maxIterations"):
        opts["max_iterations"] = int(meta["maxIterations"])
    opts.update(options)
    s = ff.create_grid_pressure_solver3(res, meta["gridSpacing"], collider_weights=cw,
                                        dirichlet=(vent, np.zeros(vent.size, np.float32)), **opts)
    b = Field("float", res).from_array(a["b"])
    return s, b, meta, a


# ------------------------------------------------------------------ 2D ----
def write_system2_arrays(path, shape, grid_spacing, b, pressure_before, pressure_after, dirichlet_mask=None,
                         gpu=None, settings=None, url="", frame=0, has_weights=False):
    """Write an export_system2 directory from host arrays."""
    nx, ny = int(shape[0]), int(shape[1])
    cells = nx * ny
    vals = {"b": b, "pressureBefore": pressure_before, "pressureAfter": pressure_after,
            "dirichletMask": dirichlet_mask}
    os.makedirs(path, exist_ok=True)
    for n, v in vals.items():
        f = os.path.join(path, n + ".bin")
        if v is None:
            if os.path.exists(f):
                os.remove(f)
            continue
        v = np.asarray(v)
        if v.size != cells:
            raise ValueError(f"write_system2: {n} has {v.size} values, expected {cells}")
        _write_bin(f, v)
    b32 = np.asarray(b, np.float32).astype(np.float64).ravel()
    pinned = int((np.asarray(dirichlet_mask) > 0.5).sum()) if dirichlet_mask is not None else 0
    meta = {"url": url, "frame": frame, "shape": [nx, ny], "gridSpacing": [float(grid_spacing[0]),
                                                                          float(grid_spacing[1])],
            "hasWeights": bool(has_weights), "settings": dict(settings or {}), "gpu": dict(gpu or {}),
            "bNorm": float(np.sqrt(np.dot(b32, b32))), "pinned": pinned, "cells": cells}
    with open(os.path.join(path, "meta.json"), "w") as fh:
        fh.write(json.dumps(meta, indent="\t"))
    return meta


def write_system2(path, solver, pressure_before, url="", frame=0):
    """A 2D solver's (create_grid_pressure_solver2, nz = 1) last solve:
    ``pressure_before`` is the pressure the solve started from (the
    previous frame's), as export_system2.mjs:83-93 saves it."""
    if solver.resolution[2] != 1:
        raise ValueError("write_system2: a 2D solver (nz = 1) is required")
    d, diag = solver.desc, solver.diagnostics
    mask = solver.dirichlet_mask.to_array().astype(np.float32)
    settings = {"tolerance": float(d.tolerance), "relativeTolerance": bool(d.relative_tolerance),
                "maxIterations": int(d.max_iterations) or None,
                "preconditioner": {v: k for k, v in PRECONDITIONERS.items()}.get(int(d.preconditioner)),
                "levels": int(d.mg_levels)}
    gpu = {"converged": diag.get("converged"), "iterations": diag.get("iterations"),
           "residual": diag.get("residual"), "stoppedBy": diag.get("stoppedBy")}
    return write_system2_arrays(path, solver.resolution[:2], solver.grid_spacing[:2], solver.b.to_array(),
                                pressure_before, solver.pressure.to_array(), mask, gpu,
                                settings, url, frame, has_weights="cw" in solver._keep)


def read_system2(path):
    return _read_dir(path, SYSTEM2_ARRAYS)
