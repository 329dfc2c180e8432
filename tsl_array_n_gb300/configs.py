"""Timings of the configurations besides the 256^3 sphere solve (which
bench.py measures): one JSON line per configuration on cuda:0.

    python -m tsl_array_n_gb300.configs [c1] [c2[:steps]] [c4] [c5[:steps]] [c5tp[:steps]] [gridstep]

- c1: 2D 128^2 cylinder, 4-level MGPCG to 1e-6 (double-single and plain
  FP32 iterate): ms per solve, iterations, residual.
- c2: 2D 1024 x 256 channel past a cylinder of radius 16 cells at x = 128
  cells, u = 1 inflow, Re = U D / nu = 200, CFL 0.5, outflow column
  Dirichlet p = 0: ms per step over 100 steps, then the run continued to
  2000 steps with the transverse velocity sampled at four probes on the
  cylinder's centre line (1, 2, 3.3 and 5 diameters behind it), from which
  the Strouhal number follows by the crossing count of the reference's
  karman_shedding.mjs:94-114 (opening 30% discarded, crossings of the mean
  with a 0.25 sigma dead band, period = 2 span / crossings).
- c4: the U-Net warm start's forward at 128^3 and 256^3 and its loss and
  backward at 128^3.
- c5: 3D FLIP dam break, 256 x 128 x 128, 2^3 particles per cell in a
  liquid column of 40% of the domain, 500 steps: ms per step; c5dump and
  c5solve save one of its pressure systems and solve it standalone.
- c5tp: the configuration as specified: the same dam break with the air
  simulated too (two-phase, liquid:air density 1000:1, variable-coefficient
  projection), 500 steps, with plain FP32, mixed and learned+mixed
  projections; c5tpdump and c5tpsolve save one of its pressure systems and
  solve it standalone.
- gridstep: the 3D grid solver step at 256^3 around the benchmark's sphere,
  with the advection and the velocity constraint timed alone.

All inputs are synthetic and seeded; every timing is taken with the device
synchronised on both sides.
"""
import json
import math
import os
import sys
import time

import numpy as np

from . import fluxflow as ff, scenes, tsl_array_n
from .tsl_array_n import Field


def _now(ctx):
    ctx.synchronize()
    return time.perf_counter()


def c1(ctx):
    sc = scenes.cylinder_scene_2d()
    n = 128
    shape, h = sc["shape"], sc["h"]
    cw = {"u": Field("float", (n + 1, n, 1)).from_array(sc["wu"]), "v": Field("float", (n, n + 1, 1)).from_array(sc["wv"]),
          "w": Field("float", (n, n, 2)).from_array(np.ones(2 * n * n, np.float32))}
    out = {"config": "C1 2D 128^2 cylinder, 4-level MGPCG, tolerance 1e-6"}
    for prec in ("mixed", "fp32"):
        s = ff.create_grid_pressure_solver2((n, n), h[:2], collider_weights=cw, dirichlet=(sc["active"], sc["target"]),
                                            multigrid={"numberOfLevels": 4}, precision=prec, tolerance=1e-6)
        grid = ff.FaceCenteredGrid3(shape, h).set(sc["u"], sc["v"], sc["w"])
        o = ff.FaceCenteredGrid3(shape, h)
        disp = s.project(grid, o)
        for _ in range(3):
            s.pressure.fill(0.0)
            d = disp()
        t0 = _now(ctx)
        for _ in range(20):
            s.pressure.fill(0.0)
            d = disp()
        out[prec] = {"ms_per_solve": round((_now(ctx) - t0) / 20 * 1e3, 3), "iterations": d["iterations"],
                     "converged": d["converged"], "residual": d["residual"]}
    return out


def strouhal(series, every, dt, diameter, speed):
    """The crossing-count estimate of karman_shedding.mjs:94-114 for one
    probe's samples (one every `every` steps of length dt): None when the
    signal crosses its mean fewer than twice."""
    raw = np.asarray(series[int(math.floor(len(series) * 0.3)):], np.float64)
    if raw.size < 20:
        return None, 0
    dev = raw - raw.mean()
    std = float(np.sqrt(np.mean(dev * dev)))
    crossings, last = 0, 0
    for d in dev:
        s = 1 if d > 0.25 * std else (-1 if d < -0.25 * std else 0)
        if s != 0 and last != 0 and s != last:
            crossings += 1
        if s != 0:
            last = s
    if crossings < 2:
        return None, crossings
    period_steps = 2.0 * raw.size * every / crossings
    return (diameter / speed) / (period_steps * dt), crossings


def c2_channel(nx=1024, ny=256, radius=16, cx=128):
    """The C2 channel (karman_shedding.mjs): a disc of `radius` cells at
    x = `cx` cells on the centre line of an nx x ny channel with h = 1/ny,
    inflow u = 1 through a box at the left wall, p = 0 on the last cell
    column, free-slip top and bottom walls, Re 200 on the diameter, dt = h/2,
    5-level mixed-precision MGPCG to 1e-6.  Returns (solver, grid, collider,
    inflow, geometry dict)."""
    h = 1.0 / ny
    cy = ny // 2
    # one cell layer with hz = h: the sphere below cuts it in a disc of
    # `radius` cells (the w faces are closed walls, so hz enters nothing else)
    res, hh = (nx, ny, 1), (h, h, h)
    grid = ff.FaceCenteredGrid3(res, hh)
    grid.set(np.ones(ny * (nx + 1), np.float32), np.zeros(nx * (ny + 1), np.float32), np.zeros(2 * nx * ny, np.float32))
    col = ff.create_sdf_static_collider3(*res, *hh)
    col.add_shapes([{"type": "sphere", "center": [cx * h, cy * h, 0.5 * h], "radius": radius * h}])
    inflow = ff.create_sdf_inflow3(*res, *hh, velocity=(1.0, 0.0, 0.0), mode="set")
    inflow.add_shapes([{"type": "box", "center": [0.0, 0.5, 0.5 * h], "halfExtents": [1.5 * h, 1.0, 1.0]}])
    active = np.zeros((ny, nx), np.uint8)
    active[:, nx - 1] = 1
    dt, speed, diameter = 0.5 * h, 1.0, 2 * radius * h
    solver = ff.create_grid_solver3(velocity_grid=grid, collider=col, inflows=[inflow], dt=dt, nu=speed * diameter / 200.0,
                                    closed_domain_boundary_flag=ff.DIRECTION_DOWN | ff.DIRECTION_UP |
                                    ff.DIRECTION_BACK | ff.DIRECTION_FRONT,
                                    dirichlet=(active.ravel(), np.zeros(nx * ny, np.float32)),
                                    pressure={"multigrid": {"numberOfLevels": 5}, "precision": "mixed", "tolerance": 1e-6})
    geo = {"res": res, "h": hh, "cx": cx, "cy": cy, "dt": dt, "speed": speed, "diameter": diameter,
           "probes": [cx + int(round(f * 2 * radius)) for f in (1.0, 2.0, 3.3, 5.0)]}
    return solver, grid, col, inflow, geo


def c2(ctx, steps=2000, timed=100, every=2):
    solver, grid, col, inflow, geo = c2_channel()
    nx, cx, cy, dt, speed, diameter = geo["res"][0], geo["cx"], geo["cy"], geo["dt"], geo["speed"], geo["diameter"]
    for _ in range(5):
        solver.on_advance_time_step()
    its = []
    t0 = _now(ctx)
    for _ in range(timed):
        its.append(solver.on_advance_time_step()["iterations"])
    ms = (_now(ctx) - t0) / timed * 1e3
    # v at the probes (cell columns radius * (2, 4, 6.6, 10) behind the centre)
    probes = geo["probes"]
    series, steps_at, sym_break = [], [], None
    done = 5 + timed
    for step in range(done, steps):
        solver.on_advance_time_step()
        if (step - done) % every == 0:
            v = grid.data_v.to_array()
            row = [float(v[i + nx * cy]) for i in probes]
            series.append(row)
            steps_at.append(step + 1)
            if sym_break is None and max(abs(x) for x in row) > 0.01 * speed:
                sym_break = step + 1

    def estimate(rows):
        st = []
        for p in range(len(probes)):
            s, crossings = strouhal([r[p] for r in rows], every, dt, diameter, speed)
            st.append({"probe_cells_behind": probes[p] - cx, "strouhal": None if s is None else round(s, 4),
                       "crossings": crossings})
        return st

    # the same estimate over the samples after the symmetry break alone, as
    # the CPU oracle's run of this channel reports it
    post = [r for r, k in zip(series, steps_at) if sym_break is not None and k > sym_break]
    if os.environ.get("FF_C2_SERIES"):
        # the probe series ([step, v at each probe] rows) for other windows
        with open(os.environ["FF_C2_SERIES"], "w") as f:
            json.dump({"probes": probes, "cx": cx, "series": [[k] + r for k, r in zip(steps_at, series)]}, f)
    return {"config": "C2 2D 1024x256 channel past a cylinder r = 16 cells, Re 200, CFL 0.5",
            "ms_per_step": round(ms, 3), "mean_iterations": float(np.mean(its)), "timed_steps": timed,
            "steps": steps, "symmetry_break_step": sym_break, "probes": estimate(series),
            "probes_post_break": estimate(post)}


def gridstep(ctx, steps=20):
    """The 3D grid solver step at 256^3 around the benchmark's sphere (radius
    24 cells, the 32-mode velocity, closed walls, one pinned cell): explicit
    viscosity, projection to 1e-6 (mixed, 6 levels, coarsest direct),
    constrainVelocity, semi-Lagrangian advection of the faces, constraint
    again; ms per step over `steps` steps, and the advection and the
    constraint timed alone with their algorithmic bytes.  Advection reads the
    three velocity arrays for the back-trace and the advected component and
    writes that component, per component (16 B a face); the constraint, per
    face: marking (value and weight read, value and int32 marker written,
    16 B), five Jacobi extrapolation passes (value and marker read and
    written, 16 B each), no-flux (12 B) and walls (8 B): 116 B a face."""
    n = 256
    sc = scenes.sphere_scene(n=n, radius_cells=24, modes=32, seed=1)
    shape, h = sc["shape"], sc["h"]
    grid = ff.FaceCenteredGrid3(shape, h).set(sc["u"], sc["v"], sc["w"])
    col = ff.create_sdf_static_collider3(*shape, *h)
    col.add_shapes(sc["shapes"])
    solver = ff.create_grid_solver3(velocity_grid=grid, collider=col, dt=0.25 / n, nu=1e-4,
                                    dirichlet=(sc["active"], sc["target"]),
                                    pressure={"multigrid": {"numberOfLevels": 6, "coarseSolve": "direct"},
                                              "precision": "mixed", "tolerance": 1e-6})
    for _ in range(3):
        solver.on_advance_time_step()
    its = []
    t0 = _now(ctx)
    for _ in range(steps):
        its.append(solver.on_advance_time_step()["iterations"])
    ms = (_now(ctx) - t0) / steps * 1e3
    faces = sum(f.count for f in (grid.data_u, grid.data_v, grid.data_w))
    out = {"config": "3D grid solver step 256^3, sphere r=24, viscosity + projection + advection + constraints",
           "ms_per_step": round(ms, 3), "mean_iterations": float(np.mean(its))}
    adv = solver.advection_solver.advect_face_centered3(solver.velocity_prev, solver._scratch)
    for name, fn, nbytes in (("advection", adv, 16 * faces),
                             ("constrain", solver.boundary_solver.constrain_velocity, 116 * faces)):
        fn()
        t0 = _now(ctx)
        for _ in range(5):
            fn()
        t = (_now(ctx) - t0) / 5
        out[name] = {"ms": round(t * 1e3, 3), "GB_s": round(nbytes / t / 1e9, 1), "bytes": int(nbytes)}
    return out


def c4(ctx, steps=None):
    """U-Net timings at 128^3 and 256^3 (``c4:128`` or ``c4:256``: that size
    alone)."""
    from .warmstart import UNetWarmStart
    out = {"config": "C4 U-Net warm start (3 levels, 16/32/64 channels)"}
    for n in ((steps,) if steps else (128, 256)):
        shp = (n, n, n)
        rng = np.random.default_rng(0)
        b = Field("float", shp).from_array(rng.standard_normal(n ** 3).astype(np.float32))
        m = Field("uint8", shp).from_array(np.zeros(n ** 3, np.uint8))
        p = Field("float", shp).from_array(rng.standard_normal(n ** 3).astype(np.float32))
        o = Field("float", shp)
        net = UNetWarmStart(seed=1)
        for _ in range(3):
            net.forward(shp, 1.0 / n, b, m, p, o)
        t0 = _now(ctx)
        for _ in range(10):
            net.forward(shp, 1.0 / n, b, m, p, o)
        r = {"forward_ms": round((_now(ctx) - t0) / 10 * 1e3, 3)}
        if n == 128:
            t = Field("float", shp).from_array(rng.standard_normal(n ** 3).astype(np.float32))
            for _ in range(2):
                net.loss_backward(shp, 1.0 / n, b, m, p, t)
            t0 = _now(ctx)
            for _ in range(5):
                net.loss_backward(shp, 1.0 / n, b, m, p, t)
            r["loss_backward_ms"] = round((_now(ctx) - t0) / 5 * 1e3, 3)
        out[f"{n}^3"] = r
        del b, m, p, o, net
    return out


def _dam_break():
    shp, hh = (256, 128, 128), (1.0 / 128,) * 3
    grid = ff.FaceCenteredGrid3(shp, hh)
    # the liquid column: 0.8 x 0.5 x 1 of the 2 x 1 x 1 domain (40%)
    seed = ff.compute_flip_box_seed3((0.0, 0.0, 0.0), (1.6, 0.5, 1.0), *hh)
    npart = seed["count"]
    # the coarsest level (16 x 8 x 8) swept, as the reference does: its
    # Dirichlet cells move every step, and a direct inverse would be
    # refactored every step
    s = ff.create_grid_flip_solver3(velocity_grid=grid, max_particles=npart, dt=0.002, flip_ratio=0.95,
                                    pressure=dict(DAM_BREAK_PRESSURE))
    s.positions.from_array(seed["positionsArray"])
    s.velocities.from_array(np.zeros(3 * npart, np.float32))
    return grid, s, npart


DAM_BREAK_PRESSURE = {"multigrid": {"numberOfLevels": 5, "coarseSolve": "sweeps"}, "tolerance": 1e-6,
                      "precision": "mixed"}


def c5(ctx, steps=500):
    grid, s, npart = _dam_break()
    for _ in range(3):
        s.on_advance_time_step()
    its, worst = [], 0.0
    t0 = _now(ctx)
    for _ in range(steps):
        a = time.perf_counter()
        its.append(s.on_advance_time_step()["iterations"])
        worst = max(worst, time.perf_counter() - a)
    ms = (_now(ctx) - t0) / steps * 1e3
    return {"config": "C5 3D FLIP dam break 256x128x128, 8 particles per cell, column 40%", "particles": npart,
            "steps": steps, "ms_per_step": round(ms, 3), "mean_iterations": float(np.mean(its)),
            "max_iterations": int(max(its)), "slowest_step_host_ms": round(worst * 1e3, 3)}


def _two_phase_dam_break(precision, n=(256, 128, 128)):
    """C5 as configured: a 3D two-phase dam break on n cells of h = 1/n[1]
    (a 2 x 1 x 1 domain), 2^3 jittered particles in every cell, the liquid
    column x < 1.6, y < 0.5 (40% of the volume) at density 1 and the rest
    gas at 0.001 (1000:1), FLIP/PIC 0.95, gravity -9.81, 5-level MGPCG whose
    coarsest level is swept (its density-weighted operator changes every
    step)."""
    h = 1.0 / n[1]
    hh = (h, h, h)
    grid = ff.FaceCenteredGrid3(n, hh)
    seed = ff.compute_two_phase_box_seed3((0.0, 0.0, 0.0), (n[0] * h, n[1] * h, n[2] * h), hh, (0.0, 0.0, 0.0),
                                          (0.8 * n[0] * h, 0.5 * n[1] * h, n[2] * h))
    npart = seed["count"]
    s = ff.create_grid_two_phase_flip_solver3(
        velocity_grid=grid, max_particles=npart, dt=0.002, liquid_density=1.0, gas_density=0.001, flip_ratio=0.95,
        pressure={"multigrid": {"numberOfLevels": 5, "coarseSolve": "sweeps"}, "tolerance": 1e-6,
                  "precision": precision})
    s.set_particles(seed["positionsArray"], np.zeros(3 * npart, np.float32), seed["phasesArray"])
    return grid, s, npart, seed


def _transfer_rates(ctx, s, grid, npart, reps=5):
    """P2G and G2P of the two-phase solver on its current particles, timed
    alone (device synchronised around `reps` calls).  Algorithmic bytes:
    P2G reads position and velocity (24 B a particle) and, per face, clears
    the two int32 accumulators, then reads them and writes the velocity and
    its valid flag (24 B a face); its 48 int32 atomics a particle go to L2.
    G2P reads position, velocity and phase and writes the velocity (40 B a
    particle) and reads the new and old face velocities (8 B a face)."""
    faces = sum(f.count for f in (grid.data_u, grid.data_v, grid.data_w))
    out = {}
    for name, nbytes in (("p2g", 24 * npart + 24 * faces), ("g2p", 40 * npart + 8 * faces)):
        s.stage(name)
        t0 = _now(ctx)
        for _ in range(reps):
            s.stage(name)
        ms = (_now(ctx) - t0) / reps * 1e3
        out[name] = {"ms": round(ms, 3), "GB_s": round(nbytes / ms / 1e6, 1), "bytes": int(nbytes),
                     "particles_per_s": float(npart / ms * 1e3)}
    return out


def c5tp(ctx, steps=500):
    """The two-phase dam break with each projection arm: plain FP32 MGPCG,
    mixed precision, and mixed with the learned warm start (the network's
    forward pass inside every step); ms per step, PCG iterations per
    projection, convergence."""
    from . import warmstart
    import os
    out = {"config": "C5 3D two-phase FLIP dam break 256x128x128, 8 particles per cell, liquid column 40%, "
                     "density 1000:1, FLIP 0.95", "steps": steps, "arms": {}}
    weights = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "unet_warmstart.npy")
    for arm in ("fp32", "mixed", "learned+mixed"):
        grid, s, npart, seed = _two_phase_dam_break("fp32" if arm == "fp32" else "mixed")
        net = None
        if arm == "learned+mixed":
            net = warmstart.UNetWarmStart(seed=1)
            if os.path.exists(weights):
                net.load(weights)
            warmstart.attach(s.pressure_solver, net)
        out["particles"] = npart
        for _ in range(3):
            s.on_advance_time_step()
        its, conv, res, stops = [], 0, [], {}
        t0 = _now(ctx)
        for _ in range(steps):
            d = s.on_advance_time_step()
            its.append(d["iterations"])
            conv += int(d["converged"])
            res.append(d["residual"] / max(d["bNorm"], 1e-300))
            stops[d["stoppedBy"]] = stops.get(d["stoppedBy"], 0) + 1
        ms = (_now(ctx) - t0) / steps * 1e3
        pos, _, ph = s.get_particles(npart)
        liquid_y = float(pos.reshape(-1, 3)[ph > 0.5, 1].mean())
        out["arms"][arm] = {"ms_per_step": round(ms, 3), "mean_iterations": float(np.mean(its)),
                            "max_iterations": int(max(its)), "converged_fraction": conv / steps,
                            "residual_rel_median": float(np.median(res)), "residual_rel_max": float(max(res)),
                            "stopped_by": stops, "liquid_centroid_y": round(liquid_y, 4)}
        if arm == "mixed":
            out["arms"][arm]["transfers"] = _transfer_rates(ctx, s, grid, npart)
        if net is not None:
            warmstart.attach(s.pressure_solver, None)
            net.close()
        s.close()
        del grid, s
    return out


def c5tpdump(ctx, steps, path):
    """Run the two-phase dam break (mixed precision) `steps` steps and save
    its last projection's system to `path` (.npz, compressed): b, the beta
    faces it was built with, the pressure the solver returned, the pinned
    cell and the projection's diagnostics."""
    grid, s, npart, _ = _two_phase_dam_break("mixed")
    for _ in range(steps):
        d = s.on_advance_time_step()
    res = grid.resolution
    np.savez_compressed(path, b=s.pressure_solver.b.to_array(), beta_u=s.beta_u.to_array(),
                        beta_v=s.beta_v.to_array(), beta_w=s.beta_w.to_array(), pressure=s.pressure.to_array(),
                        pin=np.array([res[0] // 2, res[1] - 1, res[2] // 2]), iterations=d["iterations"],
                        residual=d["residual"], b_norm=d["bNorm"])
    return {"config": f"C5 two-phase pressure system after {steps} steps", "path": path, "diagnostics": d}


def c5tpsolve(ctx, path, out=None):
    """Solve a saved two-phase system (c5tpdump) from a zero start with a
    standalone solver of the dam break's options, with the coarsest level
    swept and solved directly; `out` (.npz) keeps one V-cycle applied to b
    (coarsest level swept)."""
    z = np.load(path)
    shp, hh = (256, 128, 128), (1.0 / 128,) * 3
    n = int(np.prod(shp))
    pin = z["pin"]
    active = np.zeros(n, np.uint8)
    active[int(pin[0]) + shp[0] * (int(pin[1]) + shp[1] * int(pin[2]))] = 1
    fw = {"u": Field("float", (shp[0] + 1, shp[1], shp[2])).from_array(z["beta_u"]),
          "v": Field("float", (shp[0], shp[1] + 1, shp[2])).from_array(z["beta_v"]),
          "w": Field("float", (shp[0], shp[1], shp[2] + 1)).from_array(z["beta_w"])}
    b = Field("float", shp).from_array(z["b"])
    res = {"config": "C5 two-phase pressure system, standalone solve from zero", "path": path}
    keep = {}
    for coarse in ("sweeps", "direct"):
        ps = ff.create_grid_pressure_solver3(shp, hh, dirichlet=(active, np.zeros(n, np.float32)), face_weights=fw,
                                             multigrid={"numberOfLevels": 5, "coarseSolve": coarse},
                                             tolerance=1e-6, precision="mixed")
        ps.prepare()
        ps.pressure.fill(0.0)
        d = ps.solve(b)
        res[coarse] = {"iterations": d["iterations"], "converged": d["converged"], "stoppedBy": d["stoppedBy"],
                       "residual_rel": d["residual"] / max(d["bNorm"], 1e-300)}
        if coarse == "sweeps":
            zf = Field("float", shp)
            ps.apply_preconditioner(b, zf)
            keep = {"z": zf.to_array()}
        del ps
    if out:
        np.savez_compressed(out, **keep)
    return res


def c5dump(ctx, steps, path):
    """Run the dam break `steps` steps and save the last projection's
    system (Dirichlet active/target cells and b) to `path` (.npz)."""
    grid, s, npart = _dam_break()
    for _ in range(steps):
        d = s.on_advance_time_step()
    gf = s.grid_fields()
    np.savez(path, active=gf["dirichletActive"].to_array(), target=gf["dirichletTarget"].to_array(),
             b=s.pressure_solver.b.to_array(), iterations=d["iterations"])
    return {"config": f"C5 pressure system after {steps} steps", "path": path, "iterations": d["iterations"]}


def c5solve(ctx, path, reps=1):
    """Solve a saved dam-break system with a standalone solver of the same
    options (CUDA graphs off, so a profiler sees each kernel) and report
    the per-kernel times of ff_pressure3_profile."""
    import ctypes as C
    from . import _lib
    z = np.load(path)
    shp, hh = (256, 128, 128), (1.0 / 128,) * 3
    opts = dict(DAM_BREAK_PRESSURE)
    ps = ff.create_grid_pressure_solver3(shp, hh, dirichlet=(z["active"], z["target"]), multigrid=opts["multigrid"],
                                         tolerance=opts["tolerance"], precision=opts["precision"])
    ps.settings.useGraph = False
    b = Field("float", shp).from_array(z["b"])
    for _ in range(reps):
        ps.pressure.fill(0.0)
        d = ps.solve(b)
    out = {"config": "C5 pressure system, standalone solve", "iterations": d["iterations"],
           "converged": d["converged"], "air_fraction": round(float(np.mean(z["active"] != 0)), 4)}
    for name, kid in (("p_pAp", 0), ("x_residual", 1), ("sweep", 2), ("residual_restrict", 3), ("prolong", 5),
                      ("vcycle", 7)):
        avg = C.c_float()
        _lib.check(_lib.load().ff_pressure3_profile(ps.handle, kid, 5, C.byref(avg)))
        out[name + "_ms"] = round(avg.value, 4)
    return out


def main(argv):
    """Arguments: configuration names, each optionally with a step count
    (``c2:6000`` runs the channel 6000 steps, ``c5:200`` the dam break 200);
    ``c5dump:300:sys.npz`` saves the dam break's system after 300 steps
    (``c5tpdump`` the two-phase one's) and ``c5solve:sys.npz`` solves and
    profiles it standalone."""
    runs = []
    for a in argv:
        name, _, rest = a.partition(":")
        if name in ("c1", "c2", "c4", "c5", "c5tp", "gridstep"):
            runs.append((name, {"steps": int(rest)} if rest else {}))
        elif name in ("c5dump", "c5tpdump"):
            steps, _, path = rest.partition(":")
            runs.append((name, {"steps": int(steps), "path": path}))
        elif name == "c5solve":
            runs.append((name, {"path": rest}))
        elif name == "c5tpsolve":
            path, _, out = rest.partition(":")
            runs.append((name, {"path": path, "out": out or None}))
    ctx = tsl_array_n.init(0)
    for name, kw in runs or [(n, {}) for n in ("c1", "c2", "c4", "c5")]:
        print(json.dumps(globals()[name](ctx, **kw)), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
