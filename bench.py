"""Benchmark: ms per pressure projection (MGPCG to relative residual 1e-6) on
the 256^3 sphere configuration, on GB300.

A step is one projection of the same synthetic velocity field from a cold
start (pressure reset to zero): build b, PCG to 1e-6, circuit breaker,
velocity correction.  `value` is device time per step with the inputs
resident in HBM; `e2e` adds the host->device upload of u, v, w from pinned
memory and the device->host read of the corrected u, v, w, all through the
C ABI (ff_pressure3_project_host: each step's upload overlaps the previous
step's download, as a stream of projections runs).  The timed inputs (about 1.7 GB of fields) are larger than the 129 MB
L2, so no flush is needed between steps.

The line also carries `arms`: the same projection timed with plain FP32
MGPCG (FP32 iterate and V-cycle), BF16 V-cycle storage, and the learned
warm start (the network's forward pass and the residual test inside the
timed region) on top of the mixed solve; `oracle_error`: the pressure and
corrected velocity of the timed solve against the FP64 oracle's solution
converged to 1e-10, and the divergence left; and `cpu_baseline`: one whole
FP64 oracle projection of the same system to 1e-6, measured, with the
oracle's own iteration count.

--impl reference times the FP64 CPU restatement of the same path (the
reference is JavaScript + WebGPU and cannot run on this machine) on the
host cores: every timed step is one whole projection to 1e-6.
"""
import argparse
import datetime
import json
import os
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms/solve to 1e-6 residual at 256^3 (MGPCG pressure projection, sphere r=24)"
UNIT = "ms/solve"

# Algorithmic bytes per cell per launch (each array the kernel reads or
# writes counted once over the domain; FP32 4 B, BF16 2 B, coefficients
# 16 B FP32 / 8 B BF16, the double-single iterate 8 B).
def kernel_bytes_per_cell(precision):
    xb = 8 if precision.startswith("mixed") else 4
    if precision == "mixed-bf16":
        # per-colour kernels, BF16 coarse storage, coefficients read per cell
        return {"p_pAp": 4 + 4 + 16 + 4, "x_residual": xb + 4 + 4 + 16 + xb + 4,
                "relax": 4 + 4 + 8 + 2, "residual": 4 + 4 + 8 + 2, "restrict": 2 + 0.25,
                "prolong": 0.25 + 8, "rz": 8}
    # fused path: plain cells read no coefficients; the TMA kernels read one
    # class byte per four cells
    return {
        "p_pAp": 4 + 4 + 4,                 # z, p -> p
        "x_residual": xb + 4 + 4 + xb + 4,  # x, p, b -> x, r
        "relax": 4 + 4 + 4 + 0.25,          # one full red-black sweep: x, b, classes -> x
        # residual with the x restriction taps (x, b, classes -> half-size
        # rx), then the y/z taps (rx -> coarse b)
        "residual": 4 + 4 + 0.25 + 2 + 2 + 0.5,
        "restrict": 4 + 0.5,
        "prolong": 0.5 + 8,
        "rz": 8,
    }


PROF_IDS = {"p_pAp": 0, "x_residual": 1, "relax": 2, "residual": 3, "restrict": 4, "prolong": 5,
            "rz": 6}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        p = json.load(open(path))
        return p["hbm_gbs"], "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling every 20 ms, started before the solver is built so
    that it is running when the timed region opens.  mark() and stop() record the
    wall-clock bracket of the timed region; the summary keeps the rows whose
    nvidia-smi timestamp falls inside it (the nearest rows when none do)."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        # the raw samples: FF_CLOCKS_CSV if set, else a temporary file
        self.path = os.environ.get("FF_CLOCKS_CSV") or os.path.join(tempfile.gettempdir(),
                                                                     f"ff_clocks_{os.getpid()}.csv")
        self.t0 = self.t1 = None

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "20", "-i",
                 str(os.environ.get("LOCAL_RANK", 0))],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def mark(self):
        """the timed region opens"""
        self.t0 = datetime.datetime.now()

    def stop(self):
        if not self.proc:
            return None
        self.t1 = datetime.datetime.now()
        time.sleep(0.05)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = [[c.strip() for c in r.split(",")] for r in open(self.path).read().strip().splitlines()
                if r.count(",") >= 9]
        if not rows:
            return None
        stamp = []
        for r in rows:
            try:
                stamp.append(datetime.datetime.strptime(r[0], "%Y/%m/%d %H:%M:%S.%f"))
            except ValueError:
                stamp.append(None)
        inside = [r for r, t in zip(rows, stamp) if t is not None and self.t0 <= t <= self.t1]
        if not inside and all(t is not None for t in stamp):
            # the sample closest to the middle of the region
            mid = self.t0 + (self.t1 - self.t0) / 2
            inside = [min(zip(rows, stamp), key=lambda rt: abs((rt[1] - mid).total_seconds()))[0]]
        rows = inside or rows
        sm = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        mx = max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[6 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(inside), "interval_ms": 20}


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return rank, world, dist
    return rank, world, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ ours --
WEIGHTS = os.path.join(ROOT, "tsl_array_n_gb300", "weights", "unet_warmstart.npy")


def sphere_inputs(n):
    from tsl_array_n_gb300 import scenes
    return scenes.sphere_scene(n=n, radius_cells=24 * n // 256, modes=32, seed=1)


def make_solver(ff, sc, cw, levels, precision, coarse="direct"):
    return ff.create_grid_pressure_solver3(
        sc["shape"], sc["h"], collider_weights=cw, dirichlet=(sc["active"], sc["target"]),
        multigrid={"numberOfLevels": levels, "coarseSolve": coarse}, precision=precision, tolerance=1e-6)


def timed(lib, ctx, fn, steps, slot=4):
    """device ms per call of fn over `steps` calls (events on the context
    stream), and the last call's result"""
    import ctypes as C
    from tsl_array_n_gb300 import _lib
    ctx.synchronize()
    _lib.check(lib.ff_ctx_event_record(ctx.handle, slot))
    out = []
    for _ in range(steps):
        out.append(fn())
    _lib.check(lib.ff_ctx_event_record(ctx.handle, slot + 1))
    ms = C.c_float()
    _lib.check(lib.ff_ctx_event_elapsed(ctx.handle, slot, slot + 1, C.byref(ms)))
    ctx.synchronize()
    return ms.value / steps, out


def run_arm(ff, lib, ctx, sc, cw, grid, out, levels, arm, steps, warmup):
    """One comparison arm on the same system: ms per cold-start projection,
    iterations, convergence and residual.  'learned+mixed' runs the mixed
    solve with the U-Net warm start attached, so the network's forward pass
    and the residual comparison are inside the timed region."""
    from tsl_array_n_gb300 import warmstart
    precision = "mixed" if arm == "learned+mixed" else arm
    solver = make_solver(ff, sc, cw, levels, precision)
    net = None
    info = {}
    if arm == "learned+mixed":
        net = warmstart.UNetWarmStart(seed=1)
        if os.path.exists(WEIGHTS):
            net.load(WEIGHTS)
            info["network"] = "trained weights " + os.path.relpath(WEIGHTS, ROOT)
        else:
            info["network"] = "untrained (seeded initialisation)"
        warmstart.attach(solver, net)
    dispatch = solver.project(grid, out)

    def step():
        solver.pressure.fill(0.0)
        return dict(dispatch())

    for _ in range(warmup):
        step()
    ms, diags = timed(lib, ctx, step, steps)
    d = diags[-1]
    res = {"ms": round(ms, 4), "iterations": d["iterations"], "converged": all(x["converged"] for x in diags),
           "residual_rel": d["residual"] / d["bNorm"], "stopped_by": d["stoppedBy"],
           "max_iterations": d["maxIterations"], "steps": steps, **info}
    if net is not None:
        res["guess_used"] = sum(1 for x in diags if x["warmStart"] == 1) / len(diags)
        # the forward pass alone, for the split of the arm's time
        from tsl_array_n_gb300.tsl_array_n import Field
        g = Field("float", sc["shape"])
        h = sc["h"][0]
        fms, _ = timed(lib, ctx, lambda: net.forward(sc["shape"], h, solver.b, solver.dirichlet_mask,
                                                     solver.pressure, g), max(2, steps // 2))
        res["forward_ms"] = round(fms, 4)
        del g
        warmstart.attach(solver, None)
        net.close()
    solver.close()
    return res


def run_gb300(args):
    rank, world, dist = dist_setup(args.gpus)
    device = int(os.environ.get("LOCAL_RANK", 0))
    from tsl_array_n_gb300 import build as B
    B.build()
    import ctypes as C
    from tsl_array_n_gb300 import _lib, fluxflow as ff
    from tsl_array_n_gb300.tsl_array_n import init

    ctx = init(device)
    lib = _lib.load()
    n = args.size
    sc = sphere_inputs(n)
    shape, h = sc["shape"], sc["h"]
    col = ff.create_sdf_static_collider3(*shape, *h)
    col.add_shapes(sc["shapes"])
    cw = col.compute_face_weights()
    grid = ff.FaceCenteredGrid3(shape, h).set(sc["u"], sc["v"], sc["w"])
    out = ff.FaceCenteredGrid3(shape, h)
    levels = max(1, int(np.log2(n)) - 2)          # 256 -> 6 levels, 8^3 coarsest
    clocks = Clocks()   # sampling from here on: running well before the timed region
    if not args.profile_only:
        clocks.start()
    solver = make_solver(ff, sc, cw, levels, args.precision, args.coarse)
    if args.eager:
        solver.settings.useGraph = False
    dispatch = solver.project(grid, out)

    def step():
        solver.pressure.fill(0.0)
        return dispatch()

    for _ in range(args.warmup):
        d = step()
    iters = d["iterations"]
    if args.profile_only:
        # launch one kernel family a few times inside the "ff_profile" NVTX
        # range (for ncu --nvtx-include ff_profile/), then stop
        avg = C.c_float()
        _lib.check(lib.ff_pressure3_profile(solver.handle, PROF_IDS[args.profile_only], 3, C.byref(avg)))
        print(json.dumps({"profile_only": args.profile_only, "ms": avg.value}))
        return

    # device-resident timing
    barrier(dist)
    ctx.synchronize()
    clocks.mark()
    _lib.check(lib.ff_ctx_event_record(ctx.handle, 0))
    launches = 0
    diags = []
    for _ in range(args.steps):
        d = step()
        launches += d["kernelLaunches"] + 1
        diags.append(dict(d))
    _lib.check(lib.ff_ctx_event_record(ctx.handle, 1))
    ms = C.c_float()
    _lib.check(lib.ff_ctx_event_elapsed(ctx.handle, 0, 1, C.byref(ms)))
    ctx.synchronize()
    clk = clocks.stop()
    barrier(dist)
    ms_step = max_over_ranks(dist, ms.value / args.steps)
    # the timed solve's result, for the oracle comparison
    p_gpu = solver.pressure.to_array().astype(np.float64)
    u_gpu = [f.to_array() for f in (out.data_u, out.data_v, out.data_w)]

    # end-to-end through the C ABI with host buffers
    nb = [sc["u"].nbytes, sc["v"].nbytes, sc["w"].nbytes]
    hin, hout = [], []
    for b in nb:
        p = C.c_void_p()
        _lib.check(lib.ff_host_alloc(b, C.byref(p)))
        hin.append(p)
        q = C.c_void_p()
        _lib.check(lib.ff_host_alloc(b, C.byref(q)))
        hout.append(q)
    for p, a in zip(hin, (sc["u"], sc["v"], sc["w"])):
        C.memmove(p, a.ctypes.data, a.nbytes)

    def e2e_step():
        # ff_pressure3_project_host: u, v, w up from pinned memory, the
        # projection, the corrected u, v, w down; one call's upload overlaps
        # the previous call's download (separate copy streams)
        solver.pressure.fill(0.0)
        return solver.project_host(grid, out, hin, hout)

    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    barrier(dist)
    ctx.synchronize()
    _lib.check(lib.ff_ctx_event_record(ctx.handle, 2))
    for _ in range(args.steps):
        e2e_step()
    # the last download is inside the timed region
    _lib.check(lib.ff_ctx_join_copies(ctx.handle))
    _lib.check(lib.ff_ctx_event_record(ctx.handle, 3))
    e2e_ms = C.c_float()
    _lib.check(lib.ff_ctx_event_elapsed(ctx.handle, 2, 3, C.byref(e2e_ms)))
    e2e_ms_step = max_over_ranks(dist, e2e_ms.value / args.steps)
    uo = np.empty(sc["u"].size, np.float32)
    C.memmove(uo.ctypes.data, hout[0], uo.nbytes)
    assert np.all(np.isfinite(uo))
    for p in hin + hout:
        lib.ff_host_free(p)

    roof = None if args.no_kernel_profile else kernel_roofline(lib, solver, args, n)
    solver.close()

    arms = {}
    if args.arms != "none":
        for arm in args.arms.split(","):
            arms[arm] = run_arm(ff, lib, ctx, sc, cw, grid, out, levels, arm, args.arm_steps,
                                min(args.warmup, 2))
        arms[args.precision] = {"ms": round(ms_step, 4), "iterations": iters,
                                "converged": all(x["converged"] for x in diags),
                                "residual_rel": diags[-1]["residual"] / diags[-1]["bNorm"],
                                "stopped_by": diags[-1]["stoppedBy"], "steps": args.steps}

    cpu = err = None
    if rank == 0 and not args.no_cpu_baseline:
        wts = tuple(x.to_array().astype(np.float64) for x in (cw["u"], cw["v"], cw["w"]))
        cpu, p_ref = cpu_baseline(sc, levels, wts)
        err = oracle_error(sc, wts, p_gpu, u_gpu, p_ref)

    if rank == 0:
        emit_line(args, world, ms_step, e2e_ms_step, nb, launches, roof, cpu, clk, diags, iters, levels, n,
                  arms, err)
    if dist is not None:
        dist.destroy_process_group()


def kernel_roofline(lib, solver, args, n):
    """Per-kernel device time (CUDA events around single launches on the
    solver's stream) against the algorithmic bytes of each kernel."""
    import ctypes as C
    from tsl_array_n_gb300 import _lib
    peak, peak_kind = peaks()
    cells = n ** 3
    bpc = kernel_bytes_per_cell(args.precision)
    kern = {}
    # restrict and rz are the per-colour path's separate kernels; the fused
    # path runs the restriction with the residual and r.z inside the sweep
    fused_only = {k: v for k, v in PROF_IDS.items() if k not in ("restrict", "rz")}
    for name, kid in (PROF_IDS if args.precision == "mixed-bf16" else fused_only).items():
        avg = C.c_float()
        _lib.check(lib.ff_pressure3_profile(solver.handle, kid, 10, C.byref(avg)))
        kern[name] = {"ms": avg.value, "gbs": bpc[name] * cells / (avg.value * 1e-3) / 1e9}
    vc_ms = C.c_float()
    _lib.check(lib.ff_pressure3_profile(solver.handle, 7, 5, C.byref(vc_ms)))
    # share of the iteration: relax runs 2*(down+final) passes at level 0
    # launches per iteration at level 0: 2 down + 2 up sweeps (fused path)
    # or 8 colour passes (per-colour path)
    passes0 = 2 * (2 + 2) if args.precision == "mixed-bf16" else (2 + 2)
    shares = {"relax": kern["relax"]["ms"] * passes0, "x_residual": kern["x_residual"]["ms"],
              "p_pAp": kern["p_pAp"]["ms"], "residual": kern["residual"]["ms"]}
    dom = max(shares, key=shares.get)
    traffic = None
    prof_path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(prof_path):
        t = json.load(open(prof_path)).get(f"{dom}_{args.precision}_bytes_per_cell")
        traffic = t * cells if t else None
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(kern[dom]["gbs"], 1), "peak": peak,
            "unit": "GB/s", "frac": round(kern[dom]["gbs"] / peak, 4), "peak_kind": peak_kind,
            "traffic": traffic, "algorithmic_bytes": bpc[dom] * cells,
            "kernels": {k: {"ms": round(v["ms"], 4), "GB/s": round(v["gbs"], 1),
                            "frac": round(v["gbs"] / peak, 3)} for k, v in kern.items()},
            "vcycle_ms": round(vc_ms.value, 4)}
    return roof


def emit_line(args, world, ms_step, e2e_ms_step, nb, launches, roof, cpu, clk, diags, iters, levels, n,
              arms, err):
    cells = n ** 3
    line = {
        "metric": METRIC, "value": round(ms_step, 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": {"mixed": "f32(double-single iterate)+f64", "fp32": "f32+f64",
                  "mixed-bf16": "f32+bf16+f64"}[args.precision],
        "data": "synthetic (seeded 32-mode Fourier velocity, sphere collider)",
        "config": {"workload": f"3D MGPCG pressure projection {n}^3, sphere r={24 * n // 256} cells, "
                               f"closed walls + one pinned cell, {levels} levels, coarsest {args.coarse}, "
                               f"precision {args.precision}, tol 1e-6 relative, cold start",
                   "cells": cells, "iterations": iters,
                   "converged": all(x["converged"] for x in diags),
                   "residual_rel": diags[-1]["residual"] / diags[-1]["bNorm"],
                   "cell_updates_per_s": cells * iters / (ms_step * 1e-3),
                   "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(e2e_ms_step, 4), "unit": UNIT,
                "h2d_bytes_per_step": int(sum(nb)), "d2h_bytes_per_step": int(sum(nb))},
        "gpu_launches": launches,
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    if arms:
        line["arms"] = arms
        plain = arms.get("fp32")
        if plain:
            vs = {k: round(plain["ms"] / v["ms"], 2) for k, v in arms.items() if k != "fp32"}
            vs["note"] = ("plain FP32 MGPCG " + ("converged" if plain["converged"] else
                          f"did not reach 1e-6 (stopped by {plain['stopped_by']} at {plain['iterations']} "
                          f"iterations, residual {plain['residual_rel']:.2e})") +
                          "; ratio = plain ms / arm ms")
            line["vs_plain"] = vs
    if err:
        line["oracle_error"] = err
    print(json.dumps(line))


# --------------------------------------------------------- CPU baseline --
def _oracle_inputs(sc, weights=None):
    """Collider face weights: the GPU's baked weights when given (the oracle
    then solves exactly the system the GPU solved), else the FP64
    restatement's bake."""
    from oracle import oracle as O
    O.lib()
    if weights is not None:
        return O, weights
    _, wu, wv, ww = O.collider_bake(sc["shapes"], sc["shape"], sc["h"])
    return O, tuple(x.astype(np.float64) for x in (wu, wv, ww))


def oracle_projection(O, sc, w, levels, tol=1e-6, max_iter=None):
    """One whole projection on the FP64 CPU restatement, timed by phase:
    Dirichlet fields + build, hierarchy, PCG to `tol` with the oracle's own
    iteration count (cap ceil(1.5 max(res)), grid_pressure_solver3.js:133),
    velocity correction.  None of libff is on this path."""
    shape, h = sc["shape"], sc["h"]
    max_iter = max_iter or int(np.ceil(1.5 * max(shape)))
    t = {}
    t0 = time.perf_counter()
    mask, tgt, vent = O.dirichlet_fields(shape, sc["active"], sc["target"], w)
    b, _ = O.build_system(shape, h, sc["u"], sc["v"], sc["w"], collider_weights=w, mask=mask, target=tgt)
    t["build"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    mg = O.Multigrid(shape, h, mask, vent, w, levels=levels, coarse_direct=True)
    t["hierarchy"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    x, res, _ = O.pcg_solve(shape, h, b, None, mask, w, mg, "multigrid", tol=tol, max_iter=max_iter)
    t["pcg"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.correct(shape, h, x, sc["u"], sc["v"], sc["w"], collider_weights=w)
    t["correct"] = time.perf_counter() - t0
    return t, res, (x, b, mask, mg)


def cpu_baseline(sc, levels, weights):
    """The FP64 CPU restatement on all host cores: one whole projection of
    the same system to 1e-6, measured; then the same PCG continued to 1e-10
    for the reference pressure of the oracle comparison (not timed)."""
    O, w = _oracle_inputs(sc, weights)
    cores = os.cpu_count()
    t, res, (x, b, mask, mg) = oracle_projection(O, sc, w, levels)
    total = sum(t.values())
    shape, h = sc["shape"], sc["h"]
    x_ref, r2, _ = O.pcg_solve(shape, h, b, x, mask, w, mg, "multigrid", tol=1e-10, max_iter=200)
    n = sc["shape"][0]
    cpu = {"value": round(total * 1e3, 1), "unit": UNIT, "cores": cores, "kind": "port",
           "iterations": res["iterations"], "converged": res["converged"],
           "sample": f"measured: one whole FP64 oracle projection of the same {n}^3 system (Dirichlet fields, "
                     f"build, hierarchy, PCG to 1e-6 in {res['iterations']} iterations, correction), "
                     f"{total:.1f} s on {cores} cores (PCG {t['pcg']:.1f} s)"}
    return cpu, (x_ref, b, mask, r2)


def oracle_error(sc, w, p_gpu, u_gpu, ref):
    """Pressure and corrected velocity of the timed GPU solve against the
    oracle's solution converged to 1e-10, and the divergence the GPU's
    velocity leaves on non-Dirichlet cells (relative to the input's)."""
    from oracle import oracle as O
    x_ref, b, mask, r2 = ref
    shape, h = sc["shape"], sc["h"]

    def rel(a, r):
        return float(np.linalg.norm(np.asarray(a, np.float64) - r) / max(np.linalg.norm(r), 1e-300))

    u_ref = O.correct(shape, h, x_ref, sc["u"], sc["v"], sc["w"], collider_weights=w)
    b_after, _ = O.build_system(shape, h, *u_gpu, collider_weights=w, mask=mask,
                                target=np.zeros(mask.size))
    b_after[mask.astype(bool)] = 0.0
    fl = ~mask.astype(bool)
    e = np.asarray(p_gpu, np.float64) - x_ref
    return {"pressure_rel_l2": rel(p_gpu, x_ref),
            "pressure_rel_l2_mean_removed": float(np.linalg.norm(e[fl] - e[fl].mean()) / np.linalg.norm(x_ref)),
            "velocity_rel_l2": max(rel(g, r) for g, r in zip(u_gpu, u_ref)),
            "divergence_left_rel": float(np.linalg.norm(b_after) / np.linalg.norm(b)),
            "oracle_residual_rel": r2["residual"] / np.sqrt(r2["bb"]),
            "oracle": "FP64 CPU restatement on the GPU's face weights, PCG to 1e-10 relative"}


def run_reference(args):
    """--impl reference: the CPU restatement of the path on the host cores
    (the reference is JavaScript + WebGPU and has no CPU implementation of
    the 3D path that runs here), rank 0 only.  Every timed step is one whole
    projection of the full-size system to 1e-6 with the oracle's own
    iteration count; one warm-up step whatever --warmup says (a CPU solve
    has nothing to warm past the first)."""
    rank = int(os.environ.get("RANK", 0))
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    n = args.size
    sc = sphere_inputs(n)
    levels = max(1, int(np.log2(n)) - 2)
    O, w = _oracle_inputs(sc)
    warm = min(args.warmup, 1)
    samples, iters = [], []
    t_run = time.perf_counter()
    for i in range(warm + args.steps):
        t, res, _ = oracle_projection(O, sc, w, levels)
        if i >= warm:
            samples.append(sum(t.values()))
            iters.append(res["iterations"])
    run_s = time.perf_counter() - t_run
    value = float(np.mean(samples)) * 1e3
    cores = os.cpu_count()
    cpu = {"value": round(value, 1), "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"measured: FP64 CPU restatement (oracle/), {n}^3, every step one whole projection to 1e-6 "
                     f"({iters[-1]} iterations), {args.steps} timed steps after {warm} warm-up, "
                     f"{run_s:.0f} s in all"}
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": warm, "ms_per_step": round(value, 1),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded 32-mode Fourier velocity, sphere collider)",
        "config": {"workload": f"3D MGPCG pressure projection {n}^3, sphere r={24 * n // 256} cells, "
                               f"closed walls + one pinned cell, {levels} levels, coarsest direct, "
                               f"tol 1e-6 relative (CPU FP64 restatement)", "cells": n ** 3,
                   "iterations": iters[-1]},
        "cpu_baseline": cpu,
        "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp32", "mixed-bf16"])
    ap.add_argument("--coarse", default="direct", choices=["direct", "sweeps"])
    ap.add_argument("--arms", default="fp32,mixed-bf16,learned+mixed",
                    help="comparison arms timed on the same system ('none' to skip)")
    ap.add_argument("--arm-steps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-only", default=None, choices=sorted(PROF_IDS),
                    help="run one kernel family inside an NVTX range for ncu, then exit")
    ap.add_argument("--no-kernel-profile", action="store_true",
                    help="skip the per-kernel timing (used for clean ncu launch lists)")
    ap.add_argument("--eager", action="store_true",
                    help="launch the solve loop's kernels one by one instead of from the "
                         "conditional CUDA graph (ncu cannot list kernels inside one)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
