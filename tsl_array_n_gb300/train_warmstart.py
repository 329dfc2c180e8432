"""Training of the learned warm start at the configuration's scale: pairs of
(divergence b, Dirichlet mask, previous pressure) -> pressure that the plain
solver generates on 128^3 grids with 1-4 random sphere or box obstacles of
8-32 cells and random smooth velocity fields, then Adam on the U-Net with
the library's own forward and backward kernels, then the gain on held-out
256^3 systems (PCG iterations and milliseconds from the network's guess
against the cold start, to the same 1e-6 tolerance).

    python -m tsl_array_n_gb300.train_warmstart --pairs 4096 --res 128 \\
        --epochs 8 --out tsl_array_n_gb300/weights/unet_warmstart.npy \\
        --report train_report.json

Scenes come in twins that share their obstacles: the first twin is solved
from a cold start (previous pressure absent), the second has a velocity
field perturbed by 20% and takes the first twin's pressure as its previous
pressure, as consecutive steps of a simulation would.  Every pair stays in
device memory (about 19 MB per pair at 128^3).  The velocity fields are
built on the host by a pool of threads (numpy releases the interpreter lock
in its array loops), a bounded window of twins ahead of the GPU.  All inputs
are synthetic and seeded.
"""
import argparse
import collections
import json
import math
import os
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import scenes


# ------------------------------------------------------------ host scenes --
def _obstacles(rng, n):
    """1-4 spheres or boxes whose size is 8-32 cells, inside the domain."""
    out = []
    for _ in range(int(rng.integers(1, 5))):
        size = float(rng.uniform(8, 32)) / n          # diameter or box edge, domain units
        c = [float(rng.uniform(0.15 + size / 2, 0.85 - size / 2)) for _ in range(3)]
        if rng.random() < 0.5:
            out.append({"type": "sphere", "center": c, "radius": size / 2})
        else:
            he = [size / 2 * float(rng.uniform(0.5, 1.0)) for _ in range(3)]
            ax = rng.normal(size=3)
            out.append({"type": "box", "center": c, "halfExtents": he,
                        "rotation": {"axis": [float(a) for a in ax], "angle": float(rng.uniform(0, math.pi))}})
    return out


def _velocity(n, rng, modes=16, amplitude=1.0):
    """Smooth random MAC velocity with closed walls (zero normal velocity on
    the domain boundary)."""
    h = (1.0 / n,) * 3
    u = scenes.fourier_face_field((n + 1, n, n), h, 0, modes, amplitude, rng)
    v = scenes.fourier_face_field((n, n + 1, n), h, 1, modes, amplitude, rng)
    w = scenes.fourier_face_field((n, n, n + 1), h, 2, modes, amplitude, rng)
    u[:, :, 0] = u[:, :, n] = 0.0
    v[:, 0, :] = v[:, n, :] = 0.0
    w[0, :, :] = w[n, :, :] = 0.0
    return u.ravel(), v.ravel(), w.ravel()


def make_twin(args):
    """One twin of scenes (seeded): obstacles, a velocity field and the same
    field perturbed by 20%."""
    n, seed = args
    rng = np.random.default_rng(seed)
    shapes = _obstacles(rng, n)
    u, v, w = _velocity(n, rng)
    du, dv, dw = _velocity(n, rng, amplitude=0.2)
    return shapes, (u, v, w), (u + du, v + dv, w + dw)


# --------------------------------------------------------------- pairs --
class Pairs:
    """Solver-generated training pairs resident in device memory."""

    def __init__(self):
        self.items = []   # (b, mask, p_prev or None, target) Fields

    def __len__(self):
        return len(self.items)


def _twins(pool, n, seed, count, window):
    """The twins in order, built `window` ahead on the thread pool."""
    pending = collections.deque()
    nxt = 0
    while nxt < count or pending:
        while nxt < count and len(pending) < window:
            pending.append(pool.submit(make_twin, (n, seed * 100003 + nxt)))
            nxt += 1
        yield pending.popleft().result()


def generate(pairs, n, seed, pool, solver_levels=5, log=None, window=32):
    """`pairs` pairs at n^3 (twins of a cold and a warm pair).  Returns a
    Pairs object and the generation statistics."""
    from . import fluxflow as ff
    from .tsl_array_n import Field
    shape, h = (n, n, n), (1.0 / n,) * 3
    active = np.zeros(n ** 3, np.uint8)
    active[0] = 1
    target0 = np.zeros(n ** 3, np.float32)
    col = ff.create_sdf_static_collider3(*shape, *h)
    grid = ff.FaceCenteredGrid3(shape, h)
    out = ff.FaceCenteredGrid3(shape, h)
    solver = None
    data = Pairs()
    iters = []
    t0 = time.perf_counter()
    twins = (pairs + 1) // 2
    for k, (shapes, vel_a, vel_b) in enumerate(_twins(pool, n, seed, twins, window)):
        col.shapes = []
        col.add_shapes(shapes)
        cw = col.compute_face_weights()
        if solver is None:
            solver = ff.create_grid_pressure_solver3(
                shape, h, collider_weights=cw, dirichlet=(active, target0),
                multigrid={"numberOfLevels": solver_levels, "coarseSolve": "direct"}, precision="mixed",
                tolerance=1e-6)
        else:
            solver.set_collider_weights(cw)
        prev = None
        for vel in (vel_a, vel_b):
            if len(data) >= pairs:
                break
            grid.set(*vel)
            solver.pressure.fill(0.0)
            d = solver.project(grid, out)()
            iters.append(d["iterations"])
            b = Field("float", shape).copy_from(solver.b)
            mask = Field("uint8", shape).copy_from(solver.dirichlet_mask)
            p = Field("float", shape).copy_from(solver.pressure)
            data.items.append((b, mask, prev, p))
            prev = p
        if log and (k + 1) % 256 == 0:
            log(f"generated {len(data)} pairs in {time.perf_counter() - t0:.1f} s")
    stats = {"pairs": len(data), "resolution": n, "seconds": round(time.perf_counter() - t0, 1),
             "solver_iterations_mean": float(np.mean(iters)), "solver_iterations_max": int(np.max(iters))}
    solver.close()
    return data, stats


# -------------------------------------------------------------- training --
def train(net, data, epochs, lr, n, seed=0, holdout=64, time_budget=None, log=None):
    """Adam over the pairs in a seeded random order each epoch (cosine decay
    of the learning rate); the last `holdout` pairs are kept out and scored
    after every epoch (mean loss)."""
    rng = np.random.default_rng(seed)
    shape, h = (n, n, n), 1.0 / n
    train_idx = np.arange(len(data) - holdout)
    hold = list(range(len(data) - holdout, len(data)))
    hist = []
    t0 = time.perf_counter()
    steps = 0
    for ep in range(epochs):
        order = rng.permutation(train_idx)
        losses = []
        lr_ep = lr * 0.5 * (1.0 + math.cos(math.pi * ep / max(1, epochs)))
        for i in order:
            b, m, pp, t = data.items[i]
            losses.append(net.train_step(shape, h, b, m, pp, t, lr=lr_ep))
            steps += 1
            if time_budget and time.perf_counter() - t0 > time_budget:
                break
        held = float(np.mean([net.loss_backward(shape, h, *data.items[i]) for i in hold]))
        hist.append({"epoch": ep, "lr": lr_ep, "train_loss": float(np.mean(losses)), "holdout_loss": held,
                     "seconds": round(time.perf_counter() - t0, 1)})
        if log:
            log(json.dumps(hist[-1]))
        if time_budget and time.perf_counter() - t0 > time_budget:
            break
    return {"epochs": len(hist), "steps": steps, "history": hist,
            "ms_per_step": round((time.perf_counter() - t0) * 1e3 / max(1, steps + len(hist) * len(hold)), 3)}


# ------------------------------------------------------------ evaluation --
def evaluate(net, n=256, seeds=(1, 2, 3), repeats=3):
    """Held-out n^3 systems: the benchmark's sphere scene (seed 1) and
    random-obstacle scenes (other seeds).  Cold start against the network's
    guess, both to 1e-6 with the mixed-precision solver; ms per projection
    (CUDA events on the solver's stream) and PCG iterations."""
    import ctypes as C
    from . import _lib, fluxflow as ff, warmstart
    from .tsl_array_n import context
    lib = _lib.load()
    ctx = context()
    res = []
    for sd in seeds:
        if sd == 1:
            sc = scenes.sphere_scene(n=n, radius_cells=24 * n // 256, modes=32, seed=1)
            shapes, vel, name = sc["shapes"], (sc["u"], sc["v"], sc["w"]), "sphere r=24, 32 modes"
        else:
            shapes, vel, _ = make_twin((n, 7919 * sd))
            name = f"{len(shapes)} random obstacles, 16 modes"
        shape, h = (n, n, n), (1.0 / n,) * 3
        active = np.zeros(n ** 3, np.uint8)
        active[0] = 1
        col = ff.create_sdf_static_collider3(*shape, *h)
        col.add_shapes(shapes)
        cw = col.compute_face_weights()
        grid = ff.FaceCenteredGrid3(shape, h).set(*vel)
        out = ff.FaceCenteredGrid3(shape, h)
        levels = max(1, int(math.log2(n)) - 2)
        row = {"scene": name, "seed": sd}
        for arm in ("cold", "learned"):
            solver = ff.create_grid_pressure_solver3(
                shape, h, collider_weights=cw, dirichlet=(active, np.zeros(n ** 3, np.float32)),
                multigrid={"numberOfLevels": levels, "coarseSolve": "direct"}, precision="mixed", tolerance=1e-6)
            if arm == "learned":
                warmstart.attach(solver, net)
            disp = solver.project(grid, out)
            for _ in range(2):
                solver.pressure.fill(0.0)
                disp()
            ctx.synchronize()
            _lib.check(lib.ff_ctx_event_record(ctx.handle, 8))
            ds = []
            for _ in range(repeats):
                solver.pressure.fill(0.0)
                ds.append(dict(disp()))
            _lib.check(lib.ff_ctx_event_record(ctx.handle, 9))
            ms = C.c_float()
            _lib.check(lib.ff_ctx_event_elapsed(ctx.handle, 8, 9, C.byref(ms)))
            row[arm] = {"ms": round(ms.value / repeats, 3), "iterations": ds[-1]["iterations"],
                        "converged": all(d["converged"] for d in ds),
                        "residual_rel": ds[-1]["residual"] / ds[-1]["bNorm"]}
            if arm == "learned":
                row[arm]["guess_used"] = ds[-1]["warmStart"] == 1
                warmstart.attach(solver, None)
            solver.close()
        row["iterations_saved"] = row["cold"]["iterations"] - row["learned"]["iterations"]
        res.append(row)
    return res


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=4096, help="0: evaluate --init's weights only")
    ap.add_argument("--res", type=int, default=128)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--holdout", type=int, default=64)
    ap.add_argument("--time-budget", type=float, default=None, help="seconds of training at most")
    ap.add_argument("--workers", type=int, default=max(1, min(16, (os.cpu_count() or 2) - 1)))
    ap.add_argument("--eval-res", type=int, default=256)
    ap.add_argument("--init", default=None, help="start from these weights (.npy)")
    ap.add_argument("--out", default=None, help="save the trained weights here (.npy)")
    ap.add_argument("--report", default=None, help="write the JSON report here")
    args = ap.parse_args(argv)

    def log(msg):
        print(msg, flush=True)

    from . import tsl_array_n
    from .warmstart import UNetWarmStart
    tsl_array_n.init(0)
    net = UNetWarmStart(seed=args.seed + 1)
    if args.init:
        net.load(args.init)
    gen = tr = None
    if args.pairs > 0:
        with ThreadPoolExecutor(args.workers) as pool:
            data, gen = generate(args.pairs, args.res, args.seed, pool, log=log)
        log(json.dumps({"generated": gen}))
        tr = train(net, data, args.epochs, args.lr, args.res, seed=args.seed,
                   holdout=min(args.holdout, len(data) // 4), time_budget=args.time_budget, log=log)
        if args.out:
            os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
            net.save(args.out)
        del data
    ev = evaluate(net, n=args.eval_res)
    report = {"generation": gen, "training": tr, "evaluation": ev,
              "network": {"parameters": net.param_count, "levels": 3, "channels": [16, 32, 64]}}
    log(json.dumps({"evaluation": ev}))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(report, f, indent=1)
    return report


if __name__ == "__main__":
    main()
