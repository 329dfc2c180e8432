"""The 3D two-phase FLIP solver through the C ABI against the oracle's FP32
restatement on the same seeded inputs: density and beta faces, P2G and the
per-phase G2P blend bit for bit; the six-neighbour per-phase resampling
bit for bit; one variable-coefficient projection at a 1000:1 density ratio
against the FP64 oracle's converged pressure; and a short dam break."""
import numpy as np
import pytest

from conftest import oracle_pressure

pytestmark = pytest.mark.gpu

RES = (24, 16, 12)
H = 1.0 / 16


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def make(gas=0.001, resample=True, seed=3, precision="mixed", tol=1e-6):
    from tsl_array_n_gb300 import fluxflow as ff
    nx, ny, nz = RES
    grid = ff.FaceCenteredGrid3(RES, (H, H, H))
    sd = ff.compute_two_phase_box_seed3((0, 0, 0), (nx * H, ny * H, nz * H), (H, H, H), (0, 0, 0),
                                        (10 * H, 8 * H, nz * H))
    rng = np.random.default_rng(seed)
    vel = (0.3 * rng.standard_normal(3 * sd["count"])).astype(np.float32)
    solver = ff.create_grid_two_phase_flip_solver3(
        velocity_grid=grid, max_particles=sd["count"], dt=0.004, liquid_density=1.0, gas_density=gas,
        flip_ratio=0.95, resample={"enabled": resample},
        pressure={"multigrid": {"numberOfLevels": 3, "coarseSolve": "direct"}, "precision": precision,
                  "tolerance": tol})
    solver.set_particles(sd["positionsArray"], vel, sd["phasesArray"])
    return solver, grid, sd, vel


def faces(grid):
    return [f.to_array() for f in (grid.data_u, grid.data_v, grid.data_w)]


def test_density_beta_and_p2g_bit_exact(gpu, oracle):
    s, grid, sd, vel = make()
    s.stage("density")
    nc = int(np.prod(RES))
    cc, rho, (bu, bv, bw) = oracle.flip_concentration_grid(RES, (H,) * 3, (0, 0, 0), sd["positionsArray"],
                                                           sd["phasesArray"], np.ones(nc, np.float32),
                                                           density=(0.001, 1.0))
    assert np.array_equal(s.liquid_fraction.to_array(), cc)
    assert np.array_equal(s.density.to_array(), rho)
    for got, ref in ((s.beta_u, bu), (s.beta_v, bv), (s.beta_w, bw)):
        assert np.array_equal(got.to_array(), ref)
    assert bu.max() > 900          # gas faces carry the 1000:1 ratio
    cnt, acc = oracle.tp3_counts(RES, (H,) * 3, (0, 0, 0), sd["positionsArray"], sd["phasesArray"])
    gc, ga = s.cell_counts()
    assert np.array_equal(gc, cnt) and np.array_equal(ga, acc)
    s.stage("p2g")
    (u, v, w), _ = oracle.flip_p2g(RES, (H,) * 3, (0, 0, 0), sd["positionsArray"], vel)
    for got, ref in zip(faces(grid), (u, v, w)):
        assert np.array_equal(got, ref)


def test_per_phase_g2p_bit_exact(gpu, oracle):
    s, grid, sd, vel = make()
    rng = np.random.default_rng(11)
    old = [rng.standard_normal(f.count).astype(np.float32) for f in (grid.data_u, grid.data_v, grid.data_w)]
    new = [rng.standard_normal(f.count).astype(np.float32) for f in (grid.data_u, grid.data_v, grid.data_w)]
    grid.set(*old)
    s.stage("snapshotOld")
    grid.set(*new)
    s.stage("g2p")
    _, got, _ = s.get_particles(sd["count"])
    ref = oracle.tp3_g2p(RES, (H,) * 3, (0, 0, 0), sd["positionsArray"], vel, sd["phasesArray"], new, old,
                         flip_ratio=0.95, gas_ratio=0.90, damping=0.02)
    assert np.array_equal(got, ref)


def test_per_phase_resample_bit_exact(gpu, oracle):
    """Cells emptied and crowded on purpose: liquid and gas donors from the
    crowded cells fill the emptied ones of their phase, in the oracle's
    order."""
    s, grid, sd, vel = make()
    pos = sd["positionsArray"].reshape(-1, 3).copy()
    ph = sd["phasesArray"].copy()
    cell = np.floor(pos / H).astype(int)
    # empty a few liquid and gas cells (their particles go to crowded cells)
    rng = np.random.default_rng(5)
    for ci, cj, ck, ti, tj, tk in ((3, 3, 3, 5, 5, 5), (17, 10, 6, 20, 12, 8), (8, 4, 9, 2, 2, 2),
                                   (12, 13, 2, 22, 14, 10)):
        sel = np.all(cell == (ci, cj, ck), axis=1)
        pos[sel] = (np.array([ti, tj, tk]) + 0.25 + 0.5 * rng.random((sel.sum(), 3))) * H
    pos = pos.astype(np.float32).ravel()
    rng2 = np.random.default_rng(9)
    u, v, w = [rng2.standard_normal(f.count).astype(np.float32) for f in (grid.data_u, grid.data_v, grid.data_w)]
    s.set_particles(pos, vel, ph)
    s.stage("density")
    grid.set(u, v, w)
    s.stage("resample")
    gp, gv, _ = s.get_particles(sd["count"])
    cnt, acc = oracle.tp3_counts(RES, (H,) * 3, (0, 0, 0), pos, ph)
    rp, rv, moved, stats = oracle.tp3_resample(RES, (H,) * 3, (0, 0, 0), pos, vel, ph, u, v, w, cnt, acc,
                                               sd["count"])
    assert moved > 0 and stats[1] > 0 and stats[3] > 0
    st = s.resample_stats()
    assert [st["liquidDonors"], st["liquidRequested"], st["gasDonors"], st["gasRequested"]] == list(stats)
    assert np.array_equal(gp, rp)
    assert np.array_equal(gv, rv)


def test_projection_at_1000_to_1_matches_oracle(gpu, oracle):
    """One variable-coefficient projection (beta = 1000 on gas faces): b
    equals the oracle's build with the beta faces as face weights, and the
    pressure and corrected velocity are within 1e-5 relative L2 of the FP64
    oracle's converged solution."""
    s, grid, sd, vel = make(tol=1e-7)
    for st in ("density", "p2g", "snapshotOld", "extrapolateWeight", "constrainVelocity", "gravity",
               "constrainVelocity"):
        s.stage(st)
    u, v, w = faces(grid)
    beta = [f.to_array().astype(np.float64) for f in (s.beta_u, s.beta_v, s.beta_w)]
    s.stage("project")
    nx, ny, nz = RES
    active = np.zeros(nx * ny * nz, np.uint8)
    active[nx // 2 + nx * (ny - 1) + nx * ny * (nz // 2)] = 1
    mask, tgt, vent = oracle.dirichlet_fields(RES, active, np.zeros(active.size), None)
    b, _ = oracle.build_system(RES, (H,) * 3, u, v, w, face_weights=beta, mask=mask, target=tgt)
    assert rel(s.pressure_solver.b.to_array(), b) < 1e-6
    p = s.pressure.to_array().astype(np.float64)
    p_ref = oracle_pressure(oracle, RES, (H,) * 3, b, mask, beta, vent, levels=3, tol=1e-12, max_iter=2000)
    u2, v2, w2 = faces(grid)
    ref = oracle.correct(RES, (H,) * 3, p_ref, u, v, w, face_weights=beta)
    perr = rel(p, p_ref)
    uerr = max(rel(g, r) for g, r in zip((u2, v2, w2), ref))
    print(f"two-phase 3D 1000:1: pressure rel-L2 {perr:.3e}, velocity rel-L2 {uerr:.3e}")
    assert perr < 1e-5 and uerr < 1e-5, (perr, uerr)


def test_dam_break_steps(gpu):
    """Forty steps of a 1000:1 dam break: every projection converges, the
    velocities stay finite, the liquid particles keep their phase and the
    liquid column's centroid falls."""
    s, grid, sd, vel = make(seed=1)
    s.set_particles(sd["positionsArray"], np.zeros_like(sd["positionsArray"]), sd["phasesArray"])
    liquid = sd["phasesArray"] > 0.5
    y0 = sd["positionsArray"].reshape(-1, 3)[liquid, 1].mean()
    for _ in range(40):
        d = s.on_advance_time_step()
        assert d["converged"] and not d["rejected"], d
    pos, v, ph = s.get_particles(sd["count"])
    assert np.all(np.isfinite(pos)) and np.all(np.isfinite(v))
    assert int((ph > 0.5).sum()) == int(liquid.sum())
    y1 = pos.reshape(-1, 3)[ph > 0.5, 1].mean()
    assert y1 < y0 - 0.25 * H, (y0, y1)
