"""The 2D two-phase FLIP solver on the GPU through the C ABI.  Its own
stages (density and beta faces, the per-phase G2P blend, mixing, per-phase
resampling) are compared bit for bit with the 2D oracle; the stages it
shares with the 3D solver run on a one-cell-thick grid and are compared
with the 3D oracle at nz = 1; a bubble-rise scene checks the whole step."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SH = (32, 24)
H = (1 / 32, 1 / 24)
O = (0.0, 0.0)


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    bad = a != b
    assert not bad.any(), f"{bad.sum()} of {a.size} differ"


def scene(seed=3, n_per=5, **kw):
    from tsl_array_n_gb300 import fluxflow as ff
    grid = ff.FaceCenteredGrid2(SH, H, O)
    rng = np.random.default_rng(seed)
    n = n_per * SH[0] * SH[1]
    pos = (rng.random((n, 2)) ** 1.5).astype(np.float32)
    vel = (0.3 * rng.standard_normal((n, 2))).astype(np.float32)
    phase = (pos[:, 1] < 0.4).astype(np.float32)
    s = ff.create_grid_two_phase_flip_solver2(velocity_grid=grid, max_particles=n, dt=0.005, **kw)
    s.positions.from_array(pos)
    s.velocities.from_array(vel)
    s.phase.from_array(phase)
    return grid, s, pos.ravel(), vel.ravel(), phase, n


def faces(seed):
    rng = np.random.default_rng(seed)
    nx, ny = SH
    return (rng.standard_normal((nx + 1) * ny).astype(np.float32),
            rng.standard_normal(nx * (ny + 1)).astype(np.float32))


def test_density_and_beta_bit_exact(gpu, oracle):
    grid, s, pos, vel, phase, n = scene(gas_density=0.001, liquid_density=1.0)
    s.stage("density")
    cnt, acc, frac, rho, bu, bv = oracle.tp_density(SH, H, O, pos, phase, 0.001, 1.0)
    same(s.liquid_fraction.to_array(), frac)
    same(s.density.to_array(), rho)
    same(s.beta_u.to_array(), bu)
    same(s.beta_v.to_array(), bv)


def test_g2p_per_phase_blend_and_mix_bit_exact(gpu, oracle):
    grid, s, pos, vel, phase, n = scene(flip_ratio=0.95, gas_flip_ratio=0.8, velocity_damping=0.03, mixing=0.3,
                                        fade=0.05)
    old, new = faces(1), faces(2)
    grid.set(*old)
    s.stage("snapshotOld")
    grid.set(*new)
    s.stage("g2p")
    same(s.velocities.to_array(), oracle.tp_g2p(SH, H, O, pos, vel, phase, new, old, 0.95, 0.8, 0.03))
    s.stage("density")
    frac = s.liquid_fraction.to_array()
    s.stage("mixConcentration")
    same(s.phase.to_array(), oracle.tp_mix(SH, H, O, pos, frac, phase, 0.3, 0.05))


@pytest.mark.parametrize("mm", [(3, 8), (4, 6)])
def test_resample_bit_exact(gpu, oracle, mm):
    grid, s, pos, vel, phase, n = scene(resample={"minParticlesPerCell": mm[0], "maxParticlesPerCell": mm[1]})
    u, v = faces(4)
    grid.set(u, v)
    s.stage("density")
    s.stage("resample")
    cnt, acc, *_ = oracle.tp_density(SH, H, O, pos, phase, 0.01, 1.0)
    rp, rv, moved, stats = oracle.tp_resample(SH, H, O, pos, vel, phase, u, v, cnt, acc, n, *mm)
    assert moved > 0 and stats[1] > 0 and stats[3] > 0
    st = s.resample_stats()
    assert [st["liquidDonors"], st["liquidRequested"], st["gasDonors"], st["gasRequested"]] == list(stats)
    same(s.positions.to_array(), rp)
    same(s.velocities.to_array(), rv)


def test_shared_stages_match_the_3d_oracle_at_nz1(gpu, oracle):
    """advectParticles and P2G on the one-cell-thick grid against the 3D
    oracle with nz = 1, hz = max(hx, hy), particles on z = hz / 2."""
    grid, s, pos, vel, phase, n = scene(seed=8)
    u, v = faces(5)
    u, v = 0.5 * u, 0.5 * v
    grid.set(u, v)
    hz = max(H)
    sh3, h3, o3 = (SH[0], SH[1], 1), (H[0], H[1], hz), (0.0, 0.0, 0.0)
    p3 = np.column_stack([pos.reshape(-1, 2), np.full(n, np.float32(hz) * np.float32(0.5))]).astype(np.float32)
    w = np.zeros(SH[0] * SH[1] * 2, np.float32)
    s.stage("advectParticles")
    ref = oracle.flip_advect(sh3, h3, o3, u, v, w, None, p3, 0.005).reshape(-1, 3)
    same(s.positions.to_array().reshape(-1, 2), ref[:, :2])
    s.stage("p2g")
    v3 = np.column_stack([vel.reshape(-1, 2), np.zeros(n, np.float32)]).astype(np.float32)
    (ru, rv, _), _ = oracle.flip_p2g(sh3, h3, o3, ref.ravel(), v3)
    gu, gv = grid.get()
    same(gu, ru)
    same(gv, rv)


def test_bubble_rises(gpu):
    """A gas bubble under liquid at 100:1 in a closed box: every step's
    projection converges with the pressure pinned to 0 at the top-centre
    cell, particles stay in the box, and the bubble's centroid rises.  The
    solve uses the double-single iterate: the recomputed FP32 residual of
    this 100:1 system floors near 6e-4 (about 3e-5 of |b|), above the 1e-5
    tolerance, as the reference's own FP32 2D scenes floor."""
    from tsl_array_n_gb300 import fluxflow as ff
    nx, ny = 32, 32
    grid = ff.FaceCenteredGrid2((nx, ny), (1 / nx, 1 / ny))
    bubble = lambda p: (p[0] - 0.5) ** 2 + (p[1] - 0.3) ** 2 < 0.12 ** 2
    seed = ff.compute_two_phase_box_seed((0.0, 0.0), (1.0, 1.0), 1 / nx, 1 / ny,
                                         is_liquid=lambda p: p[1] < 0.7 and not bubble(p))
    n = seed["count"]
    s = ff.create_grid_two_phase_flip_solver2(velocity_grid=grid, max_particles=n, dt=0.004, gas_density=0.01,
                                              pressure={"tolerance": 1e-5, "precision": "mixed"})
    s.positions.from_array(seed["positionsArray"])
    s.phase.from_array(seed["phasesArray"])
    pos0 = seed["positionsArray"].reshape(-1, 2)
    in_bubble = np.array([bubble(p) for p in pos0.astype(np.float64)])
    y0 = pos0[in_bubble, 1].mean()
    for _ in range(25):
        d = s.on_advance_time_step()
        assert d["converged"] and not d["rejected"], d
    p = s.positions.to_array().reshape(-1, 2)
    assert np.all(np.isfinite(p)) and p.min() > 0 and p.max() < 1
    assert p[in_bubble, 1].mean() > y0 + 1e-3
    pr = s.pressure.to_array()
    assert pr[s.pin_cell[0] + nx * s.pin_cell[1]] == 0.0
