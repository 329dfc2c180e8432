"""FLIP stages on the GPU through the C ABI against the FP32 oracle, bit for
bit (both round every FP32 operation on its own; P2G is int32 fixed point),
and a short dam break checked for what the projection guarantees."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SH = (24, 20, 16)
H = (1 / 24, 1 / 20, 1 / 16)
O = (0.0, 0.0, 0.0)


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    bad = a != b
    assert not bad.any(), f"{bad.sum()} of {a.size} differ"


def make(n_extra=0, **kw):
    from tsl_array_n_gb300 import fluxflow as ff
    grid = ff.FaceCenteredGrid3(SH, H, O)
    seed = ff.compute_flip_box_seed3((0.0, 0.0, 0.0), (0.5, 0.6, 1.0), *H)
    n = seed["count"]
    solver = ff.create_grid_flip_solver3(velocity_grid=grid, max_particles=n, dt=0.01, **kw)
    solver.positions.from_array(seed["positionsArray"])
    solver.velocities.from_array(np.zeros(3 * n, np.float32))
    return grid, solver, seed["positionsArray"].reshape(-1, 3), n


def smooth_velocity(seed=1, amp=0.5):
    from tsl_array_n_gb300 import scenes
    rng = np.random.default_rng(seed)
    nx, ny, nz = SH
    return (scenes.fourier_face_field((nx + 1, ny, nz), H, 0, 6, amp, rng).ravel(),
            scenes.fourier_face_field((nx, ny + 1, nz), H, 1, 6, amp, rng).ravel(),
            scenes.fourier_face_field((nx, ny, nz + 1), H, 2, 6, amp, rng).ravel())


@pytest.mark.parametrize("with_collider", [False, True])
def test_advect_particles_bit_exact(gpu, oracle, with_collider):
    from tsl_array_n_gb300 import fluxflow as ff
    col = None
    if with_collider:
        col = ff.create_sdf_static_collider3(*SH, *H)
        col.add_shapes([{"type": "sphere", "center": [0.35, 0.3, 0.5], "radius": 0.12}])
    grid, solver, pos, n = make(collider=col, collider_push_thresh=0.01 if col else 0.0)
    u, v, w = smooth_velocity(amp=2.0)
    grid.set(u, v, w)
    solver.stage("advectParticles")
    ref = oracle.flip_advect(SH, H, O, u, v, w, col.phi.to_array() if col else None, pos, 0.01,
                             push_thresh=0.01 if col else 0.0)
    same(solver.positions.to_array(), ref)


def test_p2g_and_mark_bit_exact(gpu, oracle):
    grid, solver, pos, n = make()
    rng = np.random.default_rng(5)
    vel = rng.standard_normal((n, 3)).astype(np.float32)
    solver.velocities.from_array(vel)
    solver.stage("p2g")
    (ru, rv, rw), _ = oracle.flip_p2g(SH, H, O, pos, vel)
    for g, r in zip(grid.get(), (ru, rv, rw)):
        same(g, r)
    solver.stage("markFluidCells")
    same(solver.fluid_mask.to_array(), oracle.flip_mark_fluid(SH, H, O, pos))


def test_g2p_bit_exact(gpu, oracle):
    grid, solver, pos, n = make(flip_ratio=0.95, velocity_damping=0.02)
    old = smooth_velocity(2)
    new = smooth_velocity(3)
    rng = np.random.default_rng(6)
    vel = rng.standard_normal((n, 3)).astype(np.float32)
    solver.velocities.from_array(vel)
    grid.set(*old)
    solver.stage("snapshotOld")
    grid.set(*new)
    solver.stage("g2p")
    ref = oracle.flip_g2p(SH, H, O, pos, vel, new, old, flip_ratio=0.95, damping=0.02)
    same(solver.velocities.to_array(), ref)


def test_dirichlet_of_air_cells(gpu, oracle):
    grid, solver, pos, n = make()
    solver.stage("markFluidCells")
    solver.stage("project")
    f = solver.grid_fields()
    active, target = oracle.flip_dirichlet(SH, H, O, oracle.flip_mark_fluid(SH, H, O, pos), (0.0, -9.81, 0.0), 0.01)
    same(f["dirichletActive"].to_array(), active)
    same(f["dirichletTarget"].to_array(), target)


def test_concentration_beta_and_reduced_gravity_bit_exact(gpu, oracle):
    grid, solver, pos, n = make(carry_concentration=True, ambient_density=1.0, component_density=1000.0,
                                mixing=0.3, fade=0.01)
    conc = (pos[:, 1] < 0.3).astype(np.float32)
    solver.concentration.from_array(conc)
    u, v, w = smooth_velocity(4)
    grid.set(u, v, w)
    solver.stage("markFluidCells")
    solver.stage("concentrationGrid")
    mask = oracle.flip_mark_fluid(SH, H, O, pos)
    cc, rho, beta = oracle.flip_concentration_grid(SH, H, O, pos, conc, mask, density=(1.0, 1000.0))
    f = solver.grid_fields()
    same(f["cellConcentration"].to_array(), cc)
    same(f["cellDensity"].to_array(), rho)
    for g, r in zip(f["beta"], beta):
        same(g.to_array(), r)
    solver.stage("gravity")
    ref = oracle.flip_reduced_gravity(SH, H, O, rho, beta, (0.0, -9.81, 0.0), 0.01, 1000.0, u, v, w)
    for g, r in zip(grid.get(), ref):
        same(g, r)
    solver.stage("concentrationParticle")
    same(solver.concentration.to_array(), oracle.flip_mix_fade(SH, H, O, pos, cc, conc, 0.3, 0.01))


def test_dam_break_steps(gpu, oracle):
    """A water column released in a closed box: every step projects to a
    divergence-free velocity on fluid cells, particles stay inside the
    domain and the column's centre of mass falls."""
    grid, solver, pos0, n = make(pressure={"multigrid": {"numberOfLevels": 3, "coarseSolve": "direct"},
                                           "tolerance": 1e-6, "precision": "mixed"})
    y0 = pos0[:, 1].mean()
    for _ in range(8):
        d = solver.on_advance_time_step()
        assert d["converged"] and not d["rejected"], d
    p = solver.positions.to_array().reshape(-1, 3)
    assert np.all(np.isfinite(p))
    for a in range(3):
        assert p[:, a].min() > 0 and p[:, a].max() < SH[a] * H[a]
    assert p[:, 1].mean() < y0 - 1e-3
    vel = solver.velocities.to_array()
    assert np.all(np.isfinite(vel)) and np.abs(vel).max() <= 500
    # the projection's own solver (pressureSolver): its pressure is the
    # solver's, its Dirichlet cells are the air cells of the last step
    from tsl_array_n_gb300 import tsl_array_n
    ps = solver.pressure_solver
    assert ps.level_shape(0) == SH
    air = ps.dirichlet_mask.to_array() != 0
    assert 0 < air.sum() < air.size
    assert np.array_equal(solver.pressure.to_array(), ps.pressure.to_array())
    y = tsl_array_n.Field("float", SH)
    ps.apply_laplacian(solver.pressure, y)
    assert np.all(np.isfinite(y.to_array()))


@pytest.mark.parametrize("shape,n,mm", [(SH, 24000, (4, 8)), ((40, 36, 33), 160000, (3, 6))])
def test_resample_bit_exact(gpu, oracle, shape, n, mm):
    """resamplePass on the GPU: the same donors move to the same cells with
    the same sampled velocities as the oracle (ranks are prefix sums in
    index order), and the fluid mask is rebuilt from the new positions."""
    from tsl_array_n_gb300 import fluxflow as ff
    h = tuple(1.0 / s for s in shape)
    grid = ff.FaceCenteredGrid3(shape, h, O)
    rng = np.random.default_rng(11)
    pos = (rng.random((n, 3)) * np.array([0.6, 0.5, 0.7])).astype(np.float32)
    vel = rng.standard_normal((n, 3)).astype(np.float32)
    nx, ny, nz = shape
    u, v, w = (rng.standard_normal(s).astype(np.float32)
               for s in ((nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1)))
    grid.set(u, v, w)
    solver = ff.create_grid_flip_solver3(velocity_grid=grid, max_particles=n, dt=0.01,
                                         resample={"minParticlesPerCell": mm[0], "maxParticlesPerCell": mm[1]})
    solver.positions.from_array(pos)
    solver.velocities.from_array(vel)
    solver.stage("resample")
    rp, rv, moved = oracle.flip_resample(shape, h, O, pos, vel, u, v, w, *mm)
    assert moved > 0
    st = solver.resample_stats()
    assert st["moved"] == moved
    same(solver.positions.to_array(), rp)
    same(solver.velocities.to_array(), rv)
    same(solver.fluid_mask.to_array(), oracle.flip_mark_fluid(shape, h, O, rp))


def test_resample_disabled_is_a_no_op(gpu):
    grid, solver, pos, n = make(resample={"enabled": False})
    solver.positions.from_array(np.zeros((n, 3), np.float32) + 0.01)   # all in one cell
    solver.stage("resample")
    assert np.all(solver.positions.to_array() == np.float32(0.01))
    assert solver.resample_stats() == {"donors": 0, "requested": 0, "moved": 0}
