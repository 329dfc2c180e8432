"""Advection, velocity constraint and viscosity on the GPU through the C
ABI, against the FP32 oracle on the same inputs.  Both sides round every
FP32 operation on its own in the reference's evaluation order (the CUDA file
is built with -fmad=false, the oracle with -ffp-contract=off), so results
are compared bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SH = (28, 20, 24)
H = (1 / 28, 1 / 20, 1 / 24)
O = (0.0, 0.0, 0.0)
SPHERE = [{"type": "sphere", "center": [0.45, 0.5, 0.55], "radius": 0.22}]


def velocity(seed=3, amp=1.0):
    from tsl_array_n_gb300 import scenes
    rng = np.random.default_rng(seed)
    nx, ny, nz = SH
    u = scenes.fourier_face_field((nx + 1, ny, nz), H, 0, 8, amp, rng).ravel()
    v = scenes.fourier_face_field((nx, ny + 1, nz), H, 1, 8, amp, rng).ravel()
    w = scenes.fourier_face_field((nx, ny, nz + 1), H, 2, 8, amp, rng).ravel()
    return u, v, w


def collider():
    from tsl_array_n_gb300 import fluxflow as ff
    col = ff.create_sdf_static_collider3(*SH, *H)
    col.add_shapes(SPHERE)
    return col


def grid(u, v, w):
    from tsl_array_n_gb300 import fluxflow as ff
    return ff.FaceCenteredGrid3(SH, H, O).set(u, v, w)


def same(a, b):
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    assert a.shape == b.shape
    bad = ~((a == b) | (np.isnan(a) & np.isnan(b)))
    assert not bad.any(), f"{bad.sum()} of {a.size} differ, max {np.max(np.abs(a - b)[bad])}"


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("with_collider", [False, True])
def test_advect_faces_bit_exact(gpu, oracle, order, with_collider):
    from tsl_array_n_gb300 import fluxflow as ff
    u, v, w = velocity()
    vel = grid(u, v, w)
    out = grid(*(np.full_like(x, -3.0) for x in (u, v, w)))   # kept on closed faces
    col = collider() if with_collider else None
    dt = 0.02
    adv = ff.create_semi_lagrangian_advection_solver3(velocity_grid=vel, collider=col, dt=dt, order=order)
    adv.advect_face_centered3(vel, out)()
    phi = col.phi.to_array() if col else None
    ref = oracle.advect_faces(SH, H, O, u, v, w, phi, dt, order=order,
                              out=tuple(np.full_like(x, -3.0) for x in (u, v, w)))
    for g, r in zip(out.get(), ref):
        same(g, r)


@pytest.mark.parametrize("order", [1, 2])
def test_advect_scalar_bit_exact(gpu, oracle, order):
    from tsl_array_n_gb300 import fluxflow as ff
    from tsl_array_n_gb300.tsl_array_n import Field
    u, v, w = velocity(5)
    vel = grid(u, v, w)
    col = collider()
    rng = np.random.default_rng(9)
    s = rng.random(SH[0] * SH[1] * SH[2]).astype(np.float32)
    sf, so = Field("float", SH).from_array(s), Field("float", SH).from_array(np.zeros_like(s))
    adv = ff.create_semi_lagrangian_advection_solver3(velocity_grid=vel, collider=col, dt=0.03, order=order)
    adv.advect_scalar3(sf, so)()
    ref = oracle.advect_scalar(SH, H, O, u, v, w, col.phi.to_array(), s, 0.03, order=order,
                               out=np.zeros_like(s))
    same(so.to_array(), ref)


@pytest.mark.parametrize("direction", [1, -1])
def test_trace_points_bit_exact(gpu, oracle, direction):
    from tsl_array_n_gb300 import fluxflow as ff
    from tsl_array_n_gb300.tsl_array_n import Field
    u, v, w = velocity(7, amp=3.0)
    vel = grid(u, v, w)
    col = collider()
    rng = np.random.default_rng(4)
    p = (rng.random((5000, 3)) * np.array([1.0, 1.0, 1.0])).astype(np.float32)
    pin, pout = Field("vec3", (5000,)).from_array(p), Field("vec3", (5000,))
    adv = ff.create_semi_lagrangian_advection_solver3(velocity_grid=vel, collider=col, dt=0.05)
    adv.trace(pin, pout, direction)
    ref = oracle.trace(SH, H, O, u, v, w, col.phi.to_array(), p, 0.05, direction=direction)
    same(pout.to_array(), ref)


@pytest.mark.parametrize("weights", [False, True])
def test_constrain_velocity_bit_exact(gpu, oracle, weights):
    from tsl_array_n_gb300 import fluxflow as ff
    u, v, w = velocity(11, amp=2.0)
    u = u.copy()
    u[5] = 400.0
    v = v.copy()
    v[7] = np.nan
    vel = grid(u, v, w)
    col = collider()
    fw = col.compute_face_weights() if weights else None
    inflow = ff.create_sdf_inflow3(*SH, *H, velocity=(1.5, 0.0, -0.25), mode="set")
    inflow.add_shapes([{"type": "box", "center": [0.1, 0.5, 0.5], "halfExtents": [0.06, 0.2, 0.2]}])
    bc = ff.create_grid_blocked_boundary_condition_solver3(vel, *SH, *H, collider=col, inflows=[inflow],
                                                           collider_face_weights=fw)
    bc.closed_domain_boundary_flag = ff.DIRECTION_ALL_3D & ~ff.DIRECTION_RIGHT
    bc.constrain_velocity(5)
    ref = oracle.constrain_velocity(
        SH, H, O, u, v, w, phi=col.phi.to_array(),
        face_weights=tuple(fw[k].to_array() for k in "uvw") if weights else None,
        closed=63 & ~2, inflows=[(inflow.phi.to_array(), inflow.velocity, 0)], depth=5)
    for g, r in zip(vel.get(), ref):
        same(g, r)


def test_constrain_without_collider(gpu, oracle):
    from tsl_array_n_gb300 import fluxflow as ff
    u, v, w = velocity(12)
    vel = grid(u, v, w)
    bc = ff.create_grid_blocked_boundary_condition_solver3(vel, *SH, *H)
    bc.constrain_velocity()
    ref = oracle.constrain_velocity(SH, H, O, u, v, w, closed=63)
    for g, r in zip(vel.get(), ref):
        same(g, r)


def test_viscosity_bit_exact(gpu, oracle):
    from tsl_array_n_gb300 import fluxflow as ff
    u, v, w = velocity(13)
    a, b = grid(u, v, w), grid(u, v, w)
    ff.apply_viscosity3(a, b, nu=0.002, dt=0.01)
    ref = oracle.viscosity(SH, H, u, v, w, 0.002, 0.01)
    for g, r in zip(b.get(), ref):
        same(g, r)


def outflows():
    """Two outflows: a box slab at the high-x end on the velocity grid, and
    a sphere near the low-x end baked on a coarser grid of its own."""
    from tsl_array_n_gb300 import fluxflow as ff
    a = ff.create_sdf_outflow3(*SH, *H)
    a.add_shapes([{"type": "box", "center": [1.2, 0.5, 0.5], "halfExtents": [0.35, 2.0, 2.0]}])
    coarse, hc = (14, 10, 12), (1 / 14, 1 / 10, 1 / 12)
    b = ff.create_sdf_outflow3(*coarse, *hc)
    b.add_shapes([{"type": "sphere", "center": [0.05, 0.4, 0.6], "radius": 0.25}])
    return [a, b]


def orc_outflows(qs):
    return [(q.phi.to_array(), q.resolution, q.grid_spacing, q.origin) for q in qs]


@pytest.mark.parametrize("dt", [0.01, 0.2])
def test_outflow_velocity_bc_bit_exact(gpu, oracle, dt):
    from tsl_array_n_gb300 import fluxflow as ff
    u, v, w = velocity(5, amp=2.0)
    u = u + np.float32(1.0)
    vel = grid(u, v, w)
    qs = outflows()
    of = ff.create_grid_outflow_solver3(velocity_grid=vel, outflows=qs, dt=dt)
    of.apply_outflow_velocity_bc()
    ref = oracle.outflow_velocity(SH, H, O, u, v, w, dt, orc_outflows(qs))
    changed = 0
    for g, r, x in zip(vel.get(), ref, (u, v, w)):
        same(g, r)
        changed += int((r != x).sum())
    assert changed > 0
    # applyVelocityBC: false leaves the velocity alone
    vel2 = grid(u, v, w)
    ff.create_grid_outflow_solver3(velocity_grid=vel2, outflows=qs, dt=dt,
                                   apply_velocity_bc=False).apply_outflow_velocity_bc()
    for g, x in zip(vel2.get(), (u, v, w)):
        same(g, x)


def test_outflow_clear_scalar_and_dirichlet_bit_exact(gpu, oracle):
    from tsl_array_n_gb300 import fluxflow as ff
    from tsl_array_n_gb300.tsl_array_n import Field
    u, v, w = velocity(6)
    vel = grid(u, v, w)
    qs = outflows()
    of = ff.create_grid_outflow_solver3(velocity_grid=vel, outflows=qs, dt=0.01)
    rng = np.random.default_rng(9)
    s = rng.random(SH[0] * SH[1] * SH[2]).astype(np.float32) + 0.5
    f = Field("float", SH).from_array(s)
    of.clear_outflow_scalar_field(f)()
    ref = oracle.outflow_clear_scalar(SH, H, O, s, orc_outflows(qs))
    same(f.to_array(), ref)
    assert (ref == 0).any()
    a, t = of.dirichlet.fields(SH, H, O)
    ra, rt = oracle.outflow_dirichlet(SH, H, O, orc_outflows(qs))
    assert np.array_equal(a.to_array(), ra)
    same(t.to_array(), rt)
    # the standalone factory with a target
    a2, t2 = ff.create_outflow_pressure_dirichlet3(qs, target=0.5).fields(SH, H, O)
    assert np.array_equal(a2.to_array(), ra) and np.all(t2.to_array() == np.float32(0.5))


def test_projection_with_outflow_dirichlet(gpu):
    """A channel with a uniform inflow at low x and an outflow slab at high
    x: the projection pins the outflow cells to p = 0 and converges, and the
    velocity leaving the fluid region is divergence-free."""
    from tsl_array_n_gb300 import fluxflow as ff
    u, v, w = velocity(7, amp=0.5)
    u = u + np.float32(1.0)
    vel = grid(u, v, w)
    out = grid(u, v, w)
    of = ff.create_grid_outflow_solver3(velocity_grid=vel, outflows=outflows()[:1], dt=0.01)
    ps = ff.create_grid_pressure_solver3(SH, H, O, dirichlet=of.dirichlet, tolerance=1e-6)
    ps.project(vel, out)()
    d = ps.diagnostics
    assert d["converged"] and not d["rejected"], d
    a, _ = of.dirichlet.fields(SH, H, O)
    pinned = a.to_array().astype(bool)
    p = ps.pressure.to_array()
    assert pinned.any() and np.all(p[pinned] == 0)
    # combined with a host-side condition: b wins where both are active
    left = lambda x, y, z: (x < 0.1, np.full_like(x, 2.0))
    comb = ff.combine_dirichlet3(of.dirichlet, left)
    ca, ct = comb.fields(SH, H, O)
    ca, ct = ca.to_array().astype(bool), ct.to_array()
    x = ff.cell_positions(SH, H, O)[0]
    assert np.array_equal(ca, pinned | (x < 0.1))
    assert np.all(ct[x < 0.1] == 2.0) and np.all(ct[pinned & ~(x < 0.1)] == 0.0)
