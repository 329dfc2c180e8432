"""CPU checks of the FP32 restatement of the grid-velocity kernels
(advection_solver3.js, grid_blocked_boundary_condition_solver3.js, explicit
viscosity): properties the reference's formulas guarantee exactly."""
import numpy as np
import pytest


SH, H, O = (12, 10, 8), (1 / 12, 1 / 10, 1 / 8), (0.0, 0.0, 0.0)


def sizes(sh):
    nx, ny, nz = sh
    return (nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1)


def test_zero_velocity_advection_is_identity(oracle):
    su, sv, sw = sizes(SH)
    rng = np.random.default_rng(0)
    u, v, w = rng.standard_normal(su), rng.standard_normal(sv), rng.standard_normal(sw)
    z = [np.zeros(n, np.float32) for n in (su, sv, sw)]
    s = rng.standard_normal(SH[0] * SH[1] * SH[2]).astype(np.float32)
    # a zero velocity traces every point onto itself; a cubic sample at a
    # grid point is that grid value (up to the rounding of position -> index)
    out = oracle.advect_scalar(SH, H, O, *z, None, s, 0.1)
    np.testing.assert_allclose(out, s, rtol=0, atol=2e-6 * np.abs(s).max())
    for order in (1, 2):
        uo, vo, wo = oracle.advect_faces(SH, H, O, *z, None, 0.1, order=order,
                                         out=(u.astype(np.float32), v.astype(np.float32), w.astype(np.float32)))
        assert np.array_equal(uo, np.zeros(su, np.float32))


def test_uniform_velocity_translates_linear_field(oracle):
    """The monotone cubic reproduces linear data, and a uniform velocity
    traces back by exactly v dt: a linear scalar is translated."""
    su, sv, sw = sizes(SH)
    u = np.full(su, 0.3, np.float32)
    v = np.full(sv, -0.2, np.float32)
    w = np.zeros(sw, np.float32)
    nx, ny, nz = SH
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    x, y = (i + 0.5) * H[0], (j + 0.5) * H[1]
    s = (2.0 * x + 3.0 * y).astype(np.float32).ravel()
    dt = 0.05
    out = oracle.advect_scalar(SH, H, O, u, v, w, None, s, dt).reshape(nz, ny, nx)
    want = 2.0 * (x - 0.3 * dt) + 3.0 * (y + 0.2 * dt)
    # away from the edges, where the clamped taps flatten the cubic
    inner = (slice(None), slice(2, ny - 2), slice(2, nx - 2))
    np.testing.assert_allclose(out[inner], want[inner], rtol=0, atol=2e-5)


def test_constant_field_stays_constant_with_collider(oracle):
    su, sv, sw = sizes(SH)
    rng = np.random.default_rng(1)
    u, v, w = (rng.standard_normal(n).astype(np.float32) * 0.5 for n in (su, sv, sw))
    phi, _, _, _ = oracle.collider_bake([{"type": "sphere", "center": [0.5, 0.5, 0.5], "radius": 0.25}], SH, H)
    s = np.full(SH[0] * SH[1] * SH[2], 7.25, np.float32)
    for order in (1, 2):
        out = oracle.advect_scalar(SH, H, O, u, v, w, phi, s, 0.04, order=order)
        assert np.all(out == np.float32(7.25))


def test_trace_stops_at_the_collider(oracle):
    """A point pushed into a solid stops on (or just outside) its surface:
    the last substep is blended where the SDF crosses zero."""
    su, sv, sw = sizes(SH)
    u = np.full(su, -1.0, np.float32)   # back-trace moves +x
    v, w = np.zeros(sv, np.float32), np.zeros(sw, np.float32)
    shapes = [{"type": "box", "center": [0.8, 0.5, 0.5], "halfExtents": [0.1, 0.5, 0.5]}]
    phi, _, _, _ = oracle.collider_bake(shapes, SH, H)
    p = np.array([[0.3, 0.5, 0.5]], np.float32)
    q = oracle.trace(SH, H, O, u, v, w, phi, p, dt=1.0)
    assert 0.6 < q[0] < 0.72       # solid begins at x = 0.7
    free = oracle.trace(SH, H, O, u, v, w, None, p, dt=0.25)
    assert abs(free[0] - 0.55) < 1e-6


def test_constrain_walls_clamp_and_inflow(oracle):
    su, sv, sw = sizes(SH)
    nx, ny, nz = SH
    u = np.ones(su, np.float32)
    v = np.full(sv, 250.0, np.float32)
    w = np.ones(sw, np.float32)
    w[3] = np.nan
    inflow_phi, _, _, _ = oracle.collider_bake(
        [{"type": "box", "center": [0.5, 0.5, 0.5], "halfExtents": [0.2, 0.2, 0.2]}], SH, H)
    uo, vo, wo = oracle.constrain_velocity(SH, H, O, u, v, w, closed=1 | 8,
                                           inflows=[(inflow_phi, (2.0, 0.0, 0.5), 1)])
    U = uo.reshape(nz, ny, nx + 1)
    assert np.all(U[:, :, 0] == 0)           # LEFT wall
    assert np.any(U[:, :, nx] != 0)          # RIGHT open
    V = vo.reshape(nz, ny + 1, nx)
    assert np.all(V[:, ny, :] == 0)          # UP wall
    assert np.all(np.abs(vo) <= 100)         # clamp
    assert wo[3] == 0.0                      # non-finite -> 0
    assert np.any(U == np.float32(3.0))      # 'add' inflow: 1 + 2


def test_constrain_collider_closes_solid_faces(oracle):
    su, sv, sw = sizes(SH)
    rng = np.random.default_rng(2)
    u, v, w = (rng.standard_normal(n).astype(np.float32) for n in (su, sv, sw))
    shapes = [{"type": "sphere", "center": [0.5, 0.5, 0.5], "radius": 0.3}]
    phi, wu, wv, ww = oracle.collider_bake(shapes, SH, H)
    uo, vo, wo = oracle.constrain_velocity(SH, H, O, u, v, w, phi=phi, face_weights=(wu, wv, ww), closed=63)
    # faces between two solid cells carry no normal flow after the
    # constraint's no-flux projection
    nx, ny, nz = SH
    P = phi.reshape(nz, ny, nx)
    U = uo.reshape(nz, ny, nx + 1)
    both = (P[:, :, 1:] < 0) & (P[:, :, :-1] < 0)
    inner = U[:, :, 1:nx][both]
    assert np.all(np.isfinite(inner))
    assert np.all(np.abs(uo) <= 100)


def test_viscosity_constant_and_quadratic(oracle):
    su, sv, sw = sizes(SH)
    nx, ny, nz = SH
    c = [np.full(n, 1.5, np.float32) for n in (su, sv, sw)]
    out = oracle.viscosity(SH, H, *c, nu=0.01, dt=0.1)
    for o in out:
        assert np.all(o == np.float32(1.5))
    # u = y^2 on interior faces: lap = 2, out = u + dt nu 2
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx + 1), indexing="ij")
    y = (j + 0.5) * H[1]
    u = (y ** 2).astype(np.float32).ravel()
    uo, _, _ = oracle.viscosity(SH, H, u, c[1], c[2], nu=0.01, dt=0.1)
    U, U0 = uo.reshape(nz, ny, nx + 1), u.reshape(nz, ny, nx + 1)
    inner = (slice(None), slice(1, ny - 1), slice(1, nx))
    np.testing.assert_allclose(U[inner] - U0[inner], 0.002, rtol=2e-3)


# ---- outflow (grid_outflow_solver3.js) ------------------------------------
def slab_phi(sh, h, o, x0):
    """The padded outflow slab x > x0 of the reference's examples: phi =
    x0 - x at the cell centres, so the SDF gradient is (-1, 0, 0), pointing
    back into the fluid."""
    nx, ny, nz = sh
    x = o[0] + (np.arange(nx) + 0.5) * h[0]
    return np.broadcast_to((x0 - x).astype(np.float32), (nz, ny, nx)).ravel().copy()


def face_x(sh, h, o, a):
    nx, ny, nz = sh
    s = [(nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1)][a]
    off = 0.0 if a == 0 else 0.5
    return np.broadcast_to(o[0] + (np.arange(s[0]) + off) * h[0], s[::-1]).ravel()


def test_outflow_courant_one_is_an_upwind_copy(oracle):
    """A slab with a bulk velocity U dt / h >= 1: every face inside takes
    the value one spacing upstream (toward the fluid) as it was before the
    pass -- a component's relaxed values are written back only after the
    whole component is computed."""
    sh, h, o = SH, H, O
    x0 = 10 / 12
    phi = slab_phi(sh, h, o, x0)
    su, sv, sw = sizes(sh)
    rng = np.random.default_rng(3)
    u = (2.0 + 0.1 * rng.standard_normal(su)).astype(np.float32)   # outward everywhere
    v = rng.standard_normal(sv).astype(np.float32)
    w = rng.standard_normal(sw).astype(np.float32)
    dt = 1.0   # U dt / h >> 1: courant 1
    uo, vo, wo = oracle.outflow_velocity(sh, h, o, u, v, w, dt, [(phi, sh, h, o)])
    nx, ny, nz = sh
    U, Uo = u.reshape(nz, ny, nx + 1), uo.reshape(nz, ny, nx + 1)
    xu = face_x(sh, h, o, 0).reshape(nz, ny, nx + 1)
    inside = xu > x0 + 1e-6
    # outside the slab nothing changes
    assert np.array_equal(Uo[~inside], U[~inside])
    # inside: the u face one spacing toward the fluid (the upstream sample
    # lands on that face up to the rounding of pt - h)
    ii = np.nonzero(inside[0, 0])[0]
    np.testing.assert_allclose(Uo[:, :, ii], U[:, :, ii - 1], rtol=1e-5, atol=1e-6)


def test_outflow_inflow_faces_and_convexity(oracle):
    sh, h, o = SH, H, O
    phi = slab_phi(sh, h, o, 9 / 12)
    su, sv, sw = sizes(sh)
    rng = np.random.default_rng(4)
    v = rng.standard_normal(sv).astype(np.float32)
    w = rng.standard_normal(sw).astype(np.float32)
    # flow back in through the outflow: courant 0, the u faces keep their values
    u_in = np.full(su, -1.5, np.float32) + (0.01 * rng.standard_normal(su)).astype(np.float32)
    uo, _, _ = oracle.outflow_velocity(sh, h, o, u_in, v, w, 0.01, [(phi, sh, h, o)])
    assert np.array_equal(uo, u_in)
    # partial courant: each relaxed u face lies between its old value and the upstream one
    u = (1.0 + rng.random(su)).astype(np.float32)
    uo, _, _ = oracle.outflow_velocity(sh, h, o, u, v, w, 0.02, [(phi, sh, h, o)])
    nx, ny, nz = sh
    U, Uo = u.reshape(nz, ny, nx + 1), uo.reshape(nz, ny, nx + 1)
    changed = Uo != U
    assert changed.any()
    kk, jj, ii = np.nonzero(changed)
    lo = np.minimum(U[kk, jj, ii], U[kk, jj, ii - 1]) - 1e-5
    hi = np.maximum(U[kk, jj, ii], U[kk, jj, ii - 1]) + 1e-5
    assert np.all((Uo[kk, jj, ii] >= lo) & (Uo[kk, jj, ii] <= hi))


def test_outflow_clear_scalar_and_dirichlet(oracle):
    sh, h, o = SH, H, O
    x0 = 9 / 12
    phi = slab_phi(sh, h, o, x0)
    rng = np.random.default_rng(5)
    s = rng.random(np.prod(sh)).astype(np.float32) + 0.5
    out = oracle.outflow_clear_scalar(sh, h, o, s, [(phi, sh, h, o)])
    inside = phi < 0
    assert np.all(out[inside] == 0) and np.array_equal(out[~inside], s[~inside])
    active, target = oracle.outflow_dirichlet(sh, h, o, [(phi, sh, h, o)], target=0.25)
    assert np.array_equal(active.astype(bool), inside) and np.all(target == np.float32(0.25))
    # a second outflow on a coarser grid ORs in
    sh2, h2 = (6, 5, 4), (1 / 6, 1 / 5, 1 / 4)
    nx2, ny2, nz2 = sh2   # the low-x end: phi = x - 2/6
    phi2 = np.broadcast_to(((o[0] + (np.arange(nx2) + 0.5) * h2[0]) - 2 / 6).astype(np.float32),
                           (nz2, ny2, nx2)).ravel().copy()
    active2, _ = oracle.outflow_dirichlet(sh, h, o, [(phi, sh, h, o), (phi2, sh2, h2, o)])
    nx, ny, nz = sh
    xc = np.broadcast_to(o[0] + (np.arange(nx) + 0.5) * h[0], (nz, ny, nx)).ravel()
    assert np.array_equal(active2.astype(bool), (xc > x0) | (xc < 2 / 6))
