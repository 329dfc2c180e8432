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
