"""Seeded synthetic inputs with the shapes of the benchmark configurations.

No public dataset is involved: each scene is a MAC velocity field built from
random Fourier modes plus the boundary conditions its configuration names.
Arrays are float32, flat, i-fastest (cell (i,j,k) -> i + nx*(j + ny*k)).
"""
import numpy as np


def _mode_1d(n, offset, h, k, phase, kind):
    t = (np.arange(n, dtype=np.float64) + offset) * h
    arg = 2.0 * np.pi * k * t + phase
    return (np.sin(arg) if kind == 0 else np.cos(arg)).astype(np.float32)


def fourier_face_field(shape, h, stagger_axis, modes, amplitude, rng):
    """Sum of `modes` separable modes prod_a sin/cos(2 pi k_a t_a + phi_a),
    sampled at the face positions of `stagger_axis` (face index i sits at
    i*h on that axis and (i + 1/2)*h on the others)."""
    nx, ny, nz = shape
    dims = 3 if nz > 1 or stagger_axis == 2 else 2
    out = np.zeros((nz, ny, nx), np.float32)
    for _ in range(modes):
        a = np.float32(rng.normal(0.0, amplitude))
        k = rng.integers(1, 5, size=3)
        ph = rng.uniform(0, 2 * np.pi, size=3)
        kind = rng.integers(0, 2, size=3)
        fx = _mode_1d(nx, 0.0 if stagger_axis == 0 else 0.5, h[0], k[0], ph[0], kind[0])
        fy = _mode_1d(ny, 0.0 if stagger_axis == 1 else 0.5, h[1], k[1], ph[1], kind[1])
        if dims == 3:
            fz = _mode_1d(nz, 0.0 if stagger_axis == 2 else 0.5, h[2], k[2], ph[2], kind[2])
        else:
            fz = np.ones(nz, np.float32)
        out += a * (fz[:, None, None] * fy[None, :, None] * fx[None, None, :])
    return out


def sphere_scene(n=256, radius_cells=24, modes=32, seed=1):
    """3D mixed-precision MGPCG configuration: n^3 cells, h = 1/n, a sphere of
    radius `radius_cells` cells at the domain centre, closed walls (normal
    velocity zero on the domain boundary) and one pinned cell (0,0,0) with
    p = 0.  The velocity is `modes` random Fourier modes per component, seed
    `seed`.  Returns a dict of numpy arrays and parameters."""
    rng = np.random.default_rng(seed)
    h = (1.0 / n,) * 3
    shape = (n, n, n)
    u = fourier_face_field((n + 1, n, n), h, 0, modes, 1.0, rng)
    v = fourier_face_field((n, n + 1, n), h, 1, modes, 1.0, rng)
    w = fourier_face_field((n, n, n + 1), h, 2, modes, 1.0, rng)
    u[:, :, 0] = 0.0
    u[:, :, n] = 0.0
    v[:, 0, :] = 0.0
    v[:, n, :] = 0.0
    w[0, :, :] = 0.0
    w[n, :, :] = 0.0
    active = np.zeros(n * n * n, np.uint8)
    active[0] = 1
    return dict(shape=shape, h=h, origin=(0.0, 0.0, 0.0), u=u.ravel(), v=v.ravel(), w=w.ravel(),
                shapes=[{"type": "sphere", "center": [0.5, 0.5, 0.5], "radius": radius_cells / n}],
                active=active, target=np.zeros(n * n * n, np.float32))


def cylinder_scene_2d(n=128, radius_cells=8, center_cell=(32, 64), modes=16, seed=0):
    """2D plain MGPCG configuration: n x n MAC grid, h = 1/n; a solid
    cylinder (cell centre inside) of `radius_cells` at `center_cell`; inflow
    u = 1 on the left face; zero-pressure Dirichlet column at i = n-1;
    free-slip top and bottom (v = 0 there).  Velocity = inflow + `modes`
    Fourier modes with N(0, 0.1) amplitudes, seed `seed`.  Solid enters as
    0/1 face weights (0 on a face touching a solid cell)."""
    rng = np.random.default_rng(seed)
    h = (1.0 / n, 1.0 / n, 1.0)
    u = 1.0 + fourier_face_field((n + 1, n, 1), h, 0, modes, 0.1, rng)
    v = fourier_face_field((n, n + 1, 1), h, 1, modes, 0.1, rng)
    ci, cj = center_cell
    jj, ii = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    solid = ((ii - ci) ** 2 + (jj - cj) ** 2) < radius_cells ** 2   # (ny, nx)
    wu = np.ones((1, n, n + 1), np.float32)
    wv = np.ones((1, n + 1, n), np.float32)
    wu[0, :, 1:n] *= ~(solid[:, 1:] | solid[:, :-1])
    wu[0, :, 0] *= ~solid[:, 0]
    wu[0, :, n] *= ~solid[:, n - 1]
    wv[0, 1:n, :] *= ~(solid[1:, :] | solid[:-1, :])
    wv[0, 0, :] *= ~solid[0, :]
    wv[0, n, :] *= ~solid[n - 1, :]
    u[0, :, 0] = 1.0            # inflow
    v[0, 0, :] = 0.0            # free slip bottom / top
    v[0, n, :] = 0.0
    active = np.zeros((1, n, n), np.uint8)
    active[0, :, n - 1] = 1     # outflow column p = 0
    w = np.zeros((2, n, n), np.float32)
    return dict(shape=(n, n, 1), h=h, origin=(0.0, 0.0, 0.0), u=u.ravel(), v=v.ravel(),
                w=w.ravel(), wu=wu.ravel(), wv=wv.ravel(), solid=solid.ravel(),
                active=active.ravel(), target=np.zeros(n * n, np.float32))
