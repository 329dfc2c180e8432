"""FLIP seeding and oracle checks that need no GPU: mulberry32 and
computeFlipBoxSeed3 agree between libff's host code, the C oracle and a
third restatement written here from jitter_random.js's JavaScript
semantics; FLIP stage properties of the oracle."""
import ctypes as C

import numpy as np
import pytest


def mulberry32_py(seed, n):
    """jitter_random.js:29-41 with JavaScript's uint32 semantics."""
    m = 0xFFFFFFFF
    state = seed & m
    out = []
    for _ in range(n):
        state = (state + 0x6D2B79F5) & m
        t = state
        t = ((t ^ (t >> 15)) * (t | 1)) & m          # Math.imul, then >>> 0
        t ^= (t + (((t ^ (t >> 7)) * (t | 61)) & m)) & m
        out.append(((t ^ (t >> 14)) & m) / 4294967296.0)
    return np.array(out)


@pytest.mark.parametrize("seed", [0x9E3779B9, 0, 1, 12345, 0xFFFFFFFF])
def test_mulberry32_three_ways(oracle, seed):
    from tsl_array_n_gb300 import _lib
    ref = mulberry32_py(seed, 257)
    assert np.array_equal(oracle.jitter_random(seed, 257), ref)
    out = (C.c_double * 257)()
    _lib.check(_lib.load().ff_jitter_random(seed, 257, out))
    assert np.array_equal(np.array(out), ref)
    assert np.all((ref >= 0) & (ref < 1))


def test_box_seed_matches_oracle_and_layout(oracle):
    from tsl_array_n_gb300 import fluxflow as ff
    h = (1 / 32, 1 / 16, 1 / 24)
    box_min, box_max = (0.1, 0.05, 0.2), (0.45, 0.6, 0.55)
    got = ff.compute_flip_box_seed3(box_min, box_max, *h, particles_per_cell_axis=2, jitter=0.2)
    ref = oracle.flip_box_seed(box_min, box_max, h, 2, 0.2, 0x9E3779B9)
    assert got["count"] * 3 == ref.size
    assert np.array_equal(got["positionsArray"], ref)
    # every particle stays within its own sub-cell (jitter 0.2 < 0.5)
    cells = [max(1, int(np.floor((b - a) / hh + 0.5))) for a, b, hh in zip(box_min, box_max, h)]
    assert got["count"] == cells[0] * cells[1] * cells[2] * 8
    p = ref.reshape(-1, 3)
    for a in range(3):
        assert np.all(p[:, a] > box_min[a]) and np.all(p[:, a] < box_min[a] + cells[a] * h[a])


def test_p2g_partition_of_unity_and_order_independence(oracle):
    """Trilinear weights sum to one, so a uniform particle velocity maps to
    the same value on every face with weight; the int32 fixed point makes
    the sum independent of particle order."""
    sh, h, o = (10, 8, 6), (0.1, 0.125, 1 / 6), (0.0, 0.0, 0.0)
    pos = oracle.flip_box_seed((0.2, 0.2, 0.2), (0.7, 0.8, 0.8), h, 2, 0.2).reshape(-1, 3)
    vel = np.tile(np.array([[0.5, -1.25, 2.0]], np.float32), (len(pos), 1))
    (u, v, w), (vu, vv, vw) = oracle.flip_p2g(sh, h, o, pos, vel)
    # each term is rounded to 1/S (S = 65536), so faces whose weight comes
    # from a few small trilinear weights carry a larger relative error
    for x, valid, want in ((u, vu, 0.5), (v, vv, -1.25), (w, vw, 2.0)):
        err = np.abs(x[valid == 1] - want) / abs(want)
        assert np.median(err) < 1e-4 and np.mean(err < 2e-3) > 0.95
    rng = np.random.default_rng(0)
    vel2 = rng.standard_normal(pos.shape).astype(np.float32)
    a = oracle.flip_p2g(sh, h, o, pos, vel2)
    perm = rng.permutation(len(pos))
    b = oracle.flip_p2g(sh, h, o, pos[perm], vel2[perm])
    for x, y in zip(a[0] + a[1], b[0] + b[1]):
        assert np.array_equal(x, y)


def test_mark_fluid_dirichlet_and_adjacency(oracle):
    sh, h, o = (8, 8, 8), (0.125,) * 3, (0.0, 0.0, 0.0)
    pos = np.array([[0.3, 0.3, 0.3], [0.9, 0.2, 0.1], [-5.0, 2.0, 0.5]], np.float32)
    idx = oracle.flip_cell_index(sh, h, o, pos)
    assert list(idx) == [2 + 8 * (2 + 8 * 2), 7 + 8 * (1 + 8 * 0), 0 + 8 * (7 + 8 * 4)]
    mask = oracle.flip_mark_fluid(sh, h, o, pos)
    assert mask.sum() == 3 and all(mask[idx] == 1)
    active, target = oracle.flip_dirichlet(sh, h, o, mask, (0.0, -9.81, 0.0), 0.01)
    assert np.array_equal(active, (mask < 0.5).astype(np.uint8))
    # reduced pressure target -dt g.y y at the cell centre
    assert np.isclose(target[idx[0]], 0.01 * 9.81 * 0.3125, rtol=1e-6)
    au, av, aw = oracle.flip_fluid_adjacent(sh, mask)
    U = au.reshape(8, 8, 9)
    assert U[2, 2, 2] == 1 and U[2, 2, 3] == 1 and U[2, 2, 4] == 0


def test_g2p_pic_limit_and_clamp(oracle):
    """flipRatio 0 is PIC: the particle takes the sampled new grid velocity
    (damped); a non-finite result zeroes the particle."""
    sh, h, o = (6, 6, 6), (1 / 6,) * 3, (0.0, 0.0, 0.0)
    su, sv, sw = 7 * 36, 6 * 7 * 6, 36 * 7
    new = [np.full(su, 2.0, np.float32), np.full(sv, -1.0, np.float32), np.zeros(sw, np.float32)]
    old = [np.zeros(su, np.float32), np.zeros(sv, np.float32), np.zeros(sw, np.float32)]
    pos = np.array([[0.5, 0.5, 0.5], [0.2, 0.7, 0.3]], np.float32)
    vel = np.array([[9.0, 9.0, 9.0], [np.nan, 0.0, 0.0]], np.float32)
    out = oracle.flip_g2p(sh, h, o, pos, vel, new, old, flip_ratio=0.0, damping=0.5).reshape(-1, 3)
    np.testing.assert_allclose(out[0], [1.0, -0.5, 0.0], rtol=1e-6)
    assert np.all(out[1] == 0)


def test_concentration_density_and_beta(oracle):
    sh, h, o = (6, 5, 4), (1 / 6, 0.2, 0.25), (0.0, 0.0, 0.0)
    pos = oracle.flip_box_seed((0.0, 0.0, 0.0), (0.5, 0.6, 0.5), h, 2, 0.2).reshape(-1, 3)
    conc = (pos[:, 0] > 0.25).astype(np.float32)
    mask = oracle.flip_mark_fluid(sh, h, o, pos)
    cc, rho, beta = oracle.flip_concentration_grid(sh, h, o, pos, conc, mask, density=(1.0, 1000.0))
    assert np.all((cc >= 0) & (cc <= 1))
    assert np.all((rho >= 1.0) & (rho <= 1000.0))
    # beta = rho_ref / rho_face: 1 in the heavy phase, 1000 in the light one
    assert np.isclose(beta[0].max(), 1000.0) and np.isclose(beta[0].min(), 1.0)


def resample_numpy(oracle, sh, h, o, pos, vel, u, v, w, min_pc, max_pc):
    """resamplePass (grid_flip_solver3.js:621-820) a second way, vectorised:
    donors ranked by particle index, needs scanned in flat cell order,
    velocities through the oracle's G2P in its PIC limit (ratio 0, no
    damping: the interpolated grid velocity itself)."""
    nx, ny, nz = sh
    pos = np.asarray(pos, np.float32).reshape(-1, 3).copy()
    vel = np.asarray(vel, np.float32).reshape(-1, 3).copy()
    cell = oracle.flip_cell_index(sh, h, o, pos)
    cnt = np.bincount(cell, minlength=nx * ny * nz).reshape(nz, ny, nx)
    donors = np.nonzero(cnt.ravel()[cell] > max_pc)[0]
    ok = (cnt >= min_pc).astype(np.int64)
    nb = np.zeros_like(ok)
    for ax in range(3):
        lo = np.concatenate([np.take(ok, [0], axis=ax), np.take(ok, np.arange(ok.shape[ax] - 1), axis=ax)], axis=ax)
        hi = np.concatenate([np.take(ok, np.arange(1, ok.shape[ax]), axis=ax), np.take(ok, [-1], axis=ax)], axis=ax)
        nb += lo + hi
    need = np.where((cnt < min_pc) & (nb >= 3), min_pc - cnt, 0).ravel()
    cells = np.repeat(np.arange(need.size), need)[:donors.size]
    movers = donors[:cells.size]
    i, j, k = cells % nx, (cells // nx) % ny, cells // (nx * ny)
    f32 = np.float32
    for a, idx in enumerate((i, j, k)):
        cc = f32(o[a]) + f32(h[a]) * f32(0.5)
        pos[movers, a] = cc + idx.astype(f32) * f32(h[a])
    if movers.size:
        z = np.zeros((movers.size, 3), np.float32)
        vel[movers] = oracle.flip_g2p(sh, h, o, pos[movers], z, (u, v, w), (u, v, w), 0.0, 0.0).reshape(-1, 3)
    return pos.ravel(), vel.ravel(), int(movers.size), int(donors.size), int(need.sum())


def random_fluid(sh, h, n, seed, frac=(0.6, 0.5, 0.7)):
    rng = np.random.default_rng(seed)
    hi = np.array([sh[a] * h[a] * frac[a] for a in range(3)])
    return (rng.random((n, 3)) * hi).astype(np.float32)


@pytest.mark.parametrize("min_pc,max_pc", [(4, 8), (3, 5), (6, 7)])
def test_resample_matches_vectorised_restatement(oracle, min_pc, max_pc):
    sh, h, o = (12, 10, 9), (1 / 12, 0.1, 1 / 9), (0.0, -0.5, 0.25)
    n = 5 * int(12 * 0.6 * 10 * 0.5 * 9 * 0.7)
    pos = random_fluid(sh, h, n, 7)
    pos[:, 1] += -0.5
    pos[:, 2] += 0.25
    rng = np.random.default_rng(8)
    vel = rng.standard_normal((n, 3)).astype(np.float32)
    su, sv, sw = (13, 10, 9), (12, 11, 9), (12, 10, 10)
    u, v, w = (rng.standard_normal(np.prod(s)).astype(np.float32) for s in (su, sv, sw))
    p1, v1, moved = oracle.flip_resample(sh, h, o, pos, vel, u, v, w, min_pc, max_pc)
    p2, v2, moved2, donors, need = resample_numpy(oracle, sh, h, o, pos, vel, u, v, w, min_pc, max_pc)
    assert moved > 0 and moved == moved2 == min(donors, need)
    assert np.array_equal(p1, p2) and np.array_equal(v1, v2)
    changed = np.any(p1.reshape(-1, 3) != pos, axis=1)
    assert changed.sum() <= moved


def test_resample_no_donors_or_no_need(oracle):
    sh, h, o = (6, 6, 6), (1 / 6,) * 3, (0.0, 0.0, 0.0)
    u, v, w = (np.zeros(s, np.float32) for s in (7 * 36, 7 * 36, 7 * 36))
    # eight particles in every cell: nothing above max, nothing below min
    seed = oracle.flip_box_seed((0, 0, 0), (1, 1, 1), (1 / 6,) * 3, 2, 0.2, 0x9E3779B9)
    vel = np.ones(seed.size, np.float32)
    p, vv, moved = oracle.flip_resample(sh, h, o, seed, vel, u, v, w)
    assert moved == 0 and np.array_equal(p, seed) and np.array_equal(vv, vel)
    # an empty particle set
    p, vv, moved = oracle.flip_resample(sh, h, o, np.zeros(0, np.float32), np.zeros(0, np.float32), u, v, w)
    assert moved == 0 and p.size == 0


# ---- 2D two-phase (grid_two_phase_flip_solver2.js) -------------------------
def test_two_phase_box_seed():
    from tsl_array_n_gb300 import fluxflow as ff
    seed = ff.compute_two_phase_box_seed((0.0, 0.0), (1.0, 0.5), 0.125, 0.125, is_liquid=lambda p: p[1] < 0.25)
    assert seed["count"] == 8 * 4 * 4
    pos = seed["positionsArray"].reshape(-1, 2)
    assert np.array_equal(seed["phasesArray"] > 0.5, pos[:, 1] < 0.25)
    assert seed["liquidCount"] + seed["gasCount"] == seed["count"]
    # the first particle from mulberry32's first two values (jitter_random.js)
    r = mulberry32_py(0x9E3779B9, 2)
    sub = 0.125 / 2
    x = 0.0 + 0 * 0.125 + 0.5 * sub + (r[0] * 2 - 1) * 0.2 * sub
    y = 0.0 + 0 * 0.125 + 0.5 * sub + (r[1] * 2 - 1) * 0.2 * sub
    assert pos[0, 0] == np.float32(x) and pos[0, 1] == np.float32(y)
    c = ff.compute_two_phase_box_seed((0.0, 0.0), (0.5, 0.5), 0.25, 0.25, concentration_at=lambda p: 3 * p[0] - 0.5)
    assert c["phasesArray"].min() >= 0 and c["phasesArray"].max() <= 1 and 0 < c["meanConcentration"] < 1


def test_two_phase_density_and_beta(oracle):
    sh, h, o = (10, 8), (0.1, 0.125), (0.0, 0.0)
    rng = np.random.default_rng(1)
    n = 400
    pos = (rng.random((n, 2)) * [1.0, 1.0]).astype(np.float32)
    phase = (pos[:, 1] < 0.5).astype(np.float32)
    cnt, acc, frac, rho, bu, bv = oracle.tp_density(sh, h, o, pos, phase, 0.01, 1.0)
    assert cnt.sum() == n and np.all((frac >= 0) & (frac <= 1))
    empty = cnt == 0
    assert np.all(frac[empty] == 0)
    np.testing.assert_allclose(rho, 0.01 + (1.0 - 0.01) * frac, rtol=1e-6)
    R = rho.reshape(8, 10)
    BU = bu.reshape(8, 11)
    np.testing.assert_allclose(BU[:, 1:-1], 1.0 / ((R[:, :-1] + R[:, 1:]) * 0.5), rtol=1e-6)
    np.testing.assert_allclose(BU[:, 0], 1.0 / R[:, 0], rtol=1e-6)
    # the reference density is the heavier component: beta >= 1 everywhere,
    # and exactly 1 between two all-liquid cells
    c1, _, _, _, bu1, bv1 = oracle.tp_density(sh, h, o, pos, np.ones(n, np.float32), 0.01, 1.0)
    assert np.all(bu1 >= 1.0) and np.all(bv1 >= 1.0)
    occ = c1.reshape(8, 10) > 0
    assert np.all(bu1.reshape(8, 11)[:, 1:-1][occ[:, :-1] & occ[:, 1:]] == 1.0)


def tp_resample_numpy(sh, h, o, pos, vel, phase, u, v, cnt, acc, max_particles, min_pc, max_pc, cscale=4096.0):
    """The per-phase resampling a second way, vectorised."""
    nx, ny = sh
    f32 = np.float32
    pos = pos.reshape(-1, 2).copy()
    vel = vel.reshape(-1, 2).copy()
    C = cnt.reshape(ny, nx).astype(np.int64)
    A = acc.reshape(ny, nx).astype(np.int64)
    pad = lambda X: (np.concatenate([X[:, :1], X[:, :-1]], 1), np.concatenate([X[:, 1:], X[:, -1:]], 1),
                     np.concatenate([X[:1], X[:-1]], 0), np.concatenate([X[1:], X[-1:]], 0))
    nb = sum((q >= min_pc).astype(int) for q in pad(C))
    ntot = sum(pad(C)).astype(f32)
    nsum = sum(pad(A)).astype(f32) / f32(cscale)
    own = (A.astype(f32) / f32(cscale)) / np.maximum(C.astype(f32), f32(1))
    around = nsum / np.maximum(ntot, f32(1))
    liquid = np.where(C > 0, own > 0.5, around > 0.5)
    needed = min_pc - C
    need = np.where((C < min_pc) & (nb >= 2), np.where(liquid, needed, -needed), 0).ravel()
    cell = np.clip(np.floor((pos - np.array(o, f32)) / np.array(h, f32)).astype(int), 0, [nx - 1, ny - 1])
    over = cnt[cell[:, 0] + nx * cell[:, 1]] > max_pc
    half, top = max(1, max_particles // 2), max_particles - 1
    lq = np.nonzero(over & (phase > 0.5))[0]
    gs = np.nonzero(over & ~(phase > 0.5))[0]
    moved = 0
    for sign, donors in ((1, lq), (-1, gs)):
        want = np.where(sign * need > 0, sign * need, 0)
        cells = np.repeat(np.arange(need.size), want)[:min(donors.size, half)]
        movers = donors[:cells.size]
        i, j = cells % nx, cells // nx
        pos[movers, 0] = (f32(o[0]) + f32(h[0]) * f32(0.5)) + i.astype(f32) * f32(h[0])
        pos[movers, 1] = (f32(o[1]) + f32(h[1]) * f32(0.5)) + j.astype(f32) * f32(h[1])
        moved += movers.size
    return pos.ravel(), moved


@pytest.mark.parametrize("mm", [(3, 8), (4, 6)])
def test_two_phase_resample_matches_vectorised_restatement(oracle, mm):
    sh, h, o = (16, 12), (1 / 16, 1 / 12), (0.0, 0.0)
    rng = np.random.default_rng(6)
    n = 5 * 16 * 12
    pos = (rng.random((n, 2)) ** 1.7).astype(np.float32)   # crowded near the origin, sparse far from it
    vel = rng.standard_normal((n, 2)).astype(np.float32)
    phase = (rng.random(n) < 0.6).astype(np.float32)
    u = rng.standard_normal(17 * 12).astype(np.float32)
    v = rng.standard_normal(16 * 13).astype(np.float32)
    cnt, acc, *_ = oracle.tp_density(sh, h, o, pos, phase, 0.01, 1.0)
    p1, v1, moved, stats = oracle.tp_resample(sh, h, o, pos, vel, phase, u, v, cnt, acc, n, *mm)
    p2, moved2 = tp_resample_numpy(sh, h, o, pos, vel, phase, u, v, cnt, acc, n, *mm)
    assert moved > 0 and moved == moved2
    assert np.array_equal(p1, p2)
    assert stats[1] > 0 and stats[3] > 0   # both phases asked for particles


def test_tp3_oracle_on_one_cell_thick_grid_equals_2d(oracle):
    """The 3D two-phase oracle's counts and per-phase G2P on a grid one cell
    thick, with particles on the centre plane and a zero w, equal the 2D
    two-phase oracle's bit for bit (trilinear at fz = 0 is bilinear)."""
    rng = np.random.default_rng(4)
    nx, ny, h = 12, 9, 0.125
    n = 500
    xy = np.stack([rng.uniform(0, nx * h, n), rng.uniform(0, ny * h, n)], 1).astype(np.float32)
    xyz = np.concatenate([xy, np.full((n, 1), 0.5 * h, np.float32)], 1)
    ph = rng.uniform(0, 1, n).astype(np.float32)
    cnt2, acc2, *_ = oracle.tp_density((nx, ny), (h, h), (0, 0), xy.ravel(), ph, 0.01, 1.0)
    cnt3, acc3 = oracle.tp3_counts((nx, ny, 1), (h, h, h), (0, 0, 0), xyz.ravel(), ph)
    assert np.array_equal(cnt2, cnt3) and np.array_equal(acc2, acc3)
    new2 = [rng.standard_normal((nx + 1) * ny).astype(np.float32), rng.standard_normal(nx * (ny + 1)).astype(np.float32)]
    old2 = [rng.standard_normal((nx + 1) * ny).astype(np.float32), rng.standard_normal(nx * (ny + 1)).astype(np.float32)]
    vel2 = rng.standard_normal(2 * n).astype(np.float32)
    g2 = oracle.tp_g2p((nx, ny), (h, h), (0, 0), xy.ravel(), vel2, ph, new2, old2, 0.95, 0.9, 0.02)
    z = np.zeros(nx * ny * 2, np.float32)
    vel3 = np.concatenate([vel2.reshape(-1, 2), np.zeros((n, 1), np.float32)], 1).ravel()
    g3 = oracle.tp3_g2p((nx, ny, 1), (h, h, h), (0, 0, 0), xyz.ravel(), vel3, ph, new2 + [z], old2 + [z], 0.95,
                        0.9, 0.02)
    assert np.array_equal(g3.reshape(-1, 3)[:, :2].ravel(), g2)
