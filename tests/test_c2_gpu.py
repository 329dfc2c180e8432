"""The C2 channel (1024 x 256, disc of radius 16 cells, Re 200, CFL 0.5;
karman_shedding.mjs) on the device against the oracle's stage-for-stage
CPU restatement of the same grid solver step, over a stated prefix of
PREFIX steps from the impulsive start: the collider and inflow bakes (to
the last FP32 bit, solid classification exact), and after every step the
velocity fields, the probe velocities on the centre line and the PCG
iteration counts.  Both projections solve to
the same 1e-6 relative residual (the device's in a double-single iterate,
the oracle's in FP64), so the fields agree to that tolerance, not bit for
bit; the step's other stages are bit-exact against the oracle on their
own (test_grid_gpu.py).  The symmetry-break step and the Strouhal number
lie beyond this prefix (step 1646 on the device); the oracle's long run of
the same channel (test_c2_oracle.py) gives the CPU's."""
import numpy as np
import pytest

import c2_mirror as M

pytestmark = pytest.mark.gpu

PREFIX = 24


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_c2_prefix_against_oracle(gpu, oracle):
    from tsl_array_n_gb300.configs import c2_channel
    solver, grid, col, inflow, geo = c2_channel()
    g = M.geometry()
    assert geo["probes"] == g["probes"] and geo["res"] == g["res"]
    phi = col.phi.to_array()
    cw = solver.collider_face_weights
    weights = tuple(cw[k].to_array() for k in "uvw")
    iphi = inflow.phi.to_array()
    ref_phi, ref_wu, ref_wv, ref_ww = oracle.collider_bake(g["collider"], g["res"], g["h"])
    np.testing.assert_allclose(phi, ref_phi, rtol=0, atol=2e-7)
    assert np.array_equal(phi < 0, ref_phi < 0)
    for got, ref in zip(weights, (ref_wu, ref_wv, ref_ww)):
        np.testing.assert_allclose(got, ref, rtol=0, atol=2e-6)
        assert np.array_equal(got == 0, ref == 0) and np.array_equal(got == 1, ref == 1)
    ref_iphi = oracle.collider_bake(g["inflow"], g["res"], g["h"])[0]
    np.testing.assert_allclose(iphi, ref_iphi, rtol=0, atol=2e-7)
    assert np.array_equal(iphi < 0, ref_iphi < 0)
    # the CPU side steps with the device's own bakes, so that the step's
    # stages are compared on the same geometry
    cpu = M.OracleC2(oracle, g, phi, weights, iphi)
    worst = {"u": 0.0, "v": 0.0, "probe_u": 0.0, "probe_v": 0.0}
    its = []
    nx, cy = g["res"][0], g["cy"]
    for step in range(PREFIX):
        d = solver.on_advance_time_step()
        r = cpu.step()
        its.append((d["iterations"], r["iterations"]))
        assert d["converged"] and r["converged"], (step, d, r)
        u, v, w = grid.get()
        assert np.all(w == 0)
        eu, ev = rel(u, cpu.u), rel(v, cpu.v)
        pu = max(abs(float(u[i + (nx + 1) * cy]) - float(cpu.u[i + (nx + 1) * cy])) for i in g["probes"])
        pv = max(abs(a - b) for a, b in zip(M.probe_row(g, v), M.probe_row(g, cpu.v)))
        worst = {"u": max(worst["u"], eu), "v": max(worst["v"], ev), "probe_u": max(worst["probe_u"], pu),
                 "probe_v": max(worst["probe_v"], pv)}
        # no symmetry break inside the prefix, on either side
        assert max(abs(x) for x in M.probe_row(g, v)) < 0.01 and max(abs(x) for x in M.probe_row(g, cpu.v)) < 0.01
    print(f"C2 prefix of {PREFIX} steps, device vs CPU oracle: {worst}; iterations (device, oracle) {its}")
    # measured: u 5.7e-7, v 1.1e-5 (v is small beside u, so its relative
    # error is larger), probe u 6e-8, probe v 4e-8
    assert worst["u"] < 1e-5 and worst["v"] < 1e-4, worst
    assert worst["probe_u"] < 1e-6 and worst["probe_v"] < 1e-6, worst
    # iteration counts: the same median (48 on both sides, 24 steps); single
    # steps differ where one side meets a stall of about 30 iterations that
    # the other does not: both sides show such stalls, at different steps
    dev, orc = np.array([a for a, _ in its]), np.array([b for _, b in its])
    assert abs(np.median(dev) - np.median(orc)) <= 2, its
    assert abs(int(dev.sum()) - int(orc.sum())) <= 0.15 * orc.sum(), its
