"""The learned warm start inside the pressure solve: the network's guess
replaces the previous pressure only when it lowers the initial residual,
and MGPCG still iterates to the same tolerance from whichever start won."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def solver_and_grid():
    from tsl_array_n_gb300 import fluxflow as ff, scenes
    n = 32
    sc = scenes.sphere_scene(n=n, radius_cells=5, modes=8, seed=3)
    shape, h = sc["shape"], sc["h"]
    col = ff.create_sdf_static_collider3(*shape, *h)
    col.add_shapes(sc["shapes"])
    s = ff.create_grid_pressure_solver3(shape, h, collider_weights=col.compute_face_weights(),
                                        dirichlet=(sc["active"], sc["target"]),
                                        multigrid={"numberOfLevels": 3, "coarseSolve": "direct"},
                                        precision="mixed", tolerance=1e-6)
    g = ff.FaceCenteredGrid3(shape, h).set(sc["u"], sc["v"], sc["w"])
    return s, g, ff.FaceCenteredGrid3(shape, h), n


def test_guess_is_used_only_when_it_lowers_the_residual(gpu):
    from tsl_array_n_gb300.warmstart import UNetWarmStart, attach
    s, g, out, n = solver_and_grid()
    s.pressure.fill(0.0)
    d0 = s.project(g, out)()
    assert d0["converged"]
    p = s.pressure.to_array()
    # a smooth previous pressure a thousand times off (e.g. after a scene
    # change): its error needs about three more V-cycles to remove
    bad = (-1000.0 * p).astype(np.float32)
    # without the network: start from the bad previous pressure
    s.pressure.from_array(bad)
    d1 = s.project(g, out)()
    assert d1["converged"] and d1["warmStart"] == -1
    # an untrained network scales its guess by the bad pressure; one V-cycle
    # corrects it before the residual test, and whichever start has the
    # smaller residual is taken: the solve converges to the same tolerance
    # in no more iterations either way
    net = UNetWarmStart(seed=2)
    attach(s, net)
    s.pressure.from_array(bad)
    d2 = s.project(g, out)()
    assert d2["converged"] and d2["warmStart"] in (0, 1)
    assert d2["iterations"] <= d1["iterations"]
    # a network fitted to this scene (the repo's own forward, backward and
    # Adam kernels) gives a guess with the smaller residual: used, and the
    # solve from it converges with no more iterations (MGPCG removes a
    # smooth start error this size within the same 8 iterations, so the
    # count is not a sensitive measure here)
    from tsl_array_n_gb300.tsl_array_n import Field
    shape = (n, n, n)
    fb = Field("float", shape).from_array(s.b.to_array())
    fbad = Field("float", shape).from_array(bad)
    ftarget = Field("float", shape).from_array(p)
    first = last = None
    for _ in range(150):
        last = net.train_step(shape, 1.0 / n, fb, s.dirichlet_mask, fbad, ftarget, lr=2e-3)
        first = first if first is not None else last
    assert last < 0.1 * first
    s.pressure.from_array(bad)
    d3 = s.project(g, out)()
    assert d3["converged"] and d3["warmStart"] == 1
    assert d3["iterations"] <= d1["iterations"]


def test_good_previous_pressure_is_kept(gpu):
    from tsl_array_n_gb300.warmstart import UNetWarmStart, attach
    s, g, out, n = solver_and_grid()
    s.pressure.fill(0.0)
    d0 = s.project(g, out)()
    attach(s, UNetWarmStart(seed=2))
    d1 = s.project(g, out)()          # previous pressure is the converged one
    assert d1["converged"] and d1["warmStart"] == 0
    assert d1["iterations"] <= 2
