"""The C2 channel (flow past a cylinder) stepped on the CPU by the oracle,
stage for stage as GridSolver3.onAdvanceTimeStep runs it on the device
(grid_solver3.js:112-140 with the explicit viscosity stage): viscosity,
projection (FP64 MGPCG with the same multigrid options and tolerance,
warm-started from the previous pressure), constrainVelocity, copy of the
velocity, semi-Lagrangian advection of the faces through it,
constrainVelocity.  Velocities are FP32 between the stages, as on the
device.  Test infrastructure: the oracle is the checker here.

The geometry follows karman_shedding.mjs (a disc of radius 16 cells at
x = 128 cells in a 1024 x 256 channel, inflow u = 1 through a box at the
left wall, p = 0 on the last cell column, free-slip top and bottom walls,
Re 200 on the diameter, dt = h / 2)."""
import math

import numpy as np

DOWN, UP, BACK, FRONT = 4, 8, 16, 32


def geometry(nx=1024, ny=256, radius=16, cx=128):
    h = 1.0 / ny
    cy = ny // 2
    return {
        "res": (nx, ny, 1), "h": (h, h, h), "radius": radius, "cx": cx, "cy": cy, "dt": 0.5 * h,
        "nu": 1.0 * (2 * radius * h) / 200.0, "speed": 1.0, "diameter": 2 * radius * h,
        "collider": [{"type": "sphere", "center": [cx * h, cy * h, 0.5 * h], "radius": radius * h}],
        "inflow": [{"type": "box", "center": [0.0, 0.5, 0.5 * h], "halfExtents": [1.5 * h, 1.0, 1.0]}],
        "closed": DOWN | UP | BACK | FRONT,
        "probes": [cx + int(round(f * 2 * radius)) for f in (1.0, 2.0, 3.3, 5.0)],
    }


def initial_velocity(g):
    nx, ny, _ = g["res"]
    return (np.ones(ny * (nx + 1), np.float32), np.zeros(nx * (ny + 1), np.float32),
            np.zeros(2 * nx * ny, np.float32))


def dirichlet(g):
    nx, ny, _ = g["res"]
    active = np.zeros((ny, nx), np.uint8)
    active[:, nx - 1] = 1
    return active.ravel(), np.zeros(nx * ny, np.float32)


def probe_row(g, v, row_of="v"):
    """v on the faces of row cy at the probe columns."""
    nx = g["res"][0]
    return [float(v[i + nx * g["cy"]]) for i in g["probes"]]


class OracleC2:
    """The oracle's C2 step.  `phi`, `weights` and `inflow_phi` are the
    collider's cell SDF, its (u, v, w) face weights and the inflow SDF."""

    def __init__(self, O, g, phi, weights, inflow_phi, levels=5, tol=1e-6):
        self.O, self.g = O, g
        self.res, self.h = g["res"], g["h"]
        self.phi = np.asarray(phi, np.float32)
        self.fw = tuple(np.asarray(a, np.float32) for a in weights)
        self.cw = tuple(a.astype(np.float64) for a in self.fw)
        self.inflows = [(np.asarray(inflow_phi, np.float32), (g["speed"], 0.0, 0.0), 0)]
        active, target = dirichlet(g)
        self.mask, self.tgt, vent = O.dirichlet_fields(self.res, active, target, self.cw)
        self.mg = O.Multigrid(self.res, self.h, self.mask, vent, self.cw[:2] + (None,), levels=levels)
        self.tol = tol
        self.max_iter = math.ceil(1.5 * max(self.res))     # grid_pressure_solver3.js:133
        self.u, self.v, self.w = initial_velocity(g)
        self.p = np.zeros(self.res[0] * self.res[1])
        self.last = None

    def constrain(self):
        self.u, self.v, self.w = self.O.constrain_velocity(
            self.res, self.h, (0.0, 0.0, 0.0), self.u, self.v, self.w, phi=self.phi, face_weights=self.fw,
            closed=self.g["closed"], inflows=self.inflows, depth=5)

    def step(self):
        O, res, h, g = self.O, self.res, self.h, self.g
        self.u, self.v, self.w = O.viscosity(res, h, self.u, self.v, self.w, g["nu"], g["dt"])
        b, x0 = O.build_system(res, h, self.u, self.v, None, collider_weights=self.cw, mask=self.mask,
                               target=self.tgt, p=self.p)
        x, r, _ = O.pcg_solve(res, h, b, x0, self.mask, self.cw[:2] + (None,), self.mg, "multigrid",
                              tol=self.tol, max_iter=self.max_iter)
        self.p, self.last = x, r
        uo, vo, _ = O.correct(res, h, x, self.u, self.v, None, collider_weights=self.cw)
        self.u, self.v = uo.astype(np.float32), vo.astype(np.float32)
        self.constrain()
        self.u, self.v, self.w = O.advect_faces(res, h, (0.0, 0.0, 0.0), self.u, self.v, self.w, self.phi,
                                                g["dt"])
        self.constrain()
        return r
