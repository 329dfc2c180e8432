"""Host-side mirror of fluxflow's grid/ API for the GB300 path.

Names, option names, defaults and error behaviour follow the reference
(packages/fluxflow/src/grid/*.js); the work runs in libff (include/ff.h).

  create_face_centered_grid3      grid_data3.js:121-176
  create_cell_centered_grid3      grid_data3.js:205-216
  create_sdf_static_collider3     sdf_collider3.js:25-264 (addShapes, computeFaceWeights)
  create_grid_pressure_solver3    grid_pressure_solver3.js:66-574
  create_grid_pressure_solver2    grid_pressure_solver2.js:223-981 (nz == 1)
  create_semi_lagrangian_advection_solver3  advection_solver3.js:67-364
  create_sdf_inflow3              sdf_inflow_outflow3.js:15-22
  create_grid_blocked_boundary_condition_solver3
                                  grid_blocked_boundary_condition_solver3.js:48-490
  apply_viscosity3                explicit viscosity (no reference counterpart)
  create_grid_solver3             grid_solver3.js:24-149 (forces, viscosity, projection, advection)
  create_grid_flip_solver3        grid_flip_solver3.js:135-1157 (resampling on by default, :621-820)
  create_grid_two_phase_flip_solver2  grid_two_phase_flip_solver2.js:479-1622 (one-cell-thick grid)
  create_grid_two_phase_flip_solver3  the same stages on a full 3D grid (no reference counterpart)
  compute_flip_box_seed3          grid_flip_solver3.js:70-130
  create_jitter_random            jitter_random.js:29-46
"""
import ctypes as C
import math

import numpy as np

from . import _lib
from .tsl_array_n import BorrowedField, Field, context

PRECONDITIONERS = {"multigrid": 0, "jacobi": 1, "none": 2}
STOP_REASONS = {0: "none", 1: "degenerate-pAp", 2: "pAp-growth", 3: "alpha-magnitude",
                4: "degenerate-oldRZ", 5: "converged", 6: "residual-growing"}


class FaceCenteredGrid3:
    """createFaceCenteredGrid3 (grid_data3.js:121-176): u (nx+1,ny,nz),
    v (nx,ny+1,nz), w (nx,ny,nz+1), staggered origins."""

    def __init__(self, resolution, grid_spacing=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0)):
        nx, ny, nz = resolution
        self.resolution = (nx, ny, nz)
        self.grid_spacing = tuple(float(h) for h in grid_spacing)
        self.origin = tuple(float(o) for o in origin)
        self.data_size_u = (nx + 1, ny, nz)
        self.data_size_v = (nx, ny + 1, nz)
        self.data_size_w = (nx, ny, nz + 1)
        self.data_u = Field("float", self.data_size_u)
        self.data_v = Field("float", self.data_size_v)
        self.data_w = Field("float", self.data_size_w)
        hx, hy, hz = self.grid_spacing
        ox, oy, oz = self.origin
        self.data_origin_u = (ox, oy + 0.5 * hy, oz + 0.5 * hz)
        self.data_origin_v = (ox + 0.5 * hx, oy, oz + 0.5 * hz)
        self.data_origin_w = (ox + 0.5 * hx, oy + 0.5 * hy, oz)

    def set(self, u, v, w):
        self.data_u.from_array(u)
        self.data_v.from_array(v)
        self.data_w.from_array(w)
        return self

    def get(self):
        return self.data_u.to_array(), self.data_v.to_array(), self.data_w.to_array()


def create_face_centered_grid3(nx, ny, nz, hx=1.0, hy=1.0, hz=1.0, ox=0.0, oy=0.0, oz=0.0):
    return FaceCenteredGrid3((nx, ny, nz), (hx, hy, hz), (ox, oy, oz))


def cell_positions(resolution, grid_spacing, origin):
    """dataPosition of a cell-centred grid (origin + h/2), as numpy arrays in
    i-fastest order (grid_data3.js:205-216)."""
    nx, ny, nz = resolution
    hx, hy, hz = grid_spacing
    ox, oy, oz = origin
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return (ox + (i + 0.5) * hx).ravel(), (oy + (j + 0.5) * hy).ravel(), (oz + (k + 0.5) * hz).ravel()


class SDFStaticCollider3:
    """createSDFStaticCollider3 (sdf_collider3.js:25-264): the cell-centred SDF
    (solid where phi < 0, isInside :49-53) and fractional face weights."""

    FRICTION = 0.5   # sdf_collider3.js:16

    def __init__(self, resolution, grid_spacing, origin=(0.0, 0.0, 0.0)):
        self.resolution = tuple(resolution)
        self.grid_spacing = tuple(float(h) for h in grid_spacing)
        self.origin = tuple(float(o) for o in origin)
        self.phi = Field("float", self.resolution)
        self.shapes = []
        self.invert = False

    @staticmethod
    def _shape(s):
        sh = _lib.Shape()
        if s["type"] == "sphere":
            sh.type = 0
            sh.radius = float(s["radius"])
        elif s["type"] == "box":
            sh.type = 1
            sh.half_extents[:] = [float(v) for v in s["halfExtents"]]
            rot = s.get("rotation")
            if rot:
                sh.has_rotation = 1
                sh.rotation_axis[:] = [float(v) for v in rot["axis"]]
                sh.rotation_angle = float(rot["angle"])
        else:
            raise ValueError(f"primitive_sdf3: unknown shape type '{s['type']}'.")
        sh.center[:] = [float(v) for v in s["center"]]
        return sh

    def _bake(self, phi, wu, wv, ww, resolution, spacing, origin):
        arr = (_lib.Shape * max(1, len(self.shapes)))(*[self._shape(s) for s in self.shapes])
        res = (C.c_int * 3)(*resolution)
        h = (C.c_double * 3)(*spacing)
        o = (C.c_double * 3)(*origin)
        hnd = lambda f: f.handle if f is not None else None
        _lib.check(_lib.load().ff_collider3_bake(context().handle, arr, len(self.shapes), int(self.invert),
                                                 res, h, o, hnd(phi), hnd(wu), hnd(wv), hnd(ww)))

    def add_shapes(self, shapes, invert=False):
        """addShapes (sdf_collider3.js:69-99)."""
        self.shapes = list(shapes)
        self.invert = bool(invert)
        self._bake(self.phi, None, None, None, self.resolution, self.grid_spacing, self.origin)

    def add_shape(self, shape, invert=False):
        self.add_shapes([shape], invert=invert)

    def compute_face_weights(self, resolution=None, grid_spacing=None, origin=None):
        """computeFaceWeights (sdf_collider3.js:131-254): {u, v, w} fields."""
        resolution = tuple(resolution or self.resolution)
        grid_spacing = tuple(grid_spacing or self.grid_spacing)
        origin = tuple(origin or self.origin)
        nx, ny, nz = resolution
        w = {"u": Field("float", (nx + 1, ny, nz)), "v": Field("float", (nx, ny + 1, nz)),
             "w": Field("float", (nx, ny, nz + 1))}
        self._bake(None, w["u"], w["v"], w["w"], resolution, grid_spacing, origin)
        return w


def create_sdf_static_collider3(nx, ny, nz, hx, hy, hz, ox=0.0, oy=0.0, oz=0.0):
    return SDFStaticCollider3((nx, ny, nz), (hx, hy, hz), (ox, oy, oz))


class GridPressureSolver3:
    """createGridPressureSolver3 (grid_pressure_solver3.js:66-574).

    ``dirichlet`` is either a callable ``f(x, y, z) -> (active, target)`` on
    numpy arrays of cell-centre positions (the reference's ``dirichlet(pos)``
    closure, evaluated once per call of ``update_dirichlet``) or a tuple of
    arrays ``(active, target)``.  ``face_weights`` / ``collider_weights`` are
    dicts {u, v, w} of face Fields.  ``multigrid`` takes the reference's
    option names (multigrid.js:1186-1250) plus ``coarseSolve`` ('sweeps' or
    'direct').  ``precision`` is 'fp32' (the reference's arithmetic) or
    'mixed' (BF16 V-cycle storage, double-single CG iterate, FP64 scalars).
    """

    def __init__(self, resolution, grid_spacing, origin=(0.0, 0.0, 0.0), dirichlet=None,
                 face_weights=None, collider_weights=None, multigrid=None, preconditioner="multigrid",
                 tolerance=1e-6, max_iterations=None, max_iterations_factor=1.5,
                 relative_tolerance=True, max_plausible_pressure=1e6, precision="fp32",
                 vcycle_storage=None, iterate=None, **ignored):
        if preconditioner not in PRECONDITIONERS:
            raise ValueError(f"grid_pressure_solver3: unknown preconditioner '{preconditioner}' "
                             f"(expected {', '.join(PRECONDITIONERS)}).")
        resolution = tuple(int(n) for n in resolution)
        if len(resolution) == 2:
            resolution = resolution + (1,)
        grid_spacing = tuple(float(h) for h in grid_spacing)
        if len(grid_spacing) == 2:
            grid_spacing = grid_spacing + (1.0,)
        origin = tuple(float(o) for o in origin) + (0.0,) * (3 - len(origin))
        self.resolution, self.grid_spacing, self.origin = resolution, grid_spacing, origin
        mg = dict(multigrid or {})
        lib = _lib.load()
        d = _lib.PressureDesc()
        lib.ff_pressure_desc_default(C.byref(d), (C.c_int * 3)(*resolution),
                                     (C.c_double * 3)(*grid_spacing))
        d.origin[:] = origin
        d.preconditioner = PRECONDITIONERS[preconditioner]
        d.tolerance = tolerance
        self._tol = float(tolerance)
        d.max_iterations = int(max_iterations or 0)
        d.max_iterations_factor = max_iterations_factor
        d.relative_tolerance = int(bool(relative_tolerance))
        d.max_plausible_pressure = max_plausible_pressure
        d.mg_levels = int(mg.get("numberOfLevels", 1))
        d.mg_down = int(mg.get("numberOfSmoothingIterationsDown", 2))
        d.mg_up = int(mg.get("numberOfSmoothingIterationsUp", 2))
        d.mg_coarsest = int(mg.get("numberOfCoarsestIterations", 20))
        d.mg_final = int(mg.get("numberOfFinalIterations", 2))
        d.mg_sor = float(mg.get("sorFactor", 1.0))
        d.mg_coarsen_mask = int(mg.get("coarsenDirichletMask", True))
        d.mg_coarsen_weights = int(mg.get("coarsenFaceWeights", True))
        d.mg_coarse_mode = 1 if mg.get("coarseSolve", "sweeps") == "direct" else 0
        # 'fp32': the reference's arithmetic (FP32 iterate); 'mixed': FP32
        # V-cycle on the fused kernels, double-single CG iterate, FP64
        # scalars; 'mixed-bf16': as 'mixed' with BF16 V-cycle storage on the
        # coarse levels and residual buffers (measured: about twice the
        # iterations, kept for that comparison)
        if precision not in ("fp32", "mixed", "mixed-bf16"):
            raise ValueError(f"unknown precision '{precision}'")
        vs = vcycle_storage or ("bf16" if precision == "mixed-bf16" else "fp32")
        it = iterate or ("ds" if precision.startswith("mixed") else "fp32")
        d.vcycle_storage = 1 if vs == "bf16" else 0
        d.iterate = 1 if it == "ds" else 0
        self.desc = d
        h = C.c_void_p()
        _lib.check(lib.ff_pressure3_create(context().handle, C.byref(d), C.byref(h)))
        self.handle = h
        self._bind(dirichlet)
        if face_weights is not None:
            self.set_face_weights(face_weights)
        if collider_weights is not None:
            self.set_collider_weights(collider_weights)
        if dirichlet is not None:
            self.update_dirichlet()

    def _bind(self, dirichlet):
        p, b, m, v = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        _lib.check(_lib.load().ff_pressure3_fields(self.handle, C.byref(p), C.byref(b), C.byref(m), C.byref(v)))
        ctx = context()
        self.pressure = BorrowedField(p, ctx)
        self.b = BorrowedField(b, ctx)
        self.dirichlet_mask = BorrowedField(m, ctx)
        self.vent_mask = BorrowedField(v, ctx)
        self.diagnostics = {"converged": None, "rejected": False, "iterations": None,
                            "stoppedBy": None}
        self._keep = {}
        self._dirichlet = dirichlet

    @classmethod
    def borrowed(cls, handle, owner, resolution, grid_spacing, origin=(0.0, 0.0, 0.0)):
        """The pressure solver another solver owns (the FLIP solver's
        ``pressureSolver``, grid_flip_solver3.js:1144-1155): the same
        methods on its handle, which ``close`` leaves to the owner."""
        self = cls.__new__(cls)
        self.resolution = tuple(int(n) for n in resolution)
        self.grid_spacing = tuple(float(h) for h in grid_spacing)
        self.origin = tuple(float(o) for o in origin)
        self.desc = None
        self.handle = C.c_void_p(handle)
        self._owner = owner
        self._bind(None)
        return self

    # -- inputs ------------------------------------------------------------
    def set_face_weights(self, fw):
        self._keep["fw"] = fw
        h = (fw["u"].handle, fw["v"].handle, fw.get("w").handle if fw.get("w") is not None else None) \
            if fw is not None else (None, None, None)
        _lib.check(_lib.load().ff_pressure3_set_face_weights(self.handle, *h))

    def set_collider_weights(self, cw):
        self._keep["cw"] = cw
        h = (cw["u"].handle, cw["v"].handle, cw.get("w").handle if cw.get("w") is not None else None) \
            if cw is not None else (None, None, None)
        _lib.check(_lib.load().ff_pressure3_set_collider_weights(self.handle, *h))

    def update_dirichlet(self, dirichlet=None):
        """Evaluate the Dirichlet condition on the cell centres
        (updateDirichletFields, grid_pressure_solver3.js:171-206)."""
        if dirichlet is not None:
            self._dirichlet = dirichlet
        dl = self._dirichlet
        if dl is None:
            _lib.check(_lib.load().ff_pressure3_set_dirichlet(self.handle, None, None))
            return
        if hasattr(dl, "fields"):
            # evaluated on the device (outflow Dirichlet, combinations)
            a, t = dl.fields(self.resolution, self.grid_spacing, self.origin)
            self._keep["dirichlet"] = (a, t)
            _lib.check(_lib.load().ff_pressure3_set_dirichlet(self.handle, a.handle, t.handle))
            return
        if callable(dl):
            x, y, z = cell_positions(self.resolution, self.grid_spacing, self.origin)
            active, target = dl(x, y, z)
        else:
            active, target = dl
        n = int(np.prod(self.resolution))
        a = Field("uint8", self.resolution).from_array(np.broadcast_to(np.asarray(active, bool), (n,)).astype(np.uint8))
        t = Field("float", self.resolution).from_array(np.broadcast_to(np.asarray(target, np.float32), (n,)))
        self._keep["dirichlet"] = (a, t)
        _lib.check(_lib.load().ff_pressure3_set_dirichlet(self.handle, a.handle, t.handle))

    @property
    def settings(self):
        return _Settings(self)

    # -- projection ----------------------------------------------------------
    def project(self, input_grid, output_grid):
        """project(inGrid, outGrid) -> dispatch() (grid_pressure_solver3.js:339-556)."""
        if tuple(input_grid.resolution) != self.resolution[: len(input_grid.resolution)] and \
                tuple(input_grid.resolution) + (1,) != self.resolution:
            raise ValueError(f"createGridPressureSolver3: project() input resolution "
                             f"{list(input_grid.resolution)} does not match constructed resolution "
                             f"{list(self.resolution)}.")

        def dispatch():
            diag = _lib.Diag()
            w_in = input_grid.data_w.handle if getattr(input_grid, "data_w", None) is not None else None
            w_out = output_grid.data_w.handle if getattr(output_grid, "data_w", None) is not None else None
            _lib.check(_lib.load().ff_pressure3_project(
                self.handle, input_grid.data_u.handle, input_grid.data_v.handle, w_in,
                output_grid.data_u.handle, output_grid.data_v.handle, w_out, C.byref(diag)))
            self.diagnostics.update(
                converged=bool(diag.converged), rejected=bool(diag.rejected),
                iterations=int(diag.iterations), stoppedBy=STOP_REASONS[diag.stopped_by],
                residual=float(diag.residual), bNorm=float(diag.b_norm),
                badCells=int(diag.bad_cells), maxIterations=int(diag.max_iterations),
                kernelLaunches=int(diag.kernel_launches), warmStart=int(diag.warm_start))
            self.diagnostics.update(_floor_diagnostics(diag, self._tolerance()))
            return self.diagnostics

        return dispatch

    def _tolerance(self):
        return getattr(self, "_tol", None)

    def project_host(self, input_grid, output_grid, host_in, host_out):
        """project(input_grid, output_grid) with the velocity coming from
        and going to host memory: `host_in` / `host_out` are (u, v, w)
        page-locked host addresses (ints or c_void_p, w None in 2D) of the
        grids' sizes.  Uploads overlap the previous call's downloads; the
        outputs are in place after the context synchronises."""
        diag = _lib.Diag()
        ptr = lambda a: C.c_void_p(a.value if isinstance(a, C.c_void_p) else a) if a is not None else None
        w_in = input_grid.data_w.handle if getattr(input_grid, "data_w", None) is not None else None
        w_out = output_grid.data_w.handle if getattr(output_grid, "data_w", None) is not None else None
        _lib.check(_lib.load().ff_pressure3_project_host(
            self.handle, input_grid.data_u.handle, input_grid.data_v.handle, w_in, *[ptr(a) for a in host_in],
            output_grid.data_u.handle, output_grid.data_v.handle, w_out, *[ptr(a) for a in host_out],
            C.byref(diag)))
        self.diagnostics.update(
            converged=bool(diag.converged), rejected=bool(diag.rejected),
            iterations=int(diag.iterations), stoppedBy=STOP_REASONS[diag.stopped_by],
            residual=float(diag.residual), bNorm=float(diag.b_norm),
            badCells=int(diag.bad_cells), maxIterations=int(diag.max_iterations),
            kernelLaunches=int(diag.kernel_launches), warmStart=int(diag.warm_start))
        self.diagnostics.update(_floor_diagnostics(diag, self._tolerance()))
        return dict(self.diagnostics)

    def solve(self, b):
        """cg.solve on A p = b for a given b Field; returns diagnostics."""
        diag = _lib.Diag()
        _lib.check(_lib.load().ff_pressure3_solve(self.handle, b.handle, C.byref(diag)))
        self.diagnostics.update(
            converged=bool(diag.converged), rejected=bool(diag.rejected),
            iterations=int(diag.iterations), stoppedBy=STOP_REASONS[diag.stopped_by],
            residual=float(diag.residual), bNorm=float(diag.b_norm),
            badCells=int(diag.bad_cells), maxIterations=int(diag.max_iterations),
            warmStart=int(diag.warm_start))
        self.diagnostics.update(_floor_diagnostics(diag, self._tolerance()))
        return dict(self.diagnostics)

    # -- test hooks -----------------------------------------------------------
    def prepare(self, input_grid=None):
        g = input_grid
        args = (g.data_u.handle, g.data_v.handle,
                g.data_w.handle if getattr(g, "data_w", None) is not None else None) if g else (None,) * 3
        _lib.check(_lib.load().ff_pressure3_prepare(self.handle, *args))

    def apply_laplacian(self, x, y):
        _lib.check(_lib.load().ff_laplacian_apply(self.handle, x.handle, y.handle))

    def apply_preconditioner(self, r, z):
        _lib.check(_lib.load().ff_precondition_apply(self.handle, r.handle, z.handle))

    def level_shape(self, level):
        s = (C.c_int * 3)()
        _lib.check(_lib.load().ff_mg_level_info(self.handle, level, s))
        return tuple(s)

    def level_data(self, level):
        nx, ny, nz = self.level_shape(level)
        mask = np.empty(nx * ny * nz, np.uint8)
        ws = [np.empty((nx + (a == 0)) * (ny + (a == 1)) * (nz + (a == 2)), np.float32) for a in range(3)]
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        _lib.check(_lib.load().ff_mg_level_download(self.handle, level, mask.ctypes.data_as(C.POINTER(C.c_uint8)),
                                                    fp(ws[0]), fp(ws[1]), fp(ws[2])))
        return mask, ws

    def restrict(self, fine_level, fine, coarse):
        _lib.check(_lib.load().ff_mg_restrict(self.handle, fine_level, fine.handle, coarse.handle))

    def prolong_add(self, fine_level, coarse, fine):
        _lib.check(_lib.load().ff_mg_prolong_add(self.handle, fine_level, coarse.handle, fine.handle))

    def close(self):
        if getattr(self, "_owner", None) is not None:
            self.handle = None      # the owner destroys it
            return
        if getattr(self, "handle", None):
            _lib.load().ff_pressure3_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _floor_diagnostics(diag, tolerance):
    """The reportNoiseFloor diagnostics (grid_pressure_solver3.js:517-542,
    linalg.js:884-905): None while the setting is off."""
    if not diag.report_floor:
        return dict(maxResidual=None, noiseFloor=None, noiseFloorRelative=None, toleranceBelowFloor=None,
                    residualOverFloor=None)
    floor = float(diag.noise_floor)
    below = ({"requested": float(diag.floor_threshold), "floor": floor, "tolerance": tolerance}
             if diag.tolerance_below_floor else None)
    return dict(maxResidual=float(diag.max_residual), noiseFloor=floor,
                noiseFloorRelative=float(diag.noise_floor_relative) if diag.b_norm > 0 else None,
                toleranceBelowFloor=below,
                residualOverFloor=float(diag.residual) / floor if floor else None)


class _Settings:
    """The runtime ``settings`` object (grid_pressure_solver3.js:135)."""

    _KEYS = {"tolerance", "maxIterations", "relativeTolerance", "checkBadCells", "useGraph",
             "useTma", "coarseTail", "preconditioner", "sorFactor", "reportNoiseFloor"}

    def __init__(self, solver):
        object.__setattr__(self, "_s", solver)

    def __setattr__(self, key, value):
        if key not in self._KEYS:
            raise AttributeError(f"unknown setting '{key}'")
        if key == "preconditioner":
            value = PRECONDITIONERS[value]
        _lib.check(_lib.load().ff_pressure3_set(self._s.handle, key.encode(), float(value)))
        if key == "tolerance":
            self._s._tol = float(value)

    __setitem__ = __setattr__


def create_grid_pressure_solver3(resolution, grid_spacing, origin=(0.0, 0.0, 0.0), **options):
    return GridPressureSolver3(resolution, grid_spacing, origin, **options)


def create_grid_pressure_solver2(resolution, grid_spacing, origin=(0.0, 0.0), **options):
    """createGridPressureSolver2 (grid_pressure_solver2.js:223-981): the same
    solver with nz = 1 (no z axis)."""
    return GridPressureSolver3(tuple(resolution) + (1,), tuple(grid_spacing) + (1.0,),
                               tuple(origin) + (0.0,), **options)


# ------------------------------------------------------------- advection --
class SemiLagrangianAdvectionSolver3:
    """createSemiLagrangianAdvectionSolver3({velocityGrid, collider, dt,
    maxSubsteps = 32, order = 1}) (advection_solver3.js:67-364).  Methods
    return a dispatch function, as the reference returns its batch."""

    def __init__(self, velocity_grid, collider=None, dt=None, max_substeps=32, order=1):
        if dt is None:
            raise ValueError("createSemiLagrangianAdvectionSolver3: dt is required.")
        self.velocity_grid = velocity_grid
        d = _lib.AdvectDesc()
        d.resolution[:] = list(velocity_grid.resolution)
        d.grid_spacing[:] = list(velocity_grid.grid_spacing)
        d.origin[:] = list(velocity_grid.origin)
        d.dt = float(dt)
        d.max_substeps = int(max_substeps)
        d.order = int(order)
        self.handle = C.c_void_p()
        _lib.check(_lib.load().ff_advect3_create(context().handle, C.byref(d), C.byref(self.handle)))
        self.collider = collider
        _lib.check(_lib.load().ff_advect3_set_collider(self.handle, collider.phi.handle if collider else None))

    def set_dt(self, dt):
        _lib.check(_lib.load().ff_advect3_set_dt(self.handle, float(dt)))

    def _vel(self):
        g = self.velocity_grid
        return g.data_u.handle, g.data_v.handle, g.data_w.handle

    def advect_face_centered3(self, input_grid, output_grid):
        def dispatch():
            _lib.check(_lib.load().ff_advect3_faces(
                self.handle, *self._vel(), input_grid.data_u.handle, input_grid.data_v.handle,
                input_grid.data_w.handle, output_grid.data_u.handle, output_grid.data_v.handle,
                output_grid.data_w.handle))
        return dispatch

    def advect_scalar3(self, input_field, output_field):
        def dispatch():
            _lib.check(_lib.load().ff_advect3_scalar(self.handle, *self._vel(), input_field.handle,
                                                     output_field.handle))
        return dispatch

    def trace(self, points_in, points_out, direction=1):
        """trace(start, direction) of a vec3 field of points."""
        _lib.check(_lib.load().ff_advect3_trace(self.handle, *self._vel(), points_in.handle,
                                                points_out.handle, int(direction)))

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().ff_advect3_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def create_semi_lagrangian_advection_solver3(velocity_grid=None, collider=None, dt=None, max_substeps=32,
                                             order=1):
    return SemiLagrangianAdvectionSolver3(velocity_grid, collider, dt, max_substeps, order)


# ------------------------------------------------------ boundary conditions --
DIRECTION_LEFT, DIRECTION_RIGHT, DIRECTION_DOWN, DIRECTION_UP = 1, 2, 4, 8
DIRECTION_BACK, DIRECTION_FRONT = 16, 32
DIRECTION_ALL_3D = 63


class SDFInflow3(SDFStaticCollider3):
    """createSDFInflow3(..., {velocity, mode}) (sdf_inflow_outflow3.js:15-22):
    an SDF region (baked like a static collider) with a velocity that faces
    inside it take ('set') or gain ('add')."""

    def __init__(self, resolution, grid_spacing, origin=(0.0, 0.0, 0.0), velocity=(0.0, 0.0, 0.0), mode="set"):
        super().__init__(resolution, grid_spacing, origin)
        if mode not in ("set", "add"):
            raise ValueError(f"createSDFInflow3: unknown mode '{mode}'.")
        self.velocity = tuple(float(v) for v in velocity)
        self.mode = mode


def create_sdf_inflow3(nx, ny, nz, hx, hy, hz, ox=0.0, oy=0.0, oz=0.0, velocity=(0.0, 0.0, 0.0), mode="set"):
    return SDFInflow3((nx, ny, nz), (hx, hy, hz), (ox, oy, oz), velocity, mode)


class GridBlockedBoundaryConditionSolver3:
    """createGridBlockedBoundaryConditionSolver3(velocity, resolution...,
    colliderSDF, inflows, colliderFaceWeights)
    (grid_blocked_boundary_condition_solver3.js:48-490)."""

    def __init__(self, velocity, resolution, grid_spacing, origin=(0.0, 0.0, 0.0), collider=None, inflows=None,
                 collider_face_weights=None):
        self.velocity = velocity
        self.handle = C.c_void_p()
        _lib.check(_lib.load().ff_bc3_create(context().handle, (C.c_int * 3)(*resolution),
                                             (C.c_double * 3)(*grid_spacing), (C.c_double * 3)(*origin),
                                             C.byref(self.handle)))
        self._closed = DIRECTION_ALL_3D
        self.set_collider(collider, collider_face_weights)
        self.set_inflows(inflows)

    @property
    def closed_domain_boundary_flag(self):
        return self._closed

    @closed_domain_boundary_flag.setter
    def closed_domain_boundary_flag(self, flag):
        _lib.check(_lib.load().ff_bc3_set_closed(self.handle, int(flag)))
        self._closed = int(flag)

    def set_collider(self, collider, face_weights=None):
        self.collider, self.face_weights = collider, face_weights
        w = face_weights or {}
        _lib.check(_lib.load().ff_bc3_set_collider(
            self.handle, collider.phi.handle if collider else None,
            w["u"].handle if "u" in w else None, w["v"].handle if "v" in w else None,
            w["w"].handle if "w" in w else None))

    def set_inflows(self, inflows):
        lst = [] if not inflows else (list(inflows) if isinstance(inflows, (list, tuple)) else [inflows])
        self.inflows = lst
        n = len(lst)
        phis = (C.c_void_p * max(1, n))(*[q.phi.handle.value for q in lst])
        vel = (C.c_double * max(3, 3 * n))(*[c for q in lst for c in q.velocity])
        modes = (C.c_int * max(1, n))(*[0 if q.mode == "set" else 1 for q in lst])
        _lib.check(_lib.load().ff_bc3_set_inflows(self.handle, n, phis, vel, modes))

    def constrain_velocity(self, extrapolation_depth=5):
        g = self.velocity
        _lib.check(_lib.load().ff_bc3_constrain(self.handle, g.data_u.handle, g.data_v.handle, g.data_w.handle,
                                                int(extrapolation_depth)))

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().ff_bc3_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def create_grid_blocked_boundary_condition_solver3(velocity, nx, ny, nz, hx, hy, hz, ox=0.0, oy=0.0, oz=0.0,
                                                   collider=None, inflows=None, collider_face_weights=None):
    return GridBlockedBoundaryConditionSolver3(velocity, (nx, ny, nz), (hx, hy, hz), (ox, oy, oz), collider,
                                               inflows, collider_face_weights)


class SDFOutflow3(SDFStaticCollider3):
    """createSDFOutflow3 (sdf_inflow_outflow3.js:25-29): an outflow region,
    baked like a static collider (solid = inside the outflow)."""


def create_sdf_outflow3(nx, ny, nz, hx, hy, hz, ox=0.0, oy=0.0, oz=0.0):
    return SDFOutflow3((nx, ny, nz), (hx, hy, hz), (ox, oy, oz))


def _outflow_handle(res, spacing, origin, outflows, dt, apply_velocity_bc):
    n = len(outflows)
    h = C.c_void_p()
    _lib.check(_lib.load().ff_outflow3_create(
        context().handle, (C.c_int * 3)(*res), (C.c_double * 3)(*spacing), (C.c_double * 3)(*origin), n,
        (C.c_void_p * max(1, n))(*[q.phi.handle.value for q in outflows]),
        (C.c_int * max(3, 3 * n))(*[int(x) for q in outflows for x in q.resolution]),
        (C.c_double * max(3, 3 * n))(*[float(x) for q in outflows for x in q.grid_spacing]),
        (C.c_double * max(3, 3 * n))(*[float(x) for q in outflows for x in q.origin]),
        float(dt), int(bool(apply_velocity_bc)), C.byref(h)))
    return h


class OutflowPressureDirichlet3:
    """createOutflowPressureDirichlet3(outflows, {target = 0})
    (sdf_inflow_outflow3.js:44-64): Dirichlet wherever an outflow holds a
    cell centre.  GridPressureSolver3 evaluates it on the device at its own
    cell centres (``fields``)."""

    def __init__(self, outflows, target=0.0, _handle=None, _owner=None):
        self.outflows = list(outflows) if isinstance(outflows, (list, tuple)) else [outflows]
        self.target = float(target)
        self._owner = _owner
        self._own = _handle is None
        self.handle = _handle if _handle is not None else _outflow_handle((1, 1, 1), (1.0,) * 3, (0.0,) * 3,
                                                                           self.outflows, 0.0, False)

    def fields(self, resolution, grid_spacing, origin=(0.0, 0.0, 0.0)):
        a, t = Field("uint8", tuple(resolution)), Field("float", tuple(resolution))
        _lib.check(_lib.load().ff_outflow3_dirichlet(self.handle, (C.c_int * 3)(*resolution),
                                                     (C.c_double * 3)(*grid_spacing), (C.c_double * 3)(*origin),
                                                     self.target, a.handle, t.handle))
        return a, t

    def close(self):
        if self._own and getattr(self, "handle", None):
            _lib.load().ff_outflow3_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def create_outflow_pressure_dirichlet3(outflows, target=0.0):
    return OutflowPressureDirichlet3(outflows, target)


def _dirichlet_arrays(d, resolution, grid_spacing, origin):
    n = int(np.prod(resolution))
    if hasattr(d, "fields"):
        a, t = d.fields(resolution, grid_spacing, origin)
        return a.to_array().astype(bool), t.to_array()
    active, target = d(*cell_positions(resolution, grid_spacing, origin)) if callable(d) else d
    return (np.broadcast_to(np.asarray(active, bool), (n,)),
            np.broadcast_to(np.asarray(target, np.float32), (n,)))


class _CombinedDirichlet3:
    def __init__(self, a, b):
        self.a, self.b = a, b

    def fields(self, resolution, grid_spacing, origin=(0.0, 0.0, 0.0)):
        aa, at = _dirichlet_arrays(self.a, resolution, grid_spacing, origin)
        ba, bt = _dirichlet_arrays(self.b, resolution, grid_spacing, origin)
        return (Field("uint8", tuple(resolution)).from_array((aa | ba).astype(np.uint8)),
                Field("float", tuple(resolution)).from_array(np.where(ba, bt, at).astype(np.float32)))


def combine_dirichlet3(a, b):
    """combineDirichlet3 (sdf_inflow_outflow3.js:77-94): active where
    either is, b's target where b is active (b wins on overlap)."""
    if not a:
        return b
    if not b:
        return a
    return _CombinedDirichlet3(a, b)


class GridOutflowSolver3:
    """createGridOutflowSolver3({velocityGrid, velocityPrev, outflows, dt,
    applyVelocityBC}) (grid_outflow_solver3.js:79-210): the pressure
    Dirichlet of the outflow cells (``dirichlet``), the convective velocity
    condition (``apply_outflow_velocity_bc``) and scalar clearing
    (``clear_outflow_scalar_field``).  velocityPrev is accepted and unused,
    as in the reference."""

    def __init__(self, velocity_grid, outflows, dt, apply_velocity_bc=True, velocity_prev=None):
        g = velocity_grid
        self.velocity_grid = g
        self.outflows = list(outflows) if isinstance(outflows, (list, tuple)) else [outflows]
        self.handle = _outflow_handle(g.resolution, g.grid_spacing, g.origin, self.outflows, dt, apply_velocity_bc)
        self.dirichlet = OutflowPressureDirichlet3(self.outflows, 0.0, _handle=self.handle, _owner=self)

    def set_dt(self, dt):
        _lib.check(_lib.load().ff_outflow3_set_dt(self.handle, float(dt)))

    def apply_outflow_velocity_bc(self):
        g = self.velocity_grid
        _lib.check(_lib.load().ff_outflow3_apply_velocity_bc(self.handle, g.data_u.handle, g.data_v.handle,
                                                             g.data_w.handle))

    def clear_outflow_scalar_field(self, scalar, resolution=None, grid_spacing=None, origin=None):
        """Returns clear(): zero the cells of ``scalar`` (a float cell Field;
        geometry defaults to the velocity grid's) inside any outflow."""
        g = self.velocity_grid
        res = (C.c_int * 3)(*(resolution or g.resolution))
        h = (C.c_double * 3)(*(grid_spacing or g.grid_spacing))
        o = (C.c_double * 3)(*(origin or g.origin))

        def clear():
            _lib.check(_lib.load().ff_outflow3_clear_scalar(self.handle, scalar.handle, res, h, o))
        return clear

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().ff_outflow3_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def create_grid_outflow_solver3(velocity_grid=None, outflows=None, dt=None, apply_velocity_bc=True,
                                velocity_prev=None):
    return GridOutflowSolver3(velocity_grid, outflows, dt, apply_velocity_bc, velocity_prev)


def apply_viscosity3(input_grid, output_grid, nu, dt):
    """Explicit viscosity u += dt nu lap(u) (no reference counterpart:
    grid_solver3.js:104 leaves computeViscosity a no-op)."""
    g = input_grid
    _lib.check(_lib.load().ff_viscosity3_apply(
        context().handle, (C.c_int * 3)(*g.resolution), (C.c_double * 3)(*g.grid_spacing), g.data_u.handle,
        g.data_v.handle, g.data_w.handle, float(nu), float(dt), output_grid.data_u.handle,
        output_grid.data_v.handle, output_grid.data_w.handle))


# -------------------------------------------------------------------- FLIP --
DEFAULT_JITTER_SEED = 0x9E3779B9   # jitter_random.js:46


def create_jitter_random(seed):
    """createJitterRandom(seed): a function returning the next value in [0, 1)."""
    state = {"seed": int(seed) & 0xFFFFFFFF, "i": 0, "buf": []}

    def random():
        if state["i"] >= len(state["buf"]):
            n = 1024 + state["i"]
            out = (C.c_double * n)()
            _lib.check(_lib.load().ff_jitter_random(state["seed"], n, out))
            state["buf"] = list(out)
        v = state["buf"][state["i"]]
        state["i"] += 1
        return v
    return random


def compute_flip_box_seed3(box_min, box_max, grid_spacing_x, grid_spacing_y, grid_spacing_z, particles_per_cell_axis=2,
                           jitter=0.2, random_seed=DEFAULT_JITTER_SEED):
    """computeFlipBoxSeed3({boxMin, boxMax, gridSpacingX/Y/Z,
    particlesPerCellAxis, jitter, randomSeed}) -> {count, positionsArray,
    velocitiesArray}."""
    dd = lambda v: (C.c_double * 3)(*[float(x) for x in v])
    h = dd((grid_spacing_x, grid_spacing_y, grid_spacing_z))
    lib = _lib.load()
    count = C.c_int64()
    _lib.check(lib.ff_flip_box_seed3(dd(box_min), dd(box_max), h, int(particles_per_cell_axis), float(jitter),
                                     int(random_seed) & 0xFFFFFFFF, None, 0, C.byref(count)))
    pos = np.empty(3 * count.value, np.float32)
    _lib.check(lib.ff_flip_box_seed3(dd(box_min), dd(box_max), h, int(particles_per_cell_axis), float(jitter),
                                     int(random_seed) & 0xFFFFFFFF, pos.ctypes.data_as(C.POINTER(C.c_float)),
                                     count.value, C.byref(count)))
    return {"count": count.value, "positionsArray": pos, "velocitiesArray": np.zeros_like(pos)}


class GridFlipSolver3:
    """createGridFlipSolver3({velocityGrid, gridSpacing, origin, maxParticles,
    dt, gravity, reducedPressure, flipRatio, velocityDamping, p2gAtomicScale,
    weightEpsilon, closedDomainBoundaryFlag, collider, colliderPushThresh,
    colliderPushShift, carryConcentration, mixing, fade,
    concentrationAtomicScale, ambientDensity, componentDensity, pressure,
    resample}) (grid_flip_solver3.js:135-1157).  resample = {enabled=True,
    minParticlesPerCell=4, maxParticlesPerCell=8} (:178-180) moves particles
    from over-full cells to under-full cells beside the fluid each step
    (:621-820)."""

    STAGES = {"advectParticles": 0, "p2g": 1, "snapshotOld": 2, "extrapolateWeight": 3, "constrainVelocity": 4,
              "markFluidCells": 5, "concentrationGrid": 6, "gravity": 7, "project": 8, "extrapolatePressure": 9,
              "g2p": 10, "concentrationParticle": 11, "resample": 12}

    def __init__(self, velocity_grid=None, max_particles=None, dt=None, gravity=(0.0, -9.81, 0.0),
                 reduced_pressure=True, flip_ratio=0.97, velocity_damping=0.02, p2g_atomic_scale=65536.0,
                 weight_epsilon=1e-4, closed_domain_boundary_flag=None, collider=None, collider_push_thresh=0.0,
                 collider_push_shift=0.0, carry_concentration=False, mixing=0.0, fade=0.0,
                 concentration_atomic_scale=4096.0, ambient_density=None, component_density=None, pressure=None,
                 max_substeps=32, extrapolation_depth=5, resample=None):
        if velocity_grid is None:
            raise ValueError("createGridFlipSolver3: options.velocityGrid is required.")
        if not max_particles:
            raise ValueError("createGridFlipSolver3: options.maxParticles is required.")
        g = velocity_grid
        self.velocity_grid = g
        lib = _lib.load()
        d = _lib.FlipDesc()
        lib.ff_flip_desc_default(C.byref(d), (C.c_int * 3)(*g.resolution), (C.c_double * 3)(*g.grid_spacing),
                                 int(max_particles), float(dt))
        d.origin[:] = list(g.origin)
        d.gravity[:] = [float(x) for x in gravity]
        d.reduced_pressure = int(bool(reduced_pressure))
        d.flip_ratio, d.velocity_damping = float(flip_ratio), float(velocity_damping)
        d.p2g_atomic_scale, d.weight_epsilon = float(p2g_atomic_scale), float(weight_epsilon)
        if closed_domain_boundary_flag is not None:
            d.closed_flags = int(closed_domain_boundary_flag)
        d.max_substeps = int(max_substeps)
        d.collider_push_thresh, d.collider_push_shift = float(collider_push_thresh), float(collider_push_shift)
        d.carry_concentration = int(bool(carry_concentration))
        d.mixing, d.fade = float(mixing), float(fade)
        d.concentration_atomic_scale = float(concentration_atomic_scale)
        if (ambient_density is None) != (component_density is None):
            raise ValueError("createGridFlipSolver3: give both ambientDensity and componentDensity or neither.")
        if ambient_density is not None:
            d.ambient_density, d.component_density = float(ambient_density), float(component_density)
        d.extrapolation_depth = int(extrapolation_depth)
        rs = resample or {}
        d.resample_enabled = int(bool(rs.get("enabled", True)))
        d.min_particles_per_cell = int(rs.get("minParticlesPerCell", 4))
        d.max_particles_per_cell = int(rs.get("maxParticlesPerCell", 8))
        p = pressure or {}
        mg = p.get("multigrid", {})
        pd = d.pressure
        pd.preconditioner = PRECONDITIONERS[p.get("preconditioner", "multigrid")]
        pd.tolerance = float(p.get("tolerance", pd.tolerance))
        pd.mg_levels = int(mg.get("numberOfLevels", pd.mg_levels))
        pd.mg_down = int(mg.get("numberOfSmoothingIterationsDown", pd.mg_down))
        pd.mg_up = int(mg.get("numberOfSmoothingIterationsUp", pd.mg_up))
        pd.mg_coarsest = int(mg.get("numberOfCoarsestIterations", pd.mg_coarsest))
        pd.mg_coarse_mode = 1 if mg.get("coarseSolve", "sweeps") == "direct" else 0
        if "maxPlausiblePressure" in p:
            pd.max_plausible_pressure = float(p["maxPlausiblePressure"])
        if p.get("precision", "fp32") != "fp32":
            pd.iterate = 1
        self.desc = d
        self.handle = C.c_void_p()
        _lib.check(lib.ff_flip3_create(context().handle, C.byref(d), g.data_u.handle, g.data_v.handle,
                                       g.data_w.handle, C.byref(self.handle)))
        self.collider = collider
        if collider is not None:
            _lib.check(lib.ff_flip3_set_collider(self.handle, collider.phi.handle))
        hs = [C.c_void_p() for _ in range(5)]
        _lib.check(lib.ff_flip3_fields(self.handle, *[C.byref(x) for x in hs]))
        ctx = context()
        self.positions = BorrowedField(hs[0], ctx)
        self.velocities = BorrowedField(hs[1], ctx)
        self.concentration = BorrowedField(hs[2], ctx) if hs[2].value else None
        self.fluid_mask = BorrowedField(hs[3], ctx)
        self.pressure_solver = GridPressureSolver3.borrowed(hs[4].value, self, g.resolution, g.grid_spacing, g.origin)
        self.pressure = self.pressure_solver.pressure
        self.diagnostics = {}

    def grid_fields(self):
        """cellConcentration, cellDensity, (betaU, betaV, betaW) and the
        Dirichlet active/target fields of the last projection (None when
        not in use)."""
        hs = [C.c_void_p() for _ in range(7)]
        _lib.check(_lib.load().ff_flip3_grid_fields(self.handle, *[C.byref(x) for x in hs]))
        ctx = context()
        f = [BorrowedField(h, ctx) if h.value else None for h in hs]
        return {"cellConcentration": f[0], "cellDensity": f[1], "beta": tuple(f[2:5]), "dirichletActive": f[5],
                "dirichletTarget": f[6]}

    def set_particle_count(self, n):
        _lib.check(_lib.load().ff_flip3_set_count(self.handle, int(n)))

    def stage(self, name):
        _lib.check(_lib.load().ff_flip3_stage(self.handle, self.STAGES[name]))

    def resample_stats(self):
        """The last resampling pass: {"donors", "requested", "moved"}."""
        dn, rq = C.c_int64(), C.c_int64()
        _lib.check(_lib.load().ff_flip3_resample_stats(self.handle, C.byref(dn), C.byref(rq)))
        return {"donors": dn.value, "requested": rq.value, "moved": min(dn.value, rq.value)}

    def on_advance_time_step(self):
        """onAdvanceTimeStep(): returns the projection's diagnostics."""
        d = _lib.Diag()
        _lib.check(_lib.load().ff_flip3_step(self.handle, C.byref(d)))
        self.diagnostics = {"converged": bool(d.converged), "rejected": bool(d.rejected),
                            "iterations": d.iterations, "stoppedBy": STOP_REASONS.get(d.stopped_by, "none"),
                            "residual": d.residual}
        return self.diagnostics

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().ff_flip3_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def create_grid_flip_solver3(**options):
    return GridFlipSolver3(**options)


# ---------------------------------------------------------------- solver --
class FaceCenteredGrid2:
    """createFaceCenteredGrid2 (grid_data2.js): u (nx+1, ny), v (nx, ny+1),
    staggered origins; the same memory as a one-cell-thick 3D grid's u and
    v."""

    def __init__(self, resolution, grid_spacing=(1.0, 1.0), origin=(0.0, 0.0)):
        nx, ny = resolution
        self.resolution = (nx, ny)
        self.grid_spacing = tuple(float(h) for h in grid_spacing)
        self.origin = tuple(float(o) for o in origin)
        self.data_size_u = (nx + 1, ny)
        self.data_size_v = (nx, ny + 1)
        self.data_u = Field("float", self.data_size_u)
        self.data_v = Field("float", self.data_size_v)
        hx, hy = self.grid_spacing
        ox, oy = self.origin
        self.data_origin_u = (ox, oy + 0.5 * hy)
        self.data_origin_v = (ox + 0.5 * hx, oy)

    def set(self, u, v):
        self.data_u.from_array(u)
        self.data_v.from_array(v)
        return self

    def get(self):
        return self.data_u.to_array(), self.data_v.to_array()


def create_face_centered_grid2(nx, ny, hx=1.0, hy=1.0, ox=0.0, oy=0.0):
    return FaceCenteredGrid2((nx, ny), (hx, hy), (ox, oy))


PHASE_GAS, PHASE_LIQUID = 0, 1


def compute_two_phase_box_seed(box_min, box_max, grid_spacing_x, grid_spacing_y, particles_per_cell_axis=2,
                               jitter=0.2, random_seed=DEFAULT_JITTER_SEED, is_liquid=None, concentration_at=None):
    """computeTwoPhaseBoxSeed (grid_two_phase_flip_solver2.js:397-477): a
    jittered box of particles, each tagged with a phase (or a concentration
    from ``concentration_at``), computed in doubles as JavaScript does."""
    min_x, min_y = (float(x) for x in box_min)
    max_x, max_y = (float(x) for x in box_max)
    jsround = lambda x: math.floor(x + 0.5)
    cells_x = max(1, jsround((max_x - min_x) / grid_spacing_x))
    cells_y = max(1, jsround((max_y - min_y) / grid_spacing_y))
    k = int(particles_per_cell_axis)
    sub_x, sub_y = grid_spacing_x / k, grid_spacing_y / k
    rnd = create_jitter_random(random_seed)
    pos, phases = [], []
    for cj in range(cells_y):
        for ci in range(cells_x):
            for sj in range(k):
                for si in range(k):
                    jx = (rnd() * 2 - 1) * jitter * sub_x
                    jy = (rnd() * 2 - 1) * jitter * sub_y
                    x = min_x + ci * grid_spacing_x + (si + 0.5) * sub_x + jx
                    y = min_y + cj * grid_spacing_y + (sj + 0.5) * sub_y + jy
                    pos += [x, y]
                    if concentration_at is not None:
                        phases.append(min(1.0, max(0.0, float(concentration_at([x, y])))))
                    else:
                        phases.append(PHASE_LIQUID if (is_liquid is None or is_liquid([x, y])) else PHASE_GAS)
    ph = np.array(phases, np.float32)
    n = len(phases)
    return {"count": n, "positionsArray": np.array(pos, np.float32), "velocitiesArray": np.zeros(2 * n, np.float32),
            "phasesArray": ph, "liquidCount": int((ph > 0.5).sum()), "gasCount": int(n - (ph > 0.5).sum()),
            "meanConcentration": float(np.sum(ph.astype(np.float64))) / n if n else 0.0}


class _TwoPhaseParticles:
    """positions / velocities of the two-phase solver as (x, y) pairs."""

    def __init__(self, solver, which):
        self._s, self._w = solver, which

    def from_array(self, values):
        a = np.ascontiguousarray(values, np.float32).ravel()
        n = a.size // 2
        fp = a.ctypes.data_as(C.POINTER(C.c_float))
        args = (fp, None, None) if self._w == 0 else (None, fp, None)
        _lib.check(_lib.load().ff_twophase2_set_particles(self._s.handle, n, *args))
        return self

    def to_array(self):
        n = self._s.max_particles
        out = np.empty(2 * n, np.float32)
        fp = out.ctypes.data_as(C.POINTER(C.c_float))
        args = (fp, None, None) if self._w == 0 else (None, fp, None)
        _lib.check(_lib.load().ff_twophase2_get_particles(self._s.handle, n, *args))
        return out


class GridTwoPhaseFlipSolver2:
    """createGridTwoPhaseFlipSolver2({velocityGrid, gridSpacing, origin,
    maxParticles, dt, gravity, liquidDensity, gasDensity, ambientDensity,
    componentDensity, mixing, fade, concentrationAtomicScale, flipRatio,
    gasFlipRatio, velocityDamping, p2gAtomicScale, weightEpsilon,
    closedDomainBoundaryFlag, collider, colliderPushThresh,
    colliderPushShift, pressurePin, resample, pressure})
    (grid_two_phase_flip_solver2.js:479-1622)."""

    STAGES = {"advectParticles": 0, "density": 1, "p2g": 2, "snapshotOld": 3, "extrapolateWeight": 4,
              "constrainVelocity": 5, "gravity": 6, "project": 7, "g2p": 8, "mixConcentration": 9, "resample": 10}

    def __init__(self, velocity_grid=None, grid_spacing=None, origin=None, max_particles=None, dt=None,
                 gravity=(0.0, -9.81), liquid_density=1.0, gas_density=0.01, ambient_density=None,
                 component_density=None, mixing=0.0, fade=0.0, concentration_atomic_scale=4096.0, flip_ratio=0.97,
                 gas_flip_ratio=0.90, velocity_damping=0.02, p2g_atomic_scale=65536.0, weight_epsilon=1e-4,
                 closed_domain_boundary_flag=None, collider=None, collider_push_thresh=0.0, collider_push_shift=0.0,
                 pressure_pin="topCenter", resample=None, pressure=None, max_substeps=32):
        vocabulary = ambient_density is None and component_density is None
        if ambient_density is not None:
            gas_density = ambient_density
        if component_density is not None:
            liquid_density = component_density
        if velocity_grid is None:
            raise ValueError("createGridTwoPhaseFlipSolver2: options.velocityGrid is required.")
        if not max_particles:
            raise ValueError("createGridTwoPhaseFlipSolver2: options.maxParticles is required.")
        if not liquid_density > 0:
            raise ValueError("createGridTwoPhaseFlipSolver2: the concentration-1 density (liquidDensity / "
                             f"componentDensity) must be > 0, got {liquid_density}.")
        if not gas_density > 0:
            raise ValueError("createGridTwoPhaseFlipSolver2: the concentration-0 density (gasDensity / "
                             f"ambientDensity) must be > 0, got {gas_density}.")
        if vocabulary and gas_density > liquid_density:
            raise ValueError(f"createGridTwoPhaseFlipSolver2: gasDensity ({gas_density}) must not exceed "
                             f"liquidDensity ({liquid_density}) -- the two phase tags would then be named "
                             "backwards. Use ambientDensity/componentDensity for a lighter concentration-1 "
                             "component.")
        g = velocity_grid
        res = tuple(g.resolution)[:2]
        spacing = tuple(grid_spacing or g.grid_spacing)[:2]
        org = tuple(origin or g.origin)[:2]
        if pressure_pin == "topCenter":
            pin = (res[0] // 2, res[1] - 1)
        elif pressure_pin is None:
            pin = (-1, -1)
        elif isinstance(pressure_pin, (list, tuple)) and len(pressure_pin) == 2:
            pin = (int(pressure_pin[0]), int(pressure_pin[1]))
        else:
            raise ValueError("createGridTwoPhaseFlipSolver2: pressurePin must be 'topCenter', null, or an [i, j] "
                             f"cell index, got {pressure_pin!r}.")
        self.pin_cell = None if pin[0] < 0 else list(pin)
        lib = _lib.load()
        d = _lib.TwoPhaseDesc()
        lib.ff_twophase_desc_default(C.byref(d), (C.c_int * 2)(*res), (C.c_double * 2)(*spacing),
                                     int(max_particles), float(dt))
        d.origin[:] = [float(x) for x in org]
        d.gravity[:] = [float(x) for x in gravity]
        d.ambient_density, d.component_density = float(gas_density), float(liquid_density)
        d.mixing, d.fade = float(mixing), float(fade)
        d.concentration_atomic_scale = float(concentration_atomic_scale)
        d.flip_ratio, d.gas_flip_ratio = float(flip_ratio), float(gas_flip_ratio)
        d.velocity_damping = float(velocity_damping)
        d.p2g_atomic_scale, d.weight_epsilon = float(p2g_atomic_scale), float(weight_epsilon)
        if closed_domain_boundary_flag is not None:
            d.closed_flags = int(closed_domain_boundary_flag)
        d.collider_push_thresh, d.collider_push_shift = float(collider_push_thresh), float(collider_push_shift)
        d.pin_cell[:] = list(pin)
        d.max_substeps = int(max_substeps)
        rs = resample or {}
        d.resample_enabled = int(bool(rs.get("enabled", True)))
        d.min_particles_per_cell = int(rs.get("minParticlesPerCell", 3))
        d.max_particles_per_cell = int(rs.get("maxParticlesPerCell", 8))
        p = pressure or {}
        mg = p.get("multigrid", {})
        pd = d.pressure
        pd.preconditioner = PRECONDITIONERS[p.get("preconditioner", "multigrid")]
        pd.tolerance = float(p.get("tolerance", pd.tolerance))
        pd.mg_levels = int(mg.get("numberOfLevels", pd.mg_levels))
        pd.mg_down = int(mg.get("numberOfSmoothingIterationsDown", pd.mg_down))
        pd.mg_up = int(mg.get("numberOfSmoothingIterationsUp", pd.mg_up))
        pd.mg_coarsest = int(mg.get("numberOfCoarsestIterations", pd.mg_coarsest))
        pd.mg_coarse_mode = 1 if mg.get("coarseSolve", "sweeps") == "direct" else 0
        if "maxIterations" in p:
            pd.max_iterations = int(p["maxIterations"])
        if "maxPlausiblePressure" in p:
            pd.max_plausible_pressure = float(p["maxPlausiblePressure"])
        if p.get("precision", "fp32") != "fp32":
            pd.iterate = 1
        self.desc = d
        self.max_particles = int(max_particles)
        self.velocity_grid = g
        self.handle = C.c_void_p()
        _lib.check(lib.ff_twophase2_create(context().handle, C.byref(d), g.data_u.handle, g.data_v.handle,
                                           C.byref(self.handle)))
        self.collider = collider
        if collider is not None:
            _lib.check(lib.ff_twophase2_set_collider(self.handle, collider.phi.handle))
        hs = [C.c_void_p() for _ in range(6)]
        _lib.check(lib.ff_twophase2_fields(self.handle, *[C.byref(x) for x in hs]))
        ctx = context()
        self.positions = _TwoPhaseParticles(self, 0)
        self.velocities = _TwoPhaseParticles(self, 1)
        self.phase = BorrowedField(hs[0], ctx)
        self.concentration = self.phase
        self.liquid_fraction = BorrowedField(hs[1], ctx)
        self.density = BorrowedField(hs[2], ctx)
        self.beta_u = BorrowedField(hs[3], ctx)
        self.beta_v = BorrowedField(hs[4], ctx)
        pf = [C.c_void_p() for _ in range(4)]
        _lib.check(lib.ff_pressure3_fields(hs[5], *[C.byref(x) for x in pf]))
        self.pressure = BorrowedField(pf[0], ctx)
        self.diagnostics = {}

    def set_particle_count(self, n):
        _lib.check(_lib.load().ff_twophase2_set_count(self.handle, int(n)))

    def stage(self, name):
        _lib.check(_lib.load().ff_twophase2_stage(self.handle, self.STAGES[name]))

    def resample_stats(self):
        v = (C.c_int64 * 4)()
        _lib.check(_lib.load().ff_twophase2_resample_stats(self.handle, v))
        return {"liquidDonors": v[0], "liquidRequested": v[1], "gasDonors": v[2], "gasRequested": v[3]}

    def on_advance_time_step(self):
        """onAdvanceTimeStep(): returns the projection's diagnostics."""
        d = _lib.Diag()
        _lib.check(_lib.load().ff_twophase2_step(self.handle, C.byref(d)))
        self.diagnostics = {"converged": bool(d.converged), "rejected": bool(d.rejected),
                            "iterations": d.iterations, "stoppedBy": STOP_REASONS.get(d.stopped_by, "none"),
                            "residual": d.residual}
        return self.diagnostics

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().ff_twophase2_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def create_grid_two_phase_flip_solver2(**options):
    return GridTwoPhaseFlipSolver2(**options)


def compute_two_phase_box_seed3(domain_min, domain_max, grid_spacing, liquid_min, liquid_max,
                                particles_per_cell_axis=2, jitter=0.2, random_seed=DEFAULT_JITTER_SEED):
    """The whole domain seeded with k^3 jittered particles per cell
    (computeFlipBoxSeed3's mulberry32 jitter), each tagged liquid (phase 1)
    inside the box [liquid_min, liquid_max) and gas (phase 0) elsewhere; the
    3D counterpart of computeTwoPhaseBoxSeed (grid_two_phase_flip_solver2.js:
    397-477)."""
    seed = compute_flip_box_seed3(domain_min, domain_max, *grid_spacing,
                                  particles_per_cell_axis=particles_per_cell_axis, jitter=jitter,
                                  random_seed=random_seed)
    p = seed["positionsArray"].reshape(-1, 3)
    lo, hi = np.asarray(liquid_min, np.float32), np.asarray(liquid_max, np.float32)
    liquid = np.all((p >= lo) & (p < hi), axis=1)
    ph = np.where(liquid, PHASE_LIQUID, PHASE_GAS).astype(np.float32)
    return {"count": seed["count"], "positionsArray": seed["positionsArray"],
            "velocitiesArray": seed["velocitiesArray"], "phasesArray": ph, "liquidCount": int(liquid.sum()),
            "gasCount": int((~liquid).sum())}


class GridTwoPhaseFlipSolver3:
    """A 3D two-phase FLIP solver (no reference counterpart: the reference's
    two-phase solver is 2D): the stages of createGridTwoPhaseFlipSolver2 on
    a full grid, with the same option names.  ``velocity_grid`` is a
    FaceCenteredGrid3; positions and velocities are (x, y, z) triples.  The
    pressure pin defaults to the top centre cell (nx/2, ny-1, nz/2)."""

    STAGES = GridTwoPhaseFlipSolver2.STAGES

    def __init__(self, velocity_grid=None, max_particles=None, dt=None, gravity=(0.0, -9.81, 0.0),
                 liquid_density=1.0, gas_density=0.01, mixing=0.0, fade=0.0, concentration_atomic_scale=4096.0,
                 flip_ratio=0.97, gas_flip_ratio=0.90, velocity_damping=0.02, p2g_atomic_scale=65536.0,
                 weight_epsilon=1e-4, closed_domain_boundary_flag=63, collider=None, collider_push_thresh=0.0,
                 collider_push_shift=0.0, pressure_pin="topCenter", resample=None, pressure=None, max_substeps=32):
        if velocity_grid is None:
            raise ValueError("GridTwoPhaseFlipSolver3: velocityGrid is required.")
        if not max_particles:
            raise ValueError("GridTwoPhaseFlipSolver3: maxParticles is required.")
        if not (liquid_density > 0 and gas_density > 0):
            raise ValueError("GridTwoPhaseFlipSolver3: both densities must be > 0.")
        g = velocity_grid
        res = tuple(g.resolution)
        if pressure_pin == "topCenter":
            pin = (res[0] // 2, res[1] - 1, res[2] // 2)
        elif pressure_pin is None:
            pin = (-1, -1, -1)
        else:
            pin = tuple(int(x) for x in pressure_pin)
        lib = _lib.load()
        d = _lib.TwoPhase3Desc()
        lib.ff_twophase3_desc_default(C.byref(d), (C.c_int * 3)(*res), (C.c_double * 3)(*g.grid_spacing),
                                      int(max_particles), float(dt))
        d.origin[:] = [float(x) for x in g.origin]
        d.gravity[:] = [float(x) for x in gravity]
        d.ambient_density, d.component_density = float(gas_density), float(liquid_density)
        d.mixing, d.fade = float(mixing), float(fade)
        d.concentration_atomic_scale = float(concentration_atomic_scale)
        d.flip_ratio, d.gas_flip_ratio = float(flip_ratio), float(gas_flip_ratio)
        d.velocity_damping = float(velocity_damping)
        d.p2g_atomic_scale, d.weight_epsilon = float(p2g_atomic_scale), float(weight_epsilon)
        d.closed_flags = int(closed_domain_boundary_flag)
        d.collider_push_thresh, d.collider_push_shift = float(collider_push_thresh), float(collider_push_shift)
        d.pin_cell[:] = list(pin)
        d.max_substeps = int(max_substeps)
        rs = resample or {}
        d.resample_enabled = int(bool(rs.get("enabled", True)))
        d.min_particles_per_cell = int(rs.get("minParticlesPerCell", 3))
        d.max_particles_per_cell = int(rs.get("maxParticlesPerCell", 8))
        p = pressure or {}
        mg = p.get("multigrid", {})
        pd = d.pressure
        pd.preconditioner = PRECONDITIONERS[p.get("preconditioner", "multigrid")]
        pd.tolerance = float(p.get("tolerance", pd.tolerance))
        pd.mg_levels = int(mg.get("numberOfLevels", pd.mg_levels))
        pd.mg_down = int(mg.get("numberOfSmoothingIterationsDown", pd.mg_down))
        pd.mg_up = int(mg.get("numberOfSmoothingIterationsUp", pd.mg_up))
        pd.mg_coarsest = int(mg.get("numberOfCoarsestIterations", pd.mg_coarsest))
        pd.mg_coarse_mode = 1 if mg.get("coarseSolve", "sweeps") == "direct" else 0
        if "maxIterations" in p:
            pd.max_iterations = int(p["maxIterations"])
        if "maxPlausiblePressure" in p:
            pd.max_plausible_pressure = float(p["maxPlausiblePressure"])
        if p.get("precision", "fp32") != "fp32":
            pd.iterate = 1
        self.desc = d
        self.max_particles = int(max_particles)
        self.velocity_grid = g
        self.handle = C.c_void_p()
        _lib.check(lib.ff_twophase3_create(context().handle, C.byref(d), g.data_u.handle, g.data_v.handle,
                                           g.data_w.handle, C.byref(self.handle)))
        self.collider = collider
        if collider is not None:
            _lib.check(lib.ff_twophase2_set_collider(self.handle, collider.phi.handle))
        hs = [C.c_void_p() for _ in range(7)]
        _lib.check(lib.ff_twophase3_fields(self.handle, *[C.byref(x) for x in hs]))
        ctx = context()
        self.phase = BorrowedField(hs[0], ctx)
        self.concentration = self.phase
        self.liquid_fraction = BorrowedField(hs[1], ctx)
        self.density = BorrowedField(hs[2], ctx)
        self.beta_u = BorrowedField(hs[3], ctx)
        self.beta_v = BorrowedField(hs[4], ctx)
        self.beta_w = BorrowedField(hs[5], ctx)
        self.pressure_solver = GridPressureSolver3.borrowed(hs[6].value, self, res, g.grid_spacing, g.origin)
        self.pressure = self.pressure_solver.pressure
        self.diagnostics = {}

    def set_particles(self, positions=None, velocities=None, phases=None, count=None):
        """Upload (x, y, z) positions, velocities and phases; `count` (default
        the number of positions) becomes the live particle count."""
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32).ravel()
                for a in (positions, velocities, phases)]
        n = count if count is not None else (arrs[0].size // 3 if arrs[0] is not None else arrs[2].size)
        ptr = lambda a: a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None
        _lib.check(_lib.load().ff_twophase3_set_particles(self.handle, int(n), *[ptr(a) for a in arrs]))
        _lib.check(_lib.load().ff_twophase2_set_count(self.handle, int(n)))

    def get_particles(self, n=None):
        n = self.max_particles if n is None else int(n)
        pos, vel, ph = np.empty(3 * n, np.float32), np.empty(3 * n, np.float32), np.empty(n, np.float32)
        ptr = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        _lib.check(_lib.load().ff_twophase3_get_particles(self.handle, n, ptr(pos), ptr(vel), ptr(ph)))
        return pos, vel, ph

    def cell_counts(self):
        nc = int(np.prod(self.velocity_grid.resolution))
        cnt, acc = np.empty(nc, np.int32), np.empty(nc, np.int32)
        _lib.check(_lib.load().ff_twophase3_cell_counts(self.handle, cnt.ctypes.data_as(C.POINTER(C.c_int32)),
                                                         acc.ctypes.data_as(C.POINTER(C.c_int32))))
        return cnt, acc

    def stage(self, name):
        _lib.check(_lib.load().ff_twophase2_stage(self.handle, self.STAGES[name]))

    def resample_stats(self):
        v = (C.c_int64 * 4)()
        _lib.check(_lib.load().ff_twophase2_resample_stats(self.handle, v))
        return {"liquidDonors": v[0], "liquidRequested": v[1], "gasDonors": v[2], "gasRequested": v[3]}

    def on_advance_time_step(self):
        """One step; returns the projection's diagnostics."""
        d = _lib.Diag()
        _lib.check(_lib.load().ff_twophase2_step(self.handle, C.byref(d)))
        self.diagnostics = {"converged": bool(d.converged), "rejected": bool(d.rejected),
                            "iterations": d.iterations, "stoppedBy": STOP_REASONS.get(d.stopped_by, "none"),
                            "residual": d.residual, "bNorm": d.b_norm}
        return self.diagnostics

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().ff_twophase2_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def create_grid_two_phase_flip_solver3(**options):
    return GridTwoPhaseFlipSolver3(**options)


class GridSolver3:
    """createGridSolver3({velocityGrid, gridSpacing, origin, force, dirichlet,
    collider, inflows, closedDomainBoundaryFlag, dt, advection, pressure})
    (grid_solver3.js:24-149) with a uniform force vector and an explicit
    viscosity `nu` (the reference's computeViscosity is a no-op, :104; nu = 0
    keeps it so).  onAdvanceTimeStep runs external forces, viscosity, the
    projection and the advection, each followed by constrainVelocity, as
    the reference's default stages do (:112-140)."""

    def __init__(self, velocity_grid=None, force=None, dirichlet=None, collider=None, inflows=None,
                 closed_domain_boundary_flag=None, dt=None, advection=None, pressure=None, nu=0.0):
        if velocity_grid is None:
            raise ValueError("createGridSolver3: options.velocityGrid is required.")
        g = velocity_grid
        self.velocity_grid, self.dt, self.nu = g, dt, float(nu)
        self.force = tuple(float(x) for x in force) if force is not None else None
        pressure = dict(pressure or {})
        cw = pressure.pop("collider_weights", None)
        if collider is not None and cw is None:
            cw = collider.compute_face_weights(g.resolution, g.grid_spacing, g.origin)
        self.collider_face_weights = cw
        self.boundary_solver = GridBlockedBoundaryConditionSolver3(g, g.resolution, g.grid_spacing, g.origin,
                                                                   collider, inflows, cw)
        if closed_domain_boundary_flag is not None:
            self.boundary_solver.closed_domain_boundary_flag = closed_domain_boundary_flag
        self.velocity_prev = FaceCenteredGrid3(g.resolution, g.grid_spacing, g.origin)
        self._scratch = FaceCenteredGrid3(g.resolution, g.grid_spacing, g.origin)
        self.pressure_solver = create_grid_pressure_solver3(g.resolution, g.grid_spacing, g.origin,
                                                            dirichlet=dirichlet, collider_weights=cw, **pressure)
        self._project = self.pressure_solver.project(g, g)
        adv = dict(advection or {})
        self.advection_solver = SemiLagrangianAdvectionSolver3(self.velocity_prev, collider, dt, **adv)
        self._advect = self.advection_solver.advect_face_centered3(self.velocity_prev, g)
        self.pressure = self.pressure_solver.pressure

    def _copy(self, dst, src):
        lib = _lib.load()
        for a, b in ((dst.data_u, src.data_u), (dst.data_v, src.data_v), (dst.data_w, src.data_w)):
            _lib.check(lib.ff_field_copy(a.handle, b.handle))

    def on_advance_time_step(self, time_step_in_seconds=None):
        dt = float(self.dt if time_step_in_seconds is None else time_step_in_seconds)
        g = self.velocity_grid
        lib = _lib.load()
        if self.force is not None:
            _lib.check(lib.ff_velocity3_add_force(context().handle, (C.c_int * 3)(*g.resolution), g.data_u.handle,
                                                  g.data_v.handle, g.data_w.handle, *self.force, dt))
            self.boundary_solver.constrain_velocity()
        if self.nu > 0:
            apply_viscosity3(g, self._scratch, self.nu, dt)
            self._copy(g, self._scratch)
        diag = self._project()
        self.boundary_solver.constrain_velocity()
        self._copy(self.velocity_prev, g)
        self.advection_solver.set_dt(dt)
        self._advect()
        self.boundary_solver.constrain_velocity()
        return diag


def create_grid_solver3(**options):
    return GridSolver3(**options)
