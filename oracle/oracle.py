"""ctypes front end of the FP64 CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline arm of bench.py
import this module, and only to check or time against it.  The product library never
loads it.  Arrays are numpy, i-fastest (Fortran order of (nx, ny, nz)),
flattened: cell (i,j,k) -> i + nx*(j + ny*k).
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_dp = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        srcs = [os.path.join(_HERE, f) for f in os.listdir(_HERE) if f.endswith((".c", ".h"))]
        if not os.path.exists(path) or any(os.path.getmtime(s) > os.path.getmtime(path) for s in srcs):
            build()
        _LIB = C.CDLL(path)
        _declare(_LIB)
    return _LIB


class MgOpts(C.Structure):
    _fields_ = [("levels", C.c_int), ("down", C.c_int), ("up", C.c_int),
                ("coarsest", C.c_int), ("final_iters", C.c_int), ("sor", C.c_double),
                ("coarsen_mask", C.c_int), ("coarsen_weights", C.c_int),
                ("coarse_direct", C.c_int), ("store_bf16", C.c_int)]


class PcgResult(C.Structure):
    _fields_ = [("converged", C.c_int), ("iterations", C.c_int), ("stop_code", C.c_int),
                ("stopped_by", C.c_int), ("rr", C.c_double), ("bb", C.c_double),
                ("residual", C.c_double)]


def _declare(L):
    I, D = C.c_int, C.c_double
    L.orc_laplacian.argtypes = [I, I, I, D, D, D, _dp, _u8p, _dp, _dp, _dp, _dp]
    L.orc_laplacian_diag.argtypes = [I, I, I, D, D, D, _u8p, _dp, _dp, _dp, _dp]
    L.orc_cpuref_apply.argtypes = [I, I, D, D, _dp, _u8p, _dp, I]
    L.orc_cpuref_cg.argtypes = [I, I, D, D, _dp, _u8p, _dp, _dp, I, I, I, I, _dp]
    L.orc_cpuref_cg.restype = I
    L.orc_mg_create.argtypes = [I, I, I, D, D, D, C.POINTER(MgOpts)]
    L.orc_mg_create.restype = C.c_void_p
    L.orc_mg_destroy.argtypes = [C.c_void_p]
    L.orc_mg_set_system.argtypes = [C.c_void_p, _u8p, _u8p, _dp, _dp, _dp]
    L.orc_mg_refresh.argtypes = [C.c_void_p]
    L.orc_mg_apply.argtypes = [C.c_void_p, _dp, _dp]
    L.orc_mg_level_shape.argtypes = [C.c_void_p, I, C.POINTER(C.c_int)]
    L.orc_mg_level_mask.argtypes = [C.c_void_p, I, _u8p]
    L.orc_mg_level_weights.argtypes = [C.c_void_p, I, I, _dp]
    L.orc_restrict.argtypes = [I, I, I, _dp, _u8p, _u8p, _dp]
    L.orc_prolong_add.argtypes = [I, I, I, _dp, _u8p, _dp]
    L.orc_pcg_solve.argtypes = [I, I, I, D, D, D, _u8p, _dp, _dp, _dp, C.c_void_p, I, _dp,
                                _dp, D, I, I, C.POINTER(C.c_int), C.POINTER(PcgResult)]
    L.orc_pcg_solve.restype = I
    L.orc_dirichlet_fields.argtypes = [I, I, I, _u8p, _dp, _dp, _dp, _dp, _u8p, _dp, _u8p]
    L.orc_build_system.argtypes = [I, I, I, D, D, D, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                   _dp, _u8p, _dp, _dp, _dp]
    L.orc_correct.argtypes = [I, I, I, D, D, D, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                              _dp, _dp, _dp, _dp]
    L.orc_count_bad.argtypes = [I, _dp, D]
    L.orc_count_bad.restype = I
    L.orc_round_bf16.argtypes = [C.c_float]
    L.orc_round_bf16.restype = C.c_float
    L.orc_fraction_inside.argtypes = [D, D, D, D]
    L.orc_fraction_inside.restype = D
    fp = C.POINTER(C.c_float)
    L.orc_collider_bake.argtypes = [_dp, I, I, I, I, I, D, D, D, D, D, D, fp, fp, fp, fp]
    ip, F, L64 = C.POINTER(C.c_int), C.c_float, C.c_int64
    L.orc_trace.argtypes = [ip, fp, fp, fp, fp, fp, fp, F, I, F, L64, fp, fp]
    L.orc_advect_faces.argtypes = [ip, fp, fp, fp, fp, fp, fp, F, I, I, fp, fp, fp]
    L.orc_advect_scalar.argtypes = [ip, fp, fp, fp, fp, fp, fp, F, I, I, fp, fp]
    L.orc_constrain_velocity.argtypes = [ip, fp, fp, fp, fp, fp, fp, fp, fp, fp, I, I, fp, fp, ip, I]
    L.orc_viscosity.argtypes = [ip, fp, fp, fp, fp, F, F, fp, fp, fp]
    dp, i32p, u8p = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_uint8)
    L.orc_outflow_velocity.argtypes = [ip, fp, fp, fp, fp, fp, F, I, fp, ip, fp, fp]
    L.orc_outflow_clear_scalar.argtypes = [ip, fp, fp, fp, I, fp, ip, fp, fp]
    L.orc_outflow_dirichlet.argtypes = [ip, fp, fp, F, I, fp, ip, fp, fp, u8p, fp]
    L.orc_jitter_random.argtypes = [C.c_uint32, I, dp]
    L.orc_flip_box_seed.argtypes = [dp, dp, dp, I, D, C.c_uint32, fp, L64]
    L.orc_flip_box_seed.restype = L64
    L.orc_flip_cell_index.argtypes = [ip, fp, fp, L64, fp, C.POINTER(C.c_int64)]
    L.orc_flip_mark_fluid.argtypes = [ip, fp, fp, L64, fp, fp]
    L.orc_flip_dirichlet.argtypes = [ip, fp, fp, fp, fp, F, I, u8p, fp]
    L.orc_flip_p2g.argtypes = [ip, fp, fp, L64, fp, fp, F, F, fp, fp, fp, i32p, i32p, i32p]
    L.orc_flip_fluid_adjacent.argtypes = [ip, fp, i32p, i32p, i32p]
    L.orc_flip_g2p.argtypes = [ip, fp, fp, L64, fp, fp, fp, fp, fp, fp, fp, fp, F, F]
    L.orc_flip_concentration_grid.argtypes = [ip, fp, fp, L64, fp, fp, F, fp, I, F, F, fp, fp, fp, fp, fp]
    L.orc_flip_reduced_gravity.argtypes = [ip, fp, fp, fp, fp, fp, fp, fp, F, F, fp, fp, fp]
    L.orc_flip_mix_fade.argtypes = [ip, fp, fp, L64, fp, fp, F, F, fp]
    L.orc_flip_advect.argtypes = [ip, fp, fp, fp, fp, fp, fp, F, I, L64, fp, fp, F, F]
    L.orc_tp3_counts.argtypes = [ip, fp, fp, L64, fp, fp, F, i32p, i32p]
    L.orc_tp3_g2p.argtypes = [ip, fp, fp, L64, fp, fp, fp, fp, fp, fp, fp, fp, fp, F, F, F]
    L.orc_tp3_resample.argtypes = [ip, fp, fp, L64, I, fp, fp, fp, fp, fp, fp, i32p, i32p, F, I, I,
                                   C.POINTER(C.c_int64)]
    L.orc_tp3_resample.restype = L64
    L.orc_tp_density.argtypes = [ip, fp, fp, L64, fp, fp, F, F, F, i32p, i32p, fp, fp, fp, fp]
    L.orc_tp_g2p.argtypes = [ip, fp, fp, L64, fp, fp, fp, fp, fp, fp, fp, F, F, F]
    L.orc_tp_mix.argtypes = [ip, fp, fp, L64, fp, fp, F, F, fp]
    L.orc_tp_resample.argtypes = [ip, fp, fp, L64, I, fp, fp, fp, fp, fp, i32p, i32p, F, I, I,
                                  C.POINTER(C.c_int64)]
    L.orc_tp_resample.restype = L64
    L.orc_flip_resample.argtypes = [ip, fp, fp, L64, fp, fp, fp, fp, fp, I, I]
    L.orc_flip_resample.restype = L64


def _shape_row(s):
    row = [0.0] * 13
    row[0] = 0.0 if s["type"] == "sphere" else 1.0
    row[1:4] = [float(v) for v in s["center"]]
    if s["type"] == "sphere":
        row[4] = float(s["radius"])
    else:
        row[5:8] = [float(v) for v in s["halfExtents"]]
        rot = s.get("rotation")
        if rot:
            row[8] = 1.0
            row[9:12] = [float(v) for v in rot["axis"]]
            row[12] = float(rot["angle"])
    return row


def collider_bake(shapes, shape, h, origin=(0.0, 0.0, 0.0), invert=False):
    """createSDFStaticCollider3.addShapes + computeFaceWeights restated:
    returns (phi, wu, wv, ww) as float32 arrays."""
    nx, ny, nz = shape
    rows = np.array([_shape_row(s) for s in shapes] or [[0.0] * 13], np.float64).ravel()
    phi = np.empty(nx * ny * nz, np.float32)
    wu = np.empty((nx + 1) * ny * nz, np.float32)
    wv = np.empty(nx * (ny + 1) * nz, np.float32)
    ww = np.empty(nx * ny * (nz + 1), np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    lib().orc_collider_bake(rows.ctypes.data_as(_dp), len(shapes), int(invert), nx, ny, nz,
                            *h, *origin, fp(phi), fp(wu), fp(wv), fp(ww))
    return phi, wu, wv, ww


def _d(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _u8(a):
    if a is None:
        return None
    assert a.dtype == np.uint8 and a.flags.c_contiguous
    return a.ctypes.data_as(_u8p)


def f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64).ravel()


def u8(a):
    return None if a is None else np.ascontiguousarray(np.asarray(a) != 0, dtype=np.uint8).ravel()


def shape3(shape):
    return (shape[0], shape[1], shape[2] if len(shape) > 2 else 1)


def spacing3(h):
    h = list(h) if hasattr(h, "__len__") else [h, h, h]
    return (h[0], h[1], h[2] if len(h) > 2 else 1.0)


def laplacian(shape, h, x, mask=None, weights=None):
    nx, ny, nz = shape3(shape)
    hx, hy, hz = spacing3(h)
    x = f64(x)
    out = np.empty_like(x)
    wu, wv, ww = (f64(w) for w in weights) if weights is not None else (None, None, None)
    if weights is not None and nz == 1:
        ww = None
    lib().orc_laplacian(nx, ny, nz, hx, hy, hz, _d(x), _u8(u8(mask)), _d(wu), _d(wv), _d(ww), _d(out))
    return out


def laplacian_diag(shape, h, mask=None, weights=None):
    nx, ny, nz = shape3(shape)
    hx, hy, hz = spacing3(h)
    out = np.empty(nx * ny * nz)
    wu, wv, ww = (f64(w) for w in weights) if weights is not None else (None, None, None)
    lib().orc_laplacian_diag(nx, ny, nz, hx, hy, hz, _u8(u8(mask)), _d(wu), _d(wv), _d(ww), _d(out))
    return out


def cpuref_apply(shape, h, x, pinned, round_f32=False):
    nx, ny = shape[0], shape[1]
    x = f64(x)
    out = np.empty_like(x)
    lib().orc_cpuref_apply(nx, ny, h[0], h[1], _d(x), _u8(u8(pinned)), _d(out), int(round_f32))
    return out


def cpuref_cg(shape, h, b, pinned, x0=None, round_f32=False, dot_kind=0, max_iter=40000,
              recompute_every=0):
    nx, ny = shape[0], shape[1]
    b = f64(b)
    xo = np.empty_like(b)
    rel = C.c_double()
    it = lib().orc_cpuref_cg(nx, ny, h[0], h[1], _d(b), _u8(u8(pinned)), _d(f64(x0)), _d(xo),
                             int(round_f32), dot_kind, max_iter, recompute_every, C.byref(rel))
    return it, rel.value, xo


def mg_opts(levels=1, down=2, up=2, coarsest=20, final_iters=2, sor=1.0, coarsen_mask=True,
            coarsen_weights=True, coarse_direct=False, store_bf16=False):
    return MgOpts(levels, down, up, coarsest, final_iters, sor, int(coarsen_mask),
                  int(coarsen_weights), int(coarse_direct),
                  7 if store_bf16 is True else int(store_bf16))


class Multigrid:
    """createMultigridPreconditioner (multigrid.js:1213-1735) restated in FP64."""

    def __init__(self, shape, h, mask=None, vent=None, weights=None, **opts):
        self.shape = shape3(shape)
        self.h = spacing3(h)
        self._o = mg_opts(**opts)
        self._p = lib().orc_mg_create(*self.shape, *self.h, C.byref(self._o))
        if not self._p:
            raise ValueError("multigrid: shape not divisible by 2^(levels-1)")
        self._keep = []
        self.set_system(mask, vent, weights)

    def set_system(self, mask=None, vent=None, weights=None):
        m, v = u8(mask), u8(vent)
        if weights is not None:
            wu, wv = f64(weights[0]), f64(weights[1])
            ww = f64(weights[2]) if self.shape[2] > 1 else None
        else:
            wu = wv = ww = None
        self._keep = [m, v, wu, wv, ww]
        lib().orc_mg_set_system(self._p, _u8(m), _u8(v), _d(wu), _d(wv), _d(ww))
        lib().orc_mg_refresh(self._p)

    def apply(self, r):
        r = f64(r)
        z = np.empty_like(r)
        lib().orc_mg_apply(self._p, _d(r), _d(z))
        return z

    def level_shape(self, level):
        s = (C.c_int * 3)()
        lib().orc_mg_level_shape(self._p, level, s)
        return tuple(s)

    def level_mask(self, level):
        nx, ny, nz = self.level_shape(level)
        out = np.empty(nx * ny * nz, np.uint8)
        lib().orc_mg_level_mask(self._p, level, _u8(out))
        return out

    def level_weights(self, level, axis):
        nx, ny, nz = self.level_shape(level)
        n = (nx + (axis == 0)) * (ny + (axis == 1)) * (nz + (axis == 2))
        out = np.empty(n)
        lib().orc_mg_level_weights(self._p, level, axis, _d(out))
        return out

    def __del__(self):
        try:
            if self._p:
                lib().orc_mg_destroy(self._p)
                self._p = None
        except Exception:
            pass


def restrict(fine_shape, fine, fine_mask=None, coarse_mask=None):
    nx, ny, nz = shape3(fine_shape)
    cn = (nx // 2) * (ny // 2) * (nz // 2 if nz > 1 else 1)
    out = np.empty(cn)
    lib().orc_restrict(nx, ny, nz, _d(f64(fine)), _u8(u8(fine_mask)), _u8(u8(coarse_mask)), _d(out))
    return out


def prolong_add(fine_shape, coarse, fine, fine_mask=None):
    nx, ny, nz = shape3(fine_shape)
    fine = f64(fine).copy()
    lib().orc_prolong_add(nx, ny, nz, _d(f64(coarse)), _u8(u8(fine_mask)), _d(fine))
    return fine


PRE = {"multigrid": 0, "jacobi": 1, "none": 2}
STOP_NAMES = {0: "none", 1: "degenerate-pAp", 2: "pAp-growth", 3: "alpha-magnitude",
              4: "degenerate-oldRZ", 5: "converged", 6: "residual-growing"}


def pcg_solve(shape, h, b, x0=None, mask=None, weights=None, mg=None, preconditioner="multigrid",
              tol=1e-6, max_iter=100, relative=True, last_iters=4):
    """GPU-resident chunked PCG (linalg.js:1651-1911) in FP64.  Returns
    (x, result dict, last_iters)."""
    nx, ny, nz = shape3(shape)
    hx, hy, hz = spacing3(h)
    b = f64(b)
    x = np.zeros_like(b) if x0 is None else f64(x0).copy()
    m = u8(mask)
    if weights is not None:
        wu, wv = f64(weights[0]), f64(weights[1])
        ww = f64(weights[2]) if nz > 1 else None
    else:
        wu = wv = ww = None
    last = C.c_int(last_iters)
    res = PcgResult()
    lib().orc_pcg_solve(nx, ny, nz, hx, hy, hz, _u8(m), _d(wu), _d(wv), _d(ww),
                        mg._p if mg is not None else None, PRE[preconditioner], _d(b), _d(x),
                        tol, max_iter, int(relative), C.byref(last), C.byref(res))
    out = dict(converged=bool(res.converged), iterations=res.iterations,
               stop_code=res.stop_code, stopped_by=STOP_NAMES[res.stopped_by],
               rr=res.rr, bb=res.bb, residual=res.residual)
    return x, out, last.value


def dirichlet_fields(shape, active=None, target=None, collider_weights=None):
    nx, ny, nz = shape3(shape)
    n = nx * ny * nz
    mask, vent, tgt = np.empty(n, np.uint8), np.empty(n, np.uint8), np.empty(n)
    cw = [f64(w) for w in collider_weights] if collider_weights is not None else [None] * 3
    if nz == 1:
        cw[2] = None
    lib().orc_dirichlet_fields(nx, ny, nz, _u8(u8(active)), _d(f64(target)), _d(cw[0]), _d(cw[1]),
                               _d(cw[2]), _u8(mask), _d(tgt), _u8(vent))
    return mask, tgt, vent


def build_system(shape, h, u, v, w, collider_weights=None, face_weights=None, mask=None,
                 target=None, p=None):
    nx, ny, nz = shape3(shape)
    hx, hy, hz = spacing3(h)
    n = nx * ny * nz
    b = np.empty(n)
    p = np.zeros(n) if p is None else f64(p).copy()
    cw = [f64(a) for a in collider_weights] if collider_weights is not None else [None] * 3
    fw = [f64(a) for a in face_weights] if face_weights is not None else [None] * 3
    w = f64(w) if w is not None else None
    lib().orc_build_system(nx, ny, nz, hx, hy, hz, _d(f64(u)), _d(f64(v)), _d(w),
                           _d(cw[0]), _d(cw[1]), _d(cw[2]), _d(fw[0]), _d(fw[1]), _d(fw[2]),
                           _u8(u8(mask)), _d(f64(target) if target is not None else np.zeros(n)),
                           _d(b), _d(p))
    return b, p


def correct(shape, h, p, u, v, w, face_weights=None, collider_weights=None):
    nx, ny, nz = shape3(shape)
    hx, hy, hz = spacing3(h)
    u, v = f64(u), f64(v)
    w = f64(w) if w is not None else np.zeros(1)
    uo, vo, wo = u.copy(), v.copy(), w.copy()
    cw = [f64(a) for a in collider_weights] if collider_weights is not None else [None] * 3
    fw = [f64(a) for a in face_weights] if face_weights is not None else [None] * 3
    lib().orc_correct(nx, ny, nz, hx, hy, hz, _d(f64(p)), _d(fw[0]), _d(fw[1]), _d(fw[2]),
                      _d(cw[0]), _d(cw[1]), _d(cw[2]), _d(u), _d(v), _d(w), _d(uo), _d(vo), _d(wo))
    return uo, vo, wo


def count_bad(p, max_plausible=1e6):
    p = f64(p)
    return lib().orc_count_bad(p.size, _d(p), max_plausible)


def round_bf16(a):
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


# ---------------------------------------------- FP32 grid-velocity kernels --
# advection_solver3.js, grid_blocked_boundary_condition_solver3.js and the
# explicit viscosity, restated in C floats (ff_oracle_grid.c).
def _f32(a):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float32).ravel()
    return a


def _fptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def _geom(shape, h, origin):
    res = (C.c_int * 3)(*shape)
    hh = (C.c_float * 3)(*[float(x) for x in h])
    oo = (C.c_float * 3)(*[float(x) for x in origin])
    return res, hh, oo


def trace(shape, h, origin, u, v, w, phi, points, dt, direction=1, max_substeps=32):
    u, v, w, phi = _f32(u), _f32(v), _f32(w), _f32(phi)
    p = _f32(points)
    out = np.empty_like(p)
    res, hh, oo = _geom(shape, h, origin)
    lib().orc_trace(res, hh, oo, _fptr(u), _fptr(v), _fptr(w), _fptr(phi), float(dt), int(max_substeps),
                    float(-1.0 if direction == -1 else 1.0), p.size // 3, _fptr(p), _fptr(out))
    return out


def advect_faces(shape, h, origin, u, v, w, phi, dt, order=1, max_substeps=32, out=None):
    """advectFaceCentered3 of (u, v, w) through itself; `out` (u, v, w)
    gives the values kept on faces inside the collider (default: the input)."""
    u, v, w, phi = _f32(u), _f32(v), _f32(w), _f32(phi)
    uo, vo, wo = (x.copy() for x in (out if out is not None else (u, v, w)))
    uo, vo, wo = _f32(uo), _f32(vo), _f32(wo)
    res, hh, oo = _geom(shape, h, origin)
    lib().orc_advect_faces(res, hh, oo, _fptr(u), _fptr(v), _fptr(w), _fptr(phi), float(dt), int(max_substeps),
                           int(order), _fptr(uo), _fptr(vo), _fptr(wo))
    return uo, vo, wo


def advect_scalar(shape, h, origin, u, v, w, phi, s, dt, order=1, max_substeps=32, out=None):
    u, v, w, phi, s = _f32(u), _f32(v), _f32(w), _f32(phi), _f32(s)
    so = _f32(out.copy() if out is not None else s.copy())
    res, hh, oo = _geom(shape, h, origin)
    lib().orc_advect_scalar(res, hh, oo, _fptr(u), _fptr(v), _fptr(w), _fptr(phi), float(dt), int(max_substeps),
                            int(order), _fptr(s), _fptr(so))
    return so


def constrain_velocity(shape, h, origin, u, v, w, phi=None, face_weights=None, closed=63, inflows=(), depth=5):
    """constrainVelocity(depth); inflows: list of (phi, (vx, vy, vz), mode)."""
    u, v, w = (_f32(x).copy() for x in (u, v, w))
    phi = _f32(phi)
    fw = [None, None, None] if face_weights is None else [_f32(x) for x in face_weights]
    n_in = len(inflows)
    ncell = shape[0] * shape[1] * shape[2]
    phis = np.concatenate([_f32(q[0]) for q in inflows]) if n_in else np.zeros(1, np.float32)
    vel = np.array([c for q in inflows for c in q[1]] or [0.0], np.float32)
    modes = (C.c_int * max(1, n_in))(*[int(q[2]) for q in inflows])
    assert phis.size == max(1, n_in * ncell) or n_in == 0
    res, hh, oo = _geom(shape, h, origin)
    lib().orc_constrain_velocity(res, hh, oo, _fptr(u), _fptr(v), _fptr(w), _fptr(phi), _fptr(fw[0]),
                                 _fptr(fw[1]), _fptr(fw[2]), int(closed), n_in, _fptr(phis), _fptr(vel), modes,
                                 int(depth))
    return u, v, w


def viscosity(shape, h, u, v, w, nu, dt):
    u, v, w = _f32(u), _f32(v), _f32(w)
    uo, vo, wo = np.empty_like(u), np.empty_like(v), np.empty_like(w)
    res = (C.c_int * 3)(*shape)
    hh = (C.c_float * 3)(*[float(x) for x in h])
    lib().orc_viscosity(res, hh, _fptr(u), _fptr(v), _fptr(w), float(nu), float(dt), _fptr(uo), _fptr(vo),
                        _fptr(wo))
    return uo, vo, wo


def _outflows(outflows):
    """outflows: list of (phi, resolution, spacing, origin) -> C arguments"""
    n = len(outflows)
    phi = np.concatenate([_f32(q[0]) for q in outflows]) if n else np.zeros(1, np.float32)
    pres = (C.c_int * max(3, 3 * n))(*[int(x) for q in outflows for x in q[1]])
    ph = (C.c_float * max(3, 3 * n))(*[float(x) for q in outflows for x in q[2]])
    po = (C.c_float * max(3, 3 * n))(*[float(x) for q in outflows for x in q[3]])
    return n, phi, pres, ph, po


def outflow_velocity(shape, h, origin, u, v, w, dt, outflows):
    """applyOutflowVelocityBC (grid_outflow_solver3.js:98-170)"""
    u, v, w = (_f32(x).copy() for x in (u, v, w))
    res, hh, oo = _geom(shape, h, origin)
    n, phi, pres, ph, po = _outflows(outflows)
    lib().orc_outflow_velocity(res, hh, oo, _fptr(u), _fptr(v), _fptr(w), float(dt), n, _fptr(phi), pres, ph, po)
    return u, v, w


def outflow_clear_scalar(shape, h, origin, data, outflows):
    data = _f32(data).copy()
    res, hh, oo = _geom(shape, h, origin)
    n, phi, pres, ph, po = _outflows(outflows)
    lib().orc_outflow_clear_scalar(res, hh, oo, _fptr(data), n, _fptr(phi), pres, ph, po)
    return data


def outflow_dirichlet(shape, h, origin, outflows, target=0.0):
    res, hh, oo = _geom(shape, h, origin)
    n, phi, pres, ph, po = _outflows(outflows)
    nc = int(np.prod(shape))
    active, tgt = np.empty(nc, np.uint8), np.empty(nc, np.float32)
    lib().orc_outflow_dirichlet(res, hh, oo, float(target), n, _fptr(phi), pres, ph, po,
                                active.ctypes.data_as(C.POINTER(C.c_uint8)), _fptr(tgt))
    return active, tgt


# ------------------------------------------------------------------- FLIP --
# grid_flip_solver3.js stages and jitter_random.js, restated in
# ff_oracle_flip.c (FP32 stages, double-precision seeding).
def jitter_random(seed, n):
    out = np.empty(n)
    lib().orc_jitter_random(int(seed) & 0xFFFFFFFF, n, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def flip_box_seed(box_min, box_max, h, per_axis=2, jitter=0.2, seed=0x9E3779B9):
    dd = lambda v: (C.c_double * 3)(*[float(x) for x in v])
    n = lib().orc_flip_box_seed(dd(box_min), dd(box_max), dd(h), per_axis, float(jitter), seed, None, 0)
    out = np.empty(3 * n, np.float32)
    lib().orc_flip_box_seed(dd(box_min), dd(box_max), dd(h), per_axis, float(jitter), seed, _fptr(out), n)
    return out


def _i32(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def flip_cell_index(shape, h, origin, pos):
    pos = _f32(pos)
    out = np.empty(pos.size // 3, np.int64)
    res, hh, oo = _geom(shape, h, origin)
    lib().orc_flip_cell_index(res, hh, oo, pos.size // 3, _fptr(pos), out.ctypes.data_as(C.POINTER(C.c_int64)))
    return out


def flip_mark_fluid(shape, h, origin, pos):
    pos = _f32(pos)
    mask = np.empty(shape[0] * shape[1] * shape[2], np.float32)
    res, hh, oo = _geom(shape, h, origin)
    lib().orc_flip_mark_fluid(res, hh, oo, pos.size // 3, _fptr(pos), _fptr(mask))
    return mask


def flip_dirichlet(shape, h, origin, mask, gravity, dt, reduced=True):
    n = shape[0] * shape[1] * shape[2]
    active, target = np.empty(n, np.uint8), np.empty(n, np.float32)
    res, hh, oo = _geom(shape, h, origin)
    g = (C.c_float * 3)(*[float(x) for x in gravity])
    lib().orc_flip_dirichlet(res, hh, oo, _fptr(_f32(mask)), g, float(dt), int(reduced),
                             active.ctypes.data_as(C.POINTER(C.c_uint8)), _fptr(target))
    return active, target


def _face_sizes(shape):
    nx, ny, nz = shape
    return (nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1)


def flip_p2g(shape, h, origin, pos, vel, scale=65536.0, eps=1e-4):
    pos, vel = _f32(pos), _f32(vel)
    su, sv, sw = _face_sizes(shape)
    u, v, w = np.empty(su, np.float32), np.empty(sv, np.float32), np.empty(sw, np.float32)
    vu, vv, vw = np.empty(su, np.int32), np.empty(sv, np.int32), np.empty(sw, np.int32)
    res, hh, oo = _geom(shape, h, origin)
    lib().orc_flip_p2g(res, hh, oo, pos.size // 3, _fptr(pos), _fptr(vel), float(scale), float(eps), _fptr(u),
                       _fptr(v), _fptr(w), _i32(vu), _i32(vv), _i32(vw))
    return (u, v, w), (vu, vv, vw)


def flip_fluid_adjacent(shape, mask):
    su, sv, sw = _face_sizes(shape)
    au, av, aw = np.empty(su, np.int32), np.empty(sv, np.int32), np.empty(sw, np.int32)
    lib().orc_flip_fluid_adjacent((C.c_int * 3)(*shape), _fptr(_f32(mask)), _i32(au), _i32(av), _i32(aw))
    return au, av, aw


def flip_g2p(shape, h, origin, pos, vel, new, old, flip_ratio=0.97, damping=0.02):
    pos, vel = _f32(pos), _f32(vel).copy()
    new, old = [_f32(x) for x in new], [_f32(x) for x in old]
    res, hh, oo = _geom(shape, h, origin)
    lib().orc_flip_g2p(res, hh, oo, pos.size // 3, _fptr(pos), _fptr(vel), *[_fptr(x) for x in new],
                       *[_fptr(x) for x in old], float(flip_ratio), float(damping))
    return vel


def flip_advect(shape, h, origin, u, v, w, phi, pos, dt, max_substeps=32, push_thresh=0.0, push_shift=0.0):
    pos = _f32(pos).copy()
    ext = (C.c_float * 3)(*[float(shape[a] * float(h[a])) for a in range(3)])
    res, hh, oo = _geom(shape, h, origin)
    lib().orc_flip_advect(res, hh, oo, _fptr(_f32(u)), _fptr(_f32(v)), _fptr(_f32(w)), _fptr(_f32(phi)),
                          float(dt), int(max_substeps), pos.size // 3, _fptr(pos), ext, float(push_thresh),
                          float(push_shift))
    return pos


def flip_concentration_grid(shape, h, origin, pos, conc, mask, cscale=4096.0, density=None):
    """density: None or (ambient, component); returns cell concentration,
    cell density and beta faces (None without the density coupling)."""
    pos, conc = _f32(pos), _f32(conc)
    n = shape[0] * shape[1] * shape[2]
    cc, rho = np.empty(n, np.float32), np.empty(n, np.float32)
    su, sv, sw = _face_sizes(shape)
    bu, bv, bw = np.empty(su, np.float32), np.empty(sv, np.float32), np.empty(sw, np.float32)
    res, hh, oo = _geom(shape, h, origin)
    r0, r1 = density if density else (0.0, 0.0)
    lib().orc_flip_concentration_grid(res, hh, oo, pos.size // 3, _fptr(pos), _fptr(conc), float(cscale),
                                      _fptr(_f32(mask)), int(density is not None), float(r0), float(r1), _fptr(cc),
                                      _fptr(rho), _fptr(bu), _fptr(bv), _fptr(bw))
    return cc, (rho if density else None), ((bu, bv, bw) if density else None)


def flip_reduced_gravity(shape, h, origin, rho, beta, gravity, dt, rref, u, v, w):
    u, v, w = (_f32(x).copy() for x in (u, v, w))
    hh = (C.c_float * 3)(*[float(x) for x in h])
    oo = (C.c_float * 3)(*[float(x) for x in origin])
    g = (C.c_float * 3)(*[float(x) for x in gravity])
    lib().orc_flip_reduced_gravity((C.c_int * 3)(*shape), hh, oo, _fptr(_f32(rho)), *[_fptr(_f32(b)) for b in beta],
                                   g, float(dt), float(rref), _fptr(u), _fptr(v), _fptr(w))
    return u, v, w


def flip_mix_fade(shape, h, origin, pos, cell_conc, conc, mixing, fade):
    conc = _f32(conc).copy()
    res, hh, oo = _geom(shape, h, origin)
    lib().orc_flip_mix_fade(res, hh, oo, _f32(pos).size // 3, _fptr(_f32(pos)), _fptr(_f32(cell_conc)),
                            float(mixing), float(fade), _fptr(conc))
    return conc


def flip_resample(shape, h, origin, pos, vel, u, v, w, min_pc=4, max_pc=8):
    """resamplePass: returns (positions, velocities, particles moved)."""
    pos, vel = _f32(pos).copy(), _f32(vel).copy()
    res, hh, oo = _geom(shape, h, origin)
    moved = lib().orc_flip_resample(res, hh, oo, pos.size // 3, _fptr(pos), _fptr(vel), _fptr(_f32(u)),
                                    _fptr(_f32(v)), _fptr(_f32(w)), int(min_pc), int(max_pc))
    return pos, vel, int(moved)


# ------------------------------------------------------- two-phase FLIP 2D --
# grid_two_phase_flip_solver2.js, restated in 2D in ff_oracle_flip.c.
def _geom2(shape, h, origin):
    return ((C.c_int * 2)(*shape), (C.c_float * 2)(*[float(x) for x in h]),
            (C.c_float * 2)(*[float(x) for x in origin]))


def tp_density(shape, h, origin, pos, phase, rho0, rho1, cscale=4096.0):
    """returns cnt, acc (int32 cells), liquidFraction, density, betaU, betaV"""
    nx, ny = shape
    pos, phase = _f32(pos), _f32(phase)
    cnt, acc = np.empty(nx * ny, np.int32), np.empty(nx * ny, np.int32)
    frac, rho = np.empty(nx * ny, np.float32), np.empty(nx * ny, np.float32)
    bu, bv = np.empty((nx + 1) * ny, np.float32), np.empty(nx * (ny + 1), np.float32)
    res, hh, oo = _geom2(shape, h, origin)
    lib().orc_tp_density(res, hh, oo, pos.size // 2, _fptr(pos), _fptr(phase), float(cscale), float(rho0),
                         float(rho1), _i32(cnt), _i32(acc), _fptr(frac), _fptr(rho), _fptr(bu), _fptr(bv))
    return cnt, acc, frac, rho, bu, bv


def tp_g2p(shape, h, origin, pos, vel, phase, new, old, flip_ratio=0.97, gas_ratio=0.9, damping=0.02):
    vel = _f32(vel).copy()
    res, hh, oo = _geom2(shape, h, origin)
    lib().orc_tp_g2p(res, hh, oo, _f32(pos).size // 2, _fptr(_f32(pos)), _fptr(vel), _fptr(_f32(phase)),
                     _fptr(_f32(new[0])), _fptr(_f32(new[1])), _fptr(_f32(old[0])), _fptr(_f32(old[1])),
                     float(flip_ratio), float(gas_ratio), float(damping))
    return vel


def tp_mix(shape, h, origin, pos, frac, phase, mixing, fade):
    phase = _f32(phase).copy()
    res, hh, oo = _geom2(shape, h, origin)
    lib().orc_tp_mix(res, hh, oo, _f32(pos).size // 2, _fptr(_f32(pos)), _fptr(_f32(frac)), float(mixing),
                     float(fade), _fptr(phase))
    return phase


def tp_resample(shape, h, origin, pos, vel, phase, u, v, cnt, acc, max_particles, min_pc=3, max_pc=8,
                cscale=4096.0):
    """returns positions, velocities, moved, stats (liquid donors, liquid
    need, gas donors, gas need)"""
    pos, vel = _f32(pos).copy(), _f32(vel).copy()
    stats = np.zeros(4, np.int64)
    res, hh, oo = _geom2(shape, h, origin)
    moved = lib().orc_tp_resample(res, hh, oo, pos.size // 2, int(max_particles), _fptr(pos), _fptr(vel),
                                  _fptr(_f32(phase)), _fptr(_f32(u)), _fptr(_f32(v)),
                                  _i32(np.ascontiguousarray(cnt, np.int32)), _i32(np.ascontiguousarray(acc, np.int32)),
                                  float(cscale), int(min_pc), int(max_pc), stats.ctypes.data_as(C.POINTER(C.c_int64)))
    return pos, vel, int(moved), stats


def tp3_counts(shape, h, origin, pos, phase, cscale=4096.0):
    """per-cell particle count and fixed-point concentration sum (int32)"""
    n = shape[0] * shape[1] * shape[2]
    cnt, acc = np.empty(n, np.int32), np.empty(n, np.int32)
    res, hh, oo = _geom(shape, h, origin)
    pos, phase = _f32(pos), _f32(phase)
    lib().orc_tp3_counts(res, hh, oo, pos.size // 3, _fptr(pos), _fptr(phase), float(cscale), _i32(cnt), _i32(acc))
    return cnt, acc


def tp3_g2p(shape, h, origin, pos, vel, phase, new, old, flip_ratio=0.97, gas_ratio=0.9, damping=0.02):
    vel = _f32(vel).copy()
    res, hh, oo = _geom(shape, h, origin)
    lib().orc_tp3_g2p(res, hh, oo, _f32(pos).size // 3, _fptr(_f32(pos)), _fptr(vel), _fptr(_f32(phase)),
                      *[_fptr(_f32(x)) for x in new], *[_fptr(_f32(x)) for x in old], float(flip_ratio),
                      float(gas_ratio), float(damping))
    return vel


def tp3_resample(shape, h, origin, pos, vel, phase, u, v, w, cnt, acc, max_particles, min_pc=3, max_pc=8,
                 cscale=4096.0):
    """returns positions, velocities, moved, stats (liquid donors, liquid
    need, gas donors, gas need)"""
    pos, vel = _f32(pos).copy(), _f32(vel).copy()
    stats = np.zeros(4, np.int64)
    res, hh, oo = _geom(shape, h, origin)
    moved = lib().orc_tp3_resample(res, hh, oo, pos.size // 3, int(max_particles), _fptr(pos), _fptr(vel),
                                   _fptr(_f32(phase)), _fptr(_f32(u)), _fptr(_f32(v)), _fptr(_f32(w)),
                                   _i32(np.ascontiguousarray(cnt, np.int32)),
                                   _i32(np.ascontiguousarray(acc, np.int32)), float(cscale), int(min_pc), int(max_pc),
                                   stats.ctypes.data_as(C.POINTER(C.c_int64)))
    return pos, vel, int(moved), stats

