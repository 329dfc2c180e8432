"""Host-side mirror of tsl_array_n's field API (packages/tsl_array_n/src).

``init()`` replaces the WebGPU bring-up of src/context.js:74-132 with a CUDA
context; ``arrayN(type, shape)`` (src/array.js:94-133) returns a device-resident
field owned by libff.  Layout is the reference's i-fastest layout
(src/array.js:24-38): element (i, j, k) sits at i + nx*(j + ny*k), which is
C order of a numpy array shaped (nz, ny, nx).  Errors mirror array.js:4-20
(1-3 dimensions, positive integer extents, known element type).
"""
import ctypes as C

import numpy as np

from . import _lib

TYPES = {"float": 0, "int": 1, "uint8": 2, "vec3": 3}
NP_DTYPES = {0: np.float32, 1: np.int32, 2: np.uint8, 3: np.float32}
_default = None


class Context:
    def __init__(self, device=0):
        lib = _lib.load()
        h = C.c_void_p()
        _lib.check(lib.ff_ctx_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    def synchronize(self):
        _lib.check(_lib.load().ff_ctx_synchronize(self.handle))

    def close(self):
        if self.handle:
            _lib.load().ff_ctx_destroy(self.handle)
            self.handle = None


def init(device=0):
    """init(): select a CUDA device (tsl_array_n src/context.js:74-132)."""
    global _default
    if _default is None:
        _default = Context(device)
    return _default


def context():
    return init()


def compute_strides(shape):
    """computeStrides (src/array.js:24-38): i-fastest, stride[0] = 1."""
    strides, s = [], 1
    for n in shape:
        strides.append(s)
        s *= n
    return strides


def flatten_index(shape, index):
    """flattenNodeIndex (src/array.js:70-92) on host integers."""
    return sum(i * s for i, s in zip(index, compute_strides(shape)))


def _validate(type_, shape):
    if type_ not in TYPES:
        raise ValueError(f'tsl_array_n: unknown type "{type_}"')
    if not isinstance(shape, (list, tuple)) or not 1 <= len(shape) <= 3:
        raise ValueError(f"tsl_array_n: shape must have 1-3 dimensions, got {shape!r}")
    for n in shape:
        if not isinstance(n, (int, np.integer)) or n <= 0:
            raise ValueError(f"tsl_array_n: shape entries must be positive integers, got {shape!r}")


class Field:
    """A device field: arrayN(type, shape)."""

    def __init__(self, type_, shape, ctx=None):
        _validate(type_, list(shape))
        self.ctx = ctx or context()
        self.type = type_
        self.shape = tuple(int(n) for n in shape)
        self.count = int(np.prod(self.shape))
        self.dtype = NP_DTYPES[TYPES[type_]]
        self.width = 3 if type_ == "vec3" else 1
        dims = (C.c_int * len(self.shape))(*self.shape)
        h = C.c_void_p()
        _lib.check(_lib.load().ff_field_create(self.ctx.handle, TYPES[type_], len(self.shape), dims,
                                               C.byref(h)))
        self.handle = h

    @property
    def nbytes(self):
        return self.count * self.width * np.dtype(self.dtype).itemsize

    def from_array(self, values):
        """fromArray (src/array.js:124-129)."""
        a = np.ascontiguousarray(values, dtype=self.dtype).ravel()
        if a.size != self.count * self.width:
            raise ValueError(f"tsl_array_n: fromArray got {a.size} values for a field of "
                             f"{self.count * self.width}")
        _lib.check(_lib.load().ff_field_upload(self.handle, a.ctypes.data, a.nbytes))
        return self

    def to_array(self):
        """toArray (src/array.js:114-122), flat in i-fastest order."""
        out = np.empty(self.count * self.width, dtype=self.dtype)
        _lib.check(_lib.load().ff_field_download(self.handle, out.ctypes.data, out.nbytes))
        return out

    def to_numpy(self):
        """The field as a numpy array shaped (nz, ny, nx) (reversed shape)."""
        return self.to_array().reshape(tuple(reversed(self.shape)))

    def fill(self, value):
        _lib.check(_lib.load().ff_field_fill(self.handle, float(value)))
        return self

    def copy_from(self, src):
        """Device-to-device copy of a field of the same type and size."""
        _lib.check(_lib.load().ff_field_copy(self.handle, src.handle))
        return self

    def device_ptr(self):
        return _lib.load().ff_field_device_ptr(self.handle)

    def destroy(self):
        if getattr(self, "handle", None):
            _lib.load().ff_field_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            if getattr(self, "owned", True):
                self.destroy()
        except Exception:
            pass


class BorrowedField(Field):
    """A handle owned by a solver (pressure, b, masks); not freed here."""

    def __init__(self, handle, ctx):
        lib = _lib.load()
        dt, nd = C.c_int(), C.c_int()
        shp = (C.c_int * 3)()
        cnt = C.c_int64()
        _lib.check(lib.ff_field_info(handle, C.byref(dt), C.byref(nd), shp, C.byref(cnt)))
        self.ctx = ctx
        self.handle = handle
        self.owned = False
        inv = {v: k for k, v in TYPES.items()}
        self.type = inv[dt.value]
        self.shape = tuple(shp[: nd.value])
        self.count = int(cnt.value)
        self.dtype = NP_DTYPES[dt.value]
        self.width = 3 if self.type == "vec3" else 1

    def destroy(self):
        self.handle = None


def arrayN(type_, shape):
    return Field(type_, shape)


def array0(type_):
    return Field(type_, [1])


def array2(type_, nx, ny):
    return Field(type_, [nx, ny])


def array3(type_, nx, ny, nz):
    return Field(type_, [nx, ny, nz])
