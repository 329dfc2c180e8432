"""ff_collider3_bake_noalloc through the C ABI: the fixed-table variant of
the collider bake gives the same fields as ff_collider3_bake, on two
different shape sets baked back to back (the second call must not see the
first call's table), leaves the device's free memory unchanged once warm,
and rejects more shapes than its table holds.  Named to be collected last;
it also passes on its own."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SETS = [
    [{"type": "sphere", "center": [0.5, 0.5, 0.5], "radius": 0.21},
     {"type": "box", "center": [0.2, 0.3, 0.7], "halfExtents": [0.1, 0.06, 0.12],
      "rotation": {"axis": [1.0, 0.4, 0.2], "angle": 0.9}}],
    [{"type": "box", "center": [0.6, 0.55, 0.4], "halfExtents": [0.2, 0.15, 0.1]},
     {"type": "sphere", "center": [0.3, 0.7, 0.35], "radius": 0.12},
     {"type": "sphere", "center": [0.75, 0.25, 0.6], "radius": 0.09}],
]


def bake(entry, shapes, res, h, invert=0):
    from tsl_array_n_gb300 import _lib
    from tsl_array_n_gb300.fluxflow import SDFStaticCollider3
    from tsl_array_n_gb300.tsl_array_n import Field, context
    nx, ny, nz = res
    phi = Field("float", res)
    w = [Field("float", (nx + 1, ny, nz)), Field("float", (nx, ny + 1, nz)), Field("float", (nx, ny, nz + 1))]
    arr = (_lib.Shape * max(1, len(shapes)))(*[SDFStaticCollider3._shape(s) for s in shapes])
    rc = getattr(_lib.load(), entry)(context().handle, arr, len(shapes), invert, (C.c_int * 3)(*res),
                                     (C.c_double * 3)(*h), (C.c_double * 3)(0.0, 0.0, 0.0), phi.handle,
                                     w[0].handle, w[1].handle, w[2].handle)
    _lib.check(rc)
    context().synchronize()
    return [phi.to_array()] + [f.to_array() for f in w]


def test_noalloc_bake_matches_bake_twice_in_a_row(gpu):
    res, h = (36, 28, 44), (1 / 36, 1 / 28, 1 / 44)
    # the fixed-table calls back to back, then the allocating ones
    got = [bake("ff_collider3_bake_noalloc", s, res, h) for s in SETS]
    ref = [bake("ff_collider3_bake", s, res, h) for s in SETS]
    for g, r in zip(got, ref):
        for a, b in zip(g, r):
            assert np.array_equal(a, b)
    # the two shape sets give different fields, so a stale table would show
    assert not np.array_equal(got[0][0], got[1][0])


def test_noalloc_bake_inverted_and_empty(gpu):
    res, h = (32, 32, 32), (1 / 32,) * 3
    for shapes, inv in ((SETS[0], 1), ([], 0)):
        a = bake("ff_collider3_bake_noalloc", shapes, res, h, inv)
        b = bake("ff_collider3_bake", shapes, res, h, inv)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_noalloc_bake_keeps_free_memory(gpu):
    """After the first call (which looks the fixed array up), further calls
    change the device's free memory by nothing: no allocation outlives the
    call.  The output fields are created before the first reading."""
    torch = pytest.importorskip("torch")
    from tsl_array_n_gb300 import _lib
    from tsl_array_n_gb300.fluxflow import SDFStaticCollider3
    from tsl_array_n_gb300.tsl_array_n import Field, context
    lib = _lib.load()
    res, h = (48, 40, 36), (1 / 48, 1 / 40, 1 / 36)
    nx, ny, nz = res
    out = [Field("float", res), Field("float", (nx + 1, ny, nz)), Field("float", (nx, ny + 1, nz)),
           Field("float", (nx, ny, nz + 1))]
    arr = (_lib.Shape * len(SETS[1]))(*[SDFStaticCollider3._shape(s) for s in SETS[1]])

    def call():
        _lib.check(lib.ff_collider3_bake_noalloc(context().handle, arr, len(SETS[1]), 0, (C.c_int * 3)(*res),
                                                 (C.c_double * 3)(*h), (C.c_double * 3)(0.0, 0.0, 0.0),
                                                 *[f.handle for f in out]))

    torch.cuda.mem_get_info(0)   # the reading's own set-up first
    call()
    context().synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    for _ in range(3):
        call()
    context().synchronize()
    assert torch.cuda.mem_get_info(0)[0] == free0
    ref = bake("ff_collider3_bake", SETS[1], res, h)
    for f, r in zip(out, ref):
        assert np.array_equal(f.to_array(), r)


def test_noalloc_bake_rejects_oversize(gpu):
    from tsl_array_n_gb300 import _lib
    from tsl_array_n_gb300.fluxflow import SDFStaticCollider3
    from tsl_array_n_gb300.tsl_array_n import Field, context
    lib = _lib.load()
    res = (16, 16, 16)
    phi = Field("float", res)
    n = 65   # FF_BAKE_NOALLOC_MAX_SHAPES + 1
    arr = (_lib.Shape * n)(*[SDFStaticCollider3._shape({"type": "sphere", "center": [0.5] * 3, "radius": 0.1})
                             for _ in range(n)])
    rc = lib.ff_collider3_bake_noalloc(context().handle, arr, n, 0, (C.c_int * 3)(*res),
                                       (C.c_double * 3)(1 / 16, 1 / 16, 1 / 16), (C.c_double * 3)(0, 0, 0),
                                       phi.handle, None, None, None)
    assert rc == -5   # FF_E_LIMIT
    assert b"exceed the fixed table of 64" in lib.ff_last_error()
