"""tsl_array_n_gb300: GB300 (sm_103a) implementation of fluxflow's grid-fluid
hot path behind the reference's tsl_array_n field API and fluxflow grid/
projection calls.  The compute runs in libff.so (include/ff.h); this package
is the host-side mirror of the reference interface."""
from . import _lib
from .tsl_array_n import arrayN, array0, array2, array3, init, Field  # noqa: F401

__all__ = ["arrayN", "array0", "array2", "array3", "init", "Field", "load_library"]


def load_library():
    """Load libff.so; raises FFError when it is not built (no CPU fallback)."""
    return _lib.load()
