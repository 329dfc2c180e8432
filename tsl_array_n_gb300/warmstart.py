"""Learned warm start for the pressure solve (no reference counterpart):
a 3-level 3D U-Net, trained on (divergence, Dirichlet mask, previous
pressure) -> pressure pairs that the plain solver generates, whose guess
starts MGPCG when it lowers the initial residual.  The network, its
gradients and Adam run in libff (include/ff.h ff_unet_*)."""
import ctypes as C

import numpy as np

from . import _lib
from .tsl_array_n import context


class UNetWarmStart:
    def __init__(self, seed=1):
        self.handle = C.c_void_p()
        _lib.check(_lib.load().ff_unet_create(context().handle, int(seed) & 0xFFFFFFFF, C.byref(self.handle)))
        n = C.c_int64()
        _lib.check(_lib.load().ff_unet_param_count(self.handle, C.byref(n)))
        self.param_count = n.value

    @property
    def params(self):
        out = np.empty(self.param_count, np.float32)
        _lib.check(_lib.load().ff_unet_get_params(self.handle, out.ctypes.data_as(C.POINTER(C.c_float)),
                                                  self.param_count))
        return out

    @params.setter
    def params(self, values):
        a = np.ascontiguousarray(values, np.float32)
        _lib.check(_lib.load().ff_unet_set_params(self.handle, a.ctypes.data_as(C.POINTER(C.c_float)), a.size))

    @property
    def grads(self):
        out = np.empty(self.param_count, np.float32)
        _lib.check(_lib.load().ff_unet_get_grads(self.handle, out.ctypes.data_as(C.POINTER(C.c_float)),
                                                 self.param_count))
        return out

    def forward(self, resolution, h, b, mask, p_prev, out):
        """p0 = net(b, mask, p_prev) into the float cell field `out`."""
        _lib.check(_lib.load().ff_unet_forward(self.handle, (C.c_int * 3)(*resolution), float(h), b.handle,
                                               mask.handle if mask is not None else None,
                                               p_prev.handle if p_prev is not None else None, out.handle))

    def loss_backward(self, resolution, h, b, mask, p_prev, target):
        loss = C.c_double()
        _lib.check(_lib.load().ff_unet_loss_backward(self.handle, (C.c_int * 3)(*resolution), float(h), b.handle,
                                                     mask.handle if mask is not None else None,
                                                     p_prev.handle if p_prev is not None else None, target.handle,
                                                     C.byref(loss)))
        return loss.value

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        _lib.check(_lib.load().ff_unet_adam_step(self.handle, float(lr), float(beta1), float(beta2), float(eps)))

    def train_step(self, resolution, h, b, mask, p_prev, target, lr=1e-3):
        loss = self.loss_backward(resolution, h, b, mask, p_prev, target)
        self.adam_step(lr)
        return loss

    def save(self, path):
        np.save(path, self.params)

    def load(self, path):
        self.params = np.load(path)

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().ff_unet_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def attach(solver, net):
    """Use `net` for the initial guess of the solver's next solves (None
    detaches); diagnostics then report warmStart 1 (guess used) or 0."""
    _lib.check(_lib.load().ff_pressure3_set_warm_start(solver.handle, net.handle if net is not None else None))
    solver._warm = net
