"""Reverse-mode gradients of a rollout (include/kobayashi_adjoint.h)."""
import ctypes

import numpy as np

from ._lib import Params, check, dptr, lib


class GradResult(ctypes.Structure):
    _fields_ = [("loss", ctypes.c_double), ("d_delta", ctypes.c_double), ("d_K", ctypes.c_double),
                ("d_theta0", ctypes.c_double), ("d_tau", ctypes.c_double), ("d_gamma", ctypes.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class Adjoint:
    """Loss 0.5 ||phi_N - phi_target||^2 of an nsteps rollout and its gradient with respect to
    delta, K, theta0, tau, gamma and the initial T field."""

    def __init__(self, nx, ny, params, nsteps, checkpoint_every=64):
        p = Params.make(params)
        h = ctypes.c_void_p()
        check(lib().kg_adjoint_create(int(nx), int(ny), ctypes.byref(p), int(nsteps), int(checkpoint_every),
                                      ctypes.byref(h)))
        self._h = h
        self.nx, self.ny = int(nx), int(ny)

    def set_params(self, params):
        p = Params.make(params)
        check(lib().kg_adjoint_set_params(self._h, ctypes.byref(p)))

    def set_initial(self, phi0, T0, theta0=None):
        a = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (phi0, T0, theta0)]
        check(lib().kg_adjoint_set_initial(self._h, *[dptr(x) for x in a]))

    def set_target(self, phi_target):
        a = np.ascontiguousarray(phi_target, dtype=np.float64)
        check(lib().kg_adjoint_set_target(self._h, dptr(a)))

    def forward(self, want_state=False):
        loss = ctypes.c_double()
        out = [np.empty((self.ny, self.nx)) for _ in range(3)] if want_state else [None] * 3
        check(lib().kg_adjoint_forward(self._h, ctypes.byref(loss), *[dptr(x) for x in out]))
        return (loss.value, tuple(out)) if want_state else loss.value

    def gradient(self, want_dT0=True):
        r = GradResult()
        g = np.empty((self.ny, self.nx)) if want_dT0 else None
        check(lib().kg_adjoint_gradient(self._h, ctypes.byref(r), dptr(g)))
        return r.as_dict(), g

    def stream(self):
        s = ctypes.c_void_p()
        check(lib().kg_adjoint_get_stream(self._h, ctypes.byref(s)))
        return s.value

    def close(self):
        if getattr(self, "_h", None):
            lib().kg_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
