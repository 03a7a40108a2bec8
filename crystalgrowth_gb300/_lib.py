"""ctypes binding of libkobayashi_gpu.so (include/kobayashi_gpu.h).

The library is built in-tree by crystalgrowth_gb300/build.py (or
__graft_entry__.build()).  Loading fails with an exception when it is absent:
there is no fallback implementation.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libkobayashi_gpu.so")

KG_OK = 0
KG_ERR_INVALID = -1
KG_ERR_CUDA = -2
KG_ERR_NOMEM = -3
KG_ERR_TIMEOUT = -4

PARAM_FIELDS = ("dx", "dy", "dt", "tau", "eps_bar", "mu", "K", "delta", "aniso", "alpha", "gamma", "teq", "theta0")


class Params(ctypes.Structure):
    """kg_params (include/kobayashi_gpu.h)."""
    _fields_ = [(f, ctypes.c_double) for f in PARAM_FIELDS]

    @classmethod
    def make(cls, d=None, **kw):
        p = cls()
        lib().kg_params_default(ctypes.byref(p), 1e-4)
        for src in (d or {}), kw:
            for k, v in src.items():
                setattr(p, k, float(v))
        return p

    def as_dict(self):
        return {f: getattr(self, f) for f in PARAM_FIELDS}


class KgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("kg error %d: %s" % (code, msg))
        self.code = code


_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p
_lib = None

# name -> argtypes (every function returns int unless listed in _RESTYPE)
_SIGS = {
    "kg_params_default": [ctypes.POINTER(Params), ctypes.c_double],
    "kg_params_validate": [ctypes.POINTER(Params)],
    "kg_slider_range": [ctypes.c_int, _ip, _ip, _ip],
    "kg_params_from_sliders": [_ip, ctypes.c_double, ctypes.POINTER(Params)],
    "kg_create": [ctypes.c_int, ctypes.c_int, ctypes.POINTER(Params), ctypes.POINTER(_vp)],
    "kg_destroy": [_vp],
    "kg_reset": [_vp],
    "kg_seed_disks": [_vp, ctypes.c_int, _ip, _ip, _ip],
    "kg_set_params": [_vp, ctypes.POINTER(Params)],
    "kg_get_params": [_vp, ctypes.POINTER(Params)],
    "kg_step": [_vp, ctypes.c_longlong],
    "kg_update": [_vp],
    "kg_sync": [_vp],
    "kg_get_fields": [_vp, _dp, _dp, _dp],
    "kg_set_fields": [_vp, _dp, _dp, _dp],
    "kg_get_size": [_vp, _ip, _ip],
    "kg_get_counters": [_vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)],
    "kg_device_fields": [_vp, ctypes.POINTER(_dp), ctypes.POINTER(_dp), ctypes.POINTER(_dp)],
    "kg_get_stream": [_vp, ctypes.POINTER(_vp)],
    "kg_set_graph_chunk": [_vp, ctypes.c_int],
    "kg_set_tile": [_vp, ctypes.c_int, ctypes.c_int],
    "kg_colormap": [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_float)],
    "kg_save": [_vp, ctypes.c_char_p],
    "kg_load": [_vp, ctypes.c_char_p],
    "kg_colormap_device": [_vp, ctypes.c_int, _vp],
    "kg_get_tile": [_vp, _ip, _ip],
    "kg_set_tblock": [_vp, ctypes.c_int],
    "kg_get_tblock": [_vp, _ip],
    "kg_step_noalloc": [ctypes.c_int, ctypes.c_int, ctypes.POINTER(Params), _vp, _vp, _vp, ctypes.c_longlong, _vp],
    "kg_last_error": [],
    "kg_version": [],
    "kg_diag_eval": [ctypes.c_int, _dp, _dp, ctypes.c_longlong, ctypes.c_double],
    "kg_diag_barrier_timeout": [ctypes.c_int, ctypes.c_longlong, _ip],
    "kg_diag_mbar_timeout": [_ip],
    "kg_batch_create": [ctypes.c_int, _ip, _ip, ctypes.POINTER(Params), ctypes.POINTER(_vp)],
    "kg_batch_destroy": [_vp],
    "kg_batch_seed_disks": [_vp, ctypes.c_int, ctypes.c_int, _ip, _ip, _ip],
    "kg_batch_step": [_vp, ctypes.c_longlong],
    "kg_batch_sync": [_vp],
    "kg_batch_get_fields": [_vp, ctypes.c_int, _dp, _dp, _dp],
    "kg_batch_set_fields": [_vp, ctypes.c_int, _dp, _dp, _dp],
    "kg_batch_get_info": [_vp, _ip, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong), _ip],
    "kg_batch_set_tuning": [_vp, _vp],
    "kg_batch_get_tuning": [_vp, _vp],
    "kg_batch_autotune": [_vp, ctypes.c_int, _vp, ctypes.POINTER(ctypes.c_double)],
    "kg_batch_get_stream": [_vp, ctypes.POINTER(_vp)],
    "kg_adjoint_create": [ctypes.c_int, ctypes.c_int, ctypes.POINTER(Params), ctypes.c_longlong, ctypes.c_int,
                          ctypes.POINTER(_vp)],
    "kg_adjoint_destroy": [_vp],
    "kg_adjoint_set_params": [_vp, ctypes.POINTER(Params)],
    "kg_adjoint_set_initial": [_vp, _dp, _dp, _dp],
    "kg_adjoint_set_target": [_vp, _dp],
    "kg_adjoint_forward": [_vp, ctypes.POINTER(ctypes.c_double), _dp, _dp, _dp],
    "kg_adjoint_gradient": [_vp, _vp, _dp],
    "kg_adjoint_get_stream": [_vp, ctypes.POINTER(_vp)],
    "kg_diag_fp64_peak": [ctypes.POINTER(ctypes.c_double)],
    "kg_diag_fp64_probe": [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                           ctypes.POINTER(ctypes.c_double)],
    "kg_diag_inject_timeout": [_vp],
    "kg_diag_batch_inject_timeout": [_vp],
    "kg_diag_copy": [_vp, _vp, ctypes.c_longlong, _vp],
}
_RESTYPE = {"kg_last_error": ctypes.c_char_p, "kg_version": ctypes.c_char_p}


def load(path=LIB_PATH):
    """Load the library (once) and declare the signatures of every symbol it must export."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise FileNotFoundError(
                "libkobayashi_gpu.so not built at %s: run `python -c 'import __graft_entry__ as g; g.build()'`" % path)
        L = ctypes.CDLL(path)
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPE.get(name, ctypes.c_int)
        _lib = L
    return _lib


def lib():
    return load()


def check(rc):
    if rc != KG_OK:
        raise KgError(rc, lib().kg_last_error().decode(errors="replace"))
    return rc


def dptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def iptr(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)
