"""ctypes front end of the CPU oracles -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline
leg, never by the product package.

* ``Port``       -- ko_oracle.c, the FP64 C restatement of the reference step
                    (libm=True: C-library atan/sin/cos; libm=False: kg_math.h).
* ``Reference``  -- the reference's own src/Kobayashi.cpp compiled verbatim
                    (fp64=True: float->double build; fp64=False: as shipped).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_dp = ctypes.POINTER(ctypes.c_double)

PARAM_FIELDS = ("dx", "dy", "dt", "tau", "eps_bar", "mu", "K", "delta", "aniso", "alpha", "gamma", "teq", "theta0")


class KoParams(ctypes.Structure):
    _fields_ = [(f, ctypes.c_double) for f in PARAM_FIELDS]


def _ptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def build():
    import importlib.util
    spec = importlib.util.spec_from_file_location("build_oracle", os.path.join(HERE, "build_oracle.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()


_port_lib = None


def port_lib():
    global _port_lib
    if _port_lib is None:
        path = os.path.join(HERE, "libko_oracle.so")
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        lib.ko_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(KoParams), _dp, _dp, _dp,
                               ctypes.c_longlong, ctypes.c_int, ctypes.c_int]
        lib.ko_run.restype = ctypes.c_int
        lib.ko_kg_atan.argtypes = [ctypes.c_double]
        lib.ko_kg_atan.restype = ctypes.c_double
        lib.ko_kg_sincos.argtypes = [ctypes.c_double, _dp, _dp]
        lib.ko_kg_eval.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_longlong, ctypes.c_double]
        lib.ko_kg_eval.restype = ctypes.c_int
        lib.ko_tlm_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(KoParams), _dp, _dp, _dp, _dp,
                                   _dp, _dp, _dp, ctypes.c_longlong, ctypes.c_int]
        lib.ko_tlm_run.restype = ctypes.c_int
        _port_lib = lib
    return _port_lib


def params_struct(p):
    return KoParams(*[float(p[f]) for f in PARAM_FIELDS])


def port_run(phi, T, theta, params, nsteps, libm=False, threads=1):
    """Advance copies of (phi, T, theta) [ny, nx] by nsteps; returns the new arrays."""
    phi = np.array(phi, dtype=np.float64, order="C", copy=True)
    T = np.array(T, dtype=np.float64, order="C", copy=True)
    theta = np.array(theta, dtype=np.float64, order="C", copy=True)
    ny, nx = phi.shape
    ps = params_struct(params)
    rc = port_lib().ko_run(nx, ny, ctypes.byref(ps), _ptr(phi), _ptr(T), _ptr(theta), int(nsteps),
                           1 if libm else 0, int(threads))
    if rc != 0:
        raise RuntimeError("ko_run failed")
    return phi, T, theta


def tlm_run(phi, T, theta, dphi, dT, dtheta, params, dparams, nsteps, threads=1):
    """Tangent-linear rollout: returns (state, tangent) after nsteps.
    dparams: dict with any of d_delta, d_K, d_theta0, d_tau, d_gamma."""
    arrs = [np.array(a, dtype=np.float64, order="C", copy=True) for a in (phi, T, theta, dphi, dT, dtheta)]
    ny, nx = arrs[0].shape
    dp = np.array([dparams.get(k, 0.0) for k in ("d_delta", "d_K", "d_theta0", "d_tau", "d_gamma")])
    ps = params_struct(params)
    rc = port_lib().ko_tlm_run(nx, ny, ctypes.byref(ps), _ptr(dp), *[_ptr(a) for a in arrs], int(nsteps),
                               int(threads))
    if rc != 0:
        raise RuntimeError("ko_tlm_run failed")
    return tuple(arrs[:3]), tuple(arrs[3:])


def kg_atan(x):
    return port_lib().ko_kg_atan(float(x))


def kg_sincos(x):
    s = ctypes.c_double()
    c = ctypes.c_double()
    port_lib().ko_kg_sincos(float(x), ctypes.byref(s), ctypes.byref(c))
    return s.value, c.value


def kg_eval(fn, x, b=1.0):
    """host kg_math over an array: fn 0 atan, 1 sin, 2 cos, 4 x / b, 5 kg_idiv(x, b), 10 kg_twice_plus,
    11 two-rounding 2x + y, 12 kg_absorb_bound, 13 kg_gdiv, 14 x[i] / x[n-1-i] (see ko_oracle.c)"""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    if port_lib().ko_kg_eval(int(fn), _ptr(x), _ptr(y), x.size, float(b)) != 0:
        raise ValueError("ko_kg_eval failed")
    return y


class Reference:
    """The reference's own Kobayashi class (src/Kobayashi.cpp), driven through ref_harness.cpp."""

    def __init__(self, nx, ny, dt, fp64=True):
        tag = "64" if fp64 else "32"
        path = os.path.join(HERE, "_ref", "libko_ref%s.so" % tag)
        if not os.path.exists(path):
            build()
        if not os.path.exists(path):
            raise FileNotFoundError("reference oracle library not built (no reference source staged)")
        lib = ctypes.CDLL(path)
        self.pre = "ref" + tag + "_"
        f = lambda n: getattr(lib, self.pre + n)
        f("create").restype = ctypes.c_void_p
        f("create").argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double]
        for n in ("destroy", "update", "vector_init"):
            f(n).argtypes = [ctypes.c_void_p]
        f("set_params").argtypes = [ctypes.c_void_p, _dp]
        f("get_params").argtypes = [ctypes.c_void_p, _dp]
        f("set_state").argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        f("get_state").argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        f("step").argtypes = [ctypes.c_void_p, ctypes.c_longlong]
        f("frame").argtypes = [ctypes.c_void_p]
        f("frame").restype = ctypes.c_int
        f("colors").argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)]
        self.lib = lib
        self.f = f
        self.nx, self.ny = nx, ny
        self.h = f("create")(nx, ny, dt)

    def __del__(self):
        if getattr(self, "h", None):
            self.f("destroy")(self.h)
            self.h = None

    def set_params(self, p):
        arr = np.array([p[k] for k in PARAM_FIELDS[:12]], dtype=np.float64)
        self.f("set_params")(self.h, _ptr(arr))

    def get_params(self):
        arr = np.zeros(12)
        self.f("get_params")(self.h, _ptr(arr))
        return dict(zip(PARAM_FIELDS[:12], arr.tolist()))

    def set_state(self, phi, T, theta):
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (phi, T, theta)]
        self.f("set_state")(self.h, *[_ptr(x) for x in a])

    def get_state(self):
        a = [np.zeros((self.ny, self.nx)) for _ in range(3)]
        self.f("get_state")(self.h, *[_ptr(x) for x in a])
        return tuple(a)

    def step(self, n):
        self.f("step")(self.h, int(n))

    def update(self):
        self.f("update")(self.h)

    def vector_init(self):
        self.f("vector_init")(self.h)

    def frame(self):
        return self.f("frame")(self.h)

    def colors(self):
        out = np.zeros((self.nx * self.ny, 4), dtype=np.float32)
        self.f("colors")(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        return out
