"""Python mirror of the reference's Kobayashi class (src/Kobayashi.h:32-122),
headless, over the C ABI.  The same surface exists in C++ as
include/kobayashi.hpp."""
import ctypes

import numpy as np

from ._lib import Params, check, dptr, iptr, lib


class Kobayashi:
    """Kobayashi(x, y, timeStep) -- src/Kobayashi.cpp:7-67.

    Owns one FP64 grid on the current CUDA device.  ``params`` may be a dict or
    Params overriding the reference defaults (src/Kobayashi.cpp:61-63,76-84).
    """

    def __init__(self, x, y, timeStep=1e-4, params=None):
        p = Params.make(params or {}, dt=timeStep)
        h = ctypes.c_void_p()
        check(lib().kg_create(int(x), int(y), ctypes.byref(p), ctypes.byref(h)))
        self._h = h
        self.nx, self.ny = int(x), int(y)

    # -- reference surface -------------------------------------------------
    def iUpdate(self):
        """10 explicit steps (src/Kobayashi.cpp:227-239)."""
        check(lib().kg_update(self._h))

    def iResetSimulationState(self, constantBuffer=None):
        """_vectorInit: zero fields, 5-cell nucleus (src/Kobayashi.cpp:241-249)."""
        check(lib().kg_reset(self._h))

    def iGetObjectCount(self):
        return (self.nx, self.ny, 0)

    def iIsUpdated(self):
        return True

    # -- accessors and extensions -------------------------------------------
    def step(self, n):
        check(lib().kg_step(self._h, int(n)))

    def sync(self):
        check(lib().kg_sync(self._h))

    def seed_disks(self, disks):
        """disks: iterable of (cx, cy, r)."""
        d = np.asarray(list(disks), dtype=np.int32).reshape(-1, 3)
        cx, cy, r = (np.ascontiguousarray(d[:, k]) for k in range(3))
        check(lib().kg_seed_disks(self._h, len(d), iptr(cx), iptr(cy), iptr(r)))

    def fields(self, out=None):
        """(phi, T, theta) as (ny, nx) float64 arrays.  `out`: three C-contiguous float64 arrays of
        that shape to copy into (for example page-locked buffers, which the copy reaches at the
        link's full speed); new arrays otherwise."""
        if out is None:
            out = [np.empty((self.ny, self.nx)) for _ in range(3)]
        else:
            out = list(out)
            if len(out) != 3 or any(not isinstance(a, np.ndarray) or a.dtype != np.float64 or
                                    a.size != self.nx * self.ny or not a.flags.c_contiguous or
                                    not a.flags.writeable for a in out):
                raise ValueError("out: three writeable C-contiguous float64 arrays of %d x %d" % (self.ny, self.nx))
        check(lib().kg_get_fields(self._h, *[dptr(a) for a in out]))
        return tuple(out)

    def phi(self):
        return self.fields()[0]

    def T(self):
        return self.fields()[1]

    def theta(self):
        return self.fields()[2]

    def set_fields(self, phi=None, T=None, theta=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(self.ny, self.nx)
                for a in (phi, T, theta)]
        check(lib().kg_set_fields(self._h, *[dptr(a) for a in arrs]))

    def params(self):
        p = Params()
        check(lib().kg_get_params(self._h, ctypes.byref(p)))
        return p.as_dict()

    def set_params(self, **kw):
        p = Params()
        check(lib().kg_get_params(self._h, ctypes.byref(p)))
        for k, v in kw.items():
            setattr(p, k, float(v))
        check(lib().kg_set_params(self._h, ctypes.byref(p)))

    def counters(self):
        s, f = ctypes.c_longlong(), ctypes.c_longlong()
        check(lib().kg_get_counters(self._h, ctypes.byref(s), ctypes.byref(f)))
        return s.value, f.value

    def set_graph_chunk(self, chunk):
        check(lib().kg_set_graph_chunk(self._h, int(chunk)))

    def colormap(self, viewer_order=False):
        """RGBA float32 of every cell (the reference's colour ramp, src/Kobayashi.cpp:309-345);
        viewer_order=True reproduces the viewer's constant-buffer order and its transposition."""
        out = np.empty((self.nx * self.ny, 4), dtype=np.float32)
        check(lib().kg_colormap(self._h, 1 if viewer_order else 0, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return out

    def save(self, path):
        """snapshot: JSON header + phi, T, theta (FP64)"""
        check(lib().kg_save(self._h, str(path).encode()))

    def load(self, path):
        check(lib().kg_load(self._h, str(path).encode()))

    def set_tile(self, nt, bh):
        check(lib().kg_set_tile(self._h, int(nt), int(bh)))

    def set_tblock(self, k):
        """time steps per pass over HBM: 1, or 2 (temporal blocking; identical results)"""
        check(lib().kg_set_tblock(self._h, int(k)))

    def tblock(self):
        k = ctypes.c_int()
        check(lib().kg_get_tblock(self._h, ctypes.byref(k)))
        return k.value

    def tile(self):
        nt, bh = ctypes.c_int(), ctypes.c_int()
        check(lib().kg_get_tile(self._h, ctypes.byref(nt), ctypes.byref(bh)))
        return nt.value, bh.value

    def stream(self):
        s = ctypes.c_void_p()
        check(lib().kg_get_stream(self._h, ctypes.byref(s)))
        return s.value

    def device_fields(self):
        ptrs = [ctypes.POINTER(ctypes.c_double)() for _ in range(3)]
        check(lib().kg_device_fields(self._h, *[ctypes.byref(p) for p in ptrs]))
        return tuple(ctypes.cast(p, ctypes.c_void_p).value for p in ptrs)

    def close(self):
        if getattr(self, "_h", None):
            lib().kg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
