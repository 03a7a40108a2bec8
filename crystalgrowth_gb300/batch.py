"""Batched ensemble of independent grids (include/kobayashi_batch.h)."""
import ctypes

import numpy as np

from ._lib import Params, check, dptr, iptr, lib

KG_BATCH_LAUNCH = 0
KG_BATCH_PERSISTENT = 1


class Tuning(ctypes.Structure):
    _fields_ = [("nt", ctypes.c_int), ("bh", ctypes.c_int), ("mode", ctypes.c_int), ("chunk", ctypes.c_int),
                ("streams", ctypes.c_int), ("tblock", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class Batch:
    """n instances: sizes [(nx, ny), ...] and one parameter dict per instance."""

    def __init__(self, sizes, params):
        n = len(sizes)
        assert n == len(params) and n > 0
        nx = np.array([s[0] for s in sizes], dtype=np.int32)
        ny = np.array([s[1] for s in sizes], dtype=np.int32)
        parr = (Params * n)(*[Params.make(p) for p in params])
        h = ctypes.c_void_p()
        check(lib().kg_batch_create(n, iptr(nx), iptr(ny), parr, ctypes.byref(h)))
        self._h = h
        self.sizes = [(int(a), int(b)) for a, b in zip(nx, ny)]

    def seed_disks(self, k, disks):
        d = np.asarray(list(disks), dtype=np.int32).reshape(-1, 3)
        cx, cy, r = (np.ascontiguousarray(d[:, i]) for i in range(3))
        check(lib().kg_batch_seed_disks(self._h, int(k), len(d), iptr(cx), iptr(cy), iptr(r)))

    def step(self, n):
        check(lib().kg_batch_step(self._h, int(n)))

    def sync(self):
        check(lib().kg_batch_sync(self._h))

    def fields(self, k):
        nx, ny = self.sizes[k]
        out = [np.empty((ny, nx)) for _ in range(3)]
        check(lib().kg_batch_get_fields(self._h, int(k), *[dptr(a) for a in out]))
        return tuple(out)

    def set_fields(self, k, phi, T, theta):
        nx, ny = self.sizes[k]
        arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(ny, nx) for a in (phi, T, theta)]
        check(lib().kg_batch_set_fields(self._h, int(k), *[dptr(a) for a in arrs]))

    def info(self):
        n, cells, steps, nwork = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_int()
        check(lib().kg_batch_get_info(self._h, ctypes.byref(n), ctypes.byref(cells), ctypes.byref(steps),
                                      ctypes.byref(nwork)))
        return dict(n=n.value, cells=cells.value, steps=steps.value, nwork=nwork.value)

    def tuning(self):
        t = Tuning()
        check(lib().kg_batch_get_tuning(self._h, ctypes.byref(t)))
        return t.as_dict()

    def set_tuning(self, nt=128, bh=64, mode=KG_BATCH_LAUNCH, chunk=100, streams=1, tblock=1):
        """tblock: time steps per pass over HBM (1, or 2 for temporal blocking)"""
        t = Tuning(nt, bh, mode, chunk, streams, tblock)
        check(lib().kg_batch_set_tuning(self._h, ctypes.byref(t)))

    def autotune(self, trial_steps=5):
        t = Tuning()
        ms = ctypes.c_double()
        check(lib().kg_batch_autotune(self._h, int(trial_steps), ctypes.byref(t), ctypes.byref(ms)))
        return t.as_dict(), ms.value

    def stream(self):
        s = ctypes.c_void_p()
        check(lib().kg_batch_get_stream(self._h, ctypes.byref(s)))
        return s.value

    def close(self):
        if getattr(self, "_h", None):
            lib().kg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
