"""kg_step_noalloc: the step for callers that cannot allocate device memory.

A viewer loop that owns the GPU memory budget, a host recording work while a
stream is captured, or a real-time loop that must not synchronise on
cudaMalloc/cudaFree, keeps its own phi, T and theta on the device and asks the
library to advance them in place.  The library then uses a fixed device array
for the second copy of the state instead of allocating one.  This file checks,
through the C ABI, that two such calls in a row give exactly (tolerance 0, as
every other step test here) what the allocating kg_create/kg_step path gives,
and that grids above the array's 512 x 512 limit are refused.  It is collected
last on purpose, and passes alone or after the other tests.
"""
import ctypes

import numpy as np
import pytest

from crystalgrowth_gb300 import Kobayashi, KgError, Params, _lib, configs

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    return np.array_equal(np.asarray(a, np.float64).view(np.uint64), np.asarray(b, np.float64).view(np.uint64))


def test_two_noalloc_calls_match_the_allocating_step():
    torch = pytest.importorskip("torch")
    nx, ny = 300, 200
    params = dict(configs.BASE)
    disks = [(150, 100, 6), (40, 30, 4)]
    init = configs.initial_fields(nx, ny, disks)
    # the caller's own device buffers (allocated here by the caller, not by the entry point)
    bufs = [torch.tensor(a, dtype=torch.float64, device="cuda") for a in init]
    stream = torch.cuda.Stream()
    p = Params.make(params)
    ref = Kobayashi(nx, ny, params["dt"], params=params)
    ref.seed_disks(disks)
    for nsteps in (7, 10):  # an odd count (result copied back from the scratch array), then an even one
        rc = _lib.lib().kg_step_noalloc(nx, ny, ctypes.byref(p), ctypes.c_void_p(bufs[0].data_ptr()),
                                        ctypes.c_void_p(bufs[1].data_ptr()), ctypes.c_void_p(bufs[2].data_ptr()),
                                        nsteps, ctypes.c_void_p(stream.cuda_stream))
        _lib.check(rc)
        stream.synchronize()
        ref.step(nsteps)
        for got, want in zip(bufs, ref.fields()):
            assert bits_equal(got.cpu().numpy(), want)
    ref.close()


def test_noalloc_refuses_grids_above_the_limit():
    p = Params.make(configs.BASE)
    dummy = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    rc = _lib.lib().kg_step_noalloc(513, 512, ctypes.byref(p), dummy, dummy, dummy, 1, None)
    assert rc == _lib.KG_ERR_INVALID
    assert b"exceeds the no-allocation limit" in _lib.lib().kg_last_error()
