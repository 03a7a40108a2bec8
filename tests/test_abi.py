"""The C ABI library (CPU-only checks: no CUDA call is made here).

libkobayashi_gpu.so must load and export every function that
include/*.h declares; the host-only entry points (defaults, validation,
error text, version) must behave.
"""
import ctypes
import os
import re
import subprocess

import pytest

import crystalgrowth_gb300 as kg
from crystalgrowth_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"^KG_API\s+[\w\s\*]*?\b(kg_\w+)\s*\(", text, flags=re.M))
    return sorted(names)


def test_header_declares_the_abi():
    names = declared_symbols()
    for must in ("kg_create", "kg_destroy", "kg_step", "kg_update", "kg_reset", "kg_get_fields", "kg_set_fields",
                 "kg_set_params", "kg_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = kg.load()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (kg_\w+)", out))
    assert set(declared_symbols()) <= exported


def test_python_binding_covers_every_symbol():
    assert set(declared_symbols()) <= set(_lib._SIGS) | {"kg_version"}


def test_defaults_are_the_reference_defaults():
    p = kg.Params.make()
    d = p.as_dict()
    # src/Kobayashi.cpp:61-63 and 76-84
    assert d == dict(dx=0.03, dy=0.03, dt=1e-4, tau=0.0003, eps_bar=0.010, mu=1.0, K=1.6, delta=0.05, aniso=6.0,
                     alpha=0.9, gamma=10.0, teq=1.0, theta0=0.0)


@pytest.mark.parametrize("field,value", [("dx", 0.0), ("dy", -1.0), ("tau", 0.0), ("dt", 0.0), ("eps_bar", 0.0),
                                         ("aniso", 2.5), ("aniso", 0.0), ("theta0", 1e3), ("delta", float("nan")),
                                         ("K", float("inf"))])
def test_validation_rejects(field, value):
    lib = kg.load()
    p = kg.Params.make(**{field: value})
    assert lib.kg_params_validate(ctypes.byref(p)) == _lib.KG_ERR_INVALID
    assert len(lib.kg_last_error()) > 0


def test_validation_accepts_slider_ranges():
    """every value the reference's sliders can reach (src/Kobayashi.cpp:12-59) is a valid parameter"""
    lib = kg.load()
    for tau in (1e-4, 9e-4):
        for eb in (0.006, 0.015):
            for K in (1.0, 1.9):
                for delta in (0.01, 0.09):
                    for j in (2.0, 8.0):
                        p = kg.Params.make(tau=tau, eps_bar=eb, K=K, delta=delta, aniso=j, alpha=1.2, gamma=20.0,
                                           teq=1.5)
                        assert lib.kg_params_validate(ctypes.byref(p)) == 0


def test_null_handle_is_an_error_not_a_crash():
    lib = kg.load()
    assert lib.kg_step(None, 1) == _lib.KG_ERR_INVALID
    assert lib.kg_destroy(None) == 0
    assert b"null" in lib.kg_last_error()
    assert lib.kg_version().startswith(b"kobayashi-gb300")


def test_slider_model():
    """the reference's integer sliders (src/Kobayashi.cpp:12-59): ranges, default positions, and
    value = (float)position * ratio (iWMHScroll's thumb-track branch, :587-591)"""
    import numpy as np
    lib = kg.load()
    rng = []
    for k in range(9):
        lo, hi, de = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        assert lib.kg_slider_range(k, ctypes.byref(lo), ctypes.byref(hi), ctypes.byref(de)) == 0
        rng.append((lo.value, hi.value, de.value))
    assert rng == [(1, 9, 3), (6, 15, 10), (5, 14, 10), (10, 19, 16), (1, 9, 5), (2, 8, 6), (7, 12, 9), (10, 20, 10),
                   (5, 15, 10)]
    assert lib.kg_slider_range(9, None, None, None) == _lib.KG_ERR_INVALID
    pos = (ctypes.c_int * 9)(*[r[2] for r in rng])
    p = kg.Params()
    assert lib.kg_params_from_sliders(pos, 1e-4, ctypes.byref(p)) == 0
    ratios = np.array([1e-4, 1e-3, 0.1, 0.1, 0.01, 1.0, 0.1, 1.0, 0.1], dtype=np.float32)
    want = (np.array([r[2] for r in rng], dtype=np.float32) * ratios).astype(np.float64)
    got = [p.tau, p.eps_bar, p.mu, p.K, p.delta, p.aniso, p.alpha, p.gamma, p.teq]
    assert got == list(want)
    # the slider defaults reproduce the reference's defaults to float precision
    assert abs(p.tau - 0.0003) < 1e-10 and abs(p.K - 1.6) < 1e-6 and p.aniso == 6.0
    bad = (ctypes.c_int * 9)(*[r[2] for r in rng])
    bad[4] = 10
    assert lib.kg_params_from_sliders(bad, 1e-4, ctypes.byref(p)) == _lib.KG_ERR_INVALID
    assert b"outside" in lib.kg_last_error()


def test_batch_create_reports_the_failing_instance_without_a_gpu():
    """kg_batch_create validates every instance before touching the device; the message names the
    instance and carries the parameter check's own text (formatted from the previous message)"""
    lib = kg.load()
    n = 3
    nx = (ctypes.c_int * n)(64, 80, 96)
    ny = (ctypes.c_int * n)(64, 80, 96)
    params = (kg.Params * n)(kg.Params.make(), kg.Params.make(tau=0.0), kg.Params.make())
    out = ctypes.c_void_p()
    assert lib.kg_batch_create(n, nx, ny, params, ctypes.byref(out)) == _lib.KG_ERR_INVALID
    msg = lib.kg_last_error().decode()
    assert msg.startswith("kg_batch_create: instance 1: params:"), msg
    assert not out.value
