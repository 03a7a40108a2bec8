"""The headless colour ramp (kg_colormap, replacing the per-cell
iUpdateConstantBuffer of src/Kobayashi.cpp:309-345) against the reference's
own colours, and snapshots (kg_save / kg_load)."""
import json

import numpy as np
import pytest

from crystalgrowth_gb300 import Kobayashi, KgError, configs

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


def test_colormap_matches_reference_fp64_build(tmp_path):
    import os
    fx = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref64_colors_64x64.npz"))
    sim = Kobayashi(64, 64, 1e-4)
    sim.set_fields(fx["phi64"], np.zeros((64, 64)), np.zeros((64, 64)))
    viewer = sim.colormap(viewer_order=True)
    assert bits_equal(viewer, fx["rgba64"])
    grid = sim.colormap()
    # grid order: cell (i, j) at i + 64 j; the viewer order reads phi transposed
    assert bits_equal(grid.reshape(64, 64, 4).transpose(1, 0, 2).reshape(-1, 4), viewer)
    # the FP32 build of the reference computes the ramp in float from a float phi: close, not equal
    assert np.abs(viewer - fx["rgba32"]).max() < 5e-2
    sim.close()


def test_colormap_edges_and_rejects_non_square_viewer_order():
    sim = Kobayashi(5, 3, 1e-4)
    phi = np.array([[-0.5, 0.0, 0.45, 0.9, 0.905], [0.95, 0.99, 0.995, 1.0, 1.2], [np.nan, 0.3, 0.6, 0.8, 1e-300]])
    sim.set_fields(phi, np.zeros((3, 5)), np.zeros((3, 5)))
    rgba = sim.colormap()
    assert np.all(rgba[:, 3] == 1.0)
    assert rgba[1, 0] == 0.0 and rgba[8, 2] == np.float32(0.9882353)
    assert np.isnan(rgba[10, 0])
    with pytest.raises(KgError):
        sim.colormap(viewer_order=True)
    sim.close()


def test_snapshot_roundtrip_and_format(tmp_path):
    p = dict(configs.BASE, delta=0.03, theta0=0.4)
    a = Kobayashi(90, 70, p["dt"], params=p)
    a.seed_disks([(45, 35, 6)])
    a.step(123)
    a.iUpdate()
    path = tmp_path / "snap.kgs"
    a.save(path)
    raw = path.read_bytes()
    hdr = json.loads(raw[:4096].decode())
    assert hdr["nx"] == 90 and hdr["ny"] == 70 and hdr["steps"] == 133 and hdr["frames"] == 1
    assert hdr["params"]["theta0"] == 0.4 and hdr["params"]["delta"] == 0.03
    arr = np.frombuffer(raw[4096:], dtype="<f8").reshape(3, 70, 90)
    fa = a.fields()
    for k in range(3):
        assert np.array_equal(arr[k].view(np.uint64), fa[k].view(np.uint64))
    b = Kobayashi(90, 70, 1e-4)
    b.load(path)
    assert b.params() == a.params()
    assert b.counters() == a.counters()
    a.step(77)
    b.step(77)
    for x, y in zip(a.fields(), b.fields()):
        assert np.array_equal(x.view(np.uint64), y.view(np.uint64))
    # a truncated snapshot is rejected before any field reaches the device: the handle is unchanged
    short = tmp_path / "short.kgs"
    short.write_bytes(raw[:-8])
    before = b.fields()
    with pytest.raises(KgError):
        b.load(short)
    for x, y in zip(before, b.fields()):
        assert np.array_equal(x.view(np.uint64), y.view(np.uint64))
    c = Kobayashi(91, 70, 1e-4)
    with pytest.raises(KgError):
        c.load(path)
    with pytest.raises(KgError):
        c.load(tmp_path / "missing.kgs")
    for s in (a, b, c):
        s.close()


@pytest.mark.parametrize("nx,ny", [(130, 70), (33, 17), (1, 1)])
def test_page_locked_transfers_equal_pageable(nx, ny):
    """page-locked host buffers move through the copy kernel, ordinary ones through the copy engine
    (and odd cell counts, which are not whole 16-byte units, always through the copy engine): both
    paths must deliver the same bits, both ways, for the fields, the batch and the colour map"""
    import torch
    from crystalgrowth_gb300 import Batch
    p = dict(configs.BASE)
    rng = np.random.default_rng(nx * 1000 + ny)
    src = [rng.standard_normal((ny, nx)) for _ in range(3)]
    pinned = [torch.empty((ny, nx), dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
    for a, b in zip(pinned, src):
        a[...] = b
    sim = Kobayashi(nx, ny, p["dt"], params=p)
    sim.set_fields(*pinned)
    got = sim.fields()
    for a, b in zip(got, src):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    sim.set_fields(*src)
    sim.step(7)
    plain = sim.fields()
    outp = [torch.empty((ny, nx), dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
    sim.fields(out=outp)
    for a, b in zip(outp, plain):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    sim.close()
    bt = Batch([(nx, ny), (nx + 1, ny)], [p, p])
    bt.set_fields(0, *pinned)
    for a, b in zip(bt.fields(0), src):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    bt.close()
