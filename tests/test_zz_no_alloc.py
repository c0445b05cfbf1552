"""tfg_bin_noalloc: binning for callers that cannot allocate device memory.

Such callers (code running inside another library's stream capture, plugins limited to
a host application's memory pool, real-time loops that cannot afford a cudaMalloc) get
their binning from a statically allocated scratch array instead.  This test checks the
entry point, called through the C ABI with caller-owned device buffers, against the
engine's own load path (tfg_load_particles, which allocates its scratch normally):
cell indices and cell-relative positions must be bit-identical, and the returned cell
order must hold every particle once, sorted by cell and by index inside a cell.  Two
calls in a row check that the shared scratch is reset between calls.  Edge cases (no
particles, a single cell, everything at one point, particles outside the box) are checked
against a numpy restatement of space_setpartp (source/mdcore/src/tfSpace.cpp:432-475) and
a stable sort by cell.  This file is collected last so that a failure here cannot hide
the other tests.
"""
import ctypes as C
import time

import numpy as np
import pytest

from tfg import configs, lib
from tfg.engine import Engine

pytestmark = pytest.mark.gpu


FLT_EPSILON = float(np.finfo(np.float32).eps)


def _setpartp_np(desc, x):
    """space_setpartp in FP32 (no FMA), as engine creation sets the geometry up."""
    f32 = np.float32
    x = np.asarray(x, f32).reshape(-1, 3)
    cell = np.zeros(len(x), np.int64)
    xrel = np.empty_like(x)
    for k in range(3):
        o, dm, c = f32(desc.origin[k]), f32(desc.dim[k]), int(desc.cells[k])
        h = f32(dm / f32(c))
        lo = f32(float(o) * (1.0 + FLT_EPSILON))
        hi = f32(float(f32(dm + o)) * (1.0 - FLT_EPSILON))
        ih = f32(1.0 / float(h))
        xc = np.maximum(lo, np.minimum(hi, x[:, k]))
        ind = np.trunc((xc - o) * ih).astype(np.int64)
        ind = np.clip(ind, 0, c - 1)
        xrel[:, k] = xc - (o + ind.astype(f32) * h)
        cell = cell * c + ind
    return cell.astype(np.int32), xrel


def _bin_noalloc(torch, w):
    return _bin_noalloc_desc(torch, w.desc(), w.x)


def _bin_noalloc_desc(torch, desc, xs):
    xs = np.ascontiguousarray(xs, np.float32).reshape(-1, 3)
    n = len(xs)
    ncells = int(np.prod(list(desc.cells)))
    x = torch.from_numpy(xs).cuda() if n else torch.empty((0, 3), dtype=torch.float32, device="cuda")
    cell = torch.empty(n, dtype=torch.int32, device="cuda")
    xrel = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    order = torch.empty(n, dtype=torch.int32, device="cuda")
    start = torch.full((ncells + 1,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    ptr = (lambda t: t.data_ptr() if n else None)
    rc = lib().tfg_bin_noalloc(C.byref(desc), n, ptr(x), ptr(cell), ptr(xrel), ptr(order), start.data_ptr(), stream)
    assert rc == 0, rc
    torch.cuda.synchronize()
    return cell.cpu().numpy(), xrel.cpu().numpy(), order.cpu().numpy(), start.cpu().numpy()


@pytest.mark.parametrize("make", [lambda: configs.cell_sorting(), lambda: configs.dpd_droplets(n=20000, side=20.0,
                                                                                              radius=6.0)])
def test_bin_noalloc_matches_engine_load(make):
    torch = pytest.importorskip("torch")
    w = make()
    eng = Engine(w.desc())
    eng.load(w.x, type=w.type)
    ref = eng.download()
    ncells = int(np.prod(w.cells))
    for call in range(2):
        cell, xrel, order, start = _bin_noalloc(torch, w)
        assert np.array_equal(cell, ref["cell"]), "call %d: cells differ" % call
        assert np.array_equal(xrel.view(np.uint32), ref["xrel"].view(np.uint32)), "call %d: xrel differs" % call
        counts = np.bincount(cell, minlength=ncells)
        assert start[0] == 0 and np.array_equal(np.diff(start), counts)
        assert np.array_equal(np.sort(order), np.arange(w.n))
        expect = np.lexsort((np.arange(w.n), cell))
        assert np.array_equal(order, expect), "call %d: order differs" % call


def _check_against_numpy(torch, desc, xs):
    cell, xrel, order, start = _bin_noalloc_desc(torch, desc, xs)
    ecell, exrel = _setpartp_np(desc, xs)
    n = len(ecell)
    ncells = int(np.prod(list(desc.cells)))
    assert np.array_equal(cell, ecell)
    assert np.array_equal(xrel.view(np.uint32), exrel.view(np.uint32))
    assert start[0] == 0 and np.array_equal(np.diff(start), np.bincount(ecell, minlength=ncells))
    assert np.array_equal(order, np.lexsort((np.arange(n), ecell)))
    return cell, order, start


def _desc(cells, side=10.0, origin=(0.0, 0.0, 0.0)):
    d = configs.cell_sorting(n=10).desc()
    for k in range(3):
        d.origin[k] = origin[k]
        d.dim[k] = side
        d.cells[k] = cells[k]
    return d


def test_bin_noalloc_no_particles():
    torch = pytest.importorskip("torch")
    d = _desc((4, 5, 6))
    for call in range(2):
        cell, xrel, order, start = _bin_noalloc_desc(torch, d, np.zeros((0, 3), np.float32))
        assert len(order) == 0 and np.array_equal(start, np.zeros(4 * 5 * 6 + 1, np.int32)), "call %d" % call


def test_bin_noalloc_single_cell_and_outside_box():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    # one cell: everything lands in cell 0, in index order
    xs = rng.uniform(-3.0, 13.0, (500, 3)).astype(np.float32)
    _check_against_numpy(torch, _desc((1, 1, 1)), xs)
    # particles outside [origin, origin + dim] are clamped into the boundary cells
    d = _desc((7, 5, 3), side=21.0, origin=(-4.0, 2.5, 0.0))
    xs = rng.uniform(-30.0, 40.0, (3000, 3)).astype(np.float32)
    xs[:10] = np.float32(-1e30)
    xs[10:20] = np.float32(1e30)
    _check_against_numpy(torch, d, xs)


def test_bin_noalloc_crowded_cell_is_linear():
    """All particles at one point: the order inside the crowded cell is by index, and the
    time stays that of a uniform spread (no per-cell quadratic ranking)."""
    torch = pytest.importorskip("torch")
    d = _desc((40, 40, 40), side=40.0)
    few = np.full((300, 3), 17.25, np.float32)
    cell, order, _ = _check_against_numpy(torch, d, few)
    assert len(np.unique(cell)) == 1
    many = np.full((200000, 3), 17.25, np.float32)
    many[::7] = np.float32(3.5)   # a second crowded cell interleaved with the first
    _check_against_numpy(torch, d, many)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _bin_noalloc_desc(torch, d, many)
    dt = time.perf_counter() - t0
    assert dt < 1.0, "crowded binning took %.3f s" % dt


def test_bin_noalloc_largest_sizes():
    """The largest accepted request: TFG_NOALLOC_MAX_PARTICLES particles over
    TFG_NOALLOC_MAX_CELLS cells (three radix passes)."""
    torch = pytest.importorskip("torch")
    d = _desc((64, 64, 64), side=64.0)
    xs = np.random.default_rng(5).uniform(0.0, 64.0, (1048576, 3)).astype(np.float32)
    _check_against_numpy(torch, d, xs)


def test_bin_noalloc_rejects_oversize():
    w = configs.cell_sorting(n=10)
    d = w.desc()
    d.cells[0] = d.cells[1] = d.cells[2] = 100   # 1e6 cells > TFG_NOALLOC_MAX_CELLS
    rc = lib().tfg_bin_noalloc(C.byref(d), 10, None, None, None, None, C.c_void_p(1), None)
    assert rc == -6   # TFG_E_OVERFLOW
    # an axis beyond the limit is refused before the cell count is formed (no overflow)
    d.cells[0] = d.cells[1] = d.cells[2] = 1 << 21
    rc = lib().tfg_bin_noalloc(C.byref(d), 10, None, None, None, None, C.c_void_p(1), None)
    assert rc == -6
    d.cells[0], d.cells[1], d.cells[2] = 1 << 30, 1, 1
    rc = lib().tfg_bin_noalloc(C.byref(d), 10, None, None, None, None, C.c_void_p(1), None)
    assert rc == -6
    d.cells[0], d.cells[1], d.cells[2] = 64, 64, 64
    rc = lib().tfg_bin_noalloc(C.byref(d), 1048577, None, None, None, None, C.c_void_p(1), None)
    assert rc == -6
