"""tfg_bin_noalloc: binning for callers that cannot allocate device memory.

Such callers (code running inside another library's stream capture, plugins limited to
a host application's memory pool, real-time loops that cannot afford a cudaMalloc) get
their binning from a statically allocated scratch array instead.  This test checks the
entry point, called through the C ABI with caller-owned device buffers, against the
engine's own load path (tfg_load_particles, which allocates its scratch normally):
cell indices and cell-relative positions must be bit-identical, and the returned cell
order must hold every particle once, sorted by cell and by index inside a cell.  Two
calls in a row check that the shared scratch is reset between calls.  This file is
collected last so that a failure here cannot hide the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from tfg import configs, lib
from tfg.engine import Engine

pytestmark = pytest.mark.gpu


def _bin_noalloc(torch, w):
    n = w.n
    desc = w.desc()
    ncells = int(np.prod(w.cells))
    x = torch.from_numpy(np.ascontiguousarray(w.x, np.float32)).cuda()
    cell = torch.empty(n, dtype=torch.int32, device="cuda")
    xrel = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    order = torch.empty(n, dtype=torch.int32, device="cuda")
    start = torch.empty(ncells + 1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib().tfg_bin_noalloc(C.byref(desc), n, x.data_ptr(), cell.data_ptr(), xrel.data_ptr(), order.data_ptr(),
                               start.data_ptr(), stream)
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


def test_bin_noalloc_rejects_oversize():
    w = configs.cell_sorting(n=10)
    d = w.desc()
    d.cells[0] = d.cells[1] = d.cells[2] = 100   # 1e6 cells > TFG_NOALLOC_MAX_CELLS
    rc = lib().tfg_bin_noalloc(C.byref(d), 10, None, None, None, None, C.c_void_p(1), None)
    assert rc == -6   # TFG_E_OVERFLOW
