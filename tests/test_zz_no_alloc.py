"""The allocation-free neighbour-count entry point (ccake_neighbour_counts_noalloc)
agrees exactly with the allocating one (ccake_get_neighbours) on two calls in a
row.

It exists for callers that cannot call cudaMalloc while they run; its
scratch is a fixed file-scope device array shared by all calls, so the second
call checks that a call does not depend on what the previous one left there.
This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind(L):
    f = L.ccake_neighbour_counts_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
                  ctypes.c_double, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                  ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int32
    return f


@pytest.mark.parametrize("dim", [2, 3])
def test_noalloc_neighbour_counts_match_allocating_entry_point(dim):
    import torch
    from ccake_gb300 import api, build, ics

    build.build()
    L = api.lib()
    f = _bind(L)
    if dim == 2:
        # lattice spacing 2h/4: four partners of every interior particle sit
        # exactly 2h away, the case the cell edge's margin is for
        p, rc = ics.hotspots_2d(n_side=120, n_hot=8, seed=3)
        lo = (ctypes.c_double * 3)(2 * rc.xmin, 2 * rc.ymin, -rc.hT)
        hi = (ctypes.c_double * 3)(-2 * rc.xmin, -2 * rc.ymin, rc.hT)
    else:
        # (x, y, eta_s) lattice: cells over all three axes, ~280 neighbours
        p, rc = ics.hotspots_3d(n_xy=20, n_eta=16, n_hot=4, seed=3)
        lo = (ctypes.c_double * 3)(rc.xmin, rc.ymin, rc.etamin)
        hi = (ctypes.c_double * 3)(-rc.xmin, -rc.ymin, -rc.etamin)
    n = p.n
    # the allocating entry point: CSR offsets of the full neighbour list
    g = api.GpuHydro(rc)
    g.load(p)
    off, _ = g.neighbours()
    expect = np.diff(off).astype(np.int32)
    g.close()

    dev = torch.device("cuda:0")
    dx = torch.tensor(p.x, dtype=torch.float64, device=dev)
    dy = torch.tensor(p.y, dtype=torch.float64, device=dev)
    de = torch.tensor(p.eta, dtype=torch.float64, device=dev)
    out = torch.empty(n, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        out.fill_(-1)
        st = f(dx.data_ptr(), dy.data_ptr(), de.data_ptr() if dim == 3 else None, n, dim, rc.hT, lo, hi,
               out.data_ptr(), stream)
        assert st == 0, L.ccake_status_string(st)
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), expect)


def test_noalloc_rejects_oversized_input():
    from ccake_gb300 import api, build

    build.build()
    f = _bind(api.lib())
    lo = (ctypes.c_double * 3)(-1, -1, -1)
    hi = (ctypes.c_double * 3)(1, 1, 1)
    # capacity is checked before any pointer is used
    st = f(1, 1, None, (1 << 18) + 1, 2, 0.1, lo, hi, 1, None)
    assert st == 5  # CCAKE_ERR_CAPACITY
