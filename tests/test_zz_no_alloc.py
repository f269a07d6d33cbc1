"""npbmz_bt_xsolve_noalloc: the BT x sweep for callers that cannot allocate.

A caller whose device memory is owned by its own pool or garbage collector, or
whose loop cannot take the device-wide synchronisation of cudaFree, cannot let
the library call cudaMalloc for it.  The no-allocation entry point takes its
working memory from one 16 MiB device array compiled into the library.  Here
it runs through the C ABI on device arrays the test owns, twice in a row on
zones of different sizes (the second call reuses the array the first one
left behind), and must match the handle path's NPBMZ_PHASE_XSOLVE within the
FP64 tolerance of the other parity tests.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

import npbmz

pytestmark = pytest.mark.gpu

FAST_REL = 1e-12


def test_noalloc_x_sweep_matches_handle_path_on_two_calls():
    torch = pytest.importorskip("torch")
    L = npbmz.lib()
    nx, ny, nz, nbr = npbmz.zones_from_widths([8, 16], [10, 14], 6)
    geom = npbmz.Geometry(npbmz.BT, nx, ny, nz, nbr, 24, 24, 6, 2, 2)
    dt = 0.010
    ce, _ = npbmz.seeded_coefficients(5, nx, ny, nz, 24, 24, 6, 2, 2)
    p = npbmz.Problem(geom, dt, 0)
    p.setup(ce)
    p.exch_qbc()
    params = np.array([dt, 24, 24, 6, 2, 2], np.float64)
    stream = torch.cuda.current_stream().cuda_stream
    for z in (3, 0):  # 16x14x6 first, then the smaller 8x10x6
        p.phase(npbmz.PHASE_RHS, z)
        u = p.download(npbmz.U, z)
        r = p.download(npbmz.RHS, z)
        p.phase(npbmz.PHASE_XSOLVE, z)
        expect = p.download(npbmz.RHS, z)
        du = torch.tensor(u, device="cuda")
        dr = torch.tensor(r, device="cuda")
        rc = L.npbmz_bt_xsolve_noalloc(int(nx[z]), int(ny[z]), int(nz[z]), params.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                       ctypes.c_void_p(du.data_ptr()), ctypes.c_void_p(dr.data_ptr()), ctypes.c_void_p(stream))
        assert rc == 0, L.npbmz_last_error(None)
        torch.cuda.synchronize()
        got = dr.cpu().numpy()
        err = np.max(np.abs(got - expect)) / np.max(np.abs(expect))
        assert err <= FAST_REL, f"zone {z}: rel err {err:.3e}"
        np.testing.assert_array_equal(du.cpu().numpy(), u)  # u is input only


def test_noalloc_rejects_zones_beyond_its_array():
    torch = pytest.importorskip("torch")
    L = npbmz.lib()
    params = np.array([1e-4, 480, 320, 28, 16, 16], np.float64)
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = L.npbmz_bt_xsolve_noalloc(200, 200, 60, params.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                   ctypes.c_void_p(buf.data_ptr()), ctypes.c_void_p(buf.data_ptr()), None)
    assert rc == -2
    assert b"16777216" in L.npbmz_last_error(None)
