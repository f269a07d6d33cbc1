"""npbmz_bt_xsolve_noalloc: the BT x sweep for callers that cannot allocate.

A caller whose device memory is owned by its own pool or garbage collector, or
whose loop cannot take the device-wide synchronisation of cudaFree, cannot let
the library call cudaMalloc for it.  The no-allocation entry point takes its
working memory from one 16 MiB device array compiled into the library.  Here
it runs through the C ABI on device arrays the test owns, three times in a
row on zones of different sizes (each call reuses the array the previous one
left behind), and must match the handle path's NPBMZ_PHASE_XSOLVE within the
FP64 tolerance of the other parity tests.  After the first call (which looks
up the array's address and loads the kernels), the device's free memory and
torch's allocated bytes must not move across the next two calls.  This file
is collected last.
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
    pp = params.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    stream = torch.cuda.current_stream().cuda_stream
    # the handle path's x sweep of zones 3 (16x14x6) and 0 (8x10x6), and the
    # device copies of their inputs, all made before anything is measured
    cases = {}
    for z in (3, 0):
        p.phase(npbmz.PHASE_RHS, z)
        u = p.download(npbmz.U, z)
        r = p.download(npbmz.RHS, z)
        p.phase(npbmz.PHASE_XSOLVE, z)
        cases[z] = (u, r, p.download(npbmz.RHS, z), torch.tensor(u, device="cuda"), torch.empty(r.shape,
                    dtype=torch.float64, device="cuda"))
    torch.cuda.synchronize()

    def run(z):
        u, r, expect, du, dr = cases[z]
        dr.copy_(torch.from_numpy(r))
        rc = L.npbmz_bt_xsolve_noalloc(int(nx[z]), int(ny[z]), int(nz[z]), pp, ctypes.c_void_p(du.data_ptr()),
                                       ctypes.c_void_p(dr.data_ptr()), ctypes.c_void_p(stream))
        assert rc == 0, L.npbmz_last_error(None)
        torch.cuda.synchronize()
        got = dr.cpu().numpy()
        err = np.max(np.abs(got - expect)) / np.max(np.abs(expect))
        assert err <= FAST_REL, f"zone {z}: rel err {err:.3e}"
        np.testing.assert_array_equal(du.cpu().numpy(), u)  # u is input only

    run(3)  # first call on this device: address look-up, kernels loaded
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    run(0)  # two calls in a row, the second on the larger zone again
    run(3)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"device free memory moved by {free0 - free1} bytes across two calls"
    assert torch.cuda.memory_allocated() == alloc0


def test_noalloc_rejects_zones_beyond_its_array():
    torch = pytest.importorskip("torch")
    L = npbmz.lib()
    params = np.array([1e-4, 480, 320, 28, 16, 16], np.float64)
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = L.npbmz_bt_xsolve_noalloc(200, 200, 60, params.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                   ctypes.c_void_p(buf.data_ptr()), ctypes.c_void_p(buf.data_ptr()), None)
    assert rc == -2
    assert b"16777216" in L.npbmz_last_error(None)
