"""ctypes wrapper of the CPU oracle (test infrastructure only).

The oracle restates the NPBApps.jl BT-MZ/SP-MZ single-rank time step on the
CPU (oracle/npbmz_oracle.cpp).  Only tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py use it, always as the checker.
"""
import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB_PATH = _HERE / "_build" / "libnpbmz_oracle.so"
_lib = None

KIND_BT, KIND_SP = 0, 1


def build(force=False):
    if force or not _LIB_PATH.exists() or _LIB_PATH.stat().st_mtime < (_HERE / "npbmz_oracle.cpp").stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(_HERE)], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(_LIB_PATH))
        ip = ctypes.POINTER(ctypes.c_int)
        dp = ctypes.POINTER(ctypes.c_double)
        L.oracle_zone_setup.argtypes = [ctypes.c_int] * 6 + [ctypes.c_double, ip, ip, ip, ip]
        L.oracle_create.restype = ctypes.c_void_p
        L.oracle_create.argtypes = [ctypes.c_int, ctypes.c_int, ip, ip, ip, ip, ctypes.c_double] + [ctypes.c_int] * 5 + [dp, ctypes.c_int]
        L.oracle_destroy.argtypes = [ctypes.c_void_p]
        L.oracle_step.argtypes = [ctypes.c_void_p, ctypes.c_int, dp]
        L.oracle_verify.argtypes = [ctypes.c_void_p, dp, dp]
        L.oracle_phase.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.oracle_get.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, dp]
        L.oracle_set.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, dp]
        _lib = L
    return _lib


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def zone_setup(kind, gx, gy, gz, xz, yz, ratio):
    n = xz * yz
    nx = np.zeros(n, np.int32); ny = np.zeros(n, np.int32); nz = np.zeros(n, np.int32)
    nbr = np.zeros(4 * n, np.int32)
    lib().oracle_zone_setup(kind, gx, gy, gz, xz, yz, ratio, _ip(nx), _ip(ny), _ip(nz), _ip(nbr))
    return nx, ny, nz, nbr


class Oracle:
    """One multi-zone problem held by the CPU oracle."""

    def __init__(self, kind, nx, ny, nz, nbr, dt, gx, gy, gz, xz, yz, ce, solve_float=False):
        self.kind = kind
        self.nx = np.ascontiguousarray(nx, np.int32)
        self.ny = np.ascontiguousarray(ny, np.int32)
        self.nz = np.ascontiguousarray(nz, np.int32)
        self.nbr = np.ascontiguousarray(nbr, np.int32)
        self.ce = np.ascontiguousarray(ce, np.float64).reshape(65)
        self.dt = dt
        self.nzones = len(self.nx)
        self._h = lib().oracle_create(kind, self.nzones, _ip(self.nx), _ip(self.ny), _ip(self.nz), _ip(self.nbr),
                                      dt, gx, gy, gz, xz, yz, _dp(self.ce), int(solve_float))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_destroy(self._h)
            self._h = None

    def step(self, nsteps=1, norms=False):
        out = np.zeros(10 * nsteps) if norms else None
        lib().oracle_step(self._h, nsteps, _dp(out) if norms else None)
        return out.reshape(nsteps, 2, 5) if norms else None

    def verify(self):
        xcr = np.zeros(5); xce = np.zeros(5)
        lib().oracle_verify(self._h, _dp(xcr), _dp(xce))
        return xcr, xce

    def phase(self, phase, zone=0):
        rc = lib().oracle_phase(self._h, phase, zone)
        assert rc == 0, rc

    def get(self, which, zone):
        z = zone
        out = np.zeros((5, int(self.nz[z]), int(self.ny[z]), int(self.nx[z])))
        lib().oracle_get(self._h, which, z, _dp(out))
        return out

    def set(self, which, zone, arr):
        a = np.ascontiguousarray(arr, np.float64)
        assert a.shape == (5, int(self.nz[zone]), int(self.ny[zone]), int(self.nx[zone]))
        lib().oracle_set(self._h, which, zone, _dp(a))
