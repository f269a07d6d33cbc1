"""ctypes wrapper of the CPU oracle (test infrastructure only).

The oracle restates the NPBApps.jl BT-MZ/SP-MZ single-rank time step on the
CPU (oracle/npbmz_oracle.cpp).  Only tests/, __graft_entry__.smoke() and the
CPU-baseline leg and reference arm of bench.py use it: to compare against, or
to time the reference's CPU path.  The tangent
library (oracle/npbmz_tangent.cpp) is the same BT and SP restatement with
forward-mode dual numbers: the reference directional derivatives against
which tests check the GPU adjoint.  liblumz_oracle.so (oracle/lumz_oracle.cpp)
restates LU-MZ's SSOR iteration; LuOracle wraps it.
"""
import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB_PATH = _HERE / "_build" / "libnpbmz_oracle.so"
_TAN_PATH = _HERE / "_build" / "libnpbmz_tangent.so"
_LU_PATH = _HERE / "_build" / "liblumz_oracle.so"
_lib = None
_tan = None
_lu = None
TANGENT_NDIR = 16

KIND_BT, KIND_SP = 0, 1


def build(force=False):
    srcs = [_HERE / "npbmz_oracle.cpp", _HERE / "npbmz_tangent.cpp", _HERE / "lumz_oracle.cpp"]
    newest = max(p.stat().st_mtime for p in srcs)
    if force or any(not p.exists() or p.stat().st_mtime < newest for p in (_LIB_PATH, _TAN_PATH, _LU_PATH)):
        subprocess.run(["make", "-s", "-C", str(_HERE)], check=True)
    return _LIB_PATH


def tangent_lib():
    global _tan
    if _tan is None:
        build()
        L = ctypes.CDLL(str(_TAN_PATH))
        ip = ctypes.POINTER(ctypes.c_int)
        dp = ctypes.POINTER(ctypes.c_double)
        L.tangent_objective.argtypes = ([ctypes.c_int] * 2 + [ip, ip, ip, ip, ctypes.c_double] + [ctypes.c_int] * 5 +
                                        [dp, dp, dp, ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, dp])
        _tan = L
    return _tan


def tangent_objective(kind, nx, ny, nz, nbr, dt, gx, gy, gz, xz, yz, u0, forcing, u_target, nsteps, du0=None,
                      dforcing=None):
    """J = 1/2 sum (u_N - u_target)^2 after nsteps BT-MZ (KIND_BT) or SP-MZ
    (KIND_SP) steps and its derivatives along up to 16 directions, by dual
    numbers through the oracle.  Flat dense arrays (zone z: [5][nz][ny][nx],
    zones back to back); du0 / dforcing: (ndir, total) or None.  Returns
    (J, dJ[ndir], u_N)."""
    nx, ny, nz, nbr = (np.ascontiguousarray(a, np.int32) for a in (nx, ny, nz, nbr))
    u0, forcing, u_target = (np.ascontiguousarray(a, np.float64) for a in (u0, forcing, u_target))
    total = u0.size
    seeds = [a for a in (du0, dforcing) if a is not None]
    ndir = seeds[0].shape[0] if seeds else 0
    assert ndir <= TANGENT_NDIR
    du0 = None if du0 is None else np.ascontiguousarray(du0, np.float64).reshape(ndir, total)
    dforcing = None if dforcing is None else np.ascontiguousarray(dforcing, np.float64).reshape(ndir, total)
    J = np.zeros(1)
    dJ = np.zeros(max(ndir, 1))
    uN = np.zeros(total)
    rc = tangent_lib().tangent_objective(kind, len(nx), _ip(nx), _ip(ny), _ip(nz), _ip(nbr), dt, gx, gy, gz, xz, yz,
                                         _dp(u0), _dp(forcing), _dp(u_target), nsteps, ndir,
                                         _dp(du0) if du0 is not None else None,
                                         _dp(dforcing) if dforcing is not None else None, _dp(J), _dp(dJ), _dp(uN))
    assert rc == 0, rc
    return float(J[0]), dJ[:ndir], uN


def tangent_bt_objective(*args, **kw):
    """tangent_objective for BT-MZ."""
    return tangent_objective(KIND_BT, *args, **kw)


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
        L.oracle_seeded_coefficients.argtypes = [ctypes.c_uint64, ctypes.c_int, ip, ip, ip] + [ctypes.c_int] * 5 + [dp]
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


def seeded_coefficients(seed, nx, ny, nz, gx, gy, gz, xz, yz):
    """Seeded 5x13 manufactured-solution coefficients with the energy-row
    positivity rule (oracle_seeded_coefficients); returns (ce, doublings)."""
    nx, ny, nz = (np.ascontiguousarray(a, np.int32) for a in (nx, ny, nz))
    ce = np.zeros((5, 13))
    e = lib().oracle_seeded_coefficients(seed, len(nx), _ip(nx), _ip(ny), _ip(nz), gx, gy, gz, xz, yz, _dp(ce))
    if e < 0:
        raise ValueError("no positivity-preserving energy scale found")
    return ce, e


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

    def get_all(self, which):
        """One field of every zone, flat dense (zones back to back)."""
        return np.concatenate([self.get(which, z).reshape(-1) for z in range(self.nzones)])

    def get(self, which, zone):
        z = zone
        out = np.zeros((5, int(self.nz[z]), int(self.ny[z]), int(self.nx[z])))
        lib().oracle_get(self._h, which, z, _dp(out))
        return out

    def set(self, which, zone, arr):
        a = np.ascontiguousarray(arr, np.float64)
        assert a.shape == (5, int(self.nz[zone]), int(self.ny[zone]), int(self.nx[zone]))
        lib().oracle_set(self._h, which, zone, _dp(a))


def lu_lib():
    global _lu
    if _lu is None:
        build()
        L = ctypes.CDLL(str(_LU_PATH))
        ip = ctypes.POINTER(ctypes.c_int)
        dp = ctypes.POINTER(ctypes.c_double)
        L.lu_oracle_zone_setup.argtypes = [ctypes.c_int] * 5 + [ctypes.c_double, ip, ip, ip, ip]
        L.lu_oracle_create.restype = ctypes.c_void_p
        L.lu_oracle_create.argtypes = [ctypes.c_int, ip, ip, ip, ip, ctypes.c_double, ctypes.c_double, dp,
                                       ctypes.c_int]
        L.lu_oracle_destroy.argtypes = [ctypes.c_void_p]
        L.lu_oracle_iterate.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.lu_oracle_phase.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.lu_oracle_verify.argtypes = [ctypes.c_void_p] + [dp] * 6
        L.lu_oracle_get.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, dp]
        L.lu_oracle_set.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, dp]
        _lu = L
    return _lu


# LU-MZ phases of lu_oracle_phase
LU_RHS, LU_SCALE, LU_LOWER, LU_UPPER, LU_UPDATE, LU_EXCH, LU_SSOR = range(7)


def lu_zone_setup(gx, gy, gz, xz, yz, ratio=1.0):
    n = xz * yz
    nx, ny, nz = (np.zeros(n, np.int32) for _ in range(3))
    nbr = np.zeros(4 * n, np.int32)
    rc = lu_lib().lu_oracle_zone_setup(gx, gy, gz, xz, yz, ratio, _ip(nx), _ip(ny), _ip(nz), _ip(nbr))
    assert rc == 0, rc
    return nx, ny, nz, nbr


class LuOracle:
    """One LU-MZ problem held by the CPU oracle (setbv, setiv, erhs, rhs done)."""

    def __init__(self, nx, ny, nz, nbr, dt, omega=1.2, ce=None, faces_npb=False):
        self.nx, self.ny, self.nz, self.nbr = (np.ascontiguousarray(a, np.int32) for a in (nx, ny, nz, nbr))
        self.nzones = len(self.nx)
        self.ce = None if ce is None else np.ascontiguousarray(ce, np.float64).reshape(65)
        self._h = lu_lib().lu_oracle_create(self.nzones, _ip(self.nx), _ip(self.ny), _ip(self.nz), _ip(self.nbr),
                                            dt, omega, _dp(self.ce) if self.ce is not None else None,
                                            int(faces_npb))

    def __del__(self):
        if getattr(self, "_h", None):
            lu_lib().lu_oracle_destroy(self._h)
            self._h = None

    def iterate(self, niter):
        lu_lib().lu_oracle_iterate(self._h, niter)

    def phase(self, phase, zone=-1):
        rc = lu_lib().lu_oracle_phase(self._h, phase, zone)
        assert rc == 0, rc

    def verify(self, per_zone=False):
        xcr, xce, xci = np.zeros(5), np.zeros(5), np.zeros(1)
        z = [np.zeros(5 * self.nzones), np.zeros(5 * self.nzones), np.zeros(self.nzones)] if per_zone else None
        lu_lib().lu_oracle_verify(self._h, _dp(xcr), _dp(xce), _dp(xci), *((_dp(a) for a in z) if z else (None,) * 3))
        if per_zone:
            return xcr, xce, float(xci[0]), z[0].reshape(-1, 5), z[1].reshape(-1, 5), z[2]
        return xcr, xce, float(xci[0])

    def get(self, which, zone):
        out = np.zeros((5, int(self.nz[zone]), int(self.ny[zone]), int(self.nx[zone])))
        lu_lib().lu_oracle_get(self._h, which, zone, _dp(out))
        return out

    def get_all(self, which):
        return np.concatenate([self.get(which, z).reshape(-1) for z in range(self.nzones)])

    def set(self, which, zone, arr):
        a = np.ascontiguousarray(arr, np.float64)
        assert a.shape == (5, int(self.nz[zone]), int(self.ny[zone]), int(self.nx[zone]))
        lu_lib().lu_oracle_set(self._h, which, zone, _dp(a))
