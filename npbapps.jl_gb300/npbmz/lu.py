"""ctypes binding of the LU-MZ SSOR iteration (include/npbmz_lu.h).

Names mirror the reference's LU driver (src/LU/lu-node.jl, src/LU/ssor.jl):
`LuProblem.exch_qbc()`, `LuProblem.ssor(iz)`, `LuProblem.iterate(niter)`,
`LuProblem.verify()` and `go(cls)`, which runs a class and checks it against
the reference's verification norms (src/LU/verify.jl, epsilon 1e-8).
"""
import ctypes
import json
from pathlib import Path

import numpy as np

from . import CLASSES, LAYOUT_DENSE, LAYOUT_REF, NpbmzError, lib as _core_lib

LU_EXPORTS = [
    "npbmz_lu_zone_setup", "npbmz_lu_create", "npbmz_lu_setup", "npbmz_lu_upload", "npbmz_lu_download",
    "npbmz_lu_exch_qbc", "npbmz_lu_ssor", "npbmz_lu_iterate", "npbmz_lu_verify", "npbmz_lu_phase",
    "npbmz_lu_set_stream", "npbmz_lu_synchronize", "npbmz_lu_launches_per_iteration", "npbmz_lu_profile",
    "npbmz_lu_last_error", "npbmz_lu_destroy", "npbmz_lu_state_check",
]
ERR_STATE = -3  # NPBMZ_LU_ERR_STATE
STATE_DENSITY, STATE_PRESSURE, STATE_NONFINITE = 1, 2, 4

# flags, fields and phases (include/npbmz_lu.h)
FACES_NPB = 0x1
GRAPH = 0x2
FMA = 0x4
U, RSD, FRCT = 0, 1, 2
PHASE_RHS, PHASE_SCALE, PHASE_LOWER, PHASE_UPPER, PHASE_UPDATE, PHASE_EXCH, PHASE_SSOR = range(7)
PROFILE_PHASES = ("exch", "jac", "lower", "upper", "update", "rhs")
OMEGA_DEFAULT = 1.2  # src/LU/lu_data.jl

_typed = False


def lib():
    """libnpbmz_gpu.so with the LU entry points typed."""
    global _typed
    L = _core_lib()
    if not _typed:
        ip = ctypes.POINTER(ctypes.c_int)
        dp = ctypes.POINTER(ctypes.c_double)
        vp = ctypes.c_void_p
        L.npbmz_lu_zone_setup.argtypes = [ctypes.c_int] * 5 + [ctypes.c_double, ip, ip, ip, ip]
        L.npbmz_lu_create.argtypes = [ctypes.c_int, ip, ip, ip, ip, dp, ctypes.c_int, ctypes.POINTER(vp)]
        L.npbmz_lu_setup.argtypes = [vp, dp]
        L.npbmz_lu_upload.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.npbmz_lu_download.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.npbmz_lu_exch_qbc.argtypes = [vp]
        L.npbmz_lu_ssor.argtypes = [vp, ctypes.c_int]
        L.npbmz_lu_iterate.argtypes = [vp, ctypes.c_int, dp]
        L.npbmz_lu_verify.argtypes = [vp, dp, dp, dp]
        L.npbmz_lu_phase.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        L.npbmz_lu_set_stream.argtypes = [vp, vp]
        L.npbmz_lu_synchronize.argtypes = [vp]
        L.npbmz_lu_launches_per_iteration.argtypes = [vp]
        L.npbmz_lu_profile.argtypes = [vp, ctypes.c_int, dp]
        L.npbmz_lu_last_error.argtypes = [vp]
        L.npbmz_lu_last_error.restype = ctypes.c_char_p
        L.npbmz_lu_destroy.argtypes = [vp]
        L.npbmz_lu_state_check.argtypes = [vp] + [ip] * 5
        _typed = True
    return L


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def lu_zone_setup(gx, gy, gz, x_zones, y_zones, ratio=1.0):
    """src/LU/zone_setup.jl: (nx, ny, nz, nbr) with nbr = west, east, south,
    north per zone (0-based)."""
    n = x_zones * y_zones
    nx, ny, nz = (np.zeros(n, np.int32) for _ in range(3))
    nbr = np.zeros(4 * n, np.int32)
    rc = lib().npbmz_lu_zone_setup(gx, gy, gz, x_zones, y_zones, ratio, _ip(nx), _ip(ny), _ip(nz), _ip(nbr))
    if rc != 0:
        raise NpbmzError(f"npbmz_lu_zone_setup failed for {gx}x{gy}x{gz}, {x_zones}x{y_zones} zones: "
                         + lib().npbmz_lu_last_error(None).decode())
    return nx, ny, nz, nbr


def ref_elems(nx, ny, nz):
    """Doubles in the reference's [1:5, -1:nx+2, -1:ny+2, 1:nz] array."""
    return 5 * (nx + 4) * (ny + 4) * nz


class LuProblem:
    """One LU-MZ problem on the GPU (a libnpbmz_gpu.so LU handle)."""

    def __init__(self, nx, ny, nz, nbr, dt, omega=OMEGA_DEFAULT, flags=0, niter=None):
        self.nx, self.ny, self.nz, self.nbr = (np.ascontiguousarray(a, np.int32) for a in (nx, ny, nz, nbr))
        self.nzones = len(self.nx)
        self.dt, self.omega, self.flags, self.niter = dt, omega, flags, niter
        h = ctypes.c_void_p()
        params = np.array([dt, omega], np.float64)
        rc = lib().npbmz_lu_create(self.nzones, _ip(self.nx), _ip(self.ny), _ip(self.nz), _ip(self.nbr),
                                   _dp(params), flags, ctypes.byref(h))
        if rc != 0 or not h.value:
            raise NpbmzError("npbmz_lu_create failed: " + lib().npbmz_lu_last_error(None).decode())
        self._h = h

    @classmethod
    def from_class(cls, cls_name, flags=0):
        niter, dt, ratio, xz, yz, gx, gy, gz = CLASSES["LU"][cls_name]
        return cls(*lu_zone_setup(gx, gy, gz, xz, yz, ratio), dt, flags=flags, niter=niter)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().npbmz_lu_destroy(h)
            self._h = None

    def close(self):
        self.__del__()

    def _check(self, rc, what):
        if rc != 0:
            raise NpbmzError(f"{what}: " + lib().npbmz_lu_last_error(self._h).decode(), rc)

    def state_check(self):
        """(bits, (zone, i, j, k)) of the last iterate call's state check."""
        v = [ctypes.c_int(0) for _ in range(5)]
        self._check(lib().npbmz_lu_state_check(self._h, *[ctypes.byref(x) for x in v]), "state_check")
        return v[0].value, tuple(x.value for x in v[1:])

    @property
    def points(self):
        return int(np.sum(self.nx.astype(np.int64) * self.ny * self.nz))

    def setup(self, ce=None):
        c = None if ce is None else np.ascontiguousarray(ce, np.float64).reshape(65)
        self._check(lib().npbmz_lu_setup(self._h, _dp(c) if c is not None else None), "setup")

    def exch_qbc(self):
        self._check(lib().npbmz_lu_exch_qbc(self._h), "exch_qbc")

    def ssor(self, iz=-1):
        self._check(lib().npbmz_lu_ssor(self._h, iz), "ssor")

    def phase(self, phase, zone=-1):
        self._check(lib().npbmz_lu_phase(self._h, phase, zone), "phase")

    def iterate(self, niter, norms=False):
        out = np.zeros(5 * niter) if norms and niter else None
        self._check(lib().npbmz_lu_iterate(self._h, niter, _dp(out) if out is not None else None), "iterate")
        return out.reshape(niter, 5) if out is not None else None

    def verify(self):
        xcr, xce, xci = np.zeros(5), np.zeros(5), np.zeros(1)
        self._check(lib().npbmz_lu_verify(self._h, _dp(xcr), _dp(xce), _dp(xci)), "verify")
        return xcr, xce, float(xci[0])

    def synchronize(self):
        self._check(lib().npbmz_lu_synchronize(self._h), "synchronize")

    def set_stream(self, stream_ptr):
        self._check(lib().npbmz_lu_set_stream(self._h, ctypes.c_void_p(stream_ptr)), "set_stream")

    def launches_per_iteration(self):
        return int(lib().npbmz_lu_launches_per_iteration(self._h))

    def profile(self, niter):
        out = np.zeros(len(PROFILE_PHASES))
        self._check(lib().npbmz_lu_profile(self._h, niter, _dp(out)), "profile")
        return dict(zip(PROFILE_PHASES, out.tolist()))

    def download(self, zone, field, layout=LAYOUT_DENSE, out=None):
        if layout == LAYOUT_DENSE:
            shape = (5, int(self.nz[zone]), int(self.ny[zone]), int(self.nx[zone]))
            a = np.empty(shape) if out is None else out
        else:
            a = np.zeros(ref_elems(int(self.nx[zone]), int(self.ny[zone]), int(self.nz[zone]))) if out is None else out
        self._check(lib().npbmz_lu_download(self._h, zone, field, layout, a.ctypes.data), "download")
        return a

    def upload(self, zone, field, arr, layout=LAYOUT_DENSE):
        a = np.ascontiguousarray(arr, np.float64)
        self._check(lib().npbmz_lu_upload(self._h, zone, field, layout, a.ctypes.data), "upload")

    def download_all(self, field):
        return [self.download(z, field) for z in range(self.nzones)]

    def flatten(self, zones):
        return np.concatenate([a.reshape(-1) for a in zones])


def golden(cls_name):
    """The reference's LU-MZ verification values (src/LU/verify.jl)."""
    path = Path(__file__).resolve().parents[2] / "tests" / "golden" / "npb_golden_norms.json"
    d = json.loads(path.read_text())["LU"].get(cls_name)
    return None if d is None else (np.array(d["xcr"]), np.array(d["xce"]), d["xci"], d["dt"], d["niter"])


def go(cls_name, flags=FACES_NPB | GRAPH, niter=None, verbose=False):
    """The reference's LU-MZ run (src/LU/lu-driver.jl go, lu-node.jl perform)
    on the GPU: setup, niter iterations of exch_qbc + ssor, verify.  Returns
    (xcr, xce, xci, verified) with verified per src/LU/verify.jl (epsilon
    1e-8), or None when the class has no golden values.  The default flags
    copy NPB-MZ's face planes, with which the reference's own golden values
    are reached (see NPBMZ_LU_FACES_NPB)."""
    p = LuProblem.from_class(cls_name, flags)
    p.setup()
    n = p.niter if niter is None else niter
    p.iterate(n)
    xcr, xce, xci = p.verify()
    g = golden(cls_name)
    verified = None
    if g is not None and n == g[4]:
        rel = lambda a, b: np.abs((np.asarray(a) - b) / b)  # noqa: E731
        verified = bool(np.all(rel(xcr, g[0]) <= 1e-8) and np.all(rel(xce, g[1]) <= 1e-8) and rel(xci, g[2]) <= 1e-8)
    if verbose:
        print(f"LU-MZ class {cls_name}: {p.nzones} zones, {n} iterations")
        print("xcr", xcr, "\nxce", xce, "\nxci", xci, "\nverified", verified)
    p.close()
    return xcr, xce, xci, verified
