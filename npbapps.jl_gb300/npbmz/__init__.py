"""npbmz -- host-side mirror of the NPBApps.jl BT-MZ / SP-MZ time-step interface
over the C ABI of libnpbmz_gpu.so (include/npbmz.h).

The reference's seam is the pair of calls in the node time loop
(src/BT/bt-node.jl:286-395): ``exch_qbc(...)`` over all zones, then
``adi(iz, ...)`` per zone.  This module keeps those names:

    p = Problem.from_class("BT", "S")        # zone_setup + alloc + set_constants
    p.setup()                                # initialize + exact_rhs on the GPU
    for step in range(p.niter):
        exch_qbc(p)                          # zone-face exchange, on the device
        adi(p)                               # all zones batched (or adi(p, iz))
    xcr, xce = p.verify()                    # verify's node part

and ``go(kind, cls)`` runs the reference's node protocol end to end
(src/BT/bt-node.jl:93-426).  Every call checks the C status and raises
``NpbmzError`` with the library's message; nothing here falls back to a CPU
path -- without the CUDA library or a GPU the calls fail.
"""
from __future__ import annotations

import ctypes
import json
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import build as _build

BT, SP = 0, 1
KINDS = {"BT": BT, "SP": SP}

EXACT, MIXED, PERZONE, GRAPH, PERSIST, FP32_NOREFINE, REFINE_FP64, RHS_DF = 0x1, 0x2, 0x4, 0x8, 0x10, 0x20, 0x40, 0x80
U, RHS, FORCING = 0, 1, 2
LAYOUT_DENSE, LAYOUT_REF = 0, 1
PHASE_RHS, PHASE_XSOLVE, PHASE_YSOLVE, PHASE_ZSOLVE, PHASE_ADD, PHASE_EXCH, PHASE_RHSONLY = range(7)

# Exported symbols of include/npbmz.h
EXPORTS = [
    "npbmz_zone_setup", "npbmz_seeded_coefficients", "npbmz_create", "npbmz_setup", "npbmz_upload",
    "npbmz_download", "npbmz_upload_async", "npbmz_download_async", "npbmz_exch_qbc", "npbmz_adi", "npbmz_step",
    "npbmz_verify", "npbmz_phase", "npbmz_set_stream", "npbmz_synchronize", "npbmz_autotune",
    "npbmz_fp64_peak", "npbmz_launches_per_step", "npbmz_device_bytes", "npbmz_describe", "npbmz_last_error", "npbmz_destroy",
    "npbmz_bt_xsolve_noalloc", "npbmz_adjoint", "npbmz_step_profile", "npbmz_set_step_groups",
    "npbmz_step_download", "npbmz_face_plan", "npbmz_pack_faces", "npbmz_unpack_faces", "npbmz_set_step_overlap",
    "npbmz_set_copy_fusion", "npbmz_state_check", "npbmz_step_inout", "npbmz_math_check",
]
STATE_DENSITY, STATE_PRESSURE, STATE_NONFINITE = 1, 2, 4
REMOTE = -1  # NPBMZ_REMOTE: a face whose neighbour zone lives on another rank
PROF_PHASES = ("exch", "prim", "rhs", "x", "y", "z")

# Problem classes (src/BT/classes.jl:15-24, src/SP/classes.jl:16-25):
# niter, dt, ratio, x_zones, y_zones, gx, gy, gz
CLASSES = {
    "BT": {
        "S": (60, 0.010, 3.0, 2, 2, 24, 24, 6),
        "W": (200, 0.0008, 4.5, 4, 4, 64, 64, 8),
        "A": (200, 0.0008, 4.5, 4, 4, 128, 128, 16),
        "B": (200, 0.0003, 4.5, 8, 8, 304, 208, 17),
        "C": (200, 0.0001, 4.5, 16, 16, 480, 320, 28),
        "D": (250, 0.00002, 4.5, 32, 32, 1632, 1216, 34),
        "E": (250, 0.000004, 4.5, 64, 64, 4224, 3456, 92),
        "F": (250, 0.000001, 4.5, 128, 128, 12032, 8960, 250),
    },
    "SP": {
        "S": (100, 0.015, 1.0, 2, 2, 24, 24, 6),
        "W": (400, 0.0015, 1.0, 4, 4, 64, 64, 8),
        "A": (400, 0.0015, 1.0, 4, 4, 128, 128, 16),
        "B": (400, 0.001, 1.0, 8, 8, 304, 208, 17),
        "C": (400, 0.00067, 1.0, 16, 16, 480, 320, 28),
        "D": (500, 0.0003, 1.0, 32, 32, 1632, 1216, 34),
        "E": (500, 0.0002, 1.0, 64, 64, 4224, 3456, 92),
        "F": (500, 0.0001, 1.0, 128, 128, 12032, 8960, 250),
    },
    # LU-MZ (src/LU/classes.jl): itmax, dt, ratio, 4x4 zones; omega 1.2 (src/LU/lu_data.jl)
    "LU": {
        "S": (50, 0.5, 1.0, 4, 4, 24, 24, 6),
        "W": (300, 1.5e-3, 1.0, 4, 4, 64, 64, 8),
        "A": (250, 2.0, 1.0, 4, 4, 128, 128, 16),
        "B": (250, 2.0, 1.0, 4, 4, 304, 208, 17),
        "C": (250, 2.0, 1.0, 4, 4, 480, 320, 28),
        "D": (300, 1.0, 1.0, 4, 4, 1632, 1216, 34),
        "E": (300, 0.5, 1.0, 4, 4, 4224, 3456, 92),
        "F": (300, 0.2, 1.0, 4, 4, 12032, 8960, 250),
    },
}

# The reference's fixed exact-solution coefficients (src/BT/set_constants.jl:47-51), row-major [5][13].
CE_REFERENCE = np.array([
    [2.0, 0.0, 0.0, 4.0, 5.0, 3.0, 0.5, 0.02, 0.01, 0.03, 0.5, 0.4, 0.3],
    [1.0, 0.0, 0.0, 0.0, 1.0, 2.0, 3.0, 0.01, 0.03, 0.02, 0.4, 0.3, 0.5],
    [2.0, 2.0, 0.0, 0.0, 0.0, 2.0, 3.0, 0.04, 0.03, 0.05, 0.3, 0.5, 0.4],
    [2.0, 2.0, 0.0, 0.0, 0.0, 2.0, 3.0, 0.03, 0.05, 0.04, 0.2, 0.1, 0.3],
    [5.0, 4.0, 3.0, 2.0, 0.1, 0.4, 0.3, 0.05, 0.04, 0.03, 0.1, 0.3, 0.2],
])


ERR_STATE = -3  # NPBMZ_ERR_STATE: the state check found a bad density or pressure


class NpbmzError(RuntimeError):
    """A failed call: the library's message; `code` is its status."""

    def __init__(self, msg, code=-1):
        super().__init__(msg)
        self.code = code


_lib = None


def lib_path() -> Path:
    return _build.LIB


def lib(build_if_missing: bool = True):
    """Load libnpbmz_gpu.so (building it in-tree if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        _build.build()
    path = lib_path()
    if not path.exists():
        raise NpbmzError(f"{path} is missing: run npbmz.build.build()")
    L = ctypes.CDLL(str(path))
    ip = ctypes.POINTER(ctypes.c_int)
    dp = ctypes.POINTER(ctypes.c_double)
    vp = ctypes.c_void_p
    L.npbmz_zone_setup.argtypes = [ctypes.c_int] * 6 + [ctypes.c_double, ip, ip, ip, ip]
    L.npbmz_seeded_coefficients.argtypes = [ctypes.c_uint64, ctypes.c_int, ip, ip, ip] + [ctypes.c_int] * 5 + [dp]
    L.npbmz_create.argtypes = [ctypes.c_int, ctypes.c_int, ip, ip, ip, ip, dp, ctypes.c_int, ctypes.POINTER(vp)]
    L.npbmz_setup.argtypes = [vp, dp]
    for f in ("npbmz_upload", "npbmz_download", "npbmz_upload_async", "npbmz_download_async"):
        getattr(L, f).argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    L.npbmz_exch_qbc.argtypes = [vp]
    L.npbmz_adi.argtypes = [vp, ctypes.c_int]
    L.npbmz_step.argtypes = [vp, ctypes.c_int, dp]
    L.npbmz_step_download.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    L.npbmz_step_inout.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    L.npbmz_math_check.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp]
    L.npbmz_verify.argtypes = [vp, dp, dp]
    L.npbmz_phase.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.npbmz_set_stream.argtypes = [vp, vp]
    L.npbmz_synchronize.argtypes = [vp]
    L.npbmz_autotune.argtypes = [vp]
    L.npbmz_fp64_peak.argtypes = [dp]
    L.npbmz_launches_per_step.argtypes = [vp]
    L.npbmz_device_bytes.argtypes = [vp]
    L.npbmz_device_bytes.restype = ctypes.c_int64
    L.npbmz_describe.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    L.npbmz_last_error.argtypes = [vp]
    L.npbmz_last_error.restype = ctypes.c_char_p
    L.npbmz_destroy.argtypes = [vp]
    L.npbmz_bt_xsolve_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, vp, vp, vp]
    L.npbmz_adjoint.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp, dp, dp, dp]
    L.npbmz_step_profile.argtypes = [vp, ctypes.c_int, dp]
    L.npbmz_set_step_groups.argtypes = [vp, ctypes.c_int]
    L.npbmz_set_step_overlap.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.npbmz_set_copy_fusion.argtypes = [vp, ctypes.c_int]
    L.npbmz_state_check.argtypes = [vp] + [ip] * 5
    i64p = ctypes.POINTER(ctypes.c_int64)
    L.npbmz_face_plan.argtypes = [vp, ctypes.c_int, ip, ctypes.c_int, ip, i64p, i64p]
    L.npbmz_pack_faces.argtypes = [vp, vp]
    L.npbmz_unpack_faces.argtypes = [vp, vp]
    _lib = L
    return L


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def zone_setup(kind: int, gx: int, gy: int, gz: int, x_zones: int, y_zones: int, ratio: float):
    """Zone sizes and periodic neighbours (src/BT/zone_setup.jl:1-77)."""
    n = x_zones * y_zones
    nx, ny, nz = (np.zeros(n, np.int32) for _ in range(3))
    nbr = np.zeros(4 * n, np.int32)
    rc = lib().npbmz_zone_setup(kind, gx, gy, gz, x_zones, y_zones, ratio, _ip(nx), _ip(ny), _ip(nz), _ip(nbr))
    if rc != 0:
        raise NpbmzError("npbmz_zone_setup: bad arguments")
    return nx, ny, nz, nbr


def zones_from_widths(xw, yw, gz):
    """Zone geometry from explicit x / y zone widths (periodic neighbours as in
    src/BT/zone_setup.jl:61-68); for grids the reference's single ratio cannot
    produce."""
    xz, yz = len(xw), len(yw)
    n = xz * yz
    nx, ny, nz = (np.zeros(n, np.int32) for _ in range(3))
    nbr = np.zeros(4 * n, np.int32)
    for j in range(yz):
        for i in range(xz):
            z = i + j * xz
            nx[z], ny[z], nz[z] = xw[i], yw[j], gz
            nbr[4 * z + 0] = (i - 1) % xz + j * xz
            nbr[4 * z + 1] = (i + 1) % xz + j * xz
            nbr[4 * z + 2] = i + ((j - 1) % yz) * xz
            nbr[4 * z + 3] = i + ((j + 1) % yz) * xz
    return nx, ny, nz, nbr


def seeded_coefficients(seed, nx, ny, nz, gx, gy, gz, x_zones, y_zones):
    """Seeded 5x13 manufactured-solution coefficients with the positivity rule
    of npbmz_seeded_coefficients; returns (ce, energy_scale_exponent)."""
    ce = np.zeros((5, 13))
    nx = np.ascontiguousarray(nx, np.int32); ny = np.ascontiguousarray(ny, np.int32)
    nz = np.ascontiguousarray(nz, np.int32)
    e = lib().npbmz_seeded_coefficients(seed, len(nx), _ip(nx), _ip(ny), _ip(nz), gx, gy, gz, x_zones, y_zones, _dp(ce))
    if e < 0:
        raise NpbmzError("no positivity-preserving energy scale found")
    return ce, e


@dataclass
class Geometry:
    kind: int
    nx: np.ndarray
    ny: np.ndarray
    nz: np.ndarray
    nbr: np.ndarray
    gx: int
    gy: int
    gz: int
    x_zones: int
    y_zones: int

    @property
    def nzones(self):
        return len(self.nx)

    @property
    def points(self):
        return int(np.sum(self.nx.astype(np.int64) * self.ny * self.nz))


class Problem:
    """One multi-zone BT-MZ or SP-MZ problem resident on the current GPU."""

    def __init__(self, geom: Geometry, dt: float, flags: int = 0, niter: int = 0):
        self.geom = geom
        self.kind = geom.kind
        self.dt = float(dt)
        self.flags = flags
        self.niter = niter
        self._nx = np.ascontiguousarray(geom.nx, np.int32)
        self._ny = np.ascontiguousarray(geom.ny, np.int32)
        self._nz = np.ascontiguousarray(geom.nz, np.int32)
        self._nbr = np.ascontiguousarray(geom.nbr, np.int32)
        params = np.array([dt, geom.gx, geom.gy, geom.gz, geom.x_zones, geom.y_zones], np.float64)
        h = ctypes.c_void_p()
        rc = lib().npbmz_create(self.kind, geom.nzones, _ip(self._nx), _ip(self._ny), _ip(self._nz), _ip(self._nbr),
                                _dp(params), flags, ctypes.byref(h))
        if rc != 0:
            raise NpbmzError("npbmz_create: " + lib().npbmz_last_error(None).decode())
        self._h = h

    # -- construction helpers -------------------------------------------------
    @classmethod
    def from_class(cls, kind: str, cls_name: str, flags: int = 0):
        niter, dt, ratio, xz, yz, gx, gy, gz = CLASSES[kind][cls_name]
        k = KINDS[kind]
        nx, ny, nz, nbr = zone_setup(k, gx, gy, gz, xz, yz, ratio)
        return cls(Geometry(k, nx, ny, nz, nbr, gx, gy, gz, xz, yz), dt, flags, niter)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().npbmz_destroy(h)
            self._h = None

    def close(self):
        self.__del__()

    def _check(self, rc, what):
        if rc != 0:
            raise NpbmzError(f"{what}: " + lib().npbmz_last_error(self._h).decode(), rc)

    # -- reference operations ---------------------------------------------------
    def setup(self, ce=None):
        """initialize + lhsinit + exact_rhs (src/BT/bt-node.jl:97-113) on the GPU."""
        c = np.ascontiguousarray(CE_REFERENCE if ce is None else ce, np.float64).reshape(65)
        self.ce = c.reshape(5, 13).copy()
        self._check(lib().npbmz_setup(self._h, _dp(c)), "npbmz_setup")

    def exch_qbc(self):
        self._check(lib().npbmz_exch_qbc(self._h), "npbmz_exch_qbc")

    def adi(self, zone: int = -1):
        self._check(lib().npbmz_adi(self._h, zone), "npbmz_adi")

    def step(self, nsteps: int = 1, norms: bool = False):
        out = np.zeros(10 * max(nsteps, 1)) if norms else None
        self._check(lib().npbmz_step(self._h, nsteps, _dp(out) if norms else None), "npbmz_step")
        return out[: 10 * nsteps].reshape(nsteps, 2, 5) if norms else None

    def step_download(self, nsteps: int, layout: int, ptr: int):
        """nsteps steps, then u of all zones to the host buffer at ptr (layout as
        transfer_raw); with a page-locked buffer and zone-group branches the
        copies of each group overlap the other groups' work."""
        self._check(lib().npbmz_step_download(self._h, nsteps, layout, ctypes.c_void_p(ptr)), "npbmz_step_download")

    def step_inout(self, nsteps: int, layout: int, in_ptr: int, out_ptr: int):
        """u of all zones from the host buffer at in_ptr, nsteps steps, u to
        out_ptr (layout as transfer_raw); with page-locked buffers and
        zone-group branches the copies overlap the steps."""
        self._check(lib().npbmz_step_inout(self._h, nsteps, layout, ctypes.c_void_p(in_ptr), ctypes.c_void_p(out_ptr)),
                    "npbmz_step_inout")

    def step_profile(self, nsteps: int = 1):
        """Mean device milliseconds per step of each phase of the batched step
        (CUDA events on the handle's stream); advances nsteps steps."""
        out = np.zeros(len(PROF_PHASES))
        self._check(lib().npbmz_step_profile(self._h, nsteps, _dp(out)), "npbmz_step_profile")
        return dict(zip(PROF_PHASES, out.tolist()))

    def verify(self):
        xcr, xce = np.zeros(5), np.zeros(5)
        self._check(lib().npbmz_verify(self._h, _dp(xcr), _dp(xce)), "npbmz_verify")
        return xcr, xce

    def phase(self, phase: int, zone: int = -1):
        self._check(lib().npbmz_phase(self._h, phase, zone), "npbmz_phase")

    def synchronize(self):
        self._check(lib().npbmz_synchronize(self._h), "npbmz_synchronize")

    def set_stream(self, stream_ptr: int):
        self._check(lib().npbmz_set_stream(self._h, ctypes.c_void_p(stream_ptr)), "npbmz_set_stream")

    def set_step_groups(self, groups: int):
        """Zone groups of the step graph (pipelined branches), 1..8."""
        self._check(lib().npbmz_set_step_groups(self._h, groups), "npbmz_set_step_groups")

    def face_plan(self, send, recv):
        """Register the (zone, side) faces sent to and received from other
        ranks; returns the doubles of the send and receive buffers."""
        s = np.ascontiguousarray(np.asarray(send, np.int32).reshape(-1))
        r = np.ascontiguousarray(np.asarray(recv, np.int32).reshape(-1))
        ns, nr = ctypes.c_int64(0), ctypes.c_int64(0)
        self._check(lib().npbmz_face_plan(self._h, len(s) // 2, _ip(s), len(r) // 2, _ip(r), ctypes.byref(ns),
                                          ctypes.byref(nr)), "npbmz_face_plan")
        return ns.value, nr.value

    def pack_faces(self, send_ptr: int):
        self._check(lib().npbmz_pack_faces(self._h, ctypes.c_void_p(send_ptr)), "npbmz_pack_faces")

    def unpack_faces(self, recv_ptr: int):
        self._check(lib().npbmz_unpack_faces(self._h, ctypes.c_void_p(recv_ptr)), "npbmz_unpack_faces")

    def state_check(self):
        """(bits, (zone, i, j, k)) of the last step call's state check;
        bits == 0 when every point was healthy."""
        v = [ctypes.c_int(0) for _ in range(5)]
        self._check(lib().npbmz_state_check(self._h, *[ctypes.byref(x) for x in v]), "npbmz_state_check")
        return v[0].value, tuple(x.value for x in v[1:])

    def set_step_overlap(self, fp64_first: bool, sweep_ctas_per_sm: int = 0):
        """Zone-group branches: prim + compute_rhs on a high-priority stream,
        and at most sweep_ctas_per_sm resident sweep CTAs per SM (0: no cap)."""
        self._check(lib().npbmz_set_step_overlap(self._h, int(bool(fp64_first)), int(sweep_ctas_per_sm)),
                    "npbmz_set_step_overlap")

    def set_copy_fusion(self, on: bool):
        """The x sweep's x-line-major state copies in the compute_rhs launch
        (True) or by a kernel of their own (False)."""
        self._check(lib().npbmz_set_copy_fusion(self._h, int(bool(on))), "npbmz_set_copy_fusion")

    def autotune(self):
        self._check(lib().npbmz_autotune(self._h), "npbmz_autotune")

    def adjoint(self, nsteps: int, u_target, checkpoint_every: int = 10, grad_forcing: bool = True,
                grad_u0: bool = True):
        """Discrete adjoint of ``nsteps`` steps for J = 1/2 sum (u_N - u_target)^2
        over every stored point (BT only).  ``u_target``: one dense array per
        zone (or the flat concatenation).  Returns (J, dJ/dforcing, dJ/du0),
        the gradients as lists of per-zone dense arrays (None when not asked
        for).  u is left as it was."""
        total = self.dense_total()
        t = self.flatten(u_target)
        gf = np.zeros(total) if grad_forcing else None
        gu = np.zeros(total) if grad_u0 else None
        J = ctypes.c_double(0.0)
        self._check(lib().npbmz_adjoint(self._h, nsteps, checkpoint_every, _dp(t), ctypes.byref(J),
                                        _dp(gf) if gf is not None else None, _dp(gu) if gu is not None else None),
                    "npbmz_adjoint")
        return J.value, (self.split(gf) if gf is not None else None), (self.split(gu) if gu is not None else None)

    # -- all zones in the dense layout (zone z: [5][nz][ny][nx], zones back to back) --
    def dense_total(self) -> int:
        return int(5 * np.sum(self._nx.astype(np.int64) * self._ny * self._nz))

    def flatten(self, arrays):
        if isinstance(arrays, np.ndarray) and arrays.ndim == 1:
            a = np.ascontiguousarray(arrays, np.float64)
        else:
            a = np.concatenate([np.ascontiguousarray(x, np.float64).reshape(-1) for x in arrays])
        if a.size != self.dense_total():
            raise NpbmzError(f"{a.size} values for {self.dense_total()} dense elements")
        return a

    def split(self, flat):
        out, o = [], 0
        for z in range(self.geom.nzones):
            shp = self.zone_shape(z)
            n = int(np.prod(shp))
            out.append(flat[o:o + n].reshape(shp))
            o += n
        return out

    def download_all(self, field: int):
        out = np.zeros(self.dense_total())
        self._check(lib().npbmz_download(self._h, -1, field, LAYOUT_DENSE, out.ctypes.data), "npbmz_download")
        return self.split(out)

    def upload_all(self, field: int, arrays):
        a = self.flatten(arrays)
        self._check(lib().npbmz_upload(self._h, -1, field, LAYOUT_DENSE, a.ctypes.data), "npbmz_upload")

    # -- data movement -------------------------------------------------------------
    def zone_shape(self, zone):
        return (5, int(self._nz[zone]), int(self._ny[zone]), int(self._nx[zone]))

    def download(self, field: int, zone: int):
        out = np.zeros(self.zone_shape(zone))
        self._check(lib().npbmz_download(self._h, zone, field, LAYOUT_DENSE, out.ctypes.data), "npbmz_download")
        return out

    def upload(self, field: int, zone: int, arr):
        a = np.ascontiguousarray(arr, np.float64)
        if a.shape != self.zone_shape(zone):
            raise NpbmzError(f"shape {a.shape} != {self.zone_shape(zone)}")
        self._check(lib().npbmz_upload(self._h, zone, field, LAYOUT_DENSE, a.ctypes.data), "npbmz_upload")

    def transfer_raw(self, field: int, zone: int, layout: int, ptr: int, to_device: bool, sync: bool = True):
        """Upload/download through a raw host pointer (pinned buffers, reference layouts)."""
        if to_device:
            f = lib().npbmz_upload if sync else lib().npbmz_upload_async
        else:
            f = lib().npbmz_download if sync else lib().npbmz_download_async
        self._check(f(self._h, zone, field, layout, ctypes.c_void_p(ptr)), f.__name__)

    # -- queries ---------------------------------------------------------------------
    @property
    def launches_per_step(self):
        return lib().npbmz_launches_per_step(self._h)

    @property
    def device_bytes(self):
        return lib().npbmz_device_bytes(self._h)

    def describe(self):
        buf = ctypes.create_string_buffer(1024)
        lib().npbmz_describe(self._h, buf, 1024)
        return json.loads(buf.value.decode())


def ref_elems(kind: int, field: int, nx: int, ny: int, nz: int) -> int:
    """Element count of one zone's reference OffsetArray (see include/npbmz.h)."""
    IMAX, JMAX, KMAX = nx + 1, ny + 1, nz + 1
    if kind == BT:
        if field == U:
            return 5 * (IMAX + 4) * (JMAX + 4) * (KMAX + 4)
        if field == RHS:
            return 5 * (IMAX + 1) * (JMAX + 1) * (KMAX + 1)
        return 5 * IMAX * JMAX * KMAX
    IMAXP, JMAXP = (IMAX // 2) * 2 + 1, (JMAX // 2) * 2 + 1
    if field == U:
        return 5 * (IMAXP + 4) * (JMAXP + 4) * (KMAX + 4)
    return 5 * IMAXP * JMAXP * KMAX


# ---- the reference's entry points, by name ----------------------------------------
def exch_qbc(problem: Problem):
    """exch_qbc over all zones (src/BT/exchange_qbc.jl:1-122), on the device."""
    problem.exch_qbc()


def adi(problem: Problem, iz: int = -1):
    """adi for zone iz (0-based), or all zones batched when iz = -1 (src/BT/adi.jl:5-251)."""
    problem.adi(iz)


def fp64_peak_gflops() -> float:
    """Measured FP64 FMA throughput of the current GPU (GFLOP/s)."""
    g = ctypes.c_double(0.0)
    if lib().npbmz_fp64_peak(ctypes.byref(g)) != 0:
        raise NpbmzError("npbmz_fp64_peak failed")
    return g.value


def golden_norms(kind: str, cls_name: str):
    """The reference's verification norms (src/BT/verify.jl:136-348, src/SP/verify.jl:137-282)."""
    path = Path(__file__).resolve().parents[2] / "tests" / "golden" / "npb_golden_norms.json"
    d = json.loads(path.read_text())[kind].get(cls_name)
    return None if d is None else (np.array(d["xcr"]), np.array(d["xce"]), d["dt"], d["niter"])


def go(kind: str, cls_name: str, flags: int = 0, niter: int | None = None, verbose: bool = False):
    """The reference's node protocol on the GPU (src/BT/bt-node.jl:93-426):
    set_constants, initialize, exact_rhs, niter steps of exch_qbc + adi, verify.
    Returns (xcr, xce, verified) with verified per src/BT/verify.jl:361-398
    (epsilon 1e-8), or None when the class has no golden values."""
    p = Problem.from_class(kind, cls_name, flags)
    p.setup()
    n = p.niter if niter is None else niter
    p.step(n)
    xcr, xce = p.verify()
    g = golden_norms(kind, cls_name)
    verified = None
    if g is not None and n == g[3]:
        xcrref, xceref, _, _ = g
        verified = bool(np.all(np.abs((xcr - xcrref) / xcrref) <= 1e-8) and np.all(np.abs((xce - xceref) / xceref) <= 1e-8))
    if verbose:
        print(f"{kind} class {cls_name}: {p.geom.nzones} zones, {n} steps")
        print("xcr", xcr, "\nxce", xce, "\nverified", verified)
    p.close()
    return xcr, xce, verified
