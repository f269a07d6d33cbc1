"""The dual-number oracle (oracle/npbmz_tangent.cpp) on the CPU.

It is the reference gradient for the GPU adjoint, so it is pinned here:
its value part must be the double oracle's trajectory bit for bit, and its
directional derivatives must match central finite differences of the double
oracle (the oracle itself is pinned to the NPB golden norms).
"""
import math

import numpy as np
import pytest

import npbmz
from oracle import oracle


KINDS = {"BT": oracle.KIND_BT, "SP": oracle.KIND_SP}


def case(kind="BT", cls="S", seed=2):
    niter, dt, ratio, xz, yz, gx, gy, gz = npbmz.CLASSES[kind][cls]
    nx, ny, nz, nbr = oracle.zone_setup(KINDS[kind], gx, gy, gz, xz, yz, ratio)
    o = oracle.Oracle(KINDS[kind], nx, ny, nz, nbr, dt, gx, gy, gz, xz, yz, npbmz.CE_REFERENCE)
    geo = (KINDS[kind], nx, ny, nz, nbr, dt, gx, gy, gz, xz, yz)
    rng = np.random.default_rng(seed)
    u0, f0 = o.get_all(0), o.get_all(2)
    target = u0 + rng.normal(0.0, 0.05, u0.shape)
    return o, geo, u0, f0, target


def set_all(o, which, flat):
    off = 0
    for z in range(o.nzones):
        shp = (5, int(o.nz[z]), int(o.ny[z]), int(o.nx[z]))
        n = int(np.prod(shp))
        o.set(which, z, flat[off:off + n].reshape(shp))
        off += n


def oracle_terminal(geo, u0, f0, nsteps):
    kind, nx, ny, nz, nbr, dt, gx, gy, gz, xz, yz = geo
    o = oracle.Oracle(kind, nx, ny, nz, nbr, dt, gx, gy, gz, xz, yz, npbmz.CE_REFERENCE)
    set_all(o, 0, u0)
    set_all(o, 2, f0)
    o.step(nsteps)
    return o.get_all(0)


@pytest.mark.parametrize("kind", ["BT", "SP"])
def test_value_part_is_the_double_oracle_bit_for_bit(kind):
    o, geo, u0, f0, target = case(kind)
    rng = np.random.default_rng(4)
    J, dJ, uN = oracle.tangent_objective(*geo, u0, f0, target, 6, du0=rng.standard_normal((3, u0.size)))
    o.step(6)
    ref = o.get_all(0)
    np.testing.assert_array_equal(uN, ref)
    a = ref - target
    assert J == pytest.approx(0.5 * math.fsum(a * a), rel=1e-13)


@pytest.mark.parametrize("kind", ["BT", "SP"])
@pytest.mark.parametrize("which", ["u0", "forcing"])
def test_directional_derivatives_match_central_differences(kind, which):
    """Dual-number derivatives vs central differences of the double oracle
    along 4 seeded directions scaled to the field's RMS, 6 steps.  Rough
    directions in u_0 meet the stencil's strong curvature (the O(h^2) error
    is 7e-7 at h = 1e-5, 7e-9 at 1e-6), so h = 1e-6 there; the forcing enters
    through dt and is nearly linear for BT, so h = 1e-5 there, clear of
    rounding.  SP's forcing is larger and its curvature shows (worst of 4:
    2.2e-7 at h = 1e-5, 2.2e-9 at 1e-6, 1.2e-10 at 1e-7, falling as h^2), so
    SP takes h = 1e-6 for both.  SP's max() in the viscous band term selects
    the same branch at every point for these h, so the derivative of the
    selected branch is the one the differences see."""
    o, geo, u0, f0, target = case(kind)
    nsteps = 6
    h = 1e-5 if (kind, which) == ("BT", "forcing") else 1e-6
    x0 = u0 if which == "u0" else f0
    rng = np.random.default_rng(9)
    d = rng.standard_normal((4, x0.size))
    d *= math.sqrt(float(np.mean(x0 * x0)))
    _, dJ, _ = oracle.tangent_objective(*geo, u0, f0, target, nsteps,
                                        du0=d if which == "u0" else None, dforcing=d if which == "forcing" else None)
    for k in range(d.shape[0]):
        if which == "u0":
            ap = oracle_terminal(geo, u0 + h * d[k], f0, nsteps) - target
            am = oracle_terminal(geo, u0 - h * d[k], f0, nsteps) - target
        else:
            ap = oracle_terminal(geo, u0, f0 + h * d[k], nsteps) - target
            am = oracle_terminal(geo, u0, f0 - h * d[k], nsteps) - target
        fd = math.fsum(0.5 * (ap - am) * (ap + am)) / (2.0 * h)
        assert abs(fd - dJ[k]) <= 1e-7 * abs(dJ[k]), (k, fd, dJ[k])


def test_rejects_too_many_directions():
    o, geo, u0, f0, target = case()
    with pytest.raises(AssertionError):
        oracle.tangent_objective(*geo, u0, f0, target, 1, du0=np.zeros((17, u0.size)))


def test_bt_wrapper_is_the_bt_kind():
    o, geo, u0, f0, target = case()
    rng = np.random.default_rng(5)
    d = rng.standard_normal((2, u0.size))
    a = oracle.tangent_objective(*geo, u0, f0, target, 2, du0=d)
    b = oracle.tangent_bt_objective(*geo[1:], u0, f0, target, 2, du0=d)
    assert a[0] == b[0]
    np.testing.assert_array_equal(a[1], b[1])
