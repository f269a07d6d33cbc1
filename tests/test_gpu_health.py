"""The state check of npbmz_step and npbmz_step_download, through the C ABI.

Each step's primitive kernel checks the state entering that step, and a final
kernel checks the state a call leaves.  A density that is not positive and
finite, or a non-finite value, makes the call return NPBMZ_ERR_STATE with a
message naming the failure and the first bad point; so does a non-positive
pressure-like quantity rho E - |rho v|^2 / (2 rho) for SP (which takes its
square root).  For BT the latter is only reported by npbmz_state_check: the
reference carries such a state on.  The failure is made on the host: a u
with one bad point is uploaded (no device fault is involved), and a healthy
run must report nothing.
"""
import numpy as np
import pytest

import npbmz

pytestmark = pytest.mark.gpu

VARIANTS = {"fp64": 0, "exact": npbmz.EXACT, "mixed-graph": npbmz.MIXED | npbmz.GRAPH,
            "dfrhs-graph": npbmz.MIXED | npbmz.RHS_DF | npbmz.GRAPH}


def problem(kind, flags):
    niter, dt, ratio, xz, yz, gx, gy, gz = npbmz.CLASSES[kind]["S"]
    k = npbmz.KINDS[kind]
    nx, ny, nz, nbr = npbmz.zone_setup(k, gx, gy, gz, xz, yz, ratio)
    p = npbmz.Problem(npbmz.Geometry(k, nx, ny, nz, nbr, gx, gy, gz, xz, yz), dt, flags)
    p.setup()
    return p


def plant(p, zone, ijk, m, value):
    u = p.download(npbmz.U, zone)
    i, j, k = ijk
    u[m, k, j, i] = value
    p.upload(npbmz.U, zone, u)


@pytest.mark.parametrize("kind", ["BT", "SP"])
@pytest.mark.parametrize("variant", list(VARIANTS))
def test_healthy_run_reports_nothing(kind, variant):
    p = problem(kind, VARIANTS[variant])
    p.step(3)
    assert p.state_check() == (0, (-1, -1, -1, -1))
    p.step(2, norms=True)
    assert p.state_check()[0] == 0


@pytest.mark.parametrize("kind", ["BT", "SP"])
@pytest.mark.parametrize("variant", list(VARIANTS))
@pytest.mark.parametrize("what,bit,m,value", [("pressure", npbmz.STATE_PRESSURE, 4, -1.0),
                                              ("density", npbmz.STATE_DENSITY, 0, -0.5),
                                              ("non-finite", npbmz.STATE_NONFINITE, 2, float("nan")),
                                              ("density", npbmz.STATE_DENSITY, 0, float("inf"))])
def test_planted_bad_point_is_reported(kind, variant, what, bit, m, value):
    p = problem(kind, VARIANTS[variant])
    zone, ijk = 2, (3, 4, 2)
    fatal = bit != npbmz.STATE_PRESSURE or kind == "SP"
    plant(p, zone, ijk, m, value)
    # no step: the final check alone names exactly the planted point
    if fatal:
        with pytest.raises(npbmz.NpbmzError) as e:
            p.step(0)
        assert e.value.code == npbmz.ERR_STATE
        msg = str(e.value)
        assert what in msg and f"zone {zone} (i, j, k) = {ijk}" in msg, msg
    else:
        p.step(0)  # BT carries a non-positive pressure on, as the reference does
    assert p.state_check() == (bit, (zone,) + ijk)
    # one step: the step's own check sees it (the step may spread it further)
    plant(p, zone, ijk, m, value)
    if fatal:
        with pytest.raises(npbmz.NpbmzError) as e:
            p.step(1)
        assert e.value.code == npbmz.ERR_STATE and "state check failed" in str(e.value)
    else:
        p.step(1)
    assert p.state_check()[0] & bit


def test_step_download_reports_and_still_copies():
    torch = pytest.importorskip("torch")
    p = problem("BT", npbmz.MIXED | npbmz.GRAPH)
    plant(p, 1, (2, 2, 2), 0, -3.0)
    host = torch.zeros(p.dense_total(), dtype=torch.float64).pin_memory()
    with pytest.raises(npbmz.NpbmzError) as e:
        p.step_download(1, npbmz.LAYOUT_DENSE, host.data_ptr())
    assert e.value.code == npbmz.ERR_STATE
    assert np.count_nonzero(host.numpy()) > 0
    # a fresh set-up is healthy again
    p.setup()
    p.step_download(1, npbmz.LAYOUT_DENSE, host.data_ptr())
