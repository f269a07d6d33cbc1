"""The CPU oracle against the reference's own known-answer values: the NPB
verification norms of src/BT/verify.jl:136-348 and src/SP/verify.jl:137-282,
reproduced with the reference's fixed ce table (src/BT/set_constants.jl:47-51)
on the class geometries of src/BT/classes.jl / src/SP/classes.jl.  The
reference verifies with epsilon = 1e-8 (src/BT/verify.jl:113); the oracle is
held to 1e-11 relative (the golden values carry 13 significant digits)."""
import json
from pathlib import Path

import numpy as np
import pytest

from npbmz import CE_REFERENCE, CLASSES

GOLDEN = json.loads((Path(__file__).parent / "golden" / "npb_golden_norms.json").read_text())


def run_class(oracle_mod, kind, cls):
    niter, dt, ratio, xz, yz, gx, gy, gz = CLASSES[kind][cls]
    k = oracle_mod.KIND_BT if kind == "BT" else oracle_mod.KIND_SP
    nx, ny, nz, nbr = oracle_mod.zone_setup(k, gx, gy, gz, xz, yz, ratio)
    o = oracle_mod.Oracle(k, nx, ny, nz, nbr, dt, gx, gy, gz, xz, yz, CE_REFERENCE)
    o.step(niter)
    return o.verify()


@pytest.mark.parametrize(
    "kind,cls",
    [("BT", "S"), ("BT", "W"), ("SP", "S"), ("SP", "W"), ("SP", "A"),
     pytest.param("BT", "A", marks=pytest.mark.slow),
     # 304x208x17 in 64 geometric zones (ratio 4.5): the geometry of the
     # BT class B benchmark configuration, about 45 s on 8 cores
     pytest.param("BT", "B", marks=pytest.mark.slow)],
)
def test_oracle_reproduces_npb_golden_norms(oracle_mod, kind, cls):
    xcr, xce = run_class(oracle_mod, kind, cls)
    g = GOLDEN[kind][cls]
    np.testing.assert_allclose(xcr, g["xcr"], rtol=1e-11, atol=0)
    np.testing.assert_allclose(xce, g["xce"], rtol=1e-11, atol=0)


def test_golden_fixture_covers_reference_classes():
    for kind in ("BT", "SP"):
        assert set("SWABCDEF") <= set(GOLDEN[kind])
        for cls, d in GOLDEN[kind].items():
            assert len(d["xcr"]) == 5 and len(d["xce"]) == 5
            assert d["niter"] == CLASSES[kind][cls][0]
            assert abs(d["dt"] - CLASSES[kind][cls][1]) < 1e-12


def test_oracle_planted_error_is_caught(oracle_mod):
    """A mistake planted in the oracle's state (on the CPU) moves the norms far
    outside the golden tolerance, so the known-answer test has teeth."""
    niter, dt, ratio, xz, yz, gx, gy, gz = CLASSES["BT"]["S"]
    nx, ny, nz, nbr = oracle_mod.zone_setup(oracle_mod.KIND_BT, gx, gy, gz, xz, yz, ratio)
    o = oracle_mod.Oracle(oracle_mod.KIND_BT, nx, ny, nz, nbr, dt, gx, gy, gz, xz, yz, CE_REFERENCE)
    f = o.get(2, 0)
    f[:, 2, 2, 2] *= 1.0 + 1e-3
    o.set(2, 0, f)
    o.step(niter)
    xcr, xce = o.verify()
    g = GOLDEN["BT"]["S"]
    assert np.max(np.abs((xcr - g["xcr"]) / np.array(g["xcr"]))) > 1e-8
