"""The benchmark's own configuration against the FP64 oracle, at full size.

The timed workload is the 480x320x28 grid split 16x16 (4.3 M points, 256
zones), seeded manufactured solution (seed 20261203, energy row scaled by
2^2), 200 steps:

- BT-MZ: geometric zones (area ratio 20.8, the class C geometry of
  src/BT/classes.jl:20), dt 1e-4;
- SP-MZ: equal 30x20x28 zones (src/SP/classes.jl), dt 6.7e-4.

The oracle runs the 200 steps once per kind on the host cores (OpenMP over
zones).  The headline variant -- MIXED (FP32 line solves refined against the
FP64 residual) replayed as a CUDA graph, on an autotuned handle, as bench.py
times it -- must agree with it to 1e-10 relative in the final residual and
error norms and in u (per zone, max-abs error over max-abs value); the FP64
graph path to 1e-12.
"""
import numpy as np
import pytest

import npbmz

pytestmark = pytest.mark.gpu

SEED = 20261203
STEPS = 200
MIXED_REL = 1e-10
FP64_REL = 1e-12
DT = {"BT": 1e-4, "SP": 6.7e-4}


def geometry(kind):
    niter, dt, ratio, xz, yz, gx, gy, gz = npbmz.CLASSES[kind]["C"]
    k = npbmz.KINDS[kind]
    nx, ny, nz, nbr = npbmz.zone_setup(k, gx, gy, gz, xz, yz, ratio)
    return npbmz.Geometry(k, nx, ny, nz, nbr, gx, gy, gz, xz, yz)


@pytest.fixture(scope="module", params=["BT", "SP"])
def oracle_run(request, oracle_mod):
    """(kind, geometry, ce, oracle norms, oracle u per zone) after 200 steps."""
    kind = request.param
    g = geometry(kind)
    ce, e = npbmz.seeded_coefficients(SEED, g.nx, g.ny, g.nz, g.gx, g.gy, g.gz, g.x_zones, g.y_zones)
    assert e == 2
    o = oracle_mod.Oracle(g.kind, g.nx, g.ny, g.nz, g.nbr, DT[kind], g.gx, g.gy, g.gz, g.x_zones, g.y_zones, ce)
    o.step(STEPS)
    norms = np.concatenate(o.verify())
    u = [o.get(0, z) for z in range(g.nzones)]
    del o
    return kind, g, ce, norms, u


def check(p, norms, u, rel):
    p.synchronize()
    x = np.concatenate(p.verify())
    np.testing.assert_allclose(x, norms, rtol=rel, atol=0)
    worst = 0.0
    for z in range(p.geom.nzones):
        a = p.download(npbmz.U, z)
        err = np.max(np.abs(a - u[z])) / np.max(np.abs(u[z]))
        worst = max(worst, err)
        assert err <= rel, f"zone {z}: u rel err {err:.3e} > {rel:.0e}"
    return worst


def test_headline_variant_within_1e10_of_fp64_oracle(oracle_run):
    kind, g, ce, norms, u = oracle_run
    p = npbmz.Problem(g, DT[kind], npbmz.MIXED | npbmz.GRAPH)
    p.setup(ce)
    p.autotune()
    p.setup(ce)
    p.step(STEPS)
    check(p, norms, u, MIXED_REL)
    p.close()


def test_fp64_graph_path_within_1e12_of_oracle(oracle_run):
    kind, g, ce, norms, u = oracle_run
    p = npbmz.Problem(g, DT[kind], npbmz.GRAPH)
    p.setup(ce)
    p.step(STEPS)
    check(p, norms, u, FP64_REL)
    p.close()
