"""LU-MZ on the GPU (include/npbmz_lu.h) against the CPU oracle
(oracle/lumz_oracle.cpp, pinned to the reference's LU-MZ verification norms).

The kernels are built without FMA contraction and follow the reference's
statements point for point, so u, rsd and frct are compared bit for bit:
after setup (setbv, setiv, erhs, rhs), after every phase of ssor, and after
whole iterations, in both exch_qbc plane modes.  Norms (sums in another
order) are held to 1e-13.  Geometries: LU-MZ classes S, W and B (4x4 zones
of 6x6x6, 16x16x8 and 76x52x17), zones of the minimum size 5x5x5 (where the
fourth-difference boundary stencils overlap), rectangular 9x7x7 zones, 2x2
zones, and stretched zones of unequal sizes; the reference's ce table and a
perturbed one.  Whole runs of classes S to C, in the bit-exact and the FMA
build, meet the reference's verification norms (epsilon 1e-8).
"""
import numpy as np
import pytest

import npbmz
from npbmz import lu

pytestmark = pytest.mark.gpu


def oracle_lu():
    from oracle import oracle

    return oracle


def make(geom, dt, flags=0):
    """GPU problem and oracle from the same geometry, both after setup."""
    o = oracle_lu()
    nx, ny, nz, nbr = geom
    p = lu.LuProblem(nx, ny, nz, nbr, dt, flags=flags)
    p.setup()
    r = o.LuOracle(nx, ny, nz, nbr, dt, faces_npb=bool(flags & lu.FACES_NPB))
    return p, r


def assert_state_equal(p, r, fields=(lu.U, lu.RSD, lu.FRCT)):
    for z in range(p.nzones):
        for f in fields:
            np.testing.assert_array_equal(p.download(z, f), r.get(f, z), err_msg=f"zone {z} field {f}")


GEOMS = {
    "S": (lambda: lu.lu_zone_setup(24, 24, 6, 4, 4), 0.5),
    "W": (lambda: lu.lu_zone_setup(64, 64, 8, 4, 4), 1.5e-3),
    "min5": (lambda: lu.lu_zone_setup(20, 20, 5, 4, 4), 0.5),
    "rect": (lambda: lu.lu_zone_setup(36, 28, 7, 4, 4), 0.5),
    "2x2": (lambda: lu.lu_zone_setup(18, 14, 6, 2, 2), 0.5),
}


@pytest.mark.parametrize("name", list(GEOMS))
def test_setup_is_bit_exact(name):
    g, dt = GEOMS[name]
    p, r = make(g(), dt)
    assert_state_equal(p, r)


@pytest.mark.parametrize("name", ["S", "min5", "rect"])
@pytest.mark.parametrize("faces_npb", [False, True], ids=["ref-faces", "npb-faces"])
def test_phases_are_bit_exact(name, faces_npb):
    """Each phase from the same state: exch_qbc, rsd *= dt, jacld + blts,
    jacu + buts, update, rhs; then a whole ssor."""
    from oracle import oracle

    g, dt = GEOMS[name]
    p, r = make(g(), dt, lu.FACES_NPB if faces_npb else 0)
    for gp, op in [(lu.PHASE_EXCH, oracle.LU_EXCH), (lu.PHASE_SCALE, oracle.LU_SCALE),
                   (lu.PHASE_LOWER, oracle.LU_LOWER), (lu.PHASE_UPPER, oracle.LU_UPPER),
                   (lu.PHASE_UPDATE, oracle.LU_UPDATE), (lu.PHASE_RHS, oracle.LU_RHS),
                   (lu.PHASE_SSOR, oracle.LU_SSOR)]:
        p.phase(gp)
        r.phase(op)
        assert_state_equal(p, r, (lu.U, lu.RSD))


@pytest.mark.parametrize("name,niter", [("S", 50), ("W", 40), ("min5", 20), ("rect", 20), ("2x2", 20)])
@pytest.mark.parametrize("flags", [0, lu.FACES_NPB, lu.FACES_NPB | lu.GRAPH], ids=["ref", "npb", "npb-graph"])
def test_iterations_are_bit_exact(name, niter, flags):
    g, dt = GEOMS[name]
    p, r = make(g(), dt, flags)
    p.iterate(niter)
    r.iterate(niter)
    assert_state_equal(p, r, (lu.U, lu.RSD))
    a, b = p.verify(), r.verify()
    np.testing.assert_allclose(a[0], b[0], rtol=1e-13)
    np.testing.assert_allclose(a[1], b[1], rtol=1e-13)
    np.testing.assert_allclose(a[2], b[2], rtol=1e-13)


def test_per_zone_ssor_equals_batched():
    g, dt = GEOMS["rect"]
    a, _ = make(g(), dt, lu.FACES_NPB)
    b, _ = make(g(), dt, lu.FACES_NPB)
    for _ in range(3):
        a.exch_qbc()
        a.ssor(-1)
        b.exch_qbc()
        for z in range(b.nzones):
            b.ssor(z)
    for z in range(a.nzones):
        for f in (lu.U, lu.RSD):
            np.testing.assert_array_equal(a.download(z, f), b.download(z, f))


def test_iteration_norms_match_verify():
    g, dt = GEOMS["S"]
    p, _ = make(g(), dt, lu.FACES_NPB | lu.GRAPH)
    norms = p.iterate(7, norms=True)
    assert norms.shape == (7, 5) and np.all(norms > 0)
    xcr, _, _ = p.verify()
    np.testing.assert_array_equal(norms[-1], xcr)


@pytest.mark.parametrize("cls", ["S", "W", "A", "B", "C"])
def test_go_meets_the_golden_norms(cls):
    xcr, xce, xci, verified = lu.go(cls)
    assert verified, (xcr, xce, xci)


def test_reference_faces_miss_the_golden_norms_as_the_oracle_does():
    xcr, _, _, verified = lu.go("S", flags=lu.GRAPH)
    assert verified is False


def test_ref_layout_round_trip_keeps_the_halo():
    g, dt = GEOMS["rect"]
    p, r = make(g(), dt)
    z = 5
    nx, ny, nz = int(p.nx[z]), int(p.ny[z]), int(p.nz[z])
    img = np.full(lu.ref_elems(nx, ny, nz), 7.25)
    p.download(z, lu.U, npbmz.LAYOUT_REF, out=img)
    a = img.reshape(nz, ny + 4, nx + 4, 5)  # column-major [m, i, j, k] read back to front
    dense = r.get(lu.U, z)
    for m in range(5):
        np.testing.assert_array_equal(a[:, 2:ny + 2, 2:nx + 2, m], dense[m])
    assert np.all(a[:, :2, :, :] == 7.25) and np.all(a[:, :, :2, :] == 7.25)
    assert np.all(a[:, ny + 2:, :, :] == 7.25) and np.all(a[:, :, nx + 2:, :] == 7.25)
    a[:, 2:ny + 2, 2:nx + 2, :] *= 1.5
    p.upload(z, lu.U, img, npbmz.LAYOUT_REF)
    np.testing.assert_array_equal(p.download(z, lu.U), dense * 1.5)


def test_upload_download_all_zones_dense():
    g, dt = GEOMS["2x2"]
    p, r = make(g(), dt)
    flat = r.get_all(lu.FRCT) * 0.5
    lu.lib().npbmz_lu_upload(p._h, -1, lu.FRCT, npbmz.LAYOUT_DENSE, flat.ctypes.data)
    back = np.empty_like(flat)
    lu.lib().npbmz_lu_download(p._h, -1, lu.FRCT, npbmz.LAYOUT_DENSE, back.ctypes.data)
    np.testing.assert_array_equal(back, flat)


def test_create_rejects_bad_geometry():
    nx, ny, nz, nbr = lu.lu_zone_setup(16, 16, 6, 4, 4)  # zones 4 wide: below the 5-point stencil
    with pytest.raises(npbmz.NpbmzError, match="size 4x4x6"):
        lu.LuProblem(nx, ny, nz, nbr, 0.5)
    nx, ny, nz, nbr = lu.lu_zone_setup(24, 24, 6, 4, 4)
    with pytest.raises(npbmz.NpbmzError, match="unknown flags"):
        lu.LuProblem(nx, ny, nz, nbr, 0.5, flags=0x80)
    with pytest.raises(npbmz.NpbmzError, match="outside the zones"):
        lu.lu_zone_setup(24, 24, 6, 3, 2)  # the reference's neighbour rule leaves the zone range


def test_create_rejects_a_problem_larger_than_device_memory():
    """Class E (4224x3456x92, 1.34 G points, about 1.6 TB of state and Jacobian
    planes) is refused before any device allocation, and leaves no pending
    error behind: a handle created next runs."""
    with pytest.raises(npbmz.NpbmzError, match="GB of device memory"):
        lu.LuProblem.from_class("E")
    g, dt = GEOMS["S"]
    p, o = make(g(), dt)
    p.iterate(2)
    o.iterate(2)
    np.testing.assert_array_equal(p.download(0, lu.U), o.get(lu.U, 0))


def test_phase_and_zone_errors_are_reported():
    g, dt = GEOMS["S"]
    p, _ = make(g(), dt)
    with pytest.raises(npbmz.NpbmzError, match="phase"):
        p.phase(17)
    with pytest.raises(npbmz.NpbmzError, match="zone"):
        p.ssor(16)
    assert p.launches_per_iteration() == 5 + 2 * (6 + 6 + 6 - 3 - 6 + 1)


@pytest.mark.parametrize("name,niter", [("S", 50), ("W", 40), ("rect", 20)])
def test_fma_build_stays_within_rounding_of_the_oracle(name, niter):
    """NPBMZ_LU_FMA: the iteration's kernels with a*b+c contracted.  Not
    bit-for-bit; after niter iterations u stays within 1e-12 (relative to
    each variable's largest magnitude) and the norms within 1e-10 of the
    oracle, and set-up is still bit-for-bit (it runs uncontracted)."""
    g, dt = GEOMS[name]
    p, r = make(g(), dt, lu.FACES_NPB | lu.GRAPH | lu.FMA)
    for z in range(p.nzones):
        np.testing.assert_array_equal(p.download(z, lu.U), r.get(lu.U, z))
        np.testing.assert_array_equal(p.download(z, lu.FRCT), r.get(lu.FRCT, z))
    p.iterate(niter)
    r.iterate(niter)
    for z in range(p.nzones):
        a, b = p.download(z, lu.U), r.get(lu.U, z)
        scale = np.max(np.abs(b), axis=(1, 2, 3), keepdims=True)
        assert np.max(np.abs(a - b) / scale) <= 1e-12
    x, y = p.verify(), r.verify()
    np.testing.assert_allclose(x[0], y[0], rtol=1e-10)
    np.testing.assert_allclose(x[1], y[1], rtol=1e-10)
    np.testing.assert_allclose(x[2], y[2], rtol=1e-10)


@pytest.mark.parametrize("cls", ["S", "W", "A", "B", "C"])
def test_fma_build_meets_the_golden_norms(cls):
    xcr, xce, xci, verified = lu.go(cls, flags=lu.FACES_NPB | lu.GRAPH | lu.FMA)
    assert verified, (xcr, xce, xci)


def test_upper_phase_alone_uses_the_current_state():
    """jacu reads the current u (src/LU/jacu.jl): buts alone, after u has
    changed since the last lower sweep (an upload), matches the oracle's."""
    from oracle import oracle

    g, dt = GEOMS["rect"]
    p, r = make(g(), dt)
    p.phase(lu.PHASE_LOWER)
    r.phase(oracle.LU_LOWER)
    for z in (0, 7):
        u = r.get(lu.U, z)
        u[:, 2:-2, 2:-2, 2:-2] *= 1.0 + 1e-3
        r.set(lu.U, z, u)
        p.upload(z, lu.U, u)
    p.phase(lu.PHASE_UPPER)
    r.phase(oracle.LU_UPPER)
    assert_state_equal(p, r, (lu.U, lu.RSD))
    p.phase(lu.PHASE_UPDATE)
    r.phase(oracle.LU_UPDATE)
    p.phase(lu.PHASE_UPPER)
    r.phase(oracle.LU_UPPER)
    assert_state_equal(p, r, (lu.U, lu.RSD))


@pytest.mark.parametrize("flags", [0, lu.FACES_NPB], ids=["ref-faces", "npb-faces"])
def test_stretched_unequal_zones_are_bit_exact(flags):
    """zone_setup's stretched rule (ratio 3: zone widths 6..16 x 5..14): zones
    of different sizes share every hyperplane launch, each with its own
    hyperplane count and its own setcoeff constants."""
    g = lu.lu_zone_setup(40, 36, 6, 4, 4, 3.0)
    assert len(set(g[0].tolist())) > 1 and len(set(g[1].tolist())) > 1
    p, r = make(g, 0.5, flags)
    p.iterate(20)
    r.iterate(20)
    assert_state_equal(p, r, (lu.U, lu.RSD))


def test_other_coefficient_table_is_bit_exact():
    """setup from a ce table other than the reference's (each coefficient
    perturbed by a seeded 10 %): setbv, setiv, erhs and 20 iterations."""
    from oracle import oracle

    rng = np.random.default_rng(31)
    ce = np.array(npbmz.CE_REFERENCE) * (1.0 + 0.1 * rng.standard_normal((5, 13)))
    nx, ny, nz, nbr = lu.lu_zone_setup(40, 40, 8, 4, 4)
    p = lu.LuProblem(nx, ny, nz, nbr, 0.5, flags=lu.FACES_NPB | lu.GRAPH)
    p.setup(ce)
    r = oracle.LuOracle(nx, ny, nz, nbr, 0.5, ce=ce, faces_npb=True)
    assert_state_equal(p, r)
    p.iterate(20)
    r.iterate(20)
    assert_state_equal(p, r, (lu.U, lu.RSD))


def test_class_b_zones_are_bit_exact():
    """LU-MZ class B geometry (16 zones of 76x52x17, 1.07 M points), 5
    iterations."""
    niter, dt, ratio, xz, yz, gx, gy, gz = npbmz.CLASSES["LU"]["B"]
    g = lu.lu_zone_setup(gx, gy, gz, xz, yz, ratio)
    p, r = make(g, dt, lu.GRAPH)
    p.iterate(5)
    r.iterate(5)
    assert_state_equal(p, r, (lu.U, lu.RSD))


@pytest.mark.parametrize("layout", [npbmz.LAYOUT_DENSE, npbmz.LAYOUT_REF], ids=["dense", "ref"])
def test_page_locked_transfers_match_pageable(layout):
    """Page-locked host buffers are read and written in place by one kernel
    per zone: the same values as the staged path for pageable memory, and
    the reference layout's halo is left as it was."""
    torch = pytest.importorskip("torch")
    g, dt = GEOMS["rect"]
    p, r = make(g(), dt)
    sizes = [lu.ref_elems(int(p.nx[z]), int(p.ny[z]), int(p.nz[z])) if layout == npbmz.LAYOUT_REF
             else 5 * int(p.nx[z]) * int(p.ny[z]) * int(p.nz[z]) for z in range(p.nzones)]
    total = int(sum(sizes))
    pinned = torch.full((total,), 7.25, dtype=torch.float64, pin_memory=True)
    pageable = np.full(total, 7.25)
    L = lu.lib()
    assert L.npbmz_lu_download(p._h, -1, lu.U, layout, pinned.data_ptr()) == 0
    assert L.npbmz_lu_download(p._h, -1, lu.U, layout, pageable.ctypes.data) == 0
    np.testing.assert_array_equal(pinned.numpy(), pageable)
    if layout == npbmz.LAYOUT_REF:
        assert np.count_nonzero(pageable == 7.25) > 0
    # upload a scaled copy through the pinned buffer and read it back
    pinned.mul_(1.5)
    assert L.npbmz_lu_upload(p._h, -1, lu.U, layout, pinned.data_ptr()) == 0
    for z in range(p.nzones):
        np.testing.assert_array_equal(p.download(z, lu.U), r.get(lu.U, z) * 1.5)


@pytest.mark.parametrize("flags", [0, lu.GRAPH, lu.GRAPH | lu.FMA], ids=["direct", "graph", "fma-graph"])
@pytest.mark.parametrize("m,value,bit,fatal", [(2, float("nan"), lu.STATE_NONFINITE, True),
                                               (0, -0.5, lu.STATE_DENSITY, True),
                                               (4, 1e-3, lu.STATE_PRESSURE, False)],
                         ids=["nan-momentum", "negative-density", "low-energy"])
def test_state_check_reports_a_planted_point(flags, m, value, bit, fatal):
    """Each iteration's update tests the points it writes: a non-finite value
    or a density that is not positive fails npbmz_lu_iterate with
    NPBMZ_LU_ERR_STATE; a non-positive pressure is only reported by
    npbmz_lu_state_check (LU never takes its root).  Planted from the host
    into one interior point of zone 1; a healthy run reports nothing."""
    g, dt = GEOMS["S"]
    p, _ = make(g(), dt, flags)
    p.iterate(2)
    assert p.state_check() == (0, (-1, -1, -1, -1))
    u = p.download(1, lu.U)
    u[m, 2, 3, 3] = value
    p.upload(1, lu.U, u)
    if fatal:
        with pytest.raises(npbmz.NpbmzError) as e:
            p.iterate(1)
        assert e.value.code == lu.ERR_STATE and "state check failed" in str(e.value)
    else:
        p.iterate(1)
    bits, (zone, i, j, k) = p.state_check()
    assert bits & bit and zone == 1
    if bit == lu.STATE_PRESSURE:
        assert (i, j, k) == (3, 3, 2)
