"""GPU parity against the CPU oracle, through the C ABI.

NPBMZ_EXACT builds the FP64 kernels without FMA contraction in the
reference's operation order: u, rhs and forcing must then be bit-for-bit the
oracle's.  The default (FMA-contracted) FP64 path must agree to 1e-12
relative in u, rhs and the per-step norms.  Norms are reductions whose
summation order differs from the reference's sequential loops, so they are
compared to 1e-13 relative even on the exact path.
"""
import numpy as np
import pytest

import npbmz

pytestmark = pytest.mark.gpu

EXACT_REL = 0.0      # bit-for-bit
FAST_REL = 1e-12     # FMA-contracted FP64 path
NORM_REL = 1e-13     # reduction order only


def geom_class(kind, cls):
    niter, dt, ratio, xz, yz, gx, gy, gz = npbmz.CLASSES[kind][cls]
    k = npbmz.KINDS[kind]
    nx, ny, nz, nbr = npbmz.zone_setup(k, gx, gy, gz, xz, yz, ratio)
    return npbmz.Geometry(k, nx, ny, nz, nbr, gx, gy, gz, xz, yz), dt, niter


def geom_bt24_widths():
    """BT 24x24x6 split 2x2 with x widths 8/16 and y widths 10/14."""
    nx, ny, nz, nbr = npbmz.zones_from_widths([8, 16], [10, 14], 6)
    return npbmz.Geometry(npbmz.BT, nx, ny, nz, nbr, 24, 24, 6, 2, 2), 0.010, 60


def make_pair(oracle_mod, geom, dt, flags, ce):
    p = npbmz.Problem(geom, dt, flags)
    p.setup(ce)
    o = oracle_mod.Oracle(geom.kind, geom.nx, geom.ny, geom.nz, geom.nbr, dt, geom.gx, geom.gy, geom.gz,
                          geom.x_zones, geom.y_zones, ce)
    return p, o


def seeded(geom, seed=3):
    ce, _ = npbmz.seeded_coefficients(seed, geom.nx, geom.ny, geom.nz, geom.gx, geom.gy, geom.gz, geom.x_zones,
                                      geom.y_zones)
    return ce


def compare(p, o, field, rel, zones=None):
    worst = 0.0
    for z in range(p.geom.nzones) if zones is None else zones:
        a = p.download(field, z)
        b = o.get(field, z)
        if rel == 0.0:
            np.testing.assert_array_equal(a, b, err_msg=f"field {field} zone {z}")
        else:
            scale = np.max(np.abs(b)) or 1.0
            err = np.max(np.abs(a - b)) / scale
            worst = max(worst, err)
            assert err <= rel, f"field {field} zone {z}: rel err {err:.3e} > {rel:.1e}"
    return worst


GEOMS = {
    "bt_classS": lambda: geom_class("BT", "S"),
    "bt_24x24x6_widths": geom_bt24_widths,
    "sp_classS": lambda: geom_class("SP", "S"),
}


@pytest.mark.parametrize("gname", list(GEOMS))
@pytest.mark.parametrize("ce_kind", ["reference", "seeded"])
def test_setup_is_bit_exact(oracle_mod, gname, ce_kind):
    geom, dt, _ = GEOMS[gname]()
    ce = npbmz.CE_REFERENCE if ce_kind == "reference" else seeded(geom)
    p, o = make_pair(oracle_mod, geom, dt, npbmz.EXACT, ce)
    compare(p, o, npbmz.U, EXACT_REL)
    compare(p, o, npbmz.FORCING, EXACT_REL)


@pytest.mark.parametrize("gname", list(GEOMS))
def test_each_phase_is_bit_exact(oracle_mod, gname):
    geom, dt, _ = GEOMS[gname]()
    p, o = make_pair(oracle_mod, geom, dt, npbmz.EXACT, seeded(geom))
    p.phase(npbmz.PHASE_EXCH)
    o.phase(5)
    compare(p, o, npbmz.U, EXACT_REL)
    for z in range(geom.nzones):
        p.phase(npbmz.PHASE_RHS, z)
        o.phase(0, z)
        compare(p, o, npbmz.RHS, EXACT_REL, [z])
        for ph in (npbmz.PHASE_XSOLVE, npbmz.PHASE_YSOLVE, npbmz.PHASE_ZSOLVE):
            p.phase(ph, z)
            o.phase(ph, z)
            compare(p, o, npbmz.RHS, EXACT_REL, [z])
        p.phase(npbmz.PHASE_ADD, z)
        o.phase(4, z)
        compare(p, o, npbmz.U, EXACT_REL, [z])


@pytest.mark.parametrize("gname", list(GEOMS))
def test_each_phase_fast_path_within_1e12(oracle_mod, gname):
    """The FMA build's phases (compute_rhs from the point-function planes and
    the merged linear stencil, the FMA sweeps) against the oracle, one phase
    at a time from identical inputs."""
    geom, dt, _ = GEOMS[gname]()
    p, o = make_pair(oracle_mod, geom, dt, 0, seeded(geom))
    p.phase(npbmz.PHASE_EXCH)
    o.phase(5)
    for z in range(geom.nzones):
        p.phase(npbmz.PHASE_RHS, z)
        o.phase(0, z)
        compare(p, o, npbmz.RHS, FAST_REL, [z])
        p.upload(npbmz.RHS, z, o.get(npbmz.RHS, z))
        for ph in (npbmz.PHASE_XSOLVE, npbmz.PHASE_YSOLVE, npbmz.PHASE_ZSOLVE):
            p.phase(ph, z)
            o.phase(ph, z)
            compare(p, o, npbmz.RHS, FAST_REL, [z])
            p.upload(npbmz.RHS, z, o.get(npbmz.RHS, z))


DF_RHS_REL = 1e-12   # compute_rhs in double-float (FP32 pairs, about 48 bits)


@pytest.mark.parametrize("gname", list(GEOMS))
def test_double_float_compute_rhs_phase(oracle_mod, gname):
    """NPBMZ_RHS_DF handles form the primitive variables and compute_rhs (with
    SP's txinvr) in double-float arithmetic on the FP32 pipe: the compute_rhs
    phase of each zone against the oracle from identical inputs."""
    geom, dt, _ = GEOMS[gname]()
    p, o = make_pair(oracle_mod, geom, dt, npbmz.MIXED | npbmz.RHS_DF, seeded(geom))
    p.phase(npbmz.PHASE_EXCH)
    o.phase(5)
    worst = 0.0
    for z in range(geom.nzones):
        p.phase(npbmz.PHASE_RHS, z)
        o.phase(0, z)
        worst = max(worst, compare(p, o, npbmz.RHS, DF_RHS_REL, [z]))
    print(f"double-float compute_rhs: worst rel err {worst:.3e}")


@pytest.mark.parametrize("kind", ["BT", "SP"])
def test_double_float_rhs_steps_match_fp64_rhs(kind):
    """The same refined mixed step with compute_rhs in double-float
    (NPBMZ_RHS_DF) and in FP64 (default): u and the verification norms after
    20 steps of class W agree to 1e-12."""
    geom, dt, _ = geom_class(kind, "W")
    ce = seeded(geom)
    a = npbmz.Problem(geom, dt, npbmz.MIXED | npbmz.RHS_DF)
    b = npbmz.Problem(geom, dt, npbmz.MIXED)
    a.setup(ce)
    b.setup(ce)
    a.step(20)
    b.step(20)
    worst = 0.0
    for z in range(geom.nzones):
        ua, ub = a.download(npbmz.U, z), b.download(npbmz.U, z)
        worst = max(worst, float(np.max(np.abs(ua - ub)) / np.max(np.abs(ub))))
    assert worst <= 1e-12, worst
    np.testing.assert_allclose(np.concatenate(a.verify()), np.concatenate(b.verify()), rtol=1e-12, atol=0)


@pytest.mark.parametrize("gname,nsteps", [("bt_24x24x6_widths", 60), ("bt_classS", 20), ("sp_classS", 40)])
def test_steps_exact_path_bit_exact(oracle_mod, gname, nsteps):
    geom, dt, _ = GEOMS[gname]()
    p, o = make_pair(oracle_mod, geom, dt, npbmz.EXACT, seeded(geom))
    ng = p.step(nsteps, norms=True)
    no = o.step(nsteps, norms=True)
    compare(p, o, npbmz.U, EXACT_REL)
    compare(p, o, npbmz.RHS, EXACT_REL)
    np.testing.assert_allclose(ng, no, rtol=NORM_REL, atol=0)


@pytest.mark.parametrize("gname,nsteps", [("bt_24x24x6_widths", 60), ("sp_classS", 100)])
def test_steps_fast_path_within_1e12(oracle_mod, gname, nsteps):
    geom, dt, _ = GEOMS[gname]()
    p, o = make_pair(oracle_mod, geom, dt, 0, seeded(geom))
    ng = p.step(nsteps, norms=True)
    no = o.step(nsteps, norms=True)
    compare(p, o, npbmz.U, FAST_REL)
    np.testing.assert_allclose(ng, no, rtol=FAST_REL, atol=0)
    xcr_g, xce_g = p.verify()
    xcr_o, xce_o = o.verify()
    np.testing.assert_allclose(xcr_g, xcr_o, rtol=FAST_REL)
    np.testing.assert_allclose(xce_g, xce_o, rtol=FAST_REL)


@pytest.mark.parametrize("kind,cls", [("BT", "S"), ("SP", "S"), ("BT", "W"), ("SP", "W")])
@pytest.mark.parametrize("flags", [npbmz.EXACT, 0])
def test_gpu_reproduces_npb_golden_norms(kind, cls, flags):
    xcr, xce, verified = npbmz.go(kind, cls, flags)
    assert verified is True
    g = npbmz.golden_norms(kind, cls)
    np.testing.assert_allclose(xcr, g[0], rtol=1e-11)
    np.testing.assert_allclose(xce, g[1], rtol=1e-11)


@pytest.mark.parametrize("kind,cls", [(k, c) for c in "ABC" for k in ("BT", "SP")])
@pytest.mark.parametrize("flags", [npbmz.EXACT | npbmz.GRAPH, npbmz.MIXED | npbmz.GRAPH])
def test_benchmark_classes_meet_the_golden_norms(kind, cls, flags):
    """Classes A, B and C (C: the 480x320x28 grid of 256 zones the benchmark
    times) over the reference's full step count verify against its norms, both
    the bit-exact FP64 step and the mixed-precision step of the headline."""
    xcr, xce, verified = npbmz.go(kind, cls, flags)
    assert verified is True, (xcr, xce)


def test_bt_class_d_meets_the_golden_norms():
    """BT class D (1632x1216x34, 67.5 M points in 1024 zones, about 85 GB on
    the device, 250 steps) on the mixed-precision graph step verifies against
    the reference's norms."""
    xcr, xce, verified = npbmz.go("BT", "D", npbmz.MIXED | npbmz.GRAPH)
    assert verified is True, (xcr, xce)


def test_perzone_launches_equal_batched(oracle_mod):
    geom, dt, _ = geom_bt24_widths()
    ce = seeded(geom)
    a = npbmz.Problem(geom, dt, npbmz.EXACT)
    b = npbmz.Problem(geom, dt, npbmz.EXACT | npbmz.PERZONE)
    a.setup(ce)
    b.setup(ce)
    a.step(10)
    b.step(10)
    for z in range(geom.nzones):
        np.testing.assert_array_equal(a.download(npbmz.U, z), b.download(npbmz.U, z))
    assert b.launches_per_step == 1 + 5 * geom.nzones and a.launches_per_step == 6


def test_graph_replay_equals_direct_launches():
    geom, dt, _ = geom_class("BT", "S")
    ce = seeded(geom)
    a = npbmz.Problem(geom, dt, 0)
    b = npbmz.Problem(geom, dt, npbmz.GRAPH)
    a.setup(ce)
    b.setup(ce)
    a.step(12)
    b.step(12)
    b.synchronize()
    for z in range(geom.nzones):
        np.testing.assert_array_equal(a.download(npbmz.U, z), b.download(npbmz.U, z))


@pytest.mark.parametrize("kind", ["BT", "SP"])
@pytest.mark.parametrize("flags", [0, npbmz.MIXED, npbmz.MIXED | npbmz.RHS_DF], ids=["fp64", "mixed", "mixed-dfrhs"])
@pytest.mark.parametrize("groups,prio,cap", [(2, False, 0), (3, False, 0), (5, False, 0), (2, True, 0), (4, True, 3),
                                             (3, False, 2)])
def test_zone_group_graph_equals_direct_launches(kind, flags, groups, prio, cap):
    """The step graph with zone-group branches (npbmz_set_step_groups), with
    or without the priority stream for the FP64 phases and a cap on the
    sweeps' resident CTAs (npbmz_set_step_overlap), runs the same kernels per
    zone: bit-identical to direct launches of the batched step (class W
    geometry, 16 zones; uneven for BT)."""
    geom, dt, _ = geom_class(kind, "W")
    ce = seeded(geom)
    a = npbmz.Problem(geom, dt, flags)
    b = npbmz.Problem(geom, dt, flags | npbmz.GRAPH)
    a.setup(ce)
    b.setup(ce)
    b.set_step_groups(groups)
    b.set_step_overlap(prio, cap)
    a.step(6)
    b.step(6)
    b.synchronize()
    for z in range(geom.nzones):
        np.testing.assert_array_equal(a.download(npbmz.U, z), b.download(npbmz.U, z))
    np.testing.assert_array_equal(np.concatenate(a.verify()), np.concatenate(b.verify()))


@pytest.mark.parametrize("kind", ["BT", "SP"])
@pytest.mark.parametrize("flags,groups", [(npbmz.MIXED | npbmz.GRAPH, 2), (npbmz.MIXED | npbmz.GRAPH, 1),
                                          (npbmz.MIXED, 1), (0, 1)],
                         ids=["mixed-graph-2groups", "mixed-graph", "mixed-direct", "fp64-direct"])
def test_copy_fusion_changes_no_result(kind, flags, groups):
    """The x sweep's x-line-major state copies made in the compute_rhs launch
    (npbmz_set_copy_fusion) leave u, rhs and the norms bit-identical to the
    separate copy kernel; class W geometry (16 zones, uneven for BT)."""
    geom, dt, _ = geom_class(kind, "W")
    ce = seeded(geom)
    a = npbmz.Problem(geom, dt, flags)
    b = npbmz.Problem(geom, dt, flags)
    for q in (a, b):
        q.setup(ce)
        if flags & npbmz.GRAPH:
            q.set_step_groups(groups)
    assert a.describe()["copy_fusion"]  # the default
    a.set_copy_fusion(False)
    b.set_copy_fusion(True)
    assert b.describe()["copy_fusion"] and not a.describe()["copy_fusion"]
    a.step(5)
    b.step(5)
    b.synchronize()
    for z in range(geom.nzones):
        np.testing.assert_array_equal(a.download(npbmz.U, z), b.download(npbmz.U, z))
        np.testing.assert_array_equal(a.download(npbmz.RHS, z), b.download(npbmz.RHS, z))
    np.testing.assert_array_equal(np.concatenate(a.verify()), np.concatenate(b.verify()))


@pytest.mark.parametrize("kind", ["BT", "SP"])
@pytest.mark.parametrize("flags,groups", [(npbmz.MIXED | npbmz.GRAPH, 3), (npbmz.GRAPH, 2), (npbmz.MIXED, 1)],
                         ids=["mixed-graph-3groups", "fp64-graph-2groups", "mixed-direct"])
def test_step_download_equals_step_then_download(kind, flags, groups):
    """npbmz_step_download (each zone group copied out of the last step as soon
    as its z sweep is done, into page-locked memory) leaves the same host array
    as npbmz_step followed by npbmz_download, and the same device state."""
    torch = pytest.importorskip("torch")
    geom, dt, _ = geom_class(kind, "W")
    ce = seeded(geom)
    sizes = [npbmz.ref_elems(geom.kind, npbmz.U, int(geom.nx[z]), int(geom.ny[z]), int(geom.nz[z]))
             for z in range(geom.nzones)]
    a = npbmz.Problem(geom, dt, flags)
    b = npbmz.Problem(geom, dt, flags)
    a.setup(ce)
    b.setup(ce)
    if flags & npbmz.GRAPH:
        a.set_step_groups(groups)
        b.set_step_groups(groups)
    ha = torch.full((sum(sizes),), -1.0, dtype=torch.float64, pin_memory=True)
    hb = torch.full((sum(sizes),), -1.0, dtype=torch.float64, pin_memory=True)
    for _ in range(3):
        a.step(2)
        a.transfer_raw(npbmz.U, -1, npbmz.LAYOUT_REF, ha.data_ptr(), False)
        b.step_download(2, npbmz.LAYOUT_REF, hb.data_ptr())
        np.testing.assert_array_equal(ha.numpy(), hb.numpy())
    for z in range(geom.nzones):
        np.testing.assert_array_equal(a.download(npbmz.U, z), b.download(npbmz.U, z))


@pytest.mark.parametrize("kind", ["BT", "SP"])
@pytest.mark.parametrize("flags,groups,prio,cap,nsteps", [
    (npbmz.MIXED | npbmz.GRAPH, 3, False, 0, 1), (npbmz.MIXED | npbmz.GRAPH, 2, True, 3, 2),
    (npbmz.GRAPH, 4, True, 0, 3), (npbmz.MIXED, 1, False, 0, 2)],
    ids=["mixed-graph-3groups", "mixed-graph-2groups-prio-cap3", "fp64-graph-4groups-prio", "mixed-direct"])
@pytest.mark.parametrize("layout", [npbmz.LAYOUT_REF, npbmz.LAYOUT_DENSE], ids=["ref", "dense"])
def test_step_inout_equals_upload_step_download(kind, flags, groups, prio, cap, nsteps, layout):
    """npbmz_step_inout (exch_qbc's source planes uploaded first, then each
    zone group's remaining points while earlier groups compute, each group
    copied out after its last z sweep) leaves the same host array and device
    state as npbmz_upload + npbmz_step + npbmz_download, from a host array
    that differs from the device state; in place (host_in == host_out) and
    into a second buffer."""
    torch = pytest.importorskip("torch")
    geom, dt, _ = geom_class(kind, "W")
    ce = seeded(geom)
    if layout == npbmz.LAYOUT_REF:
        total = sum(npbmz.ref_elems(geom.kind, npbmz.U, int(geom.nx[z]), int(geom.ny[z]), int(geom.nz[z]))
                    for z in range(geom.nzones))
    else:
        total = 5 * int(np.sum(geom.nx.astype(np.int64) * geom.ny * geom.nz))
    a = npbmz.Problem(geom, dt, flags)
    b = npbmz.Problem(geom, dt, flags)
    for q in (a, b):
        q.setup(ce)
        if flags & npbmz.GRAPH:
            q.set_step_groups(groups)
            q.set_step_overlap(prio, cap)
    # a host u one step ahead of the device state, perturbed, halo untouched
    src = npbmz.Problem(geom, dt, flags)
    src.setup(ce)
    src.step(1)
    h0 = torch.full((total,), -7.0, dtype=torch.float64, pin_memory=True)
    src.transfer_raw(npbmz.U, -1, layout, h0.data_ptr(), False)
    v = h0.numpy()
    v[v != -7.0] *= 1.0 + 1e-3 * np.sin(np.arange(int(np.sum(v != -7.0))))
    ha = h0.clone().pin_memory()
    hb_in = h0.clone().pin_memory()
    hb_out = torch.full((total,), -7.0, dtype=torch.float64, pin_memory=True)
    for rep in range(2):
        a.transfer_raw(npbmz.U, -1, layout, ha.data_ptr(), True)
        a.step(nsteps)
        a.transfer_raw(npbmz.U, -1, layout, ha.data_ptr(), False)
        if rep == 0:
            b.step_inout(nsteps, layout, hb_in.data_ptr(), hb_out.data_ptr())
            np.testing.assert_array_equal(ha.numpy(), hb_out.numpy())
            hb_in.copy_(hb_out)
        else:
            b.step_inout(nsteps, layout, hb_in.data_ptr(), hb_in.data_ptr())
            np.testing.assert_array_equal(ha.numpy(), hb_in.numpy())
    for z in range(geom.nzones):
        np.testing.assert_array_equal(a.download(npbmz.U, z), b.download(npbmz.U, z))


@pytest.mark.parametrize("kind", ["BT", "SP"])
@pytest.mark.parametrize("flags", [0, npbmz.MIXED, npbmz.MIXED | npbmz.GRAPH, npbmz.MIXED | npbmz.RHS_DF | npbmz.GRAPH],
                         ids=["fp64", "mixed", "mixed-graph", "mixed-dfrhs-graph"])
def test_persistent_kernels_equal_one_cta_per_item(kind, flags):
    """NPBMZ_PERSIST: the same work items looped over by a resident grid --
    bit-identical u and per-step norms."""
    geom, dt, _ = geom_class(kind, "W")
    ce = seeded(geom)
    a = npbmz.Problem(geom, dt, flags)
    b = npbmz.Problem(geom, dt, flags | npbmz.PERSIST)
    a.setup(ce)
    b.setup(ce)
    a.step(4)
    b.step(4)
    na = a.step(2, norms=True)
    nb = b.step(2, norms=True)
    np.testing.assert_array_equal(na, nb)
    for z in range(geom.nzones):
        np.testing.assert_array_equal(a.download(npbmz.U, z), b.download(npbmz.U, z))


def test_reference_layout_round_trip():
    """Upload u in the reference's OffsetArray memory layout, download it dense
    and in the reference layout again (halo untouched)."""
    for kind in ("BT", "SP"):
        geom, dt, _ = geom_class(kind, "S")
        p = npbmz.Problem(geom, dt, 0)
        p.setup()
        rng = np.random.default_rng(5)
        for z in range(geom.nzones):
            nx, ny, nz = int(geom.nx[z]), int(geom.ny[z]), int(geom.nz[z])
            n = npbmz.ref_elems(geom.kind, npbmz.U, nx, ny, nz)
            ref = rng.standard_normal(n)
            p.transfer_raw(npbmz.U, z, npbmz.LAYOUT_REF, ref.ctypes.data, True)
            dense = p.download(npbmz.U, z)
            IMAX, JMAX, KMAX = nx + 1, ny + 1, nz + 1
            if geom.kind == npbmz.BT:
                v = ref.reshape(KMAX + 4, JMAX + 4, IMAX + 4, 5)  # column-major [m,i,j,k] viewed C-order
                expect = np.transpose(v[2:2 + nz, 2:2 + ny, 2:2 + nx, :], (3, 0, 1, 2))
            else:
                IMAXP, JMAXP = (IMAX // 2) * 2 + 1, (JMAX // 2) * 2 + 1
                v = ref.reshape(5, KMAX + 4, JMAXP + 4, IMAXP + 4)
                expect = v[:, 2:2 + nz, 2:2 + ny, 2:2 + nx]
            np.testing.assert_array_equal(dense, expect)
            back = np.full(n, -7.0)
            p.transfer_raw(npbmz.U, z, npbmz.LAYOUT_REF, back.ctypes.data, False)
            touched = back != -7.0
            np.testing.assert_array_equal(back[touched], ref[touched])
            assert touched.sum() == 5 * nx * ny * nz


def test_errors_are_reported_not_raised_across_the_abi():
    geom, dt, _ = geom_class("BT", "S")
    p = npbmz.Problem(geom, dt, 0)
    with pytest.raises(npbmz.NpbmzError, match="bad zone"):
        p.adi(99)
    with pytest.raises(npbmz.NpbmzError, match="bad phase"):
        p.phase(42)
    bad = npbmz.Geometry(npbmz.BT, np.array([2], np.int32), np.array([5], np.int32), np.array([5], np.int32),
                         np.zeros(4, np.int32), 2, 5, 5, 1, 1)
    with pytest.raises(npbmz.NpbmzError, match="minimum is 3"):
        npbmz.Problem(bad, 0.01, 0)


MIXED_REL = 1e-10   # FP32 line solves refined against an FP64 residual


@pytest.mark.parametrize("gname,nsteps", [("bt_24x24x6_widths", 60), ("bt_classS", 60), ("sp_classS", 100)])
@pytest.mark.parametrize("flags", [npbmz.MIXED, npbmz.MIXED | npbmz.RHS_DF, npbmz.MIXED | npbmz.REFINE_FP64],
                         ids=["df64-residual", "df64-rhs", "fp64-residual"])
def test_mixed_precision_within_1e10_of_fp64_oracle(oracle_mod, gname, nsteps, flags):
    geom, dt, _ = GEOMS[gname]()
    p, o = make_pair(oracle_mod, geom, dt, flags, seeded(geom))
    ng = p.step(nsteps, norms=True)
    no = o.step(nsteps, norms=True)
    err_u = compare(p, o, npbmz.U, MIXED_REL)
    np.testing.assert_allclose(ng, no, rtol=MIXED_REL, atol=0)
    # the unrefined FP32 solve is far from that bar: the refinement is what meets it
    q = npbmz.Problem(geom, dt, npbmz.FP32_NOREFINE)
    q.setup(seeded(geom))
    q.step(nsteps)
    err_plain = max(np.max(np.abs(q.download(npbmz.U, z) - o.get(0, z))) / np.max(np.abs(o.get(0, z)))
                    for z in range(geom.nzones))
    assert err_plain > 100 * max(err_u, 1e-16)


def test_mixed_precision_golden_norms():
    """With refinement the FP32 line solves still verify the NPB classes."""
    for kind, cls in (("BT", "W"), ("SP", "W")):
        xcr, xce, verified = npbmz.go(kind, cls, npbmz.MIXED)
        assert verified is True


def test_reference_layout_round_trip_pinned():
    """Page-locked host arrays take the zero-copy path (one kernel each way)."""
    torch = pytest.importorskip("torch")
    for kind in ("BT", "SP"):
        geom, dt, _ = geom_class(kind, "S")
        p = npbmz.Problem(geom, dt, 0)
        p.setup()
        sizes = [npbmz.ref_elems(geom.kind, npbmz.U, int(geom.nx[z]), int(geom.ny[z]), int(geom.nz[z]))
                 for z in range(geom.nzones)]
        host = torch.full((sum(sizes),), -3.0, dtype=torch.float64, pin_memory=True)
        p.transfer_raw(npbmz.U, -1, npbmz.LAYOUT_REF, host.data_ptr(), False)
        h = host.numpy().copy()
        off = 0
        for z in range(geom.nzones):
            seg = h[off:off + sizes[z]]
            assert int((seg != -3.0).sum()) == 5 * int(geom.nx[z] * geom.ny[z] * geom.nz[z])
            off += sizes[z]
        # upload a perturbed copy and read it back dense
        host2 = torch.tensor(h * 1.5, dtype=torch.float64).pin_memory()
        p.transfer_raw(npbmz.U, -1, npbmz.LAYOUT_REF, host2.data_ptr(), True)
        before = [p.download(npbmz.U, z) for z in range(geom.nzones)]
        p.transfer_raw(npbmz.U, -1, npbmz.LAYOUT_REF, host.data_ptr(), False)
        np.testing.assert_array_equal(host.numpy()[host.numpy() != -3.0], (h * 1.5)[h != -3.0])
        assert all(np.all(np.isfinite(b)) for b in before)


# ---- the benchmark configurations at full size (the oracle runs them on the host cores) ----

def test_sp_class_a_per_step_norms(oracle_mod):
    """SP-MZ 128x128x16 split 4x4 (32x32x16 zones), dt 1.5e-3, 400 steps: per-step
    residual and error norms of the FP64 GPU path within 1e-12 of the oracle."""
    geom, dt, niter = geom_class("SP", "A")
    p, o = make_pair(oracle_mod, geom, dt, 0, seeded(geom))
    ng = p.step(niter, norms=True)
    no = o.step(niter, norms=True)
    np.testing.assert_allclose(ng, no, rtol=FAST_REL, atol=0)
    compare(p, o, npbmz.U, FAST_REL)


@pytest.mark.parametrize("flags,rel", [(0, FAST_REL), (npbmz.MIXED, MIXED_REL), (npbmz.MIXED | npbmz.GRAPH, MIXED_REL)],
                         ids=["fp64", "mixed", "mixed-graph"])
def test_bt_class_b_final_norms(oracle_mod, flags, rel):
    """BT-MZ 304x208x17 split 8x8 (area ratio 20.05), dt 3e-4, 200 steps, batched:
    final norms of each variant against the FP64 oracle."""
    geom, dt, niter = geom_class("BT", "B")
    p, o = make_pair(oracle_mod, geom, dt, flags, seeded(geom))
    p.step(niter)
    o.step(niter)
    p.synchronize()
    xg = np.concatenate(p.verify())
    xo = np.concatenate(o.verify())
    np.testing.assert_allclose(xg, xo, rtol=rel, atol=0)


@pytest.mark.parametrize("flags", [0, npbmz.MIXED | npbmz.GRAPH], ids=["fp64", "mixed-graph"])
def test_bt_class_b_autotuned_launch_shapes_keep_results(oracle_mod, flags):
    """The autotuner (lines per CTA per sweep direction and zone-size bucket;
    zone-group branches for graph handles) changes launch shapes only: the
    state it leaves is the one it found, and later steps are bit-identical
    to untuned direct launches."""
    geom, dt, niter = geom_class("BT", "B")
    ce = seeded(geom)
    a = npbmz.Problem(geom, dt, flags)
    a.setup(ce)
    u_before = [a.download(npbmz.U, z) for z in range(geom.nzones)]
    a.autotune()
    d = a.describe()
    assert d["zone_size_buckets"] in (1, 3) and len(d["lines_per_cta"]) == 3
    assert d["persistent"] in (True, False)
    assert all(len(per_dir) == d["zone_size_buckets"] for per_dir in d["lines_per_cta"])
    assert all(t in (32, 64, 128) for per_dir in d["lines_per_cta"] for t in per_dir)
    for z in range(geom.nzones):
        np.testing.assert_array_equal(a.download(npbmz.U, z), u_before[z])
    b = npbmz.Problem(geom, dt, flags & ~npbmz.GRAPH)
    b.setup(ce)
    a.step(5)
    b.step(5)
    a.synchronize()
    for z in range(0, geom.nzones, 7):
        np.testing.assert_array_equal(a.download(npbmz.U, z), b.download(npbmz.U, z))


def test_fma_build_reciprocal_error_bound():
    """The FMA build's primitive kernel takes 1/rho by Newton-Raphson
    refinement of the FP32 hardware estimate (npbmz_math_check runs the same
    device function).  Against numpy's correctly rounded 1/x it stays within
    2 ulps over the range the state takes and far beyond it; outside the FP32
    range it falls back to the IEEE divide."""
    import ctypes

    rng = np.random.default_rng(17)
    x = np.concatenate([10.0 ** rng.uniform(-30, 30, 200000), rng.uniform(0.01, 100.0, 200000),
                        np.array([1.0, 2.0, 0.5, 3.0, 1e-37, 1e37, 1e-300, 1e300, 7.0, 1.0 - 2 ** -52])])
    y = np.zeros_like(x)
    dp = ctypes.POINTER(ctypes.c_double)
    assert npbmz.lib().npbmz_math_check(0, len(x), x.ctypes.data_as(dp), y.ctypes.data_as(dp)) == 0
    want = 1.0 / x
    err_ulps = np.abs(y - want) / np.spacing(want)
    assert np.max(err_ulps) <= 2, (np.max(err_ulps), x[np.argmax(err_ulps)])
