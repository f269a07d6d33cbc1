"""Discrete adjoint of the BT-MZ and SP-MZ steps (npbmz_adjoint) on the GPU.

Workload: BT-MZ 64x64x8 split 4x4 (zone_setup with per-axis ratio sqrt(6):
widths 10/13/17/24, area ratio 5.76), dt 8e-4, 50 steps, seeded polynomial
initial state, checkpoints every 10 steps.  Objective
J = 1/2 sum over every stored point (u_50 - u_target)^2 with u_target the
manufactured solution (exact_solution, src/BT/exact_solution.jl:5-18) of the
coefficients perturbed by seeded N(0, 0.01).

The gradient with respect to the forcing and to u_0 is checked against
central finite differences of the GPU forward path (npbmz_step) along 16
seeded Gaussian directions each, to 1e-6 relative.  The
difference J(x + h d) - J(x - h d) is formed as 1/2 sum (a+ - a-)(a+ + a-)
with a = u_50 - u_target, so that it carries no cancellation error from two
separately rounded sums of 160k terms.  How the directions are scaled decides
whether h = 1e-6 lies between the rounding floor of the forward run (error
~ 1/h) and the curvature of the 50-step map (error ~ h^2); measured on
this workload (max relative error over the 16 directions at h = 1e-6):
  u_0, entries of unit RMS (absolute h; rho ~ 800 and rho E ~ 6e4 in the
      seeded state): 6.4e-7;  scaled by each variable's RMS: 1.1e-4
      (curvature);
  forcing, scaled by each variable's RMS: 7.2e-7 .. 1.2e-6 (depending on
      the rounding of the forward kernels);  unit RMS: 3.6e-6 (rounding).
The forcing moves u only through dt * forcing (dt = 8e-4, forcing RMS ~ 10
against u RMS ~ 1e3), so a relative forcing perturbation of 1e-6 changes u_50
by ~1e-10 relative and its difference quotient sits on the rounding floor of
the forward run.  So u_0 directions have unit-RMS entries, at h = 2e-6 (see
the test: the forward path's current rounding puts the floor at h = 1e-6 at
1.2e-6), and forcing directions are scaled per variable at h = 1e-5 (worst
of 16: 4.6e-8; J is nearly linear in the forcing, so the O(h^2) term stays
below 1e-9).  SP-MZ (below) meets the bar at h = 1e-6 for u_0.

The gradient is also checked against forward-mode dual numbers pushed
through the CPU oracle's BT and SP steps (oracle/npbmz_tangent.cpp, the stand-in for
ForwardDiff through the reference's Julia code) along 8 directions in u_0
and 8 in the forcing, to 1e-9 relative: both are exact derivatives of the
same discrete step, apart from rounding and the FMA contraction of the GPU
forward path (1e-12 relative in u).
"""
import math

import numpy as np
import pytest

import npbmz

pytestmark = pytest.mark.gpu

ADJ_REL = 1e-6   # adjoint vs central finite differences
DUAL_REL = 1e-9  # adjoint vs dual numbers through the oracle
H = 1e-6
NDIR = 16


def geom_bt64():
    gx, gy, gz, xz, yz = 64, 64, 8, 4, 4
    nx, ny, nz, nbr = npbmz.zone_setup(npbmz.BT, gx, gy, gz, xz, yz, math.sqrt(6.0))
    return npbmz.Geometry(npbmz.BT, nx, ny, nz, nbr, gx, gy, gz, xz, yz), 0.0008, 50


def manufactured(geom, ce):
    """exact_solution at every stored point of every zone, dense per zone."""
    dnx = 1.0 / ((geom.gx - 1) / geom.x_zones)
    dny = 1.0 / ((geom.gy - 1) / geom.y_zones)
    dnz = 1.0 / (geom.gz - 1)
    out = []
    for z in range(geom.nzones):
        k, j, i = np.meshgrid(np.arange(geom.nz[z]), np.arange(geom.ny[z]), np.arange(geom.nx[z]), indexing="ij")
        xi, eta, zeta = i * dnx, j * dny, k * dnz
        u = np.empty((5,) + xi.shape)
        for m in range(5):
            c = ce[m]
            u[m] = (c[0] + xi * (c[1] + xi * (c[4] + xi * (c[7] + xi * c[10])))
                    + eta * (c[2] + eta * (c[5] + eta * (c[8] + eta * c[11])))
                    + zeta * (c[3] + zeta * (c[6] + zeta * (c[9] + zeta * c[12]))))
        out.append(u)
    return out


def build_case(geom, dt, flags=0, seed=3):
    ce, _ = npbmz.seeded_coefficients(seed, geom.nx, geom.ny, geom.nz, geom.gx, geom.gy, geom.gz, geom.x_zones,
                                      geom.y_zones)
    p = npbmz.Problem(geom, dt, flags)
    p.setup(ce)
    rng = np.random.default_rng(seed + 1000)
    target = manufactured(geom, ce + rng.normal(0.0, 0.01, ce.shape))
    return p, ce, target


def variable_scale(p, x):
    """Per-entry scale of a flat dense field: the RMS of its conserved
    variable over all zones."""
    zones = p.split(x)
    rms = [math.sqrt(math.fsum(float(np.sum(a[m] * a[m])) for a in zones) / sum(a[m].size for a in zones))
           for m in range(5)]
    return p.flatten([np.broadcast_to(np.array(rms)[:, None, None, None], a.shape) for a in zones])


def unit_directions(p, n, x, seed, per_variable):
    """n seeded Gaussian directions of unit RMS; per_variable: the entries of
    variable m scaled by the RMS of variable m in x."""
    rng = np.random.default_rng(seed)
    d = rng.standard_normal((n, x.size))
    d *= math.sqrt(x.size) / np.linalg.norm(d, axis=1, keepdims=True)
    return d * variable_scale(p, x) if per_variable else d


def terminal_state(p, field, base, base_other, other_field, nsteps):
    """u_N after nsteps from the given forcing / u_0 (flat dense arrays)."""
    p.upload_all(field, base)
    p.upload_all(other_field, base_other)
    p.step(nsteps)
    p.synchronize()
    return np.concatenate([a.reshape(-1) for a in p.download_all(npbmz.U)])


def fd_check(p, target, nsteps, every, field, seed, h=H):
    u0 = p.flatten(p.download_all(npbmz.U))
    f0 = p.flatten(p.download_all(npbmz.FORCING))
    t = p.flatten(target)
    J, gf, gu = p.adjoint(nsteps, target, checkpoint_every=every)
    grad = p.flatten(gf if field == npbmz.FORCING else gu)
    x0, other, other_field = (f0, u0, npbmz.U) if field == npbmz.FORCING else (u0, f0, npbmz.FORCING)
    errs = []
    for d in unit_directions(p, NDIR, x0, seed, per_variable=(field == npbmz.FORCING)):
        ap = terminal_state(p, field, x0 + h * d, other, other_field, nsteps) - t
        am = terminal_state(p, field, x0 - h * d, other, other_field, nsteps) - t
        fd = math.fsum(0.5 * (ap - am) * (ap + am)) / (2.0 * h)
        ad = float(np.dot(grad, d))
        errs.append(abs(fd - ad) / abs(ad))
    # restore the unperturbed state
    p.upload_all(npbmz.U, u0)
    p.upload_all(npbmz.FORCING, f0)
    return J, grad, errs


@pytest.fixture(scope="module")
def bt64():
    geom, dt, nsteps = geom_bt64()
    p, ce, target = build_case(geom, dt)
    return p, target, nsteps


@pytest.mark.parametrize("field,h", [(npbmz.FORCING, 1e-5), (npbmz.U, 2e-6)], ids=["forcing", "u0"])
def test_bt64_adjoint_matches_central_differences(bt64, field, h):
    """u_0 at h = 2e-6: with the FP64 compute_rhs that folds dt into its
    factors, the forward path's rounding puts the difference quotient's floor
    at h = 1e-6 right at the bar (worst of 16: 1.18e-6, median 1.4e-7);
    measured worst at h = 2e-6, 3e-6, 5e-6: 4.9e-7, 3.9e-7, 2.1e-7 (no
    curvature term visible yet)."""
    p, target, nsteps = bt64
    J, grad, errs = fd_check(p, target, nsteps, 10, field, seed=77, h=h)
    print(f"field {field} h {h:.0e}: worst {max(errs):.2e}, median {np.median(errs):.2e}")
    assert J > 0.0 and np.all(np.isfinite(grad))
    assert max(errs) <= ADJ_REL, f"max rel err {max(errs):.3e} over {NDIR} directions: {errs}"


def test_bt64_adjoint_matches_dual_numbers(bt64):
    from oracle import oracle

    p, target, nsteps = bt64
    g = p.geom
    u0 = p.flatten(p.download_all(npbmz.U))
    f0 = p.flatten(p.download_all(npbmz.FORCING))
    t = p.flatten(target)
    J, gf, gu = p.adjoint(nsteps, target, checkpoint_every=10)
    rng = np.random.default_rng(2024)
    du = np.zeros((16, u0.size))
    df = np.zeros((16, u0.size))
    du[:8] = rng.standard_normal((8, u0.size)) * variable_scale(p, u0)
    df[8:] = rng.standard_normal((8, u0.size)) * variable_scale(p, f0)
    Jd, dJ, _ = oracle.tangent_objective(oracle.KIND_BT, g.nx, g.ny, g.nz, g.nbr, p.dt, g.gx, g.gy, g.gz, g.x_zones,
                                         g.y_zones, u0, f0, t, nsteps, du0=du, dforcing=df)
    assert J == pytest.approx(Jd, rel=1e-10)
    ad = du @ p.flatten(gu) + df @ p.flatten(gf)
    rel = np.abs(ad - dJ) / np.abs(dJ)
    assert rel.max() <= DUAL_REL, rel


def test_bt64_objective_matches_forward_path(bt64):
    """J from the adjoint call equals J of a plain forward run, and the call
    leaves u as it was."""
    p, target, nsteps = bt64
    u0 = p.flatten(p.download_all(npbmz.U))
    J, _, _ = p.adjoint(nsteps, target, checkpoint_every=10, grad_forcing=False, grad_u0=False)
    assert np.array_equal(p.flatten(p.download_all(npbmz.U)), u0)
    p.step(nsteps)
    p.synchronize()
    a = p.flatten(p.download_all(npbmz.U)) - p.flatten(target)
    np.testing.assert_allclose(J, 0.5 * math.fsum(a * a), rtol=1e-12)
    p.upload_all(npbmz.U, u0)


def test_checkpoint_interval_does_not_change_the_gradient(bt64):
    """Recomputation is deterministic: every checkpoint interval gives the
    same bits."""
    p, target, nsteps = bt64
    ref = p.adjoint(nsteps, target, checkpoint_every=10)
    for every in (1, 7, 50, 64):
        got = p.adjoint(nsteps, target, checkpoint_every=every)
        assert got[0] == ref[0]
        for a, b in zip(got[1] + got[2], ref[1] + ref[2]):
            np.testing.assert_array_equal(a, b)


def test_single_zone_adjoint_without_exchange():
    """One zone: no exch_qbc in the step (bt-node.jl:286), so none in the
    adjoint.  12x10x7, dt 5e-3, 12 steps; h = 1e-5, where both fields sit
    clear of the rounding floor (at 1e-6 the worst of 16 directions is
    3.6e-6 for u_0 and 1.4e-6 for the forcing, at 1e-5 3.7e-7 and 1.9e-7)."""
    nx, ny, nz, nbr = npbmz.zones_from_widths([12], [10], 7)
    geom = npbmz.Geometry(npbmz.BT, nx, ny, nz, nbr, 12, 10, 7, 1, 1)
    p, _, target = build_case(geom, 0.005, seed=11)
    for field in (npbmz.FORCING, npbmz.U):
        _, _, errs = fd_check(p, target, 12, 5, field, seed=77, h=1e-5)
        assert max(errs) <= ADJ_REL, errs


def test_adjoint_rejects_bad_arguments(bt64):
    p, target, _ = bt64
    with pytest.raises(npbmz.NpbmzError, match="checkpoint_every"):
        p.adjoint(5, target, checkpoint_every=0)
    with pytest.raises(npbmz.NpbmzError, match="nsteps"):
        p.adjoint(0, target)


# ---- SP-MZ ----------------------------------------------------------------------
# SP-MZ 64x64x8 split 4x4 into equal 16x16x8 zones, dt 1.5e-3 (the class W
# geometry), 30 steps, checkpoints every 10.  The transposed pentadiagonal
# sweeps, the transposes of ninvr / pinvr / tzetar / txinvr and the
# linearisations of the bands (velocity, rhon, speed of each column's point)
# and of tzetar / txinvr in the state are SP's own; compute_rhs and exch_qbc
# share BT's adjoint.

def geom_sp():
    gx, gy, gz, xz, yz = 64, 64, 8, 4, 4
    nx, ny, nz, nbr = npbmz.zone_setup(npbmz.SP, gx, gy, gz, xz, yz, 1.0)
    return npbmz.Geometry(npbmz.SP, nx, ny, nz, nbr, gx, gy, gz, xz, yz), 0.0015, 30


@pytest.fixture(scope="module")
def sp_case():
    geom, dt, nsteps = geom_sp()
    p, ce, target = build_case(geom, dt, seed=5)
    return p, target, nsteps


@pytest.mark.parametrize("field,h", [(npbmz.FORCING, 1e-5), (npbmz.U, 1e-6)], ids=["forcing", "u0"])
def test_sp_adjoint_matches_central_differences(sp_case, field, h):
    p, target, nsteps = sp_case
    J, grad, errs = fd_check(p, target, nsteps, 10, field, seed=91, h=h)
    print(f"SP field {field} h {h:.0e}: worst {max(errs):.2e}, median {np.median(errs):.2e}")
    assert J > 0.0 and np.all(np.isfinite(grad))
    assert max(errs) <= ADJ_REL, f"max rel err {max(errs):.3e} over {NDIR} directions: {errs}"


def test_sp_adjoint_matches_dual_numbers(sp_case):
    """The SP adjoint against dual numbers through the oracle's SP step (line
    solves in FP64 there, as on this path) along 8 directions in u_0 and 8 in
    the forcing, to 1e-9 relative."""
    from oracle import oracle

    p, target, nsteps = sp_case
    g = p.geom
    u0 = p.flatten(p.download_all(npbmz.U))
    f0 = p.flatten(p.download_all(npbmz.FORCING))
    t = p.flatten(target)
    J, gf, gu = p.adjoint(nsteps, target, checkpoint_every=10)
    rng = np.random.default_rng(2025)
    du = np.zeros((16, u0.size))
    df = np.zeros((16, u0.size))
    du[:8] = rng.standard_normal((8, u0.size)) * variable_scale(p, u0)
    df[8:] = rng.standard_normal((8, u0.size)) * variable_scale(p, f0)
    Jd, dJ, _ = oracle.tangent_objective(oracle.KIND_SP, g.nx, g.ny, g.nz, g.nbr, p.dt, g.gx, g.gy, g.gz, g.x_zones,
                                         g.y_zones, u0, f0, t, nsteps, du0=du, dforcing=df)
    assert J == pytest.approx(Jd, rel=1e-10)
    ad = du @ p.flatten(gu) + df @ p.flatten(gf)
    rel = np.abs(ad - dJ) / np.abs(dJ)
    print(f"SP adjoint vs dual numbers: worst {rel.max():.2e}")
    assert rel.max() <= DUAL_REL, rel


def test_sp_checkpoint_interval_does_not_change_the_gradient(sp_case):
    p, target, nsteps = sp_case
    ref = p.adjoint(nsteps, target, checkpoint_every=10)
    for every in (1, 7, 30):
        got = p.adjoint(nsteps, target, checkpoint_every=every)
        assert got[0] == ref[0]
        for a, b in zip(got[1] + got[2], ref[1] + ref[2]):
            np.testing.assert_array_equal(a, b)


def test_sp_objective_matches_forward_path(sp_case):
    p, target, nsteps = sp_case
    u0 = p.flatten(p.download_all(npbmz.U))
    J, _, _ = p.adjoint(nsteps, target, checkpoint_every=10, grad_forcing=False, grad_u0=False)
    assert np.array_equal(p.flatten(p.download_all(npbmz.U)), u0)
    p.step(nsteps)
    p.synchronize()
    a = p.flatten(p.download_all(npbmz.U)) - p.flatten(target)
    np.testing.assert_allclose(J, 0.5 * math.fsum(a * a), rtol=1e-12)
    p.upload_all(npbmz.U, u0)


def test_torch_autograd_function(bt64):
    """TerminalObjective (the torch.autograd counterpart of the Julia rrule)
    returns the adjoint's J and gradients."""
    torch = pytest.importorskip("torch")
    from npbmz.autograd import terminal_objective

    p, target, nsteps = bt64
    u0 = p.flatten(p.download_all(npbmz.U))
    f0 = p.flatten(p.download_all(npbmz.FORCING))
    J0, gf, gu = p.adjoint(nsteps, target, checkpoint_every=10)
    f = torch.tensor(f0, requires_grad=True)
    u = torch.tensor(u0, requires_grad=True)
    J = terminal_objective(p, f, u, torch.tensor(p.flatten(target)), nsteps)
    (2.0 * J).backward()
    assert float(J.detach()) == J0
    np.testing.assert_array_equal(f.grad.numpy(), 2.0 * p.flatten(gf))
    np.testing.assert_array_equal(u.grad.numpy(), 2.0 * p.flatten(gu))
