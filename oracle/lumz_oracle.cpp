// lumz_oracle.cpp -- CPU restatement of NPBApps.jl's LU-MZ single-rank SSOR
// iteration (TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg and reference arm load liblumz_oracle.so, to
// compare the GPU LU path against or to time the reference's CPU path;
// nothing in the product links it).
//
// One MPI rank per zone, one process (the reference's single-rank case):
// every zone is a whole LU domain (row = col = 1, all four process
// neighbours -1, so ist = jst = 2, iend = nx-1, jend = ny-1, ipt = jpt = 0)
// and the exchange_1/3/4/5/6 calls inside ssor, rhs, erhs and pintgr send
// nothing.  Zones couple only through exch_qbc.
//
//   zone_setup ....... src/LU/zone_setup.jl:1-111 (LU's own neighbour rule:
//                      north/south along x, west/east along y)
//   setcoeff ......... src/LU/setcoeff.jl (per zone: dxi, tx1.. from the zone's
//                      own nx0, ny0, nz0)
//   setbv / setiv .... src/LU/setbv.jl, src/LU/setiv.jl, exact src/LU/exact.jl
//   erhs ............. src/LU/erhs.jl
//   rhs .............. src/LU/rhs.jl
//   ssor ............. src/LU/ssor.jl:9-254 (jacld/blts, jacu/buts, update, rhs)
//   jacld / blts ..... src/LU/jacld.jl, src/LU/blts.jl
//   jacu / buts ...... src/LU/jacu.jl, src/LU/buts.jl
//   exch_qbc ......... src/LU/exchange_qbc.jl:1-288
//   l2norm / error ... src/LU/l2norm.jl, src/LU/error.jl
//   pintgr ........... src/LU/pintgr.jl
//
// buts: the reference's Julia statements of the back substitution read
//   tv3 -= t34*tv4 - t35*tv5;  tv2 -= t23*tv3 - t24*tv4 - t25*tv5;
//   tv1 -= t12*tv2 - t13*tv3 - t14*tv4 - t15*tv5
// and the elimination has `tmat[5,5] -=- tmp * tmat[2,5]` (i.e. +=), where
// NPB's LU and blts in the same reference subtract every term.  They are
// restated as written; they change no value: d (jacu's diagonal block) is
// lower triangular, its strict upper triangle stays +0 through the
// elimination, and every term those signs touch is a product with it.
//
// exch_qbc: the reference copies the face planes k = 1..nz-2
// (src/LU/exchange_qbc.jl:85,109,135,160); NPB-MZ's LU-MZ copies the
// interior planes k = 2..nz-1.  Plane nz-1 is read by the solver and plane 1
// is not, so the two differ, and only k = 2..nz-1 reproduces the reference's
// own verification norms (src/LU/verify.jl).  `faces_npb` selects it; the
// default follows the reference.

// Array layout here: AoS per zone, point (i, j, k) 1-based as in the
// reference, element m (1..5) at ((k-1)*ny + (j-1))*nx + (i-1)) * 5 + m-1.
// -ffp-contract=off (oracle/Makefile): Julia never fuses a*b+c.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

const double c1 = 1.40e+00, c2 = 0.40e+00, c3 = 1.00e-01, c4 = 1.00e+00, c5 = 1.40e+00;
const double dx1 = 0.75e+00, dx2 = dx1, dx3 = dx1, dx4 = dx1, dx5 = dx1;
const double dy1 = 0.75e+00, dy2 = dy1, dy3 = dy1, dy4 = dy1, dy5 = dy1;
const double dz1 = 1.00e+00, dz2 = dz1, dz3 = dz1, dz4 = dz1, dz5 = dz1;
const double dssp = std::max(dx1, std::max(dy1, dz1)) / 4.0e+00;
const int ii1 = 2, ji1 = 2, ki1 = 3;

// the reference's ce table (src/LU/setcoeff.jl), row m = 1..5, 13 columns
const double ce_reference[5][13] = {
    {2.0e0, 0.0e0, 0.0e0, 4.0e0, 5.0e0, 3.0e0, 0.5e0, 0.02e0, 0.01e0, 0.03e0, 0.5e0, 0.4e0, 0.3e0},
    {1.0e0, 0.0e0, 0.0e0, 0.0e0, 1.0e0, 2.0e0, 3.0e0, 0.01e0, 0.03e0, 0.02e0, 0.4e0, 0.3e0, 0.5e0},
    {2.0e0, 2.0e0, 0.0e0, 0.0e0, 0.0e0, 2.0e0, 3.0e0, 0.04e0, 0.03e0, 0.05e0, 0.3e0, 0.5e0, 0.4e0},
    {2.0e0, 2.0e0, 0.0e0, 0.0e0, 0.0e0, 2.0e0, 3.0e0, 0.03e0, 0.05e0, 0.04e0, 0.2e0, 0.1e0, 0.3e0},
    {5.0e0, 4.0e0, 3.0e0, 2.0e0, 0.1e0, 0.4e0, 0.3e0, 0.05e0, 0.04e0, 0.03e0, 0.1e0, 0.3e0, 0.2e0}};

struct Coeff {  // setcoeff for one zone
  double dxi, deta, dzeta, tx1, tx2, tx3, ty1, ty2, ty3, tz1, tz2, tz3;
  int ii2, ji2, ki2;
};

Coeff setcoeff(int nx0, int ny0, int nz0) {
  Coeff C;
  C.dxi = 1.0e+00 / (nx0 - 1);
  C.deta = 1.0e+00 / (ny0 - 1);
  C.dzeta = 1.0e+00 / (nz0 - 1);
  C.tx1 = 1.0e+00 / (C.dxi * C.dxi);
  C.tx2 = 1.0e+00 / (2.0e+00 * C.dxi);
  C.tx3 = 1.0e+00 / C.dxi;
  C.ty1 = 1.0e+00 / (C.deta * C.deta);
  C.ty2 = 1.0e+00 / (2.0e+00 * C.deta);
  C.ty3 = 1.0e+00 / C.deta;
  C.tz1 = 1.0e+00 / (C.dzeta * C.dzeta);
  C.tz2 = 1.0e+00 / (2.0e+00 * C.dzeta);
  C.tz3 = 1.0e+00 / C.dzeta;
  C.ii2 = nx0 - 1;
  C.ji2 = ny0 - 2;
  C.ki2 = nz0 - 1;
  return C;
}

struct Zone {
  int nx, ny, nz;
  Coeff C;
  std::vector<double> u, rsd, frct;
  size_t P(int i, int j, int k) const { return (((size_t)(k - 1) * ny + (j - 1)) * nx + (i - 1)) * 5; }
  double& U(int m, int i, int j, int k) { return u[P(i, j, k) + m - 1]; }
  double& R(int m, int i, int j, int k) { return rsd[P(i, j, k) + m - 1]; }
  double& F(int m, int i, int j, int k) { return frct[P(i, j, k) + m - 1]; }
};

struct Problem {
  int nzones;
  double dt, omega;
  double ce[5][13];
  int faces_npb;  // exch_qbc planes k = 2..nz-1 (1) or the reference's 1..nz-2 (0)
  std::vector<int> nbr;  // per zone: west, east, south, north (0-based)
  std::vector<Zone> zones;
};

// src/LU/exact.jl
void exact(const Problem& pb, int i, int j, int k, double out[5], int nx0, int ny0, int nz0) {
  double xi = (double)(i - 1) / (nx0 - 1);
  double eta = (double)(j - 1) / (ny0 - 1);
  double zeta = (double)(k - 1) / (nz0 - 1);
  for (int m = 0; m < 5; ++m) {
    const double* c = pb.ce[m];
    out[m] = c[0] + (c[1] + (c[4] + (c[7] + c[10] * xi) * xi) * xi) * xi +
             (c[2] + (c[5] + (c[8] + c[11] * eta) * eta) * eta) * eta +
             (c[3] + (c[6] + (c[9] + c[12] * zeta) * zeta) * zeta) * zeta;
  }
}

// src/LU/setbv.jl (all four process neighbours -1)
void setbv(const Problem& pb, Zone& z) {
  const int nx = z.nx, ny = z.ny, nz = z.nz;
  double e[5];
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      exact(pb, i, j, 1, e, nx, ny, nz);
      for (int m = 1; m <= 5; ++m) z.U(m, i, j, 1) = e[m - 1];
      exact(pb, i, j, nz, e, nx, ny, nz);
      for (int m = 1; m <= 5; ++m) z.U(m, i, j, nz) = e[m - 1];
    }
  for (int k = 1; k <= nz; ++k)
    for (int i = 1; i <= nx; ++i) {
      exact(pb, i, 1, k, e, nx, ny, nz);
      for (int m = 1; m <= 5; ++m) z.U(m, i, 1, k) = e[m - 1];
    }
  for (int k = 1; k <= nz; ++k)
    for (int i = 1; i <= nx; ++i) {
      exact(pb, i, ny, k, e, nx, ny, nz);
      for (int m = 1; m <= 5; ++m) z.U(m, i, ny, k) = e[m - 1];
    }
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j) {
      exact(pb, 1, j, k, e, nx, ny, nz);
      for (int m = 1; m <= 5; ++m) z.U(m, 1, j, k) = e[m - 1];
    }
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j) {
      exact(pb, nx, j, k, e, nx, ny, nz);
      for (int m = 1; m <= 5; ++m) z.U(m, nx, j, k) = e[m - 1];
    }
}

// src/LU/setiv.jl
void setiv(const Problem& pb, Zone& z) {
  const int nx = z.nx, ny = z.ny, nz = z.nz;
  double a1[5], a2[5], b1[5], b2[5], g1[5], g2[5];
  for (int k = 2; k <= nz - 1; ++k) {
    double zeta = (double)(k - 1) / (nz - 1);
    for (int j = 1; j <= ny; ++j) {
      if (j == 1 || j == ny) continue;
      double eta = (double)(j - 1) / (ny - 1);
      for (int i = 1; i <= nx; ++i) {
        if (i == 1 || i == nx) continue;
        double xi = (double)(i - 1) / (nx - 1);
        exact(pb, 1, j, k, a1, nx, ny, nz);
        exact(pb, nx, j, k, a2, nx, ny, nz);
        exact(pb, i, 1, k, b1, nx, ny, nz);
        exact(pb, i, ny, k, b2, nx, ny, nz);
        exact(pb, i, j, 1, g1, nx, ny, nz);
        exact(pb, i, j, nz, g2, nx, ny, nz);
        for (int m = 0; m < 5; ++m) {
          double pxi = (1.0e+00 - xi) * a1[m] + xi * a2[m];
          double peta = (1.0e+00 - eta) * b1[m] + eta * b2[m];
          double pzeta = (1.0e+00 - zeta) * g1[m] + zeta * g2[m];
          z.U(m + 1, i, j, k) = pxi + peta + pzeta - pxi * peta - peta * pzeta - pzeta * pxi + pxi * peta * pzeta;
        }
      }
    }
  }
}

// The flux/viscous/dissipation operator shared by rhs (g = u, out = rsd,
// which starts at -frct) and erhs (g = the exact polynomial, out = frct,
// which starts at 0).  The reference writes it twice; the two copies differ
// only in the order of the z second difference (rhs: g(k-1) - 2 g(k) +
// g(k+1); erhs: g(k+1) - 2 g(k) + g(k-1)) and in how the viscous update of
// m = 2..5 associates (rhs `rsd += A + B`, erhs `frct = frct + A + B`), which
// `erhs_order` selects.
struct Op {
  int nx, ny, nz;
  const double* g;
  double* out;
  size_t P(int i, int j, int k) const { return (((size_t)(k - 1) * ny + (j - 1)) * nx + (i - 1)) * 5; }
  double G(int m, int i, int j, int k) const { return g[P(i, j, k) + m - 1]; }
  double& O(int m, int i, int j, int k) { return out[P(i, j, k) + m - 1]; }
};

// rhs: rsd[m] += A + B (rsd + (A + B)); erhs: frct[m] = frct[m] + A + B
// ((frct + A) + B)
inline double viscous_update(double o, double a, double b, bool erhs_order) {
  return erhs_order ? (o + a) + b : o + (a + b);
}

void flux_operator(Op& o, const Coeff& C, bool erhs_order, std::vector<double>& flux) {
  const int nx = o.nx, ny = o.ny, nz = o.nz;
  const int ist = 2, iend = nx - 1, jst = 2, jend = ny - 1;
  flux.assign((size_t)(nx + 2) * (ny + 2) * (nz + 2) * 5, 0.0);
  auto FL = [&](int m, int i, int j, int k) -> double& {
    return flux[((((size_t)k * (ny + 2) + j) * (nx + 2)) + i) * 5 + m - 1];
  };
  const double tx1 = C.tx1, tx2 = C.tx2, tx3 = C.tx3, ty1 = C.ty1, ty2 = C.ty2, ty3 = C.ty3, tz1 = C.tz1,
               tz2 = C.tz2, tz3 = C.tz3;
  // ---- xi direction
  {
    const int L1 = 1, L2 = nx, ist1 = 4, iend1 = nx - 3;
    for (int k = 2; k <= nz - 1; ++k)
      for (int j = jst; j <= jend; ++j) {
        for (int i = L1; i <= L2; ++i) {
          double g1 = o.G(1, i, j, k), g2 = o.G(2, i, j, k), g3 = o.G(3, i, j, k), g4 = o.G(4, i, j, k),
                 g5 = o.G(5, i, j, k);
          FL(1, i, j, k) = g2;
          double u21 = g2 / g1;
          double q = 0.50e+00 * (g2 * g2 + g3 * g3 + g4 * g4) / g1;
          FL(2, i, j, k) = g2 * u21 + c2 * (g5 - q);
          FL(3, i, j, k) = g3 * u21;
          FL(4, i, j, k) = g4 * u21;
          FL(5, i, j, k) = (c1 * g5 - c2 * q) * u21;
        }
        for (int i = ist; i <= iend; ++i)
          for (int m = 1; m <= 5; ++m) o.O(m, i, j, k) = o.O(m, i, j, k) - tx2 * (FL(m, i + 1, j, k) - FL(m, i - 1, j, k));
        for (int i = ist; i <= L2; ++i) {
          double tmp = 1.0e+00 / o.G(1, i, j, k);
          double u21i = tmp * o.G(2, i, j, k), u31i = tmp * o.G(3, i, j, k), u41i = tmp * o.G(4, i, j, k),
                 u51i = tmp * o.G(5, i, j, k);
          tmp = 1.0e+00 / o.G(1, i - 1, j, k);
          double u21im1 = tmp * o.G(2, i - 1, j, k), u31im1 = tmp * o.G(3, i - 1, j, k),
                 u41im1 = tmp * o.G(4, i - 1, j, k), u51im1 = tmp * o.G(5, i - 1, j, k);
          FL(2, i, j, k) = (4.0e+00 / 3.0e+00) * tx3 * (u21i - u21im1);
          FL(3, i, j, k) = tx3 * (u31i - u31im1);
          FL(4, i, j, k) = tx3 * (u41i - u41im1);
          FL(5, i, j, k) = 0.50e+00 * (1.0e+00 - c1 * c5) * tx3 *
                               ((u21i * u21i + u31i * u31i + u41i * u41i) -
                                (u21im1 * u21im1 + u31im1 * u31im1 + u41im1 * u41im1)) +
                           (1.0e+00 / 6.0e+00) * tx3 * (u21i * u21i - u21im1 * u21im1) +
                           c1 * c5 * tx3 * (u51i - u51im1);
        }
        for (int i = ist; i <= iend; ++i) {
          o.O(1, i, j, k) = o.O(1, i, j, k) +
                            dx1 * tx1 * (o.G(1, i - 1, j, k) - 2.0e+00 * o.G(1, i, j, k) + o.G(1, i + 1, j, k));
          const double dxm[5] = {dx1, dx2, dx3, dx4, dx5};
          for (int m = 2; m <= 5; ++m)
            o.O(m, i, j, k) = viscous_update(o.O(m, i, j, k), tx3 * c3 * c4 * (FL(m, i + 1, j, k) - FL(m, i, j, k)),
                                             dxm[m - 1] * tx1 * (o.G(m, i - 1, j, k) - 2.0e+00 * o.G(m, i, j, k) + o.G(m, i + 1, j, k)), erhs_order);
        }
        for (int m = 1; m <= 5; ++m) {
          o.O(m, 2, j, k) = o.O(m, 2, j, k) -
                            dssp * (+5.0e+00 * o.G(m, 2, j, k) - 4.0e+00 * o.G(m, 3, j, k) + o.G(m, 4, j, k));
          o.O(m, 3, j, k) = o.O(m, 3, j, k) - dssp * (-4.0e+00 * o.G(m, 2, j, k) + 6.0e+00 * o.G(m, 3, j, k) -
                                                      4.0e+00 * o.G(m, 4, j, k) + o.G(m, 5, j, k));
        }
        for (int i = ist1; i <= iend1; ++i)
          for (int m = 1; m <= 5; ++m)
            o.O(m, i, j, k) = o.O(m, i, j, k) -
                              dssp * (o.G(m, i - 2, j, k) - 4.0e+00 * o.G(m, i - 1, j, k) +
                                      6.0e+00 * o.G(m, i, j, k) - 4.0e+00 * o.G(m, i + 1, j, k) + o.G(m, i + 2, j, k));
        for (int m = 1; m <= 5; ++m) {
          o.O(m, nx - 2, j, k) = o.O(m, nx - 2, j, k) -
                                 dssp * (o.G(m, nx - 4, j, k) - 4.0e+00 * o.G(m, nx - 3, j, k) +
                                         6.0e+00 * o.G(m, nx - 2, j, k) - 4.0e+00 * o.G(m, nx - 1, j, k));
          o.O(m, nx - 1, j, k) = o.O(m, nx - 1, j, k) - dssp * (o.G(m, nx - 3, j, k) - 4.0e+00 * o.G(m, nx - 2, j, k) +
                                                                5.0e+00 * o.G(m, nx - 1, j, k));
        }
      }
  }
  // ---- eta direction
  {
    const int L1 = 1, L2 = ny, jst1 = 4, jend1 = ny - 3;
    for (int k = 2; k <= nz - 1; ++k) {
      for (int j = L1; j <= L2; ++j)
        for (int i = ist; i <= iend; ++i) {
          double g1 = o.G(1, i, j, k), g2 = o.G(2, i, j, k), g3 = o.G(3, i, j, k), g4 = o.G(4, i, j, k),
                 g5 = o.G(5, i, j, k);
          FL(1, i, j, k) = g3;
          double u31 = g3 / g1;
          double q = 0.50e+00 * (g2 * g2 + g3 * g3 + g4 * g4) / g1;
          FL(2, i, j, k) = g2 * u31;
          FL(3, i, j, k) = g3 * u31 + c2 * (g5 - q);
          FL(4, i, j, k) = g4 * u31;
          FL(5, i, j, k) = (c1 * g5 - c2 * q) * u31;
        }
      for (int j = jst; j <= jend; ++j)
        for (int i = ist; i <= iend; ++i)
          for (int m = 1; m <= 5; ++m) o.O(m, i, j, k) = o.O(m, i, j, k) - ty2 * (FL(m, i, j + 1, k) - FL(m, i, j - 1, k));
      for (int j = jst; j <= L2; ++j)
        for (int i = ist; i <= iend; ++i) {
          double tmp = 1.0e+00 / o.G(1, i, j, k);
          double u21j = tmp * o.G(2, i, j, k), u31j = tmp * o.G(3, i, j, k), u41j = tmp * o.G(4, i, j, k),
                 u51j = tmp * o.G(5, i, j, k);
          tmp = 1.0e+00 / o.G(1, i, j - 1, k);
          double u21jm1 = tmp * o.G(2, i, j - 1, k), u31jm1 = tmp * o.G(3, i, j - 1, k),
                 u41jm1 = tmp * o.G(4, i, j - 1, k), u51jm1 = tmp * o.G(5, i, j - 1, k);
          FL(2, i, j, k) = ty3 * (u21j - u21jm1);
          FL(3, i, j, k) = (4.0e+00 / 3.0e+00) * ty3 * (u31j - u31jm1);
          FL(4, i, j, k) = ty3 * (u41j - u41jm1);
          FL(5, i, j, k) = 0.50e+00 * (1.0e+00 - c1 * c5) * ty3 *
                               ((u21j * u21j + u31j * u31j + u41j * u41j) -
                                (u21jm1 * u21jm1 + u31jm1 * u31jm1 + u41jm1 * u41jm1)) +
                           (1.0e+00 / 6.0e+00) * ty3 * (u31j * u31j - u31jm1 * u31jm1) +
                           c1 * c5 * ty3 * (u51j - u51jm1);
        }
      for (int j = jst; j <= jend; ++j)
        for (int i = ist; i <= iend; ++i) {
          o.O(1, i, j, k) = o.O(1, i, j, k) +
                            dy1 * ty1 * (o.G(1, i, j - 1, k) - 2.0e+00 * o.G(1, i, j, k) + o.G(1, i, j + 1, k));
          const double dym[5] = {dy1, dy2, dy3, dy4, dy5};
          for (int m = 2; m <= 5; ++m)
            o.O(m, i, j, k) = viscous_update(o.O(m, i, j, k), ty3 * c3 * c4 * (FL(m, i, j + 1, k) - FL(m, i, j, k)),
                                             dym[m - 1] * ty1 * (o.G(m, i, j - 1, k) - 2.0e+00 * o.G(m, i, j, k) + o.G(m, i, j + 1, k)), erhs_order);
        }
      for (int i = ist; i <= iend; ++i)
        for (int m = 1; m <= 5; ++m) {
          o.O(m, i, 2, k) = o.O(m, i, 2, k) -
                            dssp * (+5.0e+00 * o.G(m, i, 2, k) - 4.0e+00 * o.G(m, i, 3, k) + o.G(m, i, 4, k));
          o.O(m, i, 3, k) = o.O(m, i, 3, k) - dssp * (-4.0e+00 * o.G(m, i, 2, k) + 6.0e+00 * o.G(m, i, 3, k) -
                                                      4.0e+00 * o.G(m, i, 4, k) + o.G(m, i, 5, k));
        }
      for (int j = jst1; j <= jend1; ++j)
        for (int i = ist; i <= iend; ++i)
          for (int m = 1; m <= 5; ++m)
            o.O(m, i, j, k) = o.O(m, i, j, k) -
                              dssp * (o.G(m, i, j - 2, k) - 4.0e+00 * o.G(m, i, j - 1, k) +
                                      6.0e+00 * o.G(m, i, j, k) - 4.0e+00 * o.G(m, i, j + 1, k) + o.G(m, i, j + 2, k));
      for (int i = ist; i <= iend; ++i)
        for (int m = 1; m <= 5; ++m) {
          o.O(m, i, ny - 2, k) = o.O(m, i, ny - 2, k) -
                                 dssp * (o.G(m, i, ny - 4, k) - 4.0e+00 * o.G(m, i, ny - 3, k) +
                                         6.0e+00 * o.G(m, i, ny - 2, k) - 4.0e+00 * o.G(m, i, ny - 1, k));
          o.O(m, i, ny - 1, k) = o.O(m, i, ny - 1, k) - dssp * (o.G(m, i, ny - 3, k) - 4.0e+00 * o.G(m, i, ny - 2, k) +
                                                                5.0e+00 * o.G(m, i, ny - 1, k));
        }
    }
  }
  // ---- zeta direction
  for (int k = 1; k <= nz; ++k)
    for (int j = jst; j <= jend; ++j)
      for (int i = ist; i <= iend; ++i) {
        double g1 = o.G(1, i, j, k), g2 = o.G(2, i, j, k), g3 = o.G(3, i, j, k), g4 = o.G(4, i, j, k),
               g5 = o.G(5, i, j, k);
        FL(1, i, j, k) = g4;
        double u41 = g4 / g1;
        double q = 0.50e+00 * (g2 * g2 + g3 * g3 + g4 * g4) / g1;
        FL(2, i, j, k) = g2 * u41;
        FL(3, i, j, k) = g3 * u41;
        FL(4, i, j, k) = g4 * u41 + c2 * (g5 - q);
        FL(5, i, j, k) = (c1 * g5 - c2 * q) * u41;
      }
  for (int k = 2; k <= nz - 1; ++k)
    for (int j = jst; j <= jend; ++j)
      for (int i = ist; i <= iend; ++i)
        for (int m = 1; m <= 5; ++m) o.O(m, i, j, k) = o.O(m, i, j, k) - tz2 * (FL(m, i, j, k + 1) - FL(m, i, j, k - 1));
  for (int k = 2; k <= nz; ++k)
    for (int j = jst; j <= jend; ++j)
      for (int i = ist; i <= iend; ++i) {
        double tmp = 1.0e+00 / o.G(1, i, j, k);
        double u21k = tmp * o.G(2, i, j, k), u31k = tmp * o.G(3, i, j, k), u41k = tmp * o.G(4, i, j, k),
               u51k = tmp * o.G(5, i, j, k);
        tmp = 1.0e+00 / o.G(1, i, j, k - 1);
        double u21km1 = tmp * o.G(2, i, j, k - 1), u31km1 = tmp * o.G(3, i, j, k - 1),
               u41km1 = tmp * o.G(4, i, j, k - 1), u51km1 = tmp * o.G(5, i, j, k - 1);
        FL(2, i, j, k) = tz3 * (u21k - u21km1);
        FL(3, i, j, k) = tz3 * (u31k - u31km1);
        FL(4, i, j, k) = (4.0e+00 / 3.0e+00) * tz3 * (u41k - u41km1);
        FL(5, i, j, k) = 0.50e+00 * (1.0e+00 - c1 * c5) * tz3 *
                             ((u21k * u21k + u31k * u31k + u41k * u41k) -
                              (u21km1 * u21km1 + u31km1 * u31km1 + u41km1 * u41km1)) +
                         (1.0e+00 / 6.0e+00) * tz3 * (u41k * u41k - u41km1 * u41km1) +
                         c1 * c5 * tz3 * (u51k - u51km1);
      }
  for (int k = 2; k <= nz - 1; ++k)
    for (int j = jst; j <= jend; ++j)
      for (int i = ist; i <= iend; ++i) {
        auto sd = [&](int m) {
          return erhs_order ? (o.G(m, i, j, k + 1) - 2.0e+00 * o.G(m, i, j, k) + o.G(m, i, j, k - 1))
                            : (o.G(m, i, j, k - 1) - 2.0e+00 * o.G(m, i, j, k) + o.G(m, i, j, k + 1));
        };
        o.O(1, i, j, k) = o.O(1, i, j, k) + dz1 * tz1 * sd(1);
        const double dzm[5] = {dz1, dz2, dz3, dz4, dz5};
        for (int m = 2; m <= 5; ++m)
          o.O(m, i, j, k) = viscous_update(o.O(m, i, j, k), tz3 * c3 * c4 * (FL(m, i, j, k + 1) - FL(m, i, j, k)),
                                           dzm[m - 1] * tz1 * sd(m), erhs_order);
      }
  for (int j = jst; j <= jend; ++j)
    for (int i = ist; i <= iend; ++i)
      for (int m = 1; m <= 5; ++m) {
        o.O(m, i, j, 2) = o.O(m, i, j, 2) -
                          dssp * (+5.0e+00 * o.G(m, i, j, 2) - 4.0e+00 * o.G(m, i, j, 3) + o.G(m, i, j, 4));
        o.O(m, i, j, 3) = o.O(m, i, j, 3) - dssp * (-4.0e+00 * o.G(m, i, j, 2) + 6.0e+00 * o.G(m, i, j, 3) -
                                                    4.0e+00 * o.G(m, i, j, 4) + o.G(m, i, j, 5));
      }
  for (int k = 4; k <= nz - 3; ++k)
    for (int j = jst; j <= jend; ++j)
      for (int i = ist; i <= iend; ++i)
        for (int m = 1; m <= 5; ++m)
          o.O(m, i, j, k) = o.O(m, i, j, k) -
                            dssp * (o.G(m, i, j, k - 2) - 4.0e+00 * o.G(m, i, j, k - 1) + 6.0e+00 * o.G(m, i, j, k) -
                                    4.0e+00 * o.G(m, i, j, k + 1) + o.G(m, i, j, k + 2));
  for (int j = jst; j <= jend; ++j)
    for (int i = ist; i <= iend; ++i)
      for (int m = 1; m <= 5; ++m) {
        o.O(m, i, j, nz - 2) = o.O(m, i, j, nz - 2) -
                               dssp * (o.G(m, i, j, nz - 4) - 4.0e+00 * o.G(m, i, j, nz - 3) +
                                       6.0e+00 * o.G(m, i, j, nz - 2) - 4.0e+00 * o.G(m, i, j, nz - 1));
        o.O(m, i, j, nz - 1) = o.O(m, i, j, nz - 1) - dssp * (o.G(m, i, j, nz - 3) - 4.0e+00 * o.G(m, i, j, nz - 2) +
                                                              5.0e+00 * o.G(m, i, j, nz - 1));
      }
}

// src/LU/erhs.jl: frct from the exact polynomial (non-Horner form) held in rsd
void erhs(const Problem& pb, Zone& z) {
  const int nx = z.nx, ny = z.ny, nz = z.nz;
  std::fill(z.frct.begin(), z.frct.end(), 0.0);
  for (int k = 1; k <= nz; ++k) {
    double zeta = (double)(k - 1) / (nz - 1);
    for (int j = 1; j <= ny; ++j) {
      double eta = (double)(j - 1) / (ny - 1);
      for (int i = 1; i <= nx; ++i) {
        double xi = (double)(i - 1) / (nx - 1);
        for (int m = 0; m < 5; ++m) {
          const double* c = pb.ce[m];
          z.R(m + 1, i, j, k) = c[0] + c[1] * xi + c[2] * eta + c[3] * zeta + c[4] * xi * xi + c[5] * eta * eta +
                                c[6] * zeta * zeta + c[7] * xi * xi * xi + c[8] * eta * eta * eta +
                                c[9] * zeta * zeta * zeta + c[10] * xi * xi * xi * xi + c[11] * eta * eta * eta * eta +
                                c[12] * zeta * zeta * zeta * zeta;
        }
      }
    }
  }
  Op o{nx, ny, nz, z.rsd.data(), z.frct.data()};
  std::vector<double> flux;
  flux_operator(o, z.C, true, flux);
}

// src/LU/rhs.jl
void rhs(Zone& z) {
  for (size_t e = 0; e < z.rsd.size(); ++e) z.rsd[e] = -z.frct[e];
  Op o{z.nx, z.ny, z.nz, z.u.data(), z.rsd.data()};
  static thread_local std::vector<double> flux;
  flux_operator(o, z.C, false, flux);
}

typedef double Blk[5][5];  // Blk[m-1][n-1] = the reference's blk[m, n, i]

// src/LU/jacld.jl for one point: d (diagonal), a (z, from k-1), b (y, from
// j-1), c (x, from i-1)
void jacld_point(Zone& z, const Coeff& C, double dt, int i, int j, int k, Blk d, Blk a, Blk b, Blk c) {
  const double r43 = (4.0e+00 / 3.0e+00), c1345 = c1 * c3 * c4 * c5, c34 = c3 * c4;
  const double tx1 = C.tx1, tx2 = C.tx2, ty1 = C.ty1, ty2 = C.ty2, tz1 = C.tz1, tz2 = C.tz2;
  double u1 = z.U(1, i, j, k), u2 = z.U(2, i, j, k), u3 = z.U(3, i, j, k), u4 = z.U(4, i, j, k), u5 = z.U(5, i, j, k);
  double tmp1 = 1.0e+00 / u1, tmp2 = tmp1 * tmp1, tmp3 = tmp1 * tmp2;
  d[0][0] = 1.0e+00 + dt * 2.0e+00 * (tx1 * dx1 + ty1 * dy1 + tz1 * dz1);
  d[0][1] = 0.0; d[0][2] = 0.0; d[0][3] = 0.0; d[0][4] = 0.0;
  d[1][0] = dt * 2.0e+00 * (tx1 * (-r43 * c34 * tmp2 * u2) + ty1 * (-c34 * tmp2 * u2) + tz1 * (-c34 * tmp2 * u2));
  d[1][1] = 1.0e+00 + dt * 2.0e+00 * (tx1 * r43 * c34 * tmp1 + ty1 * c34 * tmp1 + tz1 * c34 * tmp1) +
            dt * 2.0e+00 * (tx1 * dx2 + ty1 * dy2 + tz1 * dz2);
  d[1][2] = 0.0; d[1][3] = 0.0; d[1][4] = 0.0;
  d[2][0] = dt * 2.0e+00 * (tx1 * (-c34 * tmp2 * u3) + ty1 * (-r43 * c34 * tmp2 * u3) + tz1 * (-c34 * tmp2 * u3));
  d[2][1] = 0.0;
  d[2][2] = 1.0e+00 + dt * 2.0e+00 * (tx1 * c34 * tmp1 + ty1 * r43 * c34 * tmp1 + tz1 * c34 * tmp1) +
            dt * 2.0e+00 * (tx1 * dx3 + ty1 * dy3 + tz1 * dz3);
  d[2][3] = 0.0; d[2][4] = 0.0;
  d[3][0] = dt * 2.0e+00 * (tx1 * (-c34 * tmp2 * u4) + ty1 * (-c34 * tmp2 * u4) + tz1 * (-r43 * c34 * tmp2 * u4));
  d[3][1] = 0.0; d[3][2] = 0.0;
  d[3][3] = 1.0e+00 + dt * 2.0e+00 * (tx1 * c34 * tmp1 + ty1 * c34 * tmp1 + tz1 * r43 * c34 * tmp1) +
            dt * 2.0e+00 * (tx1 * dx4 + ty1 * dy4 + tz1 * dz4);
  d[3][4] = 0.0;
  d[4][0] = dt * 2.0e+00 *
            (tx1 * (-(r43 * c34 - c1345) * tmp3 * (u2 * u2) - (c34 - c1345) * tmp3 * (u3 * u3) -
                    (c34 - c1345) * tmp3 * (u4 * u4) - (c1345)*tmp2 * u5) +
             ty1 * (-(c34 - c1345) * tmp3 * (u2 * u2) - (r43 * c34 - c1345) * tmp3 * (u3 * u3) -
                    (c34 - c1345) * tmp3 * (u4 * u4) - (c1345)*tmp2 * u5) +
             tz1 * (-(c34 - c1345) * tmp3 * (u2 * u2) - (c34 - c1345) * tmp3 * (u3 * u3) -
                    (r43 * c34 - c1345) * tmp3 * (u4 * u4) - (c1345)*tmp2 * u5));
  d[4][1] = dt * 2.0e+00 *
            (tx1 * (r43 * c34 - c1345) * tmp2 * u2 + ty1 * (c34 - c1345) * tmp2 * u2 + tz1 * (c34 - c1345) * tmp2 * u2);
  d[4][2] = dt * 2.0e+00 *
            (tx1 * (c34 - c1345) * tmp2 * u3 + ty1 * (r43 * c34 - c1345) * tmp2 * u3 + tz1 * (c34 - c1345) * tmp2 * u3);
  d[4][3] = dt * 2.0e+00 *
            (tx1 * (c34 - c1345) * tmp2 * u4 + ty1 * (c34 - c1345) * tmp2 * u4 + tz1 * (r43 * c34 - c1345) * tmp2 * u4);
  d[4][4] = 1.0e+00 + dt * 2.0e+00 * (tx1 * c1345 * tmp1 + ty1 * c1345 * tmp1 + tz1 * c1345 * tmp1) +
            dt * 2.0e+00 * (tx1 * dx5 + ty1 * dy5 + tz1 * dz5);

  // a: zeta, from k-1
  u1 = z.U(1, i, j, k - 1); u2 = z.U(2, i, j, k - 1); u3 = z.U(3, i, j, k - 1); u4 = z.U(4, i, j, k - 1);
  u5 = z.U(5, i, j, k - 1);
  tmp1 = 1.0e+00 / u1; tmp2 = tmp1 * tmp1; tmp3 = tmp1 * tmp2;
  a[0][0] = -dt * tz1 * dz1;
  a[0][1] = 0.0;
  a[0][2] = 0.0;
  a[0][3] = -dt * tz2;
  a[0][4] = 0.0;
  a[1][0] = -dt * tz2 * (-(u2 * u4) * tmp2) - dt * tz1 * (-c34 * tmp2 * u2);
  a[1][1] = -dt * tz2 * (u4 * tmp1) - dt * tz1 * c34 * tmp1 - dt * tz1 * dz2;
  a[1][2] = 0.0;
  a[1][3] = -dt * tz2 * (u2 * tmp1);
  a[1][4] = 0.0;
  a[2][0] = -dt * tz2 * (-(u3 * u4) * tmp2) - dt * tz1 * (-c34 * tmp2 * u3);
  a[2][1] = 0.0;
  a[2][2] = -dt * tz2 * (u4 * tmp1) - dt * tz1 * (c34 * tmp1) - dt * tz1 * dz3;
  a[2][3] = -dt * tz2 * (u3 * tmp1);
  a[2][4] = 0.0;
  a[3][0] = -dt * tz2 * (-((u4 * tmp1) * (u4 * tmp1)) + 0.50e+00 * c2 * ((u2 * u2 + u3 * u3 + u4 * u4) * tmp2)) -
            dt * tz1 * (-r43 * c34 * tmp2 * u4);
  a[3][1] = -dt * tz2 * (-c2 * (u2 * tmp1));
  a[3][2] = -dt * tz2 * (-c2 * (u3 * tmp1));
  a[3][3] = -dt * tz2 * (2.0e+00 - c2) * (u4 * tmp1) - dt * tz1 * (r43 * c34 * tmp1) - dt * tz1 * dz4;
  a[3][4] = -dt * tz2 * c2;
  a[4][0] = -dt * tz2 * ((c2 * (u2 * u2 + u3 * u3 + u4 * u4) * tmp2 - c1 * (u5 * tmp1)) * (u4 * tmp1)) -
            dt * tz1 *
                (-(c34 - c1345) * tmp3 * (u2 * u2) - (c34 - c1345) * tmp3 * (u3 * u3) -
                 (r43 * c34 - c1345) * tmp3 * (u4 * u4) - c1345 * tmp2 * u5);
  a[4][1] = -dt * tz2 * (-c2 * (u2 * u4) * tmp2) - dt * tz1 * (c34 - c1345) * tmp2 * u2;
  a[4][2] = -dt * tz2 * (-c2 * (u3 * u4) * tmp2) - dt * tz1 * (c34 - c1345) * tmp2 * u3;
  a[4][3] = -dt * tz2 * (c1 * (u5 * tmp1) - 0.50e+00 * c2 * ((u2 * u2 + u3 * u3 + 3.0e+00 * u4 * u4) * tmp2)) -
            dt * tz1 * (r43 * c34 - c1345) * tmp2 * u4;
  a[4][4] = -dt * tz2 * (c1 * (u4 * tmp1)) - dt * tz1 * c1345 * tmp1 - dt * tz1 * dz5;

  // b: eta, from j-1
  u1 = z.U(1, i, j - 1, k); u2 = z.U(2, i, j - 1, k); u3 = z.U(3, i, j - 1, k); u4 = z.U(4, i, j - 1, k);
  u5 = z.U(5, i, j - 1, k);
  tmp1 = 1.0e+00 / u1; tmp2 = tmp1 * tmp1; tmp3 = tmp1 * tmp2;
  b[0][0] = -dt * ty1 * dy1;
  b[0][1] = 0.0;
  b[0][2] = -dt * ty2;
  b[0][3] = 0.0;
  b[0][4] = 0.0;
  b[1][0] = -dt * ty2 * (-(u2 * u3) * tmp2) - dt * ty1 * (-c34 * tmp2 * u2);
  b[1][1] = -dt * ty2 * (u3 * tmp1) - dt * ty1 * (c34 * tmp1) - dt * ty1 * dy2;
  b[1][2] = -dt * ty2 * (u2 * tmp1);
  b[1][3] = 0.0;
  b[1][4] = 0.0;
  b[2][0] = -dt * ty2 * (-((u3 * tmp1) * (u3 * tmp1)) + 0.50e+00 * c2 * ((u2 * u2 + u3 * u3 + u4 * u4) * tmp2)) -
            dt * ty1 * (-r43 * c34 * tmp2 * u3);
  b[2][1] = -dt * ty2 * (-c2 * (u2 * tmp1));
  b[2][2] = -dt * ty2 * ((2.0e+00 - c2) * (u3 * tmp1)) - dt * ty1 * (r43 * c34 * tmp1) - dt * ty1 * dy3;
  b[2][3] = -dt * ty2 * (-c2 * (u4 * tmp1));
  b[2][4] = -dt * ty2 * c2;
  b[3][0] = -dt * ty2 * (-(u3 * u4) * tmp2) - dt * ty1 * (-c34 * tmp2 * u4);
  b[3][1] = 0.0;
  b[3][2] = -dt * ty2 * (u4 * tmp1);
  b[3][3] = -dt * ty2 * (u3 * tmp1) - dt * ty1 * (c34 * tmp1) - dt * ty1 * dy4;
  b[3][4] = 0.0;
  b[4][0] = -dt * ty2 * ((c2 * (u2 * u2 + u3 * u3 + u4 * u4) * tmp2 - c1 * (u5 * tmp1)) * (u3 * tmp1)) -
            dt * ty1 *
                (-(c34 - c1345) * tmp3 * (u2 * u2) - (r43 * c34 - c1345) * tmp3 * (u3 * u3) -
                 (c34 - c1345) * tmp3 * (u4 * u4) - c1345 * tmp2 * u5);
  b[4][1] = -dt * ty2 * (-c2 * (u2 * u3) * tmp2) - dt * ty1 * (c34 - c1345) * tmp2 * u2;
  b[4][2] = -dt * ty2 * (c1 * (u5 * tmp1) - 0.50e+00 * c2 * ((u2 * u2 + 3.0e+00 * u3 * u3 + u4 * u4) * tmp2)) -
            dt * ty1 * (r43 * c34 - c1345) * tmp2 * u3;
  b[4][3] = -dt * ty2 * (-c2 * (u3 * u4) * tmp2) - dt * ty1 * (c34 - c1345) * tmp2 * u4;
  b[4][4] = -dt * ty2 * (c1 * (u3 * tmp1)) - dt * ty1 * c1345 * tmp1 - dt * ty1 * dy5;

  // c: xi, from i-1
  u1 = z.U(1, i - 1, j, k); u2 = z.U(2, i - 1, j, k); u3 = z.U(3, i - 1, j, k); u4 = z.U(4, i - 1, j, k);
  u5 = z.U(5, i - 1, j, k);
  tmp1 = 1.0e+00 / u1; tmp2 = tmp1 * tmp1; tmp3 = tmp1 * tmp2;
  c[0][0] = -dt * tx1 * dx1;
  c[0][1] = -dt * tx2;
  c[0][2] = 0.0;
  c[0][3] = 0.0;
  c[0][4] = 0.0;
  c[1][0] = -dt * tx2 * (-((u2 * tmp1) * (u2 * tmp1)) + c2 * 0.50e+00 * (u2 * u2 + u3 * u3 + u4 * u4) * tmp2) -
            dt * tx1 * (-r43 * c34 * tmp2 * u2);
  c[1][1] = -dt * tx2 * ((2.0e+00 - c2) * (u2 * tmp1)) - dt * tx1 * (r43 * c34 * tmp1) - dt * tx1 * dx2;
  c[1][2] = -dt * tx2 * (-c2 * (u3 * tmp1));
  c[1][3] = -dt * tx2 * (-c2 * (u4 * tmp1));
  c[1][4] = -dt * tx2 * c2;
  c[2][0] = -dt * tx2 * (-(u2 * u3) * tmp2) - dt * tx1 * (-c34 * tmp2 * u3);
  c[2][1] = -dt * tx2 * (u3 * tmp1);
  c[2][2] = -dt * tx2 * (u2 * tmp1) - dt * tx1 * (c34 * tmp1) - dt * tx1 * dx3;
  c[2][3] = 0.0;
  c[2][4] = 0.0;
  c[3][0] = -dt * tx2 * (-(u2 * u4) * tmp2) - dt * tx1 * (-c34 * tmp2 * u4);
  c[3][1] = -dt * tx2 * (u4 * tmp1);
  c[3][2] = 0.0;
  c[3][3] = -dt * tx2 * (u2 * tmp1) - dt * tx1 * (c34 * tmp1) - dt * tx1 * dx4;
  c[3][4] = 0.0;
  c[4][0] = -dt * tx2 * ((c2 * (u2 * u2 + u3 * u3 + u4 * u4) * tmp2 - c1 * (u5 * tmp1)) * (u2 * tmp1)) -
            dt * tx1 *
                (-(r43 * c34 - c1345) * tmp3 * (u2 * u2) - (c34 - c1345) * tmp3 * (u3 * u3) -
                 (c34 - c1345) * tmp3 * (u4 * u4) - c1345 * tmp2 * u5);
  c[4][1] = -dt * tx2 * (c1 * (u5 * tmp1) - 0.50e+00 * c2 * ((3.0e+00 * u2 * u2 + u3 * u3 + u4 * u4) * tmp2)) -
            dt * tx1 * (r43 * c34 - c1345) * tmp2 * u2;
  c[4][2] = -dt * tx2 * (-c2 * (u3 * u2) * tmp2) - dt * tx1 * (c34 - c1345) * tmp2 * u3;
  c[4][3] = -dt * tx2 * (-c2 * (u4 * u2) * tmp2) - dt * tx1 * (c34 - c1345) * tmp2 * u4;
  c[4][4] = -dt * tx2 * (c1 * (u2 * tmp1)) - dt * tx1 * c1345 * tmp1 - dt * tx1 * dx5;
}

// src/LU/jacu.jl for one point: d (diagonal), a (x, from i+1), b (y, from
// j+1), c (z, from k+1)
void jacu_point(Zone& z, const Coeff& C, double dt, int i, int j, int k, Blk d, Blk a, Blk b, Blk c) {
  const double r43 = (4.0e+00 / 3.0e+00), c1345 = c1 * c3 * c4 * c5, c34 = c3 * c4;
  const double tx1 = C.tx1, tx2 = C.tx2, ty1 = C.ty1, ty2 = C.ty2, tz1 = C.tz1, tz2 = C.tz2;
  // d is jacld's diagonal block, statement for statement
  Blk a0, b0, c0;
  jacld_point(z, C, dt, i, j, k, d, a0, b0, c0);

  // a: xi, from i+1
  double u1 = z.U(1, i + 1, j, k), u2 = z.U(2, i + 1, j, k), u3 = z.U(3, i + 1, j, k), u4 = z.U(4, i + 1, j, k),
         u5 = z.U(5, i + 1, j, k);
  double tmp1 = 1.0e+00 / u1, tmp2 = tmp1 * tmp1, tmp3 = tmp1 * tmp2;
  a[0][0] = -dt * tx1 * dx1;
  a[0][1] = dt * tx2;
  a[0][2] = 0.0;
  a[0][3] = 0.0;
  a[0][4] = 0.0;
  a[1][0] = dt * tx2 * (-((u2 * tmp1) * (u2 * tmp1)) + c2 * 0.50e+00 * (u2 * u2 + u3 * u3 + u4 * u4) * tmp2) -
            dt * tx1 * (-r43 * c34 * tmp2 * u2);
  a[1][1] = dt * tx2 * ((2.0e+00 - c2) * (u2 * tmp1)) - dt * tx1 * (r43 * c34 * tmp1) - dt * tx1 * dx2;
  a[1][2] = dt * tx2 * (-c2 * (u3 * tmp1));
  a[1][3] = dt * tx2 * (-c2 * (u4 * tmp1));
  a[1][4] = dt * tx2 * c2;
  a[2][0] = dt * tx2 * (-(u2 * u3) * tmp2) - dt * tx1 * (-c34 * tmp2 * u3);
  a[2][1] = dt * tx2 * (u3 * tmp1);
  a[2][2] = dt * tx2 * (u2 * tmp1) - dt * tx1 * (c34 * tmp1) - dt * tx1 * dx3;
  a[2][3] = 0.0;
  a[2][4] = 0.0;
  a[3][0] = dt * tx2 * (-(u2 * u4) * tmp2) - dt * tx1 * (-c34 * tmp2 * u4);
  a[3][1] = dt * tx2 * (u4 * tmp1);
  a[3][2] = 0.0;
  a[3][3] = dt * tx2 * (u2 * tmp1) - dt * tx1 * (c34 * tmp1) - dt * tx1 * dx4;
  a[3][4] = 0.0;
  a[4][0] = dt * tx2 * ((c2 * (u2 * u2 + u3 * u3 + u4 * u4) * tmp2 - c1 * (u5 * tmp1)) * (u2 * tmp1)) -
            dt * tx1 *
                (-(r43 * c34 - c1345) * tmp3 * (u2 * u2) - (c34 - c1345) * tmp3 * (u3 * u3) -
                 (c34 - c1345) * tmp3 * (u4 * u4) - c1345 * tmp2 * u5);
  a[4][1] = dt * tx2 * (c1 * (u5 * tmp1) - 0.50e+00 * c2 * ((3.0e+00 * u2 * u2 + u3 * u3 + u4 * u4) * tmp2)) -
            dt * tx1 * (r43 * c34 - c1345) * tmp2 * u2;
  a[4][2] = dt * tx2 * (-c2 * (u3 * u2) * tmp2) - dt * tx1 * (c34 - c1345) * tmp2 * u3;
  a[4][3] = dt * tx2 * (-c2 * (u4 * u2) * tmp2) - dt * tx1 * (c34 - c1345) * tmp2 * u4;
  a[4][4] = dt * tx2 * (c1 * (u2 * tmp1)) - dt * tx1 * c1345 * tmp1 - dt * tx1 * dx5;

  // b: eta, from j+1
  u1 = z.U(1, i, j + 1, k); u2 = z.U(2, i, j + 1, k); u3 = z.U(3, i, j + 1, k); u4 = z.U(4, i, j + 1, k);
  u5 = z.U(5, i, j + 1, k);
  tmp1 = 1.0e+00 / u1; tmp2 = tmp1 * tmp1; tmp3 = tmp1 * tmp2;
  b[0][0] = -dt * ty1 * dy1;
  b[0][1] = 0.0;
  b[0][2] = dt * ty2;
  b[0][3] = 0.0;
  b[0][4] = 0.0;
  b[1][0] = dt * ty2 * (-(u2 * u3) * tmp2) - dt * ty1 * (-c34 * tmp2 * u2);
  b[1][1] = dt * ty2 * (u3 * tmp1) - dt * ty1 * (c34 * tmp1) - dt * ty1 * dy2;
  b[1][2] = dt * ty2 * (u2 * tmp1);
  b[1][3] = 0.0;
  b[1][4] = 0.0;
  b[2][0] = dt * ty2 * (-((u3 * tmp1) * (u3 * tmp1)) + 0.50e+00 * c2 * ((u2 * u2 + u3 * u3 + u4 * u4) * tmp2)) -
            dt * ty1 * (-r43 * c34 * tmp2 * u3);
  b[2][1] = dt * ty2 * (-c2 * (u2 * tmp1));
  b[2][2] = dt * ty2 * ((2.0e+00 - c2) * (u3 * tmp1)) - dt * ty1 * (r43 * c34 * tmp1) - dt * ty1 * dy3;
  b[2][3] = dt * ty2 * (-c2 * (u4 * tmp1));
  b[2][4] = dt * ty2 * c2;
  b[3][0] = dt * ty2 * (-(u3 * u4) * tmp2) - dt * ty1 * (-c34 * tmp2 * u4);
  b[3][1] = 0.0;
  b[3][2] = dt * ty2 * (u4 * tmp1);
  b[3][3] = dt * ty2 * (u3 * tmp1) - dt * ty1 * (c34 * tmp1) - dt * ty1 * dy4;
  b[3][4] = 0.0;
  b[4][0] = dt * ty2 * ((c2 * (u2 * u2 + u3 * u3 + u4 * u4) * tmp2 - c1 * (u5 * tmp1)) * (u3 * tmp1)) -
            dt * ty1 *
                (-(c34 - c1345) * tmp3 * (u2 * u2) - (r43 * c34 - c1345) * tmp3 * (u3 * u3) -
                 (c34 - c1345) * tmp3 * (u4 * u4) - c1345 * tmp2 * u5);
  b[4][1] = dt * ty2 * (-c2 * (u2 * u3) * tmp2) - dt * ty1 * (c34 - c1345) * tmp2 * u2;
  b[4][2] = dt * ty2 * (c1 * (u5 * tmp1) - 0.50e+00 * c2 * ((u2 * u2 + 3.0e+00 * u3 * u3 + u4 * u4) * tmp2)) -
            dt * ty1 * (r43 * c34 - c1345) * tmp2 * u3;
  b[4][3] = dt * ty2 * (-c2 * (u3 * u4) * tmp2) - dt * ty1 * (c34 - c1345) * tmp2 * u4;
  b[4][4] = dt * ty2 * (c1 * (u3 * tmp1)) - dt * ty1 * c1345 * tmp1 - dt * ty1 * dy5;

  // c: zeta, from k+1
  u1 = z.U(1, i, j, k + 1); u2 = z.U(2, i, j, k + 1); u3 = z.U(3, i, j, k + 1); u4 = z.U(4, i, j, k + 1);
  u5 = z.U(5, i, j, k + 1);
  tmp1 = 1.0e+00 / u1; tmp2 = tmp1 * tmp1; tmp3 = tmp1 * tmp2;
  c[0][0] = -dt * tz1 * dz1;
  c[0][1] = 0.0;
  c[0][2] = 0.0;
  c[0][3] = dt * tz2;
  c[0][4] = 0.0;
  c[1][0] = dt * tz2 * (-(u2 * u4) * tmp2) - dt * tz1 * (-c34 * tmp2 * u2);
  c[1][1] = dt * tz2 * (u4 * tmp1) - dt * tz1 * c34 * tmp1 - dt * tz1 * dz2;
  c[1][2] = 0.0;
  c[1][3] = dt * tz2 * (u2 * tmp1);
  c[1][4] = 0.0;
  c[2][0] = dt * tz2 * (-(u3 * u4) * tmp2) - dt * tz1 * (-c34 * tmp2 * u3);
  c[2][1] = 0.0;
  c[2][2] = dt * tz2 * (u4 * tmp1) - dt * tz1 * (c34 * tmp1) - dt * tz1 * dz3;
  c[2][3] = dt * tz2 * (u3 * tmp1);
  c[2][4] = 0.0;
  c[3][0] = dt * tz2 * (-((u4 * tmp1) * (u4 * tmp1)) + 0.50e+00 * c2 * ((u2 * u2 + u3 * u3 + u4 * u4) * tmp2)) -
            dt * tz1 * (-r43 * c34 * tmp2 * u4);
  c[3][1] = dt * tz2 * (-c2 * (u2 * tmp1));
  c[3][2] = dt * tz2 * (-c2 * (u3 * tmp1));
  c[3][3] = dt * tz2 * (2.0e+00 - c2) * (u4 * tmp1) - dt * tz1 * (r43 * c34 * tmp1) - dt * tz1 * dz4;
  c[3][4] = dt * tz2 * c2;
  c[4][0] = dt * tz2 * ((c2 * (u2 * u2 + u3 * u3 + u4 * u4) * tmp2 - c1 * (u5 * tmp1)) * (u4 * tmp1)) -
            dt * tz1 *
                (-(c34 - c1345) * tmp3 * (u2 * u2) - (c34 - c1345) * tmp3 * (u3 * u3) -
                 (r43 * c34 - c1345) * tmp3 * (u4 * u4) - c1345 * tmp2 * u5);
  c[4][1] = dt * tz2 * (-c2 * (u2 * u4) * tmp2) - dt * tz1 * (c34 - c1345) * tmp2 * u2;
  c[4][2] = dt * tz2 * (-c2 * (u3 * u4) * tmp2) - dt * tz1 * (c34 - c1345) * tmp2 * u3;
  c[4][3] = dt * tz2 * (c1 * (u5 * tmp1) - 0.50e+00 * c2 * ((u2 * u2 + u3 * u3 + 3.0e+00 * u4 * u4) * tmp2)) -
            dt * tz1 * (r43 * c34 - c1345) * tmp2 * u4;
  c[4][4] = dt * tz2 * (c1 * (u4 * tmp1)) - dt * tz1 * c1345 * tmp1 - dt * tz1 * dz5;
}

// Gauss elimination of tmat without pivoting, with the right-hand side v,
// and the back substitution: blts (src/LU/blts.jl:106-193) or, with
// buts_form, buts as the reference states it (src/LU/buts.jl:113-200).
void block_solve(Blk t, double v[5], bool buts_form) {
  double tmp1, tmp;
  tmp1 = 1.0e+00 / t[0][0];
  for (int r = 1; r < 5; ++r) {
    tmp = tmp1 * t[r][0];
    for (int cc = 1; cc < 5; ++cc) t[r][cc] = t[r][cc] - tmp * t[0][cc];
    v[r] = v[r] - v[0] * tmp;
  }
  tmp1 = 1.0e+00 / t[1][1];
  for (int r = 2; r < 5; ++r) {
    tmp = tmp1 * t[r][1];
    for (int cc = 2; cc < 5; ++cc) {
      if (buts_form && r == 4 && cc == 4)
        t[r][cc] = t[r][cc] - (-tmp * t[1][cc]);  // tmat[5,5] -=- tmp * tmat[2,5]
      else
        t[r][cc] = t[r][cc] - tmp * t[1][cc];
    }
    v[r] = v[r] - v[1] * tmp;
  }
  tmp1 = 1.0e+00 / t[2][2];
  for (int r = 3; r < 5; ++r) {
    tmp = tmp1 * t[r][2];
    for (int cc = 3; cc < 5; ++cc) t[r][cc] = t[r][cc] - tmp * t[2][cc];
    v[r] = v[r] - v[2] * tmp;
  }
  tmp1 = 1.0e+00 / t[3][3];
  tmp = tmp1 * t[4][3];
  t[4][4] = t[4][4] - tmp * t[3][4];
  v[4] = v[4] - v[3] * tmp;
  v[4] = v[4] / t[4][4];
  v[3] = v[3] - t[3][4] * v[4];
  v[3] = v[3] / t[3][3];
  if (buts_form) {
    v[2] = v[2] - (t[2][3] * v[3] - t[2][4] * v[4]);
    v[2] = v[2] / t[2][2];
    v[1] = v[1] - (t[1][2] * v[2] - t[1][3] * v[3] - t[1][4] * v[4]);
    v[1] = v[1] / t[1][1];
    v[0] = v[0] - (t[0][1] * v[1] - t[0][2] * v[2] - t[0][3] * v[3] - t[0][4] * v[4]);
    v[0] = v[0] / t[0][0];
  } else {
    v[2] = v[2] - (t[2][3] * v[3] + t[2][4] * v[4]);
    v[2] = v[2] / t[2][2];
    v[1] = v[1] - (t[1][2] * v[2] + t[1][3] * v[3] + t[1][4] * v[4]);
    v[1] = v[1] / t[1][1];
    v[0] = v[0] - (t[0][1] * v[1] + t[0][2] * v[2] + t[0][3] * v[3] + t[0][4] * v[4]);
    v[0] = v[0] / t[0][0];
  }
}

// jacld + blts of one (j, k) row (src/LU/ssor.jl:78-99, src/LU/blts.jl)
void lower_row(Problem& pb, Zone& z, int j, int k) {
  const int ist = 2, iend = z.nx - 1;
  const double omega = pb.omega;
  std::vector<double> D((size_t)z.nx * 25), A((size_t)z.nx * 25), B((size_t)z.nx * 25), Cb((size_t)z.nx * 25);
  auto blk = [](std::vector<double>& v, int i) { return reinterpret_cast<Blk*>(&v[(size_t)i * 25]); };
  for (int i = ist; i <= iend; ++i) jacld_point(z, z.C, pb.dt, i, j, k, *blk(D, i), *blk(A, i), *blk(B, i), *blk(Cb, i));
  for (int i = ist; i <= iend; ++i) {
    Blk& ldz = *blk(A, i);
    for (int m = 0; m < 5; ++m)
      z.R(m + 1, i, j, k) = z.R(m + 1, i, j, k) -
                            omega * (ldz[m][0] * z.R(1, i, j, k - 1) + ldz[m][1] * z.R(2, i, j, k - 1) +
                                     ldz[m][2] * z.R(3, i, j, k - 1) + ldz[m][3] * z.R(4, i, j, k - 1) +
                                     ldz[m][4] * z.R(5, i, j, k - 1));
  }
  for (int i = ist; i <= iend; ++i) {
    Blk& ldy = *blk(B, i);
    Blk& ldx = *blk(Cb, i);
    for (int m = 0; m < 5; ++m)
      z.R(m + 1, i, j, k) =
          z.R(m + 1, i, j, k) -
          omega * (ldy[m][0] * z.R(1, i, j - 1, k) + ldx[m][0] * z.R(1, i - 1, j, k) + ldy[m][1] * z.R(2, i, j - 1, k) +
                   ldx[m][1] * z.R(2, i - 1, j, k) + ldy[m][2] * z.R(3, i, j - 1, k) + ldx[m][2] * z.R(3, i - 1, j, k) +
                   ldy[m][3] * z.R(4, i, j - 1, k) + ldx[m][3] * z.R(4, i - 1, j, k) + ldy[m][4] * z.R(5, i, j - 1, k) +
                   ldx[m][4] * z.R(5, i - 1, j, k));
    Blk t;
    std::memcpy(t, *blk(D, i), sizeof(Blk));
    double v[5];
    for (int m = 0; m < 5; ++m) v[m] = z.R(m + 1, i, j, k);
    block_solve(t, v, false);
    for (int m = 0; m < 5; ++m) z.R(m + 1, i, j, k) = v[m];
  }
}

// jacu + buts of one (j, k) row (src/LU/ssor.jl:113-165, src/LU/buts.jl)
void upper_row(Problem& pb, Zone& z, int j, int k) {
  const int ist = 2, iend = z.nx - 1;
  const double omega = pb.omega;
  std::vector<double> D((size_t)z.nx * 25), A((size_t)z.nx * 25), B((size_t)z.nx * 25), Cb((size_t)z.nx * 25);
  std::vector<double> tv((size_t)z.nx * 5);
  auto blk = [](std::vector<double>& v, int i) { return reinterpret_cast<Blk*>(&v[(size_t)i * 25]); };
  for (int i = ist; i <= iend; ++i) jacu_point(z, z.C, pb.dt, i, j, k, *blk(D, i), *blk(A, i), *blk(B, i), *blk(Cb, i));
  for (int i = iend; i >= ist; --i) {
    Blk& udz = *blk(Cb, i);
    for (int m = 0; m < 5; ++m)
      tv[(size_t)i * 5 + m] =
          omega * (udz[m][0] * z.R(1, i, j, k + 1) + udz[m][1] * z.R(2, i, j, k + 1) + udz[m][2] * z.R(3, i, j, k + 1) +
                   udz[m][3] * z.R(4, i, j, k + 1) + udz[m][4] * z.R(5, i, j, k + 1));
  }
  for (int i = iend; i >= ist; --i) {
    Blk& udy = *blk(B, i);
    Blk& udx = *blk(A, i);
    double v[5];
    for (int m = 0; m < 5; ++m)
      v[m] = tv[(size_t)i * 5 + m] +
             omega * (udy[m][0] * z.R(1, i, j + 1, k) + udx[m][0] * z.R(1, i + 1, j, k) +
                      udy[m][1] * z.R(2, i, j + 1, k) + udx[m][1] * z.R(2, i + 1, j, k) +
                      udy[m][2] * z.R(3, i, j + 1, k) + udx[m][2] * z.R(3, i + 1, j, k) +
                      udy[m][3] * z.R(4, i, j + 1, k) + udx[m][3] * z.R(4, i + 1, j, k) +
                      udy[m][4] * z.R(5, i, j + 1, k) + udx[m][4] * z.R(5, i + 1, j, k));
    Blk t;
    std::memcpy(t, *blk(D, i), sizeof(Blk));
    block_solve(t, v, true);
    for (int m = 0; m < 5; ++m) z.R(m + 1, i, j, k) = z.R(m + 1, i, j, k) - v[m];
  }
}

void scale_rsd(Problem& pb, Zone& z) {
  for (int k = 2; k <= z.nz - 1; ++k)
    for (int j = 2; j <= z.ny - 1; ++j)
      for (int i = 2; i <= z.nx - 1; ++i)
        for (int m = 1; m <= 5; ++m) z.R(m, i, j, k) = pb.dt * z.R(m, i, j, k);
}

void lower_sweep(Problem& pb, Zone& z) {
  for (int k = 2; k <= z.nz - 1; ++k)
    for (int j = 2; j <= z.ny - 1; ++j) lower_row(pb, z, j, k);
}

void upper_sweep(Problem& pb, Zone& z) {
  for (int k = z.nz - 1; k >= 2; --k)
    for (int j = z.ny - 1; j >= 2; --j) upper_row(pb, z, j, k);
}

void update(Problem& pb, Zone& z) {
  const double tmp = 1.0e+00 / (pb.omega * (2.0e+00 - pb.omega));
  for (int k = 2; k <= z.nz - 1; ++k)
    for (int j = 2; j <= z.ny - 1; ++j)
      for (int i = 2; i <= z.nx - 1; ++i)
        for (int m = 1; m <= 5; ++m) z.U(m, i, j, k) = z.U(m, i, j, k) + tmp * z.R(m, i, j, k);
}

void ssor(Problem& pb, Zone& z) {
  scale_rsd(pb, z);
  lower_sweep(pb, z);
  upper_sweep(pb, z);
  update(pb, z);
  rhs(z);
}

// src/LU/exchange_qbc.jl, one process: every face is packed before any is
// unpacked; unpack order south, north, west, east (corners from west/east);
// planes k = 1..nz-2 (the reference) or 2..nz-1 (faces_npb).
void exch_qbc(Problem& pb) {
  const int nzn = pb.nzones;
  std::vector<std::vector<double>> e_out(nzn), w_out(nzn), s_out(nzn), n_out(nzn);
  for (int zi = 0; zi < nzn; ++zi) {
    Zone& z = pb.zones[zi];
    const int klo = pb.faces_npb ? 2 : 1, khi = pb.faces_npb ? z.nz - 1 : z.nz - 2;
    for (int k = klo; k <= khi; ++k)  // east face: j = ny-1
      for (int i = 1; i <= z.nx; ++i)
        for (int m = 1; m <= 5; ++m) e_out[zi].push_back(z.U(m, i, z.ny - 1, k));
    for (int k = klo; k <= khi; ++k)  // west face: j = 2
      for (int i = 1; i <= z.nx; ++i)
        for (int m = 1; m <= 5; ++m) w_out[zi].push_back(z.U(m, i, 2, k));
    for (int k = klo; k <= khi; ++k)  // south face: i = nx-1
      for (int j = 1; j <= z.ny; ++j)
        for (int m = 1; m <= 5; ++m) s_out[zi].push_back(z.U(m, z.nx - 1, j, k));
    for (int k = klo; k <= khi; ++k)  // north face: i = 2
      for (int j = 1; j <= z.ny; ++j)
        for (int m = 1; m <= 5; ++m) n_out[zi].push_back(z.U(m, 2, j, k));
  }
  for (int zi = 0; zi < nzn; ++zi) {
    Zone& z = pb.zones[zi];
    const int klo = pb.faces_npb ? 2 : 1, khi = pb.faces_npb ? z.nz - 1 : z.nz - 2;
    const int w = pb.nbr[4 * zi + 0], e = pb.nbr[4 * zi + 1], s = pb.nbr[4 * zi + 2], n = pb.nbr[4 * zi + 3];
    size_t p = 0;
    for (int k = klo; k <= khi; ++k)  // south ghost i = nx <- south zone's north face
      for (int j = 1; j <= z.ny; ++j)
        for (int m = 1; m <= 5; ++m) z.U(m, z.nx, j, k) = n_out[s][p++];
    p = 0;
    for (int k = klo; k <= khi; ++k)  // north ghost i = 1 <- north zone's south face
      for (int j = 1; j <= z.ny; ++j)
        for (int m = 1; m <= 5; ++m) z.U(m, 1, j, k) = s_out[n][p++];
    p = 0;
    for (int k = klo; k <= khi; ++k)  // west ghost j = 1 <- west zone's east face
      for (int i = 1; i <= z.nx; ++i)
        for (int m = 1; m <= 5; ++m) z.U(m, i, 1, k) = e_out[w][p++];
    p = 0;
    for (int k = klo; k <= khi; ++k)  // east ghost j = ny <- east zone's west face
      for (int i = 1; i <= z.nx; ++i)
        for (int m = 1; m <= 5; ++m) z.U(m, i, z.ny, k) = w_out[e][p++];
  }
}

// src/LU/l2norm.jl (before the sqrt: the caller needs per-zone values)
void l2norm(Zone& z, double out[5]) {
  double sum[5] = {0, 0, 0, 0, 0};
  for (int k = 2; k <= z.nz - 1; ++k)
    for (int j = 2; j <= z.ny - 1; ++j)
      for (int i = 2; i <= z.nx - 1; ++i)
        for (int m = 1; m <= 5; ++m) sum[m - 1] = sum[m - 1] + z.R(m, i, j, k) * z.R(m, i, j, k);
  for (int m = 0; m < 5; ++m) out[m] = std::sqrt(sum[m] / ((double)(z.nx - 2) * (z.ny - 2) * (z.nz - 2)));
}

// src/LU/error.jl
void error_norm(const Problem& pb, Zone& z, double out[5]) {
  double sum[5] = {0, 0, 0, 0, 0}, e[5];
  for (int k = 2; k <= z.nz - 1; ++k)
    for (int j = 2; j <= z.ny - 1; ++j)
      for (int i = 2; i <= z.nx - 1; ++i) {
        exact(pb, i, j, k, e, z.nx, z.ny, z.nz);
        for (int m = 1; m <= 5; ++m) {
          double tmp = e[m - 1] - z.U(m, i, j, k);
          sum[m - 1] = sum[m - 1] + tmp * tmp;
        }
      }
  for (int m = 0; m < 5; ++m) out[m] = std::sqrt(sum[m] / ((double)(z.nx - 2) * (z.ny - 2) * (z.nz - 2)));
}

// src/LU/pintgr.jl, one process (ibeg = ii1, ifin = ii2, jbeg = ji1, jfin = ji2)
double pintgr(Zone& z) {
  const Coeff& C = z.C;
  const int ibeg = ii1, ifin = C.ii2, jbeg = ji1, jfin = C.ji2;
  const int ifin1 = ifin - 1, jfin1 = jfin - 1;
  auto phi = [&](int i, int j, int k) {
    return c2 * (z.U(5, i, j, k) - 0.50e+00 *
                                       (z.U(2, i, j, k) * z.U(2, i, j, k) + z.U(3, i, j, k) * z.U(3, i, j, k) +
                                        z.U(4, i, j, k) * z.U(4, i, j, k)) /
                                       z.U(1, i, j, k));
  };
  double frc1 = 0.0;
  for (int j = jbeg; j <= jfin1; ++j)
    for (int i = ibeg; i <= ifin1; ++i)
      frc1 = frc1 + (phi(i, j, ki1) + phi(i + 1, j, ki1) + phi(i, j + 1, ki1) + phi(i + 1, j + 1, ki1) +
                     phi(i, j, C.ki2) + phi(i + 1, j, C.ki2) + phi(i, j + 1, C.ki2) + phi(i + 1, j + 1, C.ki2));
  frc1 = C.dxi * C.deta * frc1;
  double frc2 = 0.0;
  for (int k = ki1; k <= C.ki2 - 1; ++k)
    for (int i = ibeg; i <= ifin1; ++i)
      frc2 = frc2 + (phi(i, jbeg, k) + phi(i + 1, jbeg, k) + phi(i, jbeg, k + 1) + phi(i + 1, jbeg, k + 1) +
                     phi(i, jfin, k) + phi(i + 1, jfin, k) + phi(i, jfin, k + 1) + phi(i + 1, jfin, k + 1));
  frc2 = C.dxi * C.dzeta * frc2;
  double frc3 = 0.0;
  for (int k = ki1; k <= C.ki2 - 1; ++k)
    for (int j = jbeg; j <= jfin1; ++j)
      frc3 = frc3 + (phi(ibeg, j, k) + phi(ibeg, j + 1, k) + phi(ibeg, j, k + 1) + phi(ibeg, j + 1, k + 1) +
                     phi(ifin, j, k) + phi(ifin, j + 1, k) + phi(ifin, j, k + 1) + phi(ifin, j + 1, k + 1));
  frc3 = C.deta * C.dzeta * frc3;
  return 0.25e+00 * (frc1 + frc2 + frc3);
}

}  // namespace

extern "C" {

struct lu_oracle_t;

// src/LU/zone_setup.jl: zone sizes and LU's neighbour table (west, east,
// south, north per zone, 0-based).  Returns -1 if an x or y extent is not
// an integer (the reference's Int conversion would throw) or a neighbour
// falls outside the zone range (the rule assumes x_zones == y_zones).
int lu_oracle_zone_setup(int gx, int gy, int gz, int xz, int yz, double ratio, int* nx, int* ny, int* nz, int* nbr) {
  std::vector<long> x_end(xz), y_end(yz), x_start(xz), y_start(yz), x_size(xz), y_size(yz);
  if (std::fabs(ratio - 1.0e0) > 1.0e-10) {
    double x_r = std::exp(std::log(ratio) / (xz - 1));
    double y_r = std::exp(std::log(ratio) / (yz - 1));
    double x_smallest = (double)gx * (x_r - 1.0e0) / (std::pow(x_r, xz) - 1.0e0);
    double y_smallest = (double)gy * (y_r - 1.0e0) / (std::pow(y_r, yz) - 1.0e0);
    for (int i = 1; i <= xz; ++i) x_end[i - 1] = (long)std::nearbyint(x_smallest * (std::pow(x_r, i) - 1.0e0) / (x_r - 1.0e0) + 0.45e0);
    for (int j = 1; j <= yz; ++j) y_end[j - 1] = (long)std::nearbyint(y_smallest * (std::pow(y_r, j) - 1.0e0) / (y_r - 1.0e0) + 0.45e0);
  } else {
    for (int i = 1; i <= xz; ++i) {
      if (((long)i * gx) % xz) return -1;
      x_end[i - 1] = (long)i * gx / xz;
    }
    for (int j = 1; j <= yz; ++j) {
      if (((long)j * gy) % yz) return -1;
      y_end[j - 1] = (long)j * gy / yz;
    }
  }
  x_start[0] = 1;
  for (int i = 0; i < xz; ++i) {
    if (i != xz - 1) x_start[i + 1] = x_end[i] + 1;
    x_size[i] = x_end[i] - x_start[i] + 1;
  }
  y_start[0] = 1;
  for (int j = 0; j < yz; ++j) {
    if (j != yz - 1) y_start[j + 1] = y_end[j] + 1;
    y_size[j] = y_end[j] - y_start[j] + 1;
  }
  const int nzones = xz * yz;
  for (int j = 1; j <= yz; ++j)
    for (int i = 1; i <= xz; ++i) {
      const int zone_no = (i - 1) + (j - 1) * xz + 1;
      nx[zone_no - 1] = (int)x_size[i - 1];
      ny[zone_no - 1] = (int)y_size[j - 1];
      nz[zone_no - 1] = gz;
      const int row = i, col = j;
      int north = row > 1 ? zone_no - 1 : col * xz;
      int south = row < xz ? zone_no + 1 : zone_no - xz + 1;
      int west = col > 1 ? zone_no - xz : zone_no + yz * (xz - 1);
      int east = col < yz ? zone_no + xz : zone_no - yz * (xz - 1);
      for (int q : {north, south, west, east})
        if (q < 1 || q > nzones) return -1;
      nbr[4 * (zone_no - 1) + 0] = west - 1;
      nbr[4 * (zone_no - 1) + 1] = east - 1;
      nbr[4 * (zone_no - 1) + 2] = south - 1;
      nbr[4 * (zone_no - 1) + 3] = north - 1;
    }
  return 0;
}

// setbv, setiv, erhs, and the first rhs for every zone (the reference's
// warm-up iteration is followed by setbv / setiv / rhs again, so it leaves
// no trace).  ce: 65 values row-major [5][13], or NULL for the reference's.
// faces_npb: exch_qbc copies planes k = 2..nz-1 instead of the reference's
// 1..nz-2.
lu_oracle_t* lu_oracle_create(int nzones, const int* nx, const int* ny, const int* nz, const int* nbr, double dt,
                              double omega, const double* ce, int faces_npb) {
  Problem* pb = new Problem();
  pb->nzones = nzones;
  pb->dt = dt;
  pb->omega = omega;
  pb->faces_npb = faces_npb;
  std::memcpy(pb->ce, ce ? ce : &ce_reference[0][0], sizeof(pb->ce));
  pb->nbr.assign(nbr, nbr + 4 * nzones);
  pb->zones.resize(nzones);
  for (int zi = 0; zi < nzones; ++zi) {
    Zone& z = pb->zones[zi];
    z.nx = nx[zi]; z.ny = ny[zi]; z.nz = nz[zi];
    z.C = setcoeff(z.nx, z.ny, z.nz);
    const size_t n = (size_t)z.nx * z.ny * z.nz * 5;
    z.u.assign(n, 0.0);
    z.rsd.assign(n, 0.0);
    z.frct.assign(n, 0.0);
    setbv(*pb, z);
    setiv(*pb, z);
    erhs(*pb, z);
    rhs(z);
  }
  return reinterpret_cast<lu_oracle_t*>(pb);
}

void lu_oracle_destroy(lu_oracle_t* h) { delete reinterpret_cast<Problem*>(h); }

// niter iterations of exch_qbc over all zones + ssor per zone
// (src/LU/lu-node.jl time loop)
int lu_oracle_iterate(lu_oracle_t* h, int niter) {
  Problem& pb = *reinterpret_cast<Problem*>(h);
  for (int it = 0; it < niter; ++it) {
    exch_qbc(pb);
#pragma omp parallel for schedule(dynamic, 1)
    for (int zi = 0; zi < pb.nzones; ++zi) ssor(pb, pb.zones[zi]);
  }
  return 0;
}

// phases for phase-level checks; zone -1 = every zone.
// 0 rhs, 1 rsd *= dt, 2 jacld+blts sweep, 3 jacu+buts sweep, 4 update,
// 5 exch_qbc (all zones), 6 ssor
int lu_oracle_phase(lu_oracle_t* h, int phase, int zone) {
  Problem& pb = *reinterpret_cast<Problem*>(h);
  if (phase == 5) {
    exch_qbc(pb);
    return 0;
  }
  for (int zi = 0; zi < pb.nzones; ++zi) {
    if (zone >= 0 && zi != zone) continue;
    Zone& z = pb.zones[zi];
    switch (phase) {
      case 0: rhs(z); break;
      case 1: scale_rsd(pb, z); break;
      case 2: lower_sweep(pb, z); break;
      case 3: upper_sweep(pb, z); break;
      case 4: update(pb, z); break;
      case 6: ssor(pb, z); break;
      default: return -1;
    }
  }
  return 0;
}

// Norms summed over zones as lu-node.jl does (xcr: l2norm of rsd, xce:
// error, xci: pintgr).  Per-zone values in zxcr / zxce / zxci when non-NULL.
int lu_oracle_verify(lu_oracle_t* h, double* xcr, double* xce, double* xci, double* zxcr, double* zxce, double* zxci) {
  Problem& pb = *reinterpret_cast<Problem*>(h);
  for (int m = 0; m < 5; ++m) xcr[m] = xce[m] = 0.0;
  *xci = 0.0;
  for (int zi = 0; zi < pb.nzones; ++zi) {
    Zone& z = pb.zones[zi];
    double r[5], e[5];
    error_norm(pb, z, e);
    l2norm(z, r);
    double f = pintgr(z);
    for (int m = 0; m < 5; ++m) {
      xcr[m] += r[m];
      xce[m] += e[m];
      if (zxcr) zxcr[5 * zi + m] = r[m];
      if (zxce) zxce[5 * zi + m] = e[m];
    }
    *xci += f;
    if (zxci) zxci[zi] = f;
  }
  return 0;
}

// field 0 u, 1 rsd, 2 frct; dense [5][nz][ny][nx] per zone
int lu_oracle_get(lu_oracle_t* h, int field, int zone, double* out) {
  Problem& pb = *reinterpret_cast<Problem*>(h);
  Zone& z = pb.zones[zone];
  std::vector<double>& v = field == 0 ? z.u : (field == 1 ? z.rsd : z.frct);
  const size_t np = (size_t)z.nx * z.ny * z.nz;
  for (int m = 0; m < 5; ++m)
    for (size_t p = 0; p < np; ++p) out[m * np + p] = v[p * 5 + m];
  return 0;
}

int lu_oracle_set(lu_oracle_t* h, int field, int zone, const double* in) {
  Problem& pb = *reinterpret_cast<Problem*>(h);
  Zone& z = pb.zones[zone];
  std::vector<double>& v = field == 0 ? z.u : (field == 1 ? z.rsd : z.frct);
  const size_t np = (size_t)z.nx * z.ny * z.nz;
  for (int m = 0; m < 5; ++m)
    for (size_t p = 0; p < np; ++p) v[p * 5 + m] = in[m * np + p];
  return 0;
}

}  // extern "C"
