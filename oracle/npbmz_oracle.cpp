// npbmz_oracle.cpp -- CPU restatement of the NPBApps.jl BT-MZ / SP-MZ ADI time step.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle: a scalar, loop-for-loop
// restatement of the reference's single-rank path (one MPI rank per cluster,
// ncells = 1, so cell_start = cell_end = 1 and each line solve is one stage).
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg and
// reference arm may load it: to compare against, or to time the reference's
// CPU path.  The product (libnpbmz_gpu.so) never calls it.
//
// Every arithmetic expression keeps the reference's operand order and
// parenthesisation, and the file is compiled with -ffp-contract=off, because
// Julia does not contract a*b+c into an FMA.  Reference files (paths relative
// to the NPBApps.jl source tree):
//   constants ........ src/BT/set_constants.jl:1-130, src/SP/set_constants.jl:1-130
//   zone geometry .... src/BT/zone_setup.jl:1-77, src/SP/zone_setup.jl:1-78
//   exact solution ... src/BT/exact_solution.jl:5-18
//   initialize ....... src/BT/initialize.jl:6-212, src/SP/initialize.jl:6-206
//   exact_rhs ........ src/BT/exact_rhs.jl:5-370 (SP copy: src/SP/exact_rhs.jl)
//   compute_rhs ...... src/BT/rhs.jl:4-460, src/SP/rhs.jl:3-452
//   BT line solves ... src/BT/x_solve.jl:444-488,501-1746, src/BT/y_solve.jl:443-820,
//                      src/BT/z_solve.jl:438-864, src/BT/solve_subs.jl:4-37,193-461,468-862
//   SP transforms .... src/SP/txinvr.jl:5-56, ninvr.jl:5-38, pinvr.jl:5-39, tzetar.jl:5-59
//   SP line solves ... src/SP/lhsx.jl:5-114, lhsy.jl, lhsz.jl, src/SP/x_solve.jl:8-557,
//                      src/SP/y_solve.jl, src/SP/z_solve.jl
//   add .............. src/BT/add.jl:5-24, src/SP/add.jl:6-26
//   exch_qbc ......... src/BT/exchange_qbc.jl:145-465 (semantics of the zone-face copy)
//   norms ............ src/BT/error.jl:7-79, src/SP/error.jl:7-81, src/BT/verify.jl:411-505
//   time loop ........ src/BT/bt-node.jl:93-426, src/SP/sp-node.jl:86-400
//
// Halo points outside 0..n-1 (the reference's 2-deep OffsetArray halo) are not
// stored: on the single-cell path no value computed there reaches u, rhs or a
// norm (compute_rhs evaluates primitives at -1 and n, but every stencil on the
// interior 1..n-2 reads only 0..n-1).
//
// The line solves are templated on the arithmetic type T so that the same
// restatement also runs with float line solves (the mixed-precision variant's
// expected behaviour); T = double is the reference path.
//
// The state (u, rhs, forcing and the primitive variables) has the scalar type
// `real`, double here.  oracle/npbmz_tangent.cpp includes this file with a
// forward-mode dual number as `real` (ORACLE_REAL, ORACLE_TANGENT) to push
// directional derivatives through the same BT and SP statements, with the
// line solves in `real`; the dual's value part then follows exactly the
// double operations of this file.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifndef ORACLE_REAL
#define ORACLE_REAL double
#endif
#ifndef ORACLE_TANGENT
#define ORACLE_TANGENT 0
#endif

namespace {

typedef ORACLE_REAL real;
inline double value(double x) { return x; }
// std::max(a, b) on the value part: b when a < b, else a
inline real rmax(const real& a, const real& b) { return value(a) < value(b) ? b : a; }

constexpr int KIND_BT = 0;
constexpr int KIND_SP = 1;

// ---- fixed constants (src/BT/set_constants.jl:1-45) -----------------------
const double c1 = 1.4e0, c2 = 0.4e0, c3 = 0.1e0, c4 = 1.0e0, c5 = 1.4e0;
const double bt_ = std::sqrt(0.5e0);
const double c1c2 = c1 * c2, c1c5 = c1 * c5, c3c4 = c3 * c4, c1345 = c1c5 * c3c4;
const double conz1 = (1.0e0 - c1c5);
const double dx1 = 0.75e0, dx2 = 0.75e0, dx3 = 0.75e0, dx4 = 0.75e0, dx5 = 0.75e0;
const double dy1 = 0.75e0, dy2 = 0.75e0, dy3 = 0.75e0, dy4 = 0.75e0, dy5 = 0.75e0;
const double dz1 = 1.0e0, dz2 = 1.0e0, dz3 = 1.0e0, dz4 = 1.0e0, dz5 = 1.0e0;
const double dxmax = std::max(dx3, dx4), dymax = std::max(dy2, dy4), dzmax = std::max(dz2, dz3);
const double dssp = 0.25e0 * std::max(dx1, std::max(dy1, dz1));
const double c2iv = 2.5e0, con43 = 4.0e0 / 3.0e0, con16 = 1.0e0 / 6.0e0;

// ---- derived constants (src/BT/set_constants.jl:53-130) --------------------
struct Consts {
  double dt, dnxm1, dnym1, dnzm1;
  double tx1, tx2, tx3, ty1, ty2, ty3, tz1, tz2, tz3;
  double dttx1, dttx2, dtty1, dtty2, dttz1, dttz2, c2dttx1, c2dtty1, c2dttz1;
  double dtdssp, comz1, comz4, comz5, comz6;
  double c3c4tx3, c3c4ty3, c3c4tz3;
  double dx1tx1, dx2tx1, dx3tx1, dx4tx1, dx5tx1;
  double dy1ty1, dy2ty1, dy3ty1, dy4ty1, dy5ty1;
  double dz1tz1, dz2tz1, dz3tz1, dz4tz1, dz5tz1;
  double xxcon1, xxcon2, xxcon3, xxcon4, xxcon5;
  double yycon1, yycon2, yycon3, yycon4, yycon5;
  double zzcon1, zzcon2, zzcon3, zzcon4, zzcon5;
};

Consts set_constants(double dt, int gx, int gy, int gz, int xz, int yz) {
  Consts k;
  k.dt = dt;
  k.dnxm1 = 1.0e0 / ((double)(gx - 1) / (double)xz);
  k.dnym1 = 1.0e0 / ((double)(gy - 1) / (double)yz);
  k.dnzm1 = 1.0e0 / (double)(gz - 1);
  k.tx1 = 1.0e0 / (k.dnxm1 * k.dnxm1); k.tx2 = 1.0e0 / (2.0e0 * k.dnxm1); k.tx3 = 1.0e0 / k.dnxm1;
  k.ty1 = 1.0e0 / (k.dnym1 * k.dnym1); k.ty2 = 1.0e0 / (2.0e0 * k.dnym1); k.ty3 = 1.0e0 / k.dnym1;
  k.tz1 = 1.0e0 / (k.dnzm1 * k.dnzm1); k.tz2 = 1.0e0 / (2.0e0 * k.dnzm1); k.tz3 = 1.0e0 / k.dnzm1;
  k.dttx1 = dt * k.tx1; k.dttx2 = dt * k.tx2;
  k.dtty1 = dt * k.ty1; k.dtty2 = dt * k.ty2;
  k.dttz1 = dt * k.tz1; k.dttz2 = dt * k.tz2;
  k.c2dttx1 = 2.0e0 * k.dttx1; k.c2dtty1 = 2.0e0 * k.dtty1; k.c2dttz1 = 2.0e0 * k.dttz1;
  k.dtdssp = dt * dssp;
  k.comz1 = k.dtdssp; k.comz4 = 4.0e0 * k.dtdssp; k.comz5 = 5.0e0 * k.dtdssp; k.comz6 = 6.0e0 * k.dtdssp;
  k.c3c4tx3 = c3c4 * k.tx3; k.c3c4ty3 = c3c4 * k.ty3; k.c3c4tz3 = c3c4 * k.tz3;
  k.dx1tx1 = dx1 * k.tx1; k.dx2tx1 = dx2 * k.tx1; k.dx3tx1 = dx3 * k.tx1; k.dx4tx1 = dx4 * k.tx1; k.dx5tx1 = dx5 * k.tx1;
  k.dy1ty1 = dy1 * k.ty1; k.dy2ty1 = dy2 * k.ty1; k.dy3ty1 = dy3 * k.ty1; k.dy4ty1 = dy4 * k.ty1; k.dy5ty1 = dy5 * k.ty1;
  k.dz1tz1 = dz1 * k.tz1; k.dz2tz1 = dz2 * k.tz1; k.dz3tz1 = dz3 * k.tz1; k.dz4tz1 = dz4 * k.tz1; k.dz5tz1 = dz5 * k.tz1;
  k.xxcon1 = k.c3c4tx3 * con43 * k.tx3; k.xxcon2 = k.c3c4tx3 * k.tx3; k.xxcon3 = k.c3c4tx3 * conz1 * k.tx3;
  k.xxcon4 = k.c3c4tx3 * con16 * k.tx3; k.xxcon5 = k.c3c4tx3 * c1c5 * k.tx3;
  k.yycon1 = k.c3c4ty3 * con43 * k.ty3; k.yycon2 = k.c3c4ty3 * k.ty3; k.yycon3 = k.c3c4ty3 * conz1 * k.ty3;
  k.yycon4 = k.c3c4ty3 * con16 * k.ty3; k.yycon5 = k.c3c4ty3 * c1c5 * k.ty3;
  k.zzcon1 = k.c3c4tz3 * con43 * k.tz3; k.zzcon2 = k.c3c4tz3 * k.tz3; k.zzcon3 = k.c3c4tz3 * conz1 * k.tz3;
  k.zzcon4 = k.c3c4tz3 * con16 * k.tz3; k.zzcon5 = k.c3c4tz3 * c1c5 * k.tz3;
  return k;
}

// ---- exact solution (src/BT/exact_solution.jl:5-18); ce is row-major [5][13] --
void exact_solution(double xi, double eta, double zeta, const double* ce, double out[5]) {
  for (int m = 0; m < 5; ++m) {
    const double* c = ce + 13 * m;
    out[m] = c[0] +
             xi * (c[1] + xi * (c[4] + xi * (c[7] + xi * c[10]))) +
             eta * (c[2] + eta * (c[5] + eta * (c[8] + eta * c[11]))) +
             zeta * (c[3] + zeta * (c[6] + zeta * (c[9] + zeta * c[12])));
  }
}

struct Zone {
  int nx, ny, nz;
  std::vector<real> u, rhs, forcing;                  // [k][j][i][m]
  std::vector<real> rho_i, us, vs, ws, qs, square, speed, ainv;  // [k][j][i]
  size_t P(int i, int j, int k) const { return ((size_t)k * ny + j) * nx + i; }
  real& U(int m, int i, int j, int k) { return u[P(i, j, k) * 5 + m]; }
  real& R(int m, int i, int j, int k) { return rhs[P(i, j, k) * 5 + m]; }
  real& F(int m, int i, int j, int k) { return forcing[P(i, j, k) * 5 + m]; }
};

struct Problem {
  int kind, nzones;
  Consts k;
  double ce[65];
  std::vector<Zone> zones;
  std::vector<int> nbr;   // per zone: west, east, south, north (0-based zone ids)
  int solve_float;        // 1: line solves in float (mixed-precision emulation)
};

// ---- initialize (src/BT/initialize.jl:6-212; SP halo values differ only) --
void initialize(Problem& pb, Zone& z) {
  const Consts& K = pb.k;
  double Pface1[2][5], Pface2[2][5], Pface3[2][5], temp[5];
  for (int k = 0; k < z.nz; ++k) {
    double zeta = (double)k * K.dnzm1;
    for (int j = 0; j < z.ny; ++j) {
      double eta = (double)j * K.dnym1;
      for (int i = 0; i < z.nx; ++i) {
        double xi = (double)i * K.dnxm1;
        for (int ix = 0; ix < 2; ++ix) exact_solution((double)ix, eta, zeta, pb.ce, Pface1[ix]);
        for (int iy = 0; iy < 2; ++iy) exact_solution(xi, (double)iy, zeta, pb.ce, Pface2[iy]);
        for (int iz = 0; iz < 2; ++iz) exact_solution(xi, eta, (double)iz, pb.ce, Pface3[iz]);
        for (int m = 0; m < 5; ++m) {
          double Pxi = xi * Pface1[1][m] + (1.0e0 - xi) * Pface1[0][m];
          double Peta = eta * Pface2[1][m] + (1.0e0 - eta) * Pface2[0][m];
          double Pzeta = zeta * Pface3[1][m] + (1.0e0 - zeta) * Pface3[0][m];
          z.U(m, i, j, k) = Pxi + Peta + Pzeta - Pxi * Peta - Pxi * Pzeta - Peta * Pzeta + Pxi * Peta * Pzeta;
        }
      }
    }
  }
  // boundary faces, in the reference's order: west, east, south, north, bottom, top
  for (int k = 0; k < z.nz; ++k) {
    double zeta = (double)k * K.dnzm1;
    for (int j = 0; j < z.ny; ++j) {
      double eta = (double)j * K.dnym1;
      exact_solution(0.0e0, eta, zeta, pb.ce, temp);
      for (int m = 0; m < 5; ++m) z.U(m, 0, j, k) = temp[m];
    }
  }
  for (int k = 0; k < z.nz; ++k) {
    double zeta = (double)k * K.dnzm1;
    for (int j = 0; j < z.ny; ++j) {
      double eta = (double)j * K.dnym1;
      exact_solution(1.0e0, eta, zeta, pb.ce, temp);
      for (int m = 0; m < 5; ++m) z.U(m, z.nx - 1, j, k) = temp[m];
    }
  }
  for (int k = 0; k < z.nz; ++k) {
    double zeta = (double)k * K.dnzm1;
    for (int i = 0; i < z.nx; ++i) {
      double xi = (double)i * K.dnxm1;
      exact_solution(xi, 0.0e0, zeta, pb.ce, temp);
      for (int m = 0; m < 5; ++m) z.U(m, i, 0, k) = temp[m];
    }
  }
  for (int k = 0; k < z.nz; ++k) {
    double zeta = (double)k * K.dnzm1;
    for (int i = 0; i < z.nx; ++i) {
      double xi = (double)i * K.dnxm1;
      exact_solution(xi, 1.0e0, zeta, pb.ce, temp);
      for (int m = 0; m < 5; ++m) z.U(m, i, z.ny - 1, k) = temp[m];
    }
  }
  for (int j = 0; j < z.ny; ++j) {
    double eta = (double)j * K.dnym1;
    for (int i = 0; i < z.nx; ++i) {
      double xi = (double)i * K.dnxm1;
      exact_solution(xi, eta, 0.0e0, pb.ce, temp);
      for (int m = 0; m < 5; ++m) z.U(m, i, j, 0) = temp[m];
    }
  }
  for (int j = 0; j < z.ny; ++j) {
    double eta = (double)j * K.dnym1;
    for (int i = 0; i < z.nx; ++i) {
      double xi = (double)i * K.dnxm1;
      exact_solution(xi, eta, 1.0e0, pb.ce, temp);
      for (int m = 0; m < 5; ++m) z.U(m, i, j, z.nz - 1) = temp[m];
    }
  }
}

// ---- exact_rhs (src/BT/exact_rhs.jl:5-370) --------------------------------
// ue/buf/cuf/q are line scratch over 0..n-1 (the reference's loop bound
// -2*(1-cell_start):cell_size+1-2*cell_end is 0..n-1 on one cell).
void exact_rhs(Problem& pb, Zone& z) {
  const Consts& K = pb.k;
  const int nmax = std::max(z.nx, std::max(z.ny, z.nz));
  std::vector<double> ue(nmax * 5), buf(nmax * 5), cuf(nmax), q(nmax);
  auto UE = [&](int p, int m) -> double& { return ue[p * 5 + m]; };
  auto BUF = [&](int p, int m) -> double& { return buf[p * 5 + m]; };
  double dtemp[5];
  std::fill(z.forcing.begin(), z.forcing.end(), 0.0e0);

  // xi-direction flux differences
  for (int k = 1; k <= z.nz - 2; ++k) {
    double zeta = (double)k * K.dnzm1;
    for (int j = 1; j <= z.ny - 2; ++j) {
      double eta = (double)j * K.dnym1;
      for (int i = 0; i <= z.nx - 1; ++i) {
        double xi = (double)i * K.dnxm1;
        exact_solution(xi, eta, zeta, pb.ce, dtemp);
        for (int m = 0; m < 5; ++m) UE(i, m) = dtemp[m];
        double dtpp = 1.0e0 / dtemp[0];
        for (int m = 1; m < 5; ++m) BUF(i, m) = dtpp * dtemp[m];
        cuf[i] = BUF(i, 1) * BUF(i, 1);
        BUF(i, 0) = cuf[i] + BUF(i, 2) * BUF(i, 2) + BUF(i, 3) * BUF(i, 3);
        q[i] = 0.5e0 * (BUF(i, 1) * UE(i, 1) + BUF(i, 2) * UE(i, 2) + BUF(i, 3) * UE(i, 3));
      }
      for (int i = 1; i <= z.nx - 2; ++i) {
        int im1 = i - 1, ip1 = i + 1;
        z.F(0, i, j, k) = z.F(0, i, j, k) - K.tx2 * (UE(ip1, 1) - UE(im1, 1)) +
                          K.dx1tx1 * (UE(ip1, 0) - 2.0e0 * UE(i, 0) + UE(im1, 0));
        z.F(1, i, j, k) = z.F(1, i, j, k) -
                          K.tx2 * ((UE(ip1, 1) * BUF(ip1, 1) + c2 * (UE(ip1, 4) - q[ip1])) -
                                   (UE(im1, 1) * BUF(im1, 1) + c2 * (UE(im1, 4) - q[im1]))) +
                          K.xxcon1 * (BUF(ip1, 1) - 2.0e0 * BUF(i, 1) + BUF(im1, 1)) +
                          K.dx2tx1 * (UE(ip1, 1) - 2.0e0 * UE(i, 1) + UE(im1, 1));
        z.F(2, i, j, k) = z.F(2, i, j, k) - K.tx2 * (UE(ip1, 2) * BUF(ip1, 1) - UE(im1, 2) * BUF(im1, 1)) +
                          K.xxcon2 * (BUF(ip1, 2) - 2.0e0 * BUF(i, 2) + BUF(im1, 2)) +
                          K.dx3tx1 * (UE(ip1, 2) - 2.0e0 * UE(i, 2) + UE(im1, 2));
        z.F(3, i, j, k) = z.F(3, i, j, k) - K.tx2 * (UE(ip1, 3) * BUF(ip1, 1) - UE(im1, 3) * BUF(im1, 1)) +
                          K.xxcon2 * (BUF(ip1, 3) - 2.0e0 * BUF(i, 3) + BUF(im1, 3)) +
                          K.dx4tx1 * (UE(ip1, 3) - 2.0e0 * UE(i, 3) + UE(im1, 3));
        z.F(4, i, j, k) = z.F(4, i, j, k) -
                          K.tx2 * (BUF(ip1, 1) * (c1 * UE(ip1, 4) - c2 * q[ip1]) -
                                   BUF(im1, 1) * (c1 * UE(im1, 4) - c2 * q[im1])) +
                          0.5e0 * K.xxcon3 * (BUF(ip1, 0) - 2.0e0 * BUF(i, 0) + BUF(im1, 0)) +
                          K.xxcon4 * (cuf[ip1] - 2.0e0 * cuf[i] + cuf[im1]) +
                          K.xxcon5 * (BUF(ip1, 4) - 2.0e0 * BUF(i, 4) + BUF(im1, 4)) +
                          K.dx5tx1 * (UE(ip1, 4) - 2.0e0 * UE(i, 4) + UE(im1, 4));
      }
      // fourth-order dissipation
      for (int m = 0; m < 5; ++m) {
        int i = 1;
        z.F(m, i, j, k) = z.F(m, i, j, k) - dssp * (5.0e0 * UE(i, m) - 4.0e0 * UE(i + 1, m) + UE(i + 2, m));
        i = 2;
        z.F(m, i, j, k) = z.F(m, i, j, k) -
                          dssp * (-4.0e0 * UE(i - 1, m) + 6.0e0 * UE(i, m) - 4.0e0 * UE(i + 1, m) + UE(i + 2, m));
      }
      for (int m = 0; m < 5; ++m)
        for (int i = 3; i <= z.nx - 4; ++i)
          z.F(m, i, j, k) = z.F(m, i, j, k) - dssp * (UE(i - 2, m) - 4.0e0 * UE(i - 1, m) + 6.0e0 * UE(i, m) -
                                                      4.0e0 * UE(i + 1, m) + UE(i + 2, m));
      for (int m = 0; m < 5; ++m) {
        int i = z.nx - 3;
        z.F(m, i, j, k) = z.F(m, i, j, k) -
                          dssp * (UE(i - 2, m) - 4.0e0 * UE(i - 1, m) + 6.0e0 * UE(i, m) - 4.0e0 * UE(i + 1, m));
        i = z.nx - 2;
        z.F(m, i, j, k) = z.F(m, i, j, k) - dssp * (UE(i - 2, m) - 4.0e0 * UE(i - 1, m) + 5.0e0 * UE(i, m));
      }
    }
  }

  // eta-direction flux differences
  for (int k = 1; k <= z.nz - 2; ++k) {
    double zeta = (double)k * K.dnzm1;
    for (int i = 1; i <= z.nx - 2; ++i) {
      double xi = (double)i * K.dnxm1;
      for (int j = 0; j <= z.ny - 1; ++j) {
        double eta = (double)j * K.dnym1;
        exact_solution(xi, eta, zeta, pb.ce, dtemp);
        for (int m = 0; m < 5; ++m) UE(j, m) = dtemp[m];
        double dtpp = 1.0e0 / dtemp[0];
        for (int m = 1; m < 5; ++m) BUF(j, m) = dtpp * dtemp[m];
        cuf[j] = BUF(j, 2) * BUF(j, 2);
        BUF(j, 0) = cuf[j] + BUF(j, 1) * BUF(j, 1) + BUF(j, 3) * BUF(j, 3);
        q[j] = 0.5e0 * (BUF(j, 1) * UE(j, 1) + BUF(j, 2) * UE(j, 2) + BUF(j, 3) * UE(j, 3));
      }
      for (int j = 1; j <= z.ny - 2; ++j) {
        int jm1 = j - 1, jp1 = j + 1;
        z.F(0, i, j, k) = z.F(0, i, j, k) - K.ty2 * (UE(jp1, 2) - UE(jm1, 2)) +
                          K.dy1ty1 * (UE(jp1, 0) - 2.0e0 * UE(j, 0) + UE(jm1, 0));
        z.F(1, i, j, k) = z.F(1, i, j, k) - K.ty2 * (UE(jp1, 1) * BUF(jp1, 2) - UE(jm1, 1) * BUF(jm1, 2)) +
                          K.yycon2 * (BUF(jp1, 1) - 2.0e0 * BUF(j, 1) + BUF(jm1, 1)) +
                          K.dy2ty1 * (UE(jp1, 1) - 2.0 * UE(j, 1) + UE(jm1, 1));
        z.F(2, i, j, k) = z.F(2, i, j, k) -
                          K.ty2 * ((UE(jp1, 2) * BUF(jp1, 2) + c2 * (UE(jp1, 4) - q[jp1])) -
                                   (UE(jm1, 2) * BUF(jm1, 2) + c2 * (UE(jm1, 4) - q[jm1]))) +
                          K.yycon1 * (BUF(jp1, 2) - 2.0e0 * BUF(j, 2) + BUF(jm1, 2)) +
                          K.dy3ty1 * (UE(jp1, 2) - 2.0e0 * UE(j, 2) + UE(jm1, 2));
        z.F(3, i, j, k) = z.F(3, i, j, k) - K.ty2 * (UE(jp1, 3) * BUF(jp1, 2) - UE(jm1, 3) * BUF(jm1, 2)) +
                          K.yycon2 * (BUF(jp1, 3) - 2.0e0 * BUF(j, 3) + BUF(jm1, 3)) +
                          K.dy4ty1 * (UE(jp1, 3) - 2.0e0 * UE(j, 3) + UE(jm1, 3));
        z.F(4, i, j, k) = z.F(4, i, j, k) -
                          K.ty2 * (BUF(jp1, 2) * (c1 * UE(jp1, 4) - c2 * q[jp1]) -
                                   BUF(jm1, 2) * (c1 * UE(jm1, 4) - c2 * q[jm1])) +
                          0.5e0 * K.yycon3 * (BUF(jp1, 0) - 2.0e0 * BUF(j, 0) + BUF(jm1, 0)) +
                          K.yycon4 * (cuf[jp1] - 2.0e0 * cuf[j] + cuf[jm1]) +
                          K.yycon5 * (BUF(jp1, 4) - 2.0e0 * BUF(j, 4) + BUF(jm1, 4)) +
                          K.dy5ty1 * (UE(jp1, 4) - 2.0e0 * UE(j, 4) + UE(jm1, 4));
      }
      for (int m = 0; m < 5; ++m) {
        int j = 1;
        z.F(m, i, j, k) = z.F(m, i, j, k) - dssp * (5.0e0 * UE(j, m) - 4.0e0 * UE(j + 1, m) + UE(j + 2, m));
        j = 2;
        z.F(m, i, j, k) = z.F(m, i, j, k) -
                          dssp * (-4.0e0 * UE(j - 1, m) + 6.0e0 * UE(j, m) - 4.0e0 * UE(j + 1, m) + UE(j + 2, m));
      }
      for (int m = 0; m < 5; ++m)
        for (int j = 3; j <= z.ny - 4; ++j)
          z.F(m, i, j, k) = z.F(m, i, j, k) - dssp * (UE(j - 2, m) - 4.0e0 * UE(j - 1, m) + 6.0e0 * UE(j, m) -
                                                      4.0e0 * UE(j + 1, m) + UE(j + 2, m));
      for (int m = 0; m < 5; ++m) {
        int j = z.ny - 3;
        z.F(m, i, j, k) = z.F(m, i, j, k) -
                          dssp * (UE(j - 2, m) - 4.0e0 * UE(j - 1, m) + 6.0e0 * UE(j, m) - 4.0e0 * UE(j + 1, m));
        j = z.ny - 2;
        z.F(m, i, j, k) = z.F(m, i, j, k) - dssp * (UE(j - 2, m) - 4.0e0 * UE(j - 1, m) + 5.0e0 * UE(j, m));
      }
    }
  }

  // zeta-direction flux differences
  for (int j = 1; j <= z.ny - 2; ++j) {
    double eta = (double)j * K.dnym1;
    for (int i = 1; i <= z.nx - 2; ++i) {
      double xi = (double)i * K.dnxm1;
      for (int k = 0; k <= z.nz - 1; ++k) {
        double zeta = (double)k * K.dnzm1;
        exact_solution(xi, eta, zeta, pb.ce, dtemp);
        for (int m = 0; m < 5; ++m) UE(k, m) = dtemp[m];
        double dtpp = 1.0e0 / dtemp[0];
        for (int m = 1; m < 5; ++m) BUF(k, m) = dtpp * dtemp[m];
        cuf[k] = BUF(k, 3) * BUF(k, 3);
        BUF(k, 0) = cuf[k] + BUF(k, 1) * BUF(k, 1) + BUF(k, 2) * BUF(k, 2);
        q[k] = 0.5e0 * (BUF(k, 1) * UE(k, 1) + BUF(k, 2) * UE(k, 2) + BUF(k, 3) * UE(k, 3));
      }
      for (int k = 1; k <= z.nz - 2; ++k) {
        int km1 = k - 1, kp1 = k + 1;
        z.F(0, i, j, k) = z.F(0, i, j, k) - K.tz2 * (UE(kp1, 3) - UE(km1, 3)) +
                          K.dz1tz1 * (UE(kp1, 0) - 2.0e0 * UE(k, 0) + UE(km1, 0));
        z.F(1, i, j, k) = z.F(1, i, j, k) - K.tz2 * (UE(kp1, 1) * BUF(kp1, 3) - UE(km1, 1) * BUF(km1, 3)) +
                          K.zzcon2 * (BUF(kp1, 1) - 2.0e0 * BUF(k, 1) + BUF(km1, 1)) +
                          K.dz2tz1 * (UE(kp1, 1) - 2.0e0 * UE(k, 1) + UE(km1, 1));
        z.F(2, i, j, k) = z.F(2, i, j, k) - K.tz2 * (UE(kp1, 2) * BUF(kp1, 3) - UE(km1, 2) * BUF(km1, 3)) +
                          K.zzcon2 * (BUF(kp1, 2) - 2.0e0 * BUF(k, 2) + BUF(km1, 2)) +
                          K.dz3tz1 * (UE(kp1, 2) - 2.0e0 * UE(k, 2) + UE(km1, 2));
        z.F(3, i, j, k) = z.F(3, i, j, k) -
                          K.tz2 * ((UE(kp1, 3) * BUF(kp1, 3) + c2 * (UE(kp1, 4) - q[kp1])) -
                                   (UE(km1, 3) * BUF(km1, 3) + c2 * (UE(km1, 4) - q[km1]))) +
                          K.zzcon1 * (BUF(kp1, 3) - 2.0e0 * BUF(k, 3) + BUF(km1, 3)) +
                          K.dz4tz1 * (UE(kp1, 3) - 2.0e0 * UE(k, 3) + UE(km1, 3));
        z.F(4, i, j, k) = z.F(4, i, j, k) -
                          K.tz2 * (BUF(kp1, 3) * (c1 * UE(kp1, 4) - c2 * q[kp1]) -
                                   BUF(km1, 3) * (c1 * UE(km1, 4) - c2 * q[km1])) +
                          0.5e0 * K.zzcon3 * (BUF(kp1, 0) - 2.0e0 * BUF(k, 0) + BUF(km1, 0)) +
                          K.zzcon4 * (cuf[kp1] - 2.0e0 * cuf[k] + cuf[km1]) +
                          K.zzcon5 * (BUF(kp1, 4) - 2.0e0 * BUF(k, 4) + BUF(km1, 4)) +
                          K.dz5tz1 * (UE(kp1, 4) - 2.0e0 * UE(k, 4) + UE(km1, 4));
      }
      for (int m = 0; m < 5; ++m) {
        int k = 1;
        z.F(m, i, j, k) = z.F(m, i, j, k) - dssp * (5.0e0 * UE(k, m) - 4.0e0 * UE(k + 1, m) + UE(k + 2, m));
        k = 2;
        z.F(m, i, j, k) = z.F(m, i, j, k) -
                          dssp * (-4.0e0 * UE(k - 1, m) + 6.0e0 * UE(k, m) - 4.0e0 * UE(k + 1, m) + UE(k + 2, m));
      }
      for (int m = 0; m < 5; ++m)
        for (int k = 3; k <= z.nz - 4; ++k)
          z.F(m, i, j, k) = z.F(m, i, j, k) - dssp * (UE(k - 2, m) - 4.0e0 * UE(k - 1, m) + 6.0e0 * UE(k, m) -
                                                      4.0e0 * UE(k + 1, m) + UE(k + 2, m));
      for (int m = 0; m < 5; ++m) {
        int k = z.nz - 3;
        z.F(m, i, j, k) = z.F(m, i, j, k) -
                          dssp * (UE(k - 2, m) - 4.0e0 * UE(k - 1, m) + 6.0e0 * UE(k, m) - 4.0e0 * UE(k + 1, m));
        k = z.nz - 2;
        z.F(m, i, j, k) = z.F(m, i, j, k) - dssp * (UE(k - 2, m) - 4.0e0 * UE(k - 1, m) + 5.0e0 * UE(k, m));
      }
    }
  }

  for (int k = 1; k <= z.nz - 2; ++k)
    for (int j = 1; j <= z.ny - 2; ++j)
      for (int i = 1; i <= z.nx - 2; ++i)
        for (int m = 0; m < 5; ++m) z.F(m, i, j, k) = -1.0e0 * z.F(m, i, j, k);
}

// ---- exch_qbc (src/BT/exchange_qbc.jl:145-465, one cluster, one rank) -----
// ghost i=0 <- west's i=nx_w-2; ghost i=nx-1 <- east's i=1;
// ghost j=0 <- south's j=ny_s-2; ghost j=ny-1 <- north's j=1;
// only the interior range of the other two indices, all 5 variables.
void exch_qbc(Problem& pb) {
  const int nzn = pb.nzones;
  // All sends are packed before any receive is unpacked (MPI semantics), so
  // snapshot every source plane first.
  std::vector<std::vector<real>> west_src(nzn), east_src(nzn), south_src(nzn), north_src(nzn);
  for (int zi = 0; zi < nzn; ++zi) {
    Zone& z = pb.zones[zi];
    // plane sent to the east neighbour (its west ghost): i = nx-2
    for (int m = 0; m < 5; ++m)
      for (int k = 1; k <= z.nz - 2; ++k)
        for (int j = 1; j <= z.ny - 2; ++j) east_src[zi].push_back(z.U(m, z.nx - 2, j, k));
    for (int m = 0; m < 5; ++m)
      for (int k = 1; k <= z.nz - 2; ++k)
        for (int j = 1; j <= z.ny - 2; ++j) west_src[zi].push_back(z.U(m, 1, j, k));
    for (int m = 0; m < 5; ++m)
      for (int k = 1; k <= z.nz - 2; ++k)
        for (int i = 1; i <= z.nx - 2; ++i) north_src[zi].push_back(z.U(m, i, z.ny - 2, k));
    for (int m = 0; m < 5; ++m)
      for (int k = 1; k <= z.nz - 2; ++k)
        for (int i = 1; i <= z.nx - 2; ++i) south_src[zi].push_back(z.U(m, i, 1, k));
  }
  for (int zi = 0; zi < nzn; ++zi) {
    Zone& z = pb.zones[zi];
    int w = pb.nbr[4 * zi + 0], e = pb.nbr[4 * zi + 1], s = pb.nbr[4 * zi + 2], n = pb.nbr[4 * zi + 3];
    size_t p = 0;
    for (int m = 0; m < 5; ++m)
      for (int k = 1; k <= z.nz - 2; ++k)
        for (int j = 1; j <= z.ny - 2; ++j) z.U(m, 0, j, k) = east_src[w][p++];
    p = 0;
    for (int m = 0; m < 5; ++m)
      for (int k = 1; k <= z.nz - 2; ++k)
        for (int j = 1; j <= z.ny - 2; ++j) z.U(m, z.nx - 1, j, k) = west_src[e][p++];
    p = 0;
    for (int m = 0; m < 5; ++m)
      for (int k = 1; k <= z.nz - 2; ++k)
        for (int i = 1; i <= z.nx - 2; ++i) z.U(m, i, 0, k) = north_src[s][p++];
    p = 0;
    for (int m = 0; m < 5; ++m)
      for (int k = 1; k <= z.nz - 2; ++k)
        for (int i = 1; i <= z.nx - 2; ++i) z.U(m, i, z.ny - 1, k) = south_src[n][p++];
  }
}

// ---- compute_rhs (src/BT/rhs.jl:4-460; SP src/SP/rhs.jl:3-452) --------------
void compute_rhs(Problem& pb, Zone& z) {
  const Consts& K = pb.k;
  const int nx = z.nx, ny = z.ny, nz = z.nz;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        size_t p = z.P(i, j, k);
        real rho_inv = 1.0e0 / z.U(0, i, j, k);
        z.rho_i[p] = rho_inv;
        z.us[p] = z.U(1, i, j, k) * rho_inv;
        z.vs[p] = z.U(2, i, j, k) * rho_inv;
        z.ws[p] = z.U(3, i, j, k) * rho_inv;
        z.square[p] = 0.5e0 * (z.U(1, i, j, k) * z.U(1, i, j, k) + z.U(2, i, j, k) * z.U(2, i, j, k) +
                               z.U(3, i, j, k) * z.U(3, i, j, k)) * rho_inv;
        z.qs[p] = z.square[p] * rho_inv;
        if (pb.kind == KIND_SP) {
          using std::sqrt;
          real aux = c1c2 * rho_inv * (z.U(4, i, j, k) - z.square[p]);
          aux = sqrt(aux);
          z.speed[p] = aux;
          z.ainv[p] = 1.0e0 / aux;
        }
      }
  z.rhs = z.forcing;
  auto& u = z;
  auto us = [&](int i, int j, int k) { return z.us[z.P(i, j, k)]; };
  auto vs = [&](int i, int j, int k) { return z.vs[z.P(i, j, k)]; };
  auto ws = [&](int i, int j, int k) { return z.ws[z.P(i, j, k)]; };
  auto qs = [&](int i, int j, int k) { return z.qs[z.P(i, j, k)]; };
  auto sq = [&](int i, int j, int k) { return z.square[z.P(i, j, k)]; };
  auto ri = [&](int i, int j, int k) { return z.rho_i[z.P(i, j, k)]; };

  // xi-direction fluxes
  for (int k = 1; k <= nz - 2; ++k)
    for (int j = 1; j <= ny - 2; ++j)
      for (int i = 1; i <= nx - 2; ++i) {
        real uijk = us(i, j, k), up1 = us(i + 1, j, k), um1 = us(i - 1, j, k);
        z.R(0, i, j, k) += K.dx1tx1 * (u.U(0, i + 1, j, k) - 2.0e0 * u.U(0, i, j, k) + u.U(0, i - 1, j, k)) -
                           K.tx2 * (u.U(1, i + 1, j, k) - u.U(1, i - 1, j, k));
        z.R(1, i, j, k) += K.dx2tx1 * (u.U(1, i + 1, j, k) - 2.0e0 * u.U(1, i, j, k) + u.U(1, i - 1, j, k)) +
                           K.xxcon2 * con43 * (up1 - 2.0e0 * uijk + um1) -
                           K.tx2 * (u.U(1, i + 1, j, k) * up1 - u.U(1, i - 1, j, k) * um1 +
                                    (u.U(4, i + 1, j, k) - sq(i + 1, j, k) - u.U(4, i - 1, j, k) + sq(i - 1, j, k)) * c2);
        z.R(2, i, j, k) += K.dx3tx1 * (u.U(2, i + 1, j, k) - 2.0e0 * u.U(2, i, j, k) + u.U(2, i - 1, j, k)) +
                           K.xxcon2 * (vs(i + 1, j, k) - 2.0e0 * vs(i, j, k) + vs(i - 1, j, k)) -
                           K.tx2 * (u.U(2, i + 1, j, k) * up1 - u.U(2, i - 1, j, k) * um1);
        z.R(3, i, j, k) += K.dx4tx1 * (u.U(3, i + 1, j, k) - 2.0e0 * u.U(3, i, j, k) + u.U(3, i - 1, j, k)) +
                           K.xxcon2 * (ws(i + 1, j, k) - 2.0e0 * ws(i, j, k) + ws(i - 1, j, k)) -
                           K.tx2 * (u.U(3, i + 1, j, k) * up1 - u.U(3, i - 1, j, k) * um1);
        z.R(4, i, j, k) += K.dx5tx1 * (u.U(4, i + 1, j, k) - 2.0e0 * u.U(4, i, j, k) + u.U(4, i - 1, j, k)) +
                           K.xxcon3 * (qs(i + 1, j, k) - 2.0e0 * qs(i, j, k) + qs(i - 1, j, k)) +
                           K.xxcon4 * (up1 * up1 - 2.0e0 * uijk * uijk + um1 * um1) +
                           K.xxcon5 * (u.U(4, i + 1, j, k) * ri(i + 1, j, k) - 2.0e0 * u.U(4, i, j, k) * ri(i, j, k) +
                                       u.U(4, i - 1, j, k) * ri(i - 1, j, k)) -
                           K.tx2 * ((c1 * u.U(4, i + 1, j, k) - c2 * sq(i + 1, j, k)) * up1 -
                                    (c1 * u.U(4, i - 1, j, k) - c2 * sq(i - 1, j, k)) * um1);
      }
  // xi-direction fourth-order dissipation
  for (int k = 1; k <= nz - 2; ++k)
    for (int j = 1; j <= ny - 2; ++j) {
      int i = 1;
      for (int m = 0; m < 5; ++m)
        z.R(m, i, j, k) -= dssp * (5.0e0 * u.U(m, i, j, k) - 4.0e0 * u.U(m, i + 1, j, k) + u.U(m, i + 2, j, k));
      i = 2;
      for (int m = 0; m < 5; ++m)
        z.R(m, i, j, k) -= dssp * (-4.0e0 * u.U(m, i - 1, j, k) + 6.0e0 * u.U(m, i, j, k) -
                                   4.0e0 * u.U(m, i + 1, j, k) + u.U(m, i + 2, j, k));
    }
  for (int k = 1; k <= nz - 2; ++k)
    for (int j = 1; j <= ny - 2; ++j)
      for (int i = 3; i <= nx - 4; ++i)
        for (int m = 0; m < 5; ++m)
          z.R(m, i, j, k) -= dssp * (u.U(m, i - 2, j, k) - 4.0e0 * u.U(m, i - 1, j, k) + 6.0 * u.U(m, i, j, k) -
                                     4.0e0 * u.U(m, i + 1, j, k) + u.U(m, i + 2, j, k));
  for (int k = 1; k <= nz - 2; ++k)
    for (int j = 1; j <= ny - 2; ++j) {
      int i = nx - 3;
      for (int m = 0; m < 5; ++m)
        z.R(m, i, j, k) -= dssp * (u.U(m, i - 2, j, k) - 4.0e0 * u.U(m, i - 1, j, k) + 6.0e0 * u.U(m, i, j, k) -
                                   4.0e0 * u.U(m, i + 1, j, k));
      i = nx - 2;
      for (int m = 0; m < 5; ++m)
        z.R(m, i, j, k) -= dssp * (u.U(m, i - 2, j, k) - 4.0e0 * u.U(m, i - 1, j, k) + 5.0e0 * u.U(m, i, j, k));
    }

  // eta-direction fluxes
  for (int k = 1; k <= nz - 2; ++k)
    for (int j = 1; j <= ny - 2; ++j)
      for (int i = 1; i <= nx - 2; ++i) {
        real vijk = vs(i, j, k), vp1 = vs(i, j + 1, k), vm1 = vs(i, j - 1, k);
        z.R(0, i, j, k) += K.dy1ty1 * (u.U(0, i, j + 1, k) - 2.0e0 * u.U(0, i, j, k) + u.U(0, i, j - 1, k)) -
                           K.ty2 * (u.U(2, i, j + 1, k) - u.U(2, i, j - 1, k));
        z.R(1, i, j, k) += K.dy2ty1 * (u.U(1, i, j + 1, k) - 2.0e0 * u.U(1, i, j, k) + u.U(1, i, j - 1, k)) +
                           K.yycon2 * (us(i, j + 1, k) - 2.0e0 * us(i, j, k) + us(i, j - 1, k)) -
                           K.ty2 * (u.U(1, i, j + 1, k) * vp1 - u.U(1, i, j - 1, k) * vm1);
        z.R(2, i, j, k) += K.dy3ty1 * (u.U(2, i, j + 1, k) - 2.0e0 * u.U(2, i, j, k) + u.U(2, i, j - 1, k)) +
                           K.yycon2 * con43 * (vp1 - 2.0e0 * vijk + vm1) -
                           K.ty2 * (u.U(2, i, j + 1, k) * vp1 - u.U(2, i, j - 1, k) * vm1 +
                                    (u.U(4, i, j + 1, k) - sq(i, j + 1, k) - u.U(4, i, j - 1, k) + sq(i, j - 1, k)) * c2);
        z.R(3, i, j, k) += K.dy4ty1 * (u.U(3, i, j + 1, k) - 2.0e0 * u.U(3, i, j, k) + u.U(3, i, j - 1, k)) +
                           K.yycon2 * (ws(i, j + 1, k) - 2.0e0 * ws(i, j, k) + ws(i, j - 1, k)) -
                           K.ty2 * (u.U(3, i, j + 1, k) * vp1 - u.U(3, i, j - 1, k) * vm1);
        z.R(4, i, j, k) += K.dy5ty1 * (u.U(4, i, j + 1, k) - 2.0e0 * u.U(4, i, j, k) + u.U(4, i, j - 1, k)) +
                           K.yycon3 * (qs(i, j + 1, k) - 2.0e0 * qs(i, j, k) + qs(i, j - 1, k)) +
                           K.yycon4 * (vp1 * vp1 - 2.0e0 * vijk * vijk + vm1 * vm1) +
                           K.yycon5 * (u.U(4, i, j + 1, k) * ri(i, j + 1, k) - 2.0e0 * u.U(4, i, j, k) * ri(i, j, k) +
                                       u.U(4, i, j - 1, k) * ri(i, j - 1, k)) -
                           K.ty2 * ((c1 * u.U(4, i, j + 1, k) - c2 * sq(i, j + 1, k)) * vp1 -
                                    (c1 * u.U(4, i, j - 1, k) - c2 * sq(i, j - 1, k)) * vm1);
      }
  for (int k = 1; k <= nz - 2; ++k) {
    int j = 1;
    for (int i = 1; i <= nx - 2; ++i)
      for (int m = 0; m < 5; ++m)
        z.R(m, i, j, k) -= dssp * (5.0e0 * u.U(m, i, j, k) - 4.0e0 * u.U(m, i, j + 1, k) + u.U(m, i, j + 2, k));
    j = 2;
    for (int i = 1; i <= nx - 2; ++i)
      for (int m = 0; m < 5; ++m)
        z.R(m, i, j, k) -= dssp * (-4.0e0 * u.U(m, i, j - 1, k) + 6.0e0 * u.U(m, i, j, k) -
                                   4.0e0 * u.U(m, i, j + 1, k) + u.U(m, i, j + 2, k));
  }
  for (int k = 1; k <= nz - 2; ++k)
    for (int j = 3; j <= ny - 4; ++j)
      for (int i = 1; i <= nx - 2; ++i)
        for (int m = 0; m < 5; ++m)
          z.R(m, i, j, k) -= dssp * (u.U(m, i, j - 2, k) - 4.0e0 * u.U(m, i, j - 1, k) + 6.0 * u.U(m, i, j, k) -
                                     4.0e0 * u.U(m, i, j + 1, k) + u.U(m, i, j + 2, k));
  for (int k = 1; k <= nz - 2; ++k) {
    int j = ny - 3;
    for (int i = 1; i <= nx - 2; ++i)
      for (int m = 0; m < 5; ++m)
        z.R(m, i, j, k) -= dssp * (u.U(m, i, j - 2, k) - 4.0e0 * u.U(m, i, j - 1, k) + 6.0e0 * u.U(m, i, j, k) -
                                   4.0e0 * u.U(m, i, j + 1, k));
    j = ny - 2;
    for (int i = 1; i <= nx - 2; ++i)
      for (int m = 0; m < 5; ++m)
        z.R(m, i, j, k) -= dssp * (u.U(m, i, j - 2, k) - 4.0e0 * u.U(m, i, j - 1, k) + 5.0e0 * u.U(m, i, j, k));
  }

  // zeta-direction fluxes
  for (int k = 1; k <= nz - 2; ++k)
    for (int j = 1; j <= ny - 2; ++j)
      for (int i = 1; i <= nx - 2; ++i) {
        real wijk = ws(i, j, k), wp1 = ws(i, j, k + 1), wm1 = ws(i, j, k - 1);
        z.R(0, i, j, k) += K.dz1tz1 * (u.U(0, i, j, k + 1) - 2.0e0 * u.U(0, i, j, k) + u.U(0, i, j, k - 1)) -
                           K.tz2 * (u.U(3, i, j, k + 1) - u.U(3, i, j, k - 1));
        z.R(1, i, j, k) += K.dz2tz1 * (u.U(1, i, j, k + 1) - 2.0e0 * u.U(1, i, j, k) + u.U(1, i, j, k - 1)) +
                           K.zzcon2 * (us(i, j, k + 1) - 2.0e0 * us(i, j, k) + us(i, j, k - 1)) -
                           K.tz2 * (u.U(1, i, j, k + 1) * wp1 - u.U(1, i, j, k - 1) * wm1);
        z.R(2, i, j, k) += K.dz3tz1 * (u.U(2, i, j, k + 1) - 2.0e0 * u.U(2, i, j, k) + u.U(2, i, j, k - 1)) +
                           K.zzcon2 * (vs(i, j, k + 1) - 2.0e0 * vs(i, j, k) + vs(i, j, k - 1)) -
                           K.tz2 * (u.U(2, i, j, k + 1) * wp1 - u.U(2, i, j, k - 1) * wm1);
        z.R(3, i, j, k) += K.dz4tz1 * (u.U(3, i, j, k + 1) - 2.0e0 * u.U(3, i, j, k) + u.U(3, i, j, k - 1)) +
                           K.zzcon2 * con43 * (wp1 - 2.0e0 * wijk + wm1) -
                           K.tz2 * (u.U(3, i, j, k + 1) * wp1 - u.U(3, i, j, k - 1) * wm1 +
                                    (u.U(4, i, j, k + 1) - sq(i, j, k + 1) - u.U(4, i, j, k - 1) + sq(i, j, k - 1)) * c2);
        z.R(4, i, j, k) += K.dz5tz1 * (u.U(4, i, j, k + 1) - 2.0e0 * u.U(4, i, j, k) + u.U(4, i, j, k - 1)) +
                           K.zzcon3 * (qs(i, j, k + 1) - 2.0e0 * qs(i, j, k) + qs(i, j, k - 1)) +
                           K.zzcon4 * (wp1 * wp1 - 2.0e0 * wijk * wijk + wm1 * wm1) +
                           K.zzcon5 * (u.U(4, i, j, k + 1) * ri(i, j, k + 1) - 2.0e0 * u.U(4, i, j, k) * ri(i, j, k) +
                                       u.U(4, i, j, k - 1) * ri(i, j, k - 1)) -
                           K.tz2 * ((c1 * u.U(4, i, j, k + 1) - c2 * sq(i, j, k + 1)) * wp1 -
                                    (c1 * u.U(4, i, j, k - 1) - c2 * sq(i, j, k - 1)) * wm1);
      }
  {
    int k = 1;
    for (int j = 1; j <= ny - 2; ++j)
      for (int i = 1; i <= nx - 2; ++i)
        for (int m = 0; m < 5; ++m)
          z.R(m, i, j, k) -= dssp * (5.0e0 * u.U(m, i, j, k) - 4.0e0 * u.U(m, i, j, k + 1) + u.U(m, i, j, k + 2));
    k = 2;
    for (int j = 1; j <= ny - 2; ++j)
      for (int i = 1; i <= nx - 2; ++i)
        for (int m = 0; m < 5; ++m)
          z.R(m, i, j, k) -= dssp * (-4.0e0 * u.U(m, i, j, k - 1) + 6.0e0 * u.U(m, i, j, k) -
                                     4.0e0 * u.U(m, i, j, k + 1) + u.U(m, i, j, k + 2));
  }
  for (int k = 3; k <= nz - 4; ++k)
    for (int j = 1; j <= ny - 2; ++j)
      for (int i = 1; i <= nx - 2; ++i)
        for (int m = 0; m < 5; ++m)
          z.R(m, i, j, k) -= dssp * (u.U(m, i, j, k - 2) - 4.0e0 * u.U(m, i, j, k - 1) + 6.0 * u.U(m, i, j, k) -
                                     4.0e0 * u.U(m, i, j, k + 1) + u.U(m, i, j, k + 2));
  {
    int k = nz - 3;
    for (int j = 1; j <= ny - 2; ++j)
      for (int i = 1; i <= nx - 2; ++i)
        for (int m = 0; m < 5; ++m)
          z.R(m, i, j, k) -= dssp * (u.U(m, i, j, k - 2) - 4.0e0 * u.U(m, i, j, k - 1) + 6.0e0 * u.U(m, i, j, k) -
                                     4.0e0 * u.U(m, i, j, k + 1));
    k = nz - 2;
    for (int j = 1; j <= ny - 2; ++j)
      for (int i = 1; i <= nx - 2; ++i)
        for (int m = 0; m < 5; ++m)
          z.R(m, i, j, k) -= dssp * (u.U(m, i, j, k - 2) - 4.0e0 * u.U(m, i, j, k - 1) + 5.0e0 * u.U(m, i, j, k));
  }
  for (int k = 1; k <= nz - 2; ++k)
    for (int j = 1; j <= ny - 2; ++j)
      for (int i = 1; i <= nx - 2; ++i)
        for (int m = 0; m < 5; ++m) z.R(m, i, j, k) *= K.dt;
}

// ======================= BT block-tridiagonal solves =========================
// Flux (fjac) and viscous (njac) Jacobians per sweep direction,
// src/BT/x_solve.jl:536-609, src/BT/y_solve.jl:543-613, src/BT/z_solve.jl:537-618.
// tmp1 is 1/rho (x: rho_i from compute_rhs; y,z: 1/u1 recomputed, the same value).
template <class T>
void jacobians(int dir, T tmp1, T u2, T u3, T u4, T u5, T q, T f[5][5], T n[5][5]) {
  const T C1 = (T)c1, C2 = (T)c2, C3C4 = (T)c3c4, C1345 = (T)c1345, CON43 = (T)con43;
  const T C3 = (T)c3, C4 = (T)c4;
  T tmp2 = tmp1 * tmp1;
  T tmp3 = tmp1 * tmp2;
  for (int a = 0; a < 5; ++a)
    for (int b = 0; b < 5; ++b) { f[a][b] = (T)0; n[a][b] = (T)0; }
  if (dir == 0) {
    f[0][1] = (T)1;
    f[1][0] = -(u2 * tmp2 * u2) + C2 * q;
    f[1][1] = ((T)2 - C2) * (u2 * tmp1);
    f[1][2] = -C2 * (u3 * tmp1);
    f[1][3] = -C2 * (u4 * tmp1);
    f[1][4] = C2;
    f[2][0] = -(u2 * u3) * tmp2;
    f[2][1] = u3 * tmp1;
    f[2][2] = u2 * tmp1;
    f[3][0] = -(u2 * u4) * tmp2;
    f[3][1] = u4 * tmp1;
    f[3][3] = u2 * tmp1;
    f[4][0] = (C2 * (T)2 * q - C1 * (u5 * tmp1)) * (u2 * tmp1);
    f[4][1] = C1 * u5 * tmp1 - C2 * (u2 * u2 * tmp2 + q);
    f[4][2] = -C2 * (u3 * u2) * tmp2;
    f[4][3] = -C2 * (u4 * u2) * tmp2;
    f[4][4] = C1 * (u2 * tmp1);
    n[1][0] = -CON43 * C3C4 * tmp2 * u2;
    n[1][1] = CON43 * C3C4 * tmp1;
    n[2][0] = -C3C4 * tmp2 * u3;
    n[2][2] = C3C4 * tmp1;
    n[3][0] = -C3C4 * tmp2 * u4;
    n[3][3] = C3C4 * tmp1;
    n[4][0] = -(CON43 * C3C4 - C1345) * tmp3 * (u2 * u2) - (C3C4 - C1345) * tmp3 * (u3 * u3) -
              (C3C4 - C1345) * tmp3 * (u4 * u4) - C1345 * tmp2 * u5;
    n[4][1] = (CON43 * C3C4 - C1345) * tmp2 * u2;
    n[4][2] = (C3C4 - C1345) * tmp2 * u3;
    n[4][3] = (C3C4 - C1345) * tmp2 * u4;
    n[4][4] = (C1345) * tmp1;
  } else if (dir == 1) {
    f[0][2] = (T)1;
    f[1][0] = -(u2 * u3) * tmp2;
    f[1][1] = u3 * tmp1;
    f[1][2] = u2 * tmp1;
    f[2][0] = -(u3 * u3 * tmp2) + C2 * q;
    f[2][1] = -C2 * u2 * tmp1;
    f[2][2] = ((T)2 - C2) * u3 * tmp1;
    f[2][3] = -C2 * u4 * tmp1;
    f[2][4] = C2;
    f[3][0] = -(u3 * u4) * tmp2;
    f[3][2] = u4 * tmp1;
    f[3][3] = u3 * tmp1;
    f[4][0] = (C2 * (T)2 * q - C1 * u5 * tmp1) * u3 * tmp1;
    f[4][1] = -C2 * u2 * u3 * tmp2;
    f[4][2] = C1 * u5 * tmp1 - C2 * (q + u3 * u3 * tmp2);
    f[4][3] = -C2 * (u3 * u4) * tmp2;
    f[4][4] = C1 * u3 * tmp1;
    n[1][0] = -C3C4 * tmp2 * u2;
    n[1][1] = C3C4 * tmp1;
    n[2][0] = -CON43 * C3C4 * tmp2 * u3;
    n[2][2] = CON43 * C3C4 * tmp1;
    n[3][0] = -C3C4 * tmp2 * u4;
    n[3][3] = C3C4 * tmp1;
    n[4][0] = -(C3C4 - C1345) * tmp3 * (u2 * u2) - (CON43 * C3C4 - C1345) * tmp3 * (u3 * u3) -
              (C3C4 - C1345) * tmp3 * (u4 * u4) - C1345 * tmp2 * u5;
    n[4][1] = (C3C4 - C1345) * tmp2 * u2;
    n[4][2] = (CON43 * C3C4 - C1345) * tmp2 * u3;
    n[4][3] = (C3C4 - C1345) * tmp2 * u4;
    n[4][4] = (C1345) * tmp1;
  } else {
    f[0][3] = (T)1;
    f[1][0] = -(u2 * u4) * tmp2;
    f[1][1] = u4 * tmp1;
    f[1][3] = u2 * tmp1;
    f[2][0] = -(u3 * u4) * tmp2;
    f[2][2] = u4 * tmp1;
    f[2][3] = u3 * tmp1;
    f[3][0] = -(u4 * u4 * tmp2) + C2 * q;
    f[3][1] = -C2 * u2 * tmp1;
    f[3][2] = -C2 * u3 * tmp1;
    f[3][3] = ((T)2 - C2) * u4 * tmp1;
    f[3][4] = C2;
    f[4][0] = (C2 * (T)2 * q - C1 * (u5 * tmp1)) * (u4 * tmp1);
    f[4][1] = -C2 * (u2 * u4) * tmp2;
    f[4][2] = -C2 * (u3 * u4) * tmp2;
    f[4][3] = C1 * (u5 * tmp1) - C2 * (q + u4 * u4 * tmp2);
    f[4][4] = C1 * u4 * tmp1;
    n[1][0] = -C3C4 * tmp2 * u2;
    n[1][1] = C3C4 * tmp1;
    n[2][0] = -C3C4 * tmp2 * u3;
    n[2][2] = C3C4 * tmp1;
    n[3][0] = -CON43 * C3C4 * tmp2 * u4;
    n[3][3] = CON43 * C3 * C4 * tmp1;
    n[4][0] = -(C3C4 - C1345) * tmp3 * (u2 * u2) - (C3C4 - C1345) * tmp3 * (u3 * u3) -
              (CON43 * C3C4 - C1345) * tmp3 * (u4 * u4) - C1345 * tmp2 * u5;
    n[4][1] = (C3C4 - C1345) * tmp2 * u2;
    n[4][2] = (C3C4 - C1345) * tmp2 * u3;
    n[4][3] = (CON43 * C3C4 - C1345) * tmp2 * u4;
    n[4][4] = (C1345) * tmp1;
  }
}

// binvcrhs: Gauss-Jordan on B without pivoting, applied to C and r
// (src/BT/solve_subs.jl:468-723).  For pivot p: scale row p of B (columns
// after p), of C and r; then for each other row q in increasing order:
// coeff = B[q][p]; B[q][p+1..] -= coeff*B[p][p+1..]; C[q][:] -= coeff*C[p][:];
// r[q] -= coeff*r[p].
template <class T>
void binvcrhs(T B[5][5], T C[5][5], T r[5]) {
  for (int p = 0; p < 5; ++p) {
    T pivot = (T)1 / B[p][p];
    for (int c = p + 1; c < 5; ++c) B[p][c] *= pivot;
    for (int c = 0; c < 5; ++c) C[p][c] *= pivot;
    r[p] *= pivot;
    for (int q = 0; q < 5; ++q) {
      if (q == p) continue;
      T coeff = B[q][p];
      for (int c = p + 1; c < 5; ++c) B[q][c] -= coeff * B[p][c];
      for (int c = 0; c < 5; ++c) C[q][c] -= coeff * C[p][c];
      r[q] -= coeff * r[p];
    }
  }
}

// binvrhs: the same elimination without C (src/BT/solve_subs.jl:730-862).
template <class T>
void binvrhs(T B[5][5], T r[5]) {
  for (int p = 0; p < 5; ++p) {
    T pivot = (T)1 / B[p][p];
    for (int c = p + 1; c < 5; ++c) B[p][c] *= pivot;
    r[p] *= pivot;
    for (int q = 0; q < 5; ++q) {
      if (q == p) continue;
      T coeff = B[q][p];
      for (int c = p + 1; c < 5; ++c) B[q][c] -= coeff * B[p][c];
      r[q] -= coeff * r[p];
    }
  }
}

// matvec_sub: b -= A*v, the row sum formed first (src/BT/solve_subs.jl:4-37).
template <class T>
void matvec_sub(const T A[5][5], const T v[5], T b[5]) {
  for (int m = 0; m < 5; ++m)
    b[m] -= A[m][0] * v[0] + A[m][1] * v[1] + A[m][2] * v[2] + A[m][3] * v[3] + A[m][4] * v[4];
}

// matmul_sub2: C -= A*B, one term at a time (src/BT/solve_subs.jl:333-460).
template <class T>
void matmul_sub(const T A[5][5], const T B[5][5], T C[5][5]) {
  for (int n = 0; n < 5; ++n)
    for (int m = 0; m < 5; ++m)
      C[m][n] = C[m][n] - A[m][0] * B[0][n] - A[m][1] * B[1][n] - A[m][2] * B[2][n] - A[m][3] * B[3][n] -
                A[m][4] * B[4][n];
}

// One BT line of n points (0 and n-1 are boundary points).  ul/q/ri: state;
// rl: rhs (in/out).  Restates x_solve_cell + x_backsubstitute for one (j,k).
// dtt1 = dt*t?1, dtt2 = dt*t?2, dd[5] = d?1..d?5 of the direction.
template <class T>
void bt_line(int dir, int n, const real* ul, const real* ri, const real* q, real* rl, double dtt1,
             double dtt2, const double dd[5]) {
  // per-thread line scratch, reused across lines (no allocation per line)
  static thread_local std::vector<T> fj, nj, la, lb, lc, r;
  for (auto* v : {&fj, &nj, &la, &lb, &lc}) v->resize((size_t)n * 25);
  r.resize((size_t)n * 5);
  auto F = [&](int p) { return reinterpret_cast<T(*)[5]>(&fj[(size_t)p * 25]); };
  auto N = [&](int p) { return reinterpret_cast<T(*)[5]>(&nj[(size_t)p * 25]); };
  auto A = [&](int p) { return reinterpret_cast<T(*)[5]>(&la[(size_t)p * 25]); };
  auto B = [&](int p) { return reinterpret_cast<T(*)[5]>(&lb[(size_t)p * 25]); };
  auto C = [&](int p) { return reinterpret_cast<T(*)[5]>(&lc[(size_t)p * 25]); };
  for (int p = 0; p < n * 5; ++p) r[p] = (T)rl[p];
  // lhsabinit: A = 0, B = I; the persistent lhsc is zero at boundary points.
  for (int p = 0; p < n; ++p)
    for (int a = 0; a < 5; ++a)
      for (int b = 0; b < 5; ++b) {
        A(p)[a][b] = (T)0;
        B(p)[a][b] = (a == b) ? (T)1 : (T)0;
        C(p)[a][b] = (T)0;
      }
  for (int p = 0; p < n; ++p)
    jacobians<T>(dir, (T)ri[p], (T)ul[p * 5 + 1], (T)ul[p * 5 + 2], (T)ul[p * 5 + 3], (T)ul[p * 5 + 4], (T)q[p],
                 F(p), N(p));
  const T tmp1 = (T)dtt1, tmp2 = (T)dtt2;
  for (int p = 1; p <= n - 2; ++p) {
    for (int a = 0; a < 5; ++a)
      for (int b = 0; b < 5; ++b) {
        if (a == b) {
          A(p)[a][b] = -tmp2 * F(p - 1)[a][b] - tmp1 * N(p - 1)[a][b] - tmp1 * (T)dd[a];
          B(p)[a][b] = (T)1 + tmp1 * (T)2 * N(p)[a][b] + tmp1 * (T)2 * (T)dd[a];
          C(p)[a][b] = tmp2 * F(p + 1)[a][b] - tmp1 * N(p + 1)[a][b] - tmp1 * (T)dd[a];
        } else {
          A(p)[a][b] = -tmp2 * F(p - 1)[a][b] - tmp1 * N(p - 1)[a][b];
          B(p)[a][b] = tmp1 * (T)2 * N(p)[a][b];
          C(p)[a][b] = tmp2 * F(p + 1)[a][b] - tmp1 * N(p + 1)[a][b];
        }
      }
  }
  // forward elimination (FIRST = LAST = 1)
  binvcrhs<T>(B(0), C(0), &r[0]);
  for (int p = 1; p <= n - 2; ++p) {
    matvec_sub<T>(A(p), &r[(p - 1) * 5], &r[p * 5]);
    matmul_sub<T>(A(p), C(p - 1), B(p));
    binvcrhs<T>(B(p), C(p), &r[p * 5]);
  }
  {
    int p = n - 1;
    matvec_sub<T>(A(p), &r[(p - 1) * 5], &r[p * 5]);
    matmul_sub<T>(A(p), C(p - 1), B(p));
    binvrhs<T>(B(p), &r[p * 5]);
  }
  // back substitution (x_backsubstitute, LAST = 1)
  for (int p = n - 2; p >= 0; --p)
    for (int m = 0; m < 5; ++m)
      for (int c = 0; c < 5; ++c) r[p * 5 + m] -= C(p)[m][c] * r[(p + 1) * 5 + c];
  for (int p = 0; p < n * 5; ++p) rl[p] = (real)r[p];
}

template <class T>
void bt_sweep(Problem& pb, Zone& z, int dir) {
  const Consts& K = pb.k;
  int n = dir == 0 ? z.nx : (dir == 1 ? z.ny : z.nz);
  int na = dir == 0 ? z.ny : z.nx;           // first transverse index range
  int nb = dir == 2 ? z.ny : z.nz;           // second transverse index range
  double dd[5];
  double dtt1, dtt2;
  if (dir == 0) { dd[0] = dx1; dd[1] = dx2; dd[2] = dx3; dd[3] = dx4; dd[4] = dx5; dtt1 = K.dt * K.tx1; dtt2 = K.dt * K.tx2; }
  else if (dir == 1) { dd[0] = dy1; dd[1] = dy2; dd[2] = dy3; dd[3] = dy4; dd[4] = dy5; dtt1 = K.dt * K.ty1; dtt2 = K.dt * K.ty2; }
  else { dd[0] = dz1; dd[1] = dz2; dd[2] = dz3; dd[3] = dz4; dd[4] = dz5; dtt1 = K.dt * K.tz1; dtt2 = K.dt * K.tz2; }
  std::vector<real> ul(n * 5), ri(n), q(n), rl(n * 5);
  for (int b = 1; b <= nb - 2; ++b)
    for (int a = 1; a <= na - 2; ++a) {
      for (int p = 0; p < n; ++p) {
        int i = dir == 0 ? p : a, j = dir == 1 ? p : (dir == 0 ? a : b), k = dir == 2 ? p : b;
        size_t P = z.P(i, j, k);
        for (int m = 0; m < 5; ++m) { ul[p * 5 + m] = z.U(m, i, j, k); rl[p * 5 + m] = z.R(m, i, j, k); }
        ri[p] = dir == 0 ? z.rho_i[P] : 1.0e0 / z.U(0, i, j, k);
        q[p] = z.qs[P];
      }
      bt_line<T>(dir, n, ul.data(), ri.data(), q.data(), rl.data(), dtt1, dtt2, dd);
      for (int p = 0; p < n; ++p) {
        int i = dir == 0 ? p : a, j = dir == 1 ? p : (dir == 0 ? a : b), k = dir == 2 ? p : b;
        for (int m = 0; m < 5; ++m) z.R(m, i, j, k) = rl[p * 5 + m];
      }
    }
}

// ======================= SP scalar pentadiagonal solves ======================
// txinvr (src/SP/txinvr.jl:5-56)
void txinvr(Zone& z) {
  for (int k = 1; k <= z.nz - 2; ++k)
    for (int j = 1; j <= z.ny - 2; ++j)
      for (int i = 1; i <= z.nx - 2; ++i) {
        size_t P = z.P(i, j, k);
        real ru1 = z.rho_i[P], uu = z.us[P], vv = z.vs[P], ww = z.ws[P], ac = z.speed[P];
        real ac2inv = 1.0 / (ac * ac);
        real r1 = z.R(0, i, j, k), r2 = z.R(1, i, j, k), r3 = z.R(2, i, j, k), r4 = z.R(3, i, j, k),
               r5 = z.R(4, i, j, k);
        real t1 = c2 * ac2inv * (z.qs[P] * r1 - uu * r2 - vv * r3 - ww * r4 + r5);
        real t2 = bt_ * ru1 * (uu * r1 - r2);
        real t3 = (bt_ * ru1 * ac) * t1;
        z.R(0, i, j, k) = r1 - t1;
        z.R(1, i, j, k) = -ru1 * (ww * r1 - r4);
        z.R(2, i, j, k) = ru1 * (vv * r1 - r3);
        z.R(3, i, j, k) = -t2 + t3;
        z.R(4, i, j, k) = t2 + t3;
      }
}

// One SP line: lhs assembly (lhsx/lhsy/lhsz) + Thomas forward elimination +
// back substitution (src/SP/x_solve.jl:203-313,456-512).  Boundary rows 0 and
// n-1 are the identity rows lhsinit leaves there (src/SP/initialize.jl:235-256);
// the in-place updates the reference applies to them leave them unchanged.
template <class T>
void sp_line(int n, const real* rho_i, const real* cvel, const real* speed, real* rl, const Consts& K,
             int dir) {
  double dtt1, dtt2, c2dtt1, da, db, dmax_, dc;
  if (dir == 0) { dtt1 = K.dttx1; dtt2 = K.dttx2; c2dtt1 = K.c2dttx1; da = dx2; db = dx5; dmax_ = dxmax; dc = dx1; }
  else if (dir == 1) { dtt1 = K.dtty1; dtt2 = K.dtty2; c2dtt1 = K.c2dtty1; da = dy3; db = dy5; dmax_ = dymax; dc = dy1; }
  else { dtt1 = K.dttz1; dtt2 = K.dttz2; c2dtt1 = K.c2dttz1; da = dz4; db = dz5; dmax_ = dzmax; dc = dz1; }
  static thread_local std::vector<real> rhon, cv, L64;
  static thread_local std::vector<T> L, r;
  rhon.resize(n);
  cv.resize(n);
  L.resize((size_t)n * 15);
  r.resize((size_t)n * 5);
  auto l = [&](int p, int b) -> T& { return L[(size_t)p * 15 + b]; };  // b = 0..14 (bands 1..15)
  for (int p = 0; p < n * 5; ++p) r[p] = (T)rl[p];
  for (int p = 0; p < n; ++p)
    for (int b = 0; b < 15; ++b) l(p, b) = (b == 2 || b == 7 || b == 12) ? (T)1 : (T)0;
  for (int p = 0; p < n; ++p) {
    real ru1 = c3c4 * rho_i[p];
    cv[p] = cvel[p];
    rhon[p] = rmax(rmax(rmax(da + con43 * ru1, db + c1c5 * ru1), dmax_ + ru1), real(dc));
  }
  // lhs assembly is FP64 in the reference; it is converted to T afterwards.
  L64.assign((size_t)n * 5, real(0.0));
  auto l64 = [&](int p, int b) -> real& { return L64[(size_t)p * 5 + b]; };
  for (int p = 1; p <= n - 2; ++p) {
    l64(p, 0) = 0.0e0;
    l64(p, 1) = -dtt2 * cv[p - 1] - dtt1 * rhon[p - 1];
    l64(p, 2) = 1.0e0 + c2dtt1 * rhon[p];
    l64(p, 3) = dtt2 * cv[p + 1] - dtt1 * rhon[p + 1];
    l64(p, 4) = 0.0e0;
  }
  {
    int p = 1;
    l64(p, 2) += K.comz5; l64(p, 3) -= K.comz4; l64(p, 4) += K.comz1;
    l64(p + 1, 1) -= K.comz4; l64(p + 1, 2) += K.comz6; l64(p + 1, 3) -= K.comz4; l64(p + 1, 4) += K.comz1;
  }
  for (int p = 3; p <= n - 4; ++p) {
    l64(p, 0) += K.comz1; l64(p, 1) -= K.comz4; l64(p, 2) += K.comz6; l64(p, 3) -= K.comz4; l64(p, 4) += K.comz1;
  }
  {
    int p = n - 3;
    l64(p, 0) += K.comz1; l64(p, 1) -= K.comz4; l64(p, 2) += K.comz6; l64(p, 3) -= K.comz4;
    l64(p + 1, 0) += K.comz1; l64(p + 1, 1) -= K.comz4; l64(p + 1, 2) += K.comz5;
  }
  for (int p = 1; p <= n - 2; ++p) {
    real L1 = l64(p, 0), L2 = l64(p, 1), L3 = l64(p, 2), L4 = l64(p, 3), L5 = l64(p, 4);
    l(p, 0) = (T)L1; l(p, 1) = (T)L2; l(p, 2) = (T)L3; l(p, 3) = (T)L4; l(p, 4) = (T)L5;
    l(p, 5) = (T)L1;
    l(p, 6) = (T)(L2 - dtt2 * speed[p - 1]);
    l(p, 7) = (T)L3;
    l(p, 8) = (T)(L4 + dtt2 * speed[p + 1]);
    l(p, 9) = (T)L5;
    l(p, 10) = (T)L1;
    l(p, 11) = (T)(L2 + dtt2 * speed[p - 1]);
    l(p, 12) = (T)L3;
    l(p, 13) = (T)(L4 - dtt2 * speed[p + 1]);
    l(p, 14) = (T)L5;
  }
  // forward elimination: system n=0 shared by m = 1..3, then m = 4 (n=5), m = 5 (n=10)
  auto forward = [&](int nb, int m0, int m1) {
    for (int p = 0; p <= n - 3; ++p) {
      int p1 = p + 1, p2 = p + 2;
      T fac1 = (T)1 / l(p, nb + 2);
      l(p, nb + 3) *= fac1;
      l(p, nb + 4) *= fac1;
      for (int m = m0; m <= m1; ++m) r[p * 5 + m] *= fac1;
      l(p1, nb + 2) -= l(p1, nb + 1) * l(p, nb + 3);
      l(p1, nb + 3) -= l(p1, nb + 1) * l(p, nb + 4);
      for (int m = m0; m <= m1; ++m) r[p1 * 5 + m] -= l(p1, nb + 1) * r[p * 5 + m];
      l(p2, nb + 1) -= l(p2, nb + 0) * l(p, nb + 3);
      l(p2, nb + 2) -= l(p2, nb + 0) * l(p, nb + 4);
      for (int m = m0; m <= m1; ++m) r[p2 * 5 + m] -= l(p2, nb + 0) * r[p * 5 + m];
    }
    int p = n - 2, p1 = n - 1;
    T fac1 = (T)1 / l(p, nb + 2);
    l(p, nb + 3) *= fac1;
    l(p, nb + 4) *= fac1;
    for (int m = m0; m <= m1; ++m) r[p * 5 + m] *= fac1;
    l(p1, nb + 2) -= l(p1, nb + 1) * l(p, nb + 3);
    l(p1, nb + 3) -= l(p1, nb + 1) * l(p, nb + 4);
    for (int m = m0; m <= m1; ++m) r[p1 * 5 + m] -= l(p1, nb + 1) * r[p * 5 + m];
    T fac2 = (T)1 / l(p1, nb + 2);
    l(p1, nb + 3) *= fac2;
    l(p1, nb + 4) *= fac2;
    for (int m = m0; m <= m1; ++m) r[p1 * 5 + m] *= fac2;
  };
  forward(0, 0, 2);
  forward(5, 3, 3);
  forward(10, 4, 4);
  // back substitution
  for (int m = 0; m < 5; ++m) {
    int nb = m < 3 ? 0 : (m == 3 ? 5 : 10);
    int p = n - 2, p1 = n - 1;
    r[p * 5 + m] -= l(p, nb + 3) * r[p1 * 5 + m];
    for (p = n - 3; p >= 0; --p)
      r[p * 5 + m] -= l(p, nb + 3) * r[(p + 1) * 5 + m] + l(p, nb + 4) * r[(p + 2) * 5 + m];
  }
  for (int p = 0; p < n * 5; ++p) rl[p] = (real)r[p];
}

template <class T>
void sp_sweep(Problem& pb, Zone& z, int dir) {
  int n = dir == 0 ? z.nx : (dir == 1 ? z.ny : z.nz);
  int na = dir == 0 ? z.ny : z.nx;
  int nb = dir == 2 ? z.ny : z.nz;
  std::vector<real> ri(n), cvel(n), spd(n), rl(n * 5);
  for (int b = 1; b <= nb - 2; ++b)
    for (int a = 1; a <= na - 2; ++a) {
      for (int p = 0; p < n; ++p) {
        int i = dir == 0 ? p : a, j = dir == 1 ? p : (dir == 0 ? a : b), k = dir == 2 ? p : b;
        size_t P = z.P(i, j, k);
        ri[p] = z.rho_i[P];
        cvel[p] = dir == 0 ? z.us[P] : (dir == 1 ? z.vs[P] : z.ws[P]);
        spd[p] = z.speed[P];
        for (int m = 0; m < 5; ++m) rl[p * 5 + m] = z.R(m, i, j, k);
      }
      sp_line<T>(n, ri.data(), cvel.data(), spd.data(), rl.data(), pb.k, dir);
      for (int p = 0; p < n; ++p) {
        int i = dir == 0 ? p : a, j = dir == 1 ? p : (dir == 0 ? a : b), k = dir == 2 ? p : b;
        for (int m = 0; m < 5; ++m) z.R(m, i, j, k) = rl[p * 5 + m];
      }
    }
  // transforms after each sweep: ninvr (x), pinvr (y), tzetar (z)
  for (int k = 1; k <= z.nz - 2; ++k)
    for (int j = 1; j <= z.ny - 2; ++j)
      for (int i = 1; i <= z.nx - 2; ++i) {
        real r1 = z.R(0, i, j, k), r2 = z.R(1, i, j, k), r3 = z.R(2, i, j, k), r4 = z.R(3, i, j, k),
             r5 = z.R(4, i, j, k);
        if (dir == 0) {  // src/SP/ninvr.jl:19-32
          real t1 = bt_ * r3;
          real t2 = 0.5e0 * (r4 + r5);
          z.R(0, i, j, k) = -r2;
          z.R(1, i, j, k) = r1;
          z.R(2, i, j, k) = bt_ * (r4 - r5);
          z.R(3, i, j, k) = -t1 + t2;
          z.R(4, i, j, k) = t1 + t2;
        } else if (dir == 1) {  // src/SP/pinvr.jl:20-33
          real t1 = bt_ * r1;
          real t2 = 0.5e0 * (r4 + r5);
          z.R(0, i, j, k) = bt_ * (r4 - r5);
          z.R(1, i, j, k) = -r3;
          z.R(2, i, j, k) = r2;
          z.R(3, i, j, k) = -t1 + t2;
          z.R(4, i, j, k) = t1 + t2;
        } else {  // src/SP/tzetar.jl:27-52
          size_t P = z.P(i, j, k);
          real xvel = z.us[P], yvel = z.vs[P], zvel = z.ws[P], ac = z.speed[P], acinv = z.ainv[P];
          real ac2u = ac * ac;
          real uzik1 = z.U(0, i, j, k);
          real btuz = bt_ * uzik1;
          real t1 = btuz * acinv * (r4 + r5);
          real t2 = r3 + t1;
          real t3 = btuz * (r4 - r5);
          z.R(0, i, j, k) = t2;
          z.R(1, i, j, k) = -uzik1 * r2 + xvel * t2;
          z.R(2, i, j, k) = uzik1 * r1 + yvel * t2;
          z.R(3, i, j, k) = zvel * t2 + t3;
          z.R(4, i, j, k) = uzik1 * (-xvel * r2 + yvel * r1) + z.qs[P] * t2 + c2iv * ac2u * t1 + zvel * t3;
        }
      }
}


void add(Zone& z) {
  for (int k = 1; k <= z.nz - 2; ++k)
    for (int j = 1; j <= z.ny - 2; ++j)
      for (int i = 1; i <= z.nx - 2; ++i)
        for (int m = 0; m < 5; ++m) z.U(m, i, j, k) += z.R(m, i, j, k);
}

// error_norm (sum over all zone points) and rhs_norm (interior), per zone.
void zone_norms(Problem& pb, Zone& z, double xce[5], double xcr[5]);

// adi (src/BT/adi.jl:82-251, src/SP/adi.jl:85-258).  xcr (nullable) receives
// this zone's rhs_norm of the compute_rhs output, before any transform.
void adi(Problem& pb, Zone& z, double* xcr = nullptr) {
  compute_rhs(pb, z);
  if (xcr) {
    double xce_unused[5];
    zone_norms(pb, z, xce_unused, xcr);
  }
#if ORACLE_TANGENT
  if (pb.kind == KIND_BT) {
    for (int d = 0; d < 3; ++d) bt_sweep<real>(pb, z, d);
  } else {
    txinvr(z);
    for (int d = 0; d < 3; ++d) sp_sweep<real>(pb, z, d);
  }
#else
  if (pb.kind == KIND_BT) {
    for (int d = 0; d < 3; ++d) {
      if (pb.solve_float) bt_sweep<float>(pb, z, d); else bt_sweep<double>(pb, z, d);
    }
  } else {
    txinvr(z);
    for (int d = 0; d < 3; ++d) {
      if (pb.solve_float) sp_sweep<float>(pb, z, d); else sp_sweep<double>(pb, z, d);
    }
  }
#endif
  add(z);
}

// error_norm (sum over all zone points) and rhs_norm (interior), per zone;
// src/BT/error.jl:7-79.  Returns the per-zone values before the sqrt/scale so
// callers can combine them as verify does.
void zone_norms(Problem& pb, Zone& z, double xce[5], double xcr[5]) {
  const Consts& K = pb.k;
  double rms[5] = {0, 0, 0, 0, 0}, ue[5];
  for (int k = 0; k < z.nz; ++k) {
    double zeta = (double)k * K.dnzm1;
    for (int j = 0; j < z.ny; ++j) {
      double eta = (double)j * K.dnym1;
      for (int i = 0; i < z.nx; ++i) {
        double xi = (double)i * K.dnxm1;
        exact_solution(xi, eta, zeta, pb.ce, ue);
        for (int m = 0; m < 5; ++m) {
          double a = value(z.U(m, i, j, k)) - ue[m];
          rms[m] = rms[m] + a * a;
        }
      }
    }
  }
  double denom = (double)(z.nx - 2) * (double)(z.ny - 2) * (double)(z.nz - 2);
  for (int m = 0; m < 5; ++m) xce[m] = std::sqrt(rms[m] / denom);
  double rr[5] = {0, 0, 0, 0, 0};
  for (int k = 1; k <= z.nz - 2; ++k)
    for (int j = 1; j <= z.ny - 2; ++j)
      for (int i = 1; i <= z.nx - 2; ++i)
        for (int m = 0; m < 5; ++m) {
          double a = value(z.R(m, i, j, k));
          rr[m] = rr[m] + a * a;
        }
  for (int m = 0; m < 5; ++m) xcr[m] = std::sqrt(rr[m] / denom);
}

}  // namespace

#if !ORACLE_TANGENT
// =============================== C ABI ======================================
extern "C" {

struct oracle_t;

// Zone geometry, src/BT/zone_setup.jl:1-77 (SP: src/SP/zone_setup.jl, which
// stretches whenever ratio != 1).  Outputs per zone nx, ny, nz and the
// periodic neighbours (west, east, south, north), 0-based.
int oracle_zone_setup(int kind, int gx, int gy, int gz, int xz, int yz, double ratio, int* nx, int* ny, int* nz,
                      int* nbr) {
  std::vector<long> x_end(xz), y_end(yz), x_start(xz), y_start(yz), x_size(xz), y_size(yz);
  bool stretch = std::fabs(ratio - 1.0e0) > 1.0e-10 && (kind == KIND_SP || (xz > 1 && yz > 1));
  if (stretch) {
    double x_r = std::exp(std::log(ratio) / (xz - 1));
    double y_r = std::exp(std::log(ratio) / (yz - 1));
    double x_smallest = (double)gx * (x_r - 1.0e0) / (std::pow(x_r, xz) - 1.0e0);
    double y_smallest = (double)gy * (y_r - 1.0e0) / (std::pow(y_r, yz) - 1.0e0);
    for (int i = 1; i <= xz; ++i) x_end[i - 1] = (long)std::trunc(x_smallest * (std::pow(x_r, i) - 1.0e0) / (x_r - 1.0e0) + 0.45e0);
    for (int j = 1; j <= yz; ++j) y_end[j - 1] = (long)std::trunc(y_smallest * (std::pow(y_r, j) - 1.0e0) / (y_r - 1.0e0) + 0.45e0);
  } else {
    for (int i = 1; i <= xz; ++i) x_end[i - 1] = (long)((double)(i * gx) / (double)xz);
    for (int j = 1; j <= yz; ++j) y_end[j - 1] = (long)((double)(j * gy) / (double)yz);
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
  for (int j = 1; j <= yz; ++j)
    for (int i = 1; i <= xz; ++i) {
      int zn = (i - 1) + (j - 1) * xz;
      nx[zn] = (int)x_size[i - 1];
      ny[zn] = (int)y_size[j - 1];
      nz[zn] = gz;
      int id_west = (i - 2 + xz) % xz, id_east = i % xz;
      int jd_south = (j - 2 + yz) % yz, jd_north = j % yz;
      nbr[4 * zn + 0] = id_west + (j - 1) * xz;
      nbr[4 * zn + 1] = id_east + (j - 1) * xz;
      nbr[4 * zn + 2] = (i - 1) + jd_south * xz;
      nbr[4 * zn + 3] = (i - 1) + jd_north * xz;
    }
  return 0;
}

// Seeded manufactured-solution coefficients (the benchmark's initial data;
// the reference itself uses the fixed ce table of src/BT/set_constants.jl:47-51
// instead).  All 65 entries are drawn U(0.5, 2.0) from one SplitMix64 stream
// (ce row-major [5][13], one draw each in order: the 53 high bits of the word
// scaled to [0, 1)).  Then the energy row is doubled until, at every grid
// coordinate (xi, eta, zeta) = (i dnxm1, j dnym1, k dnzm1) of the largest zone
// extents, the exact solution, its six face values and their transfinite
// interpolation (the initialize formula above) all have rho > 0, rho E > 0
// and rho E - |rho v|^2 / (2 rho) >= rho E / 4.  Returns the number of
// doublings e (0..39) or -2 when none passes; the caller's ce is written in
// every case.
int oracle_seeded_coefficients(uint64_t seed, int nzones, const int* nx, const int* ny, const int* nz, int gx, int gy,
                               int gz, int xz, int yz, double* ce) {
  if (!nx || !ny || !nz || !ce || nzones < 1) return -1;
  uint64_t state = seed;
  for (int e = 0; e < 65; ++e) {
    state += 0x9E3779B97F4A7C15ull;
    uint64_t w = state;
    w = (w ^ (w >> 30)) * 0xBF58476D1CE4E5B9ull;
    w = (w ^ (w >> 27)) * 0x94D049BB133111EBull;
    w ^= w >> 31;
    ce[e] = 0.5 + 1.5 * ((double)(w >> 11) * 0x1.0p-53);
  }
  const Consts K = set_constants(1.0, gx, gy, gz, xz, yz);
  int ex = 0, ey = 0, ez = 0;
  for (int zi = 0; zi < nzones; ++zi) {
    ex = std::max(ex, nx[zi]);
    ey = std::max(ey, ny[zi]);
    ez = std::max(ez, nz[zi]);
  }
  auto admissible = [](const double* q) {
    if (!(q[0] > 0.0) || !(q[4] > 0.0)) return false;
    const double kinetic = 0.5 * (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]) / q[0];
    return q[4] - kinetic >= 0.25 * q[4];
  };
  for (int doublings = 0; doublings < 40; ++doublings) {
    bool pass = true;
    for (int k = 0; k < ez && pass; ++k) {
      const double zeta = (double)k * K.dnzm1;
      for (int j = 0; j < ey && pass; ++j) {
        const double eta = (double)j * K.dnym1;
        for (int i = 0; i < ex && pass; ++i) {
          const double xi = (double)i * K.dnxm1;
          double q[5], fx[2][5], fy[2][5], fz[2][5], blend[5];
          exact_solution(xi, eta, zeta, ce, q);
          for (int s = 0; s < 2; ++s) {
            exact_solution((double)s, eta, zeta, ce, fx[s]);
            exact_solution(xi, (double)s, zeta, ce, fy[s]);
            exact_solution(xi, eta, (double)s, ce, fz[s]);
          }
          for (int m = 0; m < 5; ++m) {
            const double a = xi * fx[1][m] + (1.0 - xi) * fx[0][m];
            const double b = eta * fy[1][m] + (1.0 - eta) * fy[0][m];
            const double c = zeta * fz[1][m] + (1.0 - zeta) * fz[0][m];
            blend[m] = a + b + c - a * b - a * c - b * c + a * b * c;
          }
          pass = admissible(q) && admissible(blend);
          for (int s = 0; s < 2 && pass; ++s) pass = admissible(fx[s]) && admissible(fy[s]) && admissible(fz[s]);
        }
      }
    }
    if (pass) return doublings;
    for (int n = 0; n < 13; ++n) ce[4 * 13 + n] *= 2.0;
  }
  return -2;
}

// Create a problem: constants, initialize, exact_rhs (the reference's warm-up
// step is omitted: the reference re-initialises u after it, and rhs/lhs are
// rewritten before they are read, so it changes no value).
oracle_t* oracle_create(int kind, int nzones, const int* nx, const int* ny, const int* nz, const int* nbr, double dt,
                        int gx, int gy, int gz, int xz, int yz, const double* ce, int solve_float) {
  Problem* pb = new Problem();
  pb->kind = kind;
  pb->nzones = nzones;
  pb->k = set_constants(dt, gx, gy, gz, xz, yz);
  std::memcpy(pb->ce, ce, sizeof(pb->ce));
  pb->nbr.assign(nbr, nbr + 4 * nzones);
  pb->solve_float = solve_float;
  pb->zones.resize(nzones);
  for (int zi = 0; zi < nzones; ++zi) {
    Zone& z = pb->zones[zi];
    z.nx = nx[zi]; z.ny = ny[zi]; z.nz = nz[zi];
    size_t np = (size_t)z.nx * z.ny * z.nz;
    z.u.assign(np * 5, 0.0);
    z.rhs.assign(np * 5, 0.0);
    z.forcing.assign(np * 5, 0.0);
    for (auto* v : {&z.rho_i, &z.us, &z.vs, &z.ws, &z.qs, &z.square, &z.speed, &z.ainv}) v->assign(np, 0.0);
    initialize(*pb, z);
    exact_rhs(*pb, z);
  }
  return reinterpret_cast<oracle_t*>(pb);
}

void oracle_destroy(oracle_t* h) { delete reinterpret_cast<Problem*>(h); }

// One or more time steps: exch_qbc over all zones, then adi per zone
// (src/BT/bt-node.jl:280-395).  norms (nullable): 10 doubles per step,
// xcr[5] (residual norm of that step's compute_rhs, summed over zones, /dt)
// then xce[5] (error norm after the step, summed over zones).
int oracle_step(oracle_t* h, int nsteps, double* norms) {
  Problem& pb = *reinterpret_cast<Problem*>(h);
  for (int s = 0; s < nsteps; ++s) {
    if (pb.nzones > 1) exch_qbc(pb);
    std::vector<double> xcr_z(5 * pb.nzones), xce_z(5 * pb.nzones);
#pragma omp parallel for schedule(dynamic, 1)
    for (int zi = 0; zi < pb.nzones; ++zi) {
      Zone& z = pb.zones[zi];
      adi(pb, z, norms ? &xcr_z[5 * zi] : nullptr);
      if (norms) {
        double xcr_unused[5];
        zone_norms(pb, z, &xce_z[5 * zi], xcr_unused);
      }
    }
    if (norms) {
      for (int m = 0; m < 5; ++m) {
        double xcr = 0.0, xce = 0.0;
        for (int zi = 0; zi < pb.nzones; ++zi) {
          xcr = xcr + xcr_z[5 * zi + m] / pb.k.dt;
          xce = xce + xce_z[5 * zi + m];
        }
        norms[10 * s + m] = xcr;
        norms[10 * s + 5 + m] = xce;
      }
    }
  }
  return 0;
}

// verify's node part (src/BT/verify.jl:411-505): error_norm of u, then
// compute_rhs (no exchange) and rhs_norm; xcr sums rhs_norm/dt over zones.
int oracle_verify(oracle_t* h, double* xcr, double* xce) {
  Problem& pb = *reinterpret_cast<Problem*>(h);
  for (int m = 0; m < 5; ++m) { xcr[m] = 0.0; xce[m] = 0.0; }
  for (int zi = 0; zi < pb.nzones; ++zi) {
    Zone& z = pb.zones[zi];
    compute_rhs(pb, z);
    double ce_z[5], cr_z[5];
    zone_norms(pb, z, ce_z, cr_z);
    for (int m = 0; m < 5; ++m) {
      xcr[m] = xcr[m] + cr_z[m] / pb.k.dt;
      xce[m] = xce[m] + ce_z[m];
    }
  }
  return 0;
}

// Single phases on one zone (or all zones for exch_qbc), for per-phase parity:
// 0 compute_rhs (+txinvr for SP), 1 x sweep, 2 y sweep, 3 z sweep, 4 add,
// 5 exch_qbc (all zones), 6 compute_rhs only.
int oracle_phase(oracle_t* h, int phase, int zone) {
  Problem& pb = *reinterpret_cast<Problem*>(h);
  if (phase == 5) { exch_qbc(pb); return 0; }
  if (zone < 0 || zone >= pb.nzones) return -1;
  Zone& z = pb.zones[zone];
  switch (phase) {
    case 0: compute_rhs(pb, z); if (pb.kind == KIND_SP) txinvr(z); break;
    case 1: case 2: case 3:
      if (pb.kind == KIND_BT) {
        if (pb.solve_float) bt_sweep<float>(pb, z, phase - 1); else bt_sweep<double>(pb, z, phase - 1);
      } else {
        if (pb.solve_float) sp_sweep<float>(pb, z, phase - 1); else sp_sweep<double>(pb, z, phase - 1);
      }
      break;
    case 4: add(z); break;
    case 6: compute_rhs(pb, z); break;
    default: return -1;
  }
  return 0;
}

// Field access in the dense exchange layout [m][k][j][i] of one zone.
// which: 0 u, 1 rhs, 2 forcing.
int oracle_get(oracle_t* h, int which, int zone, double* out) {
  Problem& pb = *reinterpret_cast<Problem*>(h);
  if (zone < 0 || zone >= pb.nzones) return -1;
  Zone& z = pb.zones[zone];
  std::vector<double>& src = which == 0 ? z.u : (which == 1 ? z.rhs : z.forcing);
  size_t np = (size_t)z.nx * z.ny * z.nz;
  for (size_t p = 0; p < np; ++p)
    for (int m = 0; m < 5; ++m) out[m * np + p] = src[p * 5 + m];
  return 0;
}

int oracle_set(oracle_t* h, int which, int zone, const double* in) {
  Problem& pb = *reinterpret_cast<Problem*>(h);
  if (zone < 0 || zone >= pb.nzones) return -1;
  Zone& z = pb.zones[zone];
  std::vector<double>& dst = which == 0 ? z.u : (which == 1 ? z.rhs : z.forcing);
  size_t np = (size_t)z.nx * z.ny * z.nz;
  for (size_t p = 0; p < np; ++p)
    for (int m = 0; m < 5; ++m) dst[p * 5 + m] = in[m * np + p];
  return 0;
}

}  // extern "C"
#endif  // !ORACLE_TANGENT
