// npbmz_tangent.cpp -- forward-mode dual numbers through the CPU oracle's BT-MZ
// and SP-MZ time steps: the reference gradient for the discrete adjoint.
//
// TEST INFRASTRUCTURE ONLY (like npbmz_oracle.cpp, which this file compiles a
// second time): only tests/ load libnpbmz_tangent.so, to compare against the
// GPU adjoint (npbmz_adjoint).  The reference would take this gradient with
// ForwardDiff.jl dual numbers pushed through its Julia step (exch_qbc + adi,
// src/BT/bt-node.jl:280-395, src/SP/sp-node.jl:258-297); Julia is not
// available here, so the oracle's
// restatement of that step (npbmz_oracle.cpp, state type `real`) is
// instantiated with a dual number of NDIR directional parts.  The value part
// of every dual performs exactly the double operations of the oracle, so the
// primal trajectory is the oracle's bit for bit; each directional part is the
// exact derivative (up to rounding) of the discrete step along one seeded
// direction of (u_0, forcing).  The line solves run in the dual type too (the
// oracle's FP64 reference path); SP's std::max of the viscous band term
// compares value parts, so its derivative is that of the selected branch.
#include <cmath>

namespace npbmz_tangent {

constexpr int NDIR = 16;

struct Dual {
  double v;
  double d[NDIR];
  Dual() : v(0.0) {
    for (int k = 0; k < NDIR; ++k) d[k] = 0.0;
  }
  Dual(double x) : v(x) {  // NOLINT: implicit, as a constant
    for (int k = 0; k < NDIR; ++k) d[k] = 0.0;
  }
  explicit operator float() const { return (float)v; }
  Dual& operator+=(const Dual& b) {
    v += b.v;
    for (int k = 0; k < NDIR; ++k) d[k] += b.d[k];
    return *this;
  }
  Dual& operator-=(const Dual& b) {
    v -= b.v;
    for (int k = 0; k < NDIR; ++k) d[k] -= b.d[k];
    return *this;
  }
  Dual& operator*=(const Dual& b) {
    for (int k = 0; k < NDIR; ++k) d[k] = d[k] * b.v + v * b.d[k];
    v *= b.v;
    return *this;
  }
};

inline double value(const Dual& a) { return a.v; }

inline Dual operator+(const Dual& a, const Dual& b) {
  Dual r = a;
  r += b;
  return r;
}
inline Dual operator-(const Dual& a, const Dual& b) {
  Dual r = a;
  r -= b;
  return r;
}
inline Dual operator-(const Dual& a) {
  Dual r;
  r.v = -a.v;
  for (int k = 0; k < NDIR; ++k) r.d[k] = -a.d[k];
  return r;
}
inline Dual operator*(const Dual& a, const Dual& b) {
  Dual r = a;
  r *= b;
  return r;
}
inline Dual operator/(const Dual& a, const Dual& b) {
  Dual r;
  r.v = a.v / b.v;
  for (int k = 0; k < NDIR; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
  return r;
}
// mixed forms: the double operand is a constant
inline Dual operator+(const Dual& a, double b) { Dual r = a; r.v = a.v + b; return r; }
inline Dual operator+(double a, const Dual& b) { Dual r = b; r.v = a + b.v; return r; }
inline Dual operator-(const Dual& a, double b) { Dual r = a; r.v = a.v - b; return r; }
inline Dual operator-(double a, const Dual& b) {
  Dual r;
  r.v = a - b.v;
  for (int k = 0; k < NDIR; ++k) r.d[k] = -b.d[k];
  return r;
}
inline Dual operator*(const Dual& a, double b) {
  Dual r;
  r.v = a.v * b;
  for (int k = 0; k < NDIR; ++k) r.d[k] = a.d[k] * b;
  return r;
}
inline Dual operator*(double a, const Dual& b) {
  Dual r;
  r.v = a * b.v;
  for (int k = 0; k < NDIR; ++k) r.d[k] = a * b.d[k];
  return r;
}
inline Dual operator/(const Dual& a, double b) {
  Dual r;
  r.v = a.v / b;
  for (int k = 0; k < NDIR; ++k) r.d[k] = a.d[k] / b;
  return r;
}
inline Dual operator/(double a, const Dual& b) {
  Dual r;
  r.v = a / b.v;
  for (int k = 0; k < NDIR; ++k) r.d[k] = -r.v * b.d[k] / b.v;
  return r;
}
inline Dual sqrt(const Dual& a) {
  Dual r;
  r.v = std::sqrt(a.v);
  for (int k = 0; k < NDIR; ++k) r.d[k] = a.d[k] * (0.5 / r.v);
  return r;
}

}  // namespace npbmz_tangent

#define ORACLE_REAL npbmz_tangent::Dual
#define ORACLE_TANGENT 1
#include "npbmz_oracle.cpp"

extern "C" {

// J = 1/2 sum over every stored point of every zone of (u_N - u_target)^2
// after nsteps BT-MZ (kind 0) or SP-MZ (kind 1) steps (exch_qbc over all zones
// when there are several, then adi per zone) from u0 with the given forcing,
// and its derivatives dJ[d] along ndir <= 16 directions (du0[d], dforcing[d];
// either array may be NULL for zero).  Every array is the dense layout of all
// zones back to back (zone z: [5][nz][ny][nx]); du0 and dforcing hold ndir
// such arrays.  uN (nullable) receives the value part of u_N.
int tangent_objective(int kind, int nzones, const int* nx, const int* ny, const int* nz, const int* nbr, double dt,
                      int gx, int gy, int gz, int xz, int yz, const double* u0, const double* forcing,
                      const double* u_target, int nsteps, int ndir, const double* du0, const double* dforcing,
                      double* J, double* dJ, double* uN) {
  using npbmz_tangent::Dual;
  if (ndir < 0 || ndir > npbmz_tangent::NDIR || nzones < 1 || nsteps < 0) return -1;
  if (kind != KIND_BT && kind != KIND_SP) return -1;
  Problem pb;
  pb.kind = kind;
  pb.nzones = nzones;
  pb.k = set_constants(dt, gx, gy, gz, xz, yz);
  std::memset(pb.ce, 0, sizeof(pb.ce));
  pb.nbr.assign(nbr, nbr + 4 * nzones);
  pb.solve_float = 0;
  pb.zones.resize(nzones);
  size_t total = 0;
  for (int zi = 0; zi < nzones; ++zi) total += 5 * (size_t)nx[zi] * ny[zi] * nz[zi];
  size_t off = 0;
  for (int zi = 0; zi < nzones; ++zi) {
    Zone& z = pb.zones[zi];
    z.nx = nx[zi]; z.ny = ny[zi]; z.nz = nz[zi];
    const size_t np = (size_t)z.nx * z.ny * z.nz;
    z.u.assign(np * 5, Dual(0.0));
    z.rhs.assign(np * 5, Dual(0.0));
    z.forcing.assign(np * 5, Dual(0.0));
    for (auto* v : {&z.rho_i, &z.us, &z.vs, &z.ws, &z.qs, &z.square, &z.speed, &z.ainv}) v->assign(np, Dual(0.0));
    for (int m = 0; m < 5; ++m)
      for (size_t p = 0; p < np; ++p) {
        const size_t e = off + m * np + p;
        Dual& a = z.u[p * 5 + m];
        Dual& f = z.forcing[p * 5 + m];
        a.v = u0[e];
        f.v = forcing[e];
        for (int d = 0; d < ndir; ++d) {
          if (du0) a.d[d] = du0[(size_t)d * total + e];
          if (dforcing) f.d[d] = dforcing[(size_t)d * total + e];
        }
      }
    off += 5 * np;
  }
  for (int s = 0; s < nsteps; ++s) {
    if (pb.nzones > 1) exch_qbc(pb);
#pragma omp parallel for schedule(dynamic, 1)
    for (int zi = 0; zi < pb.nzones; ++zi) adi(pb, pb.zones[zi]);
  }
  Dual acc(0.0);
  off = 0;
  for (int zi = 0; zi < nzones; ++zi) {
    Zone& z = pb.zones[zi];
    const size_t np = (size_t)z.nx * z.ny * z.nz;
    for (int m = 0; m < 5; ++m)
      for (size_t p = 0; p < np; ++p) {
        const size_t e = off + m * np + p;
        const Dual a = z.u[p * 5 + m] - u_target[e];
        acc += a * a;
        if (uN) uN[e] = z.u[p * 5 + m].v;
      }
    off += 5 * np;
  }
  if (J) *J = 0.5 * acc.v;
  if (dJ)
    for (int d = 0; d < ndir; ++d) dJ[d] = 0.5 * acc.d[d];
  return 0;
}

// the BT-MZ form of tangent_objective
int tangent_bt_objective(int nzones, const int* nx, const int* ny, const int* nz, const int* nbr, double dt, int gx,
                         int gy, int gz, int xz, int yz, const double* u0, const double* forcing,
                         const double* u_target, int nsteps, int ndir, const double* du0, const double* dforcing,
                         double* J, double* dJ, double* uN) {
  return tangent_objective(KIND_BT, nzones, nx, ny, nz, nbr, dt, gx, gy, gz, xz, yz, u0, forcing, u_target, nsteps,
                           ndir, du0, dforcing, J, dJ, uN);
}

}  // extern "C"
