// lu_kernels.cuh -- the LU-MZ device code (NPBApps.jl src/LU), compiled
// twice into namespaces named by LU_NS: lu_exact.cu with -fmad=false (every
// FP64 statement rounds as the reference's Julia does, bit-for-bit the
// oracle) and lu_fast.cu with -fmad=true (a*b+c contracted to FMA).
#pragma once
#ifndef LU_NS
#error "define LU_NS before including lu_kernels.cuh"
#endif
#include "lu_types.h"

namespace npbmz_lu {
namespace LU_NS {

// ---- exact solution (src/LU/exact.jl) ---------------------------------------
__device__ inline void exact_point(const CeTable& ce, int i, int j, int k, int nx0, int ny0, int nz0, double out[5]) {
  const double xi = (double)(i - 1) / (nx0 - 1);
  const double eta = (double)(j - 1) / (ny0 - 1);
  const double zeta = (double)(k - 1) / (nz0 - 1);
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    const double* c = ce.c[m];
    out[m] = c[0] + (c[1] + (c[4] + (c[7] + c[10] * xi) * xi) * xi) * xi +
             (c[2] + (c[5] + (c[8] + c[11] * eta) * eta) * eta) * eta +
             (c[3] + (c[6] + (c[9] + c[12] * zeta) * zeta) * zeta) * zeta;
  }
}

// ---- rhs / erhs point operator (src/LU/rhs.jl, src/LU/erhs.jl) -------------
// o: the point's output, holding -frct (rhs) or 0 (erhs) on entry.  ERHS
// selects erhs's z second difference order (g(k+1) first) and its viscous
// association ((o + A) + B instead of o + (A + B)).
template <bool ERHS>
__device__ inline double visc_up(double o, double a, double b) {
  return ERHS ? (o + a) + b : o + (a + b);
}

__device__ __forceinline__ void prim_point(const double g[5], double pr[PR_COUNT]) {
  const double tmp = 1.0e+00 / g[0];
  pr[PR_RHO] = tmp;
  pr[PR_U21] = tmp * g[1];
  pr[PR_U31] = tmp * g[2];
  pr[PR_U41] = tmp * g[3];
  pr[PR_U51] = tmp * g[4];
  pr[PR_S] = pr[PR_U21] * pr[PR_U21] + pr[PR_U31] * pr[PR_U31] + pr[PR_U41] * pr[PR_U41];
  pr[PR_C21] = g[1] / g[0];
  pr[PR_C31] = g[2] / g[0];
  pr[PR_C41] = g[3] / g[0];
  pr[PR_Q] = 0.50e+00 * (g[1] * g[1] + g[2] * g[2] + g[3] * g[3]) / g[0];
}

__device__ __forceinline__ void store_prim(double* prim, long long NP, long long p, const double g[5]) {
  double pr[PR_COUNT];
  prim_point(g, pr);
#pragma unroll
  for (int q = 0; q < PR_COUNT; ++q) prim[q * NP + p] = pr[q];
}

template <bool ERHS>
__device__ void flux_point(const double* __restrict__ g, const double* __restrict__ prim, long long NP,
                           const LuZone& Z, int i, int j, int k, double o[5]) {
  const int nx = Z.nx, ny = Z.ny, nz = Z.nz;
  auto G = [&](int m, int ii, int jj, int kk) -> double { return g[m * NP + pidx(Z, ii, jj, kk)]; };
  auto P = [&](int q, int ii, int jj, int kk) -> double { return prim[q * NP + pidx(Z, ii, jj, kk)]; };
  const double tx1 = Z.tx1, tx2 = Z.tx2, tx3 = Z.tx3, ty1 = Z.ty1, ty2 = Z.ty2, ty3 = Z.ty3, tz1 = Z.tz1,
               tz2 = Z.tz2, tz3 = Z.tz3;
  // convective flux of direction D (0 x, 1 y, 2 z) at a point
  auto conv = [&](int D, int ii, int jj, int kk, double f[5]) {
    const double g2 = G(1, ii, jj, kk), g3 = G(2, ii, jj, kk), g4 = G(3, ii, jj, kk), g5 = G(4, ii, jj, kk);
    const double q = P(PR_Q, ii, jj, kk);
    if (D == 0) {
      const double u21 = P(PR_C21, ii, jj, kk);
      f[0] = g2;
      f[1] = g2 * u21 + c2 * (g5 - q);
      f[2] = g3 * u21;
      f[3] = g4 * u21;
      f[4] = (c1 * g5 - c2 * q) * u21;
    } else if (D == 1) {
      const double u31 = P(PR_C31, ii, jj, kk);
      f[0] = g3;
      f[1] = g2 * u31;
      f[2] = g3 * u31 + c2 * (g5 - q);
      f[3] = g4 * u31;
      f[4] = (c1 * g5 - c2 * q) * u31;
    } else {
      const double u41 = P(PR_C41, ii, jj, kk);
      f[0] = g4;
      f[1] = g2 * u41;
      f[2] = g3 * u41;
      f[3] = g4 * u41 + c2 * (g5 - q);
      f[4] = (c1 * g5 - c2 * q) * u41;
    }
  };
  // viscous flux of direction D between point b (the - side) and point a
  auto visc = [&](int D, double t3, int ai, int aj, int ak, int bi, int bj, int bk, double f[5]) {
    const double u21i = P(PR_U21, ai, aj, ak), u31i = P(PR_U31, ai, aj, ak), u41i = P(PR_U41, ai, aj, ak),
                 u51i = P(PR_U51, ai, aj, ak), si = P(PR_S, ai, aj, ak);
    const double u21m = P(PR_U21, bi, bj, bk), u31m = P(PR_U31, bi, bj, bk), u41m = P(PR_U41, bi, bj, bk),
                 u51m = P(PR_U51, bi, bj, bk), sm = P(PR_S, bi, bj, bk);
    f[1] = (D == 0 ? (4.0e+00 / 3.0e+00) * t3 : t3) * (u21i - u21m);
    f[2] = (D == 1 ? (4.0e+00 / 3.0e+00) * t3 : t3) * (u31i - u31m);
    f[3] = (D == 2 ? (4.0e+00 / 3.0e+00) * t3 : t3) * (u41i - u41m);
    const double ui = D == 0 ? u21i : (D == 1 ? u31i : u41i), um = D == 0 ? u21m : (D == 1 ? u31m : u41m);
    f[4] = 0.50e+00 * (1.0e+00 - c1 * c5) * t3 * (si - sm) + (1.0e+00 / 6.0e+00) * t3 * (ui * ui - um * um) +
           c1 * c5 * t3 * (u51i - u51m);
  };
  // ---------------- xi ----------------
  {
    double fp[5], fm[5];
    conv(0, i + 1, j, k, fp);
    conv(0, i - 1, j, k, fm);
#pragma unroll
    for (int m = 0; m < 5; ++m) o[m] = o[m] - tx2 * (fp[m] - fm[m]);
    visc(0, tx3, i + 1, j, k, i, j, k, fp);
    visc(0, tx3, i, j, k, i - 1, j, k, fm);
    o[0] = o[0] + dx1 * tx1 * (G(0, i - 1, j, k) - 2.0e+00 * G(0, i, j, k) + G(0, i + 1, j, k));
    const double dxm[5] = {dx1, dx2, dx3, dx4, dx5};
#pragma unroll
    for (int m = 1; m < 5; ++m)
      o[m] = visc_up<ERHS>(o[m], tx3 * c3 * c4 * (fp[m] - fm[m]),
                           dxm[m] * tx1 * (G(m, i - 1, j, k) - 2.0e+00 * G(m, i, j, k) + G(m, i + 1, j, k)));
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      if (i == 2) o[m] = o[m] - dssp * (+5.0e+00 * G(m, 2, j, k) - 4.0e+00 * G(m, 3, j, k) + G(m, 4, j, k));
      if (i == 3)
        o[m] = o[m] - dssp * (-4.0e+00 * G(m, 2, j, k) + 6.0e+00 * G(m, 3, j, k) - 4.0e+00 * G(m, 4, j, k) +
                              G(m, 5, j, k));
      if (i >= 4 && i <= nx - 3)
        o[m] = o[m] - dssp * (G(m, i - 2, j, k) - 4.0e+00 * G(m, i - 1, j, k) + 6.0e+00 * G(m, i, j, k) -
                              4.0e+00 * G(m, i + 1, j, k) + G(m, i + 2, j, k));
      if (i == nx - 2)
        o[m] = o[m] - dssp * (G(m, nx - 4, j, k) - 4.0e+00 * G(m, nx - 3, j, k) + 6.0e+00 * G(m, nx - 2, j, k) -
                              4.0e+00 * G(m, nx - 1, j, k));
      if (i == nx - 1)
        o[m] = o[m] - dssp * (G(m, nx - 3, j, k) - 4.0e+00 * G(m, nx - 2, j, k) + 5.0e+00 * G(m, nx - 1, j, k));
    }
  }
  // ---------------- eta ----------------
  {
    double fp[5], fm[5];
    conv(1, i, j + 1, k, fp);
    conv(1, i, j - 1, k, fm);
#pragma unroll
    for (int m = 0; m < 5; ++m) o[m] = o[m] - ty2 * (fp[m] - fm[m]);
    visc(1, ty3, i, j + 1, k, i, j, k, fp);
    visc(1, ty3, i, j, k, i, j - 1, k, fm);
    o[0] = o[0] + dy1 * ty1 * (G(0, i, j - 1, k) - 2.0e+00 * G(0, i, j, k) + G(0, i, j + 1, k));
    const double dym[5] = {dy1, dy2, dy3, dy4, dy5};
#pragma unroll
    for (int m = 1; m < 5; ++m)
      o[m] = visc_up<ERHS>(o[m], ty3 * c3 * c4 * (fp[m] - fm[m]),
                           dym[m] * ty1 * (G(m, i, j - 1, k) - 2.0e+00 * G(m, i, j, k) + G(m, i, j + 1, k)));
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      if (j == 2) o[m] = o[m] - dssp * (+5.0e+00 * G(m, i, 2, k) - 4.0e+00 * G(m, i, 3, k) + G(m, i, 4, k));
      if (j == 3)
        o[m] = o[m] - dssp * (-4.0e+00 * G(m, i, 2, k) + 6.0e+00 * G(m, i, 3, k) - 4.0e+00 * G(m, i, 4, k) +
                              G(m, i, 5, k));
      if (j >= 4 && j <= ny - 3)
        o[m] = o[m] - dssp * (G(m, i, j - 2, k) - 4.0e+00 * G(m, i, j - 1, k) + 6.0e+00 * G(m, i, j, k) -
                              4.0e+00 * G(m, i, j + 1, k) + G(m, i, j + 2, k));
      if (j == ny - 2)
        o[m] = o[m] - dssp * (G(m, i, ny - 4, k) - 4.0e+00 * G(m, i, ny - 3, k) + 6.0e+00 * G(m, i, ny - 2, k) -
                              4.0e+00 * G(m, i, ny - 1, k));
      if (j == ny - 1)
        o[m] = o[m] - dssp * (G(m, i, ny - 3, k) - 4.0e+00 * G(m, i, ny - 2, k) + 5.0e+00 * G(m, i, ny - 1, k));
    }
  }
  // ---------------- zeta ----------------
  {
    double fp[5], fm[5];
    conv(2, i, j, k + 1, fp);
    conv(2, i, j, k - 1, fm);
#pragma unroll
    for (int m = 0; m < 5; ++m) o[m] = o[m] - tz2 * (fp[m] - fm[m]);
    visc(2, tz3, i, j, k + 1, i, j, k, fp);
    visc(2, tz3, i, j, k, i, j, k - 1, fm);
    auto sd = [&](int m) {
      return ERHS ? (G(m, i, j, k + 1) - 2.0e+00 * G(m, i, j, k) + G(m, i, j, k - 1))
                  : (G(m, i, j, k - 1) - 2.0e+00 * G(m, i, j, k) + G(m, i, j, k + 1));
    };
    o[0] = o[0] + dz1 * tz1 * sd(0);
    const double dzm[5] = {dz1, dz2, dz3, dz4, dz5};
#pragma unroll
    for (int m = 1; m < 5; ++m) o[m] = visc_up<ERHS>(o[m], tz3 * c3 * c4 * (fp[m] - fm[m]), dzm[m] * tz1 * sd(m));
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      if (k == 2) o[m] = o[m] - dssp * (+5.0e+00 * G(m, i, j, 2) - 4.0e+00 * G(m, i, j, 3) + G(m, i, j, 4));
      if (k == 3)
        o[m] = o[m] - dssp * (-4.0e+00 * G(m, i, j, 2) + 6.0e+00 * G(m, i, j, 3) - 4.0e+00 * G(m, i, j, 4) +
                              G(m, i, j, 5));
      if (k >= 4 && k <= nz - 3)
        o[m] = o[m] - dssp * (G(m, i, j, k - 2) - 4.0e+00 * G(m, i, j, k - 1) + 6.0e+00 * G(m, i, j, k) -
                              4.0e+00 * G(m, i, j, k + 1) + G(m, i, j, k + 2));
      if (k == nz - 2)
        o[m] = o[m] - dssp * (G(m, i, j, nz - 4) - 4.0e+00 * G(m, i, j, nz - 3) + 6.0e+00 * G(m, i, j, nz - 2) -
                              4.0e+00 * G(m, i, j, nz - 1));
      if (k == nz - 1)
        o[m] = o[m] - dssp * (G(m, i, j, nz - 3) - 4.0e+00 * G(m, i, j, nz - 2) + 5.0e+00 * G(m, i, j, nz - 1));
    }
  }
}

__device__ inline bool decode(const LuZone& Z, int q, int& i, int& j, int& k) {
  if (q >= Z.np) return false;
  i = q % Z.nx + 1;
  j = (q / Z.nx) % Z.ny + 1;
  k = q / (Z.nx * Z.ny) + 1;
  return true;
}

__device__ inline bool interior(const LuZone& Z, int i, int j, int k) {
  return i >= 2 && i <= Z.nx - 1 && j >= 2 && j <= Z.ny - 1 && k >= 2 && k <= Z.nz - 1;
}

// rhs (ERHS = false: g = u, out = rsd starting at -frct) or erhs's flux part
// (ERHS = true: g = the exact polynomial in rsd, out = frct starting at 0)
template <bool ERHS>
__global__ void __launch_bounds__(TPB) k_lu_rhs(LuDev D, const LuWork* __restrict__ work, const double* g,
                                                const double* __restrict__ prim, double* out) {
  const LuWork w = work[blockIdx.x];
  const LuZone Z = D.zones[w.zone];
  int i, j, k;
  if (!decode(Z, w.first + threadIdx.x, i, j, k)) return;
  const long long p = pidx(Z, i, j, k);
  double o[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) o[m] = ERHS ? 0.0 : -D.frct[m * D.NP + p];
  if (interior(Z, i, j, k)) flux_point<ERHS>(g, prim, D.NP, Z, i, j, k, o);
#pragma unroll
  for (int m = 0; m < 5; ++m) out[m * D.NP + p] = o[m];
}

// setbv + setiv (src/LU/setbv.jl, src/LU/setiv.jl); every face point of
// setbv gets exact() of its own (i, j, k), whichever face writes it last
__global__ void __launch_bounds__(TPB) k_lu_init(LuDev D, const LuWork* __restrict__ work, CeTable ce) {
  const LuWork w = work[blockIdx.x];
  const LuZone Z = D.zones[w.zone];
  int i, j, k;
  if (!decode(Z, w.first + threadIdx.x, i, j, k)) return;
  const int nx = Z.nx, ny = Z.ny, nz = Z.nz;
  const long long p = pidx(Z, i, j, k);
  double out[5];
  if (!interior(Z, i, j, k)) {
    exact_point(ce, i, j, k, nx, ny, nz, out);
  } else {
    const double zeta = (double)(k - 1) / (nz - 1);
    const double eta = (double)(j - 1) / (ny - 1);
    const double xi = (double)(i - 1) / (nx - 1);
    double a1[5], a2[5], b1[5], b2[5], g1[5], g2[5];
    exact_point(ce, 1, j, k, nx, ny, nz, a1);
    exact_point(ce, nx, j, k, nx, ny, nz, a2);
    exact_point(ce, i, 1, k, nx, ny, nz, b1);
    exact_point(ce, i, ny, k, nx, ny, nz, b2);
    exact_point(ce, i, j, 1, nx, ny, nz, g1);
    exact_point(ce, i, j, nz, nx, ny, nz, g2);
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const double pxi = (1.0e+00 - xi) * a1[m] + xi * a2[m];
      const double peta = (1.0e+00 - eta) * b1[m] + eta * b2[m];
      const double pzeta = (1.0e+00 - zeta) * g1[m] + zeta * g2[m];
      out[m] = pxi + peta + pzeta - pxi * peta - peta * pzeta - pzeta * pxi + pxi * peta * pzeta;
    }
  }
#pragma unroll
  for (int m = 0; m < 5; ++m) D.u[m * D.NP + p] = out[m];
}

// erhs's first part: rsd = the exact polynomial (non-Horner, src/LU/erhs.jl:24-47)
__global__ void __launch_bounds__(TPB) k_lu_poly(LuDev D, const LuWork* __restrict__ work, CeTable ce) {
  const LuWork w = work[blockIdx.x];
  const LuZone Z = D.zones[w.zone];
  int i, j, k;
  if (!decode(Z, w.first + threadIdx.x, i, j, k)) return;
  const long long p = pidx(Z, i, j, k);
  const double zeta = (double)(k - 1) / (Z.nz - 1);
  const double eta = (double)(j - 1) / (Z.ny - 1);
  const double xi = (double)(i - 1) / (Z.nx - 1);
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    const double* c = ce.c[m];
    D.rsd[m * D.NP + p] = c[0] + c[1] * xi + c[2] * eta + c[3] * zeta + c[4] * xi * xi + c[5] * eta * eta +
                          c[6] * zeta * zeta + c[7] * xi * xi * xi + c[8] * eta * eta * eta +
                          c[9] * zeta * zeta * zeta + c[10] * xi * xi * xi * xi + c[11] * eta * eta * eta * eta +
                          c[12] * zeta * zeta * zeta * zeta;
  }
}

// rsd *= dt (SCALE) or u += tmp * rsd (UPDATE, with the point's prim
// planes refreshed from the new u) on the interior
template <bool UPDATE>
__global__ void __launch_bounds__(TPB) k_lu_pointwise(LuDev D, const LuWork* __restrict__ work, double tmp) {
  const LuWork w = work[blockIdx.x];
  const LuZone Z = D.zones[w.zone];
  int i, j, k;
  if (!decode(Z, w.first + threadIdx.x, i, j, k) || !interior(Z, i, j, k)) return;
  const long long p = pidx(Z, i, j, k);
  if (UPDATE) {
    double g[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      g[m] = D.u[m * D.NP + p] + tmp * D.rsd[m * D.NP + p];
      D.u[m * D.NP + p] = g[m];
    }
    double pr[PR_COUNT];
    prim_point(g, pr);
#pragma unroll
    for (int q = 0; q < PR_COUNT; ++q) D.prim[q * D.NP + p] = pr[q];
    if (D.health) {
      // on the bit patterns (integer pipe): positive and finite
      const double pres = g[4] - pr[PR_Q];
      const unsigned long long br = (unsigned long long)__double_as_longlong(g[0]);
      const unsigned long long bp = (unsigned long long)__double_as_longlong(pres);
      const bool rho_ok = br - 1ull < 0x7FEFFFFFFFFFFFFFull, p_ok = bp - 1ull < 0x7FEFFFFFFFFFFFFFull;
      if (!(rho_ok && p_ok)) {
        const bool p_finite = (bp & 0x7FF0000000000000ull) != 0x7FF0000000000000ull;
        const unsigned bits = (rho_ok ? 0u : LU_STATE_DENSITY) |
                              (p_ok ? 0u : p_finite ? LU_STATE_PRESSURE : LU_STATE_NONFINITE);
        atomicOr(D.health, (unsigned long long)bits);
        atomicMin(D.health + 1, (unsigned long long)p);
      }
    }
  } else {
#pragma unroll
    for (int m = 0; m < 5; ++m) D.rsd[m * D.NP + p] = D.dt * D.rsd[m * D.NP + p];
  }
}

// prim planes of g (u, or erhs's exact polynomial) at every point
__global__ void __launch_bounds__(TPB) k_lu_prim(LuDev D, const LuWork* __restrict__ work, const double* g) {
  const LuWork w = work[blockIdx.x];
  const LuZone Z = D.zones[w.zone];
  const int q = w.first + threadIdx.x;
  if (q >= Z.np) return;
  const long long p = Z.off + q;
  double v[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) v[m] = g[m * D.NP + p];
  store_prim(D.prim, D.NP, p, v);
}

// ---- Jacobian blocks of jacld / jacu (src/LU/jacld.jl, src/LU/jacu.jl) -----
// the diagonal block (identical in jacld and jacu) at the point's own state
__device__ __forceinline__ void jac_d(const JC& J, double r1, double u2, double u3, double u4, double u5,
                                      double d[5][5]) {
  const double dt = J.dt, tx1 = J.tx1, ty1 = J.ty1, tz1 = J.tz1;
  const double tmp1 = r1, tmp2 = tmp1 * tmp1, tmp3 = tmp1 * tmp2;
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
}

// Off-diagonal block of direction DIR (0 x, 1 y, 2 z) from the neighbour's
// state; SG = -1: jacld's (the neighbour at -1), SG = +1: jacu's (at +1).
// The entries are the reference's statements.  r1 = 1/u1 of the neighbour
// (the reference's tmp1: the PR_RHO plane).
template <int DIR, int SG>
__device__ __forceinline__ void jac_off(const JC& J, double r1, double u2, double u3, double u4, double u5,
                                        double a[5][5]) {
  const double dt = J.dt;
  const double tmp1 = r1, tmp2 = tmp1 * tmp1, tmp3 = tmp1 * tmp2;
  if (DIR == 2) {
    const double tz1 = J.tz1, tz2 = J.tz2;
    if (SG < 0) {
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
    } else {
      a[0][0] = -dt * tz1 * dz1;
      a[0][1] = 0.0;
      a[0][2] = 0.0;
      a[0][3] = dt * tz2;
      a[0][4] = 0.0;
      a[1][0] = dt * tz2 * (-(u2 * u4) * tmp2) - dt * tz1 * (-c34 * tmp2 * u2);
      a[1][1] = dt * tz2 * (u4 * tmp1) - dt * tz1 * c34 * tmp1 - dt * tz1 * dz2;
      a[1][2] = 0.0;
      a[1][3] = dt * tz2 * (u2 * tmp1);
      a[1][4] = 0.0;
      a[2][0] = dt * tz2 * (-(u3 * u4) * tmp2) - dt * tz1 * (-c34 * tmp2 * u3);
      a[2][1] = 0.0;
      a[2][2] = dt * tz2 * (u4 * tmp1) - dt * tz1 * (c34 * tmp1) - dt * tz1 * dz3;
      a[2][3] = dt * tz2 * (u3 * tmp1);
      a[2][4] = 0.0;
      a[3][0] = dt * tz2 * (-((u4 * tmp1) * (u4 * tmp1)) + 0.50e+00 * c2 * ((u2 * u2 + u3 * u3 + u4 * u4) * tmp2)) -
                dt * tz1 * (-r43 * c34 * tmp2 * u4);
      a[3][1] = dt * tz2 * (-c2 * (u2 * tmp1));
      a[3][2] = dt * tz2 * (-c2 * (u3 * tmp1));
      a[3][3] = dt * tz2 * (2.0e+00 - c2) * (u4 * tmp1) - dt * tz1 * (r43 * c34 * tmp1) - dt * tz1 * dz4;
      a[3][4] = dt * tz2 * c2;
      a[4][0] = dt * tz2 * ((c2 * (u2 * u2 + u3 * u3 + u4 * u4) * tmp2 - c1 * (u5 * tmp1)) * (u4 * tmp1)) -
                dt * tz1 *
                    (-(c34 - c1345) * tmp3 * (u2 * u2) - (c34 - c1345) * tmp3 * (u3 * u3) -
                     (r43 * c34 - c1345) * tmp3 * (u4 * u4) - c1345 * tmp2 * u5);
      a[4][1] = dt * tz2 * (-c2 * (u2 * u4) * tmp2) - dt * tz1 * (c34 - c1345) * tmp2 * u2;
      a[4][2] = dt * tz2 * (-c2 * (u3 * u4) * tmp2) - dt * tz1 * (c34 - c1345) * tmp2 * u3;
      a[4][3] = dt * tz2 * (c1 * (u5 * tmp1) - 0.50e+00 * c2 * ((u2 * u2 + u3 * u3 + 3.0e+00 * u4 * u4) * tmp2)) -
                dt * tz1 * (r43 * c34 - c1345) * tmp2 * u4;
      a[4][4] = dt * tz2 * (c1 * (u4 * tmp1)) - dt * tz1 * c1345 * tmp1 - dt * tz1 * dz5;
    }
  } else if (DIR == 1) {
    const double ty1 = J.ty1, ty2 = J.ty2;
    if (SG < 0) {
      a[0][0] = -dt * ty1 * dy1;
      a[0][1] = 0.0;
      a[0][2] = -dt * ty2;
      a[0][3] = 0.0;
      a[0][4] = 0.0;
      a[1][0] = -dt * ty2 * (-(u2 * u3) * tmp2) - dt * ty1 * (-c34 * tmp2 * u2);
      a[1][1] = -dt * ty2 * (u3 * tmp1) - dt * ty1 * (c34 * tmp1) - dt * ty1 * dy2;
      a[1][2] = -dt * ty2 * (u2 * tmp1);
      a[1][3] = 0.0;
      a[1][4] = 0.0;
      a[2][0] = -dt * ty2 * (-((u3 * tmp1) * (u3 * tmp1)) + 0.50e+00 * c2 * ((u2 * u2 + u3 * u3 + u4 * u4) * tmp2)) -
                dt * ty1 * (-r43 * c34 * tmp2 * u3);
      a[2][1] = -dt * ty2 * (-c2 * (u2 * tmp1));
      a[2][2] = -dt * ty2 * ((2.0e+00 - c2) * (u3 * tmp1)) - dt * ty1 * (r43 * c34 * tmp1) - dt * ty1 * dy3;
      a[2][3] = -dt * ty2 * (-c2 * (u4 * tmp1));
      a[2][4] = -dt * ty2 * c2;
      a[3][0] = -dt * ty2 * (-(u3 * u4) * tmp2) - dt * ty1 * (-c34 * tmp2 * u4);
      a[3][1] = 0.0;
      a[3][2] = -dt * ty2 * (u4 * tmp1);
      a[3][3] = -dt * ty2 * (u3 * tmp1) - dt * ty1 * (c34 * tmp1) - dt * ty1 * dy4;
      a[3][4] = 0.0;
      a[4][0] = -dt * ty2 * ((c2 * (u2 * u2 + u3 * u3 + u4 * u4) * tmp2 - c1 * (u5 * tmp1)) * (u3 * tmp1)) -
                dt * ty1 *
                    (-(c34 - c1345) * tmp3 * (u2 * u2) - (r43 * c34 - c1345) * tmp3 * (u3 * u3) -
                     (c34 - c1345) * tmp3 * (u4 * u4) - c1345 * tmp2 * u5);
      a[4][1] = -dt * ty2 * (-c2 * (u2 * u3) * tmp2) - dt * ty1 * (c34 - c1345) * tmp2 * u2;
      a[4][2] = -dt * ty2 * (c1 * (u5 * tmp1) - 0.50e+00 * c2 * ((u2 * u2 + 3.0e+00 * u3 * u3 + u4 * u4) * tmp2)) -
                dt * ty1 * (r43 * c34 - c1345) * tmp2 * u3;
      a[4][3] = -dt * ty2 * (-c2 * (u3 * u4) * tmp2) - dt * ty1 * (c34 - c1345) * tmp2 * u4;
      a[4][4] = -dt * ty2 * (c1 * (u3 * tmp1)) - dt * ty1 * c1345 * tmp1 - dt * ty1 * dy5;
    } else {
      a[0][0] = -dt * ty1 * dy1;
      a[0][1] = 0.0;
      a[0][2] = dt * ty2;
      a[0][3] = 0.0;
      a[0][4] = 0.0;
      a[1][0] = dt * ty2 * (-(u2 * u3) * tmp2) - dt * ty1 * (-c34 * tmp2 * u2);
      a[1][1] = dt * ty2 * (u3 * tmp1) - dt * ty1 * (c34 * tmp1) - dt * ty1 * dy2;
      a[1][2] = dt * ty2 * (u2 * tmp1);
      a[1][3] = 0.0;
      a[1][4] = 0.0;
      a[2][0] = dt * ty2 * (-((u3 * tmp1) * (u3 * tmp1)) + 0.50e+00 * c2 * ((u2 * u2 + u3 * u3 + u4 * u4) * tmp2)) -
                dt * ty1 * (-r43 * c34 * tmp2 * u3);
      a[2][1] = dt * ty2 * (-c2 * (u2 * tmp1));
      a[2][2] = dt * ty2 * ((2.0e+00 - c2) * (u3 * tmp1)) - dt * ty1 * (r43 * c34 * tmp1) - dt * ty1 * dy3;
      a[2][3] = dt * ty2 * (-c2 * (u4 * tmp1));
      a[2][4] = dt * ty2 * c2;
      a[3][0] = dt * ty2 * (-(u3 * u4) * tmp2) - dt * ty1 * (-c34 * tmp2 * u4);
      a[3][1] = 0.0;
      a[3][2] = dt * ty2 * (u4 * tmp1);
      a[3][3] = dt * ty2 * (u3 * tmp1) - dt * ty1 * (c34 * tmp1) - dt * ty1 * dy4;
      a[3][4] = 0.0;
      a[4][0] = dt * ty2 * ((c2 * (u2 * u2 + u3 * u3 + u4 * u4) * tmp2 - c1 * (u5 * tmp1)) * (u3 * tmp1)) -
                dt * ty1 *
                    (-(c34 - c1345) * tmp3 * (u2 * u2) - (r43 * c34 - c1345) * tmp3 * (u3 * u3) -
                     (c34 - c1345) * tmp3 * (u4 * u4) - c1345 * tmp2 * u5);
      a[4][1] = dt * ty2 * (-c2 * (u2 * u3) * tmp2) - dt * ty1 * (c34 - c1345) * tmp2 * u2;
      a[4][2] = dt * ty2 * (c1 * (u5 * tmp1) - 0.50e+00 * c2 * ((u2 * u2 + 3.0e+00 * u3 * u3 + u4 * u4) * tmp2)) -
                dt * ty1 * (r43 * c34 - c1345) * tmp2 * u3;
      a[4][3] = dt * ty2 * (-c2 * (u3 * u4) * tmp2) - dt * ty1 * (c34 - c1345) * tmp2 * u4;
      a[4][4] = dt * ty2 * (c1 * (u3 * tmp1)) - dt * ty1 * c1345 * tmp1 - dt * ty1 * dy5;
    }
  } else {
    const double tx1 = J.tx1, tx2 = J.tx2;
    if (SG < 0) {
      a[0][0] = -dt * tx1 * dx1;
      a[0][1] = -dt * tx2;
      a[0][2] = 0.0;
      a[0][3] = 0.0;
      a[0][4] = 0.0;
      a[1][0] = -dt * tx2 * (-((u2 * tmp1) * (u2 * tmp1)) + c2 * 0.50e+00 * (u2 * u2 + u3 * u3 + u4 * u4) * tmp2) -
                dt * tx1 * (-r43 * c34 * tmp2 * u2);
      a[1][1] = -dt * tx2 * ((2.0e+00 - c2) * (u2 * tmp1)) - dt * tx1 * (r43 * c34 * tmp1) - dt * tx1 * dx2;
      a[1][2] = -dt * tx2 * (-c2 * (u3 * tmp1));
      a[1][3] = -dt * tx2 * (-c2 * (u4 * tmp1));
      a[1][4] = -dt * tx2 * c2;
      a[2][0] = -dt * tx2 * (-(u2 * u3) * tmp2) - dt * tx1 * (-c34 * tmp2 * u3);
      a[2][1] = -dt * tx2 * (u3 * tmp1);
      a[2][2] = -dt * tx2 * (u2 * tmp1) - dt * tx1 * (c34 * tmp1) - dt * tx1 * dx3;
      a[2][3] = 0.0;
      a[2][4] = 0.0;
      a[3][0] = -dt * tx2 * (-(u2 * u4) * tmp2) - dt * tx1 * (-c34 * tmp2 * u4);
      a[3][1] = -dt * tx2 * (u4 * tmp1);
      a[3][2] = 0.0;
      a[3][3] = -dt * tx2 * (u2 * tmp1) - dt * tx1 * (c34 * tmp1) - dt * tx1 * dx4;
      a[3][4] = 0.0;
      a[4][0] = -dt * tx2 * ((c2 * (u2 * u2 + u3 * u3 + u4 * u4) * tmp2 - c1 * (u5 * tmp1)) * (u2 * tmp1)) -
                dt * tx1 *
                    (-(r43 * c34 - c1345) * tmp3 * (u2 * u2) - (c34 - c1345) * tmp3 * (u3 * u3) -
                     (c34 - c1345) * tmp3 * (u4 * u4) - c1345 * tmp2 * u5);
      a[4][1] = -dt * tx2 * (c1 * (u5 * tmp1) - 0.50e+00 * c2 * ((3.0e+00 * u2 * u2 + u3 * u3 + u4 * u4) * tmp2)) -
                dt * tx1 * (r43 * c34 - c1345) * tmp2 * u2;
      a[4][2] = -dt * tx2 * (-c2 * (u3 * u2) * tmp2) - dt * tx1 * (c34 - c1345) * tmp2 * u3;
      a[4][3] = -dt * tx2 * (-c2 * (u4 * u2) * tmp2) - dt * tx1 * (c34 - c1345) * tmp2 * u4;
      a[4][4] = -dt * tx2 * (c1 * (u2 * tmp1)) - dt * tx1 * c1345 * tmp1 - dt * tx1 * dx5;
    } else {
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
    }
  }
}

// The t-th point (0-based) of hyperplane i + j + k = l of a zone's interior,
// enumerated by k ascending, then j ascending.
__device__ inline bool hyperplane_point(const LuZone& Z, int l, int t, int& i, int& j, int& k) {
  const int klo = max(2, l - (Z.nx - 1) - (Z.ny - 1)), khi = min(Z.nz - 1, l - 4);
  for (int kk = klo; kk <= khi; ++kk) {
    const int s = l - kk;
    const int jlo = max(2, s - (Z.nx - 1)), jhi = min(Z.ny - 1, s - 2);
    const int c = jhi - jlo + 1;
    if (c <= 0) continue;
    if (t < c) {
      k = kk;
      j = jlo + t;
      i = s - j;
      return true;
    }
    t -= c;
  }
  return false;
}

__device__ __forceinline__ void load5(const double* f, long long NP, long long p, double v[5]) {
#pragma unroll
  for (int m = 0; m < 5; ++m) v[m] = f[m * NP + p];
}

template <int DIR, int S>
__device__ __forceinline__ void store_blk(double* jac, long long NP, long long h, const double b[5][5]) {
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c < 5; ++c)
      if (!off_zero(DIR, r, c)) jac[(FAC_BLK + (2 * DIR + S) * BLK_NZ + blk_idx(DIR, r, c)) * NP + h] = b[r][c];
}

// jacld's (SG = -1) and jacu's (SG = +1) blocks of direction DIR built from
// this point's state (r1 = 1/u1, u), stored at the interior consumers: the
// point at +1 in DIR reads the jacld block, the point at -1 the jacu block.
// Both signs from one state share most of their subexpressions.
template <int DIR>
__device__ __forceinline__ void jac_dir(const JC& J, double r1, const double u[5], double* __restrict__ jac,
                                        long long NP, bool lo, long long slot_lo, bool up, long long slot_up) {
  double b[5][5], c[5][5];
  if (lo && up) {
    jac_off<DIR, -1>(J, r1, u[1], u[2], u[3], u[4], b);
    jac_off<DIR, 1>(J, r1, u[1], u[2], u[3], u[4], c);
    store_blk<DIR, 0>(jac, NP, slot_lo, b);
    store_blk<DIR, 1>(jac, NP, slot_up, c);
  } else if (lo) {
    jac_off<DIR, -1>(J, r1, u[1], u[2], u[3], u[4], b);
    store_blk<DIR, 0>(jac, NP, slot_lo, b);
  } else if (up) {
    jac_off<DIR, 1>(J, r1, u[1], u[2], u[3], u[4], c);
    store_blk<DIR, 1>(jac, NP, slot_up, c);
  }
}

// jacld's and jacu's blocks and d's factors (the Jacobian work of ssor,
// taken off the wavefront): one thread per point of the zones (blockIdx.y:
// zone - z0), in the zone's full-box hyperplane order (i+j+k, then k, then
// j), so that consecutive threads write consecutive consumer slots.
// fb: per zone, l and k, the first full-box point of row k of hyperplane l;
// ri: the same for the interior points (the consumers' slots).
// HP_ORDER false: threads in the zone's natural order instead (coalesced
// reads of the point's state, scattered block writes).  The FP64-bound
// uncontracted build is faster so, the FMA build with HP_ORDER; the values
// written are the same either way.
template <bool HP_ORDER>
__global__ void __launch_bounds__(TPB) k_lu_jac(LuDev D, const int* __restrict__ fb, int fls, const int* __restrict__ ri,
                                                int ls, int ks, double* __restrict__ jac, int z0) {
  const int zone = z0 + blockIdx.y;
  const LuZone Z = D.zones[zone];
  const int T = blockIdx.x * TPB + threadIdx.x;
  if (T >= Z.np) return;
  int i, j, k;
  if (HP_ORDER) {
    const int* FB = fb + (long long)zone * fls * ks;
    int lo = 3, hi = Z.nx + Z.ny + Z.nz;  // the hyperplane: largest l starting at or before T
    while (lo < hi) {
      const int mid = (lo + hi + 1) / 2;
      if (FB[mid * ks] <= T) lo = mid; else hi = mid - 1;
    }
    const int l = lo;
    int klo = 1, khi = Z.nz;  // the row: largest k starting at or before T
    while (klo < khi) {
      const int mid = (klo + khi + 1) / 2;
      if (FB[l * ks + mid] <= T) klo = mid; else khi = mid - 1;
    }
    k = klo;
    j = max(1, l - k - Z.nx) + (T - FB[l * ks + k]);
    i = l - j - k;
  } else {
    decode(Z, T, i, j, k);
  }
  const long long NP = D.NP, p = pidx(Z, i, j, k);
  const JC J{D.dt, Z.tx1, Z.tx2, Z.ty1, Z.ty2, Z.tz1, Z.tz2};
  const int* R = ri + (long long)zone * ls * ks;
  auto slot = [&](int a, int b, int c) -> long long {
    const int l = a + b + c;
    return Z.off + R[(long long)l * ks + c] + (b - max(2, l - c - (Z.nx - 1)));
  };
  const double r1 = D.prim[PR_RHO * NP + p];
  double u[5];
  load5(D.u, NP, p, u);
  const bool ii = i >= 2 && i <= Z.nx - 1, jj = j >= 2 && j <= Z.ny - 1, kk = k >= 2 && k <= Z.nz - 1;
  if (jj && kk) {
    const bool lo = i <= Z.nx - 2, up = i >= 3;
    jac_dir<0>(J, r1, u, jac, NP, lo, lo ? slot(i + 1, j, k) : 0, up, up ? slot(i - 1, j, k) : 0);
  }
  if (ii && kk) {
    const bool lo = j <= Z.ny - 2, up = j >= 3;
    jac_dir<1>(J, r1, u, jac, NP, lo, lo ? slot(i, j + 1, k) : 0, up, up ? slot(i, j - 1, k) : 0);
  }
  if (ii && jj) {
    const bool lo = k <= Z.nz - 2, up = k >= 3;
    jac_dir<2>(J, r1, u, jac, NP, lo, lo ? slot(i, j, k + 1) : 0, up, up ? slot(i, j, k - 1) : 0);
  }
  if (ii && jj && kk) {
    const long long h = slot(i, j, k);
    double b[5][5];
    jac_d(J, r1, u[1], u[2], u[3], u[4], b);
    const double rinv0 = 1.0e+00 / b[0][0];
#pragma unroll
    for (int r = 0; r < 5; ++r) jac[(FAC_T + r) * NP + h] = b[r][r];
#pragma unroll
    for (int r = 1; r < 5; ++r) jac[(FAC_R0 + r - 1) * NP + h] = rinv0 * b[r][0];
#pragma unroll
    for (int c = 1; c <= 3; ++c) jac[(FAC_4C + c - 1) * NP + h] = (1.0e+00 / b[c][c]) * b[4][c];
  }
}

// row M of the point's block (DIR, S) dotted with w, summed left to right as
// the reference does (structural zeros skipped: a product with one is +-0
// and adding it changes no sum's value)
template <int DIR, int S, int M>
__device__ __forceinline__ double row_dot(const double* __restrict__ jac, long long NP, long long h,
                                          const double w[5]) {
  double s = 0.0;
  bool first = true;
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    if (off_zero(DIR, M, c)) continue;
    const double t = jac[(FAC_BLK + (2 * DIR + S) * BLK_NZ + blk_idx(DIR, M, c)) * NP + h] * w[c];
    s = first ? t : s + t;
    first = false;
  }
  return s;
}

// sum over c of Y[M][c] wy[c] + X[M][c] wx[c] (y term first, as blts / buts
// write it)
template <int S, int M>
__device__ __forceinline__ double row_dot2(const double* __restrict__ jac, long long NP, long long h,
                                           const double wy[5], const double wx[5]) {
  double s = 0.0;
  bool first = true;
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    if (!off_zero(1, M, c)) {
      const double t = jac[(FAC_BLK + (2 + S) * BLK_NZ + blk_idx(1, M, c)) * NP + h] * wy[c];
      s = first ? t : s + t;
      first = false;
    }
    if (!off_zero(0, M, c)) {
      const double t = jac[(FAC_BLK + S * BLK_NZ + blk_idx(0, M, c)) * NP + h] * wx[c];
      s = first ? t : s + t;
      first = false;
    }
  }
  return s;
}

// blts's two update loops for row M of one point (h: its jac index)
template <int M, bool SCALE>
__device__ __forceinline__ double lower_row(const LuDev& D, const double* __restrict__ jac, const LuZone& Z, int i,
                                            int j, int k, long long h) {
  const long long NP = D.NP, p = pidx(Z, i, j, k);
  const double omega = D.omega;
  double v = D.rsd[M * NP + p];
  if (SCALE) v = D.dt * v;
  double w[5], x[5];
  load5(D.rsd, NP, pidx(Z, i, j, k - 1), w);
  v = v - omega * row_dot<2, 0, M>(jac, NP, h, w);
  load5(D.rsd, NP, pidx(Z, i, j - 1, k), w);
  load5(D.rsd, NP, pidx(Z, i - 1, j, k), x);
  v = v - omega * row_dot2<0, M>(jac, NP, h, w, x);
  return v;
}

// d's factors row m needs, loaded before the rows are exchanged (so that
// their latency overlaps the row sums): f[0] = t_mm; rows 1..3 f[1] = tmp_m0;
// row 4 f[1..4] = tmp_40, tmp_10, tmp_20, tmp_30, f[5..7] = tmp_41..tmp_43
__device__ __forceinline__ void load_factors(const double* __restrict__ jac, long long NP, long long h, int m,
                                             double f[8]) {
  f[0] = jac[(FAC_T + m) * NP + h];
  if (m >= 1 && m <= 3) f[1] = jac[(FAC_R0 + m - 1) * NP + h];
  if (m == 4) {
    f[1] = jac[(FAC_R0 + 3) * NP + h];
#pragma unroll
    for (int c = 1; c <= 3; ++c) {
      f[1 + c] = jac[(FAC_R0 + c - 1) * NP + h];
      f[4 + c] = jac[(FAC_4C + c - 1) * NP + h];
    }
  }
}

// the forward substitution with d's factors (rows exchanged through shared
// memory); v: this thread's row, sv: every row of the point
__device__ __forceinline__ double d_solve(const double f[8], int m, double v, const double sv[5]) {
  const double v0 = sv[0];
  if (m == 0) return v / f[0];
  if (m < 4) {
    v = v - v0 * f[1];
    return v / f[0];
  }
  v = v - v0 * f[1];
#pragma unroll
  for (int c = 1; c <= 3; ++c) {
    const double vc = sv[c] - v0 * f[1 + c];  // v_c after column 0, as row c has it
    v = v - vc * f[4 + c];
  }
  return v / f[0];
}

// jacld + blts at every point of hyperplane l (blockIdx.y: zone - zone0),
// five threads per point (threadIdx.y: row).  SCALE: rsd *= dt at the point
// first (ssor's scaling, fused: blts reads only points it has already scaled
// and solved, or boundary points, which the scaling does not touch).
template <bool SCALE>
__global__ void __launch_bounds__(HP * 5) k_lu_lower(LuDev D, const double* __restrict__ jac,
                                                     const int* __restrict__ hps, int hstride, int l, int zone0) {
  __shared__ double sv[HP][5];
  const int m = threadIdx.y, a = threadIdx.x, z = zone0 + blockIdx.y;
  const LuZone Z = D.zones[z];
  const int t = blockIdx.x * HP + a;
  int i = 0, j = 0, k = 0;
  const bool ok = hyperplane_point(Z, l, t, i, j, k);
  const long long h = ok ? Z.off + hps[(long long)z * hstride + l] + t : 0;
  double v = 0.0, f[8];
  if (ok) {
    load_factors(jac, D.NP, h, m, f);
    switch (m) {
      case 0: v = lower_row<0, SCALE>(D, jac, Z, i, j, k, h); break;
      case 1: v = lower_row<1, SCALE>(D, jac, Z, i, j, k, h); break;
      case 2: v = lower_row<2, SCALE>(D, jac, Z, i, j, k, h); break;
      case 3: v = lower_row<3, SCALE>(D, jac, Z, i, j, k, h); break;
      default: v = lower_row<4, SCALE>(D, jac, Z, i, j, k, h); break;
    }
    sv[a][m] = v;
  }
  __syncthreads();
  if (!ok) return;
  D.rsd[m * D.NP + pidx(Z, i, j, k)] = d_solve(f, m, v, sv[a]);
}

// buts's two tv loops for row M of one point
template <int M>
__device__ __forceinline__ double upper_row(const LuDev& D, const double* __restrict__ jac, const LuZone& Z, int i,
                                            int j, int k, long long h) {
  const long long NP = D.NP;
  const double omega = D.omega;
  double w[5], x[5];
  load5(D.rsd, NP, pidx(Z, i, j, k + 1), w);
  double tv = omega * row_dot<2, 1, M>(jac, NP, h, w);
  load5(D.rsd, NP, pidx(Z, i, j + 1, k), w);
  load5(D.rsd, NP, pidx(Z, i + 1, j, k), x);
  tv = tv + omega * row_dot2<1, M>(jac, NP, h, w, x);
  return tv;
}

// jacu + buts at every point of hyperplane l
__global__ void __launch_bounds__(HP * 5) k_lu_upper(LuDev D, const double* __restrict__ jac,
                                                     const int* __restrict__ hps, int hstride, int l, int zone0) {
  __shared__ double sv[HP][5];
  const int m = threadIdx.y, a = threadIdx.x, z = zone0 + blockIdx.y;
  const LuZone Z = D.zones[z];
  const int t = blockIdx.x * HP + a;
  int i = 0, j = 0, k = 0;
  const bool ok = hyperplane_point(Z, l, t, i, j, k);
  const long long h = ok ? Z.off + hps[(long long)z * hstride + l] + t : 0;
  double tv = 0.0, f[8], own = 0.0;
  if (ok) {
    load_factors(jac, D.NP, h, m, f);
    own = D.rsd[m * D.NP + pidx(Z, i, j, k)];
    switch (m) {
      case 0: tv = upper_row<0>(D, jac, Z, i, j, k, h); break;
      case 1: tv = upper_row<1>(D, jac, Z, i, j, k, h); break;
      case 2: tv = upper_row<2>(D, jac, Z, i, j, k, h); break;
      case 3: tv = upper_row<3>(D, jac, Z, i, j, k, h); break;
      default: tv = upper_row<4>(D, jac, Z, i, j, k, h); break;
    }
    sv[a][m] = tv;
  }
  __syncthreads();
  if (!ok) return;
  tv = d_solve(f, m, tv, sv[a]);
  D.rsd[m * D.NP + pidx(Z, i, j, k)] = own - tv;
}

__device__ inline void face_sizes(const LuZone& Z, int nkp, long long& e, long long& s) {
  e = (long long)Z.nx * nkp;
  s = (long long)Z.ny * nkp;
}

__global__ void __launch_bounds__(TPB) k_lu_pack(LuDev D, Faces F, int nzones) {
  const int z = blockIdx.y;
  if (z >= nzones) return;
  const LuZone Z = D.zones[z];
  const int per = 2 * Z.nx + 2 * Z.ny;
  const int t = blockIdx.x * TPB + threadIdx.x;
  if (t >= per * F.nkp) return;
  const int kq = t / per, pos = t % per, k = F.klo + kq;
  long long ne, ns;
  face_sizes(Z, F.nkp, ne, ns);
  double* base = F.stage + F.zoff[z];
  int i, j;
  long long so;
  if (pos < Z.nx) {  // east face
    i = pos + 1; j = Z.ny - 1; so = 0 * ne + (long long)kq * Z.nx + pos;
  } else if (pos < 2 * Z.nx) {  // west face
    i = pos - Z.nx + 1; j = 2; so = 5 * ne + (long long)kq * Z.nx + (pos - Z.nx);
  } else if (pos < 2 * Z.nx + Z.ny) {  // south face
    i = Z.nx - 1; j = pos - 2 * Z.nx + 1; so = 10 * ne + (long long)kq * Z.ny + (j - 1);
  } else {  // north face
    i = 2; j = pos - 2 * Z.nx - Z.ny + 1; so = 10 * ne + 5 * ns + (long long)kq * Z.ny + (j - 1);
  }
  const long long p = pidx(Z, i, j, k);
  const long long stride = pos < 2 * Z.nx ? ne : ns;
#pragma unroll
  for (int m = 0; m < 5; ++m) base[so + m * stride] = D.u[m * D.NP + p];
}

// Every ghost point has one writer: j = 1 / j = ny (west / east) include the
// corners, which the reference's unpack order (south, north, west, east)
// leaves to them.
__global__ void __launch_bounds__(TPB) k_lu_unpack(LuDev D, Faces F, int nzones) {
  const int z = blockIdx.y;
  if (z >= nzones) return;
  const LuZone Z = D.zones[z];
  const int per = 2 * Z.nx + 2 * (Z.ny - 2);
  const int t = blockIdx.x * TPB + threadIdx.x;
  if (t >= per * F.nkp) return;
  const int kq = t / per, pos = t % per, k = F.klo + kq;
  int i, j, src;
  long long so, stride;
  if (pos < Z.nx) {  // west ghost j = 1 <- west zone's east face
    i = pos + 1; j = 1; src = F.nbr[4 * z + 0];
    const LuZone S = D.zones[src];
    long long ne, ns;
    face_sizes(S, F.nkp, ne, ns);
    so = F.zoff[src] + 0 * ne + (long long)kq * S.nx + (i - 1); stride = ne;
  } else if (pos < 2 * Z.nx) {  // east ghost j = ny <- east zone's west face
    i = pos - Z.nx + 1; j = Z.ny; src = F.nbr[4 * z + 1];
    const LuZone S = D.zones[src];
    long long ne, ns;
    face_sizes(S, F.nkp, ne, ns);
    so = F.zoff[src] + 5 * ne + (long long)kq * S.nx + (i - 1); stride = ne;
  } else if (pos < 2 * Z.nx + (Z.ny - 2)) {  // north ghost i = 1 <- north zone's south face
    i = 1; j = pos - 2 * Z.nx + 2; src = F.nbr[4 * z + 3];
    const LuZone S = D.zones[src];
    long long ne, ns;
    face_sizes(S, F.nkp, ne, ns);
    so = F.zoff[src] + 10 * ne + (long long)kq * S.ny + (j - 1); stride = ns;
  } else {  // south ghost i = nx <- south zone's north face
    i = Z.nx; j = pos - 2 * Z.nx - (Z.ny - 2) + 2; src = F.nbr[4 * z + 2];
    const LuZone S = D.zones[src];
    long long ne, ns;
    face_sizes(S, F.nkp, ne, ns);
    so = F.zoff[src] + 10 * ne + 5 * ns + (long long)kq * S.ny + (j - 1); stride = ns;
  }
  const long long p = pidx(Z, i, j, k);
  double g[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    g[m] = F.stage[so + m * stride];
    D.u[m * D.NP + p] = g[m];
  }
  store_prim(D.prim, D.NP, p, g);
}

// ---- norms (src/LU/l2norm.jl, src/LU/error.jl, src/LU/pintgr.jl) -----------
// WHICH 0: sum of rsd^2, 1: sum of (exact - u)^2 over the interior; one row
// of 5 partial sums per work block (fixed-order tree reduction)
template <int WHICH>
__global__ void __launch_bounds__(TPB) k_lu_norm_partial(LuDev D, const LuWork* __restrict__ work, CeTable ce,
                                                         double* partial) {
  __shared__ double sh[5][TPB];
  const LuWork w = work[blockIdx.x];
  const LuZone Z = D.zones[w.zone];
  double s[5] = {0, 0, 0, 0, 0};
  int i, j, k;
  if (decode(Z, w.first + threadIdx.x, i, j, k) && interior(Z, i, j, k)) {
    const long long p = pidx(Z, i, j, k);
    if (WHICH == 0) {
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        const double r = D.rsd[m * D.NP + p];
        s[m] = r * r;
      }
    } else {
      double e[5];
      exact_point(ce, i, j, k, Z.nx, Z.ny, Z.nz, e);
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        const double t = e[m] - D.u[m * D.NP + p];
        s[m] = t * t;
      }
    }
  }
#pragma unroll
  for (int m = 0; m < 5; ++m) sh[m][threadIdx.x] = s[m];
  __syncthreads();
  for (int h = TPB / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h)
#pragma unroll
      for (int m = 0; m < 5; ++m) sh[m][threadIdx.x] += sh[m][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x < 5) partial[(long long)blockIdx.x * 5 + threadIdx.x] = sh[threadIdx.x][0];
}

// per zone: sqrt(sum / ((nx-2)(ny-2)(nz-2))), then summed over zones in
// order into out[5] (+ out_zone[5*z + m] when non-null); one thread per m
__global__ void k_lu_norm_finish(const LuZone* zones, const int* zblock, int nzones, const double* partial,
                                 double* out, double* out_zone) {
  const int m = threadIdx.x;
  if (m >= 5) return;
  double total = 0.0;
  for (int z = 0; z < nzones; ++z) {
    double s = 0.0;
    for (int b = zblock[z]; b < zblock[z + 1]; ++b) s += partial[(long long)b * 5 + m];
    const LuZone Z = zones[z];
    const double r = sqrt(s / ((double)(Z.nx - 2) * (Z.ny - 2) * (Z.nz - 2)));
    if (out_zone) out_zone[5 * z + m] = r;
    total += r;
  }
  out[m] = total;
}

// pintgr of one zone per block (one process: ibeg = ii1, ifin = ii2,
// jbeg = ji1, jfin = ji2); frc[z] = 0.25 (frc1 + frc2 + frc3)
__global__ void __launch_bounds__(TPB) k_lu_pintgr(LuDev D, double* frc) {
  __shared__ double sh[3][TPB];
  const LuZone Z = D.zones[blockIdx.x];
  const int ibeg = ii1, ifin = Z.ii2, jbeg = ji1, jfin = Z.ji2, ifin1 = ifin - 1, jfin1 = jfin - 1;
  auto phi = [&](int i, int j, int k) {
    const long long p = pidx(Z, i, j, k);
    const double u1 = D.u[p], u2 = D.u[D.NP + p], u3 = D.u[2 * D.NP + p], u4 = D.u[3 * D.NP + p],
                 u5 = D.u[4 * D.NP + p];
    return c2 * (u5 - 0.50e+00 * (u2 * u2 + u3 * u3 + u4 * u4) / u1);
  };
  double s1 = 0.0, s2 = 0.0, s3 = 0.0;
  const int n1i = ifin1 - ibeg + 1, n1j = jfin1 - jbeg + 1, nk = Z.ki2 - 1 - ki1 + 1;
  for (int t = threadIdx.x; t < n1i * n1j; t += TPB) {
    const int i = ibeg + t % n1i, j = jbeg + t / n1i;
    s1 += (phi(i, j, ki1) + phi(i + 1, j, ki1) + phi(i, j + 1, ki1) + phi(i + 1, j + 1, ki1) + phi(i, j, Z.ki2) +
           phi(i + 1, j, Z.ki2) + phi(i, j + 1, Z.ki2) + phi(i + 1, j + 1, Z.ki2));
  }
  for (int t = threadIdx.x; t < n1i * nk; t += TPB) {
    const int i = ibeg + t % n1i, k = ki1 + t / n1i;
    s2 += (phi(i, jbeg, k) + phi(i + 1, jbeg, k) + phi(i, jbeg, k + 1) + phi(i + 1, jbeg, k + 1) + phi(i, jfin, k) +
           phi(i + 1, jfin, k) + phi(i, jfin, k + 1) + phi(i + 1, jfin, k + 1));
  }
  for (int t = threadIdx.x; t < n1j * nk; t += TPB) {
    const int j = jbeg + t % n1j, k = ki1 + t / n1j;
    s3 += (phi(ibeg, j, k) + phi(ibeg, j + 1, k) + phi(ibeg, j, k + 1) + phi(ibeg, j + 1, k + 1) + phi(ifin, j, k) +
           phi(ifin, j + 1, k) + phi(ifin, j, k + 1) + phi(ifin, j + 1, k + 1));
  }
  sh[0][threadIdx.x] = s1;
  sh[1][threadIdx.x] = s2;
  sh[2][threadIdx.x] = s3;
  __syncthreads();
  for (int h = TPB / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h)
      for (int q = 0; q < 3; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double frc1 = Z.dxi * Z.deta * sh[0][0];
    const double frc2 = Z.dxi * Z.dzeta * sh[1][0];
    const double frc3 = Z.deta * Z.dzeta * sh[2][0];
    frc[blockIdx.x] = 0.25e+00 * (frc1 + frc2 + frc3);
  }
}

// ---- layout conversion --------------------------------------------------------
// REF: [1:5, -1:nx+2, -1:ny+2, 1:nz] column-major; DENSE: [m][k][j][i].  One
// thread per double, in the host array's order (REF: the 5*nx interior
// doubles of each (j, k) row are contiguous), so that a warp's host accesses
// are contiguous: the host side may be page-locked memory read or written
// in place over the host link.
template <bool REF, bool TO_DEV>
__global__ void __launch_bounds__(TPB) k_lu_convert(LuDev D, double* field, double* host_img, int zone) {
  const LuZone Z = D.zones[zone];
  const long long t = (long long)blockIdx.x * TPB + threadIdx.x;
  if (t >= 5LL * Z.np) return;
  int m, i, j, k;
  long long h;
  if (REF) {
    const int rowlen = 5 * Z.nx;
    const int row = (int)(t / rowlen), e = (int)(t % rowlen);
    m = e % 5;
    i = e / 5 + 1;
    j = row % Z.ny + 1;
    k = row / Z.ny + 1;
    h = 5LL * (Z.nx + 4) * ((j + 1) + (long long)(Z.ny + 4) * (k - 1)) + 10 + e;
  } else {
    m = (int)(t / Z.np);
    const int q = (int)(t % Z.np);
    i = q % Z.nx + 1;
    j = (q / Z.nx) % Z.ny + 1;
    k = q / (Z.nx * Z.ny) + 1;
    h = t;
  }
  const long long p = m * D.NP + pidx(Z, i, j, k);
  if (TO_DEV)
    field[p] = host_img[h];
  else
    host_img[h] = field[p];
}

// ---- host launchers ------------------------------------------------------------
void rhs(bool erhs, const LuDev& D, const LuWork* w, int n, const double* g, const double* prim, double* out,
         cudaStream_t s) {
  if (erhs)
    k_lu_rhs<true><<<n, TPB, 0, s>>>(D, w, g, prim, out);
  else
    k_lu_rhs<false><<<n, TPB, 0, s>>>(D, w, g, prim, out);
}
void init(const LuDev& D, const LuWork* w, int n, const CeTable& ce, cudaStream_t s) {
  k_lu_init<<<n, TPB, 0, s>>>(D, w, ce);
}
void poly(const LuDev& D, const LuWork* w, int n, const CeTable& ce, cudaStream_t s) {
  k_lu_poly<<<n, TPB, 0, s>>>(D, w, ce);
}
void prim(const LuDev& D, const LuWork* w, int n, const double* g, cudaStream_t s) {
  k_lu_prim<<<n, TPB, 0, s>>>(D, w, g);
}
void pointwise(bool update, const LuDev& D, const LuWork* w, int n, double tmp, cudaStream_t s) {
  if (update)
    k_lu_pointwise<true><<<n, TPB, 0, s>>>(D, w, tmp);
  else
    k_lu_pointwise<false><<<n, TPB, 0, s>>>(D, w, tmp);
}
void jac(bool hp_order, const LuDev& D, const int* fb, int fls, const int* ri, int ls, int ks, double* jac, int z0,
         dim3 grid, cudaStream_t s) {
  if (hp_order)
    k_lu_jac<true><<<grid, TPB, 0, s>>>(D, fb, fls, ri, ls, ks, jac, z0);
  else
    k_lu_jac<false><<<grid, TPB, 0, s>>>(D, fb, fls, ri, ls, ks, jac, z0);
}
void lower(bool scale, const LuDev& D, const double* jac, const int* hps, int hstride, int l, int z0, dim3 grid,
           cudaStream_t s) {
  const dim3 b(HP, 5);
  if (scale)
    k_lu_lower<true><<<grid, b, 0, s>>>(D, jac, hps, hstride, l, z0);
  else
    k_lu_lower<false><<<grid, b, 0, s>>>(D, jac, hps, hstride, l, z0);
}
void upper(const LuDev& D, const double* jac, const int* hps, int hstride, int l, int z0, dim3 grid,
           cudaStream_t s) {
  k_lu_upper<<<grid, dim3(HP, 5), 0, s>>>(D, jac, hps, hstride, l, z0);
}
void pack(const LuDev& D, const Faces& F, int nzones, dim3 grid, cudaStream_t s) {
  k_lu_pack<<<grid, TPB, 0, s>>>(D, F, nzones);
}
void unpack(const LuDev& D, const Faces& F, int nzones, dim3 grid, cudaStream_t s) {
  k_lu_unpack<<<grid, TPB, 0, s>>>(D, F, nzones);
}
void norm_partial(int which, const LuDev& D, const LuWork* w, int n, const CeTable& ce, double* partial,
                  cudaStream_t s) {
  if (which == 0)
    k_lu_norm_partial<0><<<n, TPB, 0, s>>>(D, w, ce, partial);
  else
    k_lu_norm_partial<1><<<n, TPB, 0, s>>>(D, w, ce, partial);
}
void norm_finish(const LuZone* zones, const int* zblock, int nzones, const double* partial, double* out,
                 cudaStream_t s) {
  k_lu_norm_finish<<<1, 32, 0, s>>>(zones, zblock, nzones, partial, out, nullptr);
}
void pintgr(const LuDev& D, int nzones, double* frc, cudaStream_t s) { k_lu_pintgr<<<nzones, TPB, 0, s>>>(D, frc); }
void convert(bool ref, bool to_dev, const LuDev& D, double* field, double* img, int zone, int blocks, cudaStream_t s) {
  if (ref && to_dev)
    k_lu_convert<true, true><<<blocks, TPB, 0, s>>>(D, field, img, zone);
  else if (ref)
    k_lu_convert<true, false><<<blocks, TPB, 0, s>>>(D, field, img, zone);
  else if (to_dev)
    k_lu_convert<false, true><<<blocks, TPB, 0, s>>>(D, field, img, zone);
  else
    k_lu_convert<false, false><<<blocks, TPB, 0, s>>>(D, field, img, zone);
}

}  // namespace LU_NS
}  // namespace npbmz_lu
