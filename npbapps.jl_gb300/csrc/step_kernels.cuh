// step_kernels.cuh -- the time-step kernels: primitive variables,
// compute_rhs (+ txinvr for SP), the BT block-tridiagonal and SP scalar
// pentadiagonal line solves (with ninvr / pinvr / tzetar and add fused into
// their back substitution), and their host-side launchers.
//
// This file is compiled twice, into namespace NPBMZ_NS:
//   exact  with -fmad=false: FP64 in the reference's operation order, no FMA
//          contraction -- bit-for-bit the reference's arithmetic;
//   fast   with -fmad=true : the same FP64 code with FMA contraction, plus the
//          FP32 line-solve (mixed precision) instantiations.
// Every expression keeps the reference's operand order and parenthesisation
// (reference files cited at each kernel).
#pragma once

#include "npbmz_internal.cuh"

#ifndef NPBMZ_NS
#error "NPBMZ_NS must name the variant namespace"
#endif

namespace npbmz {
namespace NPBMZ_NS {

// ============================================================================
// Primitive variables (src/BT/rhs.jl:62-77, src/SP/rhs.jl:62-89), one thread
// per point of the padded plane (padding points compute garbage nobody reads).
// ============================================================================
// xl: x line through the point and its position on it (FP32 BT sweeps of
// the FMA build write the x-line-major state copy there), or xl < 0.
template <bool SP>
__device__ __forceinline__ void prim_point(const Fields& F, const Consts& K, int64_t p, int64_t xl, int xi) {
  const int64_t NP = F.NP;
  {
    const double u1 = F.u[p], u2 = F.u[NP + p], u3 = F.u[2 * NP + p], u4 = F.u[3 * NP + p];
#if NPBMZ_HAS_FP32
    const double rho_inv = nr_rcp(u1);  // within a few ulps of 1/u1 (FMA build)
#else
    const double rho_inv = 1.0e0 / u1;
#endif
    const double square = 0.5e0 * (u2 * u2 + u3 * u3 + u4 * u4) * rho_inv;
    health_check_ek(F, p, u1, F.u[4 * NP + p], square);
    F.prim[PR_RHOI * NP + p] = rho_inv;
    F.prim[PR_US * NP + p] = u2 * rho_inv;
    F.prim[PR_VS * NP + p] = u3 * rho_inv;
    F.prim[PR_WS * NP + p] = u4 * rho_inv;
    F.prim[PR_SQUARE * NP + p] = square;
    F.prim[PR_QS * NP + p] = square * rho_inv;
    if (SP) {
      const double u5 = F.u[4 * NP + p];
      // IEEE square root and divide in both builds: the speed of sound enters
      // the SP adjoint's finite-difference checks, which a few-ulp estimate
      // makes noisy (1/rho above stays on the Newton-Raphson estimate)
      double aux = K.c1c2 * rho_inv * (u5 - square);
      aux = sqrt(aux);
      F.prim[PR_SPEED * NP + p] = aux;
      F.prim[PR_AINV * NP + p] = 1.0e0 / aux;
    }
    if (SP && F.primf) {
      const double v[PS_HI_COUNT] = {rho_inv, u2 * rho_inv, u3 * rho_inv, u4 * rho_inv, F.prim[PR_SPEED * NP + p]};
#pragma unroll
      for (int e = 0; e < PS_HI_COUNT; ++e) {
        float hi, lo;
        split_df(v[e], hi, lo);
        F.primf[e * NP + p] = hi;
        F.primf[(PS_HI_COUNT + e) * NP + p] = lo;
        if (F.pfx && xl >= 0) {
          F.pfx[((int64_t)xi * PS_COUNT + e) * F.nlx + xl] = hi;
          F.pfx[((int64_t)xi * PS_COUNT + PS_HI_COUNT + e) * F.nlx + xl] = lo;
        }
      }
    } else if (F.primf) {
      const double v[PF_HI_COUNT] = {rho_inv, square * rho_inv, u2, u3, u4, F.u[4 * NP + p]};
#pragma unroll
      for (int e = 0; e < PF_HI_COUNT; ++e) {
        float hi, lo;
        split_df(v[e], hi, lo);
        F.primf[e * NP + p] = hi;
        F.primf[(PF_HI_COUNT + e) * NP + p] = lo;
        if (F.pfx && xl >= 0) {
          F.pfx[((int64_t)xi * PF_COUNT + e) * F.nlx + xl] = hi;
          F.pfx[((int64_t)xi * PF_COUNT + PF_HI_COUNT + e) * F.nlx + xl] = lo;
        }
      }
    }
#if NPBMZ_HAS_FP32
    if (F.flux) {
      // point functions of compute_rhs (FMA build): each is differenced by
      // both neighbours, so it is formed once here instead of twice there
      double* X = F.flux;
      const double u5 = F.u[4 * NP + p];
      const double us = u2 * rho_inv, vs = u3 * rho_inv, ws = u4 * rho_inv;
      const double press = K.c2 * (u5 - square);
      const double h = K.c1 * u5 - K.c2 * square;
      const double qs = square * rho_inv, e = u5 * rho_inv;
      X[PX_UV * NP + p] = u3 * us;
      X[PX_UW * NP + p] = u4 * us;
      X[PX_VW * NP + p] = u4 * vs;
      X[PX_XX * NP + p] = u2 * us + press;
      X[PX_YY * NP + p] = u3 * vs + press;
      X[PX_ZZ * NP + p] = u4 * ws + press;
      X[PX_EX * NP + p] = h * us;
      X[PX_EY * NP + p] = h * vs;
      X[PX_EZ * NP + p] = h * ws;
      X[PX_WX * NP + p] = K.xxcon3 * qs + K.xxcon4 * (us * us) + K.xxcon5 * e;
      X[PX_WY * NP + p] = K.yycon3 * qs + K.yycon4 * (vs * vs) + K.yycon5 * e;
      X[PX_WZ * NP + p] = K.zzcon3 * qs + K.zzcon4 * (ws * ws) + K.zzcon5 * e;
    }
#endif
  }
}

template <bool SP>
__global__ void __launch_bounds__(256) k_prim(Fields F, Consts K, int64_t lo, int64_t hi) {
  for (int64_t p = lo + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < hi; p += (int64_t)gridDim.x * blockDim.x)
    prim_point<SP>(F, K, p, -1, 0);
}

// Over the point work list (zone known): also the x-line-major state copy.
template <bool SP>
// Work-item loop (here and in the other kernels of the batched FMA step):
// CTA b takes items b, b + gridDim.x, ...; launched with one CTA per item, or
// as a persistent kernel with as many CTAs as fit on the SMs (NPBMZ_PERSIST).
__global__ void __launch_bounds__(128) k_prim_w(Fields F, Consts K, const Work* __restrict__ work, int nwork) {
  for (int it = blockIdx.x; it < nwork; it += gridDim.x) {
    const Work w = work[it];
    const ZoneDev Z = F.zones[w.zone];
    const int q = w.first + threadIdx.x;
    if (q >= Z.nx * Z.ny * Z.nz) continue;
    const int i = q % Z.nx, j = (q / Z.nx) % Z.ny, k = q / (Z.nx * Z.ny);
    prim_point<SP>(F, K, Z.off + q, xline_of(Z, j, k), i);
  }
}

// ============================================================================
// compute_rhs (src/BT/rhs.jl:4-460; SP src/SP/rhs.jl:3-452 -- the flux and
// dissipation statements are identical) and, when TX (the SP step), txinvr
// (src/SP/txinvr.jl:5-56).  One thread per zone point; boundary points copy
// the forcing, as the reference's `rhs = forcing` over the whole cell does.
// Per element the order of updates is the reference's: forcing, xi flux, xi
// dissipation, eta flux, eta dissipation, zeta flux, zeta dissipation, *dt.
// NORM: also accumulate this CTA's sum of rhs^2 (interior, before txinvr)
// into partials[blockIdx.x][5] (each CTA covers points of one zone).
// ============================================================================

// Fourth-order dissipation term at position q of an axis of n points
// (1 <= q <= n-2): the start / middle / end stencils of the reference,
// applied in the reference's order when n is so small that they overlap.
__device__ __forceinline__ void dissip(double& r, int q, int n, double dssp, double um2, double um1, double u0,
                                       double up1, double up2) {
  if (q == 1) r -= dssp * (5.0e0 * u0 - 4.0e0 * up1 + up2);
  if (q == 2) r -= dssp * (-4.0e0 * um1 + 6.0e0 * u0 - 4.0e0 * up1 + up2);
  if (q >= 3 && q <= n - 4) r -= dssp * (um2 - 4.0e0 * um1 + 6.0 * u0 - 4.0e0 * up1 + up2);
  if (q == n - 3) r -= dssp * (um2 - 4.0e0 * um1 + 6.0e0 * u0 - 4.0e0 * up1);
  if (q == n - 2) r -= dssp * (um2 - 4.0e0 * um1 + 5.0e0 * u0);
}

// Safe neighbour load along an axis: positions outside 0..n-1 are never used
// by dissip() (their stencil weight is absent), so they read the centre.
__device__ __forceinline__ double ld_axis(const double* __restrict__ a, int64_t p, int64_t st, int q, int d, int n) {
  const int qq = q + d;
  return (qq >= 0 && qq < n) ? a[p + d * st] : a[p];
}

// Weighted form of the dissipation stencils at position q of an axis of n
// points: the sum of the start / middle / end stencils that apply at q.  Used
// by the FMA build (no lane divergence at zone edges); the exact build keeps
// dissip() and the reference's operation order.
__device__ __forceinline__ void dissip_weights(int q, int n, double w[5]) {
  w[0] = w[1] = w[2] = w[3] = w[4] = 0.0;
  if (q == 1) { w[2] += 5.0; w[3] -= 4.0; w[4] += 1.0; }
  if (q == 2) { w[1] -= 4.0; w[2] += 6.0; w[3] -= 4.0; w[4] += 1.0; }
  if (q >= 3 && q <= n - 4) { w[0] += 1.0; w[1] -= 4.0; w[2] += 6.0; w[3] -= 4.0; w[4] += 1.0; }
  if (q == n - 3) { w[0] += 1.0; w[1] -= 4.0; w[2] += 6.0; w[3] -= 4.0; }
  if (q == n - 2) { w[0] += 1.0; w[1] -= 4.0; w[2] += 5.0; }
}

#if NPBMZ_HAS_FP32
#define NPBMZ_DISSIP(r, q, n, dssp, um2, um1, u0, up1, up2)                                        \
  do {                                                                                              \
    double w_[5];                                                                                   \
    dissip_weights((q), (n), w_);                                                                   \
    (r) -= (dssp) * (w_[0] * (um2) + w_[1] * (um1) + w_[2] * (u0) + w_[3] * (up1) + w_[4] * (up2)); \
  } while (0)
#else
#define NPBMZ_DISSIP(r, q, n, dssp, um2, um1, u0, up1, up2) dissip((r), (q), (n), (dssp), (um2), (um1), (u0), (up1), (up2))
#endif

// One thread per INTERIOR point of a zone (the work list counts interior
// points only): the boundary rhs equals the forcing and no solve rewrites
// it, so it is set when the forcing or rhs is set, not every step.
template <bool TX, bool NORM>
__global__ void __launch_bounds__(128) k_rhs(Fields F, Consts K, const Work* __restrict__ work,
                                             double* __restrict__ partials) {
  __shared__ double red[5 * 128];
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int64_t NP = F.NP;
  const int ix = Z.nx - 2, iy = Z.ny - 2;
  const int ni = ix * iy * (Z.nz - 2);
  const int t = w.first + threadIdx.x;
  double sq[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (t < ni) {
    const int i = 1 + t % ix, j = 1 + (t / ix) % iy, k = 1 + t / (ix * iy);
    const int64_t p = Z.off + ((int64_t)k * Z.ny + j) * Z.nx + i;
    {
      const double* __restrict__ u = F.u;
      const double* __restrict__ pr = F.prim;
      const double* us = pr + PR_US * NP;
      const double* vs = pr + PR_VS * NP;
      const double* ws = pr + PR_WS * NP;
      const double* qs = pr + PR_QS * NP;
      const double* sqr = pr + PR_SQUARE * NP;
      const double* ri = pr + PR_RHOI * NP;
      double r[5];
      for (int m = 0; m < 5; ++m) r[m] = F.forcing[m * NP + p];
      const int64_t sx = 1, sy = Z.nx, sz = (int64_t)Z.nx * Z.ny;
      const double c1 = K.c1, c2 = K.c2, con43 = K.con43, dssp = K.dssp;
      // ---------------- xi direction ----------------
      {
        const int64_t a = p + sx, b = p - sx;
        const double uijk = us[p], up1 = us[a], um1 = us[b];
        r[0] += K.dx1tx1 * (u[a] - 2.0e0 * u[p] + u[b]) - K.tx2 * (u[NP + a] - u[NP + b]);
        r[1] += K.dx2tx1 * (u[NP + a] - 2.0e0 * u[NP + p] + u[NP + b]) + K.xxcon2 * con43 * (up1 - 2.0e0 * uijk + um1) -
                K.tx2 * (u[NP + a] * up1 - u[NP + b] * um1 + (u[4 * NP + a] - sqr[a] - u[4 * NP + b] + sqr[b]) * c2);
        r[2] += K.dx3tx1 * (u[2 * NP + a] - 2.0e0 * u[2 * NP + p] + u[2 * NP + b]) +
                K.xxcon2 * (vs[a] - 2.0e0 * vs[p] + vs[b]) - K.tx2 * (u[2 * NP + a] * up1 - u[2 * NP + b] * um1);
        r[3] += K.dx4tx1 * (u[3 * NP + a] - 2.0e0 * u[3 * NP + p] + u[3 * NP + b]) +
                K.xxcon2 * (ws[a] - 2.0e0 * ws[p] + ws[b]) - K.tx2 * (u[3 * NP + a] * up1 - u[3 * NP + b] * um1);
        r[4] += K.dx5tx1 * (u[4 * NP + a] - 2.0e0 * u[4 * NP + p] + u[4 * NP + b]) +
                K.xxcon3 * (qs[a] - 2.0e0 * qs[p] + qs[b]) + K.xxcon4 * (up1 * up1 - 2.0e0 * uijk * uijk + um1 * um1) +
                K.xxcon5 * (u[4 * NP + a] * ri[a] - 2.0e0 * u[4 * NP + p] * ri[p] + u[4 * NP + b] * ri[b]) -
                K.tx2 * ((c1 * u[4 * NP + a] - c2 * sqr[a]) * up1 - (c1 * u[4 * NP + b] - c2 * sqr[b]) * um1);
        for (int m = 0; m < 5; ++m) {
          const double* um = u + m * NP;
          NPBMZ_DISSIP(r[m], i, Z.nx, dssp, ld_axis(um, p, sx, i, -2, Z.nx), um[p - sx], um[p], um[p + sx],
                       ld_axis(um, p, sx, i, 2, Z.nx));
        }
      }
      // ---------------- eta direction ----------------
      {
        const int64_t a = p + sy, b = p - sy;
        const double vijk = vs[p], vp1 = vs[a], vm1 = vs[b];
        r[0] += K.dy1ty1 * (u[a] - 2.0e0 * u[p] + u[b]) - K.ty2 * (u[2 * NP + a] - u[2 * NP + b]);
        r[1] += K.dy2ty1 * (u[NP + a] - 2.0e0 * u[NP + p] + u[NP + b]) + K.yycon2 * (us[a] - 2.0e0 * us[p] + us[b]) -
                K.ty2 * (u[NP + a] * vp1 - u[NP + b] * vm1);
        r[2] += K.dy3ty1 * (u[2 * NP + a] - 2.0e0 * u[2 * NP + p] + u[2 * NP + b]) +
                K.yycon2 * con43 * (vp1 - 2.0e0 * vijk + vm1) -
                K.ty2 * (u[2 * NP + a] * vp1 - u[2 * NP + b] * vm1 + (u[4 * NP + a] - sqr[a] - u[4 * NP + b] + sqr[b]) * c2);
        r[3] += K.dy4ty1 * (u[3 * NP + a] - 2.0e0 * u[3 * NP + p] + u[3 * NP + b]) +
                K.yycon2 * (ws[a] - 2.0e0 * ws[p] + ws[b]) - K.ty2 * (u[3 * NP + a] * vp1 - u[3 * NP + b] * vm1);
        r[4] += K.dy5ty1 * (u[4 * NP + a] - 2.0e0 * u[4 * NP + p] + u[4 * NP + b]) +
                K.yycon3 * (qs[a] - 2.0e0 * qs[p] + qs[b]) + K.yycon4 * (vp1 * vp1 - 2.0e0 * vijk * vijk + vm1 * vm1) +
                K.yycon5 * (u[4 * NP + a] * ri[a] - 2.0e0 * u[4 * NP + p] * ri[p] + u[4 * NP + b] * ri[b]) -
                K.ty2 * ((c1 * u[4 * NP + a] - c2 * sqr[a]) * vp1 - (c1 * u[4 * NP + b] - c2 * sqr[b]) * vm1);
        for (int m = 0; m < 5; ++m) {
          const double* um = u + m * NP;
          NPBMZ_DISSIP(r[m], j, Z.ny, dssp, ld_axis(um, p, sy, j, -2, Z.ny), um[p - sy], um[p], um[p + sy],
                       ld_axis(um, p, sy, j, 2, Z.ny));
        }
      }
      // ---------------- zeta direction ----------------
      {
        const int64_t a = p + sz, b = p - sz;
        const double wijk = ws[p], wp1 = ws[a], wm1 = ws[b];
        r[0] += K.dz1tz1 * (u[a] - 2.0e0 * u[p] + u[b]) - K.tz2 * (u[3 * NP + a] - u[3 * NP + b]);
        r[1] += K.dz2tz1 * (u[NP + a] - 2.0e0 * u[NP + p] + u[NP + b]) + K.zzcon2 * (us[a] - 2.0e0 * us[p] + us[b]) -
                K.tz2 * (u[NP + a] * wp1 - u[NP + b] * wm1);
        r[2] += K.dz3tz1 * (u[2 * NP + a] - 2.0e0 * u[2 * NP + p] + u[2 * NP + b]) +
                K.zzcon2 * (vs[a] - 2.0e0 * vs[p] + vs[b]) - K.tz2 * (u[2 * NP + a] * wp1 - u[2 * NP + b] * wm1);
        r[3] += K.dz4tz1 * (u[3 * NP + a] - 2.0e0 * u[3 * NP + p] + u[3 * NP + b]) +
                K.zzcon2 * con43 * (wp1 - 2.0e0 * wijk + wm1) -
                K.tz2 * (u[3 * NP + a] * wp1 - u[3 * NP + b] * wm1 + (u[4 * NP + a] - sqr[a] - u[4 * NP + b] + sqr[b]) * c2);
        r[4] += K.dz5tz1 * (u[4 * NP + a] - 2.0e0 * u[4 * NP + p] + u[4 * NP + b]) +
                K.zzcon3 * (qs[a] - 2.0e0 * qs[p] + qs[b]) + K.zzcon4 * (wp1 * wp1 - 2.0e0 * wijk * wijk + wm1 * wm1) +
                K.zzcon5 * (u[4 * NP + a] * ri[a] - 2.0e0 * u[4 * NP + p] * ri[p] + u[4 * NP + b] * ri[b]) -
                K.tz2 * ((c1 * u[4 * NP + a] - c2 * sqr[a]) * wp1 - (c1 * u[4 * NP + b] - c2 * sqr[b]) * wm1);
        for (int m = 0; m < 5; ++m) {
          const double* um = u + m * NP;
          NPBMZ_DISSIP(r[m], k, Z.nz, dssp, ld_axis(um, p, sz, k, -2, Z.nz), um[p - sz], um[p], um[p + sz],
                       ld_axis(um, p, sz, k, 2, Z.nz));
        }
      }
      for (int m = 0; m < 5; ++m) r[m] *= K.dt;
      if (NORM)
        for (int m = 0; m < 5; ++m) sq[m] = r[m] * r[m];
      if (TX) {
        // txinvr (src/SP/txinvr.jl:28-49)
        const double ru1 = ri[p], uu = us[p], vv = vs[p], ww = ws[p], ac = pr[PR_SPEED * NP + p];
        const double ac2inv = 1.0 / (ac * ac);
        const double r1 = r[0], r2 = r[1], r3 = r[2], r4 = r[3], r5 = r[4];
        const double t1 = K.c2 * ac2inv * (qs[p] * r1 - uu * r2 - vv * r3 - ww * r4 + r5);
        const double t2 = K.bt * ru1 * (uu * r1 - r2);
        const double t3 = (K.bt * ru1 * ac) * t1;
        r[0] = r1 - t1;
        r[1] = -ru1 * (ww * r1 - r4);
        r[2] = ru1 * (vv * r1 - r3);
        r[3] = -t2 + t3;
        r[4] = t2 + t3;
      }
      for (int m = 0; m < 5; ++m) F.rhs[m * NP + p] = r[m];
    }
  }
  if (NORM) {
    block_sum5(sq, red);
    if (threadIdx.x == 0)
      for (int m = 0; m < 5; ++m) partials[blockIdx.x * 5 + m] = sq[m];
  }
}

#if NPBMZ_HAS_FP32
// ============================================================================
// compute_rhs, FMA build: the same terms as k_rhs, regrouped to cut FP64
// work (this path is bound by GB300's FP64 pipe, not by HBM):
//   - the fluxes and viscous energy terms come from the point functions the
//     primitive kernel wrote (PX_*), each formed once per point;
//   - per direction and variable, the second difference d*t1*D2(u) and the
//     dissipation are one 5-point stencil with weights from LinWeights,
//     staged in shared memory;
//   - the momentum viscous terms difference the velocity planes.
// The sum is algebraically the reference's; rounding differs (within 1e-12
// of the oracle, tested).
// ============================================================================
__device__ __forceinline__ int dissip_class(int q, int n) {
  return (q == 1) | ((q == 2) << 1) | ((q >= 3 && q <= n - 4) << 2) | ((q == n - 3) << 3) | ((q == n - 2) << 4);
}

// One direction: stride st, position q of n, weights W (5; the centre one,
// W[2], is summed over the directions by the caller), flux planes of
// variables 1..4 (fx[0..3]), normal momentum plane (variable a = 1 + dir),
// velocity-term factors vc[3] (their centre term likewise), viscous energy
// plane wv, t2; every factor carries dt.
__device__ __forceinline__ void rhs_dir(double r[5], const double* __restrict__ u, int64_t NP, int64_t p, int64_t st,
                                        int q, int n, const double* __restrict__ W, const double* const fx[4],
                                        const double* __restrict__ un, const double* const vel[3], const double vc[3],
                                        const double* __restrict__ wv, double t2, double dt) {
  const int64_t pm2 = q >= 2 ? p - 2 * st : p;
  const int64_t pp2 = q + 2 <= n - 1 ? p + 2 * st : p;
  const double w0 = W[0], w1 = W[1], w3 = W[3], w4 = W[4];
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    const double* um = u + m * NP;
    double s = fma(w1, um[p - st], r[m]);
    s = fma(w3, um[p + st], s);
    s = fma(w0, um[pm2], s);
    r[m] = fma(w4, um[pp2], s);
  }
  r[0] = fma(-t2, un[p + st] - un[p - st], r[0]);
#pragma unroll
  for (int m = 0; m < 4; ++m) r[m + 1] = fma(-t2, fx[m][p + st] - fx[m][p - st], r[m + 1]);
#pragma unroll
  for (int m = 0; m < 3; ++m) r[m + 1] = fma(vc[m], vel[m][p + st] + vel[m][p - st], r[m + 1]);
  r[4] = fma(dt, (wv[p + st] + wv[p - st]) - 2.0 * wv[p], r[4]);
}

// One work item (128 interior points of one zone) of compute_rhs; wt: the
// dissipation weights in shared memory, red: the NORM reduction scratch.
template <bool TX, bool NORM>
__device__ __forceinline__ void rhs_flux_item(const Fields& F, const Consts& K, const RhsF64Consts& RC, const Work w,
                                              int it, double* __restrict__ partials, const double* wt, double* red) {
  const ZoneDev Z = F.zones[w.zone];
  const int64_t NP = F.NP;
  const int ix = Z.nx - 2, iy = Z.ny - 2;
  const int ni = ix * iy * (Z.nz - 2);
  const int t = w.first + threadIdx.x;
  double sq[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (t < ni) {
    const int i = 1 + t % ix, j = 1 + (t / ix) % iy, k = 1 + t / (ix * iy);
    const int64_t p = Z.off + ((int64_t)k * Z.ny + j) * Z.nx + i;
    const double* __restrict__ u = F.u;
    const double* __restrict__ pr = F.prim;
    const double* __restrict__ X = F.flux;
    const double* vel[3] = {pr + PR_US * NP, pr + PR_VS * NP, pr + PR_WS * NP};
    double r[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) r[m] = F.fdt[m * NP + p];
    const double* Wx = wt + (0 * 32 + dissip_class(i, Z.nx)) * 5;
    const double* Wy = wt + (1 * 32 + dissip_class(j, Z.ny)) * 5;
    const double* Wz = wt + (2 * 32 + dissip_class(k, Z.nz)) * 5;
    {
      const double* fx[4] = {X + PX_XX * NP, X + PX_UV * NP, X + PX_UW * NP, X + PX_EX * NP};
      rhs_dir(r, u, NP, p, 1, i, Z.nx, Wx, fx, u + NP, vel, RC.vc[0], X + PX_WX * NP, RC.t2[0], RC.dt);
    }
    {
      const double* fx[4] = {X + PX_UV * NP, X + PX_YY * NP, X + PX_VW * NP, X + PX_EY * NP};
      rhs_dir(r, u, NP, p, Z.nx, j, Z.ny, Wy, fx, u + 2 * NP, vel, RC.vc[1], X + PX_WY * NP, RC.t2[1], RC.dt);
    }
    {
      const double* fx[4] = {X + PX_UW * NP, X + PX_VW * NP, X + PX_ZZ * NP, X + PX_EZ * NP};
      rhs_dir(r, u, NP, p, (int64_t)Z.nx * Z.ny, k, Z.nz, Wz, fx, u + 3 * NP, vel, RC.vc[2], X + PX_WZ * NP,
              RC.t2[2], RC.dt);
    }
    // centre point: the three directions' stencil weights and velocity
    // factors summed first
    const double wc = (Wx[2] + Wy[2]) + Wz[2];
#pragma unroll
    for (int m = 0; m < 5; ++m) r[m] = fma(wc, u[m * NP + p], r[m]);
#pragma unroll
    for (int m = 0; m < 3; ++m) r[m + 1] = fma(RC.vcc[m], vel[m][p], r[m + 1]);
    if (NORM)
#pragma unroll
      for (int m = 0; m < 5; ++m) sq[m] = r[m] * r[m];
    if (TX) {
      // txinvr (src/SP/txinvr.jl:28-49); 1/speed^2 as ainv^2
      const double ru1 = pr[PR_RHOI * NP + p], uu = vel[0][p], vv = vel[1][p], ww = vel[2][p];
      const double ac = pr[PR_SPEED * NP + p], ainv = pr[PR_AINV * NP + p];
      const double ac2inv = ainv * ainv;
      const double r1 = r[0], r2 = r[1], r3 = r[2], r4 = r[3], r5 = r[4];
      const double t1 = K.c2 * ac2inv * (pr[PR_QS * NP + p] * r1 - uu * r2 - vv * r3 - ww * r4 + r5);
      const double t2 = K.bt * ru1 * (uu * r1 - r2);
      const double t3 = (K.bt * ru1 * ac) * t1;
      r[0] = r1 - t1;
      r[1] = -ru1 * (ww * r1 - r4);
      r[2] = ru1 * (vv * r1 - r3);
      r[3] = -t2 + t3;
      r[4] = t2 + t3;
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) F.rhs[m * NP + p] = r[m];
    if (F.rdx) {  // b of the x sweep, x-line-major
      const int64_t xl = xline_of(Z, j, k);
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        float hi, lo;
        split_df(r[m], hi, lo);
        F.rdx[((int64_t)i * 10 + m) * F.nlx + xl] = hi;
        F.rdx[((int64_t)i * 10 + 5 + m) * F.nlx + xl] = lo;
      }
    } else if (F.rdf) {
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        float hi, lo;
        split_df(r[m], hi, lo);
        F.rdf[m * NP + p] = hi;
        F.rdf[(5 + m) * NP + p] = lo;
      }
    }
  }
  if (NORM) {
    block_sum5(sq, red);
    if (threadIdx.x == 0)
      for (int m = 0; m < 5; ++m) partials[it * 5 + m] = sq[m];
  }
}

template <bool TX, bool NORM>
__global__ void __launch_bounds__(128) k_rhs_flux(Fields F, Consts K, RhsF64Consts RC, const Work* __restrict__ work,
                                                  int nwork, double* __restrict__ partials) {
  __shared__ double red[NORM ? 5 * 128 : 1];
  __shared__ double wt[3 * 32 * 5];
  for (int e = threadIdx.x; e < 3 * 32 * 5; e += blockDim.x) wt[e] = (&RC.w[0][0][0])[e];
  __syncthreads();
  for (int it = blockIdx.x; it < nwork; it += gridDim.x) rhs_flux_item<TX, NORM>(F, K, RC, work[it], it, partials, wt, red);
}

// The two end points of every x line in the x-line-major double-float rhs
// copy: the forcing, as rhs holds there (one thread per x line).
__global__ void __launch_bounds__(128) k_xline_ends(Fields F, const Work* __restrict__ work) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int line = w.first + threadIdx.x;
  if (line >= zone_lines(Z, 0)) return;
  int64_t base, st;
  line_geometry(Z, 0, line, base, st);
  const int64_t gl = Z.lineoff[0] + line;
  const int ends[2] = {0, Z.nx - 1};
#pragma unroll
  for (int e = 0; e < 2; ++e)
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const double v = F.forcing[m * F.NP + base + ends[e]];
      const float hi = __double2float_rn(v);
      F.rdx[((int64_t)ends[e] * 10 + m) * F.nlx + gl] = hi;
      F.rdx[((int64_t)ends[e] * 10 + 5 + m) * F.nlx + gl] = __double2float_rn(v - (double)hi);
    }
}

// dst = a * src (n values)
__global__ void __launch_bounds__(256) k_scale(const double* __restrict__ src, double* __restrict__ dst, double a,
                                               int64_t n) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    dst[t] = a * src[t];
}

// dst (double-float planes 0..4 hi, 5..9 lo) <- src (5 FP64 planes)
__global__ void __launch_bounds__(256) k_split_df(const double* __restrict__ src, float* __restrict__ dst, int64_t NP) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < 5 * NP; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = t / NP, p = t - m * NP;
    const double v = src[t];
    const float hi = __double2float_rn(v);
    dst[m * NP + p] = hi;
    dst[(5 + m) * NP + p] = __double2float_rn(v - (double)hi);
  }
}
#endif  // NPBMZ_HAS_FP32

// ============================================================================
// BT block-tridiagonal line solve, one thread per line.
// Reference: x_solve_cell / y_solve_cell / z_solve_cell and the back
// substitutions (src/BT/x_solve.jl:444-488,501-1746, src/BT/y_solve.jl:443-820,
// src/BT/z_solve.jl:438-864) with matvec_sub, matmul_sub2, binvcrhs, binvrhs
// (src/BT/solve_subs.jl:4-37,333-460,468-862).
//
// The Jacobians fjac/njac have structural zeros; terms with a structural
// zero factor are skipped.  That is exact: in the reference such a term
// contributes +-0, and x - (+-0) == x for every nonzero x.  The boundary
// steps (binvcrhs at point 0 with B = I, C = 0; binvrhs at point n-1 with
// A = 0, B = I; back substitution at point 0 with C = 0) are exact no-ops in
// the reference and are skipped for the same reason.
// C'_p (the 5x5 block left by binvcrhs) goes to the line scratch
// lhsc[(p*25 + e) * nlt + global_line] (coalesced across the CTA's lines);
// the forward-eliminated rhs goes back into rhs in place.
// ============================================================================

// Structural nonzeros of fjac / njac per sweep direction.
template <int DIR>
__host__ __device__ constexpr bool fnz(int a, int b) {
  return DIR == 0 ? (a == 0 ? b == 1 : a == 1 ? true : a == 2 ? (b <= 2) : a == 3 ? (b == 0 || b == 1 || b == 3) : true)
       : DIR == 1 ? (a == 0 ? b == 2 : a == 1 ? (b <= 2) : a == 2 ? true : a == 3 ? (b == 0 || b == 2 || b == 3) : true)
                  : (a == 0 ? b == 3 : a == 1 ? (b == 0 || b == 1 || b == 3) : a == 2 ? (b == 0 || b == 2 || b == 3) : true);
}
__host__ __device__ constexpr bool nnz(int a, int b) {
  return a == 0 ? false : a == 4 ? true : (b == 0 || b == a);
}
template <int DIR>
__host__ __device__ constexpr bool anz(int a, int b) { return fnz<DIR>(a, b) || nnz(a, b) || a == b; }
__host__ __device__ constexpr bool bnz(int a, int b) { return nnz(a, b) || a == b; }

// fjac / njac at one point (src/BT/x_solve.jl:536-609, y_solve.jl:543-613,
// z_solve.jl:537-618); only structural nonzeros are written.
template <int DIR, typename T>
__device__ __forceinline__ void bt_jac(const Consts& K, T tmp1, T u2, T u3, T u4, T u5, T q, T f[5][5], T n[5][5]) {
  const T c1 = kv<T>(K.c1, K.f_c1), c2 = kv<T>(K.c2, K.f_c2), c3c4 = kv<T>(K.c3c4, K.f_c3c4);
  const T c1345 = kv<T>(K.c1345, K.f_c1345), con43 = kv<T>(K.con43, K.f_con43);
  const T tmp2 = tmp1 * tmp1;
  const T tmp3 = tmp1 * tmp2;
  if (DIR == 0) {
    f[0][1] = (T)1.0;
    f[1][0] = -(u2 * tmp2 * u2) + c2 * q;
    f[1][1] = ((T)2.0 - c2) * (u2 * tmp1);
    f[1][2] = -c2 * (u3 * tmp1);
    f[1][3] = -c2 * (u4 * tmp1);
    f[1][4] = c2;
    f[2][0] = -(u2 * u3) * tmp2;
    f[2][1] = u3 * tmp1;
    f[2][2] = u2 * tmp1;
    f[3][0] = -(u2 * u4) * tmp2;
    f[3][1] = u4 * tmp1;
    f[3][3] = u2 * tmp1;
    f[4][0] = (c2 * (T)2.0 * q - c1 * (u5 * tmp1)) * (u2 * tmp1);
    f[4][1] = c1 * u5 * tmp1 - c2 * (u2 * u2 * tmp2 + q);
    f[4][2] = -c2 * (u3 * u2) * tmp2;
    f[4][3] = -c2 * (u4 * u2) * tmp2;
    f[4][4] = c1 * (u2 * tmp1);
    n[1][0] = -con43 * c3c4 * tmp2 * u2;
    n[1][1] = con43 * c3c4 * tmp1;
    n[2][0] = -c3c4 * tmp2 * u3;
    n[2][2] = c3c4 * tmp1;
    n[3][0] = -c3c4 * tmp2 * u4;
    n[3][3] = c3c4 * tmp1;
    n[4][0] = -(con43 * c3c4 - c1345) * tmp3 * (u2 * u2) - (c3c4 - c1345) * tmp3 * (u3 * u3) -
              (c3c4 - c1345) * tmp3 * (u4 * u4) - c1345 * tmp2 * u5;
    n[4][1] = (con43 * c3c4 - c1345) * tmp2 * u2;
    n[4][2] = (c3c4 - c1345) * tmp2 * u3;
    n[4][3] = (c3c4 - c1345) * tmp2 * u4;
    n[4][4] = (c1345) * tmp1;
  } else if (DIR == 1) {
    f[0][2] = (T)1.0;
    f[1][0] = -(u2 * u3) * tmp2;
    f[1][1] = u3 * tmp1;
    f[1][2] = u2 * tmp1;
    f[2][0] = -(u3 * u3 * tmp2) + c2 * q;
    f[2][1] = -c2 * u2 * tmp1;
    f[2][2] = ((T)2.0 - c2) * u3 * tmp1;
    f[2][3] = -c2 * u4 * tmp1;
    f[2][4] = c2;
    f[3][0] = -(u3 * u4) * tmp2;
    f[3][2] = u4 * tmp1;
    f[3][3] = u3 * tmp1;
    f[4][0] = (c2 * (T)2.0 * q - c1 * u5 * tmp1) * u3 * tmp1;
    f[4][1] = -c2 * u2 * u3 * tmp2;
    f[4][2] = c1 * u5 * tmp1 - c2 * (q + u3 * u3 * tmp2);
    f[4][3] = -c2 * (u3 * u4) * tmp2;
    f[4][4] = c1 * u3 * tmp1;
    n[1][0] = -c3c4 * tmp2 * u2;
    n[1][1] = c3c4 * tmp1;
    n[2][0] = -con43 * c3c4 * tmp2 * u3;
    n[2][2] = con43 * c3c4 * tmp1;
    n[3][0] = -c3c4 * tmp2 * u4;
    n[3][3] = c3c4 * tmp1;
    n[4][0] = -(c3c4 - c1345) * tmp3 * (u2 * u2) - (con43 * c3c4 - c1345) * tmp3 * (u3 * u3) -
              (c3c4 - c1345) * tmp3 * (u4 * u4) - c1345 * tmp2 * u5;
    n[4][1] = (c3c4 - c1345) * tmp2 * u2;
    n[4][2] = (con43 * c3c4 - c1345) * tmp2 * u3;
    n[4][3] = (c3c4 - c1345) * tmp2 * u4;
    n[4][4] = (c1345) * tmp1;
  } else {
    const T c3 = kv<T>(K.c3, K.f_c3), c4 = kv<T>(K.c4, K.f_c4);
    f[0][3] = (T)1.0;
    f[1][0] = -(u2 * u4) * tmp2;
    f[1][1] = u4 * tmp1;
    f[1][3] = u2 * tmp1;
    f[2][0] = -(u3 * u4) * tmp2;
    f[2][2] = u4 * tmp1;
    f[2][3] = u3 * tmp1;
    f[3][0] = -(u4 * u4 * tmp2) + c2 * q;
    f[3][1] = -c2 * u2 * tmp1;
    f[3][2] = -c2 * u3 * tmp1;
    f[3][3] = ((T)2.0 - c2) * u4 * tmp1;
    f[3][4] = c2;
    f[4][0] = (c2 * (T)2.0 * q - c1 * (u5 * tmp1)) * (u4 * tmp1);
    f[4][1] = -c2 * (u2 * u4) * tmp2;
    f[4][2] = -c2 * (u3 * u4) * tmp2;
    f[4][3] = c1 * (u5 * tmp1) - c2 * (q + u4 * u4 * tmp2);
    f[4][4] = c1 * u4 * tmp1;
    n[1][0] = -c3c4 * tmp2 * u2;
    n[1][1] = c3c4 * tmp1;
    n[2][0] = -c3c4 * tmp2 * u3;
    n[2][2] = c3c4 * tmp1;
    n[3][0] = -con43 * c3c4 * tmp2 * u4;
    n[3][3] = con43 * c3 * c4 * tmp1;
    n[4][0] = -(c3c4 - c1345) * tmp3 * (u2 * u2) - (c3c4 - c1345) * tmp3 * (u3 * u3) -
              (con43 * c3c4 - c1345) * tmp3 * (u4 * u4) - c1345 * tmp2 * u5;
    n[4][1] = (c3c4 - c1345) * tmp2 * u2;
    n[4][2] = (c3c4 - c1345) * tmp2 * u3;
    n[4][3] = (con43 * c3c4 - c1345) * tmp2 * u4;
    n[4][4] = (c1345) * tmp1;
  }
}

// lhsa at the point after the Jacobian point: -tmp2*f - tmp1*n - tmp1*d (diag).
template <int DIR, typename T>
__device__ __forceinline__ void bt_asm_a(const T f[5][5], const T n[5][5], T tmp1, T tmp2, const T dd[5], T A[5][5]) {
#pragma unroll
  for (int a = 0; a < 5; ++a)
#pragma unroll
    for (int b = 0; b < 5; ++b) {
      if (!anz<DIR>(a, b)) continue;
      T t;
      bool have = false;
      if (fnz<DIR>(a, b)) { t = -tmp2 * f[a][b]; have = true; }
      if (nnz(a, b)) { t = have ? t - tmp1 * n[a][b] : -(tmp1 * n[a][b]); have = true; }
      if (a == b) { t = have ? t - tmp1 * dd[a] : -(tmp1 * dd[a]); }
      A[a][b] = t;
    }
}

// lhsc at the point before the Jacobian point: tmp2*f - tmp1*n - tmp1*d (diag).
template <int DIR, typename T>
__device__ __forceinline__ void bt_asm_c(const T f[5][5], const T n[5][5], T tmp1, T tmp2, const T dd[5], T C[5][5]) {
#pragma unroll
  for (int a = 0; a < 5; ++a)
#pragma unroll
    for (int b = 0; b < 5; ++b) {
      T t = (T)0.0;
      bool have = false;
      if (fnz<DIR>(a, b)) { t = tmp2 * f[a][b]; have = true; }
      if (nnz(a, b)) { t = have ? t - tmp1 * n[a][b] : -(tmp1 * n[a][b]); have = true; }
      if (a == b) { t = have ? t - tmp1 * dd[a] : -(tmp1 * dd[a]); }
      C[a][b] = t;
    }
}

// lhsb at the Jacobian point: 1 + tmp1*2*n + tmp1*2*d (diag), tmp1*2*n off-diag.
template <typename T>
__device__ __forceinline__ void bt_asm_b(const T n[5][5], T tmp1, const T dd[5], T B[5][5]) {
#pragma unroll
  for (int a = 0; a < 5; ++a)
#pragma unroll
    for (int b = 0; b < 5; ++b) {
      if (!bnz(a, b)) continue;
      if (a == b) {
        T t = (T)1.0;
        if (nnz(a, b)) t = t + tmp1 * (T)2.0 * n[a][b];
        B[a][b] = t + tmp1 * (T)2.0 * dd[a];
      } else {
        B[a][b] = tmp1 * (T)2.0 * n[a][b];
      }
    }
}

// Pivot reciprocal: IEEE division in FP64 (the reference's arithmetic); in
// the FP32 solves, which a double-float refinement corrects, the fast
// reciprocal (within 2 ulp).
template <typename T>
__device__ __forceinline__ T pivot_recip(T b) { return (T)1.0 / b; }
template <>
__device__ __forceinline__ float pivot_recip<float>(float b) { return __fdividef(1.0f, b); }

// binvcrhs (src/BT/solve_subs.jl:468-723): Gauss-Jordan on B, no pivoting,
// applied to C and r.
template <typename T>
__device__ __forceinline__ void binvcrhs(T B[5][5], T C[5][5], T r[5]) {
#pragma unroll
  for (int p = 0; p < 5; ++p) {
    const T pivot = pivot_recip<T>(B[p][p]);
#pragma unroll
    for (int c = p + 1; c < 5; ++c) B[p][c] *= pivot;
#pragma unroll
    for (int c = 0; c < 5; ++c) C[p][c] *= pivot;
    r[p] *= pivot;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      if (q == p) continue;
      const T coeff = B[q][p];
#pragma unroll
      for (int c = p + 1; c < 5; ++c) B[q][c] -= coeff * B[p][c];
#pragma unroll
      for (int c = 0; c < 5; ++c) C[q][c] -= coeff * C[p][c];
      r[q] -= coeff * r[p];
    }
  }
}

template <int DIR, typename T>
__device__ __forceinline__ void bt_load_point(const Fields& F, int64_t pt, T& ri, T& u2, T& u3, T& u4, T& u5, T& q) {
  const int64_t NP = F.NP;
  ri = (T)F.prim[PR_RHOI * NP + pt];
  q = (T)F.prim[PR_QS * NP + pt];
  u2 = (T)F.u[NP + pt];
  u3 = (T)F.u[2 * NP + pt];
  u4 = (T)F.u[3 * NP + pt];
  u5 = (T)F.u[4 * NP + pt];
}

// out: where the forward-eliminated rhs and the solution go (rhs itself for
// the in-place solve; a separate buffer when a refinement pass follows).
template <int DIR, typename T>
__global__ void __launch_bounds__(128) k_bt_solve(Fields F, Consts K, const Work* __restrict__ work,
                                                  T* __restrict__ lhsc, int64_t nlt, int add_u,
                                                  double* __restrict__ out) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int line = w.first + threadIdx.x;
  if (line >= zone_lines(Z, DIR)) return;
  int64_t base, st;
  line_geometry(Z, DIR, line, base, st);
  const int n = zone_line_len(Z, DIR);
  const int64_t gl = Z.lineoff[DIR] + line;
  const int64_t NP = F.NP;
  double* __restrict__ rhs = F.rhs;

  const T tmp1 = kv<T>(DIR == 0 ? K.dttx1 : DIR == 1 ? K.dtty1 : K.dttz1, K.f_dtt1[DIR]);
  const T tmp2 = kv<T>(DIR == 0 ? K.dttx2 : DIR == 1 ? K.dtty2 : K.dttz2, K.f_dtt2[DIR]);
  const double d64[5] = {DIR == 0 ? K.dx1 : DIR == 1 ? K.dy1 : K.dz1, DIR == 0 ? K.dx2 : DIR == 1 ? K.dy2 : K.dz2,
                         DIR == 0 ? K.dx3 : DIR == 1 ? K.dy3 : K.dz3, DIR == 0 ? K.dx4 : DIR == 1 ? K.dy4 : K.dz4,
                         DIR == 0 ? K.dx5 : DIR == 1 ? K.dy5 : K.dz5};
  T dd[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) dd[m] = kv<T>(d64[m], K.f_d[DIR][m]);

  T rp[5];          // r' at p-1
  T Cp[5][5];       // C' at p-1
  T Acur[5][5];     // lhsa at p   (structural nonzeros only)
  T Anext[5][5];    // lhsa at p+1
  T Bcur[5][5];     // lhsb at p   (structural nonzeros only)
  T f[5][5], nj[5][5];
  T ri, u2, u3, u4, u5, q;

#pragma unroll
  for (int m = 0; m < 5; ++m) rp[m] = (T)rhs[m * NP + base];
  // Jacobian at point 0 -> lhsa at 1; at point 1 -> lhsb at 1 and lhsa at 2.
  bt_load_point<DIR, T>(F, base, ri, u2, u3, u4, u5, q);
  bt_jac<DIR, T>(K, ri, u2, u3, u4, u5, q, f, nj);
  bt_asm_a<DIR, T>(f, nj, tmp1, tmp2, dd, Acur);
  bt_load_point<DIR, T>(F, base + st, ri, u2, u3, u4, u5, q);
  bt_jac<DIR, T>(K, ri, u2, u3, u4, u5, q, f, nj);
  bt_asm_b<T>(nj, tmp1, dd, Bcur);
  if (n - 2 >= 2) bt_asm_a<DIR, T>(f, nj, tmp1, tmp2, dd, Anext);

  for (int p = 1; p <= n - 2; ++p) {
    const int64_t pt = base + p * st;
    T r[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) r[m] = (T)rhs[m * NP + pt];
    // matvec_sub(lhsa_p, r'_{p-1}, r_p): the row sum is formed first.
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      T s;
      bool have = false;
#pragma unroll
      for (int c = 0; c < 5; ++c) {
        if (!anz<DIR>(m, c)) continue;
        s = have ? s + Acur[m][c] * rp[c] : Acur[m][c] * rp[c];
        have = true;
      }
      r[m] -= s;
    }
    // lhsb_p (full) = lhsb_p - lhsa_p * C'_{p-1}, one term at a time; C'_0 = 0.
    T B[5][5];
#pragma unroll
    for (int a = 0; a < 5; ++a)
#pragma unroll
      for (int b = 0; b < 5; ++b) {
        T t = bnz(a, b) ? Bcur[a][b] : (T)0.0;
        bool have = bnz(a, b);
        if (p > 1) {
#pragma unroll
          for (int c = 0; c < 5; ++c) {
            if (!anz<DIR>(a, c)) continue;
            t = have ? t - Acur[a][c] * Cp[c][b] : -(Acur[a][c] * Cp[c][b]);
            have = true;
          }
        }
        B[a][b] = t;
      }
    // Jacobian at p+1 -> lhsc_p, lhsb_{p+1}, lhsa_{p+2}
    bt_load_point<DIR, T>(F, pt + st, ri, u2, u3, u4, u5, q);
    bt_jac<DIR, T>(K, ri, u2, u3, u4, u5, q, f, nj);
    T C[5][5];
    bt_asm_c<DIR, T>(f, nj, tmp1, tmp2, dd, C);
#pragma unroll
    for (int a = 0; a < 5; ++a)
#pragma unroll
      for (int b = 0; b < 5; ++b)
        if (anz<DIR>(a, b)) Acur[a][b] = Anext[a][b];
    if (p + 1 <= n - 2) bt_asm_b<T>(nj, tmp1, dd, Bcur);
    if (p + 2 <= n - 2) bt_asm_a<DIR, T>(f, nj, tmp1, tmp2, dd, Anext);
    binvcrhs<T>(B, C, r);
#pragma unroll
    for (int a = 0; a < 5; ++a)
#pragma unroll
      for (int b = 0; b < 5; ++b) {
        Cp[a][b] = C[a][b];
        lhsc[((int64_t)p * 25 + a * 5 + b) * nlt + gl] = C[a][b];
      }
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      rp[m] = r[m];
      out[m * NP + pt] = (double)r[m];
    }
  }
  // back substitution: r_p -= C'_p r_{p+1}, one term at a time; the boundary
  // value r_{n-1} is unchanged by the forward sweep.
  T rn[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) rn[m] = (T)rhs[m * NP + base + (n - 1) * st];
  if (out != rhs) {
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      out[m * NP + base] = rhs[m * NP + base];
      out[m * NP + base + (n - 1) * st] = rhs[m * NP + base + (n - 1) * st];
    }
  }
  for (int p = n - 2; p >= 1; --p) {
    const int64_t pt = base + p * st;
    T r[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) r[m] = (p == n - 2) ? rp[m] : (T)out[m * NP + pt];
#pragma unroll
    for (int m = 0; m < 5; ++m)
#pragma unroll
      for (int c = 0; c < 5; ++c) r[m] -= lhsc[((int64_t)p * 25 + m * 5 + c) * nlt + gl] * rn[c];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const double v = (double)r[m];
      out[m * NP + pt] = v;
      if (add_u) F.u[m * NP + pt] += v;
      rn[m] = r[m];
    }
  }
}

// ============================================================================
// Mixed-precision BT sweep (NPBMZ_MIXED): two kernels per sweep direction.
//
// Pass 1 (k_bt_mixed_solve): T x0 = b in FP32 from the FP32 state copies,
// C' and the forward-eliminated rhs kept as FP32 in the line scratch
// (30 floats per point), x0 written as FP32.
// Pass 2 (k_bt_refine): the residual r = b - T x0 in FP64, T d = r in FP32,
// x = x0 + d into rhs (and, after the z sweep, into u).  Row p of T applied
// to x is, with F_q = fjac_q x_q and N_q = njac_q x_q,
//   x_p + tmp2 (F_{p+1} - F_{p-1}) - tmp1 (N_{p-1} - 2 N_p + N_{p+1})
//       - tmp1 D (x_{p-1} - 2 x_p + x_{p+1})
// (lhsa/lhsb/lhsc of src/BT/x_solve.jl:613-708 applied to x), and F, N are
// formed from the velocities directly (bt_jx), so the FP64 work is about
// 90 operations per point.  Boundary rows are identity rows whose residual
// is exactly zero, so d = 0 there.
// ============================================================================
template <int DIR>
__device__ __forceinline__ void bt_jx(const Consts& K, double ri, double q, double u2, double u3, double u4, double u5,
                                      const double x[5], double Fx[5], double Nx[5]) {
  const double vel[3] = {u2 * ri, u3 * ri, u4 * ri};
  const double E = u5 * ri;
  constexpr int a = DIR + 1;  // the momentum component normal to the sweep
  const double vn = vel[DIR];
  const double c1 = K.c1, c2 = K.c2;
  double d[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) d[m] = x[m + 1] - vel[m] * x[0];
  double tang = 0.0;
  Fx[0] = x[a];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    if (m == DIR) continue;
    Fx[m + 1] = vn * d[m] + vel[m] * x[a];
    tang += vel[m] * x[m + 1];
  }
  Fx[a] = (c2 * q - vn * vn) * x[0] - c2 * tang + (2.0 - c2) * vn * x[a] + c2 * x[4];
  Fx[4] = (2.0 * c2 * q - c1 * E) * vn * x[0] - c2 * vn * tang + (c1 * E - c2 * (q + vn * vn)) * x[a] + c1 * vn * x[4];
  const double k43 = K.con43 * K.c3c4, c3c4 = K.c3c4, c1345 = K.c1345;
  double s4 = c1345 * (x[4] - E * x[0]);
  Nx[0] = 0.0;
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const double cm = (m == DIR) ? k43 : c3c4;
    Nx[m + 1] = cm * ri * d[m];
    s4 += (cm - c1345) * vel[m] * d[m];
  }
  Nx[4] = ri * s4;
}

// State of the FP32 block elimination carried from point p to p+1.
template <int DIR>
struct BtF32Carry {
  float Cp[5][5];     // C' at p-1
  float rp[5];        // forward-eliminated rhs at p-1
  float Acur[5][5];   // lhsa at p   (structural nonzeros)
  float Anext[5][5];  // lhsa at p+1
  float Bcur[5][5];   // lhsb at p   (structural nonzeros)
};

template <int DIR>
__device__ __forceinline__ void bt_f32_consts(const Consts& K, float& tmp1, float& tmp2, float dd[5]) {
  tmp1 = K.f_dtt1[DIR];
  tmp2 = K.f_dtt2[DIR];
#pragma unroll
  for (int m = 0; m < 5; ++m) dd[m] = K.f_d[DIR][m];
}

// Start of the elimination: Jacobians at points 0 and 1 (FP32 state s0, s1 =
// ri, u2, u3, u4, u5, q).
template <int DIR>
__device__ __forceinline__ void bt_f32_begin(const Consts& K, int n, const float s0[6], const float s1[6],
                                             BtF32Carry<DIR>& c) {
  float tmp1, tmp2, dd[5], f[5][5], nj[5][5];
  bt_f32_consts<DIR>(K, tmp1, tmp2, dd);
  bt_jac<DIR, float>(K, s0[0], s0[1], s0[2], s0[3], s0[4], s0[5], f, nj);
  bt_asm_a<DIR, float>(f, nj, tmp1, tmp2, dd, c.Acur);
  bt_jac<DIR, float>(K, s1[0], s1[1], s1[2], s1[3], s1[4], s1[5], f, nj);
  bt_asm_b<float>(nj, tmp1, dd, c.Bcur);
  if (n - 2 >= 2) bt_asm_a<DIR, float>(f, nj, tmp1, tmp2, dd, c.Anext);
}

// One forward step at point p (1..n-2): r holds the rhs of row p on entry and
// the eliminated rhs on exit; sn is the FP32 state at p+1.  C'_p and r'_p go
// to scr[(p*30 + e) * nlt + gl].
template <int DIR>
__device__ __forceinline__ void bt_f32_step(const Consts& K, int p, int n, bool skip_first_matvec, float r[5],
                                            const float sn[6], BtF32Carry<DIR>& c, float* __restrict__ scr,
                                            int64_t nlt, int64_t gl) {
  float tmp1, tmp2, dd[5];
  bt_f32_consts<DIR>(K, tmp1, tmp2, dd);
  if (p > 1 || !skip_first_matvec) {
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      float sacc = 0.f;
#pragma unroll
      for (int cc = 0; cc < 5; ++cc)
        if (anz<DIR>(m, cc)) sacc += c.Acur[m][cc] * c.rp[cc];
      r[m] -= sacc;
    }
  }
  float B[5][5];
#pragma unroll
  for (int a = 0; a < 5; ++a)
#pragma unroll
    for (int b = 0; b < 5; ++b) {
      float t = bnz(a, b) ? c.Bcur[a][b] : 0.f;
      if (p > 1) {
#pragma unroll
        for (int cc = 0; cc < 5; ++cc)
          if (anz<DIR>(a, cc)) t -= c.Acur[a][cc] * c.Cp[cc][b];
      }
      B[a][b] = t;
    }
  float f[5][5], nj[5][5], C[5][5];
  bt_jac<DIR, float>(K, sn[0], sn[1], sn[2], sn[3], sn[4], sn[5], f, nj);
  bt_asm_c<DIR, float>(f, nj, tmp1, tmp2, dd, C);
#pragma unroll
  for (int a = 0; a < 5; ++a)
#pragma unroll
    for (int b = 0; b < 5; ++b)
      if (anz<DIR>(a, b)) c.Acur[a][b] = c.Anext[a][b];
  if (p + 1 <= n - 2) bt_asm_b<float>(nj, tmp1, dd, c.Bcur);
  if (p + 2 <= n - 2) bt_asm_a<DIR, float>(f, nj, tmp1, tmp2, dd, c.Anext);
  binvcrhs<float>(B, C, r);
#pragma unroll
  for (int a = 0; a < 5; ++a)
#pragma unroll
    for (int b = 0; b < 5; ++b) {
      c.Cp[a][b] = C[a][b];
      scr[((int64_t)p * 30 + a * 5 + b) * nlt + gl] = C[a][b];
    }
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    c.rp[m] = r[m];
    scr[((int64_t)p * 30 + 25 + m) * nlt + gl] = r[m];
  }
}

__device__ __forceinline__ void load_state_f32(const Fields& F, int64_t pt, float s[6]) {
  const int64_t NP = F.NP;
  s[0] = F.primf[PF_RHOI * NP + pt];
  s[1] = F.primf[PF_U2 * NP + pt];
  s[2] = F.primf[PF_U3 * NP + pt];
  s[3] = F.primf[PF_U4 * NP + pt];
  s[4] = F.primf[PF_U5 * NP + pt];
  s[5] = F.primf[PF_QS * NP + pt];
}

__device__ __forceinline__ void load_state_f64(const Fields& F, int64_t pt, double s[6]) {
  const int64_t NP = F.NP;
  s[0] = F.prim[PR_RHOI * NP + pt];
  s[1] = F.u[NP + pt];
  s[2] = F.u[2 * NP + pt];
  s[3] = F.u[3 * NP + pt];
  s[4] = F.u[4 * NP + pt];
  s[5] = F.prim[PR_QS * NP + pt];
}

// Pass 1: T x0 = b in FP32.  Loads of point p+2 and of b_{p+1} are issued one
// step ahead so that they overlap the elimination of point p.
// IN_DF: b comes from the double-float planes F.rdf (hi part), not rhs.
template <int DIR, bool IN_DF>
__global__ void __launch_bounds__(128) k_bt_mixed_solve(Fields F, Consts K, const Work* __restrict__ work,
                                                        float* __restrict__ scr, int64_t nlt,
                                                        float* __restrict__ x0) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int line = w.first + threadIdx.x;
  if (line >= zone_lines(Z, DIR)) return;
  int64_t base, st;
  line_geometry(Z, DIR, line, base, st);
  const int n = zone_line_len(Z, DIR);
  const int64_t gl = Z.lineoff[DIR] + line;
  const int64_t NP = F.NP;
  const double* __restrict__ rhs = F.rhs;
  const float* __restrict__ bdf = F.rdf;
  auto bload = [&](int m, int64_t pt) -> float { return IN_DF ? bdf[m * NP + pt] : (float)rhs[m * NP + pt]; };
  BtF32Carry<DIR> c;
  float s0[6], s1[6];
  load_state_f32(F, base, s0);
  load_state_f32(F, base + st, s1);
#pragma unroll
  for (int m = 0; m < 5; ++m) c.rp[m] = bload(m, base);
  bt_f32_begin<DIR>(K, n, s0, s1, c);
  float sn[6], bn[5];
  load_state_f32(F, base + 2 * st, sn);
#pragma unroll
  for (int m = 0; m < 5; ++m) bn[m] = bload(m, base + st);
  for (int p = 1; p <= n - 2; ++p) {
    float r[5], s[6];
#pragma unroll
    for (int m = 0; m < 5; ++m) r[m] = bn[m];
#pragma unroll
    for (int e = 0; e < 6; ++e) s[e] = sn[e];
    if (p + 1 <= n - 2) {  // prefetch for the next step
      load_state_f32(F, base + (int64_t)(p + 2) * st, sn);
#pragma unroll
      for (int m = 0; m < 5; ++m) bn[m] = bload(m, base + (int64_t)(p + 1) * st);
    }
    bt_f32_step<DIR>(K, p, n, false, r, s, c, scr, nlt, gl);
  }
  float rn[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) rn[m] = bload(m, base + (int64_t)(n - 1) * st);
  for (int p = n - 2; p >= 1; --p) {
    float r[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) r[m] = (p == n - 2) ? c.rp[m] : scr[((int64_t)p * 30 + 25 + m) * nlt + gl];
#pragma unroll
    for (int m = 0; m < 5; ++m)
#pragma unroll
      for (int cc = 0; cc < 5; ++cc) r[m] -= scr[((int64_t)p * 30 + m * 5 + cc) * nlt + gl] * rn[cc];
    const int64_t pt = base + p * st;
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      x0[m * NP + pt] = r[m];
      rn[m] = r[m];
    }
  }
}

// Pass 2: r = b - T x0 in FP64, T d = r in FP32, x = x0 + d.  The residual
// rows are accumulated point by point: point q adds
//   -tmp2 F_q - tmp1 N_q - tmp1 D x_q          to row q+1,
//   x_q + 2 tmp1 N_q + 2 tmp1 D x_q            to row q,
//   tmp2 F_q - tmp1 N_q - tmp1 D x_q           to row q-1 (which is then complete).
template <int DIR>
__global__ void __launch_bounds__(128) k_bt_refine(Fields F, Consts K, const Work* __restrict__ work,
                                                   float* __restrict__ scr, int64_t nlt, int add_u,
                                                   const float* __restrict__ x0f) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int line = w.first + threadIdx.x;
  if (line >= zone_lines(Z, DIR)) return;
  int64_t base, st;
  line_geometry(Z, DIR, line, base, st);
  const int n = zone_line_len(Z, DIR);
  const int64_t gl = Z.lineoff[DIR] + line;
  const int64_t NP = F.NP;
  double* __restrict__ rhs = F.rhs;

  const double t1d = DIR == 0 ? K.dttx1 : DIR == 1 ? K.dtty1 : K.dttz1;
  const double t2d = DIR == 0 ? K.dttx2 : DIR == 1 ? K.dtty2 : K.dttz2;
  double ddd[5];
  if (DIR == 0) { ddd[0] = K.dx1; ddd[1] = K.dx2; ddd[2] = K.dx3; ddd[3] = K.dx4; ddd[4] = K.dx5; }
  else if (DIR == 1) { ddd[0] = K.dy1; ddd[1] = K.dy2; ddd[2] = K.dy3; ddd[3] = K.dy4; ddd[4] = K.dy5; }
  else { ddd[0] = K.dz1; ddd[1] = K.dz2; ddd[2] = K.dz3; ddd[3] = K.dz4; ddd[4] = K.dz5; }

  // x0 at point q: the FP32 first pass inside, b itself on the boundary.
  auto load_x = [&](int q, double x[5]) {
    const int64_t pt = base + (int64_t)q * st;
    if (q == 0 || q == n - 1) {
#pragma unroll
      for (int m = 0; m < 5; ++m) x[m] = rhs[m * NP + pt];
    } else {
#pragma unroll
      for (int m = 0; m < 5; ++m) x[m] = (double)x0f[m * NP + pt];
    }
  };
  double acc_c[5], acc_n[5];   // partial (T x0) of rows p and p+1
  double xq[5], sq[6];
  float s0[6], s1[6];
  // point 0: contributes to row 1 only (row 0 is an identity row)
  load_x(0, xq);
  load_state_f64(F, base, sq);
  {
    double Fq[5], Nq[5];
    bt_jx<DIR>(K, sq[0], sq[5], sq[1], sq[2], sq[3], sq[4], xq, Fq, Nq);
#pragma unroll
    for (int m = 0; m < 5; ++m) acc_c[m] = -t2d * Fq[m] - t1d * Nq[m] - t1d * ddd[m] * xq[m];
#pragma unroll
    for (int e = 0; e < 6; ++e) s0[e] = (float)sq[e];
  }
  // point 1: centre of row 1, left neighbour of row 2
  load_x(1, xq);
  load_state_f64(F, base + st, sq);
  {
    double Fq[5], Nq[5];
    bt_jx<DIR>(K, sq[0], sq[5], sq[1], sq[2], sq[3], sq[4], xq, Fq, Nq);
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      acc_c[m] += xq[m] + 2.0 * t1d * Nq[m] + 2.0 * t1d * ddd[m] * xq[m];
      acc_n[m] = -t2d * Fq[m] - t1d * Nq[m] - t1d * ddd[m] * xq[m];
    }
#pragma unroll
    for (int e = 0; e < 6; ++e) s1[e] = (float)sq[e];
  }
  BtF32Carry<DIR> c;
#pragma unroll
  for (int m = 0; m < 5; ++m) c.rp[m] = 0.f;  // the boundary residual is exactly zero
  bt_f32_begin<DIR>(K, n, s0, s1, c);
  // prefetch point 2 and b_1
  double xn[5], sn[6], bn[5];
  load_x(2, xn);
  load_state_f64(F, base + 2 * st, sn);
#pragma unroll
  for (int m = 0; m < 5; ++m) bn[m] = rhs[m * NP + base + st];

  for (int p = 1; p <= n - 2; ++p) {
    const int64_t pt = base + (int64_t)p * st;
    double b[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) { xq[m] = xn[m]; b[m] = bn[m]; }
#pragma unroll
    for (int e = 0; e < 6; ++e) sq[e] = sn[e];
    if (p + 1 <= n - 2) {
      load_x(p + 2, xn);
      load_state_f64(F, base + (int64_t)(p + 2) * st, sn);
#pragma unroll
      for (int m = 0; m < 5; ++m) bn[m] = rhs[m * NP + base + (int64_t)(p + 1) * st];
    }
    // point p+1 completes row p
    double Fq[5], Nq[5];
    bt_jx<DIR>(K, sq[0], sq[5], sq[1], sq[2], sq[3], sq[4], xq, Fq, Nq);
    float r[5], s[6];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const double tx = acc_c[m] + t2d * Fq[m] - t1d * Nq[m] - t1d * ddd[m] * xq[m];
      r[m] = (float)(b[m] - tx);
      acc_c[m] = acc_n[m] + xq[m] + 2.0 * t1d * Nq[m] + 2.0 * t1d * ddd[m] * xq[m];
      acc_n[m] = -t2d * Fq[m] - t1d * Nq[m] - t1d * ddd[m] * xq[m];
    }
#pragma unroll
    for (int e = 0; e < 6; ++e) s[e] = (float)sq[e];
    bt_f32_step<DIR>(K, p, n, true, r, s, c, scr, nlt, gl);
    (void)pt;
  }
  // back substitution of the correction d, then x = x0 + d
  float dn[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  for (int p = n - 2; p >= 1; --p) {
    const int64_t pt = base + p * st;
    float d[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) d[m] = (p == n - 2) ? c.rp[m] : scr[((int64_t)p * 30 + 25 + m) * nlt + gl];
#pragma unroll
    for (int m = 0; m < 5; ++m)
#pragma unroll
      for (int cc = 0; cc < 5; ++cc) d[m] -= scr[((int64_t)p * 30 + m * 5 + cc) * nlt + gl] * dn[cc];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const double v = (double)x0f[m * NP + pt] + (double)d[m];
      rhs[m * NP + pt] = v;
      if (add_u) F.u[m * NP + pt] += v;
      dn[m] = d[m];
    }
  }
}

// ============================================================================
// Double-float (FP32 pair) arithmetic for the residual of the refinement
// pass.  GB300 issues FP32 at 64x the FP64 rate; a value hi + lo with
// |lo| <= ulp(hi)/2 carries about 48 significant bits, enough for the
// residual r = b - T x0 (its error enters the refined solution at about
// 1e-14 relative, below the FP32 re-solve's own (eps32 * kappa)^2 term).
// Error-free transformations (Knuth two-sum, FMA two-product) are written
// with explicit round-to-nearest intrinsics so no contraction or
// reassociation can change them.
// ============================================================================
struct df64 {
  float hi, lo;
};

__device__ __forceinline__ df64 df_quick(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df64 df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ df64 df_add(df64 a, df64 b) {
  const df64 s = df_two_sum(a.hi, b.hi);
  return df_quick(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df64 df_neg(df64 a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df64 df_sub(df64 a, df64 b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df64 df_mul(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_quick(p, e);
}
__device__ __forceinline__ df64 df_scale2(df64 a) { return {2.f * a.hi, 2.f * a.lo}; }  // exact
__device__ __forceinline__ df64 f2df(float2 v) { return {v.x, v.y}; }
// FP32 -> FP64 (exact) from the bit pattern: sign, exponent rebiased by
// 1023 - 127, significand shifted into place; zero, subnormals, inf and nan
// take the conversion instruction, which on GB300 is an FP64-pipe slot.
__device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu;
  if (e - 1u >= 254u) return (double)f;
  const unsigned hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b >> 3) & 0xfffffu);
  return __hiloint2double((int)hi, (int)(b << 29));
}
__device__ __forceinline__ double df_to_double(df64 v) { return f32_to_f64(v.hi) + f32_to_f64(v.lo); }
// 1/a: FP32 estimate x, residual e = 1 - a x formed exactly to first order
// (a.hi x = p + pe exactly; 1 - p is exact since p is within 2^-23 of 1),
// then x + x e.
__device__ __forceinline__ df64 df_rcp(df64 a) {
  const float x = __frcp_rn(a.hi);
  const float p = __fmul_rn(a.hi, x);
  const float pe = __fmaf_rn(a.hi, x, -p);
  const float e = __fmaf_rn(-a.lo, x, __fsub_rn(__fsub_rn(1.f, p), pe));
  return df_quick(x, __fmul_rn(x, e));
}
__device__ __forceinline__ float2 df2f(df64 v) { return make_float2(v.hi, v.lo); }
__device__ __forceinline__ df64 df_from(double d) {
  const float h = __double2float_rn(d);
  return {h, __double2float_rn(d - (double)h)};
}

// F = fjac x and N = njac x in double-float (the formulas of bt_jx).
template <int DIR>
__device__ __forceinline__ void bt_jx_df(const df64 c1, const df64 c2, const df64 two_m_c2, const df64 k43,
                                         const df64 c3c4, const df64 c1345, const df64 k43m, const df64 c3c4m,
                                         const df64 st[6], const df64 x[5], df64 Fx[5], df64 Nx[5]) {
  // st = ri, u2, u3, u4, u5, q
  const df64 ri = st[0], q = st[5];
  const df64 vel[3] = {df_mul(st[1], ri), df_mul(st[2], ri), df_mul(st[3], ri)};
  const df64 E = df_mul(st[4], ri);
  constexpr int a = DIR + 1;
  const df64 vn = vel[DIR];
  df64 d[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) d[m] = df_sub(x[m + 1], df_mul(vel[m], x[0]));
  df64 tang = {0.f, 0.f};
  Fx[0] = x[a];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    if (m == DIR) continue;
    Fx[m + 1] = df_add(df_mul(vn, d[m]), df_mul(vel[m], x[a]));
    tang = df_add(tang, df_mul(vel[m], x[m + 1]));
  }
  const df64 c2q = df_mul(c2, q), vn2 = df_mul(vn, vn), c1E = df_mul(c1, E);
  Fx[a] = df_add(df_add(df_mul(df_sub(c2q, vn2), x[0]), df_neg(df_mul(c2, tang))),
                 df_add(df_mul(df_mul(two_m_c2, vn), x[a]), df_mul(c2, x[4])));
  Fx[4] = df_add(df_add(df_mul(df_mul(df_sub(df_scale2(c2q), c1E), vn), x[0]), df_neg(df_mul(df_mul(c2, vn), tang))),
                 df_add(df_mul(df_sub(c1E, df_mul(c2, df_add(q, vn2))), x[a]), df_mul(df_mul(c1, vn), x[4])));
  df64 s4 = df_mul(c1345, df_sub(x[4], df_mul(E, x[0])));
  const df64 k43ri = df_mul(k43, ri), c3c4ri = df_mul(c3c4, ri);
  Nx[0] = {0.f, 0.f};
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    Nx[m + 1] = df_mul(m == DIR ? k43ri : c3c4ri, d[m]);
    s4 = df_add(s4, df_mul(df_mul(m == DIR ? k43m : c3c4m, vel[m]), d[m]));
  }
  Nx[4] = df_mul(ri, s4);
}

__device__ __forceinline__ void load_state_df(const Fields& F, int64_t pt, df64 s[6]) {
  const int64_t NP = F.NP;
  const int order[6] = {PF_RHOI, PF_U2, PF_U3, PF_U4, PF_U5, PF_QS};
#pragma unroll
  for (int e = 0; e < 6; ++e) {
    s[e].hi = F.primf[order[e] * NP + pt];
    s[e].lo = F.primf[(PF_HI_COUNT + order[e]) * NP + pt];
  }
}

// Refinement pass with the residual in double-float.  Point q contributes,
// with P_q = tmp2 F_q and Q_q = tmp1 (N_q + D x_q),
//   -P_q - Q_q to row q+1,   x_q + 2 Q_q to row q,   P_q - Q_q to row q-1.
// IN_DF: b and the line's end values come from the double-float planes
// F.rdf; OUT_DF: x goes back to F.rdf as the exact double-float sum x0 + d
// instead of to rhs in FP64 (the next sweep of the same step reads it so).
template <int DIR, bool IN_DF, bool OUT_DF>
__global__ void __launch_bounds__(128) k_bt_refine_df(Fields F, Consts K, const Work* __restrict__ work,
                                                      float* __restrict__ scr, int64_t nlt, int add_u,
                                                      const float* __restrict__ x0f) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int line = w.first + threadIdx.x;
  if (line >= zone_lines(Z, DIR)) return;
  int64_t base, st;
  line_geometry(Z, DIR, line, base, st);
  const int n = zone_line_len(Z, DIR);
  const int64_t gl = Z.lineoff[DIR] + line;
  const int64_t NP = F.NP;
  double* __restrict__ rhs = F.rhs;
  float* __restrict__ bdf = F.rdf;

  const df64 t1 = f2df(K.p_dtt1[DIR]);
  const df64 t2 = f2df(K.p_dtt2[DIR]);
  df64 D[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) D[m] = f2df(K.p_d[DIR][m]);
  const df64 c1 = f2df(K.p_c1), c2 = f2df(K.p_c2), two_m_c2 = f2df(K.p_two_m_c2);
  const df64 k43 = f2df(K.p_k43), c3c4 = f2df(K.p_c3c4), c1345 = f2df(K.p_c1345);
  const df64 k43m = f2df(K.p_k43m), c3c4m = f2df(K.p_c3c4m);

  auto load_x = [&](int q, df64 x[5]) {
    const int64_t pt = base + (int64_t)q * st;
    if (q == 0 || q == n - 1) {
#pragma unroll
      for (int m = 0; m < 5; ++m) x[m] = IN_DF ? df64{bdf[m * NP + pt], bdf[(5 + m) * NP + pt]} : df_from(rhs[m * NP + pt]);
    } else {
#pragma unroll
      for (int m = 0; m < 5; ++m) x[m] = {x0f[m * NP + pt], 0.f};
    }
  };
  // P and Q of one point
  auto pq = [&](const df64 s[6], const df64 x[5], df64 P[5], df64 Q[5]) {
    df64 Fq[5], Nq[5];
    bt_jx_df<DIR>(c1, c2, two_m_c2, k43, c3c4, c1345, k43m, c3c4m, s, x, Fq, Nq);
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      P[m] = df_mul(t2, Fq[m]);
      Q[m] = df_mul(t1, df_add(Nq[m], df_mul(D[m], x[m])));
    }
  };
  df64 acc_c[5], acc_n[5], xq[5], sq[6], P[5], Q[5];
  float s0[6], s1[6];
  load_x(0, xq);
  load_state_df(F, base, sq);
  pq(sq, xq, P, Q);
#pragma unroll
  for (int m = 0; m < 5; ++m) acc_c[m] = df_neg(df_add(P[m], Q[m]));
#pragma unroll
  for (int e = 0; e < 6; ++e) s0[e] = sq[e].hi;
  load_x(1, xq);
  load_state_df(F, base + st, sq);
  pq(sq, xq, P, Q);
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    acc_c[m] = df_add(acc_c[m], df_add(xq[m], df_scale2(Q[m])));
    acc_n[m] = df_neg(df_add(P[m], Q[m]));
  }
#pragma unroll
  for (int e = 0; e < 6; ++e) s1[e] = sq[e].hi;
  BtF32Carry<DIR> c;
#pragma unroll
  for (int m = 0; m < 5; ++m) c.rp[m] = 0.f;
  // bt_f32_begin takes ri, u2, u3, u4, u5, q in that order (as sq)
  bt_f32_begin<DIR>(K, n, s0, s1, c);
  df64 xn[5], sn[6];
  // b of the next point: double-float planes (IN_DF) or FP64 rhs
  df64 bn[5];
  double bn64[5];
  auto load_b = [&](int64_t pt) {
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      if (IN_DF) bn[m] = df64{bdf[m * NP + pt], bdf[(5 + m) * NP + pt]};
      else bn64[m] = rhs[m * NP + pt];
    }
  };
  load_x(2, xn);
  load_state_df(F, base + 2 * st, sn);
  load_b(base + st);

  for (int p = 1; p <= n - 2; ++p) {
    double b[5];
    df64 bd[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      xq[m] = xn[m];
      if (IN_DF) bd[m] = bn[m];
      else b[m] = bn64[m];
    }
#pragma unroll
    for (int e = 0; e < 6; ++e) sq[e] = sn[e];
    if (p + 1 <= n - 2) {
      load_x(p + 2, xn);
      load_state_df(F, base + (int64_t)(p + 2) * st, sn);
      load_b(base + (int64_t)(p + 1) * st);
    }
    pq(sq, xq, P, Q);
    float r[5], s[6];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const df64 tx = df_add(acc_c[m], df_sub(P[m], Q[m]));
      if (IN_DF) {
        const df64 rr = df_sub(bd[m], tx);
        r[m] = rr.hi + rr.lo;
      } else {
        r[m] = __double2float_rn((b[m] - (double)tx.hi) - (double)tx.lo);
      }
      acc_c[m] = df_add(acc_n[m], df_add(xq[m], df_scale2(Q[m])));
      acc_n[m] = df_neg(df_add(P[m], Q[m]));
    }
#pragma unroll
    for (int e = 0; e < 6; ++e) s[e] = sq[e].hi;
    bt_f32_step<DIR>(K, p, n, true, r, s, c, scr, nlt, gl);
  }
  float dn[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  for (int p = n - 2; p >= 1; --p) {
    const int64_t pt = base + p * st;
    float d[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) d[m] = (p == n - 2) ? c.rp[m] : scr[((int64_t)p * 30 + 25 + m) * nlt + gl];
#pragma unroll
    for (int m = 0; m < 5; ++m)
#pragma unroll
      for (int cc = 0; cc < 5; ++cc) d[m] -= scr[((int64_t)p * 30 + m * 5 + cc) * nlt + gl] * dn[cc];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      if (OUT_DF) {
        const df64 v = df_two_sum(x0f[m * NP + pt], d[m]);
        bdf[m * NP + pt] = v.hi;
        bdf[(5 + m) * NP + pt] = v.lo;
      } else {
        const double v = (double)x0f[m * NP + pt] + (double)d[m];
        rhs[m * NP + pt] = v;
        if (add_u) F.u[m * NP + pt] += v;
      }
      dn[m] = d[m];
    }
  }
}

#if NPBMZ_HAS_FP32
// ============================================================================
// Software-pipelined refined FP32 BT sweep of a fused step (mode 4).  The
// two passes above wait on memory once per point: a line advances one point
// per DRAM round trip, and with 8-12 resident warps per SM nothing hides it.
// Here each thread streams its own line's data PIPE points ahead with
// cp.async into a ring of PIPE slots in shared memory (word e of slot s of
// thread t at ring[(s * W + e) * T + t]: a warp's copies land in consecutive
// banks), in the forward elimination and in the back substitution alike.
// The arithmetic is that of k_bt_mixed_solve<DIR, true> and
// k_bt_refine_df<DIR, true, OUT_DF>.
// ============================================================================
#ifndef NPBMZ_PIPE
#define NPBMZ_PIPE 4
#endif
constexpr int PIPE = NPBMZ_PIPE;

// Minimum resident CTAs of 128 threads per SM that the pipelined sweep
// kernels are compiled for (__launch_bounds__): it caps their registers at
// 65536 / (128 * n) and so sets their occupancy.
#ifndef NPBMZ_BT_MIXED_MINB
#define NPBMZ_BT_MIXED_MINB 1
#endif
#ifndef NPBMZ_BT_REFINE_MINB
#define NPBMZ_BT_REFINE_MINB 1
#endif
#ifndef NPBMZ_SP_MINB
#define NPBMZ_SP_MINB 3
#endif

__device__ __forceinline__ void cpa4(float* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cpa8(double* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpa_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

constexpr int PL_MIXED_W = 30;   // words per slot, first pass
constexpr int PL_REFINE_W = 35;  // words per slot, refinement pass

// Dynamic shared memory of the pipelined kernels for tpb threads.
// (the first pass keeps 5 more words per line: b at the line's last point)
__host__ __device__ constexpr size_t pl_mixed_smem(int tpb) {
  return (size_t)(PIPE * PL_MIXED_W + 5) * tpb * sizeof(float);
}
__host__ __device__ constexpr size_t pl_refine_smem(int tpb, bool out_df) {
  return (size_t)PIPE * 5 * tpb * sizeof(double) * (out_df ? 0 : 1) + (size_t)PIPE * PL_REFINE_W * tpb * sizeof(float);
}

template <int DIR>
__device__ __forceinline__ void bt_mixed_pl_item(const Fields& F, const Consts& K, const Work w,
                                                 float* __restrict__ scr, int64_t nlt, float* __restrict__ x0,
                                                 unsigned char* pl_smem) {
  const ZoneDev Z = F.zones[w.zone];
  const int line = w.first + threadIdx.x;
  if (line >= zone_lines(Z, DIR)) return;
  int64_t base, st;
  line_geometry(Z, DIR, line, base, st);
  const int n = zone_line_len(Z, DIR);
  const int64_t gl = Z.lineoff[DIR] + line;
  const int64_t NP = F.NP;
  const int T = blockDim.x;
  float* my = reinterpret_cast<float*>(pl_smem) + threadIdx.x;
  auto S = [&](int slot, int e) -> float* { return my + (slot * PL_MIXED_W + e) * T; };
  const int order[6] = {PF_RHOI, PF_U2, PF_U3, PF_U4, PF_U5, PF_QS};
  // the x sweep reads its x-line-major copies, y and z the zone layout
  auto st_at = [&](int q, int plane) -> const float* {
    return DIR == 0 ? F.pfx + ((int64_t)q * PF_COUNT + plane) * F.nlx + gl : F.primf + plane * NP + base + (int64_t)q * st;
  };
  auto b_at = [&](int q, int e) -> const float* {
    return DIR == 0 ? F.rdx + ((int64_t)q * 10 + e) * F.nlx + gl : F.rdf + e * NP + base + (int64_t)q * st;
  };
  auto x0_at = [&](int q, int m) -> float* {
    return DIR == 0 ? F.x0x + ((int64_t)q * 5 + m) * F.nlx + gl : x0 + m * NP + base + (int64_t)q * st;
  };

  // forward step p (1..n-2) consumes b_p and the state at p+1
  auto issue_fwd = [&](int p) {
    if (p <= n - 2) {
      const int slot = p % PIPE;
#pragma unroll
      for (int e = 0; e < 6; ++e) cpa4(S(slot, e), st_at(p + 1, order[e]));
#pragma unroll
      for (int m = 0; m < 5; ++m) cpa4(S(slot, 6 + m), b_at(p, m));
    }
    cpa_commit();
  };
  // the ring's first slots (and b at the last point, which the back
  // substitution starts from) go out before the line's first points are read
  // directly, so that the memory latencies overlap
#pragma unroll
  for (int m = 0; m < 5; ++m) cpa4(S(PIPE, m), b_at(n - 1, m));
#pragma unroll
  for (int q = 1; q < PIPE; ++q) issue_fwd(q);
  BtF32Carry<DIR> c;
  {
    float s0[6], s1[6];
#pragma unroll
    for (int e = 0; e < 6; ++e) {
      s0[e] = *st_at(0, order[e]);
      s1[e] = *st_at(1, order[e]);
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) c.rp[m] = *b_at(0, m);
    bt_f32_begin<DIR>(K, n, s0, s1, c);
  }
  for (int p = 1; p <= n - 2; ++p) {
    issue_fwd(p + PIPE - 1);
    cpa_wait<PIPE - 1>();
    const int slot = p % PIPE;
    float r[5], s[6];
#pragma unroll
    for (int e = 0; e < 6; ++e) s[e] = *S(slot, e);
#pragma unroll
    for (int m = 0; m < 5; ++m) r[m] = *S(slot, 6 + m);
    bt_f32_step<DIR>(K, p, n, false, r, s, c, scr, nlt, gl);
    if (p + PIPE > n - 2) {
      // the ring does not refill this slot: C'_p and r'_p stay here for the
      // back substitution, which so starts without a trip to memory
#pragma unroll
      for (int a = 0; a < 5; ++a)
#pragma unroll
        for (int b = 0; b < 5; ++b) *S(slot, a * 5 + b) = c.Cp[a][b];
#pragma unroll
      for (int m = 0; m < 5; ++m) *S(slot, 25 + m) = c.rp[m];
    }
  }
  cpa_wait<0>();
  // back substitution: step p (n-2 .. 1) consumes C'_p and r'_p from slot
  // p % PIPE: the last PIPE points as the forward pass left them, the others
  // loaded PIPE steps ahead into the slot just consumed
  auto issue_bwd = [&](int p) {
    if (p >= 1) {
      const int slot = p % PIPE;
#pragma unroll
      for (int e = 0; e < 30; ++e) cpa4(S(slot, e), scr + ((int64_t)p * 30 + e) * nlt + gl);
    }
    cpa_commit();
  };
  float rn[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) rn[m] = *S(PIPE, m);
  for (int p = n - 2; p >= 1; --p) {
    if (p + PIPE <= n - 2) cpa_wait<PIPE - 1>();
    const int slot = p % PIPE;
    float r[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      float t = *S(slot, 25 + m);
#pragma unroll
      for (int cc = 0; cc < 5; ++cc) t -= *S(slot, m * 5 + cc) * rn[cc];
      r[m] = t;
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      *x0_at(p, m) = r[m];
      rn[m] = r[m];
    }
    issue_bwd(p - PIPE);
  }
  cpa_wait<0>();
}

template <int DIR>
__global__ void __launch_bounds__(128, NPBMZ_BT_MIXED_MINB) k_bt_mixed_pl(Fields F, Consts K, const Work* __restrict__ work, int nwork,
                                                     float* __restrict__ scr, int64_t nlt, float* __restrict__ x0) {
  extern __shared__ __align__(16) unsigned char pl_smem[];
  for (int it = blockIdx.x; it < nwork; it += gridDim.x) bt_mixed_pl_item<DIR>(F, K, work[it], scr, nlt, x0, pl_smem);
}

template <int DIR, bool OUT_DF>
__device__ __forceinline__ void bt_refine_pl_item(const Fields& F, const Consts& K, const Work w,
                                                  float* __restrict__ scr, int64_t nlt, int add_u,
                                                  const float* __restrict__ x0f, unsigned char* pl_smem) {
  const ZoneDev Z = F.zones[w.zone];
  const int line = w.first + threadIdx.x;
  if (line >= zone_lines(Z, DIR)) return;
  int64_t base, st;
  line_geometry(Z, DIR, line, base, st);
  const int n = zone_line_len(Z, DIR);
  const int64_t gl = Z.lineoff[DIR] + line;
  const int64_t NP = F.NP;
  const int T = blockDim.x;
  // the FP64 ring (u, z sweep only) first: 8-byte words
  double* umy = reinterpret_cast<double*>(pl_smem) + threadIdx.x;
  float* my = reinterpret_cast<float*>(pl_smem + (OUT_DF ? 0 : (size_t)PIPE * 5 * T * sizeof(double))) + threadIdx.x;
  auto S = [&](int slot, int e) -> float* { return my + (slot * PL_REFINE_W + e) * T; };
  auto SU = [&](int slot, int m) -> double* { return umy + (slot * 5 + m) * T; };
  double* __restrict__ rhs = F.rhs;
  float* __restrict__ bdf = F.rdf;
  const int order[6] = {PF_RHOI, PF_U2, PF_U3, PF_U4, PF_U5, PF_QS};
  // the x sweep reads its x-line-major copies, y and z the zone layout; the
  // result always goes to the zone layout (the next sweep reads it there)
  auto st_at = [&](int q, int plane) -> const float* {
    return DIR == 0 ? F.pfx + ((int64_t)q * PF_COUNT + plane) * F.nlx + gl : F.primf + plane * NP + base + (int64_t)q * st;
  };
  auto b_at = [&](int q, int e) -> const float* {
    return DIR == 0 ? F.rdx + ((int64_t)q * 10 + e) * F.nlx + gl : bdf + e * NP + base + (int64_t)q * st;
  };
  auto x0_at = [&](int q, int m) -> const float* {
    return DIR == 0 ? F.x0x + ((int64_t)q * 5 + m) * F.nlx + gl : x0f + m * NP + base + (int64_t)q * st;
  };

  const df64 t1 = f2df(K.p_dtt1[DIR]);
  const df64 t2 = f2df(K.p_dtt2[DIR]);
  df64 D[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) D[m] = f2df(K.p_d[DIR][m]);
  const df64 c1 = f2df(K.p_c1), c2 = f2df(K.p_c2), two_m_c2 = f2df(K.p_two_m_c2);
  const df64 k43 = f2df(K.p_k43), c3c4 = f2df(K.p_c3c4), c1345 = f2df(K.p_c1345);
  const df64 k43m = f2df(K.p_k43m), c3c4m = f2df(K.p_c3c4m);

  auto pq = [&](const df64 s[6], const df64 x[5], df64 P[5], df64 Q[5]) {
    df64 Fq[5], Nq[5];
    bt_jx_df<DIR>(c1, c2, two_m_c2, k43, c3c4, c1345, k43m, c3c4m, s, x, Fq, Nq);
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      P[m] = df_mul(t2, Fq[m]);
      Q[m] = df_mul(t1, df_add(Nq[m], df_mul(D[m], x[m])));
    }
  };
  auto load_x = [&](int q, df64 x[5]) {  // direct loads (prologue)
#pragma unroll
    for (int m = 0; m < 5; ++m)
      x[m] = (q == 0 || q == n - 1) ? df64{*b_at(q, m), *b_at(q, 5 + m)} : df64{*x0_at(q, m), 0.f};
  };
  auto load_sdf = [&](int q, df64 s6[6]) {
#pragma unroll
    for (int e = 0; e < 6; ++e) s6[e] = df64{*st_at(q, order[e]), *st_at(q, PF_HI_COUNT + order[e])};
  };
  // forward step p (1..n-2) consumes x and the state at p+1 and b_p:
  // words 0..9 x (5 x0 values, or hi/lo of the line's end value), 10..21
  // state hi/lo, 22..31 b hi/lo
  auto issue_fwd = [&](int p) {
    if (p <= n - 2) {
      const int slot = p % PIPE;
      if (p + 1 == n - 1) {
#pragma unroll
        for (int e = 0; e < 10; ++e) cpa4(S(slot, e), b_at(p + 1, e));
      } else {
#pragma unroll
        for (int m = 0; m < 5; ++m) cpa4(S(slot, m), x0_at(p + 1, m));
      }
#pragma unroll
      for (int e = 0; e < 6; ++e) {
        cpa4(S(slot, 10 + e), st_at(p + 1, order[e]));
        cpa4(S(slot, 16 + e), st_at(p + 1, PF_HI_COUNT + order[e]));
      }
#pragma unroll
      for (int e = 0; e < 10; ++e) cpa4(S(slot, 22 + e), b_at(p, e));
    }
    cpa_commit();
  };

  // the ring's first slots go out before the line's first points are read
  // directly, so that the two memory latencies overlap
#pragma unroll
  for (int q = 1; q < PIPE; ++q) issue_fwd(q);
  df64 acc_c[5], acc_n[5], xq[5], sq[6], P[5], Q[5];
  BtF32Carry<DIR> c;
  {
    float s0[6], s1[6];
    load_x(0, xq);
    load_sdf(0, sq);
    pq(sq, xq, P, Q);
#pragma unroll
    for (int m = 0; m < 5; ++m) acc_c[m] = df_neg(df_add(P[m], Q[m]));
#pragma unroll
    for (int e = 0; e < 6; ++e) s0[e] = sq[e].hi;
    load_x(1, xq);
    load_sdf(1, sq);
    pq(sq, xq, P, Q);
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      acc_c[m] = df_add(acc_c[m], df_add(xq[m], df_scale2(Q[m])));
      acc_n[m] = df_neg(df_add(P[m], Q[m]));
    }
#pragma unroll
    for (int e = 0; e < 6; ++e) s1[e] = sq[e].hi;
#pragma unroll
    for (int m = 0; m < 5; ++m) c.rp[m] = 0.f;
    bt_f32_begin<DIR>(K, n, s0, s1, c);
  }
  for (int p = 1; p <= n - 2; ++p) {
    issue_fwd(p + PIPE - 1);
    cpa_wait<PIPE - 1>();
    const int slot = p % PIPE;
    df64 bd[5];
    if (p + 1 == n - 1) {
#pragma unroll
      for (int m = 0; m < 5; ++m) xq[m] = df64{*S(slot, m), *S(slot, 5 + m)};
    } else {
#pragma unroll
      for (int m = 0; m < 5; ++m) xq[m] = df64{*S(slot, m), 0.f};
    }
#pragma unroll
    for (int e = 0; e < 6; ++e) sq[e] = df64{*S(slot, 10 + e), *S(slot, 16 + e)};
#pragma unroll
    for (int m = 0; m < 5; ++m) bd[m] = df64{*S(slot, 22 + m), *S(slot, 27 + m)};
    pq(sq, xq, P, Q);
    float r[5], s[6];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const df64 tx = df_add(acc_c[m], df_sub(P[m], Q[m]));
      const df64 rr = df_sub(bd[m], tx);
      r[m] = rr.hi + rr.lo;
      acc_c[m] = df_add(acc_n[m], df_add(xq[m], df_scale2(Q[m])));
      acc_n[m] = df_neg(df_add(P[m], Q[m]));
    }
#pragma unroll
    for (int e = 0; e < 6; ++e) s[e] = sq[e].hi;
    bt_f32_step<DIR>(K, p, n, true, r, s, c, scr, nlt, gl);
    if (p + PIPE > n - 2) {
      // the ring does not refill this slot: C'_p and r'_p stay here for the
      // back substitution, x0_p (and u_p) are fetched now, so that it starts
      // without a trip to memory
#pragma unroll
      for (int a = 0; a < 5; ++a)
#pragma unroll
        for (int b = 0; b < 5; ++b) *S(slot, a * 5 + b) = c.Cp[a][b];
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        *S(slot, 25 + m) = c.rp[m];
        cpa4(S(slot, 30 + m), x0_at(p, m));
      }
      if (!OUT_DF && add_u) {
        const int64_t pt = base + (int64_t)p * st;
#pragma unroll
        for (int m = 0; m < 5; ++m) cpa8(SU(slot, m), F.u + m * NP + pt);
      }
      cpa_commit();
    }
  }
  cpa_wait<0>();
  // back substitution: step p (n-2 .. 1) consumes C'_p, r'_p, x0_p (and u_p)
  // from slot p % PIPE: the last PIPE points as the forward pass left them,
  // the others loaded PIPE steps ahead into the slot just consumed
  auto issue_bwd = [&](int p) {
    if (p >= 1) {
      const int slot = p % PIPE;
      const int64_t pt = base + (int64_t)p * st;
#pragma unroll
      for (int e = 0; e < 30; ++e) cpa4(S(slot, e), scr + ((int64_t)p * 30 + e) * nlt + gl);
#pragma unroll
      for (int m = 0; m < 5; ++m) cpa4(S(slot, 30 + m), x0_at(p, m));
      if (!OUT_DF && add_u) {
#pragma unroll
        for (int m = 0; m < 5; ++m) cpa8(SU(slot, m), F.u + m * NP + pt);
      }
    }
    cpa_commit();
  };
  float dn[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  for (int p = n - 2; p >= 1; --p) {
    if (p + PIPE <= n - 2) cpa_wait<PIPE - 1>();
    const int slot = p % PIPE;
    const int64_t pt = base + (int64_t)p * st;
    float d[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      float t = *S(slot, 25 + m);
#pragma unroll
      for (int cc = 0; cc < 5; ++cc) t -= *S(slot, m * 5 + cc) * dn[cc];
      d[m] = t;
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const float xv = *S(slot, 30 + m);
      if (OUT_DF) {
        // x: in place of b in the x-line-major copy (k_xline_back moves it
        // to rdf); y: rdf
        const df64 v = df_two_sum(xv, d[m]);
        float* o = DIR == 0 ? F.rdx + ((int64_t)p * 10 + m) * F.nlx + gl : bdf + m * NP + pt;
        const int64_t lo_off = DIR == 0 ? 5 * F.nlx : 5 * NP;
        o[0] = v.hi;
        o[lo_off] = v.lo;
      } else {
        // exact FP32 -> FP64 by bits (a conversion instruction takes the FP64 pipe)
        const double v = f32_to_f64(xv) + f32_to_f64(d[m]);
        rhs[m * NP + pt] = v;
        if (add_u) F.u[m * NP + pt] = *SU(slot, m) + v;
      }
      dn[m] = d[m];
    }
    issue_bwd(p - PIPE);
  }
  cpa_wait<0>();
}

template <int DIR, bool OUT_DF>
__global__ void __launch_bounds__(128, NPBMZ_BT_REFINE_MINB) k_bt_refine_pl(Fields F, Consts K, const Work* __restrict__ work, int nwork,
                                                      float* __restrict__ scr, int64_t nlt, int add_u,
                                                      const float* __restrict__ x0f) {
  extern __shared__ __align__(16) unsigned char pl_smem[];
  for (int it = blockIdx.x; it < nwork; it += gridDim.x)
    bt_refine_pl_item<DIR, OUT_DF>(F, K, work[it], scr, nlt, add_u, x0f, pl_smem);
}
#endif  // NPBMZ_HAS_FP32

// ============================================================================
// SP scalar pentadiagonal line solve, one thread per line.
// lhsx / lhsy / lhsz assembly (src/SP/lhsx.jl:27-111, lhsy.jl, lhsz.jl), the
// Thomas forward elimination and back substitution (src/SP/x_solve.jl:203-313,
// 456-512; y_solve.jl, z_solve.jl), then ninvr / pinvr / tzetar
// (src/SP/ninvr.jl:19-32, pinvr.jl:20-33, tzetar.jl:27-52) and, after the z
// sweep, add (src/SP/add.jl:14-23).  Rows 0 and n-1 are the identity rows
// lhsinit leaves in the persistent lhs (src/SP/initialize.jl:235-256); they go
// through the same elimination as in the reference.  The bands l4, l5 of each
// of the 3 systems are kept for the back substitution in
// scr[(p*6 + b) * nlt + global_line].
// ============================================================================
struct SpBands {
  double l[3][5];
};

template <int DIR, typename T, typename G>
__device__ __forceinline__ void sp_assemble(const Consts& K, int q, int n, const G cv[3], const G rhon[3],
                                            const G spd[3], T L[3][5]) {
  if (q == 0 || q == n - 1) {
#pragma unroll
    for (int s = 0; s < 3; ++s) { L[s][0] = (T)0.0; L[s][1] = (T)0.0; L[s][2] = (T)1.0; L[s][3] = (T)0.0; L[s][4] = (T)0.0; }
    return;
  }
  const G dtt1 = kv<G>(DIR == 0 ? K.dttx1 : DIR == 1 ? K.dtty1 : K.dttz1, K.f_dtt1[DIR]);
  const G dtt2 = kv<G>(DIR == 0 ? K.dttx2 : DIR == 1 ? K.dtty2 : K.dttz2, K.f_dtt2[DIR]);
  const G c2dtt1 = kv<G>(DIR == 0 ? K.c2dttx1 : DIR == 1 ? K.c2dtty1 : K.c2dttz1, K.f_c2dtt1[DIR]);
  const G comz1 = kv<G>(K.comz1, K.f_comz1), comz4 = kv<G>(K.comz4, K.f_comz4);
  const G comz5 = kv<G>(K.comz5, K.f_comz5), comz6 = kv<G>(K.comz6, K.f_comz6);
  G L1 = (G)0.0;
  G L2 = -dtt2 * cv[0] - dtt1 * rhon[0];
  G L3 = (G)1.0 + c2dtt1 * rhon[1];
  G L4 = dtt2 * cv[2] - dtt1 * rhon[2];
  G L5 = (G)0.0;
  if (q == 1) { L3 += comz5; L4 -= comz4; L5 += comz1; }
  if (q == 2) { L2 -= comz4; L3 += comz6; L4 -= comz4; L5 += comz1; }
  if (q >= 3 && q <= n - 4) { L1 += comz1; L2 -= comz4; L3 += comz6; L4 -= comz4; L5 += comz1; }
  if (q == n - 3) { L1 += comz1; L2 -= comz4; L3 += comz6; L4 -= comz4; }
  if (q == n - 2) { L1 += comz1; L2 -= comz4; L3 += comz5; }
  L[0][0] = (T)L1; L[0][1] = (T)L2; L[0][2] = (T)L3; L[0][3] = (T)L4; L[0][4] = (T)L5;
  L[1][0] = (T)L1; L[1][1] = (T)(L2 - dtt2 * spd[0]); L[1][2] = (T)L3; L[1][3] = (T)(L4 + dtt2 * spd[2]); L[1][4] = (T)L5;
  L[2][0] = (T)L1; L[2][1] = (T)(L2 + dtt2 * spd[0]); L[2][2] = (T)L3; L[2][3] = (T)(L4 - dtt2 * spd[2]); L[2][4] = (T)L5;
}

template <int DIR>
__device__ __forceinline__ void sp_geom(const Fields& F, const Consts& K, int64_t pt, double& cv, double& rhon,
                                        double& spd) {
  const int64_t NP = F.NP;
  const double ru1 = K.c3c4 * F.prim[PR_RHOI * NP + pt];
  cv = F.prim[(DIR == 0 ? PR_US : DIR == 1 ? PR_VS : PR_WS) * NP + pt];
  const double da = DIR == 0 ? K.dx2 : DIR == 1 ? K.dy3 : K.dz4;
  const double db = DIR == 0 ? K.dx5 : DIR == 1 ? K.dy5 : K.dz5;
  const double dm = DIR == 0 ? K.dxmax : DIR == 1 ? K.dymax : K.dzmax;
  const double dc = DIR == 0 ? K.dx1 : DIR == 1 ? K.dy1 : K.dz1;
  rhon = fmax(fmax(fmax(da + K.con43 * ru1, db + K.c1c5 * ru1), dm + ru1), dc);
  spd = F.prim[PR_SPEED * NP + pt];
}

// system s covers rhs components [s==0 ? 0..2 : s==1 ? 3 : 4]
#define SP_M0(s) ((s) == 0 ? 0 : (s) + 2)
#define SP_M1(s) ((s) == 0 ? 2 : (s) + 2)

// out / transform: the in-place solve writes the transformed solution into
// rhs (out == rhs, transform = 1); the first pass of the refined solve writes
// the untransformed solution of the interior points to a separate buffer.
template <int DIR, typename T>
__global__ void __launch_bounds__(128) k_sp_solve(Fields F, Consts K, const Work* __restrict__ work,
                                                  T* __restrict__ scr, int64_t nlt, int add_u,
                                                  double* __restrict__ out, int transform) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int line = w.first + threadIdx.x;
  if (line >= zone_lines(Z, DIR)) return;
  int64_t base, st;
  line_geometry(Z, DIR, line, base, st);
  const int n = zone_line_len(Z, DIR);
  const int64_t gl = Z.lineoff[DIR] + line;
  const int64_t NP = F.NP;
  double* __restrict__ rhs = F.rhs;

  // geometry window for assembling row q: values at q-1, q, q+1
  double gcv[4], grh[4], gsp[4];   // values at rows a-1 .. a+2 of a sliding window
  T cur3[3], cur4[3], cur5[3];     // row p   (l3, l4, l5), modified
  T nx2[3], nx3[3], nx4[3], nx5[3];  // row p+1 (l2..l5), modified
  T rr[3][5];                       // rhs rows p, p+1, p+2

  // rows 0 and 1: assemble
  {
    T L0[3][5], L1[3][5];
    double cv[3], rh[3], sp[3];
    // row 0 is an identity row; its geometry is not needed.
    sp_assemble<DIR, T>(K, 0, n, cv, rh, sp, L0);
    sp_geom<DIR>(F, K, base, gcv[0], grh[0], gsp[0]);
    sp_geom<DIR>(F, K, base + st, gcv[1], grh[1], gsp[1]);
    sp_geom<DIR>(F, K, base + 2 * st, gcv[2], grh[2], gsp[2]);
    cv[0] = gcv[0]; cv[1] = gcv[1]; cv[2] = gcv[2];
    rh[0] = grh[0]; rh[1] = grh[1]; rh[2] = grh[2];
    sp[0] = gsp[0]; sp[1] = gsp[1]; sp[2] = gsp[2];
    sp_assemble<DIR, T>(K, 1, n, cv, rh, sp, L1);
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      cur3[s] = L0[s][2]; cur4[s] = L0[s][3]; cur5[s] = L0[s][4];
      nx2[s] = L1[s][1]; nx3[s] = L1[s][2]; nx4[s] = L1[s][3]; nx5[s] = L1[s][4];
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      rr[0][m] = (T)rhs[m * NP + base];
      rr[1][m] = (T)rhs[m * NP + base + st];
    }
  }
  // window gcv[0..2] now holds rows 0,1,2.
  for (int p = 0; p <= n - 3; ++p) {
    // assemble row p+2 (needs geometry at p+1, p+2, p+3)
    T L2[3][5];
    {
      double cv[3], rh[3], sp[3];
      const int q = p + 2;
      if (q + 1 <= n - 1) sp_geom<DIR>(F, K, base + (int64_t)(q + 1) * st, gcv[3], grh[3], gsp[3]);
      cv[0] = gcv[1]; cv[1] = gcv[2]; cv[2] = gcv[3];
      rh[0] = grh[1]; rh[1] = grh[2]; rh[2] = grh[3];
      sp[0] = gsp[1]; sp[1] = gsp[2]; sp[2] = gsp[3];
      sp_assemble<DIR, T>(K, q, n, cv, rh, sp, L2);
      gcv[0] = gcv[1]; gcv[1] = gcv[2]; gcv[2] = gcv[3];
      grh[0] = grh[1]; grh[1] = grh[2]; grh[2] = grh[3];
      gsp[0] = gsp[1]; gsp[1] = gsp[2]; gsp[2] = gsp[3];
    }
    const int64_t pt2 = base + (int64_t)(p + 2) * st;
#pragma unroll
    for (int m = 0; m < 5; ++m) rr[2][m] = (T)rhs[m * NP + pt2];
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      const T fac1 = pivot_recip<T>(cur3[s]);
      cur4[s] *= fac1;
      cur5[s] *= fac1;
#pragma unroll
      for (int m = SP_M0(s); m <= SP_M1(s); ++m) rr[0][m] *= fac1;
      nx3[s] -= nx2[s] * cur4[s];
      nx4[s] -= nx2[s] * cur5[s];
#pragma unroll
      for (int m = SP_M0(s); m <= SP_M1(s); ++m) rr[1][m] -= nx2[s] * rr[0][m];
      T n2 = L2[s][1], n3 = L2[s][2];
      n2 -= L2[s][0] * cur4[s];
      n3 -= L2[s][0] * cur5[s];
#pragma unroll
      for (int m = SP_M0(s); m <= SP_M1(s); ++m) rr[2][m] -= L2[s][0] * rr[0][m];
      scr[((int64_t)p * 6 + 2 * s) * nlt + gl] = cur4[s];
      scr[((int64_t)p * 6 + 2 * s + 1) * nlt + gl] = cur5[s];
      // shift the window: row p+1 becomes current, row p+2 next
      cur3[s] = nx3[s]; cur4[s] = nx4[s]; cur5[s] = nx5[s];
      nx2[s] = n2; nx3[s] = n3; nx4[s] = L2[s][3]; nx5[s] = L2[s][4];
    }
    const int64_t pt = base + (int64_t)p * st;
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      if (p > 0) out[m * NP + pt] = (double)rr[0][m];
      rr[0][m] = rr[1][m];
      rr[1][m] = rr[2][m];
    }
  }
  // last two rows: p = n-2 (current), n-1 (next)
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    const T fac1 = pivot_recip<T>(cur3[s]);
    cur4[s] *= fac1;
    cur5[s] *= fac1;
#pragma unroll
    for (int m = SP_M0(s); m <= SP_M1(s); ++m) rr[0][m] *= fac1;
    nx3[s] -= nx2[s] * cur4[s];
    nx4[s] -= nx2[s] * cur5[s];
#pragma unroll
    for (int m = SP_M0(s); m <= SP_M1(s); ++m) rr[1][m] -= nx2[s] * rr[0][m];
    const T fac2 = pivot_recip<T>(nx3[s]);
    nx4[s] *= fac2;
    nx5[s] *= fac2;
#pragma unroll
    for (int m = SP_M0(s); m <= SP_M1(s); ++m) rr[1][m] *= fac2;
  }
  // back substitution; rr[0] = row n-2, rr[1] = row n-1 (the boundary row,
  // numerically unchanged).  b1 = r_{p+1}, b2 = r_{p+2} before transforms.
  T b1[5], b2[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) b2[m] = rr[1][m];
  {
    const int p = n - 2;
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const int s = m < 3 ? 0 : m - 2;
      b1[m] = rr[0][m] - cur4[s] * b2[m];
    }
    (void)p;
  }
  // Emit row n-2, then rows n-3 .. 1.
  auto emit = [&](int p, const T v[5]) {
    const int64_t pt = base + (int64_t)p * st;
    double r1 = (double)v[0], r2 = (double)v[1], r3 = (double)v[2], r4 = (double)v[3], r5 = (double)v[4];
    if (!transform) {
      out[pt] = r1; out[NP + pt] = r2; out[2 * NP + pt] = r3; out[3 * NP + pt] = r4; out[4 * NP + pt] = r5;
      return;
    }
    double o[5];
    if (DIR == 0) {  // ninvr
      const double t1 = K.bt * r3;
      const double t2 = 0.5e0 * (r4 + r5);
      o[0] = -r2; o[1] = r1; o[2] = K.bt * (r4 - r5); o[3] = -t1 + t2; o[4] = t1 + t2;
    } else if (DIR == 1) {  // pinvr
      const double t1 = K.bt * r1;
      const double t2 = 0.5e0 * (r4 + r5);
      o[0] = K.bt * (r4 - r5); o[1] = -r3; o[2] = r2; o[3] = -t1 + t2; o[4] = t1 + t2;
    } else {  // tzetar
      const double xvel = F.prim[PR_US * NP + pt], yvel = F.prim[PR_VS * NP + pt], zvel = F.prim[PR_WS * NP + pt];
      const double ac = F.prim[PR_SPEED * NP + pt], acinv = F.prim[PR_AINV * NP + pt];
      const double ac2u = ac * ac;
      const double uzik1 = F.u[pt];
      const double btuz = K.bt * uzik1;
      const double t1 = btuz * acinv * (r4 + r5);
      const double t2 = r3 + t1;
      const double t3 = btuz * (r4 - r5);
      o[0] = t2;
      o[1] = -uzik1 * r2 + xvel * t2;
      o[2] = uzik1 * r1 + yvel * t2;
      o[3] = zvel * t2 + t3;
      o[4] = uzik1 * (-xvel * r2 + yvel * r1) + F.prim[PR_QS * NP + pt] * t2 + K.c2iv * ac2u * t1 + zvel * t3;
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      rhs[m * NP + pt] = o[m];
      if (add_u) F.u[m * NP + pt] += o[m];
    }
  };
  // row n-2's transform must read u before row n-2 is updated; emit updates
  // only its own point, so the order below is safe.
  emit(n - 2, b1);
  for (int p = n - 3; p >= 1; --p) {
    const int64_t pt = base + (int64_t)p * st;
    T r[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const int s = m < 3 ? 0 : m - 2;
      const T l4 = scr[((int64_t)p * 6 + 2 * s) * nlt + gl];
      const T l5 = scr[((int64_t)p * 6 + 2 * s + 1) * nlt + gl];
      r[m] = (T)out[m * NP + pt];
      r[m] -= l4 * b1[m] + l5 * b2[m];
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) { b2[m] = b1[m]; b1[m] = r[m]; }
    emit(p, r);
  }
}

// ============================================================================
// Refinement pass of the mixed-precision SP sweep: residual r = b - L x0 of
// each scalar pentadiagonal system in FP64 (bands of lhsx/lhsy/lhsz
// assembled in FP64), FP32 Thomas solve of L d = r, x = x0 + d, then the
// sweep's transform (ninvr / pinvr / tzetar) and, after the z sweep, add.
// x0 comes from xw on interior points; boundary rows are identity rows, so
// x0 there is b itself and the residual is zero.
// ============================================================================
template <int DIR>
__device__ __forceinline__ void sp_transform(const Fields& F, const Consts& K, int64_t pt, const double v[5],
                                             double o[5]) {
  const int64_t NP = F.NP;
  const double r1 = v[0], r2 = v[1], r3 = v[2], r4 = v[3], r5 = v[4];
  if (DIR == 0) {
    const double t1 = K.bt * r3;
    const double t2 = 0.5e0 * (r4 + r5);
    o[0] = -r2; o[1] = r1; o[2] = K.bt * (r4 - r5); o[3] = -t1 + t2; o[4] = t1 + t2;
  } else if (DIR == 1) {
    const double t1 = K.bt * r1;
    const double t2 = 0.5e0 * (r4 + r5);
    o[0] = K.bt * (r4 - r5); o[1] = -r3; o[2] = r2; o[3] = -t1 + t2; o[4] = t1 + t2;
  } else {
    const double xvel = F.prim[PR_US * NP + pt], yvel = F.prim[PR_VS * NP + pt], zvel = F.prim[PR_WS * NP + pt];
    const double ac = F.prim[PR_SPEED * NP + pt], acinv = F.prim[PR_AINV * NP + pt];
    const double ac2u = ac * ac;
    const double uzik1 = F.u[pt];
    const double btuz = K.bt * uzik1;
    const double t1 = btuz * acinv * (r4 + r5);
    const double t2 = r3 + t1;
    const double t3 = btuz * (r4 - r5);
    o[0] = t2;
    o[1] = -uzik1 * r2 + xvel * t2;
    o[2] = uzik1 * r1 + yvel * t2;
    o[3] = zvel * t2 + t3;
    o[4] = uzik1 * (-xvel * r2 + yvel * r1) + F.prim[PR_QS * NP + pt] * t2 + K.c2iv * ac2u * t1 + zvel * t3;
  }
}

// Geometry of one point for the SP band assembly, generic in the type.
template <int DIR, typename G>
__device__ __forceinline__ void sp_geom_t(G ri, G cvel, G spd_in, const Consts& K, G& cv, G& rhon, G& spd) {
  const G ru1 = kv<G>(K.c3c4, K.f_c3c4) * ri;
  cv = cvel;
  const G da = kv<G>(DIR == 0 ? K.dx2 : DIR == 1 ? K.dy3 : K.dz4, K.f_d[DIR][DIR + 1]);
  const G db = kv<G>(DIR == 0 ? K.dx5 : DIR == 1 ? K.dy5 : K.dz5, K.f_d[DIR][4]);
  const G dm = kv<G>(DIR == 0 ? K.dxmax : DIR == 1 ? K.dymax : K.dzmax, K.f_dmax[DIR]);
  const G dc = kv<G>(DIR == 0 ? K.dx1 : DIR == 1 ? K.dy1 : K.dz1, K.f_d[DIR][0]);
  rhon = fmax(fmax(fmax(da + kv<G>(K.con43, K.f_con43) * ru1, db + kv<G>(K.c1c5, K.f_c1c5) * ru1), dm + ru1), dc);
  spd = spd_in;
}

// Thomas forward elimination of the three SP systems over one line, in FP32,
// with rows supplied by row_at(q, L, r) (q = 0..n-1; L[3][5] bands, r[5]).
// Bands l4, l5 and the eliminated rhs of rows 0..n-3 go to the line scratch
// scr[(p*11 + e) * nlt + gl]; rows n-2 and n-1 stay in the returned state.
struct SpF32Tail {
  float cur4[3];     // l4 of row n-2
  float r2[5];       // eliminated rhs of row n-2
  float rlast[5];    // eliminated rhs of row n-1
};

template <typename RowAt>
__device__ __forceinline__ void sp_forward_f32(int n, float* __restrict__ scr, int64_t nlt, int64_t gl, RowAt row_at,
                                               SpF32Tail& tail) {
  float cur3[3], cur4[3], cur5[3], nx2[3], nx3[3], nx4[3], nx5[3];
  float rr[3][5];
  {
    float L0[3][5], L1[3][5];
    row_at(0, L0, rr[0]);
    row_at(1, L1, rr[1]);
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      cur3[s] = L0[s][2]; cur4[s] = L0[s][3]; cur5[s] = L0[s][4];
      nx2[s] = L1[s][1]; nx3[s] = L1[s][2]; nx4[s] = L1[s][3]; nx5[s] = L1[s][4];
    }
  }
  for (int p = 0; p <= n - 3; ++p) {
    float L2[3][5];
    row_at(p + 2, L2, rr[2]);
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      const float fac1 = __fdividef(1.0f, cur3[s]);
      cur4[s] *= fac1;
      cur5[s] *= fac1;
#pragma unroll
      for (int m = SP_M0(s); m <= SP_M1(s); ++m) rr[0][m] *= fac1;
      nx3[s] -= nx2[s] * cur4[s];
      nx4[s] -= nx2[s] * cur5[s];
#pragma unroll
      for (int m = SP_M0(s); m <= SP_M1(s); ++m) rr[1][m] -= nx2[s] * rr[0][m];
      float n2 = L2[s][1], n3 = L2[s][2];
      n2 -= L2[s][0] * cur4[s];
      n3 -= L2[s][0] * cur5[s];
#pragma unroll
      for (int m = SP_M0(s); m <= SP_M1(s); ++m) rr[2][m] -= L2[s][0] * rr[0][m];
      scr[((int64_t)p * 11 + 2 * s) * nlt + gl] = cur4[s];
      scr[((int64_t)p * 11 + 2 * s + 1) * nlt + gl] = cur5[s];
      cur3[s] = nx3[s]; cur4[s] = nx4[s]; cur5[s] = nx5[s];
      nx2[s] = n2; nx3[s] = n3; nx4[s] = L2[s][3]; nx5[s] = L2[s][4];
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      scr[((int64_t)p * 11 + 6 + m) * nlt + gl] = rr[0][m];
      rr[0][m] = rr[1][m];
      rr[1][m] = rr[2][m];
    }
  }
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    const float fac1 = __fdividef(1.0f, cur3[s]);
    cur4[s] *= fac1;
    cur5[s] *= fac1;
#pragma unroll
    for (int m = SP_M0(s); m <= SP_M1(s); ++m) rr[0][m] *= fac1;
    nx3[s] -= nx2[s] * cur4[s];
    nx4[s] -= nx2[s] * cur5[s];
#pragma unroll
    for (int m = SP_M0(s); m <= SP_M1(s); ++m) rr[1][m] -= nx2[s] * rr[0][m];
    const float fac2 = __fdividef(1.0f, nx3[s]);
#pragma unroll
    for (int m = SP_M0(s); m <= SP_M1(s); ++m) rr[1][m] *= fac2;
    tail.cur4[s] = cur4[s];
  }
#pragma unroll
  for (int m = 0; m < 5; ++m) { tail.r2[m] = rr[0][m]; tail.rlast[m] = rr[1][m]; }
}

// Back substitution of the three systems; emit(p, v[5]) receives rows n-2..1.
template <typename Emit>
__device__ __forceinline__ void sp_back_f32(int n, const float* __restrict__ scr, int64_t nlt, int64_t gl,
                                            const SpF32Tail& tail, Emit emit) {
  float b1[5], b2[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    const int s = m < 3 ? 0 : m - 2;
    b2[m] = tail.rlast[m];
    b1[m] = tail.r2[m] - tail.cur4[s] * b2[m];
  }
  emit(n - 2, b1);
  for (int p = n - 3; p >= 1; --p) {
    float r[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const int s = m < 3 ? 0 : m - 2;
      const float l4 = scr[((int64_t)p * 11 + 2 * s) * nlt + gl];
      const float l5 = scr[((int64_t)p * 11 + 2 * s + 1) * nlt + gl];
      r[m] = scr[((int64_t)p * 11 + 6 + m) * nlt + gl] - (l4 * b1[m] + l5 * b2[m]);
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) { b2[m] = b1[m]; b1[m] = r[m]; }
    emit(p, r);
  }
}

// Pass 1 of the mixed SP sweep: all three systems in FP32 from the FP32
// geometry copies; x0 (untransformed) in FP32.  Geometry of point q+1 is
// fetched one row ahead.
template <int DIR>
__global__ void __launch_bounds__(128) k_sp_mixed_solve(Fields F, Consts K, const Work* __restrict__ work,
                                                        float* __restrict__ scr, int64_t nlt,
                                                        float* __restrict__ x0) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int line = w.first + threadIdx.x;
  if (line >= zone_lines(Z, DIR)) return;
  int64_t base, st;
  line_geometry(Z, DIR, line, base, st);
  const int n = zone_line_len(Z, DIR);
  const int64_t gl = Z.lineoff[DIR] + line;
  const int64_t NP = F.NP;
  const double* __restrict__ rhs = F.rhs;
  const float* pf = F.primf;
  const int PCV = DIR == 0 ? PS_US : DIR == 1 ? PS_VS : PS_WS;
  // geometry window: values at rows q-1, q, q+1 of the row being assembled
  float gcv[3], grh[3], gsp[3];
  auto geom = [&](int q, float& cv, float& rh, float& sp) {
    const int64_t pt = base + (int64_t)q * st;
    sp_geom_t<DIR, float>(pf[PS_RHOI * NP + pt], pf[PCV * NP + pt], pf[PS_SPEED * NP + pt], K, cv, rh, sp);
  };
  geom(0, gcv[1], grh[1], gsp[1]);
  geom(1, gcv[2], grh[2], gsp[2]);
  gcv[0] = gcv[1]; grh[0] = grh[1]; gsp[0] = gsp[1];
  float ncv = 0.f, nrh = 0.f, nsp = 0.f;
  if (n > 2) geom(2, ncv, nrh, nsp);
  auto row_at = [&](int q, float L[3][5], float r[5]) {
    // window holds q-1, q, q+1 on entry (q+1 from the prefetch)
    sp_assemble<DIR, float, float>(K, q, n, gcv, grh, gsp, L);
    const int64_t pt = base + (int64_t)q * st;
#pragma unroll
    for (int m = 0; m < 5; ++m) r[m] = (float)rhs[m * NP + pt];
    // shift: q, q+1, prefetched q+2
    gcv[0] = gcv[1]; grh[0] = grh[1]; gsp[0] = gsp[1];
    gcv[1] = gcv[2]; grh[1] = grh[2]; gsp[1] = gsp[2];
    gcv[2] = ncv; grh[2] = nrh; gsp[2] = nsp;
    if (q + 3 <= n - 1) geom(q + 3, ncv, nrh, nsp);
  };
  SpF32Tail tail;
  sp_forward_f32(n, scr, nlt, gl, row_at, tail);
  sp_back_f32(n, scr, nlt, gl, tail, [&](int p, const float v[5]) {
    const int64_t pt = base + (int64_t)p * st;
#pragma unroll
    for (int m = 0; m < 5; ++m) x0[m * NP + pt] = v[m];
  });
}

// Pass 2 of the mixed SP sweep: residual r = b - L x0 of each system in FP64
// (bands of lhsx/lhsy/lhsz assembled in FP64 from a geometry window), the
// FP32 Thomas solve of L d = r, x = x0 + d, the sweep's transform and, after
// the z sweep, add.  x0 is b itself on the boundary rows (identity rows).
template <int DIR>
__global__ void __launch_bounds__(128) k_sp_refine(Fields F, Consts K, const Work* __restrict__ work,
                                                   float* __restrict__ scr, int64_t nlt, int add_u,
                                                   const float* __restrict__ x0f) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int line = w.first + threadIdx.x;
  if (line >= zone_lines(Z, DIR)) return;
  int64_t base, st;
  line_geometry(Z, DIR, line, base, st);
  const int n = zone_line_len(Z, DIR);
  const int64_t gl = Z.lineoff[DIR] + line;
  const int64_t NP = F.NP;
  double* __restrict__ rhs = F.rhs;
  const int PCV = DIR == 0 ? PR_US : DIR == 1 ? PR_VS : PR_WS;
  auto geom = [&](int q, double& cv, double& rh, double& sp) {
    const int64_t pt = base + (int64_t)q * st;
    sp_geom_t<DIR, double>(F.prim[PR_RHOI * NP + pt], F.prim[PCV * NP + pt], F.prim[PR_SPEED * NP + pt], K, cv, rh,
                           sp);
  };
  auto load_x = [&](int q, double x[5]) {
    const int64_t pt = base + (int64_t)q * st;
    if (q < 0 || q > n - 1) {
#pragma unroll
      for (int m = 0; m < 5; ++m) x[m] = 0.0;
    } else if (q == 0 || q == n - 1) {
#pragma unroll
      for (int m = 0; m < 5; ++m) x[m] = rhs[m * NP + pt];
    } else {
#pragma unroll
      for (int m = 0; m < 5; ++m) x[m] = (double)x0f[m * NP + pt];
    }
  };
  // windows for the row being assembled, q: geometry at q-1, q, q+1 and x0 at
  // q-2 .. q+2
  double gcv[3], grh[3], gsp[3], ncv = 0.0, nrh = 0.0, nsp = 0.0;
  double xw[5][5], nxp[5];
  geom(0, gcv[1], grh[1], gsp[1]);
  gcv[0] = gcv[1]; grh[0] = grh[1]; gsp[0] = gsp[1];
  geom(1, gcv[2], grh[2], gsp[2]);
  if (n > 2) geom(2, ncv, nrh, nsp);
  load_x(-2, xw[0]);
  load_x(-1, xw[1]);
  load_x(0, xw[2]);
  load_x(1, xw[3]);
  load_x(2, xw[4]);
  load_x(3, nxp);
  auto row_at = [&](int q, float L[3][5], float r[5]) {
    double Ld[3][5];
    sp_assemble<DIR, double, double>(K, q, n, gcv, grh, gsp, Ld);
#pragma unroll
    for (int s = 0; s < 3; ++s)
#pragma unroll
      for (int b = 0; b < 5; ++b) L[s][b] = (float)Ld[s][b];
    if (q == 0 || q == n - 1) {
#pragma unroll
      for (int m = 0; m < 5; ++m) r[m] = 0.f;
    } else {
      const int64_t pt = base + (int64_t)q * st;
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        const int s = m < 3 ? 0 : m - 2;
        const double t = Ld[s][0] * xw[0][m] + Ld[s][1] * xw[1][m] + Ld[s][2] * xw[2][m] + Ld[s][3] * xw[3][m] +
                         Ld[s][4] * xw[4][m];
        r[m] = (float)(rhs[m * NP + pt] - t);
      }
    }
    // advance the windows to row q+1 (values of q+2 / q+3 were fetched one
    // row earlier; fetch the next ones now)
    gcv[0] = gcv[1]; grh[0] = grh[1]; gsp[0] = gsp[1];
    gcv[1] = gcv[2]; grh[1] = grh[2]; gsp[1] = gsp[2];
    gcv[2] = ncv; grh[2] = nrh; gsp[2] = nsp;
    if (q + 3 <= n - 1) geom(q + 3, ncv, nrh, nsp);
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int m = 0; m < 5; ++m) xw[k][m] = xw[k + 1][m];
#pragma unroll
    for (int m = 0; m < 5; ++m) xw[4][m] = nxp[m];
    load_x(q + 4, nxp);
  };
  SpF32Tail tail;
  sp_forward_f32(n, scr, nlt, gl, row_at, tail);
  sp_back_f32(n, scr, nlt, gl, tail, [&](int p, const float d[5]) {
    const int64_t pt = base + (int64_t)p * st;
    double v[5], o[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) v[m] = (double)x0f[m * NP + pt] + (double)d[m];
    sp_transform<DIR>(F, K, pt, v, o);
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      rhs[m * NP + pt] = o[m];
      if (add_u) F.u[m * NP + pt] += o[m];
    }
  });
}

#if NPBMZ_HAS_FP32
#include "sp_pipelined.cuh"
#include "rhs_df.cuh"
#endif

// ============================================================================
// add (src/BT/add.jl:5-24, src/SP/add.jl:6-26) as a separate phase.
// ============================================================================
__global__ void __launch_bounds__(128) k_add(Fields F, const Work* __restrict__ work) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int q = w.first + threadIdx.x;
  if (q >= Z.nx * Z.ny * Z.nz) return;
  const int i = q % Z.nx, j = (q / Z.nx) % Z.ny, k = q / (Z.nx * Z.ny);
  if (i == 0 || i == Z.nx - 1 || j == 0 || j == Z.ny - 1 || k == 0 || k == Z.nz - 1) return;
  const int64_t p = Z.off + q;
  for (int m = 0; m < 5; ++m) F.u[m * F.NP + p] += F.rhs[m * F.NP + p];
}

#ifndef NPBMZ_NO_LAUNCHERS
// ============================================================================
// host-side launchers (declared in step_launch.h)
// ============================================================================
// Grid of a work-item kernel: one CTA per item, or (persistent) as many CTAs
// as fit on the device at once, each looping over items.
// Grid of a work-list kernel: one CTA per item, or (persist) as many CTAs as
// fit on the SMs looping over the items; ctas_per_sm > 0 makes it persistent
// with at most that many CTAs per SM, which leaves room on every SM for the
// CTAs of kernels running beside it on other streams.
static int item_grid(const void* f, int nwork, int tpb, size_t smem, bool persist, int ctas_per_sm = 0) {
  if (!persist && ctas_per_sm <= 0) return nwork;
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, f, tpb, smem) != cudaSuccess || per < 1) per = 1;
  if (ctas_per_sm > 0 && ctas_per_sm < per) per = ctas_per_sm;
  return nwork < per * sms ? nwork : per * sms;
}

void launch_prim_w(bool sp, const Fields& F, const Consts& K, const Work* work, int nwork, cudaStream_t s,
                   bool persist) {
  if (nwork <= 0) return;
  if (sp) k_prim_w<true><<<item_grid((const void*)k_prim_w<true>, nwork, 128, 0, persist), 128, 0, s>>>(F, K, work, nwork);
  else k_prim_w<false><<<item_grid((const void*)k_prim_w<false>, nwork, 128, 0, persist), 128, 0, s>>>(F, K, work, nwork);
}

void launch_prim(bool sp, const Fields& F, const Consts& K, int64_t lo, int64_t hi, cudaStream_t s) {
  if (hi <= lo) return;
  int64_t g = (hi - lo + 255) / 256;
  const int grid = (int)(g > 8192 ? 8192 : g);
  if (sp) k_prim<true><<<grid, 256, 0, s>>>(F, K, lo, hi);
  else k_prim<false><<<grid, 256, 0, s>>>(F, K, lo, hi);
}

void launch_rhs(bool tx, bool norm, const Fields& F, const Consts& K, const Work* work, int nwork, double* partials,
                cudaStream_t s, const RhsF64Consts* rc, bool persist) {
  if (nwork <= 0) return;
#if NPBMZ_HAS_FP32
  if (F.flux && F.fdt && rc) {
#define NPBMZ_RHS_FLUX(A, B)                                                                                  \
  k_rhs_flux<A, B><<<item_grid((const void*)k_rhs_flux<A, B>, nwork, 128, 0, persist), 128, 0, s>>>(F, K, *rc, work, \
                                                                                                  nwork, partials)
    if (tx) {
      if (norm) NPBMZ_RHS_FLUX(true, true);
      else NPBMZ_RHS_FLUX(true, false);
    } else {
      if (norm) NPBMZ_RHS_FLUX(false, true);
      else NPBMZ_RHS_FLUX(false, false);
    }
#undef NPBMZ_RHS_FLUX
    return;
  }
#endif
  if (tx) {
    if (norm) k_rhs<true, true><<<nwork, 128, 0, s>>>(F, K, work, partials);
    else k_rhs<true, false><<<nwork, 128, 0, s>>>(F, K, work, partials);
  } else {
    if (norm) k_rhs<false, true><<<nwork, 128, 0, s>>>(F, K, work, partials);
    else k_rhs<false, false><<<nwork, 128, 0, s>>>(F, K, work, partials);
  }
}

template <typename T>
static void launch_solve_t(bool sp, int dir, const Fields& F, const Consts& K, const Work* work, int nwork, int tpb,
                           void* scratch, int64_t nlt, int add_u, double* out, int transform, cudaStream_t s) {
  T* scr = reinterpret_cast<T*>(scratch);
  if (sp) {
    if (dir == 0) k_sp_solve<0, T><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, add_u, out, transform);
    else if (dir == 1) k_sp_solve<1, T><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, add_u, out, transform);
    else k_sp_solve<2, T><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, add_u, out, transform);
  } else {
    if (dir == 0) k_bt_solve<0, T><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, add_u, out);
    else if (dir == 1) k_bt_solve<1, T><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, add_u, out);
    else k_bt_solve<2, T><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, add_u, out);
  }
}

// mode 0: FP64 in place; 1: FP32 in place; 2: FP32 + refinement with a
// double-float residual (BT; SP: FP64 residual); 3: FP32 + refinement with
// an FP64 residual (xw: a [5][NP] buffer for the first solution).
void launch_solve(bool sp, int mode, int dir, const Fields& F, const Consts& K, const Work* work, int nwork, int tpb,
                  void* scratch, int64_t nlt, int add_u, double* xw, cudaStream_t s, bool persist, int ctas_per_sm) {
  if (nwork <= 0) return;
#if NPBMZ_HAS_FP32
  if (mode == 1) { launch_solve_t<float>(sp, dir, F, K, work, nwork, tpb, scratch, nlt, add_u, F.rhs, 1, s); return; }
  if (mode == 4 && sp) {
    // one fused step, SP: the pipelined passes with a double-float residual;
    // x and y hand their transformed results on as double-float
    float* scr = reinterpret_cast<float*>(scratch);
    float* x0 = reinterpret_cast<float*>(xw);
    const size_t sm_m = pls_mixed_smem(tpb), sm_r = pls_refine_smem(tpb, dir != 2);
#define NPBMZ_SPL(D, OD)                                                                                          \
  do {                                                                                                            \
    k_sp_mixed_pl<D><<<item_grid((const void*)k_sp_mixed_pl<D>, nwork, tpb, sm_m, persist, ctas_per_sm), tpb,     \
                       sm_m, s>>>(                                                                                \
        F, K, work, nwork, scr, nlt, x0);                                                                         \
    k_sp_refine_pl<D, OD><<<item_grid((const void*)k_sp_refine_pl<D, OD>, nwork, tpb, sm_r, persist, ctas_per_sm), \
                            tpb, sm_r,                                                                            \
                            s>>>(F, K, work, nwork, scr, nlt, add_u, x0);                                         \
  } while (0)
    if (dir == 0) {
      NPBMZ_SPL(0, true);
      k_xline_back<<<nwork, 256, 0, s>>>(F, work, nwork, tpb);
    } else if (dir == 1) NPBMZ_SPL(1, true);
    else NPBMZ_SPL(2, false);
#undef NPBMZ_SPL
    return;
  }
  if (mode == 4 && !sp) {
    // one fused step: b of the x sweep comes from compute_rhs's double-float
    // copy, x and y hand their results on as double-float (x through its
    // x-line-major copy), z writes FP64 rhs (and u)
    float* scr = reinterpret_cast<float*>(scratch);
    float* x0 = reinterpret_cast<float*>(xw);
    const size_t sm_m = pl_mixed_smem(tpb), sm_r = pl_refine_smem(tpb, dir != 2);
#define NPBMZ_PL(D, OD)                                                                                          \
  do {                                                                                                           \
    k_bt_mixed_pl<D><<<item_grid((const void*)k_bt_mixed_pl<D>, nwork, tpb, sm_m, persist, ctas_per_sm), tpb,     \
                       sm_m, s>>>(                                                                                \
        F, K, work, nwork, scr, nlt, x0);                                                                        \
    k_bt_refine_pl<D, OD><<<item_grid((const void*)k_bt_refine_pl<D, OD>, nwork, tpb, sm_r, persist, ctas_per_sm), \
                            tpb, sm_r,                                                                            \
                            s>>>(F, K, work, nwork, scr, nlt, add_u, x0);                                        \
  } while (0)
    if (dir == 0) {
      NPBMZ_PL(0, true);
      k_xline_back<<<nwork, 256, 0, s>>>(F, work, nwork, tpb);
    } else if (dir == 1) NPBMZ_PL(1, true);
    else NPBMZ_PL(2, false);
#undef NPBMZ_PL
    return;
  }
  if (mode == 4) mode = 2;
  if (mode == 2 || mode == 3) {
    const bool resid64 = mode == 3;
    float* scr = reinterpret_cast<float*>(scratch);
    if (sp) {
      float* x0 = reinterpret_cast<float*>(xw);
      if (dir == 0) {
        k_sp_mixed_solve<0><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, x0);
        k_sp_refine<0><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, add_u, x0);
      } else if (dir == 1) {
        k_sp_mixed_solve<1><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, x0);
        k_sp_refine<1><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, add_u, x0);
      } else {
        k_sp_mixed_solve<2><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, x0);
        k_sp_refine<2><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, add_u, x0);
      }
    } else {
      float* x0 = reinterpret_cast<float*>(xw);
      if (dir == 0) {
        k_bt_mixed_solve<0, false><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, x0);
        if (resid64) k_bt_refine<0><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, add_u, x0);
        else k_bt_refine_df<0, false, false><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, add_u, x0);
      } else if (dir == 1) {
        k_bt_mixed_solve<1, false><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, x0);
        if (resid64) k_bt_refine<1><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, add_u, x0);
        else k_bt_refine_df<1, false, false><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, add_u, x0);
      } else {
        k_bt_mixed_solve<2, false><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, x0);
        if (resid64) k_bt_refine<2><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, add_u, x0);
        else k_bt_refine_df<2, false, false><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, add_u, x0);
      }
    }
    return;
  }
#else
  (void)xw;
#endif
  (void)mode;
  launch_solve_t<double>(sp, dir, F, K, work, nwork, tpb, scratch, nlt, add_u, F.rhs, 1, s);
}

#if NPBMZ_HAS_FP32
// Opt the pipelined sweeps into their dynamic shared memory (above 48 KB for
// 128 threads per CTA); called once per handle, outside any stream capture.
int configure_kernels() {
  size_t cap_b = pl_refine_smem(128, false);
  for (size_t b : {pl_mixed_smem(128), pls_mixed_smem(128), pls_refine_smem(128, false)})
    if (b > cap_b) cap_b = b;
  const int cap = (int)cap_b;
  cudaError_t e = cudaSuccess;
  auto set = [&](const void* f) {
    const cudaError_t r = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
    if (r != cudaSuccess) e = r;
  };
  set((const void*)k_bt_mixed_pl<0>);
  set((const void*)k_bt_mixed_pl<1>);
  set((const void*)k_bt_mixed_pl<2>);
  set((const void*)k_bt_refine_pl<0, true>);
  set((const void*)k_bt_refine_pl<1, true>);
  set((const void*)k_bt_refine_pl<2, false>);
  set((const void*)k_sp_mixed_pl<0>);
  set((const void*)k_sp_mixed_pl<1>);
  set((const void*)k_sp_mixed_pl<2>);
  set((const void*)k_sp_refine_pl<0, true>);
  set((const void*)k_sp_refine_pl<1, true>);
  set((const void*)k_sp_refine_pl<2, false>);
  return e == cudaSuccess ? 0 : -1;
}

void launch_xline_ends(const Fields& F, const Work* work, int nwork, int tpb, cudaStream_t s) {
  if (nwork > 0) k_xline_ends<<<nwork, tpb, 0, s>>>(F, work);
}

void launch_prim_df(bool sp, const Fields& F, const RhsDfConsts& C, const Work* work, int nwork, cudaStream_t s,
                    bool persist) {
  if (nwork <= 0) return;
  if (sp) k_prim_df<true><<<item_grid((const void*)k_prim_df<true>, nwork, 128, 0, persist), 128, 0, s>>>(F, C, work, nwork);
  else k_prim_df<false><<<item_grid((const void*)k_prim_df<false>, nwork, 128, 0, persist), 128, 0, s>>>(F, C, work, nwork);
}

void launch_rhs_df(bool tx, bool norm, const Fields& F, const RhsDfConsts& C, const Work* work, int nwork,
                   double* partials, cudaStream_t s, bool persist) {
  if (nwork <= 0) return;
#define NPBMZ_RHS_DF(A, B)                                                                                      \
  do {                                                                                                          \
    if (C.exact_w)                                                                                              \
      k_rhs_df<A, B, true><<<item_grid((const void*)k_rhs_df<A, B, true>, nwork, 128, 0, persist), 128, 0, s>>>(  \
          F, C, work, nwork, partials);                                                                         \
    else                                                                                                        \
      k_rhs_df<A, B, false><<<item_grid((const void*)k_rhs_df<A, B, false>, nwork, 128, 0, persist), 128, 0, s>>>( \
          F, C, work, nwork, partials);                                                                         \
  } while (0)
  if (tx) {
    if (norm) NPBMZ_RHS_DF(true, true);
    else NPBMZ_RHS_DF(true, false);
  } else {
    if (norm) NPBMZ_RHS_DF(false, true);
    else NPBMZ_RHS_DF(false, false);
  }
#undef NPBMZ_RHS_DF
}

void launch_xline_copy(bool sp, const Fields& F, const Work* work, int nwork, int lpi, cudaStream_t s) {
  if (nwork <= 0) return;
  if (sp) k_xline_copy<true><<<nwork, 256, 0, s>>>(F, work, nwork, lpi);
  else k_xline_copy<false><<<nwork, 256, 0, s>>>(F, work, nwork, lpi);
}

void launch_rhs_xc(bool tx, bool norm, const Fields& F, const Consts& K, const RhsF64Consts& rc, const Work* work,
                   int nwork, double* partials, const Work* cwork, int ncopy, int lpi, cudaStream_t s, bool persist) {
  if (nwork + ncopy <= 0) return;
#define NPBMZ_RHS_XC(A, B)                                                                                   \
  k_rhs_flux_xc<A, B><<<item_grid((const void*)k_rhs_flux_xc<A, B>, nwork + ncopy, 128, 0, persist), 128, 0, s>>>( \
      F, K, rc, work, nwork, partials, cwork, ncopy, lpi)
  if (tx) {
    if (norm) NPBMZ_RHS_XC(true, true);
    else NPBMZ_RHS_XC(true, false);
  } else {
    if (norm) NPBMZ_RHS_XC(false, true);
    else NPBMZ_RHS_XC(false, false);
  }
#undef NPBMZ_RHS_XC
}

void launch_scale(const double* src, double* dst, double a, int64_t n, cudaStream_t s) {
  int64_t g = (n + 255) / 256;
  k_scale<<<(int)(g > 8192 ? 8192 : g), 256, 0, s>>>(src, dst, a, n);
}

void launch_split_f2(const double* src, float2* dst, int64_t NP, cudaStream_t s) {
  int64_t g = (5 * NP + 255) / 256;
  k_split_f2<<<(int)(g > 8192 ? 8192 : g), 256, 0, s>>>(src, dst, NP);
}

void launch_split_df(const double* src, float* dst, int64_t NP, cudaStream_t s) {
  int64_t g = (5 * NP + 255) / 256;
  k_split_df<<<(int)(g > 8192 ? 8192 : g), 256, 0, s>>>(src, dst, NP);
}
#endif

void launch_add(const Fields& F, const Work* work, int nwork, cudaStream_t s) {
  if (nwork > 0) k_add<<<nwork, 128, 0, s>>>(F, work);
}

#endif  // NPBMZ_NO_LAUNCHERS

}  // namespace NPBMZ_NS
}  // namespace npbmz
