// adjoint.cu -- discrete adjoint of the BT-MZ and SP-MZ time steps (FP64).
//
// One time step is u' = E u (exch_qbc), r = R(u', f) (compute_rhs),
// r1 = Tx(u')^-1 r, r2 = Ty(u')^-1 r1, r3 = Tz(u')^-1 r2, and
// u_next = u' + r3 on the interior (add).  Its transpose, given the adjoint
// ub of u_next:
//   r3b = ub on the interior, vb = ub;
//   for d = z, y, x:  y = Td^-T rdb  (block-tridiagonal solve with the
//       transposed blocks),  vb -= (d(Td(v) xd)/dv)^T y  (xd = the forward
//       solution of that sweep);  the next rdb is y;
//   vb += (dR/dv)^T rb,  fb += (dR/df)^T rb;   ub_prev = E^T vb.
// The pointwise derivatives (of the flux-Jacobian products and of the
// compute_rhs flux and viscous terms) are taken with forward-mode dual
// numbers over the five conserved variables of one point.
//
// SP (src/SP/adi.jl:6-258): r0 = R(u', f), r = Tx(u') r0 (txinvr), and per
// sweep d = x, y, z: y_d = L_d(u')^-1 x_{d-1} (three scalar pentadiagonal
// systems, identity rows at the line ends), x_d = P_d y_d (ninvr, pinvr:
// constant; tzetar: state-dependent) on the interior, u_next = u' + x_z.
// The band entries of row q that depend on the state are its sub- and
// super-diagonal and diagonal, each a function of the geometry (velocity,
// rhon, speed) of its own column's point only; so the linearisation of
// L(u') y at point j gathers lambda_{j-1}, lambda_j and lambda_{j+1}.
#define NPBMZ_NS adjk
#define NPBMZ_HAS_FP32 1
#define NPBMZ_NO_LAUNCHERS
#include "step_kernels.cuh"

#include "adjoint_launch.h"

namespace npbmz {
namespace adjk {

// ---- forward-mode dual number over 5 inputs --------------------------------
struct D5 {
  double v;
  double d[5];
};
__device__ __forceinline__ D5 dconst(double a) {
  D5 r;
  r.v = a;
#pragma unroll
  for (int k = 0; k < 5; ++k) r.d[k] = 0.0;
  return r;
}
__device__ __forceinline__ D5 operator+(const D5& a, const D5& b) {
  D5 r;
  r.v = a.v + b.v;
#pragma unroll
  for (int k = 0; k < 5; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
__device__ __forceinline__ D5 operator-(const D5& a, const D5& b) {
  D5 r;
  r.v = a.v - b.v;
#pragma unroll
  for (int k = 0; k < 5; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
__device__ __forceinline__ D5 operator-(const D5& a) {
  D5 r;
  r.v = -a.v;
#pragma unroll
  for (int k = 0; k < 5; ++k) r.d[k] = -a.d[k];
  return r;
}
__device__ __forceinline__ D5 operator*(const D5& a, const D5& b) {
  D5 r;
  r.v = a.v * b.v;
#pragma unroll
  for (int k = 0; k < 5; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
__device__ __forceinline__ D5 operator*(double a, const D5& b) {
  D5 r;
  r.v = a * b.v;
#pragma unroll
  for (int k = 0; k < 5; ++k) r.d[k] = a * b.d[k];
  return r;
}
__device__ __forceinline__ D5 operator*(const D5& b, double a) { return a * b; }
__device__ __forceinline__ D5 operator+(const D5& a, double b) {
  D5 r = a;
  r.v += b;
  return r;
}
__device__ __forceinline__ D5 dinv(const D5& a) {
  D5 r;
  r.v = 1.0 / a.v;
  const double g = -r.v * r.v;
#pragma unroll
  for (int k = 0; k < 5; ++k) r.d[k] = g * a.d[k];
  return r;
}

__device__ __forceinline__ D5 dsqrt(const D5& a) {
  D5 r;
  r.v = sqrt(a.v);
  const double g = 0.5 / r.v;
#pragma unroll
  for (int k = 0; k < 5; ++k) r.d[k] = g * a.d[k];
  return r;
}
__device__ __forceinline__ D5 dmax(const D5& a, const D5& b) { return a.v >= b.v ? a : b; }
__device__ __forceinline__ D5 dval(const D5& a) { return dconst(a.v); }

__device__ __forceinline__ void seed_state(const Fields& F, int64_t pt, D5 u[5]) {
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    u[m] = dconst(F.u[m * F.NP + pt]);
    u[m].d[m] = 1.0;
  }
}

// F = fjac(u) x and N = njac(u) x with dual u (the formulas of bt_jx, with
// ri = 1/u1 and qs = square / u1 derived from u as compute_rhs does).
template <int DIR>
__device__ __forceinline__ void jx_dual(const Consts& K, const D5 u[5], const double x[5], D5 Fx[5], D5 Nx[5]) {
  const D5 ri = dinv(u[0]);
  const D5 vel[3] = {u[1] * ri, u[2] * ri, u[3] * ri};
  const D5 E = u[4] * ri;
  const D5 q = 0.5 * ((u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) * ri) * ri;
  constexpr int a = DIR + 1;
  const D5 vn = vel[DIR];
  const double c1 = K.c1, c2 = K.c2;
  D5 d[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) d[m] = dconst(x[m + 1]) - vel[m] * x[0];
  D5 tang = dconst(0.0);
  Fx[0] = dconst(x[a]);
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    if (m == DIR) continue;
    Fx[m + 1] = vn * d[m] + vel[m] * x[a];
    tang = tang + vel[m] * x[m + 1];
  }
  Fx[a] = (c2 * q - vn * vn) * x[0] - c2 * tang + ((2.0 - c2) * vn) * x[a] + dconst(c2 * x[4]);
  Fx[4] = ((2.0 * c2) * q - c1 * E) * vn * x[0] - (c2 * vn) * tang + (c1 * E - c2 * (q + vn * vn)) * x[a] +
          (c1 * vn) * x[4];
  const double k43 = K.con43 * K.c3c4, c3c4 = K.c3c4, c1345 = K.c1345;
  D5 s4 = c1345 * (dconst(x[4]) - E * x[0]);
  Nx[0] = dconst(0.0);
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const double cm = (m == DIR) ? k43 : c3c4;
    Nx[m + 1] = (cm * ri) * d[m];
    s4 = s4 + ((cm - c1345) * vel[m]) * d[m];
  }
  Nx[4] = ri * s4;
}

// ---- transposed sweep --------------------------------------------------------
// Per line: the blocks of T at point p come from the Jacobians at p-1, p, p+1;
// the blocks of row p of T^T come from the Jacobian at p alone:
//   L_p = C_{p-1}^T (zero for p = 1, where C_0 is the boundary's zero block),
//   D_p = B_p^T (identity on the boundary rows 0 and n-1),
//   U_p = A_{p+1}^T (zero for p = n-2, where A_{n-1} is zero).
// Block LU (forward: G_p, g_p to the scratch), back substitution, then the
// linearisation vb_q -= J_F(q)^T w_q + J_N(q)^T z_q with
//   w_q = tmp2 (y_{q-1} - y_{q+1}),  z_q = -tmp1 (y_{q-1} - 2 y_q + y_{q+1})
// over the interior rows only.
template <int DIR>
__global__ void __launch_bounds__(128) k_adj_solve(Fields F, Consts K, const Work* __restrict__ work,
                                                  double* __restrict__ yb, const double* __restrict__ xs,
                                                  double* __restrict__ vb, double* __restrict__ scr, int64_t nlt) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int line = w.first + threadIdx.x;
  if (line >= zone_lines(Z, DIR)) return;
  int64_t base, st;
  line_geometry(Z, DIR, line, base, st);
  const int n = zone_line_len(Z, DIR);
  const int64_t gl = Z.lineoff[DIR] + line;
  const int64_t NP = F.NP;
  const double tmp1 = DIR == 0 ? K.dttx1 : DIR == 1 ? K.dtty1 : K.dttz1;
  const double tmp2 = DIR == 0 ? K.dttx2 : DIR == 1 ? K.dtty2 : K.dttz2;
  double dd[5];
  if (DIR == 0) { dd[0] = K.dx1; dd[1] = K.dx2; dd[2] = K.dx3; dd[3] = K.dx4; dd[4] = K.dx5; }
  else if (DIR == 1) { dd[0] = K.dy1; dd[1] = K.dy2; dd[2] = K.dy3; dd[3] = K.dy4; dd[4] = K.dy5; }
  else { dd[0] = K.dz1; dd[1] = K.dz2; dd[2] = K.dz3; dd[3] = K.dz4; dd[4] = K.dz5; }
  auto G = [&](int p, int e) -> double& { return scr[((int64_t)p * 30 + e) * nlt + gl]; };

  double Gp[5][5], gp[5];
  for (int p = 0; p < n; ++p) {
    const int64_t pt = base + (int64_t)p * st;
    double f[5][5], nj[5][5];
    bt_jac<DIR, double>(K, F.prim[PR_RHOI * NP + pt], F.u[NP + pt], F.u[2 * NP + pt], F.u[3 * NP + pt],
                        F.u[4 * NP + pt], F.prim[PR_QS * NP + pt], f, nj);
    double A[5][5], B[5][5], C[5][5];
#pragma unroll
    for (int a = 0; a < 5; ++a)
#pragma unroll
      for (int b = 0; b < 5; ++b) { A[a][b] = 0.0; B[a][b] = 0.0; C[a][b] = 0.0; }
    bt_asm_a<DIR, double>(f, nj, tmp1, tmp2, dd, A);   // A_{p+1}
    bt_asm_b<double>(nj, tmp1, dd, B);                  // B_p
    bt_asm_c<DIR, double>(f, nj, tmp1, tmp2, dd, C);   // C_{p-1}
    const bool bnd = (p == 0 || p == n - 1);
    double M[5][5], U[5][5], r[5];
#pragma unroll
    for (int a = 0; a < 5; ++a) {
      r[a] = yb[a * NP + pt];
#pragma unroll
      for (int b = 0; b < 5; ++b) {
        M[a][b] = bnd ? (a == b ? 1.0 : 0.0) : B[b][a];
        U[a][b] = (p <= n - 3) ? A[b][a] : 0.0;
      }
    }
    if (p >= 2) {  // L_p = C_{p-1}^T; M -= L G_{p-1}; r -= L g_{p-1}
#pragma unroll
      for (int a = 0; a < 5; ++a) {
#pragma unroll
        for (int b = 0; b < 5; ++b) {
          double t = M[a][b];
#pragma unroll
          for (int c = 0; c < 5; ++c) t -= C[c][a] * Gp[c][b];
          M[a][b] = t;
        }
        double t = r[a];
#pragma unroll
        for (int c = 0; c < 5; ++c) t -= C[c][a] * gp[c];
        r[a] = t;
      }
    }
    binvcrhs<double>(M, U, r);
#pragma unroll
    for (int a = 0; a < 5; ++a) {
      gp[a] = r[a];
      G(p, 25 + a) = r[a];
#pragma unroll
      for (int b = 0; b < 5; ++b) {
        Gp[a][b] = U[a][b];
        G(p, a * 5 + b) = U[a][b];
      }
    }
  }
  // back substitution y_p = g_p - G_p y_{p+1}; linearisation of point q = p+1
  double y_next[5], y_cur[5], y_nn[5];  // y_{p+1}, y_p, y_{p+2}
#pragma unroll
  for (int m = 0; m < 5; ++m) { y_next[m] = gp[m]; y_nn[m] = 0.0; }
#pragma unroll
  for (int m = 0; m < 5; ++m) yb[m * NP + base + (int64_t)(n - 1) * st] = y_next[m];
  auto lin = [&](int q, const double ym[5], const double yc[5], const double yp[5]) {
    // rows outside 1..n-2 do not depend on the state
    const double km = (q - 1 >= 1 && q - 1 <= n - 2) ? 1.0 : 0.0;
    const double kc = (q >= 1 && q <= n - 2) ? 1.0 : 0.0;
    const double kp = (q + 1 >= 1 && q + 1 <= n - 2) ? 1.0 : 0.0;
    double wv[5], zv[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      wv[m] = tmp2 * (km * ym[m] - kp * yp[m]);
      zv[m] = -tmp1 * (km * ym[m] - 2.0 * kc * yc[m] + kp * yp[m]);
    }
    const int64_t pt = base + (int64_t)q * st;
    D5 u[5], Fx[5], Nx[5];
    seed_state(F, pt, u);
    double x[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) x[m] = xs[m * NP + pt];
    jx_dual<DIR>(K, u, x, Fx, Nx);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      double g = 0.0;
#pragma unroll
      for (int a = 0; a < 5; ++a) g += wv[a] * Fx[a].d[c] + zv[a] * Nx[a].d[c];
      vb[c * NP + pt] -= g;
    }
  };
  for (int p = n - 2; p >= 0; --p) {
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      double t = G(p, 25 + m);
#pragma unroll
      for (int c = 0; c < 5; ++c) t -= G(p, m * 5 + c) * y_next[c];
      y_cur[m] = t;
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) yb[m * NP + base + (int64_t)p * st] = y_cur[m];
    lin(p + 1, y_cur, y_next, y_nn);
#pragma unroll
    for (int m = 0; m < 5; ++m) { y_nn[m] = y_next[m]; y_next[m] = y_cur[m]; }
  }
  {
    double zero[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    lin(0, zero, y_next, y_nn);
  }
}

// ---- compute_rhs adjoint --------------------------------------------------------
// Per direction the interior rhs is
//   r_p += psiV(p+1) - 2 psiV(p) + psiV(p-1) - (psiF(p+1) - psiF(p-1))
//          - dssp * sum_o w_o(p) u(p+o),
// with the viscous and convective point functions psiV, psiF of one point's
// state (see psi_dir), then r_p *= dt.  rb holds the adjoint of the rhs
// output; at interior points rho = dt * rb feeds the stencil adjoint.
template <int DIR>
__device__ __forceinline__ void psi_dir(const Consts& K, const D5 u[5], D5 V[5], D5 Fl[5]) {
  const D5 ri = dinv(u[0]);
  const D5 vel[3] = {u[1] * ri, u[2] * ri, u[3] * ri};
  const D5 sq = 0.5 * ((u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) * ri);
  const D5 qs = sq * ri;
  constexpr int a = DIR + 1;
  const D5 vn = vel[DIR];
  const double t2 = DIR == 0 ? K.tx2 : DIR == 1 ? K.ty2 : K.tz2;
  const double d1 = DIR == 0 ? K.dx1tx1 : DIR == 1 ? K.dy1ty1 : K.dz1tz1;
  const double d2 = DIR == 0 ? K.dx2tx1 : DIR == 1 ? K.dy2ty1 : K.dz2tz1;
  const double d3 = DIR == 0 ? K.dx3tx1 : DIR == 1 ? K.dy3ty1 : K.dz3tz1;
  const double d4 = DIR == 0 ? K.dx4tx1 : DIR == 1 ? K.dy4ty1 : K.dz4tz1;
  const double d5 = DIR == 0 ? K.dx5tx1 : DIR == 1 ? K.dy5ty1 : K.dz5tz1;
  const double con2 = DIR == 0 ? K.xxcon2 : DIR == 1 ? K.yycon2 : K.zzcon2;
  const double con3 = DIR == 0 ? K.xxcon3 : DIR == 1 ? K.yycon3 : K.zzcon3;
  const double con4 = DIR == 0 ? K.xxcon4 : DIR == 1 ? K.yycon4 : K.zzcon4;
  const double con5 = DIR == 0 ? K.xxcon5 : DIR == 1 ? K.yycon5 : K.zzcon5;
  const double dm[5] = {d1, d2, d3, d4, d5};
  V[0] = dm[0] * u[0];
#pragma unroll
  for (int m = 1; m <= 3; ++m) V[m] = dm[m] * u[m] + ((m == a ? con2 * K.con43 : con2) * vel[m - 1]);
  V[4] = dm[4] * u[4] + con3 * qs + con4 * (vn * vn) + con5 * (u[4] * ri);
  Fl[0] = t2 * u[a];
#pragma unroll
  for (int m = 1; m <= 3; ++m) {
    D5 g = u[m] * vn;
    if (m == a) g = g + K.c2 * (u[4] - sq);
    Fl[m] = t2 * g;
  }
  Fl[4] = t2 * ((K.c1 * u[4] - K.c2 * sq) * vn);
}

__device__ __forceinline__ void dweights(int q, int n, double w[5]) {
  w[0] = w[1] = w[2] = w[3] = w[4] = 0.0;
  if (q == 1) { w[2] += 5.0; w[3] -= 4.0; w[4] += 1.0; }
  if (q == 2) { w[1] -= 4.0; w[2] += 6.0; w[3] -= 4.0; w[4] += 1.0; }
  if (q >= 3 && q <= n - 4) { w[0] += 1.0; w[1] -= 4.0; w[2] += 6.0; w[3] -= 4.0; w[4] += 1.0; }
  if (q == n - 3) { w[0] += 1.0; w[1] -= 4.0; w[2] += 6.0; w[3] -= 4.0; }
  if (q == n - 2) { w[0] += 1.0; w[1] -= 4.0; w[2] += 5.0; }
}

__global__ void __launch_bounds__(128) k_adj_rhs(Fields F, Consts K, const Work* __restrict__ work,
                                                 const double* __restrict__ rb, double* __restrict__ vb,
                                                 double* __restrict__ fb) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int qi = w.first + threadIdx.x;
  if (qi >= Z.nx * Z.ny * Z.nz) return;
  const int i = qi % Z.nx, j = (qi / Z.nx) % Z.ny, k = qi / (Z.nx * Z.ny);
  const int64_t NP = F.NP;
  const int64_t pt = Z.off + qi;
  const int pos[3] = {i, j, k};
  const int len[3] = {Z.nx, Z.ny, Z.nz};
  const int64_t strd[3] = {1, Z.nx, (int64_t)Z.nx * Z.ny};
  auto interior = [&](int ii, int jj, int kk) {
    return ii >= 1 && ii <= Z.nx - 2 && jj >= 1 && jj <= Z.ny - 2 && kk >= 1 && kk <= Z.nz - 2;
  };
  // forcing: rhs = dt (forcing + ...) inside, rhs = forcing on the rest
  const bool inside = interior(i, j, k);
#pragma unroll
  for (int m = 0; m < 5; ++m) fb[m * NP + pt] += inside ? K.dt * rb[m * NP + pt] : rb[m * NP + pt];
  // rho at a neighbour along d at offset o (zero outside the interior)
  auto rho = [&](int d, int o, int m) -> double {
    int c[3] = {i, j, k};
    c[d] += o;
    if (!interior(c[0], c[1], c[2])) return 0.0;
    return K.dt * rb[m * NP + pt + o * strd[d]];
  };
  D5 u[5];
  seed_state(F, pt, u);
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    D5 V[5], Fl[5];
    if (d == 0) psi_dir<0>(K, u, V, Fl);
    else if (d == 1) psi_dir<1>(K, u, V, Fl);
    else psi_dir<2>(K, u, V, Fl);
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const double rm = rho(d, -1, m), r0 = rho(d, 0, m), rp = rho(d, 1, m);
      const double sv = rm - 2.0 * r0 + rp;
      const double sf = rp - rm;
#pragma unroll
      for (int c = 0; c < 5; ++c) acc[c] += sv * V[m].d[c] + sf * Fl[m].d[c];
      // dissipation: rows p = q - o use weight w_o(p) on u(q)
      double ds = 0.0;
#pragma unroll
      for (int o = -2; o <= 2; ++o) {
        const int pp = pos[d] - o;
        if (pp < 1 || pp > len[d] - 2) continue;
        double wv[5];
        dweights(pp, len[d], wv);
        ds += wv[o + 2] * rho(d, -o, m);
      }
      acc[m] -= K.dssp * ds;
    }
  }
#pragma unroll
  for (int m = 0; m < 5; ++m) vb[m * NP + pt] += acc[m];
}

// ---- exch_qbc adjoint: ub = vb, then each ghost's adjoint moves to its source.
// faces [f0, f1): 0 west, 1 east, 2 south, 3 north (no source is shared
// within {0,1} or within {2,3}).
__global__ void __launch_bounds__(256) k_adj_exch(Fields F, const int* __restrict__ nbr, const double* __restrict__ vb,
                                                  double* __restrict__ ub, int f0) {
  const int z = blockIdx.y / 2, face = f0 + blockIdx.y % 2;
  const ZoneDev Z = F.zones[z];
  const ZoneDev S = F.zones[nbr[4 * z + face]];
  const int nt = face < 2 ? Z.ny - 2 : Z.nx - 2;
  const int count = 5 * nt * (Z.nz - 2);
  const int64_t NP = F.NP;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < count; t += gridDim.x * blockDim.x) {
    const int a = t % nt, k = 1 + (t / nt) % (Z.nz - 2), m = t / (nt * (Z.nz - 2));
    int64_t dst, src;
    if (face == 0) {
      dst = Z.off + ((int64_t)k * Z.ny + (1 + a)) * Z.nx + 0;
      src = S.off + ((int64_t)k * S.ny + (1 + a)) * S.nx + (S.nx - 2);
    } else if (face == 1) {
      dst = Z.off + ((int64_t)k * Z.ny + (1 + a)) * Z.nx + (Z.nx - 1);
      src = S.off + ((int64_t)k * S.ny + (1 + a)) * S.nx + 1;
    } else if (face == 2) {
      dst = Z.off + ((int64_t)k * Z.ny + 0) * Z.nx + (1 + a);
      src = S.off + ((int64_t)k * S.ny + (S.ny - 2)) * S.nx + (1 + a);
    } else {
      dst = Z.off + ((int64_t)k * Z.ny + (Z.ny - 1)) * Z.nx + (1 + a);
      src = S.off + ((int64_t)k * S.ny + 1) * S.nx + (1 + a);
    }
    ub[m * NP + src] += vb[m * NP + dst];
    ub[m * NP + dst] = 0.0;
  }
}

// out = a - b (or a when b is null) at every stored point of the CTA's zone
// share, zeroed outside the interior when interior_only (the adjoint of add);
// partial: this CTA's sums of out^2 (the objective).
__global__ void __launch_bounds__(128) k_adj_seed(Fields F, const Work* __restrict__ work, const double* __restrict__ a,
                                                  const double* __restrict__ b, double* __restrict__ out,
                                                  double* __restrict__ partial, int interior_only) {
  __shared__ double red[5 * 128];
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int qi = w.first + threadIdx.x;
  double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (qi < Z.nx * Z.ny * Z.nz) {
    const int i = qi % Z.nx, j = (qi / Z.nx) % Z.ny, k = qi / (Z.nx * Z.ny);
    const bool in = !interior_only || (i >= 1 && i <= Z.nx - 2 && j >= 1 && j <= Z.ny - 2 && k >= 1 && k <= Z.nz - 2);
    const int64_t pt = Z.off + qi;
    for (int m = 0; m < 5; ++m) {
      const double d = in ? (b ? a[m * F.NP + pt] - b[m * F.NP + pt] : a[m * F.NP + pt]) : 0.0;
      out[m * F.NP + pt] = d;
      v[m] = d * d;
    }
  }
  if (partial) {
    block_sum5(v, red);
    if (threadIdx.x == 0)
      for (int m = 0; m < 5; ++m) partial[blockIdx.x * 5 + m] = v[m];
  }
}

// ---- SP ------------------------------------------------------------------------
// Primitive variables of one point's state, as the primitive kernel forms
// them (src/SP/rhs.jl:62-89).
struct SpPrim {
  D5 ri, vel[3], sq, qs, speed, ainv;
};
__device__ __forceinline__ SpPrim sp_prim(const Consts& K, const D5 u[5]) {
  SpPrim P;
  P.ri = dinv(u[0]);
#pragma unroll
  for (int d = 0; d < 3; ++d) P.vel[d] = u[d + 1] * P.ri;
  P.sq = 0.5 * ((u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) * P.ri);
  P.qs = P.sq * P.ri;
  P.speed = dsqrt(K.c1c2 * (P.ri * (u[4] - P.sq)));
  P.ainv = dinv(P.speed);
  return P;
}
__device__ __forceinline__ SpPrim sp_prim_value(const SpPrim& a) {  // derivatives dropped
  SpPrim P;
  P.ri = dval(a.ri);
#pragma unroll
  for (int d = 0; d < 3; ++d) P.vel[d] = dval(a.vel[d]);
  P.sq = dval(a.sq);
  P.qs = dval(a.qs);
  P.speed = dval(a.speed);
  P.ainv = dval(a.ainv);
  return P;
}

// txinvr (src/SP/txinvr.jl:28-49), 1/speed^2 as ainv^2 like the forward kernel
__device__ __forceinline__ void sp_txinvr(const Consts& K, const SpPrim& P, const D5 r[5], D5 o[5]) {
  const D5 ac2inv = P.ainv * P.ainv;
  const D5 t1 = K.c2 * (ac2inv * (P.qs * r[0] - P.vel[0] * r[1] - P.vel[1] * r[2] - P.vel[2] * r[3] + r[4]));
  const D5 t2 = K.bt * (P.ri * (P.vel[0] * r[0] - r[1]));
  const D5 t3 = (K.bt * (P.ri * P.speed)) * t1;
  o[0] = r[0] - t1;
  o[1] = -(P.ri * (P.vel[2] * r[0] - r[3]));
  o[2] = P.ri * (P.vel[1] * r[0] - r[2]);
  o[3] = t3 - t2;
  o[4] = t2 + t3;
}

// The transform after sweep DIR: ninvr (src/SP/ninvr.jl:19-32), pinvr
// (src/SP/pinvr.jl:20-33), tzetar (src/SP/tzetar.jl:27-52; uzik1 = u1).
template <int DIR>
__device__ __forceinline__ void sp_post(const Consts& K, const SpPrim& P, const D5& uzik1, const D5 r[5], D5 o[5]) {
  if (DIR == 0) {
    const D5 t1 = K.bt * r[2];
    const D5 t2 = 0.5 * (r[3] + r[4]);
    o[0] = -r[1]; o[1] = r[0]; o[2] = K.bt * (r[3] - r[4]); o[3] = t2 - t1; o[4] = t1 + t2;
  } else if (DIR == 1) {
    const D5 t1 = K.bt * r[0];
    const D5 t2 = 0.5 * (r[3] + r[4]);
    o[0] = K.bt * (r[3] - r[4]); o[1] = -r[2]; o[2] = r[1]; o[3] = t2 - t1; o[4] = t1 + t2;
  } else {
    const D5 btuz = K.bt * uzik1;
    const D5 t1 = (btuz * P.ainv) * (r[3] + r[4]);
    const D5 t2 = r[2] + t1;
    const D5 t3 = btuz * (r[3] - r[4]);
    o[0] = t2;
    o[1] = P.vel[0] * t2 - uzik1 * r[1];
    o[2] = uzik1 * r[0] + P.vel[1] * t2;
    o[3] = P.vel[2] * t2 + t3;
    o[4] = uzik1 * (P.vel[1] * r[0] - P.vel[0] * r[1]) + P.qs * t2 + (K.c2iv * (P.speed * P.speed)) * t1 +
           P.vel[2] * t3;
  }
}

// ybar = T^T xbar for a map o = T r linear in r (T at fixed primitives).
template <typename Map>
__device__ __forceinline__ void transpose_apply(Map map, const double xb[5], double yb[5]) {
  D5 rs[5], o[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    rs[m] = dconst(0.0);
    rs[m].d[m] = 1.0;
  }
  map(rs, o);
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    double t = 0.0;
#pragma unroll
    for (int m = 0; m < 5; ++m) t += o[m].d[j] * xb[m];
    yb[j] = t;
  }
}

// Forward recomputation: the transform of sweep DIR applied to the
// untransformed solution ys, into rhs, at the interior points.
template <int DIR>
__global__ void __launch_bounds__(128) k_sp_apply_post(Fields F, Consts K, const Work* __restrict__ work,
                                                       const double* __restrict__ ys) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int qi = w.first + threadIdx.x;
  if (qi >= Z.nx * Z.ny * Z.nz) return;
  const int i = qi % Z.nx, j = (qi / Z.nx) % Z.ny, k = qi / (Z.nx * Z.ny);
  if (i < 1 || i > Z.nx - 2 || j < 1 || j > Z.ny - 2 || k < 1 || k > Z.nz - 2) return;
  const int64_t NP = F.NP, pt = Z.off + qi;
  double v[5], o[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) v[m] = ys[m * NP + pt];
  sp_transform<DIR>(F, K, pt, v, o);
#pragma unroll
  for (int m = 0; m < 5; ++m) F.rhs[m * NP + pt] = o[m];
}

// txinvr adjoint at the interior points: vb += (d(Tx(u') r0)/du')^T rb, then
// rb <- Tx^T rb (rb in: adjoint of txinvr's output, out: of compute_rhs's).
__global__ void __launch_bounds__(128) k_adj_sp_txinvr(Fields F, Consts K, const Work* __restrict__ work,
                                                       double* __restrict__ rb, const double* __restrict__ r0,
                                                       double* __restrict__ vb) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int qi = w.first + threadIdx.x;
  if (qi >= Z.nx * Z.ny * Z.nz) return;
  const int i = qi % Z.nx, j = (qi / Z.nx) % Z.ny, k = qi / (Z.nx * Z.ny);
  if (i < 1 || i > Z.nx - 2 || j < 1 || j > Z.ny - 2 || k < 1 || k > Z.nz - 2) return;
  const int64_t NP = F.NP, pt = Z.off + qi;
  D5 u[5];
  seed_state(F, pt, u);
  const SpPrim P = sp_prim(K, u);
  double xb[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) xb[m] = rb[m * NP + pt];
  {
    D5 rc[5], o[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) rc[m] = dconst(r0[m * NP + pt]);
    sp_txinvr(K, P, rc, o);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      double g = 0.0;
#pragma unroll
      for (int m = 0; m < 5; ++m) g += xb[m] * o[m].d[c];
      vb[c * NP + pt] += g;
    }
  }
  const SpPrim Pv = sp_prim_value(P);
  double yt[5];
  transpose_apply([&](const D5 rs[5], D5 o[5]) { sp_txinvr(K, Pv, rs, o); }, xb, yt);
#pragma unroll
  for (int m = 0; m < 5; ++m) rb[m * NP + pt] = yt[m];
}

// Transposed SP sweep DIR, one thread per line.  yb in: adjoint of the
// sweep's output (transformed on the interior), out: of its input; ys: the
// forward untransformed solution (with the line's end values); vb gets the
// linearisations of the transform (tzetar) and of the bands.  Line scratch
// per point (30 doubles): bands of the three systems (0..14), the
// eliminated upper bands (15..20), the right-hand side / lambda (21..25),
// the geometry cv, rhon, speed (26..28).
template <int DIR>
__global__ void __launch_bounds__(128) k_adj_sp_solve(Fields F, Consts K, const Work* __restrict__ work,
                                                     double* __restrict__ yb, const double* __restrict__ ys,
                                                     double* __restrict__ vb, double* __restrict__ scr, int64_t nlt) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int line = w.first + threadIdx.x;
  if (line >= zone_lines(Z, DIR)) return;
  int64_t base, st;
  line_geometry(Z, DIR, line, base, st);
  const int n = zone_line_len(Z, DIR);
  const int64_t gl = Z.lineoff[DIR] + line;
  const int64_t NP = F.NP;
  const double dtt1 = DIR == 0 ? K.dttx1 : DIR == 1 ? K.dtty1 : K.dttz1;
  const double dtt2 = DIR == 0 ? K.dttx2 : DIR == 1 ? K.dtty2 : K.dttz2;
  const double c2dtt1 = DIR == 0 ? K.c2dttx1 : DIR == 1 ? K.c2dtty1 : K.c2dttz1;
  auto S = [&](int p, int e) -> double& { return scr[((int64_t)p * 30 + e) * nlt + gl]; };
  // geometry and bands (the forward solve's sp_geom / sp_assemble)
  for (int p = 0; p < n; ++p) sp_geom<DIR>(F, K, base + (int64_t)p * st, S(p, 26), S(p, 27), S(p, 28));
  for (int q = 0; q < n; ++q) {
    double cv[3], rh[3], sp[3], L[3][5];
#pragma unroll
    for (int o = 0; o < 3; ++o) {
      const int r = min(max(q + o - 1, 0), n - 1);
      cv[o] = S(r, 26); rh[o] = S(r, 27); sp[o] = S(r, 28);
    }
    sp_assemble<DIR, double, double>(K, q, n, cv, rh, sp, L);
#pragma unroll
    for (int s = 0; s < 3; ++s)
#pragma unroll
      for (int b = 0; b < 5; ++b) S(q, 5 * s + b) = L[s][b];
  }
  // right-hand side: the transform's transpose on the interior (tzetar also
  // linearised in the state)
  for (int p = 0; p < n; ++p) {
    const int64_t pt = base + (int64_t)p * st;
    double xb[5], yt[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) xb[m] = yb[m * NP + pt];
    if (p >= 1 && p <= n - 2) {
      D5 u[5];
      seed_state(F, pt, u);
      const SpPrim P = sp_prim(K, u);
      if (DIR == 2) {
        D5 yc[5], o[5];
#pragma unroll
        for (int m = 0; m < 5; ++m) yc[m] = dconst(ys[m * NP + pt]);
        sp_post<2>(K, P, u[0], yc, o);
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          double g = 0.0;
#pragma unroll
          for (int m = 0; m < 5; ++m) g += xb[m] * o[m].d[c];
          vb[c * NP + pt] += g;
        }
      }
      const SpPrim Pv = sp_prim_value(P);
      const D5 uz = dval(u[0]);
      transpose_apply([&](const D5 rs[5], D5 o[5]) { sp_post<DIR>(K, Pv, uz, rs, o); }, xb, yt);
    } else {
#pragma unroll
      for (int m = 0; m < 5; ++m) yt[m] = xb[m];
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) S(p, 21 + m) = yt[m];
  }
  // L^T lambda = ybar per system: row q of L^T holds column q of L,
  // L^T[q][q + c - 2] = band (4 - c) of row q + c - 2
  auto LT = [&](int q, int s, int c) -> double {
    const int r = q + c - 2;
    return (r < 0 || r > n - 1) ? 0.0 : S(r, 5 * s + 4 - c);
  };
  for (int q = 0; q < n; ++q) {
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      double a2 = LT(q, s, 0), a1 = LT(q, s, 1), d = LT(q, s, 2), e1 = LT(q, s, 3);
      const double e2 = LT(q, s, 4);
      double b[3];
      const int m0 = SP_M0(s), m1 = SP_M1(s);
      for (int m = m0; m <= m1; ++m) b[m - m0] = S(q, 21 + m);
      if (q >= 2) {
        a1 -= a2 * S(q - 2, 15 + 2 * s);
        d -= a2 * S(q - 2, 16 + 2 * s);
        for (int m = m0; m <= m1; ++m) b[m - m0] -= a2 * S(q - 2, 21 + m);
      }
      if (q >= 1) {
        d -= a1 * S(q - 1, 15 + 2 * s);
        e1 -= a1 * S(q - 1, 16 + 2 * s);
        for (int m = m0; m <= m1; ++m) b[m - m0] -= a1 * S(q - 1, 21 + m);
      }
      const double inv = 1.0 / d;
      S(q, 15 + 2 * s) = e1 * inv;
      S(q, 16 + 2 * s) = e2 * inv;
      for (int m = m0; m <= m1; ++m) S(q, 21 + m) = b[m - m0] * inv;
    }
  }
  for (int q = n - 2; q >= 0; --q) {
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const int s = m < 3 ? 0 : m - 2;
      double t = S(q, 21 + m) - S(q, 15 + 2 * s) * S(q + 1, 21 + m);
      if (q + 2 <= n - 1) t -= S(q, 16 + 2 * s) * S(q + 2, 21 + m);
      S(q, 21 + m) = t;
    }
  }
  // linearisation of the bands at each point j, and the output
  const double da = DIR == 0 ? K.dx2 : DIR == 1 ? K.dy3 : K.dz4;
  const double db = DIR == 0 ? K.dx5 : DIR == 1 ? K.dy5 : K.dz5;
  const double dm = DIR == 0 ? K.dxmax : DIR == 1 ? K.dymax : K.dzmax;
  const double dc = DIR == 0 ? K.dx1 : DIR == 1 ? K.dy1 : K.dz1;
  for (int j = 0; j < n; ++j) {
    const int64_t pt = base + (int64_t)j * st;
    double y[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) y[m] = ys[m * NP + pt];
    // dot(q, s) = lambda_q . y_j over the components of system s
    auto dot = [&](int q, int s) -> double {
      if (q < 1 || q > n - 2) return 0.0;  // identity rows do not depend on the state
      double t = 0.0;
      for (int m = SP_M0(s); m <= SP_M1(s); ++m) t += S(q, 21 + m) * y[m];
      return t;
    };
    double gcv = 0.0, grh = 0.0, gsp = 0.0;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      const double up = dot(j - 1, s), mid = dot(j, s), dn = dot(j + 1, s);
      gcv += dtt2 * (up - dn);
      grh += -dtt1 * dn + c2dtt1 * mid - dtt1 * up;
      if (s == 1) gsp += dtt2 * (up - dn);
      if (s == 2) gsp += dtt2 * (dn - up);
    }
    if (gcv != 0.0 || grh != 0.0 || gsp != 0.0) {
      D5 u[5];
      seed_state(F, pt, u);
      const SpPrim P = sp_prim(K, u);
      const D5 ru1 = K.c3c4 * P.ri;
      const D5 rhon = dmax(dmax(dmax(ru1 * K.con43 + da, ru1 * K.c1c5 + db), ru1 + dm), dconst(dc));
      const D5& cv = P.vel[DIR];
#pragma unroll
      for (int c = 0; c < 5; ++c) vb[c * NP + pt] -= gcv * cv.d[c] + grh * rhon.d[c] + gsp * P.speed.d[c];
    }
  }
#pragma unroll 1
  for (int p = 0; p < n; ++p)
#pragma unroll
    for (int m = 0; m < 5; ++m) yb[m * NP + base + (int64_t)p * st] = S(p, 21 + m);
}

}  // namespace adjk

// ================================ launchers ================================
void adj_launch_solve(int dir, const Fields& F, const Consts& K, const Work* work, int nwork, int tpb, double* yb,
                      const double* xs, double* vb, double* scr, int64_t nlt, cudaStream_t s) {
  if (nwork <= 0) return;
  // one CTA of tpb (<= 128) threads per work item of tpb lines
  if (dir == 0) adjk::k_adj_solve<0><<<nwork, tpb, 0, s>>>(F, K, work, yb, xs, vb, scr, nlt);
  else if (dir == 1) adjk::k_adj_solve<1><<<nwork, tpb, 0, s>>>(F, K, work, yb, xs, vb, scr, nlt);
  else adjk::k_adj_solve<2><<<nwork, tpb, 0, s>>>(F, K, work, yb, xs, vb, scr, nlt);
}

void adj_launch_rhs(const Fields& F, const Consts& K, const Work* work, int nwork, const double* rb, double* vb,
                    double* fb, cudaStream_t s) {
  if (nwork > 0) adjk::k_adj_rhs<<<nwork, 128, 0, s>>>(F, K, work, rb, vb, fb);
}

void adj_launch_exch(const Fields& F, const int* nbr, int nzones, int max_face, const double* vb, double* ub,
                     cudaStream_t s) {
  int gx = (max_face + 255) / 256;
  if (gx < 1) gx = 1;
  if (gx > 64) gx = 64;
  dim3 grid(gx, 2 * nzones);
  adjk::k_adj_exch<<<grid, 256, 0, s>>>(F, nbr, vb, ub, 0);
  adjk::k_adj_exch<<<grid, 256, 0, s>>>(F, nbr, vb, ub, 2);
}

void adj_launch_seed(const Fields& F, const Work* work, int nwork, const double* a, const double* b, double* out,
                     double* partial, int interior_only, cudaStream_t s) {
  if (nwork > 0) adjk::k_adj_seed<<<nwork, 128, 0, s>>>(F, work, a, b, out, partial, interior_only);
}

void sp_fwd_launch_solve(int dir, const Fields& F, const Consts& K, const Work* work, int nwork, int tpb, double* ys,
                         double* scr, int64_t nlt, cudaStream_t s) {
  if (nwork <= 0) return;
  if (dir == 0) adjk::k_sp_solve<0, double><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, 0, ys, 0);
  else if (dir == 1) adjk::k_sp_solve<1, double><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, 0, ys, 0);
  else adjk::k_sp_solve<2, double><<<nwork, tpb, 0, s>>>(F, K, work, scr, nlt, 0, ys, 0);
}

void sp_fwd_launch_post(int dir, const Fields& F, const Consts& K, const Work* work, int nwork, const double* ys,
                        cudaStream_t s) {
  if (nwork <= 0) return;
  if (dir == 0) adjk::k_sp_apply_post<0><<<nwork, 128, 0, s>>>(F, K, work, ys);
  else if (dir == 1) adjk::k_sp_apply_post<1><<<nwork, 128, 0, s>>>(F, K, work, ys);
  else adjk::k_sp_apply_post<2><<<nwork, 128, 0, s>>>(F, K, work, ys);
}

void adj_launch_sp_solve(int dir, const Fields& F, const Consts& K, const Work* work, int nwork, int tpb, double* yb,
                         const double* ys, double* vb, double* scr, int64_t nlt, cudaStream_t s) {
  if (nwork <= 0) return;
  if (dir == 0) adjk::k_adj_sp_solve<0><<<nwork, tpb, 0, s>>>(F, K, work, yb, ys, vb, scr, nlt);
  else if (dir == 1) adjk::k_adj_sp_solve<1><<<nwork, tpb, 0, s>>>(F, K, work, yb, ys, vb, scr, nlt);
  else adjk::k_adj_sp_solve<2><<<nwork, tpb, 0, s>>>(F, K, work, yb, ys, vb, scr, nlt);
}

void adj_launch_sp_txinvr(const Fields& F, const Consts& K, const Work* work, int nwork, double* rb, const double* r0,
                          double* vb, cudaStream_t s) {
  if (nwork > 0) adjk::k_adj_sp_txinvr<<<nwork, 128, 0, s>>>(F, K, work, rb, r0, vb);
}

}  // namespace npbmz
