// lu_types.h -- types and constants shared by the LU-MZ kernels
// (lu_kernels.cuh, compiled twice: lu_exact.cu without FMA contraction,
// lu_fast.cu with it) and the host side of the LU C ABI (lu.cu).
#pragma once
#include <cuda_runtime.h>

namespace npbmz_lu {

constexpr double c1 = 1.40e+00, c2 = 0.40e+00, c3 = 1.00e-01, c4 = 1.00e+00, c5 = 1.40e+00;
constexpr double dx1 = 0.75e+00, dx2 = dx1, dx3 = dx1, dx4 = dx1, dx5 = dx1;
constexpr double dy1 = 0.75e+00, dy2 = dy1, dy3 = dy1, dy4 = dy1, dy5 = dy1;
constexpr double dz1 = 1.00e+00, dz2 = dz1, dz3 = dz1, dz4 = dz1, dz5 = dz1;
constexpr double dssp = 1.00e+00 / 4.0e+00;  // max(dx1, dy1, dz1) / 4 (src/LU/setcoeff.jl)
constexpr int ii1 = 2, ji1 = 2, ki1 = 3;
constexpr int TPB = 128;

struct CeTable {
  double c[5][13];
};

// setcoeff of one zone (src/LU/setcoeff.jl) and its place in HBM
struct LuZone {
  long long off;
  int nx, ny, nz, np;
  double dxi, deta, dzeta, tx1, tx2, tx3, ty1, ty2, ty3, tz1, tz2, tz3;
  int ii2, ji2, ki2;
};

struct LuDev {
  double* u;
  double* rsd;
  double* frct;
  double* prim;  // PR_COUNT planes of per-point flux quantities of u
  long long NP;
  const LuZone* zones;
  double dt, omega;
  // state check of the update (null: off): word 0 ORs LU_STATE_* bits of every
  // point found bad, word 1 keeps the smallest such point index
  unsigned long long* health = nullptr;
};

// The state check's bits: the density is not positive and finite; the
// pressure-like quantity u5 - (u2^2 + u3^2 + u4^2) / (2 u1) is finite but not
// positive; it is not finite (a NaN or an infinity in u).
constexpr unsigned LU_STATE_DENSITY = 1u, LU_STATE_PRESSURE = 2u, LU_STATE_NONFINITE = 4u;

struct LuWork {  // one block of TPB consecutive points of one zone
  int zone, first;
};

__host__ __device__ inline long long pidx(const LuZone& Z, int i, int j, int k) {
  return Z.off + ((long long)(k - 1) * Z.ny + (j - 1)) * Z.nx + (i - 1);
}

// Per-point quantities of the flux functions (planes of `prim`), each the
// reference's own expression evaluated once per point instead of once per
// use (rhs.jl and erhs.jl evaluate them at every neighbour):
//   PR_RHO  1/g1                          (the viscous tmp, jacld's tmp1)
//   PR_U21..PR_U51  tmp*g2 .. tmp*g5      (the viscous u21i .. u51i)
//   PR_S    u21^2 + u31^2 + u41^2         (their sum of squares)
//   PR_C21, PR_C31, PR_C41  g2/g1, g3/g1, g4/g1  (the convective u21, u31, u41)
//   PR_Q    0.5 (g2^2 + g3^2 + g4^2) / g1 (the convective q)
enum { PR_RHO = 0, PR_U21, PR_U31, PR_U41, PR_U51, PR_S, PR_C21, PR_C31, PR_C41, PR_Q, PR_COUNT };

struct JC {
  double dt, tx1, tx2, ty1, ty2, tz1, tz2;
};
constexpr double r43 = (4.0e+00 / 3.0e+00);
constexpr double c1345 = c1 * c3 * c4 * c5;
constexpr double c34 = c3 * c4;

// The entries the reference assigns a literal 0.0 in each off-diagonal block
// (the same pattern in jacld and jacu).  A product with one is +-0 and
// adding it changes no sum's value, so the row sums below skip them.
__host__ __device__ constexpr bool off_zero(int dir, int r, int c) {
  return dir == 2 ? ((r == 0 && (c == 1 || c == 2 || c == 4)) || (r == 1 && (c == 2 || c == 4)) ||
                     (r == 2 && (c == 1 || c == 4)))
       : dir == 1 ? ((r == 0 && (c == 1 || c == 3 || c == 4)) || (r == 1 && (c == 3 || c == 4)) ||
                     (r == 3 && (c == 1 || c == 4)))
                  : ((r == 0 && (c == 2 || c == 3 || c == 4)) || (r == 2 && (c == 3 || c == 4)) ||
                     (r == 3 && (c == 2 || c == 4)));
}

// Position of entry (r, c) among the 18 entries of block DIR that are not
// structural zeros, row-major.
__host__ __device__ constexpr int blk_idx(int dir, int r, int c) {
  int n = 0;
  for (int rr = 0; rr < 5; ++rr)
    for (int cc = 0; cc < 5; ++cc) {
      if (rr == r && cc == c) return n;
      if (!off_zero(dir, rr, cc)) ++n;
    }
  return n;
}
constexpr int BLK_NZ = 18;

// The 5x5 solve of blts / buts (src/LU/blts.jl:106-193, src/LU/buts.jl:113-200)
// with tmat = d.  d is lower triangular with d[2][1] = d[3][1] = d[3][2] = 0
// (jacld.jl / jacu.jl assign those 0.0), so the elimination leaves every
// entry of tmat as it was, and every update the reference makes with a zero
// multiplier (including buts's `tmat[5,5] -=- tmp * tmat[2,5]` and its back
// substitution signs, whose terms are all products with zeros) leaves the
// value it updates unchanged.  What remains, statement for statement:
//   tmp_r0 = (1/t00) t_r0,  v_r <- v_r - v_0 tmp_r0         (r = 1..4)
//   tmp_4c = (1/t_cc) t_4c, v_4 <- v_4 - v_c tmp_4c         (c = 1, 2, 3)
//   v_r <- v_r / t_rr                                       (r = 4..0)
// `jac` planes per interior point, stored at the point's hyperplane-ordered
// index h = zone.off + hps[l] + t (t: its place in hyperplane l = i+j+k,
// k then j ascending; hps[l]: the zone's interior points with i+j+k < l), so
// that the sweeps, which run one hyperplane per launch, read them coalesced.
// Written by k_lu_jac before the sweeps (u does not change until the
// update), each block by the point whose state it is built from:
//   FAC_T + r, FAC_R0 + r-1, FAC_4C + c-1   t_rr, tmp_r0, tmp_4c of d
//   FAC_BLK + (2 dir + s) * 18 + blk_idx    the non-zero entries of the
//       off-diagonal block of direction dir: s = 0 jacld's (from the point
//       at -1 in dir), s = 1 jacu's (from the point at +1)
enum { FAC_T = 0, FAC_R0 = 5, FAC_4C = 9, FAC_BLK = 12, FAC_COUNT = 12 + 6 * 18 };

constexpr int HP = 32;  // points per block of the sweep kernels (x 5 rows)

// ---- exch_qbc (src/LU/exchange_qbc.jl) --------------------------------------
// Staging per zone: east face (j = ny-1) and west face (j = 2), nx*nkp points
// each; south face (i = nx-1) and north face (i = 2), ny*nkp points each;
// planes k = klo..klo+nkp-1; element [m][k][pos].
struct Faces {
  double* stage;
  const long long* zoff;  // staging offset of each zone
  const int* nbr;         // west, east, south, north per zone
  int klo, nkp;
};

}  // namespace npbmz_lu
