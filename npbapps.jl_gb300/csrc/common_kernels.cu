// common_kernels.cu -- set-up, zone-face exchange, norm and layout kernels.
// Compiled with -fmad=false: initialize / exact_rhs are bit-for-bit the
// reference's arithmetic.
#include "common_launch.h"
#include "npbmz_internal.cuh"

namespace npbmz {

// exact_solution (src/BT/exact_solution.jl:5-18); ce row-major [5][13].
struct Coeffs {
  double c[65];
};

__device__ __forceinline__ void exact_solution(double xi, double eta, double zeta, const Coeffs& ce, double out[5]) {
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    const double* c = ce.c + 13 * m;
    out[m] = c[0] + xi * (c[1] + xi * (c[4] + xi * (c[7] + xi * c[10]))) +
             eta * (c[2] + eta * (c[5] + eta * (c[8] + eta * c[11]))) +
             zeta * (c[3] + zeta * (c[6] + zeta * (c[9] + zeta * c[12])));
  }
}

// ---------------------------------------------------------------------------
// initialize (src/BT/initialize.jl:37-212): transfinite interpolation, then
// the six boundary faces written in the reference's order west, east, south,
// north, bottom, top -- a point on several faces keeps the last one.  Also
// writes the exact solution (error norm reference) at every point.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_initialize(Fields F, Consts K, Coeffs ce, const Work* __restrict__ work,
                                                    double* __restrict__ uex) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int q = w.first + threadIdx.x;
  if (q >= Z.nx * Z.ny * Z.nz) return;
  const int i = q % Z.nx, j = (q / Z.nx) % Z.ny, k = q / (Z.nx * Z.ny);
  const int64_t p = Z.off + q, NP = F.NP;
  const double xi = (double)i * K.dnxm1, eta = (double)j * K.dnym1, zeta = (double)k * K.dnzm1;
  double out[5];
  int face = -1;
  if (i == 0) face = 0;
  if (i == Z.nx - 1) face = 1;
  if (j == 0) face = 2;
  if (j == Z.ny - 1) face = 3;
  if (k == 0) face = 4;
  if (k == Z.nz - 1) face = 5;
  if (face < 0) {
    double P1[2][5], P2[2][5], P3[2][5];
    exact_solution(0.0, eta, zeta, ce, P1[0]);
    exact_solution(1.0, eta, zeta, ce, P1[1]);
    exact_solution(xi, 0.0, zeta, ce, P2[0]);
    exact_solution(xi, 1.0, zeta, ce, P2[1]);
    exact_solution(xi, eta, 0.0, ce, P3[0]);
    exact_solution(xi, eta, 1.0, ce, P3[1]);
    for (int m = 0; m < 5; ++m) {
      const double Pxi = xi * P1[1][m] + (1.0e0 - xi) * P1[0][m];
      const double Peta = eta * P2[1][m] + (1.0e0 - eta) * P2[0][m];
      const double Pzeta = zeta * P3[1][m] + (1.0e0 - zeta) * P3[0][m];
      out[m] = Pxi + Peta + Pzeta - Pxi * Peta - Pxi * Pzeta - Peta * Pzeta + Pxi * Peta * Pzeta;
    }
  } else {
    const double fx = face == 0 ? 0.0e0 : face == 1 ? 1.0e0 : xi;
    const double fy = face == 2 ? 0.0e0 : face == 3 ? 1.0e0 : eta;
    const double fz = face == 4 ? 0.0e0 : face == 5 ? 1.0e0 : zeta;
    exact_solution(fx, fy, fz, ce, out);
  }
  for (int m = 0; m < 5; ++m) F.u[m * NP + p] = out[m];
  double ex[5];
  exact_solution(xi, eta, zeta, ce, ex);
  for (int m = 0; m < 5; ++m) uex[m * NP + p] = ex[m];
}

// ---------------------------------------------------------------------------
// exact_rhs (src/BT/exact_rhs.jl:41-362): forcing = 0 everywhere, then on
// the interior the xi, eta and zeta flux differences and fourth-order
// dissipation of the exact solution, then forcing = -1 * forcing.  One
// thread per interior point; per element the reference's order of updates.
// ---------------------------------------------------------------------------
struct LinePt {
  double ue[5], buf[5], cuf, q;
};

// dir: 0 xi (velocity index 1), 1 eta (2), 2 zeta (3)
__device__ __forceinline__ void exact_line_point(double xi, double eta, double zeta, int dir, const Coeffs& ce,
                                                 LinePt& o) {
  exact_solution(xi, eta, zeta, ce, o.ue);
  const double dtpp = 1.0e0 / o.ue[0];
  for (int m = 1; m < 5; ++m) o.buf[m] = dtpp * o.ue[m];
  const int a = dir + 1;
  const int b = dir == 0 ? 2 : 1;
  const int c = dir == 2 ? 2 : 3;
  o.cuf = o.buf[a] * o.buf[a];
  o.buf[0] = o.cuf + o.buf[b] * o.buf[b] + o.buf[c] * o.buf[c];
  o.q = 0.5e0 * (o.buf[1] * o.ue[1] + o.buf[2] * o.ue[2] + o.buf[3] * o.ue[3]);
}

__device__ __forceinline__ void exact_dissip(double& f, int q, int n, double dssp, double um2, double um1, double u0,
                                             double up1, double up2) {
  if (q == 1) f = f - dssp * (5.0e0 * u0 - 4.0e0 * up1 + up2);
  if (q == 2) f = f - dssp * (-4.0e0 * um1 + 6.0e0 * u0 - 4.0e0 * up1 + up2);
  if (q >= 3 && q <= n - 4) f = f - dssp * (um2 - 4.0e0 * um1 + 6.0e0 * u0 - 4.0e0 * up1 + up2);
  if (q == n - 3) f = f - dssp * (um2 - 4.0e0 * um1 + 6.0e0 * u0 - 4.0e0 * up1);
  if (q == n - 2) f = f - dssp * (um2 - 4.0e0 * um1 + 5.0e0 * u0);
}

__global__ void __launch_bounds__(128) k_exact_rhs(Fields F, Consts K, Coeffs ce, const Work* __restrict__ work,
                                                   double* __restrict__ forcing) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int q = w.first + threadIdx.x;
  if (q >= Z.nx * Z.ny * Z.nz) return;
  const int i = q % Z.nx, j = (q / Z.nx) % Z.ny, k = q / (Z.nx * Z.ny);
  const int64_t p = Z.off + q, NP = F.NP;
  double f[5] = {0.0e0, 0.0e0, 0.0e0, 0.0e0, 0.0e0};
  const bool interior = i > 0 && i < Z.nx - 1 && j > 0 && j < Z.ny - 1 && k > 0 && k < Z.nz - 1;
  if (interior) {
    const double xi = (double)i * K.dnxm1, eta = (double)j * K.dnym1, zeta = (double)k * K.dnzm1;
    const double c1 = K.c1, c2 = K.c2, dssp = K.dssp;
    for (int dir = 0; dir < 3; ++dir) {
      const int pos = dir == 0 ? i : dir == 1 ? j : k;
      const int n = dir == 0 ? Z.nx : dir == 1 ? Z.ny : Z.nz;
      LinePt L[5] = {};  // positions pos-2 .. pos+2 (outside 0..n-1: unused)
      for (int d = -2; d <= 2; ++d) {
        const int pp = pos + d;
        if (pp < 0 || pp > n - 1) continue;
        const double cx = dir == 0 ? (double)pp * K.dnxm1 : xi;
        const double cy = dir == 1 ? (double)pp * K.dnym1 : eta;
        const double cz = dir == 2 ? (double)pp * K.dnzm1 : zeta;
        exact_line_point(cx, cy, cz, dir, ce, L[d + 2]);
      }
      const LinePt &Lm = L[1], &L0 = L[2], &Lp = L[3];
      const int a = dir + 1;  // the velocity component of this direction
      const double t2 = dir == 0 ? K.tx2 : dir == 1 ? K.ty2 : K.tz2;
      const double d1 = dir == 0 ? K.dx1tx1 : dir == 1 ? K.dy1ty1 : K.dz1tz1;
      const double d2 = dir == 0 ? K.dx2tx1 : dir == 1 ? K.dy2ty1 : K.dz2tz1;
      const double d3 = dir == 0 ? K.dx3tx1 : dir == 1 ? K.dy3ty1 : K.dz3tz1;
      const double d4 = dir == 0 ? K.dx4tx1 : dir == 1 ? K.dy4ty1 : K.dz4tz1;
      const double d5 = dir == 0 ? K.dx5tx1 : dir == 1 ? K.dy5ty1 : K.dz5tz1;
      const double con1 = dir == 0 ? K.xxcon1 : dir == 1 ? K.yycon1 : K.zzcon1;
      const double con2 = dir == 0 ? K.xxcon2 : dir == 1 ? K.yycon2 : K.zzcon2;
      const double con3 = dir == 0 ? K.xxcon3 : dir == 1 ? K.yycon3 : K.zzcon3;
      const double con4 = dir == 0 ? K.xxcon4 : dir == 1 ? K.yycon4 : K.zzcon4;
      const double con5 = dir == 0 ? K.xxcon5 : dir == 1 ? K.yycon5 : K.zzcon5;
      const double dd[5] = {d1, d2, d3, d4, d5};
      // flux differences: continuity, the momentum component along dir (with
      // pressure), the two transverse momenta, energy
      f[0] = f[0] - t2 * (Lp.ue[a] - Lm.ue[a]) + d1 * (Lp.ue[0] - 2.0e0 * L0.ue[0] + Lm.ue[0]);
      for (int m = 1; m <= 3; ++m) {
        if (m == a) {
          f[m] = f[m] - t2 * ((Lp.ue[m] * Lp.buf[a] + c2 * (Lp.ue[4] - Lp.q)) -
                              (Lm.ue[m] * Lm.buf[a] + c2 * (Lm.ue[4] - Lm.q))) +
                 con1 * (Lp.buf[m] - 2.0e0 * L0.buf[m] + Lm.buf[m]) +
                 dd[m] * (Lp.ue[m] - 2.0e0 * L0.ue[m] + Lm.ue[m]);
        } else {
          f[m] = f[m] - t2 * (Lp.ue[m] * Lp.buf[a] - Lm.ue[m] * Lm.buf[a]) +
                 con2 * (Lp.buf[m] - 2.0e0 * L0.buf[m] + Lm.buf[m]) +
                 dd[m] * (Lp.ue[m] - 2.0e0 * L0.ue[m] + Lm.ue[m]);
        }
      }
      f[4] = f[4] - t2 * (Lp.buf[a] * (c1 * Lp.ue[4] - c2 * Lp.q) - Lm.buf[a] * (c1 * Lm.ue[4] - c2 * Lm.q)) +
             0.5e0 * con3 * (Lp.buf[0] - 2.0e0 * L0.buf[0] + Lm.buf[0]) +
             con4 * (Lp.cuf - 2.0e0 * L0.cuf + Lm.cuf) + con5 * (Lp.buf[4] - 2.0e0 * L0.buf[4] + Lm.buf[4]) +
             d5 * (Lp.ue[4] - 2.0e0 * L0.ue[4] + Lm.ue[4]);
      for (int m = 0; m < 5; ++m)
        exact_dissip(f[m], pos, n, dssp, L[0].ue[m], L[1].ue[m], L[2].ue[m], L[3].ue[m], L[4].ue[m]);
    }
    for (int m = 0; m < 5; ++m) f[m] = -1.0e0 * f[m];
  }
  for (int m = 0; m < 5; ++m) forcing[m * NP + p] = f[m];
}

// ---------------------------------------------------------------------------
// exch_qbc (src/BT/exchange_qbc.jl:145-465): for face f of zone z, copy the
// neighbour's interior plane into z's ghost plane.  Faces: 0 west (i=0 <-
// west's i=nx-2), 1 east (i=nx-1 <- east's i=1), 2 south (j=0 <- south's
// j=ny-2), 3 north (j=ny-1 <- north's j=1); transverse indices 1..n-2.
// blockIdx.y = zone*4 + face.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_exch_qbc(Fields F, const int* __restrict__ nbr, int zone_lo) {
  const int z = zone_lo + blockIdx.y / 4, face = blockIdx.y % 4;
  const int src_zone = nbr[4 * z + face];
  if (src_zone < 0) return;  // a face of a zone on another rank: npbmz_unpack_faces fills it
  const ZoneDev Z = F.zones[z];
  const ZoneDev S = F.zones[src_zone];
  const int nt = face < 2 ? Z.ny - 2 : Z.nx - 2;  // transverse length
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
    F.u[m * NP + dst] = F.u[m * NP + src];
  }
}

// ---------------------------------------------------------------------------
// Faces exchanged with zones on other ranks (the inter-process part of
// exch_qbc, src/BT/exchange_qbc.jl:145-465).  Face f of the list is (zone,
// side); its 5 (n-2)(nz-2) values sit at buf[off..] in the reference's packing
// order: variable m outermost, then k = 1..nz-2, then the transverse index
// (j for west/east, i for south/north) = 1..n-2.
//   pack (side s): the interior plane the neighbour on side s reads --
//     west i = 1, east i = nx-2, south j = 1, north j = ny-2;
//   unpack (side s): the ghost plane on side s --
//     west i = 0, east i = nx-1, south j = 0, north j = ny-1.
// blockIdx.y = face.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t face_point(const ZoneDev& Z, int side, bool ghost, int a, int k) {
  const int i_w = ghost ? 0 : 1, i_e = ghost ? Z.nx - 1 : Z.nx - 2;
  const int j_s = ghost ? 0 : 1, j_n = ghost ? Z.ny - 1 : Z.ny - 2;
  if (side == 0) return Z.off + ((int64_t)k * Z.ny + (1 + a)) * Z.nx + i_w;
  if (side == 1) return Z.off + ((int64_t)k * Z.ny + (1 + a)) * Z.nx + i_e;
  if (side == 2) return Z.off + ((int64_t)k * Z.ny + j_s) * Z.nx + (1 + a);
  return Z.off + ((int64_t)k * Z.ny + j_n) * Z.nx + (1 + a);
}

template <bool PACK>
__global__ void __launch_bounds__(256) k_faces(Fields F, const FaceDesc* __restrict__ faces, double* __restrict__ buf) {
  const FaceDesc f = faces[blockIdx.y];
  const ZoneDev Z = F.zones[f.zone];
  const int nt = f.side < 2 ? Z.ny - 2 : Z.nx - 2;
  const int count = 5 * nt * (Z.nz - 2);
  const int64_t NP = F.NP;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < count; t += gridDim.x * blockDim.x) {
    const int a = t % nt, k = 1 + (t / nt) % (Z.nz - 2), m = t / (nt * (Z.nz - 2));
    const int64_t p = m * NP + face_point(Z, f.side, !PACK, a, k);
    if (PACK) buf[f.off + t] = F.u[p];
    else F.u[p] = buf[f.off + t];
  }
}

// ---------------------------------------------------------------------------
// error_norm partial sums (src/BT/error.jl:7-44): (u - u_exact)^2 over all
// points of the CTA's zone share.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_err_partials(Fields F, const Work* __restrict__ work,
                                                      double* __restrict__ partials) {
  __shared__ double red[5 * 128];
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int q = w.first + threadIdx.x;
  double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (q < Z.nx * Z.ny * Z.nz) {
    const int64_t p = Z.off + q;
    for (int m = 0; m < 5; ++m) {
      const double a = F.u[m * F.NP + p] - F.uex[m * F.NP + p];
      v[m] = a * a;
    }
  }
  block_sum5(v, red);
  if (threadIdx.x == 0)
    for (int m = 0; m < 5; ++m) partials[blockIdx.x * 5 + m] = v[m];
}

// Combine per-CTA partial sums into the reference's zone-summed norms:
// out[m] = sum_z scale * sqrt(S_z[m] / ((nx-2)(ny-2)(nz-2))), zones in order.
// zblk[2z], zblk[2z+1] bound the CTAs of zone z.  One CTA of 32 threads; m < 5.
__global__ void k_norm_finish(const ZoneDev* __restrict__ zones, const double* __restrict__ partials,
                              const int* __restrict__ zblk, int nzones, double scale, double* __restrict__ out) {
  const int m = threadIdx.x;
  if (m >= 5) return;
  double total = 0.0;
  for (int z = 0; z < nzones; ++z) {
    double s = 0.0;
    for (int b = zblk[2 * z]; b < zblk[2 * z + 1]; ++b) s = s + partials[b * 5 + m];
    const ZoneDev Z = zones[z];
    const double denom = (double)(Z.nx - 2) * (double)(Z.ny - 2) * (double)(Z.nz - 2);
    total = total + sqrt(s / denom) * scale;
  }
  out[m] = total;
}

// ---------------------------------------------------------------------------
// Layout conversion between the device planes and a staging copy of one
// zone's host array (dense [m][k][j][i] or the reference's OffsetArray).
// dir = 0: staging -> device, 1: device -> staging.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t ref_index(int kind, int field, const ZoneDev& Z, int m, int i, int j, int k) {
  const int IMAX = Z.nx + 1, JMAX = Z.ny + 1, KMAX = Z.nz + 1;
  if (kind == 0) {  // BT, AoS [1:5, ...]
    if (field == 0)  // u: [1:5, -2:IMAX+1, -2:JMAX+1, -2:KMAX+1]
      return m + 5 * ((int64_t)(i + 2) + (int64_t)(IMAX + 4) * ((j + 2) + (int64_t)(JMAX + 4) * (k + 2)));
    if (field == 1)  // rhs: [1:5, -1:IMAX-1, ...]
      return m + 5 * ((int64_t)(i + 1) + (int64_t)(IMAX + 1) * ((j + 1) + (int64_t)(JMAX + 1) * (k + 1)));
    return m + 5 * ((int64_t)i + (int64_t)IMAX * (j + (int64_t)JMAX * k));  // forcing [1:5, 0:IMAX-1, ...]
  }
  const int IMAXP = (IMAX / 2) * 2 + 1, JMAXP = (JMAX / 2) * 2 + 1;
  if (field == 0) {  // SP u: [-2:IMAXP+1, -2:JMAXP+1, -2:KMAX+1, 1:5]
    const int64_t ni = IMAXP + 4, nj = JMAXP + 4, nk = KMAX + 4;
    return (i + 2) + ni * ((j + 2) + nj * ((k + 2) + nk * (int64_t)m));
  }
  // SP rhs / forcing: [0:IMAXP-1, 0:JMAXP-1, 0:KMAX-1, 1:5]
  const int64_t ni = IMAXP, nj = JMAXP, nk = KMAX;
  return i + ni * (j + nj * (k + nk * (int64_t)m));
}

// blockIdx.y = zone index within [zone_lo, zone_lo + gridDim.y), or the
// zone zlist[blockIdx.y] when zlist is given.  The host
// side array of zone z starts at element soff[z] - sub of `stage`, which is
// either the device staging buffer (sub = 0) or the device mapping of a
// page-locked host buffer holding zones from zone_lo (sub = soff[zone_lo]).
// layout 0: dense [m][k][j][i]; 1: the reference OffsetArray (with halo);
// 2: compact reference order without halo (BT [k][j][i][m], SP = dense).
// part (uploads split around exch_qbc): 0 every point; 1 only the interior
// planes exch_qbc reads (i = 1, nx-2 and j = 1, ny-2, transverse indices
// 1..n-2); 2 every point but the ghost planes exch_qbc writes (i = 0, nx-1
// and j = 0, ny-1, transverse indices 1..n-2).
__device__ __forceinline__ bool exch_point(const ZoneDev& Z, int i, int j, int k, bool ghost) {
  if (k < 1 || k > Z.nz - 2) return false;
  const int ilo = ghost ? 0 : 1, ihi = ghost ? Z.nx - 1 : Z.nx - 2;
  const int jlo = ghost ? 0 : 1, jhi = ghost ? Z.ny - 1 : Z.ny - 2;
  const bool xface = (i == ilo || i == ihi) && j >= 1 && j <= Z.ny - 2;
  const bool yface = (j == jlo || j == jhi) && i >= 1 && i <= Z.nx - 2;
  return xface || yface;
}

__global__ void __launch_bounds__(256) k_convert(Fields F, double* __restrict__ field_planes,
                                                 double* __restrict__ stage, const int64_t* __restrict__ soff,
                                                 int64_t sub, int zone_lo, int kind, int field, int layout, int dir,
                                                 const int* __restrict__ zlist, int part) {
  const int zone = zlist ? zlist[blockIdx.y] : zone_lo + blockIdx.y;
  const ZoneDev Z = F.zones[zone];
  const int np = Z.nx * Z.ny * Z.nz;
  double* st = stage + (soff[zone] - sub);
  // BT's reference arrays are variable-fastest (AoS): there consecutive
  // threads take consecutive variables of a point, so a warp reads or writes
  // one contiguous run of host memory (over NVLink-C2C for page-locked
  // buffers) and the device side splits it across the five planes.
  const bool aos = kind == 0 && layout != 0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 5 * np; t += gridDim.x * blockDim.x) {
    const int m = aos ? t % 5 : t / np, q = aos ? t / 5 : t % np;
    const int i = q % Z.nx, j = (q / Z.nx) % Z.ny, k = q / (Z.nx * Z.ny);
    if (part == 1 && !exch_point(Z, i, j, k, false)) continue;
    if (part == 2 && exch_point(Z, i, j, k, true)) continue;
    int64_t s;
    if (layout == 0) s = t;
    else if (layout == 1) s = ref_index(kind, field, Z, m, i, j, k);
    else s = kind == 0 ? (int64_t)q * 5 + m : (int64_t)t;
    const int64_t d = m * F.NP + Z.off + q;
    if (dir == 0) field_planes[d] = st[s];
    else st[s] = field_planes[d];
  }
}

// ---------------------------------------------------------------------------
// State check of u over the point work list (one thread per zone point): the
// health word of Fields (see health_check) for the state a call leaves.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_state_check(Fields F, const Work* __restrict__ work) {
  const Work w = work[blockIdx.x];
  const ZoneDev Z = F.zones[w.zone];
  const int q = w.first + threadIdx.x;
  if (q >= Z.nx * Z.ny * Z.nz) return;
  const int64_t p = Z.off + q, NP = F.NP;
  const double rho = F.u[p], m1 = F.u[NP + p], m2 = F.u[2 * NP + p], m3 = F.u[3 * NP + p], e = F.u[4 * NP + p];
  health_check(F, p, rho, e - 0.5 * (m1 * m1 + m2 * m2 + m3 * m3) / rho);
}

__global__ void k_fill(double* __restrict__ a, int64_t n, double v) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) a[t] = v;
}

// ============================== launchers ==================================
void launch_initialize(const Fields& F, const Consts& K, const double* ce, const Work* work, int nwork, double* uex,
                       cudaStream_t s) {
  Coeffs c;
  for (int e = 0; e < 65; ++e) c.c[e] = ce[e];
  if (nwork > 0) k_initialize<<<nwork, 128, 0, s>>>(F, K, c, work, uex);
}

void launch_exact_rhs(const Fields& F, const Consts& K, const double* ce, const Work* work, int nwork, double* forcing,
                      cudaStream_t s) {
  Coeffs c;
  for (int e = 0; e < 65; ++e) c.c[e] = ce[e];
  if (nwork > 0) k_exact_rhs<<<nwork, 128, 0, s>>>(F, K, c, work, forcing);
}

void launch_exch_qbc(const Fields& F, const int* nbr_dev, int zone_lo, int nz_count, int max_face, cudaStream_t s) {
  if (nz_count <= 0) return;
  int gx = (max_face + 255) / 256;
  if (gx < 1) gx = 1;
  if (gx > 64) gx = 64;
  dim3 grid(gx, 4 * nz_count);
  k_exch_qbc<<<grid, 256, 0, s>>>(F, nbr_dev, zone_lo);
}

void launch_err_partials(const Fields& F, const Work* work, int nwork, double* partials, cudaStream_t s) {
  if (nwork > 0) k_err_partials<<<nwork, 128, 0, s>>>(F, work, partials);
}

void launch_norm_finish(const ZoneDev* zones, const double* partials, const int* zblk, int nzones, double scale,
                        double* out, cudaStream_t s) {
  k_norm_finish<<<1, 32, 0, s>>>(zones, partials, zblk, nzones, scale, out);
}

void launch_convert(const Fields& F, double* planes, double* stage, const int64_t* soff, int64_t sub, int zone_lo,
                    int nzn, int max_np, int kind, int field, int layout, int dir, cudaStream_t s, const int* zlist,
                    int part) {
  if (nzn <= 0) return;
  int gx = (5 * max_np + 255) / 256;
  if (gx > 512) gx = 512;
  dim3 grid(gx, nzn);
  k_convert<<<grid, 256, 0, s>>>(F, planes, stage, soff, sub, zone_lo, kind, field, layout, dir, zlist, part);
}

void launch_faces(bool pack, const Fields& F, const FaceDesc* faces, int nfaces, int max_face, double* buf,
                  cudaStream_t s) {
  if (nfaces <= 0) return;
  int gx = (max_face + 255) / 256;
  if (gx < 1) gx = 1;
  if (gx > 64) gx = 64;
  dim3 grid(gx, nfaces);
  if (pack) k_faces<true><<<grid, 256, 0, s>>>(F, faces, buf);
  else k_faces<false><<<grid, 256, 0, s>>>(F, faces, buf);
}

// The FMA build's FP64 reciprocal (nr_rcp of npbmz_internal.cuh), for
// npbmz_math_check.
__global__ void k_math_check(int which, int n, const double* __restrict__ x, double* __restrict__ y) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n || which != 0) return;
  y[t] = nr_rcp(x[t]);
}

void launch_math_check(int which, int n, const double* x, double* y, cudaStream_t s) {
  if (n > 0) k_math_check<<<(n + 255) / 256, 256, 0, s>>>(which, n, x, y);
}

void launch_state_check(const Fields& F, const Work* work, int nwork, cudaStream_t s) {
  if (nwork > 0 && F.health) k_state_check<<<nwork, 128, 0, s>>>(F, work);
}

void launch_fill(double* a, int64_t n, double v, cudaStream_t s) {
  int64_t g = (n + 255) / 256;
  k_fill<<<(int)(g > 4096 ? 4096 : (g < 1 ? 1 : g)), 256, 0, s>>>(a, n, v);
}

// ---------------------------------------------------------------------------
// FP64 FMA throughput probe (roofline denominator for the FP64-bound
// kernels): 8 independent dependent chains of fma() per thread.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_fp64_probe(double* __restrict__ sink, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) x[c] = (double)(threadIdx.x + c) * 1e-3;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += x[c];
  if (s == 123.456) sink[threadIdx.x] = s;  // keeps the chains live
}

int probe_fp64(double* gflops) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double* sink = nullptr;
  if (cudaMalloc(&sink, 256 * sizeof(double)) != cudaSuccess) return -1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, iters = 4096;
  k_fp64_probe<<<blocks, 256>>>(sink, 64, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0);
  k_fp64_probe<<<blocks, 256>>>(sink, iters, 0.999999, 1e-7);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (err != cudaSuccess || ms <= 0.f) return -1;
  *gflops = 2.0 * 8.0 * iters * (double)blocks * 256.0 / (ms * 1e-3) / 1e9;
  return 0;
}

}  // namespace npbmz
