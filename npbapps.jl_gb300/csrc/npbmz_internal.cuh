// npbmz_internal.cuh -- device-side data layout and constants shared by the
// kernels of libnpbmz_gpu.so.
//
// HBM layout: every field is variable-major structure-of-arrays over the
// points of ALL zones: field[m * NP + zone.off + (k * ny + j) * nx + i].
// Zone offsets are multiples of 32 points (256 B), NP is the padded total.
// Each zone stores its points 0..n-1 on every axis (0 and n-1 are the ghost /
// physical-boundary planes); the reference's 2-deep OffsetArray halo is not
// stored because no value computed there reaches u, rhs or a norm.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace npbmz {

// set_constants (src/BT/set_constants.jl:1-130), evaluated on the host.
struct Consts {
  double dt, dnxm1, dnym1, dnzm1;
  double c1, c2, c3, c4, c5, bt, c1c2, c1c5, c3c4, c1345, conz1, con43, con16, c2iv, dssp;
  double dx1, dx2, dx3, dx4, dx5, dy1, dy2, dy3, dy4, dy5, dz1, dz2, dz3, dz4, dz5, dxmax, dymax, dzmax;
  double tx1, tx2, tx3, ty1, ty2, ty3, tz1, tz2, tz3;
  double dttx1, dttx2, dtty1, dtty2, dttz1, dttz2, c2dttx1, c2dtty1, c2dttz1;
  double comz1, comz4, comz5, comz6;
  double dx1tx1, dx2tx1, dx3tx1, dx4tx1, dx5tx1;
  double dy1ty1, dy2ty1, dy3ty1, dy4ty1, dy5ty1;
  double dz1tz1, dz2tz1, dz3tz1, dz4tz1, dz5tz1;
  double xxcon1, xxcon2, xxcon3, xxcon4, xxcon5;
  double yycon1, yycon2, yycon3, yycon4, yycon5;
  double zzcon1, zzcon2, zzcon3, zzcon4, zzcon5;
  // FP32 values (f_) and double-float pairs (p_: {rn(v), rn(v - rn(v))}) of
  // the constants that the FP32 sweeps and their refinement passes read,
  // formed on the host so that no kernel converts them: on GB300 every
  // FP64-to-FP32 conversion is an instruction of the 1/64-rate FP64 pipe.
  // Index [d] is the sweep direction; f_d / p_d hold dx1..dx5, dy1..dy5,
  // dz1..dz5.
  float f_c1, f_c2, f_c3, f_c4, f_c3c4, f_c1345, f_con43, f_c1c5, f_comz1, f_comz4, f_comz5, f_comz6;
  float f_dtt1[3], f_dtt2[3], f_c2dtt1[3], f_d[3][5], f_dmax[3];
  float2 p_c1, p_c2, p_two_m_c2, p_k43, p_c3c4, p_c1345, p_k43m, p_c3c4m;
  float2 p_con43, p_c1c5, p_comz1, p_comz4, p_comz5, p_comz6, p_bt, p_c2iv;
  float2 p_dtt1[3], p_dtt2[3], p_c2dtt1[3], p_d[3][5], p_dmax[3];
};

// The FP32 (T = float) or FP64 (T = double) copy of a constant.
template <typename T>
__host__ __device__ inline T kv(double d, float f);
template <>
__host__ __device__ inline float kv<float>(double, float f) { return f; }
template <>
__host__ __device__ inline double kv<double>(double d, float) { return d; }

struct ZoneDev {
  int nx, ny, nz, pad;
  int64_t off;          // first point of the zone in every field plane
  int64_t lineoff[3];   // first global line index of the zone, per sweep direction
};

// One face exchanged with another rank: (zone, side 0..3 = west, east, south,
// north) and the offset of its values in the exchange buffer.
struct FaceDesc {
  int zone, side;
  int64_t off;
};

// One work item = one CTA's share: `first` is the first point (point lists)
// or the first line (line lists) of zone `zone` that the CTA handles.
struct Work {
  int zone;
  int first;
};

// Primitive-variable planes written by the primitive kernel.
enum { PR_RHOI = 0, PR_US, PR_VS, PR_WS, PR_QS, PR_SQUARE, PR_SPEED, PR_AINV, PR_COUNT };

// FP32 copies of the state read by the FP32 line-solve passes: planes
// 0..5 hold the rounded values (hi), planes 6..11 the remainders (lo), so
// that hi + lo carries the FP64 value to about 48 bits (double-float).
enum { PF_RHOI = 0, PF_QS, PF_U2, PF_U3, PF_U4, PF_U5, PF_HI_COUNT, PF_COUNT = 2 * PF_HI_COUNT };
// SP: FP32 copies of 1/rho, the three velocities and the speed of sound:
// planes 0..4 the rounded values (hi), 5..9 the remainders (lo).
enum { PS_RHOI = 0, PS_US, PS_VS, PS_WS, PS_SPEED, PS_HI_COUNT, PS_COUNT = 2 * PS_HI_COUNT };

// Point functions of compute_rhs written by the primitive kernel of the FMA
// build (one value per point, shared by both neighbours that difference it):
// the off-diagonal momentum fluxes (u2 u3 / u1 = u3 us = u2 vs, ...), the
// normal momentum fluxes with the pressure term, the energy fluxes and the
// viscous energy terms of each direction.
enum {
  PX_UV = 0, PX_UW, PX_VW,   // u2*u3/u1, u2*u4/u1, u3*u4/u1
  PX_XX, PX_YY, PX_ZZ,       // u2*us + c2*(u5 - square), u3*vs + ..., u4*ws + ...
  PX_EX, PX_EY, PX_EZ,       // (c1*u5 - c2*square) * us / vs / ws
  PX_WX, PX_WY, PX_WZ,       // con3*qs + con4*vel^2 + con5*u5/u1 with the x / y / z constants
  PX_COUNT
};

// Double-float point planes of compute_rhs for the refined mixed step
// (float2 {hi, lo} per point, one plane per quantity): the twelve PX_*
// functions, then the three velocities and (SP) qs for txinvr.
enum { XD_US = PX_COUNT, XD_VS, XD_WS, XD_QS, XD_COUNT };

// Double-float constants of compute_rhs and the primitive kernel of the
// refined mixed step, split on the host ({hi, lo} = rn(c), rn(c - hi)).
struct RhsDfConsts {
  float2 w[3][32][5];  // LinWeights
  float2 vc[3][3];     // velocity second-difference factors per direction, variables 2..4
  float2 vcc[3];       // centre point: -2 * sum over the directions of vc
  float2 t2[3];        // tx2, ty2, tz2
  float2 dt, c1, c2, c1c2, bt;
  float2 con3[3], con4[3], con5[3];  // xxcon3..5, yycon3..5, zzcon3..5
  int exact_w;  // the low words of every w and t2 are at most 2^-47 of the high: left out
};

struct Fields {
  double* u;        // [5][NP]
  double* rhs;      // [5][NP]
  const double* forcing;  // [5][NP]
  double* prim;     // [PR_COUNT][NP]
  const double* uex;      // [5][NP] exact solution (error norm)
  const ZoneDev* zones;
  int64_t NP;
  float* primf;     // [PF_COUNT][NP] or null
  double* flux = nullptr;  // [PX_COUNT][NP] or null (FMA build's compute_rhs)
  // [10][NP] double-float copy of rhs (planes 0..4 hi, 5..9 lo) that the
  // refined FP32 BT sweeps of one step hand to each other, or null
  float* rdf = nullptr;
  // x-line-major copies for the refined FP32 BT x sweep, so that the lines of
  // a warp (consecutive j, nx points apart in the zone layout) read adjacent
  // words: element e of point i of x line g at [(i * E + e) * nlx + g]
  float* pfx = nullptr;  // E = PF_COUNT: FP32 state hi / lo (primitive kernel)
  float* rdx = nullptr;  // E = 10: double-float rhs (compute_rhs; line ends: the forcing)
  float* x0x = nullptr;  // E = 5: first-pass solution
  int64_t nlx = 0;       // x lines of all zones
  // refined mixed step with the double-float compute_rhs (else null):
  float2* ud = nullptr;        // [5][NP] u
  float2* xd = nullptr;        // [XD_COUNT][NP] point functions of compute_rhs
  const float2* fd = nullptr;  // [5][NP] forcing
  const double* fdt = nullptr;  // [5][NP] dt * forcing (FMA build's compute_rhs)
  // the primitive kernel writes the FP64 planes prim (single phases; SP's
  // z sweep reads us, vs, ws, speed, ainv, qs in every step)
  bool prim64 = true;
  // compute_rhs writes rhs in FP64 as well as its double-float copy
  bool rhs64 = true;
  // state check (null: off): word 0 ORs the HEALTH_* bits of every point
  // found bad, word 1 keeps the smallest such global point index (all ones
  // while none)
  unsigned long long* health = nullptr;
};

// ---- state check ------------------------------------------------------------
// A point of u is healthy when its density rho and its pressure-like quantity
// rho E - |rho v|^2 / (2 rho) are both positive and finite.  Bits: the
// density is not positive and finite; the pressure is finite but not
// positive; the pressure is not finite (a NaN or infinity anywhere in u).
constexpr unsigned HEALTH_DENSITY = 1u;
constexpr unsigned HEALTH_PRESSURE = 2u;
constexpr unsigned HEALTH_NONFINITE = 4u;

// v > 0 and finite, on the bit pattern (integer pipe): the positive finite
// doubles are exactly the patterns 1 .. 0x7FEFFFFFFFFFFFFF; zero, negatives,
// infinities and NaNs all fall outside.
__device__ __forceinline__ bool positive_finite(double v) {
  return (unsigned long long)__double_as_longlong(v) - 1ull < 0x7FEFFFFFFFFFFFFFull;
}

// Record a bad point p (global index).  The padding points between zones
// hold u = (1, 0, 0, 0, 1) from creation on (nothing writes them later), so
// kernels over the padded plane find nothing there.
__device__ __forceinline__ void health_report(const Fields& F, int64_t p, unsigned bits) {
  atomicOr(F.health, (unsigned long long)bits);
  atomicMin(F.health + 1, (unsigned long long)p);
}

__device__ __forceinline__ bool positive_finite(float v) { return (unsigned)__float_as_uint(v) - 1u < 0x7F7FFFFFu; }
__device__ __forceinline__ bool finite_bits(double v) {
  return ((unsigned long long)__double_as_longlong(v) & 0x7FF0000000000000ull) != 0x7FF0000000000000ull;
}
__device__ __forceinline__ bool finite_bits(float v) { return (__float_as_uint(v) & 0x7F800000u) != 0x7F800000u; }

// rho and pressure in FP64, or (the double-float kernels) as the high words
// of their double-float values
// The same from the energy e = rho E and k = |rho v|^2 / (2 rho) without
// forming e - k (an FP64 instruction): for e positive and finite, e - k > 0
// exactly when e > k, and for k >= 0 that order is the order of the bit
// patterns; a negative k (negative rho) leaves e - k positive.
__device__ __forceinline__ void health_check_ek(const Fields& F, int64_t p, double rho, double e, double k) {
  if (!F.health) return;
  const long long be = __double_as_longlong(e), bk = __double_as_longlong(k);
  const bool ok = positive_finite(rho) && positive_finite(e) && finite_bits(k) && (bk < 0 || be > bk);
  if (__builtin_expect(ok, 1)) return;
  const bool finite = finite_bits(e) && finite_bits(k);
  const unsigned bits = (positive_finite(rho) ? 0u : HEALTH_DENSITY) |
                        (!finite ? HEALTH_NONFINITE : (bk < 0 || (be > bk && be > 0)) ? 0u : HEALTH_PRESSURE);
  health_report(F, p, bits);
}

template <typename R>
__device__ __forceinline__ void health_check(const Fields& F, int64_t p, R rho, R pressure) {
  if (!F.health) return;
  if (__builtin_expect(positive_finite(rho) && positive_finite(pressure), 1)) return;
  const unsigned bits = (positive_finite(rho) ? 0u : HEALTH_DENSITY) |
                        (positive_finite(pressure) ? 0u : finite_bits(pressure) ? HEALTH_PRESSURE : HEALTH_NONFINITE);
  health_report(F, p, bits);
}

// x line through interior point (j, k) of zone z (-1 when j or k is a face).
__host__ __device__ inline int64_t xline_of(const ZoneDev& z, int j, int k) {
  if (j < 1 || j > z.ny - 2 || k < 1 || k > z.nz - 2) return -1;
  return z.lineoff[0] + (j - 1) + (int64_t)(k - 1) * (z.ny - 2);
}

// The linear part of compute_rhs along one direction -- the second
// difference d*t1*(u[q-1] - 2u[q] + u[q+1]) of each variable and the
// fourth-order dissipation -- as one 5-point stencil whose weights depend on
// the position class of q (bit 0: q == 1, 1: q == 2, 2: 3 <= q <= n-4,
// 3: q == n-3, 4: q == n-2; several bits when the reference's stencils
// overlap on a short axis).  Valid when the d*t1 factor is the same for the
// five variables of a direction, as set_constants makes it.
struct LinWeights {
  double w[3][32][5];
};

// The constants of the FMA build's compute_rhs with dt folded in (its rhs is
// dt * (forcing + terms); here the forcing comes as dt * forcing and every
// term's factor carries dt): LinWeights times dt, dt*t2 per direction, the
// velocity second-difference factors times dt per direction, and the centre
// point's velocity factor -2 * sum over the directions.
struct RhsF64Consts {
  double w[3][32][5];
  double t2[3];
  double vc[3][3];
  double vcc[3];
  double dt;
};

// FP64 value -> FP32 pair (hi = rn(v), lo = rn(v - hi)), the same bits as the
// conversions __double2float_rn(v) and __double2float_rn(v - (double)hi),
// formed with integer operations from v's bit pattern: on GB300 each FP64
// conversion or subtraction takes a slot of the 1/64-rate FP64 pipe, and the
// kernels that split are FP64-pipe bound.  hi keeps the top 24 significand
// bits rounded to nearest even; the 29 bits below (minus 2^29 when hi rounded
// up) are the exact v - hi in units of 2^(e-52), converted to float (one
// rounding) and scaled by that power of two (exact while 2^(e-52) is a normal
// float, e >= -74).  Outside -74 <= e <= 126 (zero, subnormal, tiny, huge,
// inf, nan) it falls back to the conversions.
__device__ __forceinline__ void split_df(double v, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ffull) - 1023;
  if (e < -74 || e > 126) {
    hi = __double2float_rn(v);
    lo = __double2float_rn(v - (double)hi);
    return;
  }
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const unsigned long long man = b & 0xfffffffffffffull;
  const unsigned r = (unsigned)(man & 0x1fffffffull);    // the 29 bits below hi
  const unsigned mhi = (unsigned)(man >> 29);             // 23 stored bits of hi
  const bool up = r > 0x10000000u || (r == 0x10000000u && (mhi & 1u));
  hi = __uint_as_float(sign | ((((unsigned)(e + 127) << 23) | mhi) + (up ? 1u : 0u)));
  const int L = up ? (int)r - 0x20000000 : (int)r;       // v - hi = L * 2^(e-52), |L| <= 2^28
  const float mag = (float)L * __int_as_float((e - 52 + 127) << 23);
  lo = sign ? -mag : mag;
}

// ---- FP64 reciprocal without an FP64 divide ------------------------------------
// Newton-Raphson refinement of the FP32 hardware estimate (the method of
// P. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Dev. 34(1), 1990): the estimate is taken
// of x's leading 24 bits, the operands move between the formats by bit
// manipulation (integer pipe; a conversion instruction would take the FP64
// pipe), and each FP64 FMA step squares the relative error -- about 2^-22 for
// the estimate, 2^-44 after one step, within 2 ulps after the second.  Used
// for 1/rho by the FMA build's primitive kernel, where the IEEE divide cost a
// large share of its FP64 instructions.  Positive x inside the FP32 normal
// range only; anything else takes the IEEE divide.
__device__ __forceinline__ bool f64_to_f32_bits(double x, float& xf) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ffull) - 1023;
  if ((b >> 63) || e < -125 || e > 125) return false;
  xf = __uint_as_float(((unsigned)(e + 127) << 23) | (unsigned)((b >> 29) & 0x7fffffull));
  return true;
}

__device__ __forceinline__ double f32_to_f64_bits(float y) {  // y positive and normal
  const unsigned f = __float_as_uint(y);
  const unsigned long long e = (unsigned long long)((f >> 23) & 0xffu) - 127ull + 1023ull;
  return __longlong_as_double((long long)((e << 52) | ((unsigned long long)(f & 0x7fffffu) << 29)));
}

__device__ __forceinline__ double nr_rcp(double x) {
  float xf, yf;
  if (!f64_to_f32_bits(x, xf)) return 1.0 / x;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(xf));
  double y = f32_to_f64_bits(yf);
  double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  return fma(y, e, y);
}

// Lines per sweep direction of a zone (interior transverse indices only).
__host__ __device__ inline int zone_lines(const ZoneDev& z, int dir) {
  return dir == 0 ? (z.ny - 2) * (z.nz - 2) : (dir == 1 ? (z.nx - 2) * (z.nz - 2) : (z.nx - 2) * (z.ny - 2));
}

__host__ __device__ inline int zone_line_len(const ZoneDev& z, int dir) {
  return dir == 0 ? z.nx : (dir == 1 ? z.ny : z.nz);
}

// First point and point stride of line `line` of zone z in direction dir.
__host__ __device__ inline void line_geometry(const ZoneDev& z, int dir, int line, int64_t& base, int64_t& stride) {
  if (dir == 0) {
    int j = 1 + line % (z.ny - 2), k = 1 + line / (z.ny - 2);
    base = z.off + ((int64_t)k * z.ny + j) * z.nx;
    stride = 1;
  } else if (dir == 1) {
    int i = 1 + line % (z.nx - 2), k = 1 + line / (z.nx - 2);
    base = z.off + (int64_t)k * z.ny * z.nx + i;
    stride = z.nx;
  } else {
    int i = 1 + line % (z.nx - 2), j = 1 + line / (z.nx - 2);
    base = z.off + (int64_t)j * z.nx + i;
    stride = (int64_t)z.nx * z.ny;
  }
}

// Deterministic CTA sum of 5 values per thread (fixed tree shape); the result
// is valid in thread 0.  scratch must hold 5 * blockDim.x doubles.
__device__ inline void block_sum5(double v[5], double* scratch) {
  const int t = threadIdx.x, n = blockDim.x;
  for (int m = 0; m < 5; ++m) scratch[m * n + t] = v[m];
  __syncthreads();
  for (int s = n / 2; s > 0; s >>= 1) {
    if (t < s)
      for (int m = 0; m < 5; ++m) scratch[m * n + t] = scratch[m * n + t] + scratch[m * n + t + s];
    __syncthreads();
  }
  if (t == 0)
    for (int m = 0; m < 5; ++m) v[m] = scratch[m * n];
  __syncthreads();
}

}  // namespace npbmz
