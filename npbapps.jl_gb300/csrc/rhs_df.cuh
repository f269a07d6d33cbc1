// rhs_df.cuh -- the primitive kernel and compute_rhs of the refined mixed
// step in double-float arithmetic, included by step_kernels.cuh in the FMA
// build.
//
// GB300 runs FP64 at 1/64 of the FP32 rate, and the FP64 forms of these two
// kernels (k_prim_w, k_rhs_flux) are bound by the FP64 pipe.  Here every
// quantity is an unevaluated sum hi + lo of two FP32 values (about 48
// significand bits) and every operation is built from error-free
// transformations on the FP32 pipe: Knuth's two-sum, the FMA two-product,
// Dekker's normalisation, and one Newton step for 1/x and sqrt(x) from the
// FP32 estimate.  No FP64 arithmetic runs except the conversions of the
// planes that stay FP64 outside a fused step (prim, rhs).
//
// The statements are compute_rhs's (src/BT/rhs.jl:62-460, SP
// src/SP/rhs.jl:62-452 and txinvr src/SP/txinvr.jl:28-49) in the regrouped
// form of k_rhs_flux: the point functions (fluxes, viscous energy terms,
// velocities) come from the primitive kernel, the second difference and the
// dissipation are one 5-point stencil per direction with the LinWeights
// weights, and the centre point's weights of the three directions are summed
// first.  Each thread sums its terms in a compensated accumulator: the FP32
// running sum, plus the exact rounding errors and product tails in a second
// FP32 word, normalised once at the end, so that the result carries an error
// of a few units of 2^-48 of the largest partial sum (compare 2^-53 for the
// FP64 kernel).  The sweeps read the result as their double-float b.

// Running sum s with its compensation c (the sum is s + c).
struct DAcc {
  float s, c;
};

__device__ __forceinline__ void acc_exact(DAcc& a, float p) {  // a += p, the rounding error into c
  const float s = __fadd_rn(a.s, p);
  const float bb = __fsub_rn(s, a.s);
  const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  a.c = __fadd_rn(a.c, err);
  a.s = s;
}
// a += w * x (w, x double-float): the FP32 product to s, its exact rounding
// error and the two cross terms to c (w.lo * x.lo is below 2^-48)
// (WX: w.lo is negligible and left out)
template <bool WX = false>
__device__ __forceinline__ void acc_mul(DAcc& a, float2 w, float2 x) {
  const float p = __fmul_rn(w.x, x.x);
  a.c = __fadd_rn(a.c, __fmaf_rn(w.x, x.x, -p));
  a.c = __fmaf_rn(w.x, x.y, a.c);
  if (!WX) a.c = __fmaf_rn(w.y, x.x, a.c);
  acc_exact(a, p);
}
// a - b and a + b of double-float values: the rounded FP32 difference (sum)
// of the high words, its exact error plus the low words' difference (sum) in
// the second word (not renormalised)
__device__ __forceinline__ float2 df_diff(float2 a, float2 b) {
  const float s = __fsub_rn(a.x, b.x);
  const float bb = __fsub_rn(s, a.x);
  const float err = __fsub_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fadd_rn(b.x, bb));
  return make_float2(s, __fadd_rn(err, __fsub_rn(a.y, b.y)));
}
__device__ __forceinline__ float2 df_sum(float2 a, float2 b) {
  const float s = __fadd_rn(a.x, b.x);
  const float bb = __fsub_rn(s, a.x);
  const float err = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
  return make_float2(s, __fadd_rn(err, __fadd_rn(a.y, b.y)));
}
__device__ __forceinline__ void acc_add(DAcc& a, float2 x) {  // a += x
  a.c = __fadd_rn(a.c, x.y);
  acc_exact(a, x.x);
}
__device__ __forceinline__ void acc_sub2(DAcc& a, float2 x) {  // a -= 2x (exact scaling)
  a.c = __fmaf_rn(-2.f, x.y, a.c);
  acc_exact(a, __fmul_rn(-2.f, x.x));
}


// sqrt(a), a > 0: FP32 estimate x, a - x^2 formed exactly to first order,
// then x + (a - x^2) / (2x).
__device__ __forceinline__ df64 df_sqrt(df64 a) {
  const float x = __fsqrt_rn(a.hi);
  const float p = __fmul_rn(x, x);
  const float pe = __fmaf_rn(x, x, -p);
  const float d = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), pe), a.lo);
  return df_quick(x, __fmul_rn(d, __frcp_rn(__fmul_rn(2.f, x))));
}

// ---- primitive kernel --------------------------------------------------------
// Per point: u in double-float (exact split), 1/rho, the velocities, square
// and qs (src/BT/rhs.jl:62-77; SP src/SP/rhs.jl:62-89 with the speed of
// sound), the point functions of compute_rhs, the FP32 state pairs of the
// sweeps, and the FP64 prim planes that are read in FP64.  The x-line-major
// copies of the state pairs come from k_xline_copy.
template <bool SP>
__device__ __forceinline__ void prim_df_point(const Fields& F, const RhsDfConsts& C, int64_t p) {
  const int64_t NP = F.NP;
  df64 u[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    split_df(F.u[m * NP + p], u[m].hi, u[m].lo);
    F.ud[m * NP + p] = df2f(u[m]);
  }
  const df64 ri = df_rcp(u[0]);
  const df64 us = df_mul(u[1], ri), vs = df_mul(u[2], ri), ws = df_mul(u[3], ri);
  const df64 square = df_half(df_add(df_add(df_mul(u[1], us), df_mul(u[2], vs)), df_mul(u[3], ws)));
  const df64 qs = df_mul(square, ri);
  health_check(F, p, u[0].hi, df_sub(u[4], square).hi);
  {
    float2* X = F.xd;
    const df64 c1 = f2df(C.c1), c2 = f2df(C.c2);
    const df64 press = df_mul(c2, df_sub(u[4], square));
    const df64 h = df_sub(df_mul(c1, u[4]), df_mul(c2, square));
    const df64 e = df_mul(u[4], ri);
    X[PX_UV * NP + p] = df2f(df_mul(u[2], us));
    X[PX_UW * NP + p] = df2f(df_mul(u[3], us));
    X[PX_VW * NP + p] = df2f(df_mul(u[3], vs));
    X[PX_XX * NP + p] = df2f(df_add(df_mul(u[1], us), press));
    X[PX_YY * NP + p] = df2f(df_add(df_mul(u[2], vs), press));
    X[PX_ZZ * NP + p] = df2f(df_add(df_mul(u[3], ws), press));
    X[PX_EX * NP + p] = df2f(df_mul(h, us));
    X[PX_EY * NP + p] = df2f(df_mul(h, vs));
    X[PX_EZ * NP + p] = df2f(df_mul(h, ws));
    const df64 vel[3] = {us, vs, ws};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const df64 wv = df_add(df_add(df_mul(f2df(C.con3[d]), qs), df_mul(f2df(C.con4[d]), df_mul(vel[d], vel[d]))),
                             df_mul(f2df(C.con5[d]), e));
      X[(PX_WX + d) * NP + p] = df2f(wv);
      X[(XD_US + d) * NP + p] = df2f(vel[d]);
    }
    if (SP) X[XD_QS * NP + p] = df2f(qs);
  }
  if (SP) {
    const df64 speed = df_sqrt(df_mul(f2df(C.c1c2), df_mul(ri, df_sub(u[4], square))));
    const df64 v[PS_HI_COUNT] = {ri, us, vs, ws, speed};
#pragma unroll
    for (int e = 0; e < PS_HI_COUNT; ++e) {
      F.primf[e * NP + p] = v[e].hi;
      F.primf[(PS_HI_COUNT + e) * NP + p] = v[e].lo;
    }
    if (F.prim64) {  // the FP64 SP sweeps of single phases read these
      F.prim[PR_US * NP + p] = df_to_double(us);
      F.prim[PR_VS * NP + p] = df_to_double(vs);
      F.prim[PR_WS * NP + p] = df_to_double(ws);
      F.prim[PR_QS * NP + p] = df_to_double(qs);
      F.prim[PR_SPEED * NP + p] = df_to_double(speed);
      F.prim[PR_AINV * NP + p] = df_to_double(df_rcp(speed));
    }
  } else {
    const df64 v[PF_HI_COUNT] = {ri, qs, u[1], u[2], u[3], u[4]};
#pragma unroll
    for (int e = 0; e < PF_HI_COUNT; ++e) {
      F.primf[e * NP + p] = v[e].hi;
      F.primf[(PF_HI_COUNT + e) * NP + p] = v[e].lo;
    }
  }
  if (F.prim64) {
    F.prim[PR_RHOI * NP + p] = df_to_double(ri);
    F.prim[PR_SQUARE * NP + p] = df_to_double(square);
    if (!SP) {
      F.prim[PR_US * NP + p] = df_to_double(us);
      F.prim[PR_VS * NP + p] = df_to_double(vs);
      F.prim[PR_WS * NP + p] = df_to_double(ws);
      F.prim[PR_QS * NP + p] = df_to_double(qs);
    }
  }
}

template <bool SP>
__global__ void __launch_bounds__(128) k_prim_df(Fields F, RhsDfConsts C, const Work* __restrict__ work, int nwork) {
  for (int it = blockIdx.x; it < nwork; it += gridDim.x) {
    const Work w = work[it];
    const ZoneDev Z = F.zones[w.zone];
    const int q = w.first + threadIdx.x;
    if (q >= Z.nx * Z.ny * Z.nz) continue;
    prim_df_point<SP>(F, C, Z.off + q);
  }
}

// ---- compute_rhs -------------------------------------------------------------
// One direction (stride st, position q of n): the stencil's four off-centre
// points (weights W), the differences of the normal momentum and the fluxes
// (-t2), the sums of the velocities' off-centre points (vc) and the viscous
// energy term (1, -2, 1).  WX: the low words of the weights and t2 are left
// out (RhsDfConsts::exact_w).
template <bool WX>
__device__ __forceinline__ void rhs_dir_df(DAcc a[5], const float2* __restrict__ ud, int64_t NP, int64_t p, int64_t st,
                                           int q, int n, const float2* __restrict__ W, const float2* const fx[4],
                                           const float2* __restrict__ un, const float2* const vel[3],
                                           const float2 vc[3], const float2* __restrict__ wv, float2 t2) {
  const int64_t pm2 = q >= 2 ? p - 2 * st : p;  // weight 0 there
  const int64_t pp2 = q + 2 <= n - 1 ? p + 2 * st : p;
  const float2 w0 = W[0], w1 = W[1], w3 = W[3], w4 = W[4];
  const float2 mt2 = make_float2(-t2.x, -t2.y);
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    const float2* um = ud + m * NP;
    acc_mul<WX>(a[m], w1, um[p - st]);
    acc_mul<WX>(a[m], w3, um[p + st]);
    acc_mul<WX>(a[m], w0, um[pm2]);
    acc_mul<WX>(a[m], w4, um[pp2]);
  }
  acc_mul<WX>(a[0], mt2, df_diff(un[p + st], un[p - st]));
#pragma unroll
  for (int m = 0; m < 4; ++m) acc_mul<WX>(a[m + 1], mt2, df_diff(fx[m][p + st], fx[m][p - st]));
#pragma unroll
  for (int m = 0; m < 3; ++m) acc_mul(a[m + 1], vc[m], df_sum(vel[m][p + st], vel[m][p - st]));
  acc_add(a[4], wv[p + st]);
  acc_add(a[4], wv[p - st]);
  acc_sub2(a[4], wv[p]);
}

// One thread per interior point; TX: txinvr after *dt (SP); NORM: this CTA's
// sum of rhs^2 (before txinvr) into partials[item][5]; WX: the low words of
// the stencil weights and t2 are left out (RhsDfConsts::exact_w).
template <bool TX, bool NORM, bool WX>
__global__ void __launch_bounds__(128) k_rhs_df(Fields F, RhsDfConsts C, const Work* __restrict__ work, int nwork,
                                                double* __restrict__ partials) {
  __shared__ double red[NORM ? 5 * 128 : 1];
  __shared__ float2 wt[3 * 32 * 5];
  for (int e = threadIdx.x; e < 3 * 32 * 5; e += blockDim.x) wt[e] = (&C.w[0][0][0])[e];
  __syncthreads();
  for (int it = blockIdx.x; it < nwork; it += gridDim.x) {
    const Work w = work[it];
    const ZoneDev Z = F.zones[w.zone];
    const int64_t NP = F.NP;
    const int ix = Z.nx - 2, iy = Z.ny - 2;
    const int ni = ix * iy * (Z.nz - 2);
    const int t = w.first + threadIdx.x;
    double sq[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (t < ni) {
      const int i = 1 + t % ix, j = 1 + (t / ix) % iy, k = 1 + t / (ix * iy);
      const int64_t p = Z.off + ((int64_t)k * Z.ny + j) * Z.nx + i;
      const float2* __restrict__ ud = F.ud;
      const float2* __restrict__ X = F.xd;
      const float2* vel[3] = {X + XD_US * NP, X + XD_VS * NP, X + XD_WS * NP};
      DAcc a[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        const float2 f = F.fd[m * NP + p];
        a[m] = DAcc{f.x, f.y};
      }
      const float2* Wx = wt + (0 * 32 + dissip_class(i, Z.nx)) * 5;
      const float2* Wy = wt + (1 * 32 + dissip_class(j, Z.ny)) * 5;
      const float2* Wz = wt + (2 * 32 + dissip_class(k, Z.nz)) * 5;
      {
        const float2* fx[4] = {X + PX_XX * NP, X + PX_UV * NP, X + PX_UW * NP, X + PX_EX * NP};
        rhs_dir_df<WX>(a, ud, NP, p, 1, i, Z.nx, Wx, fx, ud + NP, vel, C.vc[0], X + PX_WX * NP, C.t2[0]);
      }
      {
        const float2* fx[4] = {X + PX_UV * NP, X + PX_YY * NP, X + PX_VW * NP, X + PX_EY * NP};
        rhs_dir_df<WX>(a, ud, NP, p, Z.nx, j, Z.ny, Wy, fx, ud + 2 * NP, vel, C.vc[1], X + PX_WY * NP, C.t2[1]);
      }
      {
        const float2* fx[4] = {X + PX_UW * NP, X + PX_VW * NP, X + PX_ZZ * NP, X + PX_EZ * NP};
        rhs_dir_df<WX>(a, ud, NP, p, (int64_t)Z.nx * Z.ny, k, Z.nz, Wz, fx, ud + 3 * NP, vel, C.vc[2], X + PX_WZ * NP,
                   C.t2[2]);
      }
      // centre point: the three directions' weights summed first
      const float2 wc = df2f(df_add(df_add(f2df(Wx[2]), f2df(Wy[2])), f2df(Wz[2])));
#pragma unroll
      for (int m = 0; m < 5; ++m) acc_mul(a[m], wc, ud[m * NP + p]);
#pragma unroll
      for (int m = 0; m < 3; ++m) acc_mul(a[m + 1], C.vcc[m], vel[m][p]);
      df64 r[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) r[m] = df_mul(df_two_sum(a[m].s, a[m].c), f2df(C.dt));
      if (NORM)
#pragma unroll
        for (int m = 0; m < 5; ++m) {
          const double v = df_to_double(r[m]);
          sq[m] = v * v;
        }
      if (TX) {
        // txinvr (src/SP/txinvr.jl:28-49)
        const float* pf = F.primf;
        const df64 ru1 = {pf[PS_RHOI * NP + p], pf[(PS_HI_COUNT + PS_RHOI) * NP + p]};
        const df64 ac = {pf[PS_SPEED * NP + p], pf[(PS_HI_COUNT + PS_SPEED) * NP + p]};
        const df64 uu = f2df(vel[0][p]), vv = f2df(vel[1][p]), ww = f2df(vel[2][p]);
        const df64 qs = f2df(X[XD_QS * NP + p]);
        const df64 ac2inv = df_rcp(df_mul(ac, ac));
        const df64 r1 = r[0], r2 = r[1], r3 = r[2], r4 = r[3], r5 = r[4];
        df64 s = df_sub(df_mul(qs, r1), df_mul(uu, r2));
        s = df_sub(s, df_mul(vv, r3));
        s = df_add(df_sub(s, df_mul(ww, r4)), r5);
        const df64 t1 = df_mul(df_mul(f2df(C.c2), ac2inv), s);
        const df64 btru1 = df_mul(f2df(C.bt), ru1);
        const df64 t2 = df_mul(btru1, df_sub(df_mul(uu, r1), r2));
        const df64 t3 = df_mul(df_mul(btru1, ac), t1);
        r[0] = df_sub(r1, t1);
        r[1] = df_neg(df_mul(ru1, df_sub(df_mul(ww, r1), r4)));
        r[2] = df_mul(ru1, df_sub(df_mul(vv, r1), r3));
        r[3] = df_sub(t3, t2);
        r[4] = df_add(t2, t3);
      }
      if (F.rhs64)
#pragma unroll
        for (int m = 0; m < 5; ++m) F.rhs[m * NP + p] = df_to_double(r[m]);
      if (F.rdx) {  // b of the x sweep, x-line-major
        const int64_t xl = xline_of(Z, j, k);
#pragma unroll
        for (int m = 0; m < 5; ++m) {
          F.rdx[((int64_t)i * 10 + m) * F.nlx + xl] = r[m].hi;
          F.rdx[((int64_t)i * 10 + 5 + m) * F.nlx + xl] = r[m].lo;
        }
      } else {
#pragma unroll
        for (int m = 0; m < 5; ++m) {
          F.rdf[m * NP + p] = r[m].hi;
          F.rdf[(5 + m) * NP + p] = r[m].lo;
        }
      }
    }
    if (NORM) {
      block_sum5(sq, red);
      if (threadIdx.x == 0)
        for (int m = 0; m < 5; ++m) partials[it * 5 + m] = sq[m];
    }
  }
}

// ---- x-line-major copies of the state pairs ---------------------------------
// The x sweep gives each thread one x line, so that a warp's lines sit nx
// points apart in the zone layout; it reads x-line-major copies of the FP32
// state pairs instead (plane e of point i of line g at [(i * E + e) * nlx +
// g]).  This kernel makes them for the lines of each x-sweep work item (lpi
// lines of one zone from `first`, every point of each line): 32-line x
// 32-point tiles of PB planes at a time go through shared memory, so that
// the zone-layout reads (along i) and the x-line-major writes (along g) are
// both coalesced, with 4 * PB loads in flight per thread.
// Shared tile of PB planes (default: half of the E planes per pass).
template <bool SP, int PBV = 0>
struct XlineTile {
  static constexpr int E = SP ? (int)PS_COUNT : (int)PF_COUNT;
  static constexpr int PB = PBV ? PBV : E / 2;
  float t[PB][32][33];
};

// One work item of the copy, by a CTA of NW warps: the 32 rows of a tile in
// 32 / (4 NW) passes of 4 rows per thread, 4 PB loads in flight per thread.
template <bool SP, int NW, int PBV = 0>
__device__ __forceinline__ void xline_copy_item(const Fields& F, const Work w, int lpi, XlineTile<SP, PBV>& T) {
  constexpr int E = XlineTile<SP, PBV>::E, PB = XlineTile<SP, PBV>::PB, R = 4, PASSES = 32 / (R * NW);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int64_t NP = F.NP;
  const ZoneDev Z = F.zones[w.zone];
  const int l1 = min(w.first + lpi, zone_lines(Z, 0));
  const int iy = Z.ny - 2;
  for (int l0 = w.first; l0 < l1; l0 += 32)
    for (int i0 = 0; i0 < Z.nx; i0 += 32)
#pragma unroll 1
      for (int e0 = 0; e0 < E; e0 += PB) {
#pragma unroll 1
        for (int h = 0; h < PASSES; ++h) {
          float v[PB][R];
#pragma unroll
          for (int r = 0; r < R; ++r) {  // row ty + NW (R h + r): a line, column tx: point i0 + tx
            const int l = l0 + ty + NW * (R * h + r), i = i0 + tx;
            const bool ok = l < l1 && i < Z.nx;
            const int64_t p = ok ? Z.off + ((int64_t)(1 + l / iy) * Z.ny + 1 + l % iy) * Z.nx + i : 0;
#pragma unroll
            for (int b = 0; b < PB; ++b) v[b][r] = ok ? F.primf[(int64_t)(e0 + b) * NP + p] : 0.f;
          }
#pragma unroll
          for (int b = 0; b < PB; ++b)
#pragma unroll
            for (int r = 0; r < R; ++r) T.t[b][ty + NW * (R * h + r)][tx] = v[b][r];
        }
        __syncthreads();
#pragma unroll 1
        for (int h = 0; h < PASSES; ++h)
#pragma unroll
          for (int r = 0; r < R; ++r) {  // point i0 + ty + NW (R h + r) of line l0 + tx
            const int i = i0 + ty + NW * (R * h + r), l = l0 + tx;
            if (l < l1 && i < Z.nx)
#pragma unroll
              for (int b = 0; b < PB; ++b)
                F.pfx[((int64_t)i * E + e0 + b) * F.nlx + Z.lineoff[0] + l] = T.t[b][tx][ty + NW * (R * h + r)];
          }
        __syncthreads();
      }
}

template <bool SP>
__global__ void __launch_bounds__(256) k_xline_copy(Fields F, const Work* __restrict__ work, int nwork, int lpi) {
  __shared__ XlineTile<SP> tile;
  for (int it = blockIdx.x; it < nwork; it += gridDim.x) xline_copy_item<SP, 8>(F, work[it], lpi, tile);
}

// compute_rhs (k_rhs_flux) and the x-line-major state copies (k_xline_copy)
// in one launch: both read what the primitive kernel wrote, and the copy's
// memory traffic runs beside compute_rhs, which the FP64 pipe binds.  The
// copy's tile holds 2 planes (8.4 KB): with half the planes per pass (25 KB)
// the BT-C step graph ran 3.22 ms per step against 3.08 ms.  Item b
// of the nwork + ncopy is a copy item when (b + 1) is a multiple of s = total
// / ncopy (the copies spread evenly over the launch), otherwise the compute_rhs
// item b minus the copies before it.
template <bool TX, bool NORM>
__global__ void __launch_bounds__(128) k_rhs_flux_xc(Fields F, Consts K, RhsF64Consts RC, const Work* __restrict__ work,
                                                     int nwork, double* __restrict__ partials,
                                                     const Work* __restrict__ cwork, int ncopy, int lpi) {
  __shared__ double red[NORM ? 5 * 128 : 1];
  __shared__ double wt[3 * 32 * 5];
  __shared__ XlineTile<TX, 2> tile;
  for (int e = threadIdx.x; e < 3 * 32 * 5; e += blockDim.x) wt[e] = (&RC.w[0][0][0])[e];
  __syncthreads();
  const int total = nwork + ncopy;
  const int s = ncopy > 0 ? total / ncopy : total + 1;
  for (int b = blockIdx.x; b < total; b += gridDim.x) {
    const int q = (b + 1) / s;
    if ((b + 1) % s == 0 && q <= ncopy) {
      xline_copy_item<TX, 4, 2>(F, cwork[q - 1], lpi, tile);
    } else {
      const int it = b - min(ncopy, b / s);
      rhs_flux_item<TX, NORM>(F, K, RC, work[it], it, partials, wt, red);
    }
  }
}

// The reverse copy for the refined x sweep's result: its double-float x
// (10 planes, interior points) goes from the x-line-major rdx, where each
// thread wrote its own line, to the zone-layout rdf that the y sweep reads.
__global__ void __launch_bounds__(256) k_xline_back(Fields F, const Work* __restrict__ work, int nwork, int lpi) {
  constexpr int PB = 5;
  __shared__ float tile[PB][32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 8 warps
  const int64_t NP = F.NP;
  for (int it = blockIdx.x; it < nwork; it += gridDim.x) {
    const Work w = work[it];
    const ZoneDev Z = F.zones[w.zone];
    const int l1 = min(w.first + lpi, zone_lines(Z, 0));
    const int iy = Z.ny - 2;
    for (int l0 = w.first; l0 < l1; l0 += 32)
      for (int i0 = 1; i0 < Z.nx - 1; i0 += 32)
#pragma unroll 1
        for (int e0 = 0; e0 < 10; e0 += PB) {
          float v[PB][4];
#pragma unroll
          for (int r4 = 0; r4 < 4; ++r4) {  // row ty + 8 r4: point i0 + row, column tx: line l0 + tx
            const int i = i0 + ty + 8 * r4, l = l0 + tx;
            const bool ok = l < l1 && i < Z.nx - 1;
#pragma unroll
            for (int b = 0; b < PB; ++b)
              v[b][r4] = ok ? F.rdx[((int64_t)i * 10 + e0 + b) * F.nlx + Z.lineoff[0] + l] : 0.f;
          }
#pragma unroll
          for (int b = 0; b < PB; ++b)
#pragma unroll
            for (int r4 = 0; r4 < 4; ++r4) tile[b][ty + 8 * r4][tx] = v[b][r4];
          __syncthreads();
#pragma unroll
          for (int r4 = 0; r4 < 4; ++r4) {  // line l0 + ty + 8 r4, point i0 + tx
            const int l = l0 + ty + 8 * r4, i = i0 + tx;
            if (l < l1 && i < Z.nx - 1) {
              const int64_t p = Z.off + ((int64_t)(1 + l / iy) * Z.ny + 1 + l % iy) * Z.nx + i;
#pragma unroll
              for (int b = 0; b < PB; ++b) F.rdf[(int64_t)(e0 + b) * NP + p] = tile[b][tx][ty + 8 * r4];
            }
          }
          __syncthreads();
        }
  }
}

// dst[m][p] = {rn(v), rn(v - rn(v))} of src[m][p] (5 planes)
__global__ void __launch_bounds__(256) k_split_f2(const double* __restrict__ src, float2* __restrict__ dst, int64_t NP) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < 5 * NP; t += (int64_t)gridDim.x * blockDim.x) {
    float hi, lo;
    split_df(src[t], hi, lo);
    dst[t] = make_float2(hi, lo);
  }
}
