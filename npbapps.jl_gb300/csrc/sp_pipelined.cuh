// sp_pipelined.cuh -- refined FP32 SP sweep of a fused step (mode 4), included
// by step_kernels.cuh in the FMA build.
//
// The same three pentadiagonal systems per line as k_sp_solve (lhsx / lhsy /
// lhsz assembly, src/SP/lhsx.jl:27-111; Thomas elimination and back
// substitution, src/SP/x_solve.jl:203-313,456-512), solved as
//   pass 1: L x0 = b in FP32 (bands from the FP32 state copies);
//   pass 2: r = b - L x0 with the bands assembled in double-float from the
//           FP32 pairs of the state, L d = r in FP32, x = x0 + d,
// so that no FP64 arithmetic runs except in the z sweep's output: add
// (src/SP/add.jl:14-23) in FP64, after tzetar (src/SP/tzetar.jl:27-52) in
// FP64 from the FP64 primitives, or in double-float from the double-float
// ones of the double-float compute_rhs (NPBMZ_RHS_DF).  The x and y sweeps hand
// their transformed results (ninvr, src/SP/ninvr.jl:19-32; pinvr,
// src/SP/pinvr.jl:20-33, applied in double-float) to the next sweep as
// double-float planes.  Each thread streams its line's data PIPE points ahead
// with cp.async into a ring in shared memory, in both passes' forward
// elimination and back substitution; the x sweep reads its x-line-major copies.

// words per ring slot
constexpr int PLS_MIXED_W = 11;   // forward: state of q+1 (3) + b_q (5); back: l4, l5 of 3 systems + r' (11)
constexpr int PLS_REFINE_W = 26;  // forward: state pairs of q+1 (6) + x_{q+2} (10) + b_q pair (10); back: 11 + x0 (5)
constexpr int PLS_Z64 = 11;       // z refinement, FP64 words per slot: u (5) + us, vs, ws, speed, ainv, qs

__host__ __device__ constexpr size_t pls_mixed_smem(int tpb) { return (size_t)PIPE * PLS_MIXED_W * tpb * sizeof(float); }
__host__ __device__ constexpr size_t pls_refine_smem(int tpb, bool out_df) {
  return (size_t)PIPE * PLS_Z64 * tpb * sizeof(double) * (out_df ? 0 : 1) +
         (size_t)PIPE * PLS_REFINE_W * tpb * sizeof(float);
}

// Double-float constants of one SP sweep direction.
struct SpDfK {
  df64 dtt1, dtt2, c2dtt1, comz1, comz4, comz5, comz6, c3c4, con43, c1c5, da, db, dm, dc, bt;
};

template <int DIR>
__device__ __forceinline__ SpDfK sp_df_consts(const Consts& K) {
  SpDfK c;
  c.dtt1 = f2df(K.p_dtt1[DIR]);
  c.dtt2 = f2df(K.p_dtt2[DIR]);
  c.c2dtt1 = f2df(K.p_c2dtt1[DIR]);
  c.comz1 = f2df(K.p_comz1);
  c.comz4 = f2df(K.p_comz4);
  c.comz5 = f2df(K.p_comz5);
  c.comz6 = f2df(K.p_comz6);
  c.c3c4 = f2df(K.p_c3c4);
  c.con43 = f2df(K.p_con43);
  c.c1c5 = f2df(K.p_c1c5);
  c.da = f2df(K.p_d[DIR][DIR + 1]);
  c.db = f2df(K.p_d[DIR][4]);
  c.dm = f2df(K.p_dmax[DIR]);
  c.dc = f2df(K.p_d[DIR][0]);
  c.bt = f2df(K.p_bt);
  return c;
}

__device__ __forceinline__ df64 df_max(df64 a, df64 b) {
  return (a.hi > b.hi || (a.hi == b.hi && a.lo >= b.lo)) ? a : b;
}
// a * b with b an FP32 value (exact in double-float)
__device__ __forceinline__ df64 df_mulf(df64 a, float b) {
  const float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  return df_quick(p, e);
}
__device__ __forceinline__ df64 df_half(df64 a) { return {0.5f * a.hi, 0.5f * a.lo}; }  // exact

// rhon, the viscous factor of the band assembly, in double-float
// (fmax(fmax(fmax(da + con43 ru1, db + c1c5 ru1), dm + ru1), dc), ru1 = c3c4 ri).
__device__ __forceinline__ df64 sp_rhon_df(const SpDfK& c, df64 ri) {
  const df64 ru1 = df_mul(c.c3c4, ri);
  const df64 a = df_add(c.da, df_mul(c.con43, ru1));
  const df64 b = df_add(c.db, df_mul(c.c1c5, ru1));
  const df64 d = df_add(c.dm, ru1);
  return df_max(df_max(df_max(a, b), d), c.dc);
}

// Bands of interior row q (1..n-2) of the three systems in double-float from
// cv, rhon and speed at q-1, q, q+1 (the statements of sp_assemble).
__device__ __forceinline__ void sp_assemble_df(const SpDfK& c, int q, int n, const df64 cv[3], const df64 rh[3],
                                               const df64 sp[3], df64 L[3][5]) {
  const df64 z = {0.f, 0.f};
  df64 L1 = z;
  df64 L2 = df_sub(df_neg(df_mul(c.dtt2, cv[0])), df_mul(c.dtt1, rh[0]));
  df64 L3 = df_add(df64{1.f, 0.f}, df_mul(c.c2dtt1, rh[1]));
  df64 L4 = df_sub(df_mul(c.dtt2, cv[2]), df_mul(c.dtt1, rh[2]));
  df64 L5 = z;
  if (q == 1) { L3 = df_add(L3, c.comz5); L4 = df_sub(L4, c.comz4); L5 = df_add(L5, c.comz1); }
  if (q == 2) { L2 = df_sub(L2, c.comz4); L3 = df_add(L3, c.comz6); L4 = df_sub(L4, c.comz4); L5 = df_add(L5, c.comz1); }
  if (q >= 3 && q <= n - 4) {
    L1 = df_add(L1, c.comz1); L2 = df_sub(L2, c.comz4); L3 = df_add(L3, c.comz6); L4 = df_sub(L4, c.comz4);
    L5 = df_add(L5, c.comz1);
  }
  if (q == n - 3) { L1 = df_add(L1, c.comz1); L2 = df_sub(L2, c.comz4); L3 = df_add(L3, c.comz6); L4 = df_sub(L4, c.comz4); }
  if (q == n - 2) { L1 = df_add(L1, c.comz1); L2 = df_sub(L2, c.comz4); L3 = df_add(L3, c.comz5); }
  const df64 s0 = df_mul(c.dtt2, sp[0]), s2 = df_mul(c.dtt2, sp[2]);
  L[0][0] = L1; L[0][1] = L2; L[0][2] = L3; L[0][3] = L4; L[0][4] = L5;
  L[1][0] = L1; L[1][1] = df_sub(L2, s0); L[1][2] = L3; L[1][3] = df_add(L4, s2); L[1][4] = L5;
  L[2][0] = L1; L[2][1] = df_add(L2, s0); L[2][2] = L3; L[2][3] = df_sub(L4, s2); L[2][4] = L5;
}

// FP32 Thomas elimination state of the three systems (rows p and p+1).
struct SpElim {
  float cur3[3], cur4[3], cur5[3], nx2[3], nx3[3], nx4[3], nx5[3];
  float rr[2][5];
};

// Eliminate with row p+2 (bands L2, rhs r2): the loop body of sp_forward_f32.
// Writes l4, l5 and the eliminated rhs of row p to the line scratch (and, with
// sl set, to words 0..10 of this thread's ring slot, word k at sl[k * T]).
__device__ __forceinline__ void sp_elim_step(SpElim& e, int p, const float L2[3][5], const float r2[5],
                                             float* __restrict__ scr, int64_t nlt, int64_t gl,
                                             float* sl = nullptr, int T = 0) {
  float rr2[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) rr2[m] = r2[m];
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    const float fac1 = __fdividef(1.0f, e.cur3[s]);
    e.cur4[s] *= fac1;
    e.cur5[s] *= fac1;
#pragma unroll
    for (int m = SP_M0(s); m <= SP_M1(s); ++m) e.rr[0][m] *= fac1;
    e.nx3[s] -= e.nx2[s] * e.cur4[s];
    e.nx4[s] -= e.nx2[s] * e.cur5[s];
#pragma unroll
    for (int m = SP_M0(s); m <= SP_M1(s); ++m) e.rr[1][m] -= e.nx2[s] * e.rr[0][m];
    float n2 = L2[s][1], n3 = L2[s][2];
    n2 -= L2[s][0] * e.cur4[s];
    n3 -= L2[s][0] * e.cur5[s];
#pragma unroll
    for (int m = SP_M0(s); m <= SP_M1(s); ++m) rr2[m] -= L2[s][0] * e.rr[0][m];
    scr[((int64_t)p * 11 + 2 * s) * nlt + gl] = e.cur4[s];
    scr[((int64_t)p * 11 + 2 * s + 1) * nlt + gl] = e.cur5[s];
    if (sl) {
      sl[(2 * s) * T] = e.cur4[s];
      sl[(2 * s + 1) * T] = e.cur5[s];
    }
    e.cur3[s] = e.nx3[s]; e.cur4[s] = e.nx4[s]; e.cur5[s] = e.nx5[s];
    e.nx2[s] = n2; e.nx3[s] = n3; e.nx4[s] = L2[s][3]; e.nx5[s] = L2[s][4];
  }
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    scr[((int64_t)p * 11 + 6 + m) * nlt + gl] = e.rr[0][m];
    if (sl) sl[(6 + m) * T] = e.rr[0][m];
    e.rr[0][m] = e.rr[1][m];
    e.rr[1][m] = rr2[m];
  }
}

// Last two rows (n-2, n-1) of the elimination; returns the tail.
__device__ __forceinline__ void sp_elim_finish(SpElim& e, SpF32Tail& tail) {
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    const float fac1 = __fdividef(1.0f, e.cur3[s]);
    e.cur4[s] *= fac1;
    e.cur5[s] *= fac1;
#pragma unroll
    for (int m = SP_M0(s); m <= SP_M1(s); ++m) e.rr[0][m] *= fac1;
    e.nx3[s] -= e.nx2[s] * e.cur4[s];
    e.nx4[s] -= e.nx2[s] * e.cur5[s];
#pragma unroll
    for (int m = SP_M0(s); m <= SP_M1(s); ++m) e.rr[1][m] -= e.nx2[s] * e.rr[0][m];
    const float fac2 = __fdividef(1.0f, e.nx3[s]);
#pragma unroll
    for (int m = SP_M0(s); m <= SP_M1(s); ++m) e.rr[1][m] *= fac2;
    tail.cur4[s] = e.cur4[s];
  }
#pragma unroll
  for (int m = 0; m < 5; ++m) { tail.r2[m] = e.rr[0][m]; tail.rlast[m] = e.rr[1][m]; }
}

__device__ __forceinline__ void sp_elim_begin(SpElim& e, const float L0[3][5], const float r0[5], const float L1[3][5],
                                              const float r1[5]) {
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    e.cur3[s] = L0[s][2]; e.cur4[s] = L0[s][3]; e.cur5[s] = L0[s][4];
    e.nx2[s] = L1[s][1]; e.nx3[s] = L1[s][2]; e.nx4[s] = L1[s][3]; e.nx5[s] = L1[s][4];
  }
#pragma unroll
  for (int m = 0; m < 5; ++m) { e.rr[0][m] = r0[m]; e.rr[1][m] = r1[m]; }
}

__device__ __forceinline__ void sp_identity_rows(float L[3][5]) {
#pragma unroll
  for (int s = 0; s < 3; ++s) { L[s][0] = 0.f; L[s][1] = 0.f; L[s][2] = 1.f; L[s][3] = 0.f; L[s][4] = 0.f; }
}

// Addresses of one line's inputs: the x sweep reads x-line-major copies
// (element e of point q at [(q * E + e) * nlx + gl]), y and z the zone layout.
template <int DIR>
struct SpLine {
  const Fields* F;
  int64_t base, st, gl, NP;
  float* x0;  // zone-layout first-pass solution (y, z)
  __device__ const float* state(int q, int plane) const {  // PS planes: hi 0..4, lo 5..9
    return DIR == 0 ? F->pfx + ((int64_t)q * PS_COUNT + plane) * F->nlx + gl : F->primf + plane * NP + base + (int64_t)q * st;
  }
  __device__ const float* b(int q, int e) const {  // 0..4 hi, 5..9 lo
    return DIR == 0 ? F->rdx + ((int64_t)q * 10 + e) * F->nlx + gl : F->rdf + e * NP + base + (int64_t)q * st;
  }
  __device__ float* x0_at(int q, int m) const {
    return DIR == 0 ? F->x0x + ((int64_t)q * 5 + m) * F->nlx + gl : x0 + m * NP + base + (int64_t)q * st;
  }
};

constexpr int SP_CV = 0, SP_RI = 1, SP_SPD = 2;  // order of the state words in a slot
template <int DIR>
__device__ __forceinline__ int sp_cv_plane() { return DIR == 0 ? PS_US : DIR == 1 ? PS_VS : PS_WS; }

// ---- pass 1 -------------------------------------------------------------
template <int DIR>
__device__ __forceinline__ void sp_mixed_pl_item(const Fields& F, const Consts& K, const Work w,
                                                 float* __restrict__ scr, int64_t nlt, float* __restrict__ x0,
                                                 unsigned char* pl_smem) {
  const ZoneDev Z = F.zones[w.zone];
  const int line = w.first + threadIdx.x;
  if (line >= zone_lines(Z, DIR)) return;
  SpLine<DIR> Ln;
  Ln.F = &F;
  line_geometry(Z, DIR, line, Ln.base, Ln.st);
  Ln.gl = Z.lineoff[DIR] + line;
  Ln.NP = F.NP;
  Ln.x0 = x0;
  const int n = zone_line_len(Z, DIR);
  const int T = blockDim.x;
  float* my = reinterpret_cast<float*>(pl_smem) + threadIdx.x;
  auto S = [&](int slot, int e) -> float* { return my + (slot * PLS_MIXED_W + e) * T; };
  const int pcv = sp_cv_plane<DIR>();
  // row q consumes b_q and the state at q+1 (the bands of row q need q-1..q+1)
  auto issue_fwd = [&](int q) {
    if (q <= n - 1) {
      const int slot = q % PIPE;
      if (q + 1 <= n - 1) {
        cpa4(S(slot, SP_CV), Ln.state(q + 1, pcv));
        cpa4(S(slot, SP_RI), Ln.state(q + 1, PS_RHOI));
        cpa4(S(slot, SP_SPD), Ln.state(q + 1, PS_SPEED));
      }
#pragma unroll
      for (int m = 0; m < 5; ++m) cpa4(S(slot, 3 + m), Ln.b(q, m));
    }
    cpa_commit();
  };
  // the ring's first slots go out before the line's first point is read
  // directly, so that the two memory latencies overlap
#pragma unroll
  for (int q = 0; q < PIPE - 1; ++q) issue_fwd(q);
  float gcv[3], grh[3], gsp[3];  // geometry at q-1, q, q+1
  {
    float cv, rh, sp;
    sp_geom_t<DIR, float>(*Ln.state(0, PS_RHOI), *Ln.state(0, pcv), *Ln.state(0, PS_SPEED), K, cv, rh, sp);
    gcv[1] = cv; grh[1] = rh; gsp[1] = sp;
    gcv[0] = cv; grh[0] = rh; gsp[0] = sp;
  }
  auto row = [&](int q, float L[3][5], float r[5]) {
    cpa_wait<PIPE - 1>();
    const int slot = q % PIPE;
    if (q + 1 <= n - 1) {
      float cv, rh, sp;
      sp_geom_t<DIR, float>(*S(slot, SP_RI), *S(slot, SP_CV), *S(slot, SP_SPD), K, cv, rh, sp);
      gcv[2] = cv; grh[2] = rh; gsp[2] = sp;
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) r[m] = *S(slot, 3 + m);
    if (q == 0 || q == n - 1) sp_identity_rows(L);
    else sp_assemble<DIR, float, float>(K, q, n, gcv, grh, gsp, L);
    gcv[0] = gcv[1]; grh[0] = grh[1]; gsp[0] = gsp[1];
    gcv[1] = gcv[2]; grh[1] = grh[2]; gsp[1] = gsp[2];
  };
  SpElim e;
  {
    float L0[3][5], L1[3][5], r0[5], r1[5];
    issue_fwd(PIPE - 1);
    row(0, L0, r0);
    issue_fwd(PIPE);
    row(1, L1, r1);
    sp_elim_begin(e, L0, r0, L1, r1);
  }
  for (int p = 0; p <= n - 3; ++p) {
    float L2[3][5], r2[5];
    issue_fwd(p + 2 + PIPE - 1);
    row(p + 2, L2, r2);
    // the ring does not refill the slot row p + 2 came in: row p's words stay
    // there for the back substitution, which so starts without a trip to memory
    const bool keep = p + 2 + PIPE > n - 1;
    sp_elim_step(e, p, L2, r2, scr, nlt, Ln.gl, keep ? S((p + 2) % PIPE, 0) : nullptr, T);
  }
  SpF32Tail tail;
  sp_elim_finish(e, tail);
  cpa_wait<0>();
  // back substitution: row p (n-3 .. 1) consumes l4, l5, r' of row p from
  // slot (p + 2) % PIPE: the last rows as the forward pass left them, the
  // others loaded PIPE rows ahead into the slot just consumed
  auto issue_bwd = [&](int p) {
    if (p >= 1) {
      const int slot = (p + 2) % PIPE;
#pragma unroll
      for (int k = 0; k < 11; ++k) cpa4(S(slot, k), scr + ((int64_t)p * 11 + k) * nlt + Ln.gl);
    }
    cpa_commit();
  };
  float b1[5], b2[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    const int s = m < 3 ? 0 : m - 2;
    b2[m] = tail.rlast[m];
    b1[m] = tail.r2[m] - tail.cur4[s] * b2[m];
    *Ln.x0_at(n - 2, m) = b1[m];
  }
  for (int p = n - 3; p >= 1; --p) {
    if (p + 2 + PIPE <= n - 1) cpa_wait<PIPE - 1>();
    const int slot = (p + 2) % PIPE;
    float r[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const int s = m < 3 ? 0 : m - 2;
      r[m] = *S(slot, 6 + m) - (*S(slot, 2 * s) * b1[m] + *S(slot, 2 * s + 1) * b2[m]);
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      b2[m] = b1[m];
      b1[m] = r[m];
      *Ln.x0_at(p, m) = r[m];
    }
    issue_bwd(p - PIPE);
  }
  cpa_wait<0>();
}

template <int DIR>
__global__ void __launch_bounds__(128, NPBMZ_SP_MINB) k_sp_mixed_pl(Fields F, Consts K, const Work* __restrict__ work, int nwork,
                                                     float* __restrict__ scr, int64_t nlt, float* __restrict__ x0) {
  extern __shared__ __align__(16) unsigned char pl_smem[];
  for (int it = blockIdx.x; it < nwork; it += gridDim.x) sp_mixed_pl_item<DIR>(F, K, work[it], scr, nlt, x0, pl_smem);
}

// ---- pass 2 -------------------------------------------------------------
template <int DIR, bool OUT_DF>
__device__ __forceinline__ void sp_refine_pl_item(const Fields& F, const Consts& K, const Work w,
                                                  float* __restrict__ scr, int64_t nlt, int add_u,
                                                  float* __restrict__ x0f, unsigned char* pl_smem) {
  const ZoneDev Z = F.zones[w.zone];
  const int line = w.first + threadIdx.x;
  if (line >= zone_lines(Z, DIR)) return;
  SpLine<DIR> Ln;
  Ln.F = &F;
  line_geometry(Z, DIR, line, Ln.base, Ln.st);
  Ln.gl = Z.lineoff[DIR] + line;
  Ln.NP = F.NP;
  Ln.x0 = x0f;
  const int64_t NP = F.NP;
  const int n = zone_line_len(Z, DIR);
  const int T = blockDim.x;
  double* umy = reinterpret_cast<double*>(pl_smem) + threadIdx.x;
  float* my = reinterpret_cast<float*>(pl_smem + (OUT_DF ? 0 : (size_t)PIPE * PLS_Z64 * T * sizeof(double))) + threadIdx.x;
  auto S = [&](int slot, int e) -> float* { return my + (slot * PLS_REFINE_W + e) * T; };
  auto SU = [&](int slot, int e) -> double* { return umy + (slot * PLS_Z64 + e) * T; };
  const int pcv = sp_cv_plane<DIR>();
  const SpDfK c = sp_df_consts<DIR>(K);

  // row q consumes the state pairs at q+1 (words 0..5: cv, ri, speed hi then
  // lo), x_{q+2} (words 6..15: x0 in 6..10, or the b pair at the line's end)
  // and the b pair of q (words 16..25)
  auto issue_fwd = [&](int q) {
    if (q <= n - 1) {
      const int slot = q % PIPE;
      if (q + 1 <= n - 1) {
        cpa4(S(slot, 0), Ln.state(q + 1, pcv));
        cpa4(S(slot, 1), Ln.state(q + 1, PS_RHOI));
        cpa4(S(slot, 2), Ln.state(q + 1, PS_SPEED));
        cpa4(S(slot, 3), Ln.state(q + 1, PS_HI_COUNT + pcv));
        cpa4(S(slot, 4), Ln.state(q + 1, PS_HI_COUNT + PS_RHOI));
        cpa4(S(slot, 5), Ln.state(q + 1, PS_HI_COUNT + PS_SPEED));
      }
      const int qx = q + 2;
      if (qx == n - 1) {
#pragma unroll
        for (int k = 0; k < 10; ++k) cpa4(S(slot, 6 + k), Ln.b(qx, k));
      } else if (qx < n - 1) {
#pragma unroll
        for (int m = 0; m < 5; ++m) cpa4(S(slot, 6 + m), Ln.x0_at(qx, m));
      }
#pragma unroll
      for (int k = 0; k < 10; ++k) cpa4(S(slot, 16 + k), Ln.b(q, k));
    }
    cpa_commit();
  };
  // the ring's first slots go out before the line's first points are read
  // directly, so that the two memory latencies overlap
#pragma unroll
  for (int q = 0; q < PIPE - 1; ++q) issue_fwd(q);
  // geometry window (cv, rhon, speed at q-1, q, q+1) and x window (q-2 .. q+2)
  df64 gcv[3], grh[3], gsp[3];
  df64 xw[5][5];
  const df64 z0 = {0.f, 0.f};
  {
    const df64 cv = {*Ln.state(0, pcv), *Ln.state(0, PS_HI_COUNT + pcv)};
    const df64 ri = {*Ln.state(0, PS_RHOI), *Ln.state(0, PS_HI_COUNT + PS_RHOI)};
    const df64 sp = {*Ln.state(0, PS_SPEED), *Ln.state(0, PS_HI_COUNT + PS_SPEED)};
    const df64 rh = sp_rhon_df(c, ri);
    gcv[0] = gcv[1] = cv; grh[0] = grh[1] = rh; gsp[0] = gsp[1] = sp;
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      xw[0][m] = z0;
      xw[1][m] = z0;
      xw[2][m] = df64{*Ln.b(0, m), *Ln.b(0, 5 + m)};     // row 0 is an identity row: x = b
      xw[3][m] = df64{*Ln.x0_at(1, m), 0.f};              // n >= 3: point 1 is interior
    }
  }
  auto row = [&](int q, float L[3][5], float r[5]) {
    cpa_wait<PIPE - 1>();
    const int slot = q % PIPE;
    if (q + 1 <= n - 1) {
      gcv[2] = df64{*S(slot, 0), *S(slot, 3)};
      const df64 ri = {*S(slot, 1), *S(slot, 4)};
      grh[2] = sp_rhon_df(c, ri);
      gsp[2] = df64{*S(slot, 2), *S(slot, 5)};
    }
    const int qx = q + 2;
#pragma unroll
    for (int m = 0; m < 5; ++m)
      xw[4][m] = qx > n - 1 ? z0 : (qx == n - 1 ? df64{*S(slot, 6 + m), *S(slot, 11 + m)} : df64{*S(slot, 6 + m), 0.f});
    if (q == 0 || q == n - 1) {
      sp_identity_rows(L);
#pragma unroll
      for (int m = 0; m < 5; ++m) r[m] = 0.f;  // x = b on the identity rows: no correction
    } else {
      df64 Ld[3][5];
      sp_assemble_df(c, q, n, gcv, grh, gsp, Ld);
#pragma unroll
      for (int s = 0; s < 3; ++s)
#pragma unroll
        for (int k = 0; k < 5; ++k) L[s][k] = Ld[s][k].hi;
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        const int s = m < 3 ? 0 : m - 2;
        df64 t = df_mul(Ld[s][2], xw[2][m]);
        t = df_add(t, df_mul(Ld[s][1], xw[1][m]));
        t = df_add(t, df_mul(Ld[s][3], xw[3][m]));
        t = df_add(t, df_mul(Ld[s][0], xw[0][m]));
        t = df_add(t, df_mul(Ld[s][4], xw[4][m]));
        const df64 b = {*S(slot, 16 + m), *S(slot, 21 + m)};
        const df64 rr = df_sub(b, t);
        r[m] = rr.hi + rr.lo;
      }
    }
    gcv[0] = gcv[1]; grh[0] = grh[1]; gsp[0] = gsp[1];
    gcv[1] = gcv[2]; grh[1] = grh[2]; gsp[1] = gsp[2];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int m = 0; m < 5; ++m) xw[k][m] = xw[k + 1][m];
  };
  SpElim e;
  {
    float L0[3][5], L1[3][5], r0[5], r1[5];
    issue_fwd(PIPE - 1);
    row(0, L0, r0);
    issue_fwd(PIPE);
    row(1, L1, r1);
    sp_elim_begin(e, L0, r0, L1, r1);
  }
  // back substitution: row p (n-2 .. 1) consumes l4, l5, r' (rows <= n-3), x0
  // and, in the z sweep, u and the primitives tzetar reads, from slot
  // (p + 2) % PIPE.  issue_rest: all but l4, l5, r'
  auto issue_rest = [&](int p, int slot) {
    const int64_t pt = Ln.base + (int64_t)p * Ln.st;
#pragma unroll
    for (int m = 0; m < 5; ++m) cpa4(S(slot, 11 + m), Ln.x0_at(p, m));
      if (!OUT_DF) {
        if (add_u) {
#pragma unroll
          for (int m = 0; m < 5; ++m) cpa8(SU(slot, m), F.u + m * NP + pt);
        } else {
          cpa8(SU(slot, 0), F.u + pt);
        }
        if (F.xd) {  // double-float primitives (8-byte words: float2 pairs)
          const float2* X = F.xd;
          cpa8(SU(slot, 5), X + XD_US * NP + pt);
          cpa8(SU(slot, 6), X + XD_VS * NP + pt);
          cpa8(SU(slot, 7), X + XD_WS * NP + pt);
          float* spd = reinterpret_cast<float*>(SU(slot, 8));
          cpa4(spd, F.primf + PS_SPEED * NP + pt);
          cpa4(spd + 1, F.primf + (PS_HI_COUNT + PS_SPEED) * NP + pt);
          cpa8(SU(slot, 9), X + XD_QS * NP + pt);
          cpa8(SU(slot, 10), F.ud + pt);
        } else {
          cpa8(SU(slot, 5), F.prim + PR_US * NP + pt);
          cpa8(SU(slot, 6), F.prim + PR_VS * NP + pt);
          cpa8(SU(slot, 7), F.prim + PR_WS * NP + pt);
          cpa8(SU(slot, 8), F.prim + PR_SPEED * NP + pt);
          cpa8(SU(slot, 9), F.prim + PR_AINV * NP + pt);
          cpa8(SU(slot, 10), F.prim + PR_QS * NP + pt);
        }
      }
  };
  for (int p = 0; p <= n - 3; ++p) {
    float L2[3][5], r2[5];
    issue_fwd(p + 2 + PIPE - 1);
    row(p + 2, L2, r2);
    // rows n-1-PIPE .. n-2 stay in the slots the ring does not refill (row p
    // in the one row p + 2 came in), so that the back substitution starts
    // without a trip to memory: l4, l5, r' written here, the rest fetched now
    const bool keep = p >= n - 1 - PIPE;
    sp_elim_step(e, p, L2, r2, scr, nlt, Ln.gl, keep ? S((p + 2) % PIPE, 0) : nullptr, T);
    if (keep) {
      if (p >= 1) issue_rest(p, (p + 2) % PIPE);
      if (p == (n - 1 - PIPE > 0 ? n - 1 - PIPE : 0)) issue_rest(n - 2, n % PIPE);
      cpa_commit();
    }
  }
  SpF32Tail tail;
  sp_elim_finish(e, tail);
  cpa_wait<0>();
  // the other rows PIPE ahead into the slot just consumed
  auto issue_bwd = [&](int p) {
    if (p >= 1) {
      const int slot = (p + 2) % PIPE;
#pragma unroll
      for (int k = 0; k < 11; ++k) cpa4(S(slot, k), scr + ((int64_t)p * 11 + k) * nlt + Ln.gl);
      issue_rest(p, slot);
    }
    cpa_commit();
  };
  auto emit = [&](int p, int slot, const float d[5]) {
    const int64_t pt = Ln.base + (int64_t)p * Ln.st;
    if (OUT_DF) {
      df64 v[5], o[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) v[m] = df_two_sum(*S(slot, 11 + m), d[m]);
      const df64 t2 = df_half(df_add(v[3], v[4]));
      if (DIR == 0) {  // ninvr
        const df64 t1 = df_mul(c.bt, v[2]);
        o[0] = df_neg(v[1]); o[1] = v[0]; o[2] = df_mul(c.bt, df_sub(v[3], v[4]));
        o[3] = df_sub(t2, t1); o[4] = df_add(t1, t2);
      } else {  // pinvr
        const df64 t1 = df_mul(c.bt, v[0]);
        o[0] = df_mul(c.bt, df_sub(v[3], v[4])); o[1] = df_neg(v[2]); o[2] = v[1];
        o[3] = df_sub(t2, t1); o[4] = df_add(t1, t2);
      }
      // x: in place of b in the x-line-major copy (k_xline_back moves it
      // to rdf); y: rdf
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        float* dst = DIR == 0 ? F.rdx + ((int64_t)p * 10 + m) * F.nlx + Ln.gl : F.rdf + m * NP + pt;
        const int64_t lo_off = DIR == 0 ? 5 * F.nlx : 5 * NP;
        dst[0] = o[m].hi;
        dst[lo_off] = o[m].lo;
      }
    } else if (F.xd) {  // tzetar in double-float, then add in FP64
      df64 r[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) r[m] = df_two_sum(*S(slot, 11 + m), d[m]);
      auto w2 = [&](int e) -> df64 { const float* q = reinterpret_cast<const float*>(SU(slot, e)); return {q[0], q[1]}; };
      const df64 xvel = w2(5), yvel = w2(6), zvel = w2(7), ac = w2(8), qs = w2(9), uzik1 = w2(10);
      const df64 acinv = df_rcp(ac);
      const df64 btuz = df_mul(f2df(K.p_bt), uzik1);
      const df64 t1 = df_mul(df_mul(btuz, acinv), df_add(r[3], r[4]));
      const df64 t2 = df_add(r[2], t1);
      const df64 t3 = df_mul(btuz, df_sub(r[3], r[4]));
      df64 o[5];
      o[0] = t2;
      o[1] = df_add(df_neg(df_mul(uzik1, r[1])), df_mul(xvel, t2));
      o[2] = df_add(df_mul(uzik1, r[0]), df_mul(yvel, t2));
      o[3] = df_add(df_mul(zvel, t2), t3);
      o[4] = df_add(df_add(df_mul(uzik1, df_sub(df_mul(yvel, r[0]), df_mul(xvel, r[1]))), df_mul(qs, t2)),
                    df_add(df_mul(df_mul(f2df(K.p_c2iv), df_mul(ac, ac)), t1), df_mul(zvel, t3)));
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        const double v = df_to_double(o[m]);
        F.rhs[m * NP + pt] = v;
        if (add_u) F.u[m * NP + pt] = *SU(slot, m) + v;
      }
    } else {  // tzetar in FP64, then add
      double r[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) r[m] = f32_to_f64(*S(slot, 11 + m)) + f32_to_f64(d[m]);  // exact, by bits
      const double xvel = *SU(slot, 5), yvel = *SU(slot, 6), zvel = *SU(slot, 7);
      const double ac = *SU(slot, 8), acinv = *SU(slot, 9), qs = *SU(slot, 10);
      const double ac2u = ac * ac;
      const double uzik1 = *SU(slot, 0);
      const double btuz = K.bt * uzik1;
      const double t1 = btuz * acinv * (r[3] + r[4]);
      const double t2 = r[2] + t1;
      const double t3 = btuz * (r[3] - r[4]);
      double o[5];
      o[0] = t2;
      o[1] = -uzik1 * r[1] + xvel * t2;
      o[2] = uzik1 * r[0] + yvel * t2;
      o[3] = zvel * t2 + t3;
      o[4] = uzik1 * (-xvel * r[1] + yvel * r[0]) + qs * t2 + K.c2iv * ac2u * t1 + zvel * t3;
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        F.rhs[m * NP + pt] = o[m];
        if (add_u) F.u[m * NP + pt] = *SU(slot, m) + o[m];
      }
    }
  };
  float b1[5], b2[5];
  {
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const int s = m < 3 ? 0 : m - 2;
      b2[m] = tail.rlast[m];
      b1[m] = tail.r2[m] - tail.cur4[s] * b2[m];
    }
    emit(n - 2, n % PIPE, b1);
    issue_bwd(n - 2 - PIPE);
  }
  for (int p = n - 3; p >= 1; --p) {
    if (p <= n - 2 - PIPE) cpa_wait<PIPE - 1>();
    const int slot = (p + 2) % PIPE;
    float r[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const int s = m < 3 ? 0 : m - 2;
      r[m] = *S(slot, 6 + m) - (*S(slot, 2 * s) * b1[m] + *S(slot, 2 * s + 1) * b2[m]);
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) { b2[m] = b1[m]; b1[m] = r[m]; }
    emit(p, slot, r);
    issue_bwd(p - PIPE);
  }
  cpa_wait<0>();
}

template <int DIR, bool OUT_DF>
__global__ void __launch_bounds__(128, NPBMZ_SP_MINB) k_sp_refine_pl(Fields F, Consts K, const Work* __restrict__ work, int nwork,
                                                      float* __restrict__ scr, int64_t nlt, int add_u,
                                                      float* __restrict__ x0f) {
  extern __shared__ __align__(16) unsigned char pl_smem[];
  for (int it = blockIdx.x; it < nwork; it += gridDim.x)
    sp_refine_pl_item<DIR, OUT_DF>(F, K, work[it], scr, nlt, add_u, x0f, pl_smem);
}
