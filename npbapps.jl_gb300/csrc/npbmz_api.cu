// npbmz_api.cu -- the C ABI of libnpbmz_gpu.so (declared in include/npbmz.h):
// handle, HBM buffers, zone x point / zone x line work lists, phase
// orchestration, CUDA-graph capture of a step, norms and the autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/npbmz.h"
#include "adjoint_launch.h"
#include "common_launch.h"
#include "npbmz_internal.cuh"
#include "step_launch.h"

using namespace npbmz;

namespace {

constexpr int PTS_TPB = 128;   // points per CTA of the point kernels (power of two)

// error text of the calls without a handle, per host thread
thread_local std::string g_create_error;

Consts make_consts(double dt, int gx, int gy, int gz, int xz, int yz) {
  // set_constants, src/BT/set_constants.jl:1-130 (SP: the same file body)
  Consts k;
  std::memset(&k, 0, sizeof(k));
  k.c1 = 1.4e0; k.c2 = 0.4e0; k.c3 = 0.1e0; k.c4 = 1.0e0; k.c5 = 1.4e0;
  k.bt = std::sqrt(0.5e0);
  k.c1c2 = k.c1 * k.c2; k.c1c5 = k.c1 * k.c5; k.c3c4 = k.c3 * k.c4; k.c1345 = k.c1c5 * k.c3c4;
  k.conz1 = (1.0e0 - k.c1c5);
  k.dx1 = k.dx2 = k.dx3 = k.dx4 = k.dx5 = 0.75e0;
  k.dy1 = k.dy2 = k.dy3 = k.dy4 = k.dy5 = 0.75e0;
  k.dz1 = k.dz2 = k.dz3 = k.dz4 = k.dz5 = 1.0e0;
  k.dxmax = std::max(k.dx3, k.dx4); k.dymax = std::max(k.dy2, k.dy4); k.dzmax = std::max(k.dz2, k.dz3);
  k.dssp = 0.25e0 * std::max(k.dx1, std::max(k.dy1, k.dz1));
  k.c2iv = 2.5e0; k.con43 = 4.0e0 / 3.0e0; k.con16 = 1.0e0 / 6.0e0;
  k.dt = dt;
  k.dnxm1 = 1.0e0 / ((double)(gx - 1) / (double)xz);
  k.dnym1 = 1.0e0 / ((double)(gy - 1) / (double)yz);
  k.dnzm1 = 1.0e0 / (double)(gz - 1);
  k.tx1 = 1.0e0 / (k.dnxm1 * k.dnxm1); k.tx2 = 1.0e0 / (2.0e0 * k.dnxm1); k.tx3 = 1.0e0 / k.dnxm1;
  k.ty1 = 1.0e0 / (k.dnym1 * k.dnym1); k.ty2 = 1.0e0 / (2.0e0 * k.dnym1); k.ty3 = 1.0e0 / k.dnym1;
  k.tz1 = 1.0e0 / (k.dnzm1 * k.dnzm1); k.tz2 = 1.0e0 / (2.0e0 * k.dnzm1); k.tz3 = 1.0e0 / k.dnzm1;
  k.dttx1 = dt * k.tx1; k.dttx2 = dt * k.tx2; k.dtty1 = dt * k.ty1; k.dtty2 = dt * k.ty2;
  k.dttz1 = dt * k.tz1; k.dttz2 = dt * k.tz2;
  k.c2dttx1 = 2.0e0 * k.dttx1; k.c2dtty1 = 2.0e0 * k.dtty1; k.c2dttz1 = 2.0e0 * k.dttz1;
  const double dtdssp = dt * k.dssp;
  k.comz1 = dtdssp; k.comz4 = 4.0e0 * dtdssp; k.comz5 = 5.0e0 * dtdssp; k.comz6 = 6.0e0 * dtdssp;
  const double c3c4tx3 = k.c3c4 * k.tx3, c3c4ty3 = k.c3c4 * k.ty3, c3c4tz3 = k.c3c4 * k.tz3;
  k.dx1tx1 = k.dx1 * k.tx1; k.dx2tx1 = k.dx2 * k.tx1; k.dx3tx1 = k.dx3 * k.tx1; k.dx4tx1 = k.dx4 * k.tx1; k.dx5tx1 = k.dx5 * k.tx1;
  k.dy1ty1 = k.dy1 * k.ty1; k.dy2ty1 = k.dy2 * k.ty1; k.dy3ty1 = k.dy3 * k.ty1; k.dy4ty1 = k.dy4 * k.ty1; k.dy5ty1 = k.dy5 * k.ty1;
  k.dz1tz1 = k.dz1 * k.tz1; k.dz2tz1 = k.dz2 * k.tz1; k.dz3tz1 = k.dz3 * k.tz1; k.dz4tz1 = k.dz4 * k.tz1; k.dz5tz1 = k.dz5 * k.tz1;
  k.xxcon1 = c3c4tx3 * k.con43 * k.tx3; k.xxcon2 = c3c4tx3 * k.tx3; k.xxcon3 = c3c4tx3 * k.conz1 * k.tx3;
  k.xxcon4 = c3c4tx3 * k.con16 * k.tx3; k.xxcon5 = c3c4tx3 * k.c1c5 * k.tx3;
  k.yycon1 = c3c4ty3 * k.con43 * k.ty3; k.yycon2 = c3c4ty3 * k.ty3; k.yycon3 = c3c4ty3 * k.conz1 * k.ty3;
  k.yycon4 = c3c4ty3 * k.con16 * k.ty3; k.yycon5 = c3c4ty3 * k.c1c5 * k.ty3;
  k.zzcon1 = c3c4tz3 * k.con43 * k.tz3; k.zzcon2 = c3c4tz3 * k.tz3; k.zzcon3 = c3c4tz3 * k.conz1 * k.tz3;
  k.zzcon4 = c3c4tz3 * k.con16 * k.tz3; k.zzcon5 = c3c4tz3 * k.c1c5 * k.tz3;
  // FP32 and double-float copies for the FP32 sweeps
  auto pr = [](double v) {
    const float hi = (float)v;
    return make_float2(hi, (float)(v - (double)hi));
  };
  k.f_c1 = (float)k.c1; k.f_c2 = (float)k.c2; k.f_c3 = (float)k.c3; k.f_c4 = (float)k.c4;
  k.f_c3c4 = (float)k.c3c4; k.f_c1345 = (float)k.c1345; k.f_con43 = (float)k.con43; k.f_c1c5 = (float)k.c1c5;
  k.f_comz1 = (float)k.comz1; k.f_comz4 = (float)k.comz4; k.f_comz5 = (float)k.comz5; k.f_comz6 = (float)k.comz6;
  const double dtt1[3] = {k.dttx1, k.dtty1, k.dttz1}, dtt2[3] = {k.dttx2, k.dtty2, k.dttz2};
  const double c2dtt1[3] = {k.c2dttx1, k.c2dtty1, k.c2dttz1}, dmax[3] = {k.dxmax, k.dymax, k.dzmax};
  const double dd[3][5] = {{k.dx1, k.dx2, k.dx3, k.dx4, k.dx5}, {k.dy1, k.dy2, k.dy3, k.dy4, k.dy5},
                           {k.dz1, k.dz2, k.dz3, k.dz4, k.dz5}};
  for (int d = 0; d < 3; ++d) {
    k.f_dtt1[d] = (float)dtt1[d]; k.f_dtt2[d] = (float)dtt2[d]; k.f_c2dtt1[d] = (float)c2dtt1[d];
    k.f_dmax[d] = (float)dmax[d];
    k.p_dtt1[d] = pr(dtt1[d]); k.p_dtt2[d] = pr(dtt2[d]); k.p_c2dtt1[d] = pr(c2dtt1[d]); k.p_dmax[d] = pr(dmax[d]);
    for (int m = 0; m < 5; ++m) { k.f_d[d][m] = (float)dd[d][m]; k.p_d[d][m] = pr(dd[d][m]); }
  }
  k.p_c1 = pr(k.c1); k.p_c2 = pr(k.c2); k.p_two_m_c2 = pr(2.0 - k.c2);
  k.p_k43 = pr(k.con43 * k.c3c4); k.p_c3c4 = pr(k.c3c4); k.p_c1345 = pr(k.c1345);
  k.p_k43m = pr(k.con43 * k.c3c4 - k.c1345); k.p_c3c4m = pr(k.c3c4 - k.c1345);
  k.p_con43 = pr(k.con43); k.p_c1c5 = pr(k.c1c5); k.p_comz1 = pr(k.comz1); k.p_comz4 = pr(k.comz4);
  k.p_comz5 = pr(k.comz5); k.p_comz6 = pr(k.comz6); k.p_bt = pr(k.bt); k.p_c2iv = pr(k.c2iv);
  return k;
}

// Weights of the linear 5-point stencil of compute_rhs per direction and
// position class (see LinWeights): the second difference d*t1*(1, -2, 1) of
// x/y/z plus -dssp times the sum of the reference's dissipation stencils that
// apply at that position (src/BT/rhs.jl:124-160 and its eta/zeta copies).
// False when the d*t1 factors differ between variables of a direction.
bool make_lin_weights(const Consts& k, LinWeights& lw) {
  const double a[3][5] = {{k.dx1tx1, k.dx2tx1, k.dx3tx1, k.dx4tx1, k.dx5tx1},
                          {k.dy1ty1, k.dy2ty1, k.dy3ty1, k.dy4ty1, k.dy5ty1},
                          {k.dz1tz1, k.dz2tz1, k.dz3tz1, k.dz4tz1, k.dz5tz1}};
  static const int stencil[5][5] = {{0, 0, 5, -4, 1},    // q == 1
                                    {0, -4, 6, -4, 1},   // q == 2
                                    {1, -4, 6, -4, 1},   // 3 <= q <= n-4
                                    {1, -4, 6, -4, 0},   // q == n-3
                                    {1, -4, 5, 0, 0}};   // q == n-2
  static const double second[5] = {0.0, 1.0, -2.0, 1.0, 0.0};
  for (int d = 0; d < 3; ++d) {
    for (int m = 1; m < 5; ++m)
      if (a[d][m] != a[d][0]) return false;
    for (int c = 0; c < 32; ++c)
      for (int o = 0; o < 5; ++o) {
        int wsum = 0;
        for (int b = 0; b < 5; ++b)
          if (c >> b & 1) wsum += stencil[b][o];
        lw.w[d][c][o] = a[d][0] * second[o] - k.dssp * (double)wsum;
      }
  }
  return true;
}

// The FMA build's compute_rhs constants: every factor times dt.
void make_rhs_f64_consts(const Consts& k, const LinWeights& lw, RhsF64Consts& c) {
  for (int d = 0; d < 3; ++d)
    for (int cl = 0; cl < 32; ++cl)
      for (int o = 0; o < 5; ++o) c.w[d][cl][o] = k.dt * lw.w[d][cl][o];
  const double vc[3][3] = {{k.xxcon2 * k.con43, k.xxcon2, k.xxcon2},
                           {k.yycon2, k.yycon2 * k.con43, k.yycon2},
                           {k.zzcon2, k.zzcon2, k.zzcon2 * k.con43}};
  for (int d = 0; d < 3; ++d)
    for (int m = 0; m < 3; ++m) c.vc[d][m] = k.dt * vc[d][m];
  for (int m = 0; m < 3; ++m) c.vcc[m] = -2.0 * (c.vc[0][m] + c.vc[1][m] + c.vc[2][m]);
  c.t2[0] = k.dttx2;
  c.t2[1] = k.dtty2;
  c.t2[2] = k.dttz2;
  c.dt = k.dt;
}

float2 split_const(double v) {
  const float hi = (float)v;
  return make_float2(hi, (float)(v - (double)hi));
}

// The double-float constants of the primitive kernel and compute_rhs.
void make_rhs_df_consts(const Consts& k, const LinWeights& lw, RhsDfConsts& c) {
  for (int d = 0; d < 3; ++d)
    for (int cl = 0; cl < 32; ++cl)
      for (int o = 0; o < 5; ++o) c.w[d][cl][o] = split_const(lw.w[d][cl][o]);
  const double vc[3][3] = {{k.xxcon2 * k.con43, k.xxcon2, k.xxcon2},
                           {k.yycon2, k.yycon2 * k.con43, k.yycon2},
                           {k.zzcon2, k.zzcon2, k.zzcon2 * k.con43}};
  for (int d = 0; d < 3; ++d)
    for (int m = 0; m < 3; ++m) c.vc[d][m] = split_const(vc[d][m]);
  for (int m = 0; m < 3; ++m) c.vcc[m] = split_const(-2.0 * (vc[0][m] + vc[1][m] + vc[2][m]));
  c.t2[0] = split_const(k.tx2);
  c.t2[1] = split_const(k.ty2);
  c.t2[2] = split_const(k.tz2);
  c.dt = split_const(k.dt);
  c.c1 = split_const(k.c1);
  c.c2 = split_const(k.c2);
  c.c1c2 = split_const(k.c1c2);
  c.bt = split_const(k.bt);
  const double c3[3] = {k.xxcon3, k.yycon3, k.zzcon3}, c4[3] = {k.xxcon4, k.yycon4, k.zzcon4},
               c5[3] = {k.xxcon5, k.yycon5, k.zzcon5};
  for (int d = 0; d < 3; ++d) {
    c.con3[d] = split_const(c3[d]);
    c.con4[d] = split_const(c4[d]);
    c.con5[d] = split_const(c5[d]);
  }
  // The low words of the stencil weights and t2 are dropped when none
  // exceeds 2^-47 of its high word: below the compensated sum's own rounding
  // (a few units of 2^-48 of the largest term), as for the class grids,
  // whose d*t1 factors are integers plus a few FP64 roundings.
  auto small_lo = [](float2 v) { return std::fabs((double)v.y) <= std::ldexp(std::fabs((double)v.x), -47); };
  c.exact_w = 1;
  for (int d = 0; d < 3; ++d) {
    if (!small_lo(c.t2[d])) c.exact_w = 0;
    for (int cl = 0; cl < 32; ++cl)
      for (int o = 0; o < 5; ++o)
        if (!small_lo(c.w[d][cl][o])) c.exact_w = 0;
  }
}

// A contiguous slice of a work list: items [lo, hi) belong to one zone.
struct Range {
  int lo = 0, hi = 0;
};

}  // namespace

struct HandleLimits {
  static constexpr int MAXB = 3;  // zone-size buckets per sweep direction
};

struct npbmz_handle {
  int kind = 0, nzones = 0, flags = 0;
  Consts K;
  std::vector<ZoneDev> zh;
  std::vector<int> nbr;
  int64_t NP = 0;
  int max_face = 0, max_np = 0;
  // device buffers
  ZoneDev* zones_d = nullptr;
  int* nbr_d = nullptr;
  double* u = nullptr;
  double* rhs = nullptr;
  double* forcing = nullptr;
  double* prim = nullptr;
  double* uex = nullptr;
  double* xw = nullptr;      // first-pass line solution of the refined mixed solve
  float* primf = nullptr;    // FP32 state copies for the mixed line solves
  double* flux = nullptr;    // compute_rhs point functions (FMA build)
  float* rdf = nullptr;      // double-float rhs handed between the refined FP32 BT sweeps of a step
  float* pfx = nullptr;      // x-line-major copies for the refined FP32 BT x sweep (see Fields)
  float* rdx = nullptr;
  float* x0x = nullptr;
  LinWeights lw;             // compute_rhs linear stencil weights (FMA build)
  RhsF64Consts rc64;         // the FMA build's compute_rhs constants (dt folded in)
  double* fdt = nullptr;     // [5][NP] dt * forcing (FMA build's compute_rhs)
  // refined mixed step with the double-float primitive kernel and compute_rhs
  bool dfrhs = false;
  float2* ud = nullptr;      // [5][NP] u
  float2* xd = nullptr;      // [XD_COUNT][NP] point functions
  float2* fd = nullptr;      // [5][NP] forcing
  RhsDfConsts rdc;
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  // y and z line scratch of the grouped step graph, where sweeps of
  // different directions (of different zone groups) run at the same time
  void* scratch_yz[2] = {nullptr, nullptr};
  double* part_rhs = nullptr;
  double* part_err = nullptr;
  double* norms_d = nullptr;
  int norms_cap = 0;
  double* stage = nullptr;
  size_t stage_elems = 0;
  int64_t* soff_d[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
  std::vector<int64_t> soff_h[2][3];   // per layout, field: zone offsets (+ total at [nzones])
  // work lists
  Work* wpts_d = nullptr;
  int nwpts = 0;
  std::vector<Range> pts_range;   // per zone
  int* zblk_pts_d = nullptr;      // [2*nzones] CTA ranges of each zone (point list)
  Work* wint_d = nullptr;         // interior-point list (compute_rhs)
  int nwint = 0;
  std::vector<Range> int_range;
  int* zblk_int_d = nullptr;
  bool bnd_dirty = true;          // boundary rhs must be reset to the forcing
  Work* wline_d[3] = {nullptr, nullptr, nullptr};
  int nwline[3] = {0, 0, 0};
  std::vector<Range> line_range[3];
  // zone groups of the pipelined step graph: every work list is ordered
  // group-major, so group g owns one contiguous slice of each list
  int ngroups = 1;
  std::vector<int> zone_group;     // per zone
  std::vector<Range> grp_pts, grp_int, grp_line[3];
  int cur_group = -1;              // >= 0 while the phases of one group are issued
  cudaStream_t grp_stream[8] = {};
  // the x sweep's x-line-major state copies made by the compute_rhs launch
  // (k_rhs_flux_xc) instead of a kernel of their own (npbmz_set_copy_fusion)
  bool copy_fusion = true;
  // the zone groups' streams of the npbmz_step_inout graph: priorities fall
  // with the group number, so that the groups finish in the order their copies
  // came in and each one's copy out starts while later groups compute
  cudaStream_t io_grp_stream[8] = {};
  // the zone groups' primitive kernels and compute_rhs (FP64 pipe) on one
  // stream of the device's greatest priority, so that their CTAs go to SMs
  // ahead of the waiting CTAs of the sweeps (FP32 pipe) they run beside
  bool fp64_prio = false;
  cudaStream_t prio_stream = nullptr;
  // resident CTAs per SM of the pipelined sweep kernels (0: one CTA per work
  // item): a cap leaves registers on every SM for the FP64 kernels of the
  // next zone group
  int sweep_cap = 0;
  cudaEvent_t grp_ev[2 * 8 + 1] = {};
  // npbmz_step_download: the graph records grp_out_ev[g] (an external event)
  // when group g's z sweep has written its zones' u; io_stream then copies
  // those zones out while the other groups compute.
  cudaEvent_t grp_out_ev[8] = {};
  cudaStream_t io_stream = nullptr;
  cudaEvent_t io_done = nullptr;
  int* grp_zones_d = nullptr;        // zones of each group, group-major
  std::vector<int> grp_zone_off;     // group g's zones at [off[g], off[g+1])
  // Lines per CTA of the line solves, per sweep direction and zone-size
  // bucket: zones are split by line length into nbkt buckets per direction
  // (npbmz_autotune sets 3 and picks each bucket's lines per CTA).
  int nbkt = 1;
  std::vector<int> zone_bucket[3];
  int tpb_bkt[3][HandleLimits::MAXB] = {{64, 64, 64}, {64, 64, 64}, {64, 64, 64}};
  std::vector<Range> gb_line[3];   // per (group, bucket): slice of the line list
  int cur_bucket = -1;             // >= 0: line launches of that bucket only
  int64_t nlines[3] = {0, 0, 0};
  // execution
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaGraphExec_t graph_exec = nullptr;
  // npbmz_step_inout's first step: the grouped graph without exch_qbc, whose
  // group g waits for the upload of its zones (up_ev[g], recorded on
  // io_stream before the launch)
  cudaGraphExec_t graph_inout = nullptr;
  cudaEvent_t up_ev[8] = {};
  cudaEvent_t exch_ev = nullptr;
  // its copies of whole zone arrays by the copy engines: a device image of
  // the caller's buffer, one H2D and one D2H stream, per-group events
  double* io_image = nullptr;
  size_t io_image_elems = 0;
  cudaStream_t io_h2d = nullptr, io_d2h = nullptr;
  cudaEvent_t dma_ev[8] = {}, conv_ev[8] = {};
  cudaStream_t graph_stream = nullptr;
  cudaStream_t aux_stream = nullptr;   // graph replay when the handle's stream is the legacy one
  cudaEvent_t fence[2] = {nullptr, nullptr};
  int launches_per_step = 0;
  int64_t device_bytes = 0;
  // faces exchanged with other ranks (npbmz_face_plan): packed and unpacked
  // through caller-owned device buffers
  bool has_remote = false;
  FaceDesc* send_faces_d = nullptr;
  FaceDesc* recv_faces_d = nullptr;
  int nsend = 0, nrecv = 0;
  // state check: the device word of Fields::health and its page-locked copy
  unsigned long long* health_d = nullptr;
  unsigned long long* health_h = nullptr;
  unsigned health_bits = 0;   // of the last npbmz_step / npbmz_step_download
  int64_t health_point = -1;
  std::string err;
};

namespace {

int fail(npbmz_t* h, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (h) h->err = buf;
  else g_create_error = buf;
  return -1;
}

#define CK(h, call)                                                                               \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess) return fail((h), "%s failed: %s", #call, cudaGetErrorString(e_));      \
  } while (0)

#define CKL(h)                                                                                    \
  do {                                                                                            \
    cudaError_t e_ = cudaGetLastError();                                                          \
    if (e_ != cudaSuccess) return fail((h), "kernel launch failed: %s", cudaGetErrorString(e_));  \
  } while (0)

template <typename T>
int dalloc(npbmz_t* h, T** p, size_t count) {
  size_t bytes = count * sizeof(T);
  if (bytes == 0) bytes = sizeof(T);
  CK(h, cudaMalloc((void**)p, bytes));
  h->device_bytes += (int64_t)bytes;
  return 0;
}

Fields fields(const npbmz_t* h) {
  Fields F;
  F.u = h->u;
  F.rhs = h->rhs;
  F.forcing = h->forcing;
  F.prim = h->prim;
  F.uex = h->uex;
  F.zones = h->zones_d;
  F.NP = h->NP;
  F.primf = (h->flags & NPBMZ_MIXED) && !(h->flags & NPBMZ_FP32_NOREFINE) ? h->primf : nullptr;
  F.flux = (h->flags & NPBMZ_EXACT) ? nullptr : h->flux;
  F.rdf = h->rdf;
  F.pfx = h->pfx;
  F.rdx = h->rdx;
  F.x0x = h->x0x;
  F.nlx = h->nlines[0];
  F.ud = h->ud;
  F.xd = h->xd;
  F.fd = h->fd;
  F.fdt = h->fdt;
  F.health = h->health_d;
  return F;
}

bool use_exact(const npbmz_t* h) { return (h->flags & NPBMZ_EXACT) != 0; }
bool use_fp32(const npbmz_t* h) { return (h->flags & (NPBMZ_MIXED | NPBMZ_FP32_NOREFINE)) != 0; }

// Reference-layout element count of one zone's array (see include/npbmz.h).
int64_t ref_elems(int kind, int field, const ZoneDev& z) {
  const int64_t IMAX = z.nx + 1, JMAX = z.ny + 1, KMAX = z.nz + 1;
  if (kind == NPBMZ_BT) {
    if (field == NPBMZ_U) return 5 * (IMAX + 4) * (JMAX + 4) * (KMAX + 4);
    if (field == NPBMZ_RHS) return 5 * (IMAX + 1) * (JMAX + 1) * (KMAX + 1);
    return 5 * IMAX * JMAX * KMAX;
  }
  const int64_t IMAXP = (IMAX / 2) * 2 + 1, JMAXP = (JMAX / 2) * 2 + 1;
  if (field == NPBMZ_U) return 5 * (IMAXP + 4) * (JMAXP + 4) * (KMAX + 4);
  return 5 * IMAXP * JMAXP * KMAX;
}

// Zones into ngroups groups of near-equal point counts (largest zone first
// into the lightest group).
// Zone groups are runs of consecutive zones, so that each group's host arrays
// are one contiguous range of the caller's buffer (npbmz_step_inout moves a
// group with one copy each way).  With 4 or more groups the first and the
// last hold half the points of the others: the first step of
// npbmz_step_inout waits for the first group's copy in, and its end for the
// last group's copy out.  Group g starts at the first zone whose prefix holds
// its share of the points, and every group keeps at least one zone.
void assign_zone_groups(npbmz_t* h) {
  const int nz = h->nzones;
  const int G = std::max(1, std::min(h->ngroups, nz));
  h->ngroups = G;
  std::vector<int64_t> cum(nz + 1, 0);
  for (int z = 0; z < nz; ++z) cum[z + 1] = cum[z] + (int64_t)h->zh[z].nx * h->zh[z].ny * h->zh[z].nz;
  // weights in halves: 1 for the end groups, 2 for the others (G >= 4)
  std::vector<int64_t> wcum(G + 1, 0);
  for (int g = 0; g < G; ++g) wcum[g + 1] = wcum[g] + ((G >= 4 && (g == 0 || g == G - 1)) ? 1 : 2);
  std::vector<int> start(G + 1, 0);
  start[G] = nz;
  for (int g = 1; g < G; ++g) {
    int z = start[g - 1] + 1;
    while (z < nz - (G - g) && cum[z] * wcum[G] < cum[nz] * wcum[g]) ++z;
    start[g] = z;
  }
  h->zone_group.assign(nz, 0);
  for (int g = 0; g < G; ++g)
    for (int z = start[g]; z < start[g + 1]; ++z) h->zone_group[z] = g;
}

// Zones group-major, each group's zones by decreasing key (the longest work
// first, each zone contiguous).
template <typename Key>
std::vector<int> group_order(const npbmz_t* h, Key key) {
  std::vector<int> order(h->nzones);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    if (h->zone_group[a] != h->zone_group[b]) return h->zone_group[a] < h->zone_group[b];
    return key(a) > key(b);
  });
  return order;
}

// Per-group slices [lo, hi) of a work list from its per-zone ranges.
std::vector<Range> group_ranges(const npbmz_t* h, const std::vector<Range>& zr) {
  std::vector<Range> gr(h->ngroups);
  for (int g = 0; g < h->ngroups; ++g) { gr[g].lo = 1 << 30; gr[g].hi = 0; }
  for (int z = 0; z < h->nzones; ++z) {
    Range& r = gr[h->zone_group[z]];
    r.lo = std::min(r.lo, zr[z].lo);
    r.hi = std::max(r.hi, zr[z].hi);
  }
  for (Range& r : gr)
    if (r.hi < r.lo) r.lo = r.hi = 0;
  return gr;
}

int build_work_lists(npbmz_t* h) {
  const int nz = h->nzones;
  if ((int)h->zone_group.size() != nz) assign_zone_groups(h);
  for (void** b : {(void**)&h->wpts_d, (void**)&h->zblk_pts_d, (void**)&h->wint_d, (void**)&h->zblk_int_d,
                   (void**)&h->part_rhs, (void**)&h->part_err})
    if (*b) { cudaFree(*b); *b = nullptr; }
  const std::vector<int> order =
      group_order(h, [&](int z) { return (int64_t)h->zh[z].nx * h->zh[z].ny * h->zh[z].nz; });
  std::vector<Work> w;
  h->pts_range.assign(nz, Range());
  for (int z : order) {
    const int np = h->zh[z].nx * h->zh[z].ny * h->zh[z].nz;
    h->pts_range[z].lo = (int)w.size();
    for (int f = 0; f < np; f += PTS_TPB) w.push_back(Work{z, f});
    h->pts_range[z].hi = (int)w.size();
  }
  h->nwpts = (int)w.size();
  if (dalloc(h, &h->wpts_d, w.size())) return -1;
  CK(h, cudaMemcpy(h->wpts_d, w.data(), w.size() * sizeof(Work), cudaMemcpyHostToDevice));
  std::vector<int> zb(2 * nz);
  for (int z = 0; z < nz; ++z) { zb[2 * z] = h->pts_range[z].lo; zb[2 * z + 1] = h->pts_range[z].hi; }
  if (dalloc(h, &h->zblk_pts_d, zb.size())) return -1;
  CK(h, cudaMemcpy(h->zblk_pts_d, zb.data(), zb.size() * sizeof(int), cudaMemcpyHostToDevice));
  // interior points (compute_rhs and the residual norm)
  std::vector<Work> wi;
  h->int_range.assign(nz, Range());
  for (int z : order) {
    const ZoneDev& d = h->zh[z];
    const int ni = (d.nx - 2) * (d.ny - 2) * (d.nz - 2);
    h->int_range[z].lo = (int)wi.size();
    for (int f = 0; f < ni; f += PTS_TPB) wi.push_back(Work{z, f});
    h->int_range[z].hi = (int)wi.size();
  }
  h->nwint = (int)wi.size();
  if (dalloc(h, &h->wint_d, wi.size())) return -1;
  CK(h, cudaMemcpy(h->wint_d, wi.data(), wi.size() * sizeof(Work), cudaMemcpyHostToDevice));
  std::vector<int> zi(2 * nz);
  for (int z = 0; z < nz; ++z) { zi[2 * z] = h->int_range[z].lo; zi[2 * z + 1] = h->int_range[z].hi; }
  if (dalloc(h, &h->zblk_int_d, zi.size())) return -1;
  CK(h, cudaMemcpy(h->zblk_int_d, zi.data(), zi.size() * sizeof(int), cudaMemcpyHostToDevice));
  if (dalloc(h, &h->part_rhs, (size_t)h->nwint * 5)) return -1;
  if (dalloc(h, &h->part_err, (size_t)h->nwpts * 5)) return -1;
  h->grp_pts = group_ranges(h, h->pts_range);
  h->grp_int = group_ranges(h, h->int_range);
  return 0;
}

template <typename Fn>
int line_launches(npbmz_t* h, int dir, int zone, Fn fn);

// The boundary points of rhs hold the forcing (compute_rhs sets rhs = forcing
// on the whole cell, src/BT/rhs.jl:85-93, and no solve rewrites them); the
// rhs kernel only visits interior points, so reset them after an upload.
int flush_boundary(npbmz_t* h) {
  if (!h->bnd_dirty) return 0;
  CK(h, cudaMemcpyAsync(h->rhs, h->forcing, 5 * h->NP * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  if (h->rdf) {
    fast::launch_split_df(h->forcing, h->rdf, h->NP, h->stream);
    CKL(h);
  }
  if (h->fd) {
    fast::launch_split_f2(h->forcing, h->fd, h->NP, h->stream);
    CKL(h);
  }
  if (h->fdt) {
    fast::launch_scale(h->forcing, h->fdt, h->K.dt, 5 * h->NP, h->stream);
    CKL(h);
  }
  if (h->rdx) {
    const Fields F = fields(h);
    const int saved = h->cur_group;
    h->cur_group = -1;
    const int rc = line_launches(h, 0, -1, [&](int lo, int hi, int tpb) {
      fast::launch_xline_ends(F, h->wline_d[0] + lo, hi - lo, tpb, h->stream);
      CKL(h);
      return 0;
    });
    h->cur_group = saved;
    if (rc) return -1;
  }
  h->bnd_dirty = false;
  return 0;
}

// Zone-size buckets of one sweep direction: zones by decreasing line length
// cut into nbkt runs of near-equal line counts.
void assign_buckets(npbmz_t* h, int dir) {
  const int nz = h->nzones;
  std::vector<int> order(nz);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return zone_line_len(h->zh[a], dir) > zone_line_len(h->zh[b], dir);
  });
  int64_t total = 0;
  for (int z = 0; z < nz; ++z) total += zone_lines(h->zh[z], dir);
  h->zone_bucket[dir].assign(nz, 0);
  int64_t acc = 0;
  for (int z : order) {
    h->zone_bucket[dir][z] = (int)std::min<int64_t>(h->nbkt - 1, acc * h->nbkt / std::max<int64_t>(total, 1));
    acc += zone_lines(h->zh[z], dir);
  }
}

int build_line_lists(npbmz_t* h) {
  const int nz = h->nzones;
  for (int dir = 0; dir < 3; ++dir) {
    if (h->wline_d[dir]) { cudaFree(h->wline_d[dir]); h->wline_d[dir] = nullptr; }
    if ((int)h->zone_bucket[dir].size() != nz) assign_buckets(h, dir);
    const std::vector<int>& bk = h->zone_bucket[dir];
    // group-major, then bucket, then the longest lines first
    std::vector<int> order(nz);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
      if (h->zone_group[a] != h->zone_group[b]) return h->zone_group[a] < h->zone_group[b];
      if (bk[a] != bk[b]) return bk[a] < bk[b];
      return zone_line_len(h->zh[a], dir) > zone_line_len(h->zh[b], dir);
    });
    std::vector<Work> w;
    h->line_range[dir].assign(nz, Range());
    h->gb_line[dir].assign((size_t)h->ngroups * h->nbkt, Range());
    for (Range& r : h->gb_line[dir]) { r.lo = 1 << 30; r.hi = 0; }
    for (int z : order) {
      const int tpb = h->tpb_bkt[dir][bk[z]];
      const int nl = zone_lines(h->zh[z], dir);
      h->line_range[dir][z].lo = (int)w.size();
      for (int f = 0; f < nl; f += tpb) w.push_back(Work{z, f});
      h->line_range[dir][z].hi = (int)w.size();
      Range& r = h->gb_line[dir][(size_t)h->zone_group[z] * h->nbkt + bk[z]];
      r.lo = std::min(r.lo, h->line_range[dir][z].lo);
      r.hi = std::max(r.hi, h->line_range[dir][z].hi);
    }
    for (Range& r : h->gb_line[dir])
      if (r.hi < r.lo) r.lo = r.hi = 0;
    h->nwline[dir] = (int)w.size();
    CK(h, cudaMalloc((void**)&h->wline_d[dir], std::max<size_t>(1, w.size()) * sizeof(Work)));
    CK(h, cudaMemcpy(h->wline_d[dir], w.data(), w.size() * sizeof(Work), cudaMemcpyHostToDevice));
    h->grp_line[dir] = group_ranges(h, h->line_range[dir]);
  }
  return 0;
}

// Every launch over a line list goes through here: fn(lo, hi, tpb) for each
// slice whose work items were built with tpb lines -- one zone, the current
// zone group or all groups, bucket by bucket (the current bucket only when
// one is set).
template <typename Fn>
int line_launches(npbmz_t* h, int dir, int zone, Fn fn) {
  if (zone >= 0) {
    const Range r = h->line_range[dir][zone];
    return r.hi > r.lo ? fn(r.lo, r.hi, h->tpb_bkt[dir][h->zone_bucket[dir][zone]]) : 0;
  }
  if (h->cur_group < 0 && h->cur_bucket < 0 && h->nbkt == 1)  // one shape: the whole list in one launch
    return h->nwline[dir] > 0 ? fn(0, h->nwline[dir], h->tpb_bkt[dir][0]) : 0;
  const int g0 = h->cur_group >= 0 ? h->cur_group : 0, g1 = h->cur_group >= 0 ? h->cur_group + 1 : h->ngroups;
  for (int g = g0; g < g1; ++g)
    for (int b = 0; b < h->nbkt; ++b) {
      if (h->cur_bucket >= 0 && b != h->cur_bucket) continue;
      const Range r = h->gb_line[dir][(size_t)g * h->nbkt + b];
      if (r.hi > r.lo && fn(r.lo, r.hi, h->tpb_bkt[dir][b])) return -1;
    }
  return 0;
}

// ---- phases ---------------------------------------------------------------
// The x sweep of a fused step reads x-line-major copies of the FP32 state.
// With copy fusion on and the x-sweep work list of this launch scope one
// slice (one line shape), the compute_rhs launch makes them (k_rhs_flux_xc),
// so that their memory traffic runs beside the FP64-bound compute_rhs;
// otherwise the primitive phase launches k_xline_copy per slice.
struct XSlices {
  int n = 0, lo = 0, hi = 0, tpb = 0;
};
XSlices x_slices(npbmz_t* h, int zone) {
  XSlices x;
  line_launches(h, 0, zone, [&](int lo, int hi, int tpb) {
    ++x.n;
    x.lo = lo;
    x.hi = hi;
    x.tpb = tpb;
    return 0;
  });
  return x;
}
bool copy_in_rhs(npbmz_t* h, int zone, bool fused) {
  return fused && h->copy_fusion && h->pfx && h->flux && h->fdt && !h->dfrhs && !use_exact(h) &&
         x_slices(h, zone).n == 1;
}

// fused: part of a whole step (run_adi): with the double-float primitive
// kernel, the FP64 prim planes that only single phases read are skipped.
int phase_prim(npbmz_t* h, int zone, bool fused = false) {
  Fields F = fields(h);
  F.prim64 = !fused;
  int64_t lo = 0, hi = h->NP;
  if (zone >= 0) {
    lo = h->zh[zone].off;
    hi = lo + (int64_t)h->zh[zone].nx * h->zh[zone].ny * h->zh[zone].nz;
  }
  const bool sp = h->kind == NPBMZ_SP;
  if (use_exact(h)) {
    exact::launch_prim(sp, F, h->K, lo, hi, h->stream);
  } else {
    // over the point work list
    int wlo = 0, whi = h->nwpts;
    if (zone >= 0) { wlo = h->pts_range[zone].lo; whi = h->pts_range[zone].hi; }
    else if (h->cur_group >= 0) { wlo = h->grp_pts[h->cur_group].lo; whi = h->grp_pts[h->cur_group].hi; }
    Fields Fp = F;
    Fp.pfx = nullptr;  // the x-line-major state copies come from k_xline_copy
    if (h->dfrhs)
      fast::launch_prim_df(sp, Fp, h->rdc, h->wpts_d + wlo, whi - wlo, h->stream, (h->flags & NPBMZ_PERSIST) != 0);
    else
      fast::launch_prim_w(sp, Fp, h->K, h->wpts_d + wlo, whi - wlo, h->stream, (h->flags & NPBMZ_PERSIST) != 0);
    CKL(h);
    // the x sweep of a fused step reads x-line-major copies of the state
    if (fused && h->pfx && !copy_in_rhs(h, zone, fused) &&
        line_launches(h, 0, zone, [&](int llo, int lhi, int tpb) {
          fast::launch_xline_copy(sp, F, h->wline_d[0] + llo, lhi - llo, tpb, h->stream);
          CKL(h);
          return 0;
        }))
      return -1;
  }
  CKL(h);
  return 0;
}

// fused: part of a whole step, whose sweeps read only the double-float copy
// of rhs (the z sweep rewrites rhs in FP64).
int phase_rhs(npbmz_t* h, int zone, bool tx, bool norm, bool fused = false) {
  if (flush_boundary(h)) return -1;
  Fields F = fields(h);
  F.rhs64 = !fused;
  int lo = 0, hi = h->nwint;
  if (zone >= 0) { lo = h->int_range[zone].lo; hi = h->int_range[zone].hi; }
  else if (h->cur_group >= 0) { lo = h->grp_int[h->cur_group].lo; hi = h->grp_int[h->cur_group].hi; }
  if (use_exact(h)) exact::launch_rhs(tx, norm, F, h->K, h->wint_d + lo, hi - lo, h->part_rhs + 5 * lo, h->stream);
  else if (h->dfrhs)
    fast::launch_rhs_df(tx, norm, F, h->rdc, h->wint_d + lo, hi - lo, h->part_rhs + 5 * lo, h->stream,
                        (h->flags & NPBMZ_PERSIST) != 0);
  else if (copy_in_rhs(h, zone, fused)) {
    const XSlices x = x_slices(h, zone);
    fast::launch_rhs_xc(tx, norm, F, h->K, h->rc64, h->wint_d + lo, hi - lo, h->part_rhs + 5 * lo,
                        h->wline_d[0] + x.lo, x.hi - x.lo, x.tpb, h->stream, (h->flags & NPBMZ_PERSIST) != 0);
  } else fast::launch_rhs(tx, norm, F, h->K, h->wint_d + lo, hi - lo, h->part_rhs + 5 * lo, h->stream, &h->rc64,
                          (h->flags & NPBMZ_PERSIST) != 0);
  CKL(h);
  return 0;
}

// fused: part of a whole step (run_adi), where the refined FP32 BT sweeps
// hand their results on as double-float; otherwise each sweep reads and
// writes rhs in FP64 (single phases, the adjoint's recomputation).
void* line_scratch(npbmz_t* h, int dir) {
  return (dir > 0 && h->scratch_yz[dir - 1]) ? h->scratch_yz[dir - 1] : h->scratch;
}

int phase_solve(npbmz_t* h, int dir, int zone, int add_u, bool fused = false) {
  const Fields F = fields(h);
  const bool sp = h->kind == NPBMZ_SP;
  const int mode = use_exact(h) ? 0
                   : !use_fp32(h) ? 0
                   : (h->flags & NPBMZ_FP32_NOREFINE) ? 1
                   : (h->flags & NPBMZ_REFINE_FP64) ? 3
                   : (fused && h->rdf ? 4 : 2);
  return line_launches(h, dir, zone, [&](int lo, int hi, int tpb) {
    if (use_exact(h))
      exact::launch_solve(sp, 0, dir, F, h->K, h->wline_d[dir] + lo, hi - lo, tpb, line_scratch(h, dir),
                          h->nlines[dir], add_u, nullptr, h->stream);
    else
      fast::launch_solve(sp, mode, dir, F, h->K, h->wline_d[dir] + lo, hi - lo, tpb, line_scratch(h, dir),
                         h->nlines[dir], add_u, h->xw, h->stream, (h->flags & NPBMZ_PERSIST) != 0, h->sweep_cap);
    CKL(h);
    return 0;
  });
}

int phase_add(npbmz_t* h, int zone) {
  const Fields F = fields(h);
  int lo = 0, hi = h->nwpts;
  if (zone >= 0) { lo = h->pts_range[zone].lo; hi = h->pts_range[zone].hi; }
  if (use_exact(h)) exact::launch_add(F, h->wpts_d + lo, hi - lo, h->stream);
  else fast::launch_add(F, h->wpts_d + lo, hi - lo, h->stream);
  CKL(h);
  return 0;
}

int phase_exch(npbmz_t* h) {
  // the reference skips exch_qbc for a one-zone problem (bt-node.jl:286); a
  // rank's one zone of a larger problem still copies the faces it owns
  if (h->nzones < 2 && !h->has_remote) return 0;
  launch_exch_qbc(fields(h), h->nbr_d, 0, h->nzones, h->max_face, h->stream);
  CKL(h);
  return 0;
}

// adi for one zone or all zones (batched); norm: rhs partials for this step.
int run_adi(npbmz_t* h, int zone, bool norm) {
  const bool sp = h->kind == NPBMZ_SP;
  if (zone < 0 && (h->flags & NPBMZ_PERZONE)) {
    for (int z = 0; z < h->nzones; ++z)
      if (run_adi(h, z, norm)) return -1;
    return 0;
  }
  if (phase_prim(h, zone, true)) return -1;
  if (phase_rhs(h, zone, sp, norm, true)) return -1;
  if (phase_solve(h, 0, zone, 0, true)) return -1;
  if (phase_solve(h, 1, zone, 0, true)) return -1;
  if (phase_solve(h, 2, zone, 1, true)) return -1;  // add fused into the z sweep
  return 0;
}

int finish_norms(npbmz_t* h, double* out_rhs, double* out_err) {
  if (out_rhs) launch_norm_finish(h->zones_d, h->part_rhs, h->zblk_int_d, h->nzones, 1.0 / h->K.dt, out_rhs, h->stream);
  if (out_err) launch_norm_finish(h->zones_d, h->part_err, h->zblk_pts_d, h->nzones, 1.0, out_err, h->stream);
  CKL(h);
  return 0;
}

int err_partials(npbmz_t* h) {
  launch_err_partials(fields(h), h->wpts_d, h->nwpts, h->part_err, h->stream);
  CKL(h);
  return 0;
}

int one_step(npbmz_t* h, bool norm, double* norm_slot) {
  if (phase_exch(h)) return -1;
  if (run_adi(h, -1, norm)) return -1;
  if (norm) {
    if (err_partials(h)) return -1;
    if (finish_norms(h, norm_slot, norm_slot + 5)) return -1;
  }
  return 0;
}

void drop_graph(npbmz_t* h) {
  if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
  if (h->graph_inout) cudaGraphExecDestroy(h->graph_inout);
  h->graph_exec = nullptr;
  h->graph_inout = nullptr;
}

// One step as zone-group branches (captured into the step graph): after
// exch_qbc, group g runs prim, compute_rhs and its three sweeps on its own
// stream; its primitive kernel waits for group g-1's compute_rhs.  So the
// FP32 sweeps of group g (FP32 / issue bound) run beside the FP64
// primitive and compute_rhs kernels of group g+1 (FP64-pipe bound).
// inout: the first step of npbmz_step_inout -- exch_qbc is left out (the
// caller runs it between the two parts of the upload) and group g's branch
// first waits for up_ev[g], the upload of its zones.
int grouped_step(npbmz_t* h, cudaStream_t cs, bool inout) {
  const int G = h->ngroups;
  const bool sp = h->kind == NPBMZ_SP;
  if (!inout && phase_exch(h)) return -1;
  cudaEvent_t start = h->grp_ev[2 * G];
  CK(h, cudaEventRecord(start, cs));
  int rc = 0;
  for (int g = 0; g < G && !rc; ++g) {
    cudaStream_t S = inout ? h->io_grp_stream[g] : h->grp_stream[g];
    // prim + compute_rhs of group g: on the priority stream (in group order),
    // or on the group's own stream after group g-1's compute_rhs (always so
    // in the npbmz_step_inout graph, whose group streams carry the priorities)
    cudaStream_t P = h->fp64_prio && !inout ? h->prio_stream : S;
    rc |= cudaStreamWaitEvent(P, start, 0) != cudaSuccess;
    if (inout) rc |= cudaStreamWaitEvent(P, h->up_ev[g], cudaEventWaitExternal) != cudaSuccess;
    if (g > 0 && P == S) rc |= cudaStreamWaitEvent(S, h->grp_ev[2 * (g - 1)], 0) != cudaSuccess;
    h->stream = P;
    h->cur_group = g;
    if (!rc) rc = phase_prim(h, -1, true);
    if (!rc) rc = phase_rhs(h, -1, sp, false, true);
    if (!rc) rc = cudaEventRecord(h->grp_ev[2 * g], P) != cudaSuccess;
    if (!rc && P != S) rc = cudaStreamWaitEvent(S, h->grp_ev[2 * g], 0) != cudaSuccess;
    h->stream = S;
    for (int dir = 0; dir < 3 && !rc; ++dir) rc = phase_solve(h, dir, -1, dir == 2 ? 1 : 0, true);
    // group g's u is final: an event that work outside the graph can wait on
    if (!rc) rc = cudaEventRecordWithFlags(h->grp_out_ev[g], S, cudaEventRecordExternal) != cudaSuccess;
    if (!rc) rc = cudaEventRecord(h->grp_ev[2 * g + 1], S) != cudaSuccess;
  }
  h->stream = cs;
  h->cur_group = -1;
  for (int g = 0; g < G && !rc; ++g) rc = cudaStreamWaitEvent(cs, h->grp_ev[2 * g + 1], 0) != cudaSuccess;
  if (rc && h->err.empty()) h->err = "grouped step capture failed";
  return rc ? -1 : 0;
}

bool use_groups(const npbmz_t* h) {
  return h->ngroups > 1 && !use_exact(h) && !(h->flags & NPBMZ_PERZONE);
}

int capture_step_graph(npbmz_t* h, bool inout = false) {
  cudaGraphExec_t& exec = inout ? h->graph_inout : h->graph_exec;
  if (exec) cudaGraphExecDestroy(exec);
  exec = nullptr;
  if (inout && !use_groups(h)) return fail(h, "the overlapped upload needs zone-group branches");
  if (use_groups(h)) {
    for (int g = 0; g < h->ngroups; ++g)
      if (!h->grp_stream[g]) CK(h, cudaStreamCreateWithFlags(&h->grp_stream[g], cudaStreamNonBlocking));
    for (int e = 0; e < 2 * h->ngroups + 1; ++e)
      if (!h->grp_ev[e]) CK(h, cudaEventCreateWithFlags(&h->grp_ev[e], cudaEventDisableTiming));
    for (int g = 0; g < h->ngroups; ++g) {
      if (!h->grp_out_ev[g]) CK(h, cudaEventCreateWithFlags(&h->grp_out_ev[g], cudaEventDisableTiming));
      if (!h->up_ev[g]) CK(h, cudaEventCreateWithFlags(&h->up_ev[g], cudaEventDisableTiming));
    }
    if (h->fp64_prio && !h->prio_stream) {
      int least = 0, greatest = 0;
      CK(h, cudaDeviceGetStreamPriorityRange(&least, &greatest));
      CK(h, cudaStreamCreateWithPriority(&h->prio_stream, cudaStreamNonBlocking, greatest));
    }
    if (inout) {
      int least = 0, greatest = 0;
      CK(h, cudaDeviceGetStreamPriorityRange(&least, &greatest));
      const int levels = least - greatest + 1;  // greatest is the numerically smaller
      for (int g = 0; g < h->ngroups; ++g) {
        if (h->io_grp_stream[g]) {
          CK(h, cudaStreamSynchronize(h->io_grp_stream[g]));
          CK(h, cudaStreamDestroy(h->io_grp_stream[g]));
        }
        // group 0 at the greatest priority, the last groups at the least
        const int prio = greatest + g * levels / h->ngroups;
        CK(h, cudaStreamCreateWithPriority(&h->io_grp_stream[g], cudaStreamNonBlocking, prio));
      }
    }
  }
  if (flush_boundary(h)) return -1;  // keep the one-off reset out of the graph
  // Capture is not allowed on the legacy default stream: capture and replay
  // on an owned stream, fenced against the caller's stream by events.
  cudaStream_t cs = h->stream;
  if (cs == nullptr) {
    if (!h->aux_stream) CK(h, cudaStreamCreateWithFlags(&h->aux_stream, cudaStreamNonBlocking));
    if (!h->fence[0]) {
      CK(h, cudaEventCreateWithFlags(&h->fence[0], cudaEventDisableTiming));
      CK(h, cudaEventCreateWithFlags(&h->fence[1], cudaEventDisableTiming));
    }
    cs = h->aux_stream;
  }
  cudaGraph_t g = nullptr;
  cudaStream_t saved = h->stream;
  h->stream = cs;
  CK(h, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
  int rc = use_groups(h) ? grouped_step(h, cs, inout) : one_step(h, false, nullptr);
  cudaError_t e = cudaStreamEndCapture(cs, &g);
  h->stream = saved;
  if (rc) { if (g) cudaGraphDestroy(g); return -1; }
  if (e != cudaSuccess) return fail(h, "stream capture failed: %s", cudaGetErrorString(e));
  // kernel nodes keep the priority of the stream they were captured from
  e = cudaGraphInstantiate(&exec, g,
                           use_groups(h) && (h->fp64_prio || inout) ? cudaGraphInstantiateFlagUseNodePriority : 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(h, "graph instantiate failed: %s", cudaGetErrorString(e));
  h->graph_stream = h->stream;
  return 0;
}

int replay_graph(npbmz_t* h, int nsteps) {
  if (h->stream != nullptr) {
    for (int s = 0; s < nsteps; ++s) CK(h, cudaGraphLaunch(h->graph_exec, h->stream));
    return 0;
  }
  CK(h, cudaEventRecord(h->fence[0], nullptr));
  CK(h, cudaStreamWaitEvent(h->aux_stream, h->fence[0], 0));
  for (int s = 0; s < nsteps; ++s) CK(h, cudaGraphLaunch(h->graph_exec, h->aux_stream));
  CK(h, cudaEventRecord(h->fence[1], h->aux_stream));
  CK(h, cudaStreamWaitEvent(nullptr, h->fence[1], 0));
  return 0;
}

// ---- state check (the health word) ----------------------------------------
// Every step's primitive kernel checks the state entering that step; at the
// end of a call k_state_check checks the state the call leaves.  The word is
// cleared when a call starts and read once when it ends.
int health_begin(npbmz_t* h) {
  CK(h, cudaMemsetAsync(h->health_d, 0, sizeof(unsigned long long), h->stream));
  CK(h, cudaMemsetAsync(h->health_d + 1, 0xFF, sizeof(unsigned long long), h->stream));
  return 0;
}

// Enqueue the final check and the read-back (the caller synchronises).
int health_read(npbmz_t* h) {
  launch_state_check(fields(h), h->wpts_d, h->nwpts, h->stream);
  CKL(h);
  CK(h, cudaMemcpyAsync(h->health_h, h->health_d, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
  return 0;
}

// After the stream is synchronised: NPBMZ_ERR_STATE with the first bad point
// when the state has a non-positive or non-finite density or a non-finite
// value, and for SP also a non-positive pressure (SP takes its square root,
// src/SP/rhs.jl:84-88; BT never does, and the reference carries such a state
// on: npbmz_state_check reports it).
int health_verdict(npbmz_t* h, const char* what) {
  const unsigned long long bits = h->health_h[0], p = h->health_h[1];
  h->health_bits = (unsigned)bits;
  h->health_point = bits ? (int64_t)p : -1;
  const unsigned fatal = HEALTH_DENSITY | HEALTH_NONFINITE | (h->kind == NPBMZ_SP ? HEALTH_PRESSURE : 0u);
  if (!(bits & fatal)) return 0;
  int z = 0;
  while (z + 1 < h->nzones && (unsigned long long)h->zh[z + 1].off <= p) ++z;
  const ZoneDev& d = h->zh[z];
  const int64_t q = (int64_t)p - d.off;
  std::string kinds;
  if (bits & HEALTH_DENSITY) kinds += "non-positive or non-finite density";
  if (bits & HEALTH_NONFINITE) kinds += std::string(kinds.empty() ? "" : " and ") + "a non-finite value";
  if (bits & HEALTH_PRESSURE)
    kinds += std::string(kinds.empty() ? "" : " and ") + "non-positive pressure (rho E - |rho v|^2 / (2 rho))";
  fail(h, "state check failed after %s: %s in u; first bad point zone %d (i, j, k) = (%d, %d, %d)", what,
       kinds.c_str(), z, (int)(q % d.nx), (int)((q / d.nx) % d.ny), (int)(q / ((int64_t)d.nx * d.ny)));
  return NPBMZ_ERR_STATE;
}

// Kernel launches of one npbmz_step step: exch_qbc, then per batch (all
// zones, each zone with PERZONE, each zone group in the grouped graph) the
// primitive kernel, compute_rhs and the three sweeps (two kernels each when
// the FP32 solves are refined).
int count_launches(npbmz_t* h) {
  const bool refined = (h->flags & NPBMZ_MIXED) && !(h->flags & NPBMZ_FP32_NOREFINE);
  // prim, its x-line-major copy (double-float compute_rhs), compute_rhs,
  // two kernels per refined sweep and the x result's copy back
  const int adi = 2 + (h->pfx && !h->copy_fusion ? 1 : 0) + 3 * (refined ? 2 : 1) + (h->rdx ? 1 : 0);
  int batches = 1;
  if (h->flags & NPBMZ_PERZONE) batches = h->nzones;
  else if ((h->flags & NPBMZ_GRAPH) && h->ngroups > 1 && !(h->flags & NPBMZ_EXACT)) batches = h->ngroups;
  return (h->nzones > 1 ? 1 : 0) + adi * batches;
}

int ensure_stage(npbmz_t* h, size_t elems) {
  if (elems <= h->stage_elems) return 0;
  if (h->stage) { cudaFree(h->stage); h->device_bytes -= (int64_t)(h->stage_elems * sizeof(double)); }
  h->stage = nullptr;
  h->stage_elems = 0;
  if (dalloc(h, &h->stage, elems)) return -1;
  h->stage_elems = elems;
  return 0;
}

double* field_ptr(npbmz_t* h, int field) {
  return field == NPBMZ_U ? h->u : field == NPBMZ_RHS ? h->rhs : h->forcing;
}

// Reference-array geometry of one zone: extents (fastest first, elements)
// and the position of point (0,0,0) inside the halo.
struct RefBox {
  int64_t di, dj, dk;
  int oi, oj, ok;
};

RefBox ref_box(int kind, int field, const ZoneDev& z) {
  const int64_t IMAX = z.nx + 1, JMAX = z.ny + 1, KMAX = z.nz + 1;
  if (kind == NPBMZ_BT) {
    if (field == NPBMZ_U) return {IMAX + 4, JMAX + 4, KMAX + 4, 2, 2, 2};
    if (field == NPBMZ_RHS) return {IMAX + 1, JMAX + 1, KMAX + 1, 1, 1, 1};
    return {IMAX, JMAX, KMAX, 0, 0, 0};
  }
  const int64_t IMAXP = (IMAX / 2) * 2 + 1, JMAXP = (JMAX / 2) * 2 + 1;
  if (field == NPBMZ_U) return {IMAXP + 4, JMAXP + 4, KMAX + 4, 2, 2, 2};
  return {IMAXP, JMAXP, KMAX, 0, 0, 0};
}

// Copy the interior box of one zone's reference array between host memory
// and the compact staging order (BT: [k][j][i][m], SP: [m][k][j][i]); the
// halo of the host array is neither read nor written.
int ref_box_copy(npbmz_t* h, int zone, int field, double* host_zone, double* stage_zone, cudaMemcpyKind kind) {
  const ZoneDev& z = h->zh[zone];
  const RefBox b = ref_box(h->kind, field, z);
  const int vars = h->kind == NPBMZ_BT ? 1 : 5;
  const size_t w = h->kind == NPBMZ_BT ? 5 : 1;  // doubles per i step in the host array
  const int64_t np = (int64_t)z.nx * z.ny * z.nz;
  for (int m = 0; m < vars; ++m) {
    double* hz = host_zone + (h->kind == NPBMZ_BT ? 0 : (int64_t)m * b.di * b.dj * b.dk);
    double* sz = stage_zone + (h->kind == NPBMZ_BT ? 0 : m * np);
    cudaMemcpy3DParms p;
    std::memset(&p, 0, sizeof(p));
    cudaPitchedPtr hp = make_cudaPitchedPtr(hz, w * b.di * sizeof(double), w * b.di, b.dj);
    cudaPitchedPtr sp = make_cudaPitchedPtr(sz, w * z.nx * sizeof(double), w * z.nx, z.ny);
    const cudaPos hpos = make_cudaPos(w * b.oi * sizeof(double), b.oj, b.ok);
    if (kind == cudaMemcpyHostToDevice) { p.srcPtr = hp; p.srcPos = hpos; p.dstPtr = sp; }
    else { p.srcPtr = sp; p.dstPtr = hp; p.dstPos = hpos; }
    p.extent = make_cudaExtent(w * z.nx * sizeof(double), z.ny, z.nz);
    p.kind = kind;
    CK(h, cudaMemcpy3DAsync(&p, h->stream));
  }
  return 0;
}

int transfer(npbmz_t* h, int zone, int field, int layout, void* host, int dir, bool sync) {
  if (!h) return fail(nullptr, "null handle");
  if (field < 0 || field > 2) return fail(h, "bad field %d", field);
  if (layout != NPBMZ_LAYOUT_DENSE && layout != NPBMZ_LAYOUT_REF) return fail(h, "bad layout %d", layout);
  if (zone < -1 || zone >= h->nzones) return fail(h, "bad zone %d", zone);
  if (!host) return fail(h, "null host buffer");
  if (dir == 0 && field != NPBMZ_U) h->bnd_dirty = true;
  const std::vector<int64_t>& so = h->soff_h[layout][field];
  const int zlo = zone < 0 ? 0 : zone, zn = zone < 0 ? h->nzones : 1;
  const int64_t first = so[zlo], count = so[zlo + zn] - first;
  double* planes = field_ptr(h, field);
  const Fields F = fields(h);
  // Page-locked (mapped) host memory: one kernel reads / writes it directly.
  cudaPointerAttributes attr;
  std::memset(&attr, 0, sizeof(attr));
  if (cudaPointerGetAttributes(&attr, host) == cudaSuccess && attr.type == cudaMemoryTypeHost && attr.devicePointer) {
    launch_convert(F, planes, reinterpret_cast<double*>(attr.devicePointer), h->soff_d[layout][field], first, zlo, zn,
                   h->max_np, h->kind, field, layout, dir, h->stream);
    CKL(h);
  } else {
    cudaGetLastError();  // cudaPointerGetAttributes on pageable memory is not an error to keep
    if (ensure_stage(h, (size_t)so[h->nzones])) return -1;
    if (dir == 0) {
      CK(h, cudaMemcpyAsync(h->stage + first, host, count * sizeof(double), cudaMemcpyHostToDevice, h->stream));
      launch_convert(F, planes, h->stage, h->soff_d[layout][field], 0, zlo, zn, h->max_np, h->kind, field, layout, 0,
                     h->stream);
      CKL(h);
    } else if (layout == NPBMZ_LAYOUT_DENSE) {
      launch_convert(F, planes, h->stage, h->soff_d[layout][field], 0, zlo, zn, h->max_np, h->kind, field, layout, 1,
                     h->stream);
      CKL(h);
      CK(h, cudaMemcpyAsync(host, h->stage + first, count * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    } else {
      // compact staging (dense offsets), then the interior box of each zone
      const std::vector<int64_t>& sd = h->soff_h[NPBMZ_LAYOUT_DENSE][field];
      launch_convert(F, planes, h->stage, h->soff_d[NPBMZ_LAYOUT_DENSE][field], 0, zlo, zn, h->max_np, h->kind, field,
                     2, 1, h->stream);
      CKL(h);
      double* hb = reinterpret_cast<double*>(host);
      for (int z = zlo; z < zlo + zn; ++z)
        if (ref_box_copy(h, z, field, hb + (so[z] - first), h->stage + sd[z], cudaMemcpyDeviceToHost)) return -1;
    }
  }
  if (sync) CK(h, cudaStreamSynchronize(h->stream));
  return 0;
}

// ---- seeded coefficients ----------------------------------------------------
uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void exact_host(double xi, double eta, double zeta, const double* ce, double out[5]) {
  for (int m = 0; m < 5; ++m) {
    const double* c = ce + 13 * m;
    out[m] = c[0] + xi * (c[1] + xi * (c[4] + xi * (c[7] + xi * c[10]))) +
             eta * (c[2] + eta * (c[5] + eta * (c[8] + eta * c[11]))) +
             zeta * (c[3] + zeta * (c[6] + zeta * (c[9] + zeta * c[12])));
  }
}

bool state_ok(const double u[5], double margin) {
  if (!(u[0] > 0.0)) return false;
  const double ke = 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / u[0];
  return u[4] - ke >= margin * u[4] && u[4] > 0.0;
}

}  // namespace

namespace npbmz {
// Error text for calls without a handle, reported by npbmz_last_error(NULL).
void set_global_error(const char* msg) { g_create_error = msg; }
}  // namespace npbmz

// ---- discrete adjoint of the BT step ----------------------------------------
namespace {

// Device buffers of one npbmz_adjoint call, freed on every exit path.
struct AdjointBuffers {
  std::vector<void*> owned;
  ~AdjointBuffers() {
    for (void* p : owned) cudaFree(p);
  }
  template <typename T>
  int get(npbmz_t* h, T** p, size_t count) {
    *p = nullptr;
    CK(h, cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T)));
    owned.push_back(*p);
    return 0;
  }
};

// All zones' planes <-> a host array of the dense layout ([m][k][j][i] per
// zone, zones back to back), synchronous.
int dense_io(npbmz_t* h, double* planes, double* host, int dir) {
  const std::vector<int64_t>& so = h->soff_h[NPBMZ_LAYOUT_DENSE][NPBMZ_U];
  const int64_t total = so[h->nzones];
  if (ensure_stage(h, (size_t)total)) return -1;
  const Fields F = fields(h);
  const int64_t* soff = h->soff_d[NPBMZ_LAYOUT_DENSE][NPBMZ_U];
  if (dir == 0) {
    CK(h, cudaMemcpyAsync(h->stage, host, total * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    launch_convert(F, planes, h->stage, soff, 0, 0, h->nzones, h->max_np, h->kind, NPBMZ_U, 0, 0, h->stream);
    CKL(h);
  } else {
    launch_convert(F, planes, h->stage, soff, 0, 0, h->nzones, h->max_np, h->kind, NPBMZ_U, 0, 1, h->stream);
    CKL(h);
    CK(h, cudaMemcpyAsync(host, h->stage, total * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  }
  CK(h, cudaStreamSynchronize(h->stream));
  return 0;
}

// Forward step n recomputed from u_n (in h->u): h->u becomes v = exch_qbc(u_n)
// (the state every Jacobian of the step is taken at), x[d] the solution of
// sweep d.  The update u_{n+1} = v + x[2] is not applied.
int adjoint_recompute(npbmz_t* h, double* const x[3]) {
  const size_t bytes = 5 * (size_t)h->NP * sizeof(double);
  if (phase_exch(h)) return -1;
  if (phase_prim(h, -1)) return -1;
  if (phase_rhs(h, -1, false, false)) return -1;
  for (int dir = 0; dir < 3; ++dir) {
    if (phase_solve(h, dir, -1, 0)) return -1;
    CK(h, cudaMemcpyAsync(x[dir], h->rhs, bytes, cudaMemcpyDeviceToDevice, h->stream));
  }
  return 0;
}

// SP: step n recomputed from u_n (FP64): h->u becomes v = exch_qbc(u_n),
// r0 the compute_rhs output before txinvr, y[d] sweep d's untransformed
// solution (its input at the line ends).
int adjoint_recompute_sp(npbmz_t* h, double* const y[3], double* r0, double* scr) {
  const size_t bytes = 5 * (size_t)h->NP * sizeof(double);
  if (phase_exch(h)) return -1;
  if (phase_prim(h, -1)) return -1;
  if (phase_rhs(h, -1, false, false)) return -1;
  CK(h, cudaMemcpyAsync(r0, h->rhs, bytes, cudaMemcpyDeviceToDevice, h->stream));
  if (phase_rhs(h, -1, true, false)) return -1;
  const Fields F = fields(h);
  for (int dir = 0; dir < 3; ++dir) {
    CK(h, cudaMemcpyAsync(y[dir], h->rhs, bytes, cudaMemcpyDeviceToDevice, h->stream));
    if (line_launches(h, dir, -1, [&](int lo, int hi, int tpb) {
          sp_fwd_launch_solve(dir, F, h->K, h->wline_d[dir] + lo, hi - lo, tpb, y[dir], scr, h->nlines[dir],
                              h->stream);
          CKL(h);
          return 0;
        }))
      return -1;
    sp_fwd_launch_post(dir, F, h->K, h->wpts_d, h->nwpts, y[dir], h->stream);
    CKL(h);
  }
  return 0;
}

// SP: ub <- (d u_{n+1} / d u_n)^T ub, fb += (d u_{n+1} / d forcing)^T ub,
// after adjoint_recompute_sp of step n.
int adjoint_back_step_sp(npbmz_t* h, double* const y[3], const double* r0, double* ub, double* vb, double* yb,
                         double* fb, double* scr) {
  const size_t bytes = 5 * (size_t)h->NP * sizeof(double);
  const Fields F = fields(h);
  CK(h, cudaMemcpyAsync(vb, ub, bytes, cudaMemcpyDeviceToDevice, h->stream));
  adj_launch_seed(F, h->wpts_d, h->nwpts, ub, nullptr, yb, nullptr, 1, h->stream);
  CKL(h);
  for (int dir = 2; dir >= 0; --dir) {
    if (line_launches(h, dir, -1, [&](int lo, int hi, int tpb) {
          adj_launch_sp_solve(dir, F, h->K, h->wline_d[dir] + lo, hi - lo, tpb, yb, y[dir], vb, scr, h->nlines[dir],
                              h->stream);
          CKL(h);
          return 0;
        }))
      return -1;
  }
  adj_launch_sp_txinvr(F, h->K, h->wpts_d, h->nwpts, yb, r0, vb, h->stream);
  CKL(h);
  adj_launch_rhs(F, h->K, h->wpts_d, h->nwpts, yb, vb, fb, h->stream);
  CKL(h);
  CK(h, cudaMemcpyAsync(ub, vb, bytes, cudaMemcpyDeviceToDevice, h->stream));
  if (h->nzones > 1) {
    adj_launch_exch(F, h->nbr_d, h->nzones, h->max_face, vb, ub, h->stream);
    CKL(h);
  }
  return 0;
}

// ub <- (d u_{n+1} / d u_n)^T ub and fb += (d u_{n+1} / d forcing)^T ub,
// after adjoint_recompute of step n.
int adjoint_back_step(npbmz_t* h, double* const x[3], double* ub, double* vb, double* yb, double* fb, double* scr) {
  const size_t bytes = 5 * (size_t)h->NP * sizeof(double);
  const Fields F = fields(h);
  // add: u_{n+1} = v + x3 on the interior
  CK(h, cudaMemcpyAsync(vb, ub, bytes, cudaMemcpyDeviceToDevice, h->stream));
  adj_launch_seed(F, h->wpts_d, h->nwpts, ub, nullptr, yb, nullptr, 1, h->stream);
  CKL(h);
  // the sweeps in reverse order
  for (int dir = 2; dir >= 0; --dir) {
    if (line_launches(h, dir, -1, [&](int lo, int hi, int tpb) {
          adj_launch_solve(dir, F, h->K, h->wline_d[dir] + lo, hi - lo, tpb, yb, x[dir], vb, scr, h->nlines[dir],
                           h->stream);
          CKL(h);
          return 0;
        }))
      return -1;
  }
  // compute_rhs (yb is now the adjoint of rhs)
  adj_launch_rhs(F, h->K, h->wpts_d, h->nwpts, yb, vb, fb, h->stream);
  CKL(h);
  // exch_qbc
  CK(h, cudaMemcpyAsync(ub, vb, bytes, cudaMemcpyDeviceToDevice, h->stream));
  if (h->nzones > 1) {
    adj_launch_exch(F, h->nbr_d, h->nzones, h->max_face, vb, ub, h->stream);
    CKL(h);
  }
  return 0;
}

int adjoint_run(npbmz_t* h, int nsteps, int every, const double* u_target, double* J, double* grad_forcing,
                double* grad_u0) {
  const cudaStream_t s = h->stream;
  const size_t F5 = 5 * (size_t)h->NP, bytes = F5 * sizeof(double);
  const int nck = (nsteps + every - 1) / every;
  const int seglen = std::min(every, nsteps);
  int64_t scr_elems = 0;
  for (int dir = 0; dir < 3; ++dir) {
    int maxlen = 0;
    for (const ZoneDev& z : h->zh) maxlen = std::max(maxlen, zone_line_len(z, dir));
    scr_elems = std::max<int64_t>(scr_elems, 30 * (int64_t)maxlen * h->nlines[dir]);
  }
  AdjointBuffers B;
  const bool sp = h->kind == NPBMZ_SP;
  double *ck, *seg, *x[3], *yb, *vb, *ub, *fb, *tgt, *scr, *part, *r0 = nullptr;
  if (B.get(h, &ck, (size_t)nck * F5) || B.get(h, &seg, (size_t)seglen * F5) || B.get(h, &x[0], F5) ||
      B.get(h, &x[1], F5) || B.get(h, &x[2], F5) || B.get(h, &yb, F5) || B.get(h, &vb, F5) || B.get(h, &ub, F5) ||
      B.get(h, &fb, F5) || B.get(h, &tgt, F5) || B.get(h, &scr, (size_t)scr_elems) || B.get(h, &part, 5 * (size_t)h->nwpts) ||
      (sp && B.get(h, &r0, F5)))
    return -1;
  CK(h, cudaMemsetAsync(fb, 0, bytes, s));
  CK(h, cudaMemsetAsync(tgt, 0, bytes, s));
  CK(h, cudaMemcpyAsync(ck, h->u, bytes, cudaMemcpyDeviceToDevice, s));
  int rc = 0;
  // forward pass, keeping u every `every` steps
  for (int n = 0; n < nsteps && !rc; ++n) {
    if (n % every == 0 && n > 0) rc = cudaMemcpyAsync(ck + (size_t)(n / every) * F5, h->u, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess;
    if (!rc) rc = one_step(h, false, nullptr);
  }
  // objective: J = 1/2 sum over every stored point of (u_N - u_target)^2
  if (!rc) rc = dense_io(h, tgt, const_cast<double*>(u_target), 0);
  if (!rc) {
    adj_launch_seed(fields(h), h->wpts_d, h->nwpts, h->u, tgt, ub, part, 0, s);
    rc = cudaGetLastError() != cudaSuccess;
  }
  if (!rc) {
    std::vector<double> ph(5 * (size_t)h->nwpts);
    rc = cudaMemcpyAsync(ph.data(), part, ph.size() * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
         cudaStreamSynchronize(s) != cudaSuccess;
    double sum = 0.0;
    for (double v : ph) sum += v;
    if (J) *J = 0.5 * sum;
  }
  // reverse pass, one checkpoint segment at a time
  for (int c = nck - 1; c >= 0 && !rc; --c) {
    const int n0 = c * every, n1 = std::min(n0 + every, nsteps);
    rc = cudaMemcpyAsync(h->u, ck + (size_t)c * F5, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess;
    for (int n = n0; n < n1 && !rc; ++n) {
      rc = cudaMemcpyAsync(seg + (size_t)(n - n0) * F5, h->u, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess;
      if (!rc && n + 1 < n1) rc = one_step(h, false, nullptr);
    }
    for (int n = n1 - 1; n >= n0 && !rc; --n) {
      rc = cudaMemcpyAsync(h->u, seg + (size_t)(n - n0) * F5, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess;
      if (sp) {
        if (!rc) rc = adjoint_recompute_sp(h, x, r0, scr);
        if (!rc) rc = adjoint_back_step_sp(h, x, r0, ub, vb, yb, fb, scr);
      } else {
        if (!rc) rc = adjoint_recompute(h, x);
        if (!rc) rc = adjoint_back_step(h, x, ub, vb, yb, fb, scr);
      }
    }
  }
  if (!rc && grad_forcing) rc = dense_io(h, fb, grad_forcing, 1);
  if (!rc && grad_u0) rc = dense_io(h, ub, grad_u0, 1);
  // the handle's state is u_0 again
  const bool restored = cudaMemcpyAsync(h->u, ck, bytes, cudaMemcpyDeviceToDevice, s) == cudaSuccess &&
                        cudaStreamSynchronize(s) == cudaSuccess;
  if (rc) {
    if (h->err.empty()) h->err = std::string("adjoint failed: ") + cudaGetErrorString(cudaGetLastError());
    return -1;
  }
  if (!restored) return fail(h, "adjoint: restoring u_0 failed: %s", cudaGetErrorString(cudaGetLastError()));
  return 0;
}

}  // namespace

// =============================== C ABI ======================================
extern "C" {

int npbmz_zone_setup(int kind, int gx, int gy, int gz, int xz, int yz, double ratio, int* nx, int* ny, int* nz,
                     int* nbr) {
  if (xz < 1 || yz < 1 || gx < 3 || gy < 3 || gz < 3 || !nx || !ny || !nz || !nbr) return -1;
  std::vector<long> x_end(xz), y_end(yz), x_start(xz), y_start(yz), x_size(xz), y_size(yz);
  const bool stretch = std::fabs(ratio - 1.0e0) > 1.0e-10 && (kind == NPBMZ_SP || (xz > 1 && yz > 1));
  if (stretch) {
    // geometric zone widths, src/BT/zone_setup.jl:5-22
    const double x_r = std::exp(std::log(ratio) / (xz - 1));
    const double y_r = std::exp(std::log(ratio) / (yz - 1));
    const double x_smallest = (double)gx * (x_r - 1.0e0) / (std::pow(x_r, xz) - 1.0e0);
    const double y_smallest = (double)gy * (y_r - 1.0e0) / (std::pow(y_r, yz) - 1.0e0);
    for (int i = 1; i <= xz; ++i)
      x_end[i - 1] = (long)std::trunc(x_smallest * (std::pow(x_r, i) - 1.0e0) / (x_r - 1.0e0) + 0.45e0);
    for (int j = 1; j <= yz; ++j)
      y_end[j - 1] = (long)std::trunc(y_smallest * (std::pow(y_r, j) - 1.0e0) / (y_r - 1.0e0) + 0.45e0);
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
      const int zn = (i - 1) + (j - 1) * xz;
      nx[zn] = (int)x_size[i - 1];
      ny[zn] = (int)y_size[j - 1];
      nz[zn] = gz;
      nbr[4 * zn + 0] = (i - 2 + xz) % xz + (j - 1) * xz;
      nbr[4 * zn + 1] = i % xz + (j - 1) * xz;
      nbr[4 * zn + 2] = (i - 1) + ((j - 2 + yz) % yz) * xz;
      nbr[4 * zn + 3] = (i - 1) + (j % yz) * xz;
    }
  return 0;
}

int npbmz_seeded_coefficients(uint64_t seed, int nzones, const int* nx, const int* ny, const int* nz, int gx, int gy,
                              int gz, int xz, int yz, double* ce) {
  if (!nx || !ny || !nz || !ce || nzones < 1) return -1;
  uint64_t s = seed;
  for (int e = 0; e < 65; ++e) {
    const double r = (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);  // [0, 1)
    ce[e] = 0.5 + 1.5 * r;
  }
  const Consts K = make_consts(1.0, gx, gy, gz, xz, yz);
  int mx = 0, my = 0, mz = 0;
  for (int z = 0; z < nzones; ++z) { mx = std::max(mx, nx[z]); my = std::max(my, ny[z]); mz = std::max(mz, nz[z]); }
  const double margin = 0.25;
  for (int e = 0; e < 40; ++e) {
    bool ok = true;
    double st[5], P1[2][5], P2[2][5], P3[2][5], ui[5];
    for (int k = 0; k < mz && ok; ++k)
      for (int j = 0; j < my && ok; ++j)
        for (int i = 0; i < mx && ok; ++i) {
          const double xi = (double)i * K.dnxm1, eta = (double)j * K.dnym1, zeta = (double)k * K.dnzm1;
          exact_host(xi, eta, zeta, ce, st);
          if (!state_ok(st, margin)) { ok = false; break; }
          exact_host(0.0, eta, zeta, ce, P1[0]); exact_host(1.0, eta, zeta, ce, P1[1]);
          exact_host(xi, 0.0, zeta, ce, P2[0]); exact_host(xi, 1.0, zeta, ce, P2[1]);
          exact_host(xi, eta, 0.0, ce, P3[0]); exact_host(xi, eta, 1.0, ce, P3[1]);
          for (int m = 0; m < 5; ++m) {
            const double Pxi = xi * P1[1][m] + (1.0 - xi) * P1[0][m];
            const double Peta = eta * P2[1][m] + (1.0 - eta) * P2[0][m];
            const double Pzeta = zeta * P3[1][m] + (1.0 - zeta) * P3[0][m];
            ui[m] = Pxi + Peta + Pzeta - Pxi * Peta - Pxi * Pzeta - Peta * Pzeta + Pxi * Peta * Pzeta;
          }
          if (!state_ok(ui, margin)) ok = false;
          for (int f = 0; f < 2 && ok; ++f)
            if (!state_ok(P1[f], margin) || !state_ok(P2[f], margin) || !state_ok(P3[f], margin)) ok = false;
        }
    if (ok) return e;
    for (int n = 0; n < 13; ++n) ce[4 * 13 + n] *= 2.0;
  }
  return -2;
}

int npbmz_create(int kind, int nzones, const int* nx, const int* ny, const int* nz, const int* nbr,
                 const double* params, int variant_flags, npbmz_t** out) {
  if (!out) return fail(nullptr, "out is null");
  *out = nullptr;
  if (kind != NPBMZ_BT && kind != NPBMZ_SP) return fail(nullptr, "kind must be NPBMZ_BT or NPBMZ_SP");
  if (nzones < 1 || !nx || !ny || !nz || !nbr || !params) return fail(nullptr, "bad geometry arguments");
  if ((variant_flags & NPBMZ_EXACT) && (variant_flags & (NPBMZ_MIXED | NPBMZ_FP32_NOREFINE)))
    return fail(nullptr, "NPBMZ_EXACT and the FP32 line-solve variants are exclusive");
  for (int z = 0; z < nzones; ++z) {
    // src/BT/make_set.jl:100-105 aborts on a cell size <= 2
    if (nx[z] < 3 || ny[z] < 3 || nz[z] < 3) return fail(nullptr, "zone %d: size %dx%dx%d, minimum is 3", z, nx[z], ny[z], nz[z]);
    if ((int64_t)nx[z] * ny[z] * nz[z] > (1 << 30)) return fail(nullptr, "zone %d too large", z);
    for (int f = 0; f < 4; ++f)
      if (nbr[4 * z + f] < NPBMZ_REMOTE || nbr[4 * z + f] >= nzones) return fail(nullptr, "zone %d: bad neighbour", z);
  }
  bool remote = false;
  for (int z = 0; z < nzones; ++z)
    for (int f = 0; f < 4; ++f) {
      const int o = nbr[4 * z + f];
      if (o == NPBMZ_REMOTE) { remote = true; continue; }  // its size is the exchange plan's business
      const bool ok = f < 2 ? (ny[o] == ny[z] && nz[o] == nz[z]) : (nx[o] == nx[z] && nz[o] == nz[z]);
      if (!ok) return fail(nullptr, "zone %d: neighbour face sizes do not match", z);
    }
  npbmz_t* h = new npbmz_t();
  h->kind = kind;
  h->nzones = nzones;
  h->flags = variant_flags;
  h->K = make_consts(params[0], (int)params[1], (int)params[2], (int)params[3], (int)params[4], (int)params[5]);
  h->nbr.assign(nbr, nbr + 4 * nzones);
  h->has_remote = remote;
  h->zh.resize(nzones);
  int64_t off = 0, lines[3] = {0, 0, 0};
  int64_t scratch_elems = 0;
  for (int z = 0; z < nzones; ++z) {
    ZoneDev& d = h->zh[z];
    d.nx = nx[z]; d.ny = ny[z]; d.nz = nz[z]; d.pad = 0;
    d.off = off;
    const int64_t np = (int64_t)d.nx * d.ny * d.nz;
    off += (np + 31) / 32 * 32;
    for (int dir = 0; dir < 3; ++dir) {
      d.lineoff[dir] = lines[dir];
      lines[dir] += zone_lines(d, dir);
    }
    h->max_np = std::max<int>(h->max_np, (int)np);
    h->max_face = std::max(h->max_face, 5 * std::max(d.nx, d.ny) * d.nz);
  }
  h->NP = std::max<int64_t>(off, 32);
  for (int dir = 0; dir < 3; ++dir) {
    h->nlines[dir] = lines[dir];
    int maxlen = 0;
    for (int z = 0; z < nzones; ++z) maxlen = std::max(maxlen, zone_line_len(h->zh[z], dir));
    scratch_elems = std::max<int64_t>(scratch_elems, (int64_t)maxlen * lines[dir]);
  }
  // line scratch: BT keeps 25 values per point (C'; 30 with the FP32
  // forward rhs of the refined mixed solve), SP 6 (l4, l5 of 3 systems)
  const bool refined = (variant_flags & NPBMZ_MIXED) && !(variant_flags & NPBMZ_FP32_NOREFINE);
  const int per = kind == NPBMZ_BT ? (refined ? 30 : 25) : (refined ? 11 : 6);
  if (variant_flags & NPBMZ_FP32_NOREFINE) variant_flags |= NPBMZ_MIXED;
  h->flags = variant_flags;
  const size_t esz = (variant_flags & NPBMZ_MIXED) ? sizeof(float) : sizeof(double);
  h->scratch_bytes = (size_t)scratch_elems * per * esz;

  int rc = 0;
  rc |= dalloc(h, &h->zones_d, nzones);
  rc |= dalloc(h, &h->health_d, 2);
  if (!rc && cudaMallocHost((void**)&h->health_h, 2 * sizeof(unsigned long long)) != cudaSuccess) rc = -1;
  rc |= dalloc(h, &h->nbr_d, 4 * (size_t)nzones);
  rc |= dalloc(h, &h->u, 5 * (size_t)h->NP);
  rc |= dalloc(h, &h->rhs, 5 * (size_t)h->NP);
  rc |= dalloc(h, &h->forcing, 5 * (size_t)h->NP);
  rc |= dalloc(h, &h->prim, (size_t)PR_COUNT * h->NP);
  rc |= dalloc(h, &h->uex, 5 * (size_t)h->NP);
  if (variant_flags & NPBMZ_MIXED) rc |= dalloc(h, &h->xw, 5 * (size_t)h->NP);
  if (refined) rc |= dalloc(h, &h->primf, (size_t)(kind == NPBMZ_BT ? (int)PF_COUNT : (int)PS_COUNT) * h->NP);
  if (!(variant_flags & NPBMZ_EXACT) && make_lin_weights(h->K, h->lw)) {
    h->dfrhs = refined && !(variant_flags & NPBMZ_REFINE_FP64) && (variant_flags & NPBMZ_RHS_DF);
    if (h->dfrhs) {
      make_rhs_df_consts(h->K, h->lw, h->rdc);
      rc |= dalloc(h, &h->ud, 5 * (size_t)h->NP);
      rc |= dalloc(h, &h->xd, (size_t)XD_COUNT * h->NP);
      rc |= dalloc(h, &h->fd, 5 * (size_t)h->NP);
    } else {
      make_rhs_f64_consts(h->K, h->lw, h->rc64);
      rc |= dalloc(h, &h->flux, (size_t)PX_COUNT * h->NP);
      rc |= dalloc(h, &h->fdt, 5 * (size_t)h->NP);
    }
    if (refined && !(variant_flags & NPBMZ_REFINE_FP64)) {
      rc |= dalloc(h, &h->rdf, 10 * (size_t)h->NP);
      int maxnx = 0;
      for (int z = 0; z < nzones; ++z) maxnx = std::max(maxnx, nx[z]);
      const size_t xpts = (size_t)maxnx * (size_t)std::max<int64_t>(lines[0], 1);
      rc |= dalloc(h, &h->pfx, (size_t)PF_COUNT * xpts);
      rc |= dalloc(h, &h->rdx, 10 * xpts);
      rc |= dalloc(h, &h->x0x, 5 * xpts);
    }
  }
  if (!rc) {
    if (cudaMalloc(&h->scratch, std::max<size_t>(h->scratch_bytes, 16)) != cudaSuccess) rc = fail(h, "scratch alloc failed");
    else h->device_bytes += (int64_t)h->scratch_bytes;
  }
  if (!rc && cudaMemcpy(h->zones_d, h->zh.data(), nzones * sizeof(ZoneDev), cudaMemcpyHostToDevice) != cudaSuccess) rc = -1;
  if (!rc && cudaMemcpy(h->nbr_d, nbr, 4 * nzones * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) rc = -1;
  if (!rc && h->rdf && fast::configure_kernels()) rc = fail(h, "cudaFuncSetAttribute failed: %s", cudaGetErrorString(cudaGetLastError()));
  if (!rc) rc = build_work_lists(h);
  if (!rc) rc = build_line_lists(h);
  // staging offsets per layout and field
  for (int layout = 0; layout < 2 && !rc; ++layout)
    for (int field = 0; field < 3 && !rc; ++field) {
      std::vector<int64_t>& so = h->soff_h[layout][field];
      so.assign(nzones + 1, 0);
      for (int z = 0; z < nzones; ++z) {
        const ZoneDev& d = h->zh[z];
        const int64_t n = layout == NPBMZ_LAYOUT_DENSE ? 5 * (int64_t)d.nx * d.ny * d.nz : ref_elems(kind, field, d);
        so[z + 1] = so[z] + n;
      }
      rc = dalloc(h, &h->soff_d[layout][field], (size_t)nzones + 1);
      if (!rc && cudaMemcpy(h->soff_d[layout][field], so.data(), so.size() * sizeof(int64_t), cudaMemcpyHostToDevice) !=
                     cudaSuccess)
        rc = -1;
    }
  if (!rc) {
    // fields start defined: u = (1, 0, 0, 0, 1) on padding keeps the
    // primitive kernel finite there; rhs and forcing zero.
    const Fields F = fields(h);
    (void)F;
    for (int m = 0; m < 5; ++m) launch_fill(h->u + m * h->NP, h->NP, (m == 0 || m == 4) ? 1.0 : 0.0, nullptr);
    if (cudaMemset(h->rhs, 0, 5 * h->NP * sizeof(double)) != cudaSuccess) rc = -1;
    if (cudaMemset(h->forcing, 0, 5 * h->NP * sizeof(double)) != cudaSuccess) rc = -1;
    if (cudaMemset(h->prim, 0, PR_COUNT * h->NP * sizeof(double)) != cudaSuccess) rc = -1;
    if (cudaMemset(h->uex, 0, 5 * h->NP * sizeof(double)) != cudaSuccess) rc = -1;
    if (h->dfrhs) {
      if (cudaMemset(h->ud, 0, 5 * h->NP * sizeof(float2)) != cudaSuccess) rc = -1;
      if (cudaMemset(h->xd, 0, XD_COUNT * h->NP * sizeof(float2)) != cudaSuccess) rc = -1;
      if (cudaMemset(h->fd, 0, 5 * h->NP * sizeof(float2)) != cudaSuccess) rc = -1;
    }
    if (cudaDeviceSynchronize() != cudaSuccess) rc = -1;
  }
  if (rc) {
    const std::string msg = h->err.empty() ? std::string("device allocation or copy failed: ") +
                                                 cudaGetErrorString(cudaGetLastError())
                                           : h->err;
    npbmz_destroy(h);
    return fail(nullptr, "%s", msg.c_str());
  }
  cudaStream_t s;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess) { h->stream = s; h->own_stream = true; }
  h->launches_per_step = count_launches(h);
  *out = h;
  // the step graph of a batched FMA-build step runs in zone-group branches
  if ((variant_flags & NPBMZ_GRAPH) && !(variant_flags & (NPBMZ_EXACT | NPBMZ_PERZONE)) && nzones >= 8 &&
      npbmz_set_step_groups(h, 2)) {
    const std::string msg = h->err;
    npbmz_destroy(h);
    *out = nullptr;
    return fail(nullptr, "%s", msg.c_str());
  }
  return 0;
}

int npbmz_setup(npbmz_t* h, const double* ce) {
  if (!h || !ce) return fail(h, "null argument");
  const Fields F = fields(h);
  launch_initialize(F, h->K, ce, h->wpts_d, h->nwpts, h->uex, h->stream);
  CKL(h);
  launch_exact_rhs(F, h->K, ce, h->wpts_d, h->nwpts, h->forcing, h->stream);
  CKL(h);
  // rhs starts as the forcing (its boundary values are never rewritten)
  h->bnd_dirty = true;
  if (flush_boundary(h)) return -1;
  CK(h, cudaStreamSynchronize(h->stream));
  return 0;
}

int npbmz_upload(npbmz_t* h, int zone, int field, int layout, const double* host) {
  return transfer(h, zone, field, layout, const_cast<double*>(host), 0, true);
}
int npbmz_download(npbmz_t* h, int zone, int field, int layout, double* host) {
  return transfer(h, zone, field, layout, host, 1, true);
}
int npbmz_upload_async(npbmz_t* h, int zone, int field, int layout, const double* host) {
  return transfer(h, zone, field, layout, const_cast<double*>(host), 0, false);
}
int npbmz_download_async(npbmz_t* h, int zone, int field, int layout, double* host) {
  return transfer(h, zone, field, layout, host, 1, false);
}

int npbmz_exch_qbc(npbmz_t* h) {
  if (!h) return fail(nullptr, "null handle");
  return phase_exch(h);
}

int npbmz_adi(npbmz_t* h, int zone) {
  if (!h) return fail(nullptr, "null handle");
  if (zone < -1 || zone >= h->nzones) return fail(h, "bad zone %d", zone);
  return run_adi(h, zone, false);
}

int npbmz_step(npbmz_t* h, int nsteps, double* norms) {
  if (!h) return fail(nullptr, "null handle");
  if (nsteps < 0) return fail(h, "nsteps < 0");
  if (norms && nsteps > h->norms_cap) {
    if (h->norms_d) { cudaFree(h->norms_d); h->device_bytes -= (int64_t)h->norms_cap * 10 * sizeof(double); }
    h->norms_d = nullptr;
    h->norms_cap = 0;
    if (dalloc(h, &h->norms_d, 10 * (size_t)std::max(nsteps, 1))) return -1;
    h->norms_cap = std::max(nsteps, 1);
  }
  if (h->flags & NPBMZ_GRAPH && !norms) {
    if (!h->graph_exec || h->graph_stream != h->stream)
      if (capture_step_graph(h)) return -1;
    if (flush_boundary(h)) return -1;
    if (health_begin(h) || replay_graph(h, nsteps)) return -1;
  } else {
    if (health_begin(h)) return -1;
    for (int s = 0; s < nsteps; ++s)
      if (one_step(h, norms != nullptr, norms ? h->norms_d + 10 * s : nullptr)) return -1;
    if (norms)
      CK(h, cudaMemcpyAsync(norms, h->norms_d, 10 * sizeof(double) * nsteps, cudaMemcpyDeviceToHost, h->stream));
  }
  if (health_read(h)) return -1;
  CK(h, cudaStreamSynchronize(h->stream));
  return health_verdict(h, "the steps");
}

int npbmz_step_download(npbmz_t* h, int nsteps, int layout, double* host) {
  if (!h) return fail(nullptr, "null handle");
  if (nsteps < 1) return fail(h, "nsteps must be >= 1");
  if (!host) return fail(h, "null host buffer");
  if (layout != NPBMZ_LAYOUT_DENSE && layout != NPBMZ_LAYOUT_REF) return fail(h, "bad layout %d", layout);
  cudaPointerAttributes attr;
  std::memset(&attr, 0, sizeof(attr));
  const bool mapped = cudaPointerGetAttributes(&attr, host) == cudaSuccess && attr.type == cudaMemoryTypeHost &&
                      attr.devicePointer != nullptr;
  cudaGetLastError();
  if (!mapped || !(h->flags & NPBMZ_GRAPH) || !use_groups(h) || h->stream == nullptr) {
    // a failed state check still copies u out (and keeps its message)
    const int rc = npbmz_step(h, nsteps, nullptr);
    if (rc && rc != NPBMZ_ERR_STATE) return rc;
    const std::string msg = h->err;
    if (transfer(h, -1, NPBMZ_U, layout, host, 1, true)) return -1;
    if (rc) h->err = msg;
    return rc;
  }
  if (!h->graph_exec || h->graph_stream != h->stream)
    if (capture_step_graph(h)) return -1;
  if (flush_boundary(h)) return -1;
  if (health_begin(h)) return -1;
  if (nsteps > 1 && replay_graph(h, nsteps - 1)) return -1;
  CK(h, cudaGraphLaunch(h->graph_exec, h->stream));
  if (!h->io_stream) CK(h, cudaStreamCreateWithFlags(&h->io_stream, cudaStreamNonBlocking));
  if (!h->io_done) CK(h, cudaEventCreateWithFlags(&h->io_done, cudaEventDisableTiming));
  const Fields F = fields(h);
  for (int g = 0; g < h->ngroups; ++g) {
    const int z0 = h->grp_zone_off[g], nz = h->grp_zone_off[g + 1] - z0;
    CK(h, cudaStreamWaitEvent(h->io_stream, h->grp_out_ev[g], 0));
    launch_convert(F, h->u, reinterpret_cast<double*>(attr.devicePointer), h->soff_d[layout][NPBMZ_U], 0, 0, nz,
                   h->max_np, h->kind, NPBMZ_U, layout, 1, h->io_stream, h->grp_zones_d + z0);
    CKL(h);
  }
  CK(h, cudaEventRecord(h->io_done, h->io_stream));
  if (health_read(h)) return -1;
  CK(h, cudaStreamWaitEvent(h->stream, h->io_done, 0));
  CK(h, cudaStreamSynchronize(h->stream));
  return health_verdict(h, "the steps");
}

int npbmz_step_inout(npbmz_t* h, int nsteps, int layout, const double* host_in, double* host_out) {
  if (!h) return fail(nullptr, "null handle");
  if (nsteps < 1) return fail(h, "nsteps must be >= 1");
  if (!host_in || !host_out) return fail(h, "null host buffer");
  if (layout != NPBMZ_LAYOUT_DENSE && layout != NPBMZ_LAYOUT_REF) return fail(h, "bad layout %d", layout);
  auto mapped = [](const void* p) -> double* {
    cudaPointerAttributes a;
    std::memset(&a, 0, sizeof(a));
    const bool ok = cudaPointerGetAttributes(&a, p) == cudaSuccess && a.type == cudaMemoryTypeHost && a.devicePointer;
    cudaGetLastError();
    return ok ? reinterpret_cast<double*>(a.devicePointer) : nullptr;
  };
  double* din = mapped(host_in);
  double* dout = mapped(host_out);
  if (!din || !dout || !(h->flags & NPBMZ_GRAPH) || !use_groups(h) || h->stream == nullptr || h->has_remote) {
    // the same result in sequence: upload, steps with the copy-out
    if (transfer(h, -1, NPBMZ_U, layout, const_cast<double*>(host_in), 0, false)) return -1;
    return npbmz_step_download(h, nsteps, layout, host_out);
  }
  if (!h->graph_exec || h->graph_stream != h->stream)
    if (capture_step_graph(h)) return -1;
  if (!h->graph_inout || h->graph_stream != h->stream)
    if (capture_step_graph(h, true)) return -1;
  if (flush_boundary(h)) return -1;
  const std::vector<int64_t>& soh = h->soff_h[layout][NPBMZ_U];
  const size_t img = (size_t)soh[h->nzones];
  if (h->io_image_elems < img) {
    if (h->io_image) { cudaFree(h->io_image); h->device_bytes -= (int64_t)h->io_image_elems * 8; }
    h->io_image = nullptr;
    h->io_image_elems = 0;
    CK(h, cudaMalloc((void**)&h->io_image, img * sizeof(double)));
    h->io_image_elems = img;
    h->device_bytes += (int64_t)img * 8;
  }
  // the copies and their short conversion kernels on streams of the greatest
  // priority: their CTAs reach the SMs ahead of the queued step kernels
  if (!h->io_h2d) {
    int least = 0, greatest = 0;
    CK(h, cudaDeviceGetStreamPriorityRange(&least, &greatest));
    if (h->io_stream) { CK(h, cudaStreamSynchronize(h->io_stream)); CK(h, cudaStreamDestroy(h->io_stream)); }
    h->io_stream = nullptr;
    for (cudaStream_t* st : {&h->io_stream, &h->io_h2d, &h->io_d2h})
      CK(h, cudaStreamCreateWithPriority(st, cudaStreamNonBlocking, greatest));
  }
  for (cudaEvent_t* e : {&h->io_done, &h->exch_ev})
    if (!*e) CK(h, cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  for (int g = 0; g < h->ngroups; ++g) {
    if (!h->dma_ev[g]) CK(h, cudaEventCreateWithFlags(&h->dma_ev[g], cudaEventDisableTiming));
    if (!h->conv_ev[g]) CK(h, cudaEventCreateWithFlags(&h->conv_ev[g], cudaEventDisableTiming));
  }
  const Fields F = fields(h);
  const int64_t* so = h->soff_d[layout][NPBMZ_U];
  // zone groups are runs of consecutive zones: group g's arrays are
  // [soh[z0], soh[z1]) of the caller's buffer and of the device image
  auto span = [&](int g, int64_t& off, size_t& bytes) {
    const int z0 = h->grp_zone_off[g], z1 = h->grp_zone_off[g + 1];
    off = soh[z0];
    bytes = (size_t)(soh[z1] - soh[z0]) * sizeof(double);
  };
  if (health_begin(h)) return -1;
  // 1. the planes exch_qbc reads, of every zone, straight from host memory,
  //    then exch_qbc; the copy engine starts on the zone arrays once those
  //    planes are in (sharing the link, both would finish late: 0.6 ms for
  //    the planes instead of 0.18 ms on BT-C)
  launch_convert(F, h->u, din, so, 0, 0, h->nzones, h->max_np, h->kind, NPBMZ_U, layout, 0, h->stream, nullptr, 1);
  CKL(h);
  // (exch_ev is recorded again after exch_qbc below; each wait binds to the
  // record made before it)
  CK(h, cudaEventRecord(h->exch_ev, h->stream));
  CK(h, cudaStreamWaitEvent(h->io_h2d, h->exch_ev, 0));
  for (int g = 0; g < h->ngroups; ++g) {
    int64_t off;
    size_t bytes;
    span(g, off, bytes);
    CK(h, cudaMemcpyAsync(h->io_image + off, host_in + off, bytes, cudaMemcpyHostToDevice, h->io_h2d));
    CK(h, cudaEventRecord(h->dma_ev[g], h->io_h2d));
  }
  if (phase_exch(h)) return -1;
  CK(h, cudaEventRecord(h->exch_ev, h->stream));
  // 2. each group's other points from the device image once its copy is in
  CK(h, cudaStreamWaitEvent(h->io_stream, h->exch_ev, 0));
  for (int g = 0; g < h->ngroups; ++g) {
    const int z0 = h->grp_zone_off[g], nz = h->grp_zone_off[g + 1] - z0;
    CK(h, cudaStreamWaitEvent(h->io_stream, h->dma_ev[g], 0));
    launch_convert(F, h->u, h->io_image, so, 0, z0, nz, h->max_np, h->kind, NPBMZ_U, layout, 0, h->io_stream,
                   nullptr, 2);
    CKL(h);
    CK(h, cudaEventRecord(h->up_ev[g], h->io_stream));
  }
  CK(h, cudaGraphLaunch(h->graph_inout, h->stream));
  if (nsteps > 1 && replay_graph(h, nsteps - 1)) return -1;
  // 3. each group out when its last z sweep is done: interior points into the
  //    device image (which holds the caller's halo from the copy in), then the
  //    group's arrays back by the copy engine -- in place only; into another
  //    buffer the points go straight to host memory (its halo is not ours)
  const bool in_place = host_out == host_in || layout == NPBMZ_LAYOUT_DENSE;
  for (int g = 0; g < h->ngroups; ++g) {
    const int z0 = h->grp_zone_off[g], nz = h->grp_zone_off[g + 1] - z0;
    CK(h, cudaStreamWaitEvent(h->io_stream, h->grp_out_ev[g], 0));
    launch_convert(F, h->u, in_place ? h->io_image : dout, so, 0, z0, nz, h->max_np, h->kind, NPBMZ_U, layout, 1,
                   h->io_stream);
    CKL(h);
    if (in_place) {
      CK(h, cudaEventRecord(h->conv_ev[g], h->io_stream));
      int64_t off;
      size_t bytes;
      span(g, off, bytes);
      CK(h, cudaStreamWaitEvent(h->io_d2h, h->conv_ev[g], 0));
      CK(h, cudaMemcpyAsync(host_out + off, h->io_image + off, bytes, cudaMemcpyDeviceToHost, h->io_d2h));
    }
  }
  CK(h, cudaEventRecord(h->io_done, in_place ? h->io_d2h : h->io_stream));
  if (health_read(h)) return -1;
  CK(h, cudaStreamWaitEvent(h->stream, h->io_done, 0));
  CK(h, cudaStreamSynchronize(h->stream));
  return health_verdict(h, "the steps");
}

int npbmz_step_profile(npbmz_t* h, int nsteps, double* phase_ms) {
  if (!h) return fail(nullptr, "null handle");
  if (nsteps < 1 || !phase_ms) return fail(h, "nsteps must be >= 1 and phase_ms non-null");
  constexpr int NE = NPBMZ_PROF_COUNT + 1;
  std::vector<cudaEvent_t> ev((size_t)nsteps * NE, nullptr);
  int rc = 0;
  for (auto& e : ev)
    if (!rc && cudaEventCreate(&e) != cudaSuccess) rc = fail(h, "cudaEventCreate failed");
  if (!rc && flush_boundary(h)) rc = -1;
  for (int st = 0; st < nsteps && !rc; ++st) {
    cudaEvent_t* E = &ev[(size_t)st * NE];
    rc |= cudaEventRecord(E[0], h->stream) != cudaSuccess;
    if (!rc) rc = phase_exch(h);
    rc |= cudaEventRecord(E[1], h->stream) != cudaSuccess;
    if (!rc) rc = phase_prim(h, -1, true);
    rc |= cudaEventRecord(E[2], h->stream) != cudaSuccess;
    if (!rc) rc = phase_rhs(h, -1, h->kind == NPBMZ_SP, false, true);
    rc |= cudaEventRecord(E[3], h->stream) != cudaSuccess;
    for (int dir = 0; dir < 3 && !rc; ++dir) {
      rc = phase_solve(h, dir, -1, dir == 2 ? 1 : 0, true);
      rc |= cudaEventRecord(E[4 + dir], h->stream) != cudaSuccess;
    }
  }
  if (!rc && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = fail(h, "profiled steps failed: %s", cudaGetErrorString(cudaGetLastError()));
  if (!rc) {
    for (int k = 0; k < NPBMZ_PROF_COUNT; ++k) phase_ms[k] = 0.0;
    for (int st = 0; st < nsteps; ++st)
      for (int k = 0; k < NPBMZ_PROF_COUNT; ++k) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[(size_t)st * NE + k], ev[(size_t)st * NE + k + 1]);
        phase_ms[k] += ms / nsteps;
      }
  }
  for (auto& e : ev)
    if (e) cudaEventDestroy(e);
  if (rc && h->err.empty()) h->err = "profiled steps failed";
  return rc ? -1 : 0;
}

int npbmz_verify(npbmz_t* h, double* xcr, double* xce) {
  if (!h || !xcr || !xce) return fail(h, "null argument");
  if (!h->norms_d) {
    if (dalloc(h, &h->norms_d, 10)) return -1;
    h->norms_cap = 1;
  }
  if (err_partials(h)) return -1;
  if (finish_norms(h, nullptr, h->norms_d + 5)) return -1;
  if (phase_prim(h, -1)) return -1;
  if (phase_rhs(h, -1, false, true)) return -1;
  if (finish_norms(h, h->norms_d, nullptr)) return -1;
  double buf[10];
  CK(h, cudaMemcpyAsync(buf, h->norms_d, sizeof(buf), cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  for (int m = 0; m < 5; ++m) { xcr[m] = buf[m]; xce[m] = buf[5 + m]; }
  return 0;
}

int npbmz_adjoint(npbmz_t* h, int nsteps, int checkpoint_every, const double* u_target, double* J,
                  double* grad_forcing, double* grad_u0) {
  if (!h) return fail(nullptr, "null handle");
  if (nsteps < 1 || checkpoint_every < 1) return fail(h, "nsteps and checkpoint_every must be >= 1");
  if (!u_target) return fail(h, "u_target is null");
  if (h->has_remote) return fail(h, "the adjoint needs every zone of the problem on this handle (no NPBMZ_REMOTE faces)");
  h->err.clear();
  CK(h, cudaStreamSynchronize(h->stream));
  return adjoint_run(h, nsteps, checkpoint_every, u_target, J, grad_forcing, grad_u0);
}

int npbmz_phase(npbmz_t* h, int phase, int zone) {
  if (!h) return fail(nullptr, "null handle");
  if (zone < -1 || zone >= h->nzones) return fail(h, "bad zone %d", zone);
  const bool sp = h->kind == NPBMZ_SP;
  switch (phase) {
    case NPBMZ_PHASE_RHS:
      if (phase_prim(h, zone)) return -1;
      return phase_rhs(h, zone, sp, false);
    case NPBMZ_PHASE_RHSONLY:
      if (phase_prim(h, zone)) return -1;
      return phase_rhs(h, zone, false, false);
    case NPBMZ_PHASE_XSOLVE: return phase_solve(h, 0, zone, 0);
    case NPBMZ_PHASE_YSOLVE: return phase_solve(h, 1, zone, 0);
    case NPBMZ_PHASE_ZSOLVE: return phase_solve(h, 2, zone, 0);
    case NPBMZ_PHASE_ADD: return phase_add(h, zone);
    case NPBMZ_PHASE_EXCH: return phase_exch(h);
    default: return fail(h, "bad phase %d", phase);
  }
}

int npbmz_set_step_groups(npbmz_t* h, int groups) {
  if (!h) return fail(nullptr, "null handle");
  if (groups < 1 || groups > 8) return fail(h, "groups must be 1..8");
  CK(h, cudaStreamSynchronize(h->stream));
  drop_graph(h);
  h->ngroups = groups;
  assign_zone_groups(h);
  if (build_work_lists(h) || build_line_lists(h)) return -1;
  {  // zones of each group (npbmz_step_download)
    std::vector<int> zl;
    h->grp_zone_off.assign(h->ngroups + 1, 0);
    for (int g = 0; g < h->ngroups; ++g) {
      for (int z = 0; z < h->nzones; ++z)
        if (h->zone_group[z] == g) zl.push_back(z);
      h->grp_zone_off[g + 1] = (int)zl.size();
    }
    if (!h->grp_zones_d) CK(h, cudaMalloc((void**)&h->grp_zones_d, std::max(1, h->nzones) * sizeof(int)));
    CK(h, cudaMemcpy(h->grp_zones_d, zl.data(), zl.size() * sizeof(int), cudaMemcpyHostToDevice));
  }
  if (h->ngroups > 1 && !h->scratch_yz[0])
    for (int d = 0; d < 2; ++d) {
      CK(h, cudaMalloc(&h->scratch_yz[d], std::max<size_t>(h->scratch_bytes, 16)));
      h->device_bytes += (int64_t)h->scratch_bytes;
    }
  h->launches_per_step = count_launches(h);
  return 0;
}

int npbmz_state_check(npbmz_t* h, int* bits, int* zone, int* i, int* j, int* k) {
  if (!h || !bits) return fail(h, "null argument");
  *bits = (int)h->health_bits;
  int z = -1, ii = -1, jj = -1, kk = -1;
  if (h->health_bits) {
    const int64_t p = h->health_point;
    z = 0;
    while (z + 1 < h->nzones && h->zh[z + 1].off <= p) ++z;
    const ZoneDev& d = h->zh[z];
    const int64_t q = p - d.off;
    ii = (int)(q % d.nx);
    jj = (int)((q / d.nx) % d.ny);
    kk = (int)(q / ((int64_t)d.nx * d.ny));
  }
  if (zone) *zone = z;
  if (i) *i = ii;
  if (j) *j = jj;
  if (k) *k = kk;
  return 0;
}

int npbmz_set_step_overlap(npbmz_t* h, int fp64_first, int sweep_ctas_per_sm) {
  if (!h) return fail(nullptr, "null handle");
  if (sweep_ctas_per_sm < 0 || sweep_ctas_per_sm > 32) return fail(h, "sweep_ctas_per_sm must be 0..32");
  CK(h, cudaStreamSynchronize(h->stream));
  drop_graph(h);
  h->fp64_prio = fp64_first != 0;
  h->sweep_cap = sweep_ctas_per_sm;
  return 0;
}

int npbmz_set_copy_fusion(npbmz_t* h, int on) {
  if (!h) return fail(nullptr, "null handle");
  CK(h, cudaStreamSynchronize(h->stream));
  drop_graph(h);
  h->copy_fusion = on != 0;
  h->launches_per_step = count_launches(h);
  return 0;
}

int npbmz_set_stream(npbmz_t* h, void* stream) {
  if (!h) return fail(nullptr, "null handle");
  if (h->own_stream && h->stream) {
    cudaStreamSynchronize(h->stream);
    cudaStreamDestroy(h->stream);
  }
  h->own_stream = false;
  h->stream = reinterpret_cast<cudaStream_t>(stream);
  drop_graph(h);
  return 0;
}

int npbmz_synchronize(npbmz_t* h) {
  if (!h) return fail(nullptr, "null handle");
  CK(h, cudaStreamSynchronize(h->stream));
  CK(h, cudaGetLastError());
  return 0;
}

int npbmz_autotune(npbmz_t* h) {
  if (!h) return fail(nullptr, "null handle");
  // 1. Lines per CTA of each sweep direction and zone-size bucket: the zones
  //    of a direction are split by line length into up to 3 buckets, and each
  //    bucket's candidates are timed on its own launches.  2. For graph
  //    handles, the number of zone-group branches of the step graph, timed on
  //    whole steps.  3. Persistent kernels (NPBMZ_PERSIST) on or off, timed
  //    on whole steps.  4. The x sweep's state copies in the compute_rhs
  //    launch or on their own (before 2 and after 3).  Timed on a snapshot of
  //    u and rhs, restored afterwards; no choice changes the results.
  const int cand[] = {32, 64, 128};
  const size_t bytes = 5 * (size_t)h->NP * sizeof(double);
  double* usave = nullptr;
  double* rsave = nullptr;
  CK(h, cudaMalloc(&usave, bytes));
  if (cudaMalloc(&rsave, bytes) != cudaSuccess) { cudaFree(usave); return fail(h, "autotune alloc"); }
  cudaMemcpyAsync(usave, h->u, bytes, cudaMemcpyDeviceToDevice, h->stream);
  cudaMemcpyAsync(rsave, h->rhs, bytes, cudaMemcpyDeviceToDevice, h->stream);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto elapsed = [&]() {
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    return ms;
  };
  drop_graph(h);
  int rc = 0;
  h->nbkt = std::min(HandleLimits::MAXB, h->nzones);
  for (int dir = 0; dir < 3; ++dir) {
    assign_buckets(h, dir);
    for (int bk = 0; bk < HandleLimits::MAXB; ++bk) h->tpb_bkt[dir][bk] = 64;
  }
  if (build_line_lists(h)) rc = -1;
  // prim + rhs once so that the solves read defined data
  if (!rc) rc = phase_prim(h, -1, true);
  if (!rc) rc = phase_rhs(h, -1, h->kind == NPBMZ_SP, false, true);
  for (int dir = 0; dir < 3 && !rc; ++dir)
    for (int bk = 0; bk < h->nbkt && !rc; ++bk) {
      float best = 1e30f;
      int best_tpb = h->tpb_bkt[dir][bk];
      for (int c : cand) {
        h->tpb_bkt[dir][bk] = c;
        if (build_line_lists(h)) { rc = -1; break; }
        h->cur_bucket = bk;
        float tot = 0.f;
        for (int rep = 0; rep < 4 && !rc; ++rep) {  // warm-up + 3 timed
          cudaMemcpyAsync(h->rhs, rsave, bytes, cudaMemcpyDeviceToDevice, h->stream);
          cudaEventRecord(e0, h->stream);
          rc |= phase_solve(h, dir, -1, 0, true);
          cudaEventRecord(e1, h->stream);
          const float ms = elapsed();
          if (rep > 0) tot += ms;
        }
        h->cur_bucket = -1;
        if (tot < best) { best = tot; best_tpb = c; }
      }
      h->tpb_bkt[dir][bk] = best_tpb;
    }
  if (!rc) rc = build_line_lists(h);
  // Whole steps decide: the bucket-tuned shapes against one bucket of 64
  // lines per CTA, then (graph handles) the number of zone-group branches,
  // then persistent kernels; each candidate runs 2 + 6 steps from the saved
  // state, three times, and counts its fastest run.
  auto step_ms = [&]() -> float {
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaMemcpyAsync(h->u, usave, bytes, cudaMemcpyDeviceToDevice, h->stream);
      cudaMemcpyAsync(h->rhs, rsave, bytes, cudaMemcpyDeviceToDevice, h->stream);
      if (npbmz_step(h, 2, nullptr)) return -1.f;
      cudaEventRecord(e0, h->stream);
      if (npbmz_step(h, 6, nullptr)) return -1.f;
      cudaEventRecord(e1, h->stream);
      best = std::min(best, elapsed());
    }
    return best;
  };
  if (!rc) {
    int tuned[3][HandleLimits::MAXB];
    std::memcpy(tuned, h->tpb_bkt, sizeof(tuned));
    const int tuned_nbkt = h->nbkt;
    drop_graph(h);
    const float t_tuned = step_ms();
    h->nbkt = 1;
    for (int dir = 0; dir < 3; ++dir) { assign_buckets(h, dir); h->tpb_bkt[dir][0] = 64; }
    drop_graph(h);
    if (build_line_lists(h)) rc = -1;
    const float t_plain = rc ? -1.f : step_ms();
    if (t_tuned < 0.f || t_plain < 0.f) rc = -1;
    else if (t_tuned < t_plain) {
      h->nbkt = tuned_nbkt;
      for (int dir = 0; dir < 3; ++dir) assign_buckets(h, dir);
      std::memcpy(h->tpb_bkt, tuned, sizeof(tuned));
      drop_graph(h);
      if (build_line_lists(h)) rc = -1;
    }
  }
  // the x-line-major copies in the compute_rhs launch or on their own: timed
  // before the group stage (whose choices depend on it) and again after the
  // last stage
  auto tune_copy_fusion = [&]() -> int {
    if (!h->pfx || (h->flags & NPBMZ_EXACT)) return 0;
    drop_graph(h);
    const float t_now = step_ms();
    h->copy_fusion = !h->copy_fusion;
    drop_graph(h);
    const float t_other = step_ms();
    if (t_now < 0.f || t_other < 0.f) return -1;
    if (t_now <= t_other) h->copy_fusion = !h->copy_fusion;  // keep the first
    return 0;
  };
  if (!rc) rc = tune_copy_fusion();
  if (!rc && (h->flags & NPBMZ_GRAPH) && !(h->flags & (NPBMZ_EXACT | NPBMZ_PERZONE)) && h->nzones >= 8) {
    // zone-group branches; with more than one, the priority stream for the
    // FP64 phases and a cap on the sweeps' resident CTAs per SM
    const int gcand[] = {1, 2, 3, 4, 6, 8};
    const int ccand[] = {0, 3, 2};
    float best = 1e30f;
    int best_g = h->ngroups, best_c = h->sweep_cap;
    bool best_p = h->fp64_prio;
    for (int G : gcand)
      for (int prio = 0; prio < (G > 1 ? 2 : 1) && !rc; ++prio)
        for (int ci = 0; ci < (G > 1 ? 3 : 1) && !rc; ++ci) {
          if (G > h->nzones || npbmz_set_step_groups(h, G)) continue;
          h->fp64_prio = prio != 0;
          h->sweep_cap = ccand[ci];
          const float ms = step_ms();
          if (ms < 0.f) { rc = -1; break; }
          if (ms < best) { best = ms; best_g = G; best_p = prio != 0; best_c = ccand[ci]; }
        }
    h->fp64_prio = best_p;
    h->sweep_cap = best_c;
    if (!rc) rc = npbmz_set_step_groups(h, best_g);
  }
  if (!rc && !(h->flags & (NPBMZ_EXACT | NPBMZ_PERZONE))) {
    drop_graph(h);
    const float t_now = step_ms();
    h->flags ^= NPBMZ_PERSIST;
    drop_graph(h);
    const float t_other = step_ms();
    if (t_now < 0.f || t_other < 0.f) rc = -1;
    else if (t_now <= t_other) h->flags ^= NPBMZ_PERSIST;  // keep the first
  }
  if (!rc) rc = tune_copy_fusion();
  cudaMemcpyAsync(h->u, usave, bytes, cudaMemcpyDeviceToDevice, h->stream);
  cudaMemcpyAsync(h->rhs, rsave, bytes, cudaMemcpyDeviceToDevice, h->stream);
  cudaStreamSynchronize(h->stream);
  cudaFree(usave);
  cudaFree(rsave);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  drop_graph(h);
  h->launches_per_step = count_launches(h);
  return rc ? -1 : 0;
}

int npbmz_math_check(int which, int n, const double* x, double* y) {
  if (which != 0 || n < 0 || (n && (!x || !y))) return fail(nullptr, "npbmz_math_check: bad arguments");
  if (n == 0) return 0;
  double* d = nullptr;
  if (cudaMalloc((void**)&d, 2 * (size_t)n * sizeof(double)) != cudaSuccess)
    return fail(nullptr, "npbmz_math_check: device allocation failed");
  int rc = 0;
  if (cudaMemcpy(d, x, n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) rc = -1;
  if (!rc) launch_math_check(which, n, d, d + n, nullptr);
  if (!rc && cudaMemcpy(y, d + n, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) rc = -1;
  cudaFree(d);
  return rc ? fail(nullptr, "npbmz_math_check: %s", cudaGetErrorString(cudaGetLastError())) : 0;
}

int npbmz_fp64_peak(double* gflops) {
  if (!gflops) return -1;
  return probe_fp64(gflops);
}

int npbmz_launches_per_step(npbmz_t* h) { return h ? h->launches_per_step : -1; }
int64_t npbmz_device_bytes(npbmz_t* h) { return h ? h->device_bytes : -1; }

int npbmz_describe(npbmz_t* h, char* buf, size_t n) {
  if (!h || !buf || n == 0) return fail(h, "bad arguments");
  std::string tp = "[";
  for (int d = 0; d < 3; ++d) {
    tp += d ? ",[" : "[";
    for (int b = 0; b < h->nbkt; ++b) tp += (b ? "," : "") + std::to_string(h->tpb_bkt[d][b]);
    tp += "]";
  }
  tp += "]";
  snprintf(buf, n, "{\"kind\":\"%s\",\"zones\":%d,\"points\":%lld,\"flags\":%d,\"lines_per_cta\":%s,"
           "\"zone_size_buckets\":%d,\"step_groups\":%d,\"fp64_priority\":%s,\"sweep_ctas_per_sm\":%d,"
           "\"persistent\":%s,\"copy_fusion\":%s,\"launches_per_step\":%d,\"device_bytes\":%lld}",
           h->kind == NPBMZ_BT ? "BT" : "SP", h->nzones, (long long)h->NP, h->flags, tp.c_str(), h->nbkt, h->ngroups,
           h->fp64_prio ? "true" : "false", h->sweep_cap, (h->flags & NPBMZ_PERSIST) ? "true" : "false",
           h->copy_fusion ? "true" : "false", h->launches_per_step, (long long)h->device_bytes);
  return 0;
}

const char* npbmz_last_error(npbmz_t* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int npbmz_face_plan(npbmz_t* h, int nsend, const int* send, int nrecv, const int* recv, int64_t* send_count,
                    int64_t* recv_count) {
  if (!h) return fail(nullptr, "null handle");
  if (nsend < 0 || nrecv < 0 || (nsend && !send) || (nrecv && !recv) || !send_count || !recv_count)
    return fail(h, "bad face lists");
  auto build = [&](int n, const int* list, bool incoming, std::vector<FaceDesc>& out, int64_t& total) -> int {
    total = 0;
    for (int f = 0; f < n; ++f) {
      const int z = list[2 * f], side = list[2 * f + 1];
      if (z < 0 || z >= h->nzones || side < 0 || side > 3) return fail(h, "face %d: bad zone %d or side %d", f, z, side);
      // a received face must be one the handle was told is remote
      if (incoming && h->nbr[4 * z + side] != NPBMZ_REMOTE)
        return fail(h, "face %d: zone %d side %d is not an NPBMZ_REMOTE face", f, z, side);
      const ZoneDev& d = h->zh[z];
      out.push_back({z, side, total});
      total += 5 * (int64_t)((side < 2 ? d.ny : d.nx) - 2) * (d.nz - 2);
    }
    return 0;
  };
  std::vector<FaceDesc> sf, rf;
  int64_t ns = 0, nr = 0;
  if (build(nsend, send, false, sf, ns) || build(nrecv, recv, true, rf, nr)) return -1;
  if (h->send_faces_d) { cudaFree(h->send_faces_d); h->send_faces_d = nullptr; }
  if (h->recv_faces_d) { cudaFree(h->recv_faces_d); h->recv_faces_d = nullptr; }
  h->nsend = h->nrecv = 0;
  if (nsend) {
    CK(h, cudaMalloc((void**)&h->send_faces_d, sf.size() * sizeof(FaceDesc)));
    CK(h, cudaMemcpy(h->send_faces_d, sf.data(), sf.size() * sizeof(FaceDesc), cudaMemcpyHostToDevice));
  }
  if (nrecv) {
    CK(h, cudaMalloc((void**)&h->recv_faces_d, rf.size() * sizeof(FaceDesc)));
    CK(h, cudaMemcpy(h->recv_faces_d, rf.data(), rf.size() * sizeof(FaceDesc), cudaMemcpyHostToDevice));
  }
  h->nsend = nsend;
  h->nrecv = nrecv;
  *send_count = ns;
  *recv_count = nr;
  return 0;
}

int npbmz_pack_faces(npbmz_t* h, double* send_buf) {
  if (!h) return fail(nullptr, "null handle");
  if (h->nsend && !send_buf) return fail(h, "null send buffer");
  launch_faces(true, fields(h), h->send_faces_d, h->nsend, h->max_face, send_buf, h->stream);
  CKL(h);
  return 0;
}

int npbmz_unpack_faces(npbmz_t* h, const double* recv_buf) {
  if (!h) return fail(nullptr, "null handle");
  if (h->nrecv && !recv_buf) return fail(h, "null receive buffer");
  launch_faces(false, fields(h), h->recv_faces_d, h->nrecv, h->max_face, const_cast<double*>(recv_buf), h->stream);
  CKL(h);
  return 0;
}

int npbmz_destroy(npbmz_t* h) {
  if (!h) return 0;
  if (h->stream) cudaStreamSynchronize(h->stream);
  drop_graph(h);
  void* bufs[] = {h->zones_d, h->nbr_d, h->u, h->rhs, h->forcing, h->prim, h->uex, h->xw, h->primf, h->flux, h->fdt, h->ud, h->xd, h->fd, h->rdf, h->pfx, h->rdx, h->x0x, h->scratch, h->scratch_yz[0], h->scratch_yz[1], h->part_rhs,
                  h->part_err, h->norms_d, h->stage, h->wpts_d, h->zblk_pts_d, h->wint_d, h->zblk_int_d,
                  h->wline_d[0], h->wline_d[1],
                  h->wline_d[2]};
  for (void* b : bufs)
    if (b) cudaFree(b);
  for (int l = 0; l < 2; ++l)
    for (int f = 0; f < 3; ++f)
      if (h->soff_d[l][f]) cudaFree(h->soff_d[l][f]);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  if (h->aux_stream) { cudaStreamSynchronize(h->aux_stream); cudaStreamDestroy(h->aux_stream); }
  for (cudaStream_t gs : h->grp_stream)
    if (gs) { cudaStreamSynchronize(gs); cudaStreamDestroy(gs); }
  for (cudaStream_t gs : h->io_grp_stream)
    if (gs) { cudaStreamSynchronize(gs); cudaStreamDestroy(gs); }
  if (h->prio_stream) { cudaStreamSynchronize(h->prio_stream); cudaStreamDestroy(h->prio_stream); }
  for (cudaEvent_t e : h->grp_ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : h->grp_out_ev)
    if (e) cudaEventDestroy(e);
  if (h->io_stream) { cudaStreamSynchronize(h->io_stream); cudaStreamDestroy(h->io_stream); }
  if (h->io_done) cudaEventDestroy(h->io_done);
  for (cudaEvent_t e : h->up_ev)
    if (e) cudaEventDestroy(e);
  if (h->exch_ev) cudaEventDestroy(h->exch_ev);
  for (cudaStream_t st : {h->io_h2d, h->io_d2h})
    if (st) { cudaStreamSynchronize(st); cudaStreamDestroy(st); }
  for (int g = 0; g < 8; ++g) {
    if (h->dma_ev[g]) cudaEventDestroy(h->dma_ev[g]);
    if (h->conv_ev[g]) cudaEventDestroy(h->conv_ev[g]);
  }
  if (h->io_image) cudaFree(h->io_image);
  if (h->grp_zones_d) cudaFree(h->grp_zones_d);
  if (h->health_d) cudaFree(h->health_d);
  if (h->send_faces_d) cudaFree(h->send_faces_d);
  if (h->recv_faces_d) cudaFree(h->recv_faces_d);
  if (h->health_h) cudaFreeHost(h->health_h);
  for (cudaEvent_t e : h->fence)
    if (e) cudaEventDestroy(e);
  delete h;
  return 0;
}

}  // extern "C"
