// lu.cu -- the host side of LU-MZ's SSOR iteration (NPBApps.jl src/LU) on
// the GPU: its C ABI (include/npbmz_lu.h).  The kernels are in
// lu_kernels.cuh, built twice: lu_exact (-fmad=false: every FP64 statement
// rounds as the reference's Julia does, no a*b+c contraction, so the result
// is bit-for-bit the oracle's; the default) and lu_fast (-fmad=true; the hot
// kernels of an NPBMZ_LU_FMA handle).
//
// Data in HBM: u, rsd, frct variable-major over the points of all zones,
// field[m*NP + zone.off + ((k-1)*ny + (j-1))*nx + (i-1)] (1-based i, j, k as
// in the reference; zone offsets rounded to 32 points).
//
// One iteration (src/LU/lu-node.jl:233-270 with ssor src/LU/ssor.jl:9-254):
//   exch_qbc       k_lu_pack + k_lu_unpack (every face packed before any is
//                  unpacked, as the reference's sends are)
//   rsd *= dt      fused into the first touch of each point in k_lu_lower
//   Jacobians      k_lu_jac: jacld's and jacu's off-diagonal blocks and the
//                  factors of d at every point, fully parallel
//   flux prims     per-point quantities of the flux functions (1/u1, the
//                  viscous u21.., the convective u21 and q), refreshed where
//                  u changes: k_lu_unpack (ghost faces), k_lu_pointwise<1>
//                  (update), uploads; read by the sweeps and rhs
//   blts           k_lu_lower, one launch per hyperplane i+j+k = l, five
//                  threads per point (one per row of the 5x5 blocks)
//   buts           k_lu_upper, one launch per hyperplane, l descending
//   update         k_lu_pointwise<1>
//   rhs            k_lu_rhs<false>, one thread per point
// blts / buts make point (i,j,k) depend on (i-1,j,k), (i,j-1,k), (i,j,k-1)
// (resp. +1): within a hyperplane every point is independent, and every
// zone's hyperplane l runs in the same launch.  The arithmetic of each point
// is the reference's, statement for statement; only the order in which
// independent points are visited changes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/npbmz_lu.h"
#include "lu_launch.h"

using namespace npbmz_lu;

namespace {

// the reference's ce table (src/LU/setcoeff.jl), row m, 13 columns
const double ce_reference[5][13] = {
    {2.0e0, 0.0e0, 0.0e0, 4.0e0, 5.0e0, 3.0e0, 0.5e0, 0.02e0, 0.01e0, 0.03e0, 0.5e0, 0.4e0, 0.3e0},
    {1.0e0, 0.0e0, 0.0e0, 0.0e0, 1.0e0, 2.0e0, 3.0e0, 0.01e0, 0.03e0, 0.02e0, 0.4e0, 0.3e0, 0.5e0},
    {2.0e0, 2.0e0, 0.0e0, 0.0e0, 0.0e0, 2.0e0, 3.0e0, 0.04e0, 0.03e0, 0.05e0, 0.3e0, 0.5e0, 0.4e0},
    {2.0e0, 2.0e0, 0.0e0, 0.0e0, 0.0e0, 2.0e0, 3.0e0, 0.03e0, 0.05e0, 0.04e0, 0.2e0, 0.1e0, 0.3e0},
    {5.0e0, 4.0e0, 3.0e0, 2.0e0, 0.1e0, 0.4e0, 0.3e0, 0.05e0, 0.04e0, 0.03e0, 0.1e0, 0.3e0, 0.2e0}};

}  // namespace


// ============================== C ABI =========================================
struct npbmz_lu_handle {
  int nzones = 0, flags = 0;
  bool fast = false;  // NPBMZ_LU_FMA: the hot kernels from lu_fast
  double dt = 0, omega = 0;
  long long NP = 0;
  std::vector<LuZone> zh;
  std::vector<int> nbr;
  LuZone* zones_d = nullptr;
  int* nbr_d = nullptr;
  double *u = nullptr, *rsd = nullptr, *frct = nullptr;
  double* prim = nullptr;  // PR_COUNT planes (PR_RHO first: 1/u1 for the sweeps)
  double* fac = nullptr;  // FAC_COUNT planes per point: d's factors and the off-diagonal blocks
  int* hps_d = nullptr;   // per zone, hstride ints: interior points with i+j+k < l
  std::vector<char> jac_ok;  // per zone: fac holds the blocks of the current u
  int* ri_d = nullptr;       // per zone, l and k: slot of the first interior point of row k of hyperplane l
  int ri_ks = 0;
  int* fb_d = nullptr;       // per zone, l and k: the first point of row k of hyperplane l in the full box
  int fb_ls = 0;
  int hstride = 0;
  int max_interior = 0;
  // work lists: all zones, and per zone a contiguous range
  std::vector<LuWork> work_h;
  std::vector<int> zblock;  // first block of each zone, nzones+1 entries
  LuWork* work_d = nullptr;
  int* zblock_d = nullptr;
  double* partial = nullptr;  // 5 per work block
  double* norms_d = nullptr;  // per-iteration rsd norms, 5 per iteration (grown on demand)
  int norms_cap = 0;
  double* zone_out_d = nullptr;  // 5*nzones + nzones scratch
  // exch_qbc staging
  double* stage = nullptr;
  long long* zoff_d = nullptr;
  int klo = 1, nkp = 0;
  int lmin = 6, lmax = 6;
  std::vector<int> lcount;  // max points over zones per hyperplane l
  double* img = nullptr;    // host-image staging for transfers
  size_t img_cap = 0;
  cudaStream_t own = nullptr, stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  CeTable ce{};
  // state check of npbmz_lu_iterate (LuDev::health) and its page-locked copy
  unsigned long long* health_d = nullptr;
  unsigned long long* health_h = nullptr;
  unsigned health_bits = 0;
  long long health_point = -1;
  std::string err;
  std::mutex mu;
};

namespace {

// error text of the calls without a handle (npbmz_lu_zone_setup, a failed
// npbmz_lu_create), reported by npbmz_lu_last_error(NULL)
thread_local std::string g_lu_error;

int fail(npbmz_lu_t* h, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (h) h->err = buf;
  else g_lu_error = buf;
  return -1;
}

#define LU_CK(h, call)                                                                                      \
  do {                                                                                                      \
    cudaError_t e_ = (call);                                                                                \
    if (e_ != cudaSuccess) return fail(h, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

LuDev dev(npbmz_lu_t* h) {
  return LuDev{h->u, h->rsd, h->frct, h->prim, h->NP, h->zones_d, h->dt, h->omega, h->health_d};
}

// zone and 0-based (i, j, k) of point index p (LU's interior indexing: pidx)
void lu_point(const npbmz_lu_t* h, long long p, int* zone, int* i, int* j, int* k) {
  int z = 0;
  while (z + 1 < h->nzones && h->zh[z + 1].off <= p) ++z;
  const LuZone& Z = h->zh[z];
  const long long q = p - Z.off;
  *zone = z;
  *i = (int)(q % Z.nx);
  *j = (int)((q / Z.nx) % Z.ny);
  *k = (int)(q / ((long long)Z.nx * Z.ny));
}

Faces faces(npbmz_lu_t* h) { return Faces{h->stage, h->zoff_d, h->nbr_d, h->klo, h->nkp}; }

int hp_count(const LuZone& Z, int l) {
  int n = 0;
  for (int k = std::max(2, l - (Z.nx - 1) - (Z.ny - 1)); k <= std::min(Z.nz - 1, l - 4); ++k) {
    const int s = l - k;
    n += std::max(0, std::min(Z.ny - 1, s - 2) - std::max(2, s - (Z.nx - 1)) + 1);
  }
  return n;
}

// blocks of one zone (zone >= 0) or all zones
void work_range(npbmz_lu_t* h, int zone, const LuWork** w, int* n) {
  if (zone < 0) {
    *w = h->work_d;
    *n = (int)h->work_h.size();
  } else {
    *w = h->work_d + h->zblock[zone];
    *n = h->zblock[zone + 1] - h->zblock[zone];
  }
}

// u of zones z0..z0+nzs-1 changed: their blocks must be made again
void jac_stale(npbmz_lu_t* h, int z0, int nzs) {
  for (int z = z0; z < z0 + nzs; ++z) h->jac_ok[z] = 0;
}

int launch_exch(npbmz_lu_t* h) {
  jac_stale(h, 0, h->nzones);
  int maxper = 0;
  for (const LuZone& Z : h->zh) maxper = std::max(maxper, 2 * Z.nx + 2 * Z.ny);
  const dim3 g((maxper * h->nkp + TPB - 1) / TPB, h->nzones);
  lu_exact::pack(dev(h), faces(h), h->nzones, g, h->stream);
  if (h->fast)
    lu_fast::unpack(dev(h), faces(h), h->nzones, g, h->stream);
  else
    lu_exact::unpack(dev(h), faces(h), h->nzones, g, h->stream);
  LU_CK(h, cudaGetLastError());
  return 0;
}

int launch_jac(npbmz_lu_t* h, int z0, int nzs) {
  int maxnp = 0;
  for (int z = z0; z < z0 + nzs; ++z) {
    h->jac_ok[z] = 1;
    maxnp = std::max(maxnp, h->zh[z].np);
  }
  const dim3 g((maxnp + TPB - 1) / TPB, nzs);
  // thread order: hyperplane order (coalesced block writes) for the FMA
  // build, natural order (coalesced state reads) for the FP64-bound exact one
  (h->fast ? lu_fast::jac : lu_exact::jac)(h->fast, dev(h), h->fb_d, h->fb_ls, h->ri_d, h->hstride, h->ri_ks, h->fac,
                                          z0, g, h->stream);
  LU_CK(h, cudaGetLastError());
  return 0;
}

int launch_lower(npbmz_lu_t* h, bool scale, int z0, int nzs) {
  for (int l = h->lmin; l <= h->lmax; ++l) {
    int c = 0;
    for (int z = z0; z < z0 + nzs; ++z) c = std::max(c, hp_count(h->zh[z], l));
    if (!c) continue;
    const dim3 g((c + HP - 1) / HP, nzs);
    (h->fast ? lu_fast::lower : lu_exact::lower)(scale, dev(h), h->fac, h->hps_d, h->hstride, l, z0, g, h->stream);
  }
  LU_CK(h, cudaGetLastError());
  return 0;
}

int launch_phase(npbmz_lu_t* h, int phase, int zone) {
  const LuWork* w;
  int n;
  work_range(h, zone, &w, &n);
  const int z0 = zone < 0 ? 0 : zone, nzs = zone < 0 ? h->nzones : 1;
  switch (phase) {
    case NPBMZ_LU_PHASE_RHS:
      (h->fast ? lu_fast::rhs : lu_exact::rhs)(false, dev(h), w, n, h->u, h->prim, h->rsd, h->stream);
      break;
    case NPBMZ_LU_PHASE_SCALE:
      lu_exact::pointwise(false, dev(h), w, n, 0.0, h->stream);
      break;
    case NPBMZ_LU_PHASE_UPDATE:
      jac_stale(h, z0, nzs);
      (h->fast ? lu_fast::pointwise : lu_exact::pointwise)(true, dev(h), w, n,
                                                            1.0e+00 / (h->omega * (2.0e+00 - h->omega)), h->stream);
      break;
    case NPBMZ_LU_PHASE_EXCH:
      return launch_exch(h);
    case NPBMZ_LU_PHASE_LOWER:
    case NPBMZ_LU_PHASE_SSOR + 100: {  // lower with the scaling fused
      // the blocks and d's factors of every interior point, then the wavefront
      int rc = launch_jac(h, z0, nzs);
      if (!rc) rc = launch_lower(h, phase != NPBMZ_LU_PHASE_LOWER, z0, nzs);
      return rc;
    }
    case NPBMZ_LU_PHASE_UPPER: {
      // the blocks and factors k_lu_jac made before the lower sweep (u does
      // not change between the sweeps), made again where u has changed since
      bool stale = false;
      for (int z = z0; z < z0 + nzs; ++z) stale = stale || !h->jac_ok[z];
      if (stale && launch_jac(h, z0, nzs)) return -1;
      for (int l = h->lmax; l >= h->lmin; --l) {
        int c = 0;
        for (int z = z0; z < z0 + nzs; ++z) c = std::max(c, hp_count(h->zh[z], l));
        if (!c) continue;
        const dim3 g((c + HP - 1) / HP, nzs);
        (h->fast ? lu_fast::upper : lu_exact::upper)(dev(h), h->fac, h->hps_d, h->hstride, l, z0, g, h->stream);
      }
      break;
    }
    case NPBMZ_LU_PHASE_SSOR: {
      int rc = launch_phase(h, NPBMZ_LU_PHASE_SSOR + 100, zone);
      if (!rc) rc = launch_phase(h, NPBMZ_LU_PHASE_UPPER, zone);
      if (!rc) rc = launch_phase(h, NPBMZ_LU_PHASE_UPDATE, zone);
      if (!rc) rc = launch_phase(h, NPBMZ_LU_PHASE_RHS, zone);
      return rc;
    }
    default:
      return fail(h, "unknown LU phase %d", phase);
  }
  LU_CK(h, cudaGetLastError());
  return 0;
}

int launch_iteration(npbmz_lu_t* h) {
  int rc = launch_exch(h);
  if (!rc) rc = launch_phase(h, NPBMZ_LU_PHASE_SSOR, -1);
  return rc;
}

int launch_rsd_norm(npbmz_lu_t* h, double* out) {
  lu_exact::norm_partial(0, dev(h), h->work_d, (int)h->work_h.size(), h->ce, h->partial, h->stream);
  lu_exact::norm_finish(h->zones_d, h->zblock_d, h->nzones, h->partial, out, h->stream);
  LU_CK(h, cudaGetLastError());
  return 0;
}

int ensure_img(npbmz_lu_t* h, size_t bytes) {
  if (h->img_cap >= bytes) return 0;
  if (h->img) cudaFree(h->img);
  h->img = nullptr;
  h->img_cap = 0;
  LU_CK(h, cudaMalloc(&h->img, bytes));
  h->img_cap = bytes;
  return 0;
}

size_t zone_elems(const LuZone& Z, int layout) {
  return layout == NPBMZ_LAYOUT_REF ? (size_t)5 * (Z.nx + 4) * (Z.ny + 4) * Z.nz : (size_t)5 * Z.np;
}

double* field_ptr(npbmz_lu_t* h, int field) {
  return field == NPBMZ_LU_U ? h->u : (field == NPBMZ_LU_RSD ? h->rsd : (field == NPBMZ_LU_FRCT ? h->frct : nullptr));
}

int transfer(npbmz_lu_t* h, int zone, int field, int layout, double* host, bool up) {
  double* f = field_ptr(h, field);
  if (!f) return fail(h, "unknown field %d", field);
  if (layout != NPBMZ_LAYOUT_DENSE && layout != NPBMZ_LAYOUT_REF) return fail(h, "unknown layout %d", layout);
  if (zone < -1 || zone >= h->nzones) return fail(h, "zone %d out of range", zone);
  if (!host) return fail(h, "null host buffer");
  const int z0 = zone < 0 ? 0 : zone, z1 = zone < 0 ? h->nzones : zone + 1;
  // Page-locked (mapped) host memory: one kernel per zone reads or writes it
  // in place (the reference layout's halo is not touched), one synchronise
  // at the end.
  cudaPointerAttributes attr;
  std::memset(&attr, 0, sizeof(attr));
  const bool mapped = cudaPointerGetAttributes(&attr, host) == cudaSuccess && attr.type == cudaMemoryTypeHost &&
                      attr.devicePointer != nullptr;
  cudaGetLastError();  // pageable memory is not an error to keep
  if (mapped) {
    double* dhost = reinterpret_cast<double*>(attr.devicePointer);
    for (int z = z0; z < z1; ++z) {
      const LuZone& Z = h->zh[z];
      const int blocks = (int)((5LL * Z.np + TPB - 1) / TPB);
      lu_exact::convert(layout == NPBMZ_LAYOUT_REF, up, dev(h), f, dhost, z, blocks, h->stream);
      if (up && field == NPBMZ_LU_U) {
        jac_stale(h, z, 1);
        (h->fast ? lu_fast::prim : lu_exact::prim)(dev(h), h->work_d + h->zblock[z], h->zblock[z + 1] - h->zblock[z],
                                                  h->u, h->stream);
      }
      dhost += zone_elems(Z, layout);
    }
    LU_CK(h, cudaGetLastError());
    LU_CK(h, cudaStreamSynchronize(h->stream));
    return 0;
  }
  for (int z = z0; z < z1; ++z) {
    const LuZone& Z = h->zh[z];
    const size_t n = zone_elems(Z, layout);
    if (ensure_img(h, n * sizeof(double))) return -1;
    const int blocks = (int)((5LL * Z.np + TPB - 1) / TPB);
    if (up) {
      LU_CK(h, cudaMemcpyAsync(h->img, host, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
      lu_exact::convert(layout == NPBMZ_LAYOUT_REF, true, dev(h), f, h->img, z, blocks, h->stream);
      if (field == NPBMZ_LU_U) {
        jac_stale(h, z, 1);
        (h->fast ? lu_fast::prim : lu_exact::prim)(dev(h), h->work_d + h->zblock[z], h->zblock[z + 1] - h->zblock[z],
                                                  h->u, h->stream);
      }
    } else {
      if (layout == NPBMZ_LAYOUT_REF)  // keep the host halo: start from the host image
        LU_CK(h, cudaMemcpyAsync(h->img, host, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
      lu_exact::convert(layout == NPBMZ_LAYOUT_REF, false, dev(h), f, h->img, z, blocks, h->stream);
      LU_CK(h, cudaMemcpyAsync(host, h->img, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    }
    LU_CK(h, cudaGetLastError());
    LU_CK(h, cudaStreamSynchronize(h->stream));
    host += n;
  }
  return 0;
}

void free_all(npbmz_lu_t* h) {
  if (h->graph) cudaGraphExecDestroy(h->graph);
  for (void* p : {(void*)h->zones_d, (void*)h->nbr_d, (void*)h->u, (void*)h->rsd, (void*)h->frct, (void*)h->prim,
                  (void*)h->fac, (void*)h->work_d,
                  (void*)h->zblock_d, (void*)h->partial, (void*)h->norms_d, (void*)h->zone_out_d, (void*)h->stage,
                  (void*)h->zoff_d, (void*)h->img, (void*)h->hps_d, (void*)h->ri_d, (void*)h->fb_d,
                  (void*)h->health_d})
    if (p) cudaFree(p);
  if (h->health_h) cudaFreeHost(h->health_h);
  if (h->own) cudaStreamDestroy(h->own);
}

}  // namespace

extern "C" {

int npbmz_lu_zone_setup(int gx, int gy, int gz, int xz, int yz, double ratio, int* nx, int* ny, int* nz, int* nbr) {
  if (xz < 1 || yz < 1 || gx < 1 || gy < 1 || gz < 1 || !nx || !ny || !nz || !nbr)
    return fail(nullptr, "zone_setup: bad arguments");
  std::vector<long> x_end(xz), y_end(yz), x_start(xz), y_start(yz), x_size(xz), y_size(yz);
  if (std::fabs(ratio - 1.0e0) > 1.0e-10) {
    if (xz < 2 || yz < 2) return fail(nullptr, "zone_setup: a stretched split needs 2 zones per axis");
    const double x_r = std::exp(std::log(ratio) / (xz - 1));
    const double y_r = std::exp(std::log(ratio) / (yz - 1));
    const double x_smallest = (double)gx * (x_r - 1.0e0) / (std::pow(x_r, xz) - 1.0e0);
    const double y_smallest = (double)gy * (y_r - 1.0e0) / (std::pow(y_r, yz) - 1.0e0);
    // Julia's round: to nearest, ties to even
    for (int i = 1; i <= xz; ++i)
      x_end[i - 1] = (long)std::nearbyint(x_smallest * (std::pow(x_r, i) - 1.0e0) / (x_r - 1.0e0) + 0.45e0);
    for (int j = 1; j <= yz; ++j)
      y_end[j - 1] = (long)std::nearbyint(y_smallest * (std::pow(y_r, j) - 1.0e0) / (y_r - 1.0e0) + 0.45e0);
  } else {
    for (int i = 1; i <= xz; ++i) {
      if (((long)i * gx) % xz) return fail(nullptr, "zone_setup: %d points do not split into %d equal zones", gx, xz);
      x_end[i - 1] = (long)i * gx / xz;
    }
    for (int j = 1; j <= yz; ++j) {
      if (((long)j * gy) % yz) return fail(nullptr, "zone_setup: %d points do not split into %d equal zones", gy, yz);
      y_end[j - 1] = (long)j * gy / yz;
    }
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
  const int nzones = xz * yz;
  for (int j = 1; j <= yz; ++j)
    for (int i = 1; i <= xz; ++i) {
      const int zn = (i - 1) + (j - 1) * xz + 1;
      nx[zn - 1] = (int)x_size[i - 1];
      ny[zn - 1] = (int)y_size[j - 1];
      nz[zn - 1] = gz;
      const int north = i > 1 ? zn - 1 : j * xz;
      const int south = i < xz ? zn + 1 : zn - xz + 1;
      const int west = j > 1 ? zn - xz : zn + yz * (xz - 1);
      const int east = j < yz ? zn + xz : zn - yz * (xz - 1);
      for (int q : {north, south, west, east})
        if (q < 1 || q > nzones) return fail(nullptr, "zone_setup: zone %d's neighbour %d is outside the zones", zn - 1, q - 1);
      nbr[4 * (zn - 1) + 0] = west - 1;
      nbr[4 * (zn - 1) + 1] = east - 1;
      nbr[4 * (zn - 1) + 2] = south - 1;
      nbr[4 * (zn - 1) + 3] = north - 1;
    }
  return 0;
}

int npbmz_lu_create(int nzones, const int* nx, const int* ny, const int* nz, const int* nbr, const double* params,
                    int flags, npbmz_lu_t** out) {
  if (!out) return fail(nullptr, "out is null");
  *out = nullptr;
  if (nzones < 1 || !nx || !ny || !nz || !nbr || !params) return fail(nullptr, "bad geometry arguments");
  if (flags & ~(NPBMZ_LU_FACES_NPB | NPBMZ_LU_GRAPH | NPBMZ_LU_FMA)) return fail(nullptr, "unknown flags 0x%x", flags);
  npbmz_lu_t* h = new npbmz_lu_t();
  h->nzones = nzones;
  h->flags = flags;
  h->fast = (flags & NPBMZ_LU_FMA) != 0;
  h->dt = params[0];
  h->omega = params[1];
  std::memcpy(h->ce.c, ce_reference, sizeof(h->ce.c));
  h->nbr.assign(nbr, nbr + 4 * nzones);
  long long off = 0;
  int gz = nz[0];
  for (int z = 0; z < nzones; ++z) {
    // ssor's stencils and pintgr need 5 points per axis (the reference's
    // SUBDOMAIN SIZE check asks for 3; its fourth-difference dissipation
    // reads 5)
    if (nx[z] < 5 || ny[z] < 5 || nz[z] < 5 || nz[z] != gz) {
      delete h;
      return fail(nullptr, "zone %d: size %dx%dx%d (each extent >= 5, nz equal in all zones)", z, nx[z], ny[z], nz[z]);
    }
    if ((long long)nx[z] * ny[z] * nz[z] > (1LL << 30)) {
      delete h;
      return fail(nullptr, "zone %d: more than 2^30 points", z);
    }
    for (int q = 0; q < 4; ++q)
      if (nbr[4 * z + q] < 0 || nbr[4 * z + q] >= nzones) {
        delete h;
        return fail(nullptr, "zone %d: neighbour %d outside the zones", z, nbr[4 * z + q]);
      }
    LuZone Z{};
    Z.off = off;
    Z.nx = nx[z]; Z.ny = ny[z]; Z.nz = nz[z];
    Z.np = nx[z] * ny[z] * nz[z];
    Z.dxi = 1.0e+00 / (Z.nx - 1);
    Z.deta = 1.0e+00 / (Z.ny - 1);
    Z.dzeta = 1.0e+00 / (Z.nz - 1);
    Z.tx1 = 1.0e+00 / (Z.dxi * Z.dxi);
    Z.tx2 = 1.0e+00 / (2.0e+00 * Z.dxi);
    Z.tx3 = 1.0e+00 / Z.dxi;
    Z.ty1 = 1.0e+00 / (Z.deta * Z.deta);
    Z.ty2 = 1.0e+00 / (2.0e+00 * Z.deta);
    Z.ty3 = 1.0e+00 / Z.deta;
    Z.tz1 = 1.0e+00 / (Z.dzeta * Z.dzeta);
    Z.tz2 = 1.0e+00 / (2.0e+00 * Z.dzeta);
    Z.tz3 = 1.0e+00 / Z.dzeta;
    Z.ii2 = Z.nx - 1;
    Z.ji2 = Z.ny - 2;
    Z.ki2 = Z.nz - 1;
    h->zh.push_back(Z);
    off += ((long long)Z.np + 31) / 32 * 32;
  }
  // faces between neighbours must match: west/east share nx, south/north ny
  for (int z = 0; z < nzones; ++z) {
    if (h->zh[h->nbr[4 * z + 0]].nx != h->zh[z].nx || h->zh[h->nbr[4 * z + 1]].nx != h->zh[z].nx ||
        h->zh[h->nbr[4 * z + 2]].ny != h->zh[z].ny || h->zh[h->nbr[4 * z + 3]].ny != h->zh[z].ny) {
      delete h;
      return fail(nullptr, "zone %d: neighbour face sizes do not match", z);
    }
  }
  h->NP = off;
  {
    // u, rsd, frct, the flux quantities and the Jacobian planes, checked
    // before anything is allocated
    const double need = (double)(15 + PR_COUNT + FAC_COUNT) * (double)off * sizeof(double);
    size_t free_b = 0, total_b = 0;
    const cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) {
      cudaGetLastError();
      delete h;
      return fail(nullptr, "no usable CUDA device: %s", cudaGetErrorString(e));
    }
    if (need > (double)free_b) {
      delete h;
      return fail(nullptr, "%lld points need %.1f GB of device memory, %.1f GB free", off, need / 1e9,
                  (double)free_b / 1e9);
    }
  }
  h->klo = (flags & NPBMZ_LU_FACES_NPB) ? 2 : 1;
  h->nkp = gz - 2;
  h->lmin = 6;
  h->lmax = 6;
  for (const LuZone& Z : h->zh) h->lmax = std::max(h->lmax, Z.nx + Z.ny + Z.nz - 3);
  h->hstride = h->lmax + 2;
  std::vector<int> hps((size_t)nzones * h->hstride, 0);
  for (int z = 0; z < nzones; ++z) {
    int acc = 0;
    for (int l = 0; l < h->hstride; ++l) {
      hps[(size_t)z * h->hstride + l] = acc;
      if (l >= 6) acc += hp_count(h->zh[z], l);
    }
    h->max_interior = std::max(h->max_interior, acc);
  }
  int maxnz = 0, maxl = 0;
  for (const LuZone& Z : h->zh) {
    maxnz = std::max(maxnz, Z.nz);
    maxl = std::max(maxl, Z.nx + Z.ny + Z.nz);
  }
  h->ri_ks = maxnz + 2;
  // the full-box hyperplane order of every zone's points (k_lu_jac's threads)
  h->fb_ls = maxl + 2;
  std::vector<int> fb((size_t)nzones * h->fb_ls * h->ri_ks, 0);
  for (int z = 0; z < nzones; ++z) {
    const LuZone& Z = h->zh[z];
    int F = 0;
    for (int l = 0; l < h->fb_ls; ++l) {
      int R = 0;
      for (int k = 0; k < h->ri_ks; ++k) {
        fb[((size_t)z * h->fb_ls + l) * h->ri_ks + k] = F + R;
        if (k >= 1 && k <= Z.nz && l >= 3 && l <= Z.nx + Z.ny + Z.nz)
          R += std::max(0, std::min(Z.ny, l - k - 1) - std::max(1, l - k - Z.nx) + 1);
      }
      F += R;
    }
  }
  std::vector<int> ri((size_t)nzones * h->hstride * h->ri_ks, 0);
  for (int z = 0; z < nzones; ++z) {
    const LuZone& Z = h->zh[z];
    for (int l = 0; l < h->hstride; ++l) {
      int R = 0;
      for (int k = 0; k < h->ri_ks; ++k) {
        ri[((size_t)z * h->hstride + l) * h->ri_ks + k] = hps[(size_t)z * h->hstride + l] + R;
        if (k >= 2 && k <= Z.nz - 1 && l >= 6 && l <= Z.nx + Z.ny + Z.nz - 3) {
          const int s = l - k;
          R += std::max(0, std::min(Z.ny - 1, s - 2) - std::max(2, s - (Z.nx - 1)) + 1);
        }
      }
    }
  }
  h->jac_ok.assign(nzones, 0);
  h->zblock.push_back(0);
  for (int z = 0; z < nzones; ++z) {
    for (int f = 0; f < h->zh[z].np; f += TPB) h->work_h.push_back(LuWork{z, f});
    h->zblock.push_back((int)h->work_h.size());
  }
  std::vector<long long> zoff(nzones);
  long long so = 0;
  for (int z = 0; z < nzones; ++z) {
    zoff[z] = so;
    so += 10LL * h->zh[z].nx * h->nkp + 10LL * h->zh[z].ny * h->nkp;
  }
  auto bail = [&](const char* what) {
    fail(nullptr, "%s: %s", what, cudaGetErrorString(cudaGetLastError()));
    free_all(h);
    delete h;
    return -1;
  };
  const size_t F = (size_t)5 * h->NP * sizeof(double);
  if (cudaStreamCreateWithFlags(&h->own, cudaStreamNonBlocking) != cudaSuccess) return bail("stream");
  h->stream = h->own;
  if (cudaMalloc(&h->zones_d, nzones * sizeof(LuZone)) || cudaMalloc(&h->nbr_d, 4 * nzones * sizeof(int)) ||
      cudaMalloc(&h->u, F) || cudaMalloc(&h->rsd, F) || cudaMalloc(&h->frct, F) ||
      cudaMalloc(&h->prim, (size_t)PR_COUNT * h->NP * sizeof(double)) ||
      cudaMalloc(&h->fac, (size_t)FAC_COUNT * h->NP * sizeof(double)) ||
      cudaMalloc(&h->work_d, h->work_h.size() * sizeof(LuWork)) ||
      cudaMalloc(&h->zblock_d, h->zblock.size() * sizeof(int)) ||
      cudaMalloc(&h->partial, h->work_h.size() * 5 * sizeof(double)) ||
      cudaMalloc(&h->zone_out_d, (6 * (size_t)nzones + 16) * sizeof(double)) ||
      cudaMalloc(&h->stage, so * sizeof(double)) || cudaMalloc(&h->zoff_d, nzones * sizeof(long long)) ||
      cudaMalloc(&h->hps_d, hps.size() * sizeof(int)) || cudaMalloc(&h->ri_d, ri.size() * sizeof(int)) ||
      cudaMalloc(&h->fb_d, fb.size() * sizeof(int)) || cudaMalloc(&h->health_d, 2 * sizeof(unsigned long long)) ||
      cudaMallocHost(&h->health_h, 2 * sizeof(unsigned long long)))
    return bail("device allocation failed");
  if (cudaMemcpy(h->zones_d, h->zh.data(), nzones * sizeof(LuZone), cudaMemcpyHostToDevice) ||
      cudaMemcpy(h->nbr_d, h->nbr.data(), 4 * nzones * sizeof(int), cudaMemcpyHostToDevice) ||
      cudaMemcpy(h->work_d, h->work_h.data(), h->work_h.size() * sizeof(LuWork), cudaMemcpyHostToDevice) ||
      cudaMemcpy(h->zblock_d, h->zblock.data(), h->zblock.size() * sizeof(int), cudaMemcpyHostToDevice) ||
      cudaMemcpy(h->zoff_d, zoff.data(), nzones * sizeof(long long), cudaMemcpyHostToDevice) ||
      cudaMemcpy(h->hps_d, hps.data(), hps.size() * sizeof(int), cudaMemcpyHostToDevice) ||
      cudaMemcpy(h->ri_d, ri.data(), ri.size() * sizeof(int), cudaMemcpyHostToDevice) ||
      cudaMemcpy(h->fb_d, fb.data(), fb.size() * sizeof(int), cudaMemcpyHostToDevice) ||
      cudaMemset(h->u, 0, F) || cudaMemset(h->rsd, 0, F) || cudaMemset(h->frct, 0, F) ||
      cudaMemset(h->prim, 0, (size_t)PR_COUNT * h->NP * sizeof(double)) ||
      cudaMemset(h->fac, 0, (size_t)FAC_COUNT * h->NP * sizeof(double)))
    return bail("device initialisation failed");
  *out = h;
  return 0;
}

int npbmz_lu_setup(npbmz_lu_t* h, const double* ce) {
  if (!h) return fail(nullptr, "null handle");
  std::lock_guard<std::mutex> g(h->mu);
  std::memcpy(h->ce.c, ce ? ce : &ce_reference[0][0], sizeof(h->ce.c));
  const int n = (int)h->work_h.size();
  jac_stale(h, 0, h->nzones);
  // setbv, setiv and erhs always without contraction: both builds start from
  // the same u and frct; the flux quantities of u and the first rhs come from
  // the iteration's build, as every later one does
  lu_exact::init(dev(h), h->work_d, n, h->ce, h->stream);
  lu_exact::poly(dev(h), h->work_d, n, h->ce, h->stream);
  lu_exact::prim(dev(h), h->work_d, n, h->rsd, h->stream);
  lu_exact::rhs(true, dev(h), h->work_d, n, h->rsd, h->prim, h->frct, h->stream);
  (h->fast ? lu_fast::prim : lu_exact::prim)(dev(h), h->work_d, n, h->u, h->stream);
  (h->fast ? lu_fast::rhs : lu_exact::rhs)(false, dev(h), h->work_d, n, h->u, h->prim, h->rsd, h->stream);
  LU_CK(h, cudaGetLastError());
  return 0;
}

int npbmz_lu_upload(npbmz_lu_t* h, int zone, int field, int layout, const double* host) {
  if (!h) return fail(nullptr, "null handle");
  std::lock_guard<std::mutex> g(h->mu);
  return transfer(h, zone, field, layout, const_cast<double*>(host), true);
}

int npbmz_lu_download(npbmz_lu_t* h, int zone, int field, int layout, double* host) {
  if (!h) return fail(nullptr, "null handle");
  std::lock_guard<std::mutex> g(h->mu);
  return transfer(h, zone, field, layout, host, false);
}

int npbmz_lu_exch_qbc(npbmz_lu_t* h) {
  if (!h) return fail(nullptr, "null handle");
  std::lock_guard<std::mutex> g(h->mu);
  return launch_exch(h);
}

int npbmz_lu_ssor(npbmz_lu_t* h, int zone) {
  if (!h) return fail(nullptr, "null handle");
  std::lock_guard<std::mutex> g(h->mu);
  if (zone < -1 || zone >= h->nzones) return fail(h, "zone %d out of range", zone);
  return launch_phase(h, NPBMZ_LU_PHASE_SSOR, zone);
}

int npbmz_lu_phase(npbmz_lu_t* h, int phase, int zone) {
  if (!h) return fail(nullptr, "null handle");
  std::lock_guard<std::mutex> g(h->mu);
  if (zone < -1 || zone >= h->nzones) return fail(h, "zone %d out of range", zone);
  if (phase < 0 || phase > NPBMZ_LU_PHASE_SSOR) return fail(h, "unknown LU phase %d", phase);
  return launch_phase(h, phase, zone);
}

int npbmz_lu_iterate(npbmz_lu_t* h, int niter, double* rsdnm) {
  if (!h) return fail(nullptr, "null handle");
  std::lock_guard<std::mutex> g(h->mu);
  if (niter < 0) return fail(h, "niter < 0");
  LU_CK(h, cudaMemsetAsync(h->health_d, 0, sizeof(unsigned long long), h->stream));
  LU_CK(h, cudaMemsetAsync(h->health_d + 1, 0xFF, sizeof(unsigned long long), h->stream));
  if (rsdnm && niter > h->norms_cap) {
    if (h->norms_d) cudaFree(h->norms_d);
    h->norms_d = nullptr;
    h->norms_cap = 0;
    LU_CK(h, cudaMalloc(&h->norms_d, (size_t)5 * niter * sizeof(double)));
    h->norms_cap = niter;
  }
  if ((h->flags & NPBMZ_LU_GRAPH) && !h->graph) {
    cudaGraph_t gr;
    LU_CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    gr = nullptr;
    const int rc = launch_iteration(h);
    const cudaError_t e = cudaStreamEndCapture(h->stream, &gr);
    if (rc || e != cudaSuccess) {
      if (gr) cudaGraphDestroy(gr);
      if (rc) return rc;
      LU_CK(h, e);
    }
    const cudaError_t ie = cudaGraphInstantiate(&h->graph, gr, 0);
    cudaGraphDestroy(gr);
    LU_CK(h, ie);
  }
  for (int it = 0; it < niter; ++it) {
    if (h->graph) {
      LU_CK(h, cudaGraphLaunch(h->graph, h->stream));
    } else if (int rc = launch_iteration(h)) {
      return rc;
    }
    if (rsdnm && launch_rsd_norm(h, h->norms_d + 5 * (size_t)it)) return -1;
  }
  if (rsdnm && niter > 0)
    LU_CK(h, cudaMemcpyAsync(rsdnm, h->norms_d, (size_t)5 * niter * sizeof(double), cudaMemcpyDeviceToHost,
                             h->stream));
  LU_CK(h, cudaMemcpyAsync(h->health_h, h->health_d, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           h->stream));
  LU_CK(h, cudaStreamSynchronize(h->stream));
  // every iteration's update checks the points it writes; a non-positive or
  // non-finite density or a non-finite value fails the call (LU takes no
  // square root of the pressure, so a non-positive one is only reported)
  h->health_bits = (unsigned)h->health_h[0];
  h->health_point = h->health_bits ? (long long)h->health_h[1] : -1;
  if (h->health_bits & (LU_STATE_DENSITY | LU_STATE_NONFINITE)) {
    int z, i, j, k;
    lu_point(h, h->health_point, &z, &i, &j, &k);
    fail(h, "state check failed after the iterations: %s%s%s in u; first bad point zone %d (i, j, k) = (%d, %d, %d)",
         (h->health_bits & LU_STATE_DENSITY) ? "non-positive or non-finite density" : "",
         (h->health_bits & LU_STATE_DENSITY) && (h->health_bits & LU_STATE_NONFINITE) ? " and " : "",
         (h->health_bits & LU_STATE_NONFINITE) ? "a non-finite value" : "", z, i, j, k);
    return NPBMZ_LU_ERR_STATE;
  }
  return 0;
}

int npbmz_lu_state_check(npbmz_lu_t* h, int* bits, int* zone, int* i, int* j, int* k) {
  if (!h || !bits) return fail(h, "null argument");
  std::lock_guard<std::mutex> g(h->mu);
  *bits = (int)h->health_bits;
  int z = -1, ii = -1, jj = -1, kk = -1;
  if (h->health_bits) lu_point(h, h->health_point, &z, &ii, &jj, &kk);
  if (zone) *zone = z;
  if (i) *i = ii;
  if (j) *j = jj;
  if (k) *k = kk;
  return 0;
}

int npbmz_lu_verify(npbmz_lu_t* h, double* xcr, double* xce, double* xci) {
  if (!h) return fail(nullptr, "null handle");
  std::lock_guard<std::mutex> g(h->mu);
  if (!xcr || !xce || !xci) return fail(h, "null output");
  double* o = h->zone_out_d;  // [0,5) xcr, [5,10) xce, [16, 16+nzones) frc per zone
  if (launch_rsd_norm(h, o)) return -1;
  lu_exact::norm_partial(1, dev(h), h->work_d, (int)h->work_h.size(), h->ce, h->partial, h->stream);
  lu_exact::norm_finish(h->zones_d, h->zblock_d, h->nzones, h->partial, o + 5, h->stream);
  lu_exact::pintgr(dev(h), h->nzones, o + 16, h->stream);
  LU_CK(h, cudaGetLastError());
  std::vector<double> host(16 + h->nzones);
  LU_CK(h, cudaMemcpyAsync(host.data(), o, host.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  LU_CK(h, cudaStreamSynchronize(h->stream));
  for (int m = 0; m < 5; ++m) {
    xcr[m] = host[m];
    xce[m] = host[5 + m];
  }
  double f = 0.0;
  for (int z = 0; z < h->nzones; ++z) f += host[16 + z];
  *xci = f;
  return 0;
}

int npbmz_lu_set_stream(npbmz_lu_t* h, void* stream) {
  if (!h) return fail(nullptr, "null handle");
  std::lock_guard<std::mutex> g(h->mu);
  h->stream = stream ? (cudaStream_t)stream : h->own;
  return 0;
}

int npbmz_lu_synchronize(npbmz_lu_t* h) {
  if (!h) return fail(nullptr, "null handle");
  LU_CK(h, cudaStreamSynchronize(h->stream));
  return 0;
}

int npbmz_lu_launches_per_iteration(npbmz_lu_t* h) {
  if (!h) return fail(nullptr, "null handle");
  int n = 2 + 3;  // exch (pack, unpack) + jac + update + rhs
  for (int l = h->lmin; l <= h->lmax; ++l) {
    int c = 0;
    for (const LuZone& Z : h->zh) c = std::max(c, hp_count(Z, l));
    if (c) n += 2;
  }
  return n;
}

int npbmz_lu_profile(npbmz_lu_t* h, int niter, double* phase_ms) {
  if (!h) return fail(nullptr, "null handle");
  if (!phase_ms || niter < 1) return fail(h, "profile needs phase_ms and niter >= 1");
  std::lock_guard<std::mutex> g(h->mu);
  constexpr int NPH = 6;  // exch, jac, lower, upper, update, rhs
  cudaEvent_t ev[NPH + 1];
  for (auto& e : ev) LU_CK(h, cudaEventCreate(&e));
  for (int q = 0; q < NPH; ++q) phase_ms[q] = 0.0;
  int rc = 0;
  for (int it = 0; it < niter && !rc; ++it) {
    cudaEventRecord(ev[0], h->stream);
    rc = launch_exch(h);
    cudaEventRecord(ev[1], h->stream);
    if (!rc) rc = launch_jac(h, 0, h->nzones);
    cudaEventRecord(ev[2], h->stream);
    if (!rc) rc = launch_lower(h, true, 0, h->nzones);
    cudaEventRecord(ev[3], h->stream);
    if (!rc) rc = launch_phase(h, NPBMZ_LU_PHASE_UPPER, -1);
    cudaEventRecord(ev[4], h->stream);
    if (!rc) rc = launch_phase(h, NPBMZ_LU_PHASE_UPDATE, -1);
    cudaEventRecord(ev[5], h->stream);
    if (!rc) rc = launch_phase(h, NPBMZ_LU_PHASE_RHS, -1);
    cudaEventRecord(ev[6], h->stream);
    if (cudaEventSynchronize(ev[NPH]) != cudaSuccess) rc = fail(h, "event synchronisation failed");
    for (int q = 0; q < NPH && !rc; ++q) {
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, ev[q], ev[q + 1]);
      phase_ms[q] += ms;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return rc;
}

const char* npbmz_lu_last_error(npbmz_lu_t* h) { return h ? h->err.c_str() : g_lu_error.c_str(); }

int npbmz_lu_destroy(npbmz_lu_t* h) {
  if (!h) return fail(nullptr, "null handle");
  cudaStreamSynchronize(h->stream);
  free_all(h);
  delete h;
  return 0;
}

}  // extern "C"
