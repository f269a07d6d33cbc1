// noalloc.cu -- a BT x sweep for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc at the point where they
// want a line solve: a host runtime that owns every byte of device memory
// through its own pool or garbage collector (a cudaMalloc behind its back can
// fail under its memory cap or fragment its pool), or a time-stepping loop
// that must not pay the device-wide synchronisation that cudaFree implies.
// npbmz_bt_xsolve_noalloc serves them: it runs the primitive-variable kernel
// and the FP64 BT x-sweep kernel of the handle path on one zone whose u and
// rhs the caller already holds on the device, and takes all of its working
// memory from one file-scope device array instead of allocating.
//
// The array is NOALLOC_SCRATCH_BYTES (16 MiB) on every GPU that loads the
// library, held until the process exits.  It is shared by every call: two
// calls whose kernels overlap on the GPU (different streams, or different
// host threads) race on it and must be serialised by the caller.  Nothing in
// it has to start at zero: the primitive kernel writes every plane element the
// sweep reads, and the sweep writes each 5x5 block before reading it back.
//
// The device addresses of the arrays are looked up once per device, on the
// first call made with that device current, under a lock (host threads may
// make their first calls at the same time).  cudaDeviceReset unloads the
// library's module on that device: a process that resets a device must not
// call this entry point on it afterwards.
#define NPBMZ_NS noalloc
#define NPBMZ_HAS_FP32 0
#include "step_kernels.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/npbmz.h"

namespace npbmz {
void set_global_error(const char* msg);  // npbmz_last_error(NULL) reports it
}

namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = 16u << 20;
constexpr size_t NOALLOC_SCRATCH_DOUBLES = NOALLOC_SCRATCH_BYTES / sizeof(double);
constexpr int NOALLOC_TPB = 64;          // lines per CTA
constexpr int NOALLOC_MAX_WORK = 4096;   // CTAs of one call
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];
static __device__ npbmz::ZoneDev g_noalloc_zone;
static __device__ npbmz::Work g_noalloc_work[NOALLOC_MAX_WORK];

// Device addresses of the three arrays, looked up once per device.
struct DeviceSymbols {
  double* scratch = nullptr;
  npbmz::ZoneDev* zone = nullptr;
  npbmz::Work* work = nullptr;
};
DeviceSymbols g_symbols[NOALLOC_MAX_DEVICES];
std::mutex g_symbols_lock;  // guards the first lookup on each device
int noalloc_fail(const char* msg, cudaError_t e = cudaSuccess, int code = -1) {
  char buf[320];
  if (e != cudaSuccess) snprintf(buf, sizeof(buf), "npbmz_bt_xsolve_noalloc: %s: %s", msg, cudaGetErrorString(e));
  else snprintf(buf, sizeof(buf), "npbmz_bt_xsolve_noalloc: %s", msg);
  npbmz::set_global_error(buf);
  return code;
}

// Writes the one-zone descriptor and the CTA work list into their file-scope
// arrays (device code names them directly; no host copy is involved).
__global__ void k_noalloc_tables(int nx, int ny, int nz, int nwork, int tpb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    g_noalloc_zone.nx = nx;
    g_noalloc_zone.ny = ny;
    g_noalloc_zone.nz = nz;
    g_noalloc_zone.pad = 0;
    g_noalloc_zone.off = 0;
    g_noalloc_zone.lineoff[0] = g_noalloc_zone.lineoff[1] = g_noalloc_zone.lineoff[2] = 0;
  }
  if (i < nwork) {
    g_noalloc_work[i].zone = 0;
    g_noalloc_work[i].first = i * tpb;
  }
}

// Set-up for the current device: the host-side names of the arrays are not
// device addresses, so ask the runtime for the addresses (this needs the
// device current, which it is: the caller's current device).
int symbols_for_current_device(DeviceSymbols** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail("cudaGetDevice failed", e);
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return noalloc_fail("device index out of range");
  std::lock_guard<std::mutex> guard(g_symbols_lock);
  DeviceSymbols& s = g_symbols[dev];
  if (!s.scratch) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return noalloc_fail("cudaGetSymbolAddress(scratch) failed", e);
    void* z = nullptr;
    e = cudaGetSymbolAddress(&z, g_noalloc_zone);
    if (e != cudaSuccess) return noalloc_fail("cudaGetSymbolAddress(zone) failed", e);
    void* w = nullptr;
    e = cudaGetSymbolAddress(&w, g_noalloc_work);
    if (e != cudaSuccess) return noalloc_fail("cudaGetSymbolAddress(work) failed", e);
    s.zone = static_cast<npbmz::ZoneDev*>(z);
    s.work = static_cast<npbmz::Work*>(w);
    s.scratch = static_cast<double*>(p);
  }
  *out = &s;
  return 0;
}

// set_constants (src/BT/set_constants.jl:53-130), as the handle path does.
npbmz::Consts noalloc_consts(const double* params) {
  const double dt = params[0];
  const int gx = (int)params[1], gy = (int)params[2], gz = (int)params[3], xz = (int)params[4], yz = (int)params[5];
  npbmz::Consts k;
  std::memset(&k, 0, sizeof(k));
  k.c1 = 1.4e0; k.c2 = 0.4e0; k.c3 = 0.1e0; k.c4 = 1.0e0; k.c5 = 1.4e0;
  k.bt = std::sqrt(0.5e0);
  k.c1c2 = k.c1 * k.c2; k.c1c5 = k.c1 * k.c5; k.c3c4 = k.c3 * k.c4; k.c1345 = k.c1c5 * k.c3c4;
  k.conz1 = (1.0e0 - k.c1c5);
  k.dx1 = k.dx2 = k.dx3 = k.dx4 = k.dx5 = 0.75e0;
  k.dy1 = k.dy2 = k.dy3 = k.dy4 = k.dy5 = 0.75e0;
  k.dz1 = k.dz2 = k.dz3 = k.dz4 = k.dz5 = 1.0e0;
  k.dssp = 0.25e0;
  k.con43 = 4.0e0 / 3.0e0; k.con16 = 1.0e0 / 6.0e0; k.c2iv = 2.5e0;
  k.dt = dt;
  k.dnxm1 = 1.0e0 / ((double)(gx - 1) / (double)xz);
  k.dnym1 = 1.0e0 / ((double)(gy - 1) / (double)yz);
  k.dnzm1 = 1.0e0 / (double)(gz - 1);
  k.tx1 = 1.0e0 / (k.dnxm1 * k.dnxm1); k.tx2 = 1.0e0 / (2.0e0 * k.dnxm1);
  k.dttx1 = dt * k.tx1; k.dttx2 = dt * k.tx2;
  return k;
}

}  // namespace

extern "C" int npbmz_bt_xsolve_noalloc(int nx, int ny, int nz, const double* params, const double* u, double* rhs,
                                       void* stream) {
  if (!params || !u || !rhs) return noalloc_fail("null argument");
  if (nx < 3 || ny < 3 || nz < 3) return noalloc_fail("zone sizes must be at least 3");
  // the handle path's npbmz_create checks: the constants divide by gx-1, gy-1,
  // gz-1 and the zone counts, and a non-finite dt would poison every value
  if (!std::isfinite(params[0])) return noalloc_fail("params[0] (dt) must be finite");
  for (int q = 1; q < 6; ++q)
    if (!std::isfinite(params[q]) || params[q] != std::floor(params[q]) || params[q] > 1e9)
      return noalloc_fail("params[1..5] (gx, gy, gz, x_zones, y_zones) must be whole numbers");
  if (params[1] < 2 || params[2] < 2 || params[3] < 2)
    return noalloc_fail("params[1..3] (gx, gy, gz) must be at least 2");
  if (params[4] < 1 || params[5] < 1) return noalloc_fail("params[4..5] (x_zones, y_zones) must be at least 1");
  const int64_t np = (int64_t)nx * ny * nz;
  const int64_t lines = (int64_t)(ny - 2) * (nz - 2);
  const int64_t prim_doubles = ((int64_t)npbmz::PR_COUNT * np + 31) / 32 * 32;
  const int64_t need = prim_doubles + 25 * (int64_t)nx * lines;
  if (need > (int64_t)NOALLOC_SCRATCH_DOUBLES) {
    char msg[200];
    snprintf(msg, sizeof(msg),
             "zone %dx%dx%d needs %lld bytes of working memory; npbmz_bt_xsolve_noalloc has %zu (use a handle)", nx, ny,
             nz, (long long)(need * 8), NOALLOC_SCRATCH_BYTES);
    return noalloc_fail(msg, cudaSuccess, -2);
  }
  const int nwork = (int)((lines + NOALLOC_TPB - 1) / NOALLOC_TPB);
  if (nwork > NOALLOC_MAX_WORK) return noalloc_fail("too many lines for one call");
  // An error left pending by the caller's own earlier work is reported, not
  // consumed: cudaPeekAtLastError leaves it for the caller to read.
  const cudaError_t before = cudaPeekAtLastError();
  if (before != cudaSuccess) return noalloc_fail("a CUDA error from earlier work is pending", before);
  DeviceSymbols* sym = nullptr;
  if (symbols_for_current_device(&sym)) return -1;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);

  k_noalloc_tables<<<(nwork + 127) / 128, 128, 0, s>>>(nx, ny, nz, nwork, NOALLOC_TPB);

  npbmz::Fields F;
  F.u = const_cast<double*>(u);
  F.rhs = rhs;
  F.forcing = nullptr;
  F.prim = sym->scratch;
  F.uex = nullptr;
  F.zones = sym->zone;
  F.NP = np;
  F.primf = nullptr;
  const npbmz::Consts K = noalloc_consts(params);
  npbmz::noalloc::launch_prim(false, F, K, 0, np, s);
  npbmz::noalloc::launch_solve(false, 0, 0, F, K, sym->work, nwork, NOALLOC_TPB, sym->scratch + prim_doubles, lines, 0,
                               nullptr, s, false, 0);
  // nothing was pending before the three launches, so this is theirs
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail("kernel launch failed", e);
  return 0;
}
