// common_launch.h -- host launchers of common_kernels.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "npbmz_internal.cuh"

namespace npbmz {
void launch_initialize(const Fields& F, const Consts& K, const double* ce, const Work* work, int nwork, double* uex,
                       cudaStream_t s);
void launch_exact_rhs(const Fields& F, const Consts& K, const double* ce, const Work* work, int nwork, double* forcing,
                      cudaStream_t s);
void launch_exch_qbc(const Fields& F, const int* nbr_dev, int zone_lo, int nz_count, int max_face, cudaStream_t s);
void launch_err_partials(const Fields& F, const Work* work, int nwork, double* partials, cudaStream_t s);
void launch_norm_finish(const ZoneDev* zones, const double* partials, const int* zblk, int nzones, double scale,
                        double* out, cudaStream_t s);
// zlist (optional, device): the nzn zones to convert instead of [zone_lo, zone_lo + nzn);
// part: which points of an upload (k_convert: 0 all, 1 exch_qbc's sources,
// 2 all but exch_qbc's destinations)
void launch_convert(const Fields& F, double* planes, double* stage, const int64_t* soff, int64_t sub, int zone_lo,
                    int nzn, int max_np, int kind, int field, int layout, int dir, cudaStream_t s,
                    const int* zlist = nullptr, int part = 0);
void launch_fill(double* a, int64_t n, double v, cudaStream_t s);
void launch_state_check(const Fields& F, const Work* work, int nwork, cudaStream_t s);
void launch_math_check(int which, int n, const double* x, double* y, cudaStream_t s);
// pack (true) or unpack the listed faces to / from the device buffer buf
void launch_faces(bool pack, const Fields& F, const FaceDesc* faces, int nfaces, int max_face, double* buf,
                  cudaStream_t s);
int probe_fp64(double* gflops);
}  // namespace npbmz
