// step_launch.h -- host launchers of the time-step kernels, one set per build
// variant (exact: -fmad=false, fast: -fmad=true).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "npbmz_internal.cuh"

namespace npbmz {
#define NPBMZ_DECLARE_LAUNCHERS(NS)                                                                                  \
  namespace NS {                                                                                                     \
  void launch_prim(bool sp, const Fields& F, const Consts& K, int64_t lo, int64_t hi, cudaStream_t s);                                   \
  void launch_prim_w(bool sp, const Fields& F, const Consts& K, const Work* work, int nwork, cudaStream_t s,        \
                     bool persist = false);                                                                          \
  void launch_rhs(bool tx, bool norm, const Fields& F, const Consts& K, const Work* work, int nwork,                 \
                  double* partials, cudaStream_t s, const RhsF64Consts* rc = nullptr, bool persist = false);         \
  void launch_solve(bool sp, int mode, int dir, const Fields& F, const Consts& K, const Work* work, int nwork,       \
                    int tpb, void* scratch, int64_t nlt, int add_u, double* xw, cudaStream_t s,                      \
                    bool persist = false, int ctas_per_sm = 0);                                                      \
  void launch_add(const Fields& F, const Work* work, int nwork, cudaStream_t s);                                     \
  }
NPBMZ_DECLARE_LAUNCHERS(exact)
NPBMZ_DECLARE_LAUNCHERS(fast)
#undef NPBMZ_DECLARE_LAUNCHERS
namespace fast {
// dst (10 float planes: double-float hi 0..4, lo 5..9) <- src (5 FP64 planes)
void launch_split_df(const double* src, float* dst, int64_t NP, cudaStream_t s);
// dst = a * src (n values)
void launch_scale(const double* src, double* dst, double a, int64_t n, cudaStream_t s);
// dst (5 float2 planes {hi, lo}) <- src (5 FP64 planes)
void launch_split_f2(const double* src, float2* dst, int64_t NP, cudaStream_t s);
// primitive kernel and compute_rhs of the refined mixed step in double-float
void launch_prim_df(bool sp, const Fields& F, const RhsDfConsts& C, const Work* work, int nwork, cudaStream_t s,
                    bool persist);
void launch_rhs_df(bool tx, bool norm, const Fields& F, const RhsDfConsts& C, const Work* work, int nwork,
                   double* partials, cudaStream_t s, bool persist);
// x-line-major copies of the FP32 state pairs for the x-sweep items
// work[0..nwork) of lpi lines each
void launch_xline_copy(bool sp, const Fields& F, const Work* work, int nwork, int lpi, cudaStream_t s);
// compute_rhs (the FP64 kernel with the point functions) and those copies in
// one launch: work[0..nwork) compute_rhs items, cwork[0..ncopy) copy items
void launch_rhs_xc(bool tx, bool norm, const Fields& F, const Consts& K, const RhsF64Consts& rc, const Work* work,
                   int nwork, double* partials, const Work* cwork, int ncopy, int lpi, cudaStream_t s, bool persist);
// the forcing at both ends of every x line into Fields::rdx
void launch_xline_ends(const Fields& F, const Work* work, int nwork, int tpb, cudaStream_t s);
// dynamic shared memory limits of the pipelined sweeps; 0 on success
int configure_kernels();
}  // namespace fast
}  // namespace npbmz
