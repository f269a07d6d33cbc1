// lu_launch.h -- host launchers of the LU-MZ kernels, one set per build
// (lu_exact: -fmad=false, the reference's rounding; lu_fast: -fmad=true).
#pragma once
#include "lu_types.h"

namespace npbmz_lu {
#define NPBMZ_LU_DECLARE_LAUNCHERS(NS)                                                                              \
  namespace NS {                                                                                                     \
  void rhs(bool erhs, const LuDev& D, const LuWork* w, int n, const double* g, const double* prim, double* out,     \
           cudaStream_t s);                                                                                          \
  void init(const LuDev& D, const LuWork* w, int n, const CeTable& ce, cudaStream_t s);                              \
  void poly(const LuDev& D, const LuWork* w, int n, const CeTable& ce, cudaStream_t s);                              \
  void prim(const LuDev& D, const LuWork* w, int n, const double* g, cudaStream_t s);                                \
  void pointwise(bool update, const LuDev& D, const LuWork* w, int n, double tmp, cudaStream_t s);                   \
  void jac(bool hp_order, const LuDev& D, const int* fb, int fls, const int* ri, int ls, int ks, double* jac,      \
           int z0, dim3 grid, cudaStream_t s);                                                                       \
  void lower(bool scale, const LuDev& D, const double* jac, const int* hps, int hstride, int l, int z0, dim3 grid,  \
             cudaStream_t s);                                                                                        \
  void upper(const LuDev& D, const double* jac, const int* hps, int hstride, int l, int z0, dim3 grid,              \
             cudaStream_t s);                                                                                        \
  void pack(const LuDev& D, const Faces& F, int nzones, dim3 grid, cudaStream_t s);                                  \
  void unpack(const LuDev& D, const Faces& F, int nzones, dim3 grid, cudaStream_t s);                                \
  void norm_partial(int which, const LuDev& D, const LuWork* w, int n, const CeTable& ce, double* partial,          \
                    cudaStream_t s);                                                                                 \
  void norm_finish(const LuZone* zones, const int* zblock, int nzones, const double* partial, double* out,          \
                   cudaStream_t s);                                                                                  \
  void pintgr(const LuDev& D, int nzones, double* frc, cudaStream_t s);                                              \
  void convert(bool ref, bool to_dev, const LuDev& D, double* field, double* img, int zone, int blocks,              \
               cudaStream_t s);                                                                                      \
  }
NPBMZ_LU_DECLARE_LAUNCHERS(lu_exact)
NPBMZ_LU_DECLARE_LAUNCHERS(lu_fast)
#undef NPBMZ_LU_DECLARE_LAUNCHERS
}  // namespace npbmz_lu
