// adjoint_launch.h -- host launchers of adjoint.cu (discrete adjoint of the
// BT-MZ step).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "npbmz_internal.cuh"

namespace npbmz {
// Transposed block-tridiagonal sweep `dir` over the line work list (tpb lines
// per item): yb (in: adjoint of the sweep's output, out: of its input),
// vb -= the state linearisation; xs is the forward sweep's solution; scr
// holds 30 doubles per line point ([(p*30+e)*nlt + line]).
void adj_launch_solve(int dir, const Fields& F, const Consts& K, const Work* work, int nwork, int tpb, double* yb,
                      const double* xs, double* vb, double* scr, int64_t nlt, cudaStream_t s);
// compute_rhs adjoint over the all-points work list (128 points per item).
void adj_launch_rhs(const Fields& F, const Consts& K, const Work* work, int nwork, const double* rb, double* vb,
                    double* fb, cudaStream_t s);
// exch_qbc adjoint: ub must hold vb on entry.
void adj_launch_exch(const Fields& F, const int* nbr, int nzones, int max_face, const double* vb, double* ub,
                     cudaStream_t s);
void adj_launch_seed(const Fields& F, const Work* work, int nwork, const double* a, const double* b, double* out,
                     double* partial, int interior_only, cudaStream_t s);
}  // namespace npbmz
