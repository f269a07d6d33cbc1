// adjoint_launch.h -- host launchers of adjoint.cu (discrete adjoint of the
// BT-MZ and SP-MZ steps).
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
// SP forward recomputation: sweep dir's untransformed FP64 solution of the
// lines into ys (ys must hold the sweep's input, whose line ends it keeps;
// scr: 6 doubles per line point), and its transform from ys into rhs.
void sp_fwd_launch_solve(int dir, const Fields& F, const Consts& K, const Work* work, int nwork, int tpb, double* ys,
                         double* scr, int64_t nlt, cudaStream_t s);
void sp_fwd_launch_post(int dir, const Fields& F, const Consts& K, const Work* work, int nwork, const double* ys,
                        cudaStream_t s);
// SP transposed sweep dir (yb in/out as adj_launch_solve; ys the forward
// untransformed solution; scr 30 doubles per line point) and the txinvr
// adjoint (rb in: adjoint of txinvr's output, out: of compute_rhs's; r0 the
// forward compute_rhs output) over the all-points work list.
void adj_launch_sp_solve(int dir, const Fields& F, const Consts& K, const Work* work, int nwork, int tpb, double* yb,
                         const double* ys, double* vb, double* scr, int64_t nlt, cudaStream_t s);
void adj_launch_sp_txinvr(const Fields& F, const Consts& K, const Work* work, int nwork, double* rb, const double* r0,
                          double* vb, cudaStream_t s);
}  // namespace npbmz
