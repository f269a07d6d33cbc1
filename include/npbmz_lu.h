/* npbmz_lu.h -- C ABI of the LU-MZ SSOR iteration in libnpbmz_gpu.so
 * (GB300, sm_103a): the third NPB-MZ application of NPBApps.jl.
 *
 * The reference's seam is, as for BT-MZ and SP-MZ, the pair of calls in the
 * node time loop (src/LU/lu-node.jl:233-303): exch_qbc(...) over all zones,
 * then ssor(iz, ...) per zone under Threads.@threads.  One LU-MZ zone is a
 * whole LU domain with its own unit-cube coordinates (src/LU/setcoeff.jl,
 * src/LU/exact.jl); one process per zone (the single-rank case: no
 * exchange_1/3/4/5/6 traffic inside a zone).  Every call returns an int
 * status (0 = success, negative = error, text from npbmz_lu_last_error; for
 * npbmz_lu_zone_setup, a failed npbmz_lu_create and a NULL handle,
 * npbmz_lu_last_error(NULL), kept per host thread).  A handle is not
 * re-entrant.  Device work is issued on the handle's stream.
 *
 * Host layouts (one zone):
 *   NPBMZ_LAYOUT_DENSE  [m][k][j][i], m = 0..4, k < nz, j < ny, i < nx
 *                       (i fastest), 5*nx*ny*nz doubles;
 *   NPBMZ_LAYOUT_REF    the reference's OffsetArray memory, column-major,
 *                       pointer to the first element of the parent array:
 *                         u, rsd, frct [1:5, -1:nx+2, -1:ny+2, 1:nz]
 *                         (src/LU/lu_data.jl:96-103)
 *                       only points 1..nx, 1..ny are read or written; the
 *                       halo is left untouched.
 */
#ifndef NPBMZ_LU_H
#define NPBMZ_LU_H

#include <stddef.h>
#include <stdint.h>

#include "npbmz.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct npbmz_lu_handle npbmz_lu_t;

/* flags */
#define NPBMZ_LU_FACES_NPB 0x1 /* exch_qbc copies the zone-face planes
                                  k = 2..nz-1, as NPB-MZ's LU-MZ does; the
                                  default copies the reference's k = 1..nz-2
                                  (src/LU/exchange_qbc.jl:85,109,135,160),
                                  which leaves plane nz-1 of every ghost face
                                  at its setbv value, so the reference's own
                                  verify norms (src/LU/verify.jl) are met only
                                  with this flag */
#define NPBMZ_LU_GRAPH 0x2     /* npbmz_lu_iterate replays one captured CUDA
                                  graph per iteration */
#define NPBMZ_LU_FMA 0x4       /* the iteration's kernels built with FMA
                                  contraction (a*b+c rounded once): faster on
                                  the FP64 pipe, no longer bit-for-bit the
                                  reference's rounding (setbv, setiv, erhs,
                                  exch_qbc's face copies and the norms stay
                                  uncontracted; the flux quantities of u and
                                  every rhs, the first included, come from the
                                  contracted build) */

/* fields */
#define NPBMZ_LU_U 0
#define NPBMZ_LU_RSD 1
#define NPBMZ_LU_FRCT 2

/* phases of npbmz_lu_phase */
#define NPBMZ_LU_PHASE_RHS 0    /* rhs (src/LU/rhs.jl) */
#define NPBMZ_LU_PHASE_SCALE 1  /* rsd *= dt on the interior (src/LU/ssor.jl:62-70) */
#define NPBMZ_LU_PHASE_LOWER 2  /* jacld + blts over k = 2..nz-1 (src/LU/ssor.jl:72-106) */
#define NPBMZ_LU_PHASE_UPPER 3  /* jacu + buts over k = nz-1..2 (src/LU/ssor.jl:112-172) */
#define NPBMZ_LU_PHASE_UPDATE 4 /* u += rsd / (omega (2 - omega)) (src/LU/ssor.jl:180-190) */
#define NPBMZ_LU_PHASE_EXCH 5   /* exch_qbc over all zones (zone ignored) */
#define NPBMZ_LU_PHASE_SSOR 6   /* the whole ssor call */

/* Zone sizes and neighbours of src/LU/zone_setup.jl:1-111: zone number
 * (i-1)+(j-1)*x_zones; nbr receives 4 ints per zone: west, east, south,
 * north (0-based), LU's rule (north/south step along x, west/east along y).
 * Returns an error where the reference's Int conversion of an extent would
 * throw or a neighbour falls outside the zones (its rule assumes
 * x_zones == y_zones). */
int npbmz_lu_zone_setup(int gx, int gy, int gz, int x_zones, int y_zones, double ratio, int* nx, int* ny, int* nz,
                        int* nbr);

/* Create a handle on the current CUDA device and allocate its buffers
 * (about 1.2 KB per point; a problem that does not fit in the device's free
 * memory is rejected before anything is allocated).
 * params = {dt, omega} (the reference: dt from the class, omega_default 1.2,
 * src/LU/lu_data.jl:2).  setcoeff (src/LU/setcoeff.jl) is evaluated per zone.
 * Replaces alloc_field_space + setcoeff (src/LU/lu_data.jl:92, lu-node.jl:86-97). */
int npbmz_lu_create(int nzones, const int* nx, const int* ny, const int* nz, const int* nbr, const double* params,
                    int flags, npbmz_lu_t** out);

/* setbv, setiv, erhs and the first rhs of every zone on the device, from the
 * 5x13 coefficient table ce (row-major [5][13]; NULL: the reference's table,
 * src/LU/setcoeff.jl).  Replaces lu-node.jl:93-152 (the warm-up iteration
 * that follows there is undone by setbv / setiv / rhs and leaves no trace). */
int npbmz_lu_setup(npbmz_lu_t* h, const double* ce);

/* Host <-> device transfer of one field of one zone (zone >= 0) or of all
 * zones (zone = -1, arrays back to back in zone order).  Synchronous. */
int npbmz_lu_upload(npbmz_lu_t* h, int zone, int field, int layout, const double* host);
int npbmz_lu_download(npbmz_lu_t* h, int zone, int field, int layout, double* host);

/* exch_qbc over all zones (src/LU/exchange_qbc.jl:1-288), on the device. */
int npbmz_lu_exch_qbc(npbmz_lu_t* h);

/* ssor of one zone (zone >= 0) or of all zones batched (zone = -1):
 * rsd *= dt, jacld + blts, jacu + buts, update, rhs (src/LU/ssor.jl:9-254). */
int npbmz_lu_ssor(npbmz_lu_t* h, int zone);

/* niter iterations of the time loop body (src/LU/lu-node.jl:233-270):
 * exch_qbc over all zones, then ssor of every zone.  rsdnm (nullable)
 * receives 5 doubles per iteration: the l2norm of rsd after that
 * iteration, summed over zones (src/LU/l2norm.jl).  Synchronous.  State
 * check: every iteration's update tests the points it writes; a density
 * that is not positive and finite, or a non-finite value, makes the call
 * return NPBMZ_LU_ERR_STATE after its iterations, with the first bad point
 * in npbmz_lu_last_error; a non-positive pressure-like quantity
 * u5 - (u2^2 + u3^2 + u4^2) / (2 u1) is only reported (npbmz_lu_state_check):
 * LU takes no root of it and the reference carries such a state on. */
#define NPBMZ_LU_ERR_STATE (-3)
int npbmz_lu_iterate(npbmz_lu_t* h, int niter, double* rsdnm);

/* What the state check of the last npbmz_lu_iterate found: bits =
 * NPBMZ_LU_STATE_* (0 when healthy) and the first bad point's zone and
 * 0-based (i, j, k) of the dense layout (all -1 when none); nullable.  No
 * counterpart in the reference. */
#define NPBMZ_LU_STATE_DENSITY 1
#define NPBMZ_LU_STATE_PRESSURE 2
#define NPBMZ_LU_STATE_NONFINITE 4
int npbmz_lu_state_check(npbmz_lu_t* h, int* bits, int* zone, int* i, int* j, int* k);

/* The end-of-run norms of lu-node.jl:306-321, summed over zones: xcr (l2norm
 * of rsd), xce (error against exact), xci (pintgr surface integral).
 * Synchronous. */
int npbmz_lu_verify(npbmz_lu_t* h, double* xcr, double* xce, double* xci);

/* One phase (NPBMZ_LU_PHASE_*) of one zone (>= 0) or all zones (-1). */
int npbmz_lu_phase(npbmz_lu_t* h, int phase, int zone);

/* Stream (cudaStream_t; NULL: the handle's own) and synchronisation. */
int npbmz_lu_set_stream(npbmz_lu_t* h, void* stream);
int npbmz_lu_synchronize(npbmz_lu_t* h);

/* Kernel launches of one batched iteration (exch_qbc + ssor). */
int npbmz_lu_launches_per_iteration(npbmz_lu_t* h);

/* Per-phase device time of niter batched iterations from CUDA events on the
 * handle's stream, summed: {exch, jac (jacld's and jacu's blocks of every
 * point), lower (blts, rsd *= dt fused), upper (buts), update, rhs} in ms.
 * Advances the state. */
int npbmz_lu_profile(npbmz_lu_t* h, int niter, double* phase_ms);

const char* npbmz_lu_last_error(npbmz_lu_t* h);
int npbmz_lu_destroy(npbmz_lu_t* h);

#ifdef __cplusplus
}
#endif

#endif /* NPBMZ_LU_H */
