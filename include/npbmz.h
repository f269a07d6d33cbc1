/* npbmz.h -- C ABI of libnpbmz_gpu.so, the GB300 (sm_103a) ADI time step of
 * the NPBApps.jl BT-MZ and SP-MZ solvers.
 *
 * The reference has no plugin API: its seam is the pair of Julia calls in the
 * node time loop, exch_qbc(...) then adi(iz, ...) per zone
 * (src/BT/bt-node.jl:286-395, src/SP/sp-node.jl:258-397).  Each entry point
 * below names the reference function it replaces.  Every call returns an int
 * status (0 = success, negative = error; npbmz_last_error() gives the text);
 * no C++ exception crosses the ABI.  A handle is not re-entrant: calls on one
 * handle must come from one thread at a time.  All device work of a handle is
 * issued on the handle's stream (npbmz_set_stream), asynchronously unless the
 * entry point says otherwise.
 *
 * Field arrays exchanged with the host use one of two layouts:
 *   NPBMZ_LAYOUT_DENSE  per zone, [m][k][j][i] with m = 0..4, k < nz, j < ny,
 *                       i < nx (i fastest), nx*ny*nz*5 doubles;
 *   NPBMZ_LAYOUT_REF    the reference's own OffsetArray memory for one zone
 *                       (ncells = 1), column-major, pointer to the first
 *                       element of the parent array:
 *                         BT u       [1:5, -2:IMAX+1, -2:JMAX+1, -2:KMAX+1]  (src/BT/bt_data.jl:143-144)
 *                         BT rhs     [1:5, -1:IMAX-1, -1:JMAX-1, -1:KMAX-1]  (src/BT/bt_data.jl:148-149)
 *                         BT forcing [1:5,  0:IMAX-1,  0:JMAX-1,  0:KMAX-1]  (src/BT/bt_data.jl:138-139)
 *                         SP u       [-2:IMAXP+1, -2:JMAXP+1, -2:KMAX+1, 1:5] (src/SP/sp_data.jl:115-116)
 *                         SP rhs, forcing [0:IMAXP-1, 0:JMAXP-1, 0:KMAX-1, 1:5] (src/SP/sp_data.jl:160-166)
 *                       with IMAX = nx+1, JMAX = ny+1, KMAX = nz+1,
 *                       IMAXP = 2*(IMAX/2)+1, JMAXP = 2*(JMAX/2)+1.
 *                       Only the points 0..n-1 of each axis are read or
 *                       written; the halo is left untouched.
 */
#ifndef NPBMZ_H
#define NPBMZ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct npbmz_handle npbmz_t;

/* problem kinds */
#define NPBMZ_BT 0
#define NPBMZ_SP 1

/* variant flags (npbmz_create) */
#define NPBMZ_EXACT   0x1  /* FP64 kernels built without FMA contraction, in the
                              reference's operation order: bit-for-bit the
                              reference's arithmetic */
#define NPBMZ_MIXED   0x2  /* line solves in FP32 as a defect correction on
                              the FP64 rhs: refined once against a residual of
                              the line operator formed in double-float (FP32
                              pairs, about 48 bits), in FP64 with
                              NPBMZ_REFINE_FP64; compute_rhs, add, exch_qbc
                              and the norms stay FP64, so the fixed point is
                              the FP64 one */
#define NPBMZ_PERZONE 0x4  /* one launch per zone per phase, the reference's
                              per-zone adi order; default is all zones batched
                              in one launch per phase */
#define NPBMZ_GRAPH   0x8  /* npbmz_step replays one captured CUDA graph per step */
#define NPBMZ_PERSIST 0x10 /* the batched step's primitive, compute_rhs and
                              pipelined FP32 sweep kernels (FMA build) run
                              persistent: as many CTAs as fit on the SMs at
                              once, each looping over zone x point or
                              zone x line work items; results are unchanged */
#define NPBMZ_REFINE_FP64 0x40 /* with NPBMZ_MIXED: the refinement residual in
                              FP64 instead of double-float */
#define NPBMZ_RHS_DF 0x80  /* with NPBMZ_MIXED: the primitive kernel and
                              compute_rhs in double-float too (FP32 pairs on
                              the FP32 pipe; faster on GB300, but compute_rhs
                              is then not FP64: the fixed point moves at the
                              1e-14 relative level) */
#define NPBMZ_FP32_NOREFINE 0x20 /* FP32 line solves without the refinement
                              pass (the error of plain FP32 solves, for
                              comparison); implies NPBMZ_MIXED */

/* field selectors */
#define NPBMZ_U       0
#define NPBMZ_RHS     1
#define NPBMZ_FORCING 2

/* host layouts */
#define NPBMZ_LAYOUT_DENSE 0
#define NPBMZ_LAYOUT_REF   1

/* single phases (npbmz_phase) */
#define NPBMZ_PHASE_RHS     0  /* compute_rhs, plus txinvr for SP */
#define NPBMZ_PHASE_XSOLVE  1  /* x sweep (+ ninvr for SP) */
#define NPBMZ_PHASE_YSOLVE  2  /* y sweep (+ pinvr for SP) */
#define NPBMZ_PHASE_ZSOLVE  3  /* z sweep (+ tzetar for SP), without add */
#define NPBMZ_PHASE_ADD     4  /* u += rhs on the interior */
#define NPBMZ_PHASE_EXCH    5  /* exch_qbc over all zones */
#define NPBMZ_PHASE_RHSONLY 6  /* compute_rhs only (SP: no txinvr) */

/* Zone geometry of src/BT/zone_setup.jl:1-77 (SP: src/SP/zone_setup.jl:1-78).
 * nx, ny, nz receive x_zones*y_zones sizes (zone number (i-1)+(j-1)*x_zones);
 * nbr receives 4 ints per zone: west, east, south, north (0-based). */
int npbmz_zone_setup(int kind, int gx, int gy, int gz, int x_zones, int y_zones, double ratio, int* nx, int* ny,
                     int* nz, int* nbr);

/* Seeded manufactured-solution coefficients, written row-major [5][13] into
 * ce.  Every coefficient is drawn U(0.5, 2.0) from a SplitMix64 stream seeded
 * with `seed`; the energy row is then multiplied by the smallest power of two
 * 2^e (e >= 0) such that rho > 0 and rhoE - |rho v|^2/(2 rho) >= 0.25 rhoE
 * hold for the exact solution and for the transfinite interpolation of its
 * face values at every grid coordinate the zones of this geometry use
 * (i*dnxm1 for i < max nx, and so on).  Returns e (>= 0) or a negative error.
 * No counterpart in the reference, whose ce table is fixed
 * (src/BT/set_constants.jl:47-51). */
int npbmz_seeded_coefficients(uint64_t seed, int nzones, const int* nx, const int* ny, const int* nz, int gx, int gy,
                              int gz, int x_zones, int y_zones, double* ce);

/* Create a handle on the current CUDA device and allocate every device buffer
 * it will use.  params = {dt, gx, gy, gz, x_zones, y_zones}: set_constants
 * (src/BT/set_constants.jl:53-130) is evaluated from them.  nbr as written by
 * npbmz_zone_setup.  Replaces alloc_field_space + set_constants
 * (src/BT/bt_data.jl:106, src/BT/bt-node.jl:63-93). */
int npbmz_create(int kind, int nzones, const int* nx, const int* ny, const int* nz, const int* nbr,
                 const double* params, int variant_flags, npbmz_t** out);

/* Device-side initialize + exact_rhs for all zones from the 5x13
 * coefficient table ce (row-major [5][13]); also records the exact solution
 * for the error norm.  Replaces initialize, lhsinit and exact_rhs
 * (src/BT/initialize.jl:6,229; src/BT/exact_rhs.jl:5; SP counterparts). */
int npbmz_setup(npbmz_t* h, const double* ce);

/* Host <-> device transfer of one field of one zone (zone >= 0), or of all
 * zones (zone = -1: the host buffer holds every zone's array back to back in
 * zone order).  The host buffer is read/written before the call returns. */
int npbmz_upload(npbmz_t* h, int zone, int field, int layout, const double* host);
int npbmz_download(npbmz_t* h, int zone, int field, int layout, double* host);

/* Asynchronous variants: the host buffer must stay valid (and, for full
 * overlap, be page-locked) until the stream has passed the copy. */
int npbmz_upload_async(npbmz_t* h, int zone, int field, int layout, const double* host);
int npbmz_download_async(npbmz_t* h, int zone, int field, int layout, double* host);

/* exch_qbc: copy every zone's interior boundary planes into its periodic
 * neighbours' ghost planes on the device.  Replaces exch_qbc
 * (src/BT/exchange_qbc.jl:1-122, src/SP/exchange_qbc.jl:1-122). */
int npbmz_exch_qbc(npbmz_t* h);

/* ---- zones of one problem spread over several ranks (one GPU each) ----
 * A rank creates its handle with only its own zones (npbmz_create, zones
 * renumbered 0..n-1) and marks each face whose neighbour zone lives on
 * another rank with NPBMZ_REMOTE in nbr.  npbmz_exch_qbc and npbmz_step then
 * copy only the faces between the rank's own zones; the others travel
 * through caller-owned device buffers, once per step, before the step:
 *     npbmz_pack_faces(h, send) -> the caller moves send to the peers'
 *     recv (NCCL send/recv, a peer copy) -> npbmz_unpack_faces(h, recv).
 * This is the inter-process part of exch_qbc: exch_qbc_send / exch_qbc_recv
 * (src/BT/exchange_qbc.jl:145-465, src/SP/exchange_qbc.jl:145-465), with the
 * zone-to-rank map of map_zones (src/BT/setup_mpi.jl:123-433) computed on the
 * host (npbmz/shard.py). */
#define NPBMZ_REMOTE (-1)

/* Register the faces this rank sends and receives: send[2f], send[2f+1] =
 * (zone, side) of face f, side 0..3 = west, east, south, north; recv likewise
 * (each must be an NPBMZ_REMOTE face).  A sent face (z, s) is the interior
 * plane the neighbour on side s reads (west i = 1, east i = nx-2, south
 * j = 1, north j = ny-2); a received face (z, s) is z's ghost plane on side s
 * (west i = 0, east i = nx-1, south j = 0, north j = ny-1).  Each face holds
 * 5 (n-2)(nz-2) doubles (n = ny for west/east, nx for south/north) in the
 * reference's packing order -- variable, then k = 1..nz-2, then the
 * transverse index 1..n-2 (src/BT/exchange_qbc.jl:201-210) -- and the faces
 * follow one another in list order.  Returns the doubles of the send and the
 * receive buffer.  Synchronous.  No counterpart in the reference (which posts
 * one MPI message per face). */
int npbmz_face_plan(npbmz_t* h, int nsend, const int* send, int nrecv, const int* recv, int64_t* send_count,
                    int64_t* recv_count);

/* Pack the registered send faces of u into the device buffer send_buf
 * (exch_qbc_send's packing, src/BT/exchange_qbc.jl:145-320). */
int npbmz_pack_faces(npbmz_t* h, double* send_buf);

/* Write the registered receive faces of the device buffer recv_buf into u's
 * ghost planes (exch_qbc_recv's unpacking, src/BT/exchange_qbc.jl:323-465). */
int npbmz_unpack_faces(npbmz_t* h, const double* recv_buf);

/* adi: one ADI step (compute_rhs, x/y/z solves, add) for one zone, or for all
 * zones (zone = -1, batched).  Replaces adi (src/BT/adi.jl:5-251,
 * src/SP/adi.jl:6-258). */
int npbmz_adi(npbmz_t* h, int zone);

/* nsteps time steps of exch_qbc + adi(all zones), the body of the node time
 * loop (src/BT/bt-node.jl:280-395).  norms (nullable, host) receives 10
 * doubles per step: xcr[5] (sum over zones of rhs_norm/dt of that step's
 * compute_rhs) then xce[5] (sum over zones of error_norm after the step).
 * Synchronous.  State check: the primitive kernel of every step checks the
 * state entering that step, and one kernel checks the state the call leaves
 * (npbmz_state_check returns what they found).  When some point has a density
 * rho that is not positive and finite, or a non-finite value, the call
 * returns NPBMZ_ERR_STATE after its steps and npbmz_last_error names the
 * failure and the first such point (zone, i, j, k); for SP also when the
 * pressure-like quantity rho E - |rho v|^2 / (2 rho) is not positive, whose
 * square root SP takes (src/SP/rhs.jl:84-88).  BT never takes that root and
 * the reference carries such a state on, so for BT a non-positive pressure is
 * only reported by npbmz_state_check.  The reference has no such check: a
 * diverging run continues until its final norms (src/BT/verify.jl). */
#define NPBMZ_ERR_STATE (-3)
int npbmz_step(npbmz_t* h, int nsteps, double* norms);

/* What the state check of the last npbmz_step / npbmz_step_download found:
 * bits = NPBMZ_STATE_* (0 when every point was healthy), and the first bad
 * point's zone and (i, j, k) (all -1 when none).  zone, i, j, k nullable.  No
 * counterpart in the reference. */
#define NPBMZ_STATE_DENSITY 1   /* rho not positive and finite */
#define NPBMZ_STATE_PRESSURE 2  /* rho E - |rho v|^2 / (2 rho) finite, not positive */
#define NPBMZ_STATE_NONFINITE 4 /* a NaN or an infinity in u */
int npbmz_state_check(npbmz_t* h, int* bits, int* zone, int* i, int* j, int* k);

/* nsteps steps, then u of every zone to `host` (layout as npbmz_download,
 * zone = -1): the same result as npbmz_step followed by npbmz_download.  For
 * NPBMZ_GRAPH handles with zone-group branches and a page-locked `host`, each
 * group's zones are copied out as soon as the last step's z sweep has written
 * them, while the other groups still compute.  Synchronous.  The state check
 * of npbmz_step applies (NPBMZ_ERR_STATE; u is copied out all the same).  No
 * counterpart in the reference (whose u lives in host memory). */
int npbmz_step_download(npbmz_t* h, int nsteps, int layout, double* host);

/* u of every zone from host_in, nsteps steps, u of every zone to host_out
 * (layout as npbmz_download, zone = -1; host_out may be host_in): the same
 * result as npbmz_upload + npbmz_step_download, the reference's loop with u
 * kept in host memory.  For NPBMZ_GRAPH handles with zone-group branches and
 * page-locked buffers the copies overlap the steps: the planes exch_qbc
 * reads are uploaded first and exch_qbc runs; the rest of each zone group's
 * points then arrive while earlier groups already compute, and each group
 * leaves as soon as its last z sweep is done.  Handles with NPBMZ_REMOTE
 * faces take the sequential path.  Synchronous; the state check of
 * npbmz_step applies.  No counterpart in the reference. */
int npbmz_step_inout(npbmz_t* h, int nsteps, int layout, const double* host_in, double* host_out);

/* The node part of verify (src/BT/verify.jl:411-505): error_norm of u, then
 * compute_rhs without an exchange, rhs_norm; sums over zones.  Synchronous. */
int npbmz_verify(npbmz_t* h, double* xcr, double* xce);

/* One phase (NPBMZ_PHASE_*) for one zone or all zones (zone = -1). */
int npbmz_phase(npbmz_t* h, int phase, int zone);

/* Discrete adjoint of nsteps BT-MZ time steps (exch_qbc + adi of all zones,
 * the loop body of src/BT/bt-node.jl:280-395) from the handle's current u
 * and forcing, for the terminal objective
 *     J = 1/2 * sum over every stored point of every zone of (u_N - u_target)^2.
 * u_target, grad_forcing and grad_u0 are host arrays of the dense layout for
 * all zones back to back (zone z: [5][nz][ny][nx]).  grad_forcing receives
 * dJ/dforcing and grad_u0 dJ/du_0 (either may be NULL); J (nullable) the
 * objective.  The forward pass keeps u every checkpoint_every steps; the
 * reverse pass recomputes the steps of one checkpoint interval at a time.
 * u is left as it was on entry; rhs is overwritten.  BT only.  No
 * counterpart in the reference (its gradient would come from ForwardDiff
 * dual numbers pushed through the Julia step).  Synchronous. */
int npbmz_adjoint(npbmz_t* h, int nsteps, int checkpoint_every, const double* u_target, double* J,
                  double* grad_forcing, double* grad_u0);

/* Zone groups of the step graph (NPBMZ_GRAPH, FMA build), 1..8.  With G > 1
 * the zones are split into G groups of near-equal size, and the captured
 * step runs each group's primitive kernel, compute_rhs and sweeps as one
 * branch.  Each branch starts when the previous group's compute_rhs is done,
 * so FP64-bound phases of one group run beside the FP32 sweeps of the
 * previous one.  Results are unchanged (zones are independent within a step
 * after exch_qbc).  npbmz_create sets 2 groups for NPBMZ_GRAPH handles with
 * at least 8 zones (not NPBMZ_EXACT or NPBMZ_PERZONE).  No counterpart in the
 * reference. */
int npbmz_set_step_groups(npbmz_t* h, int groups);

/* How the zone-group branches of the step graph share the SMs.
 * fp64_first != 0 issues every group's primitive kernel and compute_rhs
 * (FP64-pipe bound) on one stream of the device's greatest priority, in
 * group order, so that their CTAs reach the SMs ahead of the queued CTAs of
 * the sweeps (FP32 pipe) they overlap; the graph is instantiated with
 * per-node priorities.  sweep_ctas_per_sm > 0 runs the pipelined sweep
 * kernels as persistent grids of at most that many CTAs per SM, leaving
 * registers on every SM for the FP64 kernels beside them (0: one CTA per
 * work item).  Launch configuration only: results are unchanged.
 * npbmz_autotune chooses both with the group count.  No counterpart in the
 * reference. */
int npbmz_set_step_overlap(npbmz_t* h, int fp64_first, int sweep_ctas_per_sm);

/* Where a step of the FMA build makes the x sweep's x-line-major copies of
 * the FP32 state: on != 0 (the default) in the compute_rhs launch (one
 * kernel whose blocks each do either compute_rhs points or copy tiles, the
 * copies spread evenly over the launch), when the x-sweep work list of the
 * launch is one line shape; 0 by a copy kernel of their own after the
 * primitive kernel.  Launch configuration only: results are unchanged.
 * npbmz_autotune chooses it on whole steps.  No counterpart in the
 * reference. */
int npbmz_set_copy_fusion(npbmz_t* h, int on);

/* Use `stream` (a cudaStream_t, NULL = the legacy default stream) for all
 * later work of the handle. */
int npbmz_set_stream(npbmz_t* h, void* stream);
int npbmz_synchronize(npbmz_t* h);

/* Autotune the launch shapes (threads per block and work-item size per
 * phase and zone-size bucket), the number of zone-group branches of the step
 * graph (NPBMZ_GRAPH) and persistent kernels on or off (the NPBMZ_PERSIST bit
 * of the handle's flags) by timing candidates on the handle's own data; none
 * of them changes the results.  Leaves u, rhs and forcing as they were.
 * Synchronous.  No counterpart in the reference. */
int npbmz_autotune(npbmz_t* h);

/* The FP64 reciprocal (which = 0, the only one) that the FMA build's
 * primitive kernel uses for 1/rho instead of the IEEE divide (Newton-Raphson
 * refinement of the FP32 hardware estimate), applied on the current device
 * to x[0..n) (host) into y (host).  For the library's tests, which hold it to
 * its error bound.  No counterpart in the reference.  Synchronous. */
int npbmz_math_check(int which, int n, const double* x, double* y);

/* Measured FP64 FMA throughput of the current device in GFLOP/s (an FMA
 * counts 2 flops): the denominator of the FP64 roofline of the step kernels.
 * No counterpart in the reference. */
int npbmz_fp64_peak(double* gflops);

/* Per-phase device time of the batched step: nsteps steps launched directly
 * (the kernels npbmz_step and its graph run), with CUDA events around each
 * phase on the handle's stream; phase_ms[NPBMZ_PROF_COUNT] receives the mean
 * milliseconds per step of exch_qbc, the primitive kernel, compute_rhs and
 * the x, y and z sweeps (each sweep: all its kernels).  Advances the state
 * by nsteps steps.  No counterpart in the reference.  Synchronous. */
#define NPBMZ_PROF_EXCH 0
#define NPBMZ_PROF_PRIM 1
#define NPBMZ_PROF_RHS 2
#define NPBMZ_PROF_X 3
#define NPBMZ_PROF_Y 4
#define NPBMZ_PROF_Z 5
#define NPBMZ_PROF_COUNT 6
int npbmz_step_profile(npbmz_t* h, int nsteps, double* phase_ms);

/* Query: number of kernel launches npbmz_step issues per step, device bytes
 * held by the handle, and (info, n) a small summary string. */
int npbmz_launches_per_step(npbmz_t* h);
int64_t npbmz_device_bytes(npbmz_t* h);
int npbmz_describe(npbmz_t* h, char* buf, size_t n);

/* The FP64 BT x sweep of one zone (compute the primitive variables from u,
 * then x_solve, as NPBMZ_PHASE_XSOLVE of a handle created without NPBMZ_EXACT
 * does) for callers that cannot allocate device memory when they need it --
 * a host runtime whose own pool or garbage collector owns all device memory,
 * or a loop that cannot afford the device-wide synchronisation of cudaFree.
 * No counterpart in the reference.  u and rhs are device pointers in the dense
 * per-zone layout [m][k][j][i] of an nx*ny*nz zone; rhs is solved in place.
 * params = {dt, gx, gy, gz, x_zones, y_zones} as for npbmz_create.  All
 * working memory comes from one 16 MiB device array built into the library
 * (held by every GPU that loads it until the process exits); a zone needing
 * more (8*nx*ny*nz + 25*nx*(ny-2)*(nz-2) doubles) is rejected with -2.  The
 * call allocates nothing.  Its first call on a device looks up the array's
 * device address; make that first call before any stream capture.  Calls
 * share the array: calls whose kernels may overlap on the GPU race and must
 * be serialised by the caller.  Non-finite dt, gx/gy/gz < 2 or zone counts
 * < 1 are rejected before anything runs.  A CUDA error already pending on the
 * calling thread is reported (-1) and left pending.  After cudaDeviceReset of
 * a device, do not call it on that device again.  Errors:
 * npbmz_last_error(NULL). */
int npbmz_bt_xsolve_noalloc(int nx, int ny, int nz, const double* params, const double* u, double* rhs,
                            void* stream);

/* Error text of the last failing call on h (h may be NULL for create and for
 * npbmz_bt_xsolve_noalloc: the last such failure on the calling host
 * thread). */
const char* npbmz_last_error(npbmz_t* h);

/* Free every device buffer and the handle. */
int npbmz_destroy(npbmz_t* h);

#ifdef __cplusplus
}
#endif
#endif /* NPBMZ_H */
