/*
 * dadi_gb300 -- C ABI of the GB300 (sm_103a) diffusion integrator.
 *
 * Every entry point takes plain pointers and sizes, returns an int status
 * (DGB_OK == 0, negative on error, see dgb_status_string) and never throws.
 * Array arguments are DEVICE pointers unless a comment says "host".  Arrays
 * are C-ordered float64 with every axis of length L (dadi's square grids,
 * dadi/integration_c.pyx:74-161).  `stream` is a cudaStream_t (NULL = legacy
 * default stream); all work is enqueued on it and no call synchronises unless
 * it says so.  `ws`/`ws_bytes` is caller-owned device scratch; query the size
 * with dgb_workspace_bytes.  Calls are re-entrant: no global mutable state.
 *
 * Parameter tables.  A time loop (dadi/Integration.py:178-727) is described
 * by one row per step, evaluated on the host exactly as the reference does
 * (parameters at the *next* time, dt from the *current* ones):
 *   row[0] = this_dt, row[1] = theta0, row[2+k] = nu_k, row[2+P+k] = gamma_k,
 *   row[2+2P+k] = h_k, row[2+3P] = beta (1-D only, else 1),
 *   row[3+3P+...] = m_kj for k = 0..P-1, j != k in increasing j.
 * so a row holds DGB_ROW_STRIDE(P) doubles.
 */
#ifndef DADI_GB300_H
#define DADI_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DGB_OK 0
#define DGB_ERR_ARG (-1)         /* invalid argument (ValueError on the Python side) */
#define DGB_ERR_CUDA (-2)        /* a CUDA call failed */
#define DGB_ERR_UNSUPPORTED (-3) /* size or mode outside what the kernels handle */
#define DGB_ERR_WORKSPACE (-4)   /* workspace missing or too small */
#define DGB_ERR_TOO_LARGE (-5)   /* grid larger than dgb_integrate2d_noalloc's static scratch */

#define DGB_MAX_DIM 5
#define DGB_ROW_STRIDE(P) (3 + 3 * (P) + (P) * ((P)-1))

/* Parametric time dependence of one parameter, evaluated on the device.
 * Forms: CONST a; EXPGROW a*(b/a)**(t/c) (dadi/Demographics2D.py:302-303);
 * EXPLOG a*exp(log(b/a)*t/c); LINEAR a + b*t. */
#define DGB_PF_CONST 0
#define DGB_PF_EXPGROW 1
#define DGB_PF_EXPLOG 2
#define DGB_PF_LINEAR 3
typedef struct {
    int kind;
    int pad_;
    double a, b, c;
} dgb_pform;

/* One 2-population integration for the batched engine: the arguments of
 * Integration.two_pops (dadi/Integration.py:260-263) in parametric form. */
typedef struct {
    double T, initial_t;
    dgb_pform nu[2], m12, m21, gamma[2], h[2], theta0;
    int frozen_mask, nomut_mask;
} dgb_inst2d;

/* Per-instance status bits written by the batched engine. */
#define DGB_ST_BADPARAM 1  /* a negative size/migration/theta0 or zero size */
#define DGB_ST_STEPCAP 2   /* exceeded the per-integration step cap */
#define DGB_ST_NONFINITE 4 /* dt or phi became non-finite */
#define DGB_ST_ZERODT 8    /* timestep is zero (dadi/Integration.py:173-175) */

/* Timestep settings read at call time (dadi/Integration.py:25,39,42-44). */
typedef struct {
    double timescale_factor;     /* default 1e-3 */
    double old_timescale_factor; /* default 0.1 */
    int use_old_timestep;        /* default 0 */
    int use_delj_trick;          /* default 0 */
    int gam_placement;           /* batched engine: 0 auto, 1 shared memory, 2 workspace */
    int threads;                 /* batched engine: threads per CTA, 0 auto (the fewest
                                    warps, 2-4, that give every line of the largest grid a
                                    lane; for a launch over one grid of 73-128 points, two
                                    work items per CTA on ceil(2L/32) warps where that fills
                                    the lanes better), or 64 / 96 /
                                    128 where that many threads hold every line (else
                                    auto), one item per CTA, or -2: as auto but with two
                                    items per CTA at any L where that fills the warps'
                                    lanes better */
    int line_solver;             /* batched N-dimensional engine: 0 Thomas, one line per
                                    thread (dadi/tridiag.c:14-34); 1 parallel cyclic
                                    reduction, one warp per line (L <= 128); 2 partitioned
                                    Thomas, `segments` threads per line (L >= 3 segments);
                                    1 and 2 without the delj trick */
    int segments;                /* line_solver 2: segments per line, 2, 4 or 8 (0: 4) */
} dgb_settings;

int dgb_abi_version(void);
const char *dgb_status_string(int status);

/* Load every kernel of the library on the current device now.  CUDA loads a
 * kernel at its first launch by default, and that load can wait for the
 * device to go idle, so a first launch on one stream would serialise behind
 * work in flight on others; call this once before concurrent use
 * (DGB_ERR_CUDA if a kernel cannot be loaded). */
int dgb_preload(void);

/* Scratch bytes needed by a call.  kind: 0 = dgb_integrate_table /
 * dgb_integrate_table_states / dgb_integrate_precalc / the single sweeps
 * (for 3-5 populations and 2-D grids too large for shared memory: per-step
 * coefficient records, see dgb_integrate_table), 1 = dgb_batch2d_integrate
 * and dgb_items2d_integrate (with n = number of work items), 2 =
 * dgb_tridiag_batch, 3 = dgb_items2d_integrate with one_per_cta, 4 =
 * dgb_adjoint_table_nd. */
size_t dgb_workspace_bytes(int kind, int ndim, int L, long n);

/* Batched Numerical-Recipes tridiagonal solve of `batch` independent systems
 * of size n, system s stored at [s*n, (s+1)*n).  Replaces
 * tridiag_cython.tridiag (dadi/tridiag_cython.pyx:14-18, dadi/tridiag.c:14-40). */
int dgb_tridiag_batch(const double *a, const double *b, const double *c,
                      const double *r, double *u, int n, int batch,
                      void *ws, size_t ws_bytes, void *stream);

/* One fully implicit sweep of phi along `axis`, in place.  mig (host, ndim
 * doubles) holds the migration rates into the swept population from each
 * other population (mig[axis] ignored).  Replaces integration_c.implicit_1Dx,
 * implicit_2Dx/2Dy, implicit_3Dx/3Dy/3Dz and implicit_4Dx/4Dy/4Dz/4Da
 * (dadi/integration_c.pyx:68-161; dadi/integration1D.c:7-66,
 * integration2D.c:19-160, integration3D.c:13-239, integration4D.c:13-321). */
int dgb_implicit_sweep(double *phi, int ndim, int L, int axis, const double *xx,
                       double nu, const double *mig, double gamma, double h,
                       double beta, double dt, int use_delj_trick,
                       void *ws, size_t ws_bytes, void *stream);

/* One constant-coefficient sweep: b excludes 1/dt; b+1/dt and r = phi/dt per
 * element.  Replaces integration_c.implicit_precalc_2Dx/2Dy/3Dx/3Dy/3Dz
 * (dadi/integration_c.pyx:86-131; dadi/integration2D.c:162-217,
 * integration3D.c:241-345). */
int dgb_implicit_precalc_sweep(double *phi, int ndim, int L, int axis,
                               const double *a, const double *b, const double *c,
                               double dt, void *ws, size_t ws_bytes, void *stream);

/* A whole time loop of `nsteps` steps described by a parameter table (device,
 * nsteps rows of DGB_ROW_STRIDE(ndim) doubles).  Each step injects mutations
 * (skipped for populations in frozen_mask | nomut_mask) and sweeps every axis
 * not in frozen_mask.  2-D grids up to the shared-memory limit run as one
 * CTA with phi resident in shared memory for the whole loop; other shapes
 * run one fused sweep kernel per axis per step.  Replaces the loops of
 * Integration.one_pop/two_pops/three_pops/four_pops (dadi/Integration.py:
 * 224-257, 340-386, 514-553, 635-726) and dadi.cuda.Integration.
 * _two_pops_temporal_params / _three_pops_temporal_params /
 * _four_pops_temporal_params (dadi/cuda/Integration.py:163-291, 376-545,
 * 547-750). */
int dgb_integrate_table(double *phi, int ndim, int L, const double *xx,
                        const double *table, int nsteps, int frozen_mask,
                        int nomut_mask, int use_delj_trick,
                        void *ws, size_t ws_bytes, void *stream);

/* dgb_integrate_table for one 2-population integration spread over a
 * thread-block cluster of `cluster` CTAs (2, 4, 8 or 16), one SM each: each
 * CTA holds a block of rows of phi in shared memory, the x sweep is a
 * partitioned Thomas solve across the cluster (segment end rows exchanged
 * through distributed shared memory), the y sweep one within each CTA.  For
 * a lone integration, whose one CTA would be bound by one SM's FP64 pipe.
 * Agrees with dgb_integrate_table to rounding; default delta_j only (no
 * use_delj_trick argument); 24 <= L <= 128, 3 cluster <= L <= 16 cluster
 * (else DGB_ERR_UNSUPPORTED).  No workspace. */
int dgb_integrate2d_cluster(double *phi, int L, const double *xx, const double *table,
                            int nsteps, int frozen_mask, int nomut_mask, int cluster,
                            void *stream);

/* A whole constant-coefficient time loop: abc holds 3*ndim arrays of L^ndim
 * doubles (a_0, b_0, c_0, a_1, ...; b without 1/dt, as built by
 * dadi/Integration.py:1057-1095, 1145-1222); dts (device) the nsteps step
 * lengths; theta0 the mutation scale.  Replaces the precalc loops of
 * _two_pops_const_params / _three_pops_const_params (dadi/Integration.py:
 * 1108-1117, 1231-1241) and dadi.cuda.Integration._two_pops_const_params /
 * _three_pops_const_params (dadi/cuda/Integration.py:89-161, 293-374). */
int dgb_integrate_precalc(double *phi, int ndim, int L, const double *xx,
                          const double *abc, const double *dts, int nsteps,
                          double theta0, int frozen_mask, int nomut_mask,
                          void *ws, size_t ws_bytes, void *stream);

/* Batched 2-population engine, step 1: the per-step parameter rows of many
 * parametric two_pops integrations (the loop of dadi/Integration.py:346-386:
 * dt from the current parameters by _compute_dt, :147-176, parameters at the
 * next time, the reference's validation), one device thread per schedule.
 * Run it twice: fill == 0 writes row_cnt[s]; after the caller's exclusive
 * scan of row_cnt into row_off, fill == 1 writes the rows (DGB_ROW_STRIDE(2)
 * doubles each) at table + row_off[s]*11 and ORs DGB_ST_* bits into
 * status[instance] (caller zeroes it).  Or once: with row_cnt[s] holding an
 * upper bound on the rows of schedule s and row_off its exclusive scan,
 * fill == 2 writes the rows there and replaces row_cnt[s] by their number
 * (a walk that would pass the bound stops with DGB_ST_STEPCAP).  There is
 * one schedule per instance,
 * or per (instance, grid) when settings->use_old_timestep makes dt depend on
 * the grid; dx0s (device) holds each grid's first spacing.
 *   insts  device, ninst dgb_inst2d */
int dgb_sched2d(const dgb_inst2d *insts, int ninst, int ngrids, const double *dx0s,
                const dgb_settings *settings, long max_steps, int fill, int *row_cnt,
                const long *row_off, double *table, int *status, void *stream);

/* Batched 2-population engine, step 2: ninst integrations x ngrids grids as
 * one persistent launch; each (instance, grid) pair is a work item that keeps
 * phi in shared memory for its whole loop and reads its schedule's rows.
 *   masks    device, ninst ints: frozen_mask | nomut_mask << 8 (null: none)
 *   Ls       host, ngrids grid sizes
 *   xx_all   device, concatenated grids (sum of Ls doubles)
 *   phi0_all device, concatenated initial densities (sum of L^2), shared by
 *            every instance
 *   phi_out  device, for grid g the block of ninst*L_g^2 doubles starting
 *            after the blocks of grids < g (instance-major inside a block)
 *   table, row_off, row_cnt  the rows of step 1
 *   order    device, ninst*ngrids work ids (inst*ngrids + g) in start order
 *            (longest first balances best)
 * Many calls of Integration.two_pops become one launch; the reference runs
 * such batches as host processes (dadi/DFE/Cache2D_mod.py:117-167). */
int dgb_batch2d_integrate(const int *masks, int ninst, const int *Ls, int ngrids,
                          const double *xx_all, const double *phi0_all, double *phi_out,
                          const double *table, const long *row_off, const int *row_cnt,
                          const int *order, const dgb_settings *settings,
                          void *ws, size_t ws_bytes, void *stream);

/* Adjoint (reverse-mode) gradients of the batched 2-population engine with
 * respect to DGB_AD_NPAR model parameters theta.  dgb_seed2d holds, per
 * instance, d(T)/dtheta, d(initial_t)/dtheta and d(coefficient)/dtheta for
 * the a, b, c coefficients of the nine parametric forms of dgb_inst2d in the
 * order nu[0], nu[1], m12, m21, gamma[0], gamma[1], h[0], h[1], theta0. */
#define DGB_AD_NPAR 6
typedef struct {
    double dT[DGB_AD_NPAR];
    double dt0[DGB_AD_NPAR];
    double dform[9][3][DGB_AD_NPAR];
} dgb_seed2d;

/* Forward-mode pass over the same schedules as dgb_sched2d(fill=1): writes,
 * for each step, d(q)/dtheta (DGB_AD_NPAR doubles) for q = dt, nu1, nu2, m12,
 * m21, gamma1, gamma2, h1, h2, theta0 (60 doubles per step) at
 * drows + row_off[s]*60, following the value walk branch for branch
 * (dadi/Integration.py:147-176, 355-366).  insts/seeds device arrays.  It
 * reads no value rows, so it may run on another stream concurrently with
 * the forward integration (one lane per schedule and parameter). */
int dgb_sched2d_deriv(const dgb_inst2d *insts, const dgb_seed2d *seeds, int ninst, int ngrids,
                      const double *dx0s, const dgb_settings *settings, const int *row_cnt,
                      const long *row_off, double *drows, void *stream);

/* dgb_batch2d_integrate that also stores, for every work item, phi before
 * every ckpt_every-th step (row-major L*L doubles each) at
 * ckpt + ckpt_off[work id] -- the checkpoints the adjoint restarts from. */
int dgb_batch2d_integrate_ckpt(const int *masks, int ninst, const int *Ls, int ngrids,
                               const double *xx_all, const double *phi0_all, double *phi_out,
                               const double *table, const long *row_off, const int *row_cnt,
                               const int *order, const dgb_settings *settings, double *ckpt,
                               const long *ckpt_off, int ckpt_every, void *ws, size_t ws_bytes,
                               void *stream);

/* dgb_batch2d_integrate_ckpt over the work items order[0 .. norder) only,
 * leaving reserve_sms SMs to other launches: the rest of a batch whose
 * longest items run at the same time on clusters
 * (dgb_items2d_integrate_cluster with checkpoints). */
int dgb_batch2d_integrate_ckpt_part(const int *masks, int ninst, const int *Ls, int ngrids,
                                    const double *xx_all, const double *phi0_all,
                                    double *phi_out, const double *table, const long *row_off,
                                    const int *row_cnt, const int *order, int norder,
                                    int reserve_sms, const dgb_settings *settings, double *ckpt,
                                    const long *ckpt_off, int ckpt_every, void *ws,
                                    size_t ws_bytes, void *stream);

/* Discrete adjoint of those integrations.  lam (device, phi_out layout) holds
 * dJ/dphi_final on entry and is overwritten; grad (device, ninst x ngrids x
 * DGB_AD_NPAR) receives each (instance, grid) work item's part of
 * dJ/dtheta (written, not accumulated, so the caller's sum over the grids is
 * in a fixed order and the result does not depend on CTA timing).
 * Each work item recomputes its checkpoint segments forward and walks them
 * backwards through the transposed tridiagonal solves.  Scratch per CTA:
 * dgb_adjoint2d_scratch_bytes; ws = 256 bytes of counter + that scratch for
 * as many CTAs as it holds.  The delj trick is not supported here
 * (DGB_ERR_UNSUPPORTED).  The reference has no adjoint; its gradients come
 * from finite differences (dadi/Godambe.py:131-185). */
size_t dgb_adjoint2d_scratch_bytes(int Lmax, int ckpt_every, int nblocks);
int dgb_adjoint2d(const int *masks, int ninst, const int *Ls, int ngrids, const double *xx_all,
                  const double *table, const double *drows, const long *row_off,
                  const int *row_cnt, const double *ckpt, const long *ckpt_off, int ckpt_every,
                  double *lam, double *grad, const int *order, const dgb_settings *settings,
                  void *ws, size_t ws_bytes, void *stream);

/* dgb_adjoint2d with every checkpoint segment of every work item recomputed
 * at once, one CTA per (work item, segment), before the backward walks: a
 * long integration's recomputation no longer runs serially on its own
 * CTA.  traj (device) holds, for work item w at traj_off[w], the densities
 * phi_0..phi_n followed by the x-sweep outputs chi_0..chi_{n-1}
 * ((2 n_w + 1) L_g^2 doubles, n_w its steps); seg_off (device, nwork + 1
 * longs) is the exclusive scan of each work item's segment count
 * ceil(n_w / ckpt_every).  ws: dgb_adjoint2d_traj_ws_bytes(Lmax, nblocks)
 * for nblocks CTAs.  The same arithmetic as dgb_adjoint2d, so the same
 * gradients bit for bit. */
size_t dgb_adjoint2d_traj_ws_bytes(int Lmax, int nblocks);
int dgb_adjoint2d_traj(const int *masks, int ninst, const int *Ls, int ngrids,
                       const double *xx_all, const double *table, const double *drows,
                       const long *row_off, const int *row_cnt, const double *ckpt,
                       const long *ckpt_off, int ckpt_every, double *traj, const long *traj_off,
                       const long *seg_off, double *lam, double *grad, const int *order,
                       const dgb_settings *settings, void *ws, size_t ws_bytes, void *stream);

/* dgb_adjoint2d / dgb_adjoint2d_traj over part of the work items: the walk
 * covers order[0 .. norder) (work ids inst * ngrids + grid) on at most
 * max_blocks CTAs (<= 0: no cap), so that two calls on two streams share
 * the GPU -- e.g. the longest items in trajectory mode (traj non-null;
 * seg_off over all ninst * ngrids work ids, zero segments for the others)
 * and the rest with per-CTA segment recomputation (traj null: ws as for
 * dgb_adjoint2d).  Each item's lambda and gradient part are those of the
 * whole-batch calls, bit for bit.  cluster (trajectory mode only): walk
 * each item on a thread-block cluster of that many CTAs (2, 4, 8, 16), the
 * transposed solves partitioned across them as dgb_integrate2d_cluster
 * partitions the forward -- for a few long items, whose walk on one CTA is
 * bound by one SM's FP64 pipe; every grid within that function's range (else
 * DGB_ERR_UNSUPPORTED); lambda and gradients then agree with the one-CTA
 * walk to rounding. */
int dgb_adjoint2d_part(const int *masks, int ninst, const int *Ls, int ngrids,
                       const double *xx_all, const double *table, const double *drows,
                       const long *row_off, const int *row_cnt, const double *ckpt,
                       const long *ckpt_off, int ckpt_every, double *traj,
                       const long *traj_off, const long *seg_off, double *lam, double *grad,
                       const int *order, int norder, int max_blocks, int cluster,
                       const dgb_settings *settings, void *ws, size_t ws_bytes, void *stream);

/* One work item of dgb_items2d_integrate: a 2-D integration on grid
 * xx_all[xx_off .. xx_off+L) whose density sits at phi_out + out_off (initial
 * density on entry, result on exit), driven by schedule `sched` (index into
 * row_off / row_cnt), with masks = frozen_mask | nomut_mask << 8. */
typedef struct {
    int L;
    int masks;
    long xx_off;
    long out_off;
    long sched;
} dgb_item2d;

/* The batched 2-D integration over an explicit list of work items, so one
 * launch mixes grids of different sizes and integrations of different
 * requests (the serving engine's continuous batches).  Lmax bounds every
 * item's L; order (device, optional) gives the start order.  one_per_cta = 0:
 * a persistent launch sized to the device whose CTAs pull items from a queue
 * (ws from dgb_workspace_bytes kind 1); one_per_cta = 1: one CTA per item,
 * each retiring after its item, so launches on other streams take SMs as
 * soon as any CTA finishes (ws from kind 3 with n = nitems).
 * settings->gam_placement: 0 Thomas scratch in shared memory when it fits
 * and costs no CTAs per SM, else the workspace; 1 shared memory
 * (DGB_ERR_UNSUPPORTED if it does not fit); 2 the workspace. */
int dgb_items2d_integrate(const dgb_item2d *items, int nitems, int Lmax, const double *xx_all,
                          double *phi_out, const double *table, const long *row_off,
                          const int *row_cnt, const int *order, const dgb_settings *settings,
                          int one_per_cta, void *ws, size_t ws_bytes, void *stream);

/* dgb_items2d_integrate with one thread-block cluster of `cluster` CTAs per
 * item (the kernel of dgb_integrate2d_cluster): for a few items, which one
 * CTA each would leave bound by one SM's FP64 pipe.  Lmin / Lmax (host)
 * bound every item's L and must satisfy dgb_integrate2d_cluster's range
 * (else DGB_ERR_UNSUPPORTED); an item outside them is skipped.  With ckpt
 * (device, optional) the density before every ckpt_every-th step is stored,
 * row-major, from ckpt + ckpt_off[i] for item i (ckpt_off: device, nitems
 * longs; the checkpoints of dgb_batch2d_integrate_ckpt).  Default delta_j
 * only; no order, settings or workspace.  Results agree with
 * dgb_items2d_integrate to rounding. */
int dgb_items2d_integrate_cluster(const dgb_item2d *items, int nitems, int Lmin, int Lmax,
                                  const double *xx_all, double *phi_out, const double *table,
                                  const long *row_off, const int *row_cnt, int cluster,
                                  double *ckpt, const long *ckpt_off, int ckpt_every,
                                  void *stream);

/* dgb_sched2d evaluated in C on the host (all arrays HOST): table == NULL
 * counts rows into row_cnt; otherwise writes the rows at table +
 * row_off[i]*11 and ORs status bits into status[i].  One schedule per
 * instance on a grid with first spacing dx0.  For callers that must not wait
 * on the device (the serving loop forms batches while kernels run). */
int dgb_sched2d_host(const dgb_inst2d *insts, int ninst, const dgb_settings *settings,
                     long max_steps, double dx0, int *row_cnt, const long *row_off,
                     double *table, int *status);

/* Host helper: the number of steps of each schedule, evaluated in C on the
 * host (insts is a HOST array here); the same walk as dgb_sched2d. */
int dgb_batch2d_count_steps(const dgb_inst2d *insts, int ninst,
                            const dgb_settings *settings, long max_steps,
                            long *steps_out);

/* Discrete adjoint of the N-dimensional table-driven time loop (1-4
 * populations), for any parameter table.
 *
 * dgb_integrate_table_states: dgb_integrate_table through the per-axis
 * sweeps that also records the density at the start of every step and at the
 * end: states (device) holds (nsteps + 1) x L^ndim doubles.  (The delj trick
 * is not differentiated.)  ws: as dgb_integrate_table (kind 0); a smaller
 * workspace (or none) only costs speed.
 *
 * dgb_adjoint_table_nd: lam (device, L^ndim) holds dJ/dphi_final on entry
 * and dJ/dphi_initial on exit; gpart (device,
 * nsteps x dgb_adjoint_table_nd_gpart_doubles) receives per step the partial
 * sums of dJ/d(table row entries): for each swept axis j (in sweep order)
 * one DGB_ROW_STRIDE(ndim) row per CTA of that sweep, followed by two
 * doubles, the injection's dJ/d(dt) and dJ/d(theta0).  Summing a step's
 * rows (any fixed order) and adding those two to entries 0 and 1 gives
 * dJ/d(row) for that step.  ws: (active axes - 1) x L^ndim doubles, and
 * with dgb_workspace_bytes(4, ...) bytes also the coefficient records of the
 * recomputed sweeps (faster, same results).  The
 * reference has no adjoint; its gradients come from finite differences
 * (dadi/Godambe.py:131-185). */
int dgb_integrate_table_states(double *phi, int ndim, int L, const double *xx,
                               const double *table, int nsteps, int frozen_mask,
                               int nomut_mask, double *states, void *ws, size_t ws_bytes,
                               void *stream);
size_t dgb_adjoint_table_nd_gpart_doubles(int ndim, int L);
int dgb_adjoint_table_nd(double *lam, int ndim, int L, const double *xx, const double *table,
                         int nsteps, int frozen_mask, int nomut_mask, const double *states,
                         double *gpart, double *ws, size_t ws_bytes, void *stream);

/* Batched N-dimensional engine: nitems integrations of ndim populations
 * (1-5) on one grid xx of L points advance together; each step sweeps every
 * axis once over the lines of every integration still running.  Replaces
 * many calls of Integration.three_pops / four_pops / five_pops
 * (dadi/Integration.py:389-554, 556-727, 729-937; the reference runs them one
 * at a time, or as host processes, dadi/DFE/Cache2D_mod.py:117-167).  Each
 * integration's density is bitwise the one dgb_integrate_table computes for
 * it alone.
 *   items   device, nitems dgb_itemnd, longest first (nsteps non-increasing)
 *   nsteps  HOST, the same nitems step counts (they drive the launches)
 *   phi_all device, the densities (each L^ndim doubles at its phi_off):
 *           initial densities on entry, results on exit
 *   table   device, parameter rows (DGB_ROW_STRIDE(ndim) doubles each, the
 *           layout above); integration i uses rows row_off .. row_off+nsteps
 *   settings use_delj_trick; threads = lines per CTA (0 auto, 32, 64, 128);
 *           gam_placement 0 auto (workspace), 1 shared memory, 2 workspace;
 *           line_solver / segments (Thomas by default; the partitioned
 *           Thomas solve with one item is the fast form of a lone 3-D grid
 *           of few lines, e.g. 63 ms instead of 92 ms for 675 steps at L=70)
 *   ws      dgb_batchnd_workspace_bytes(ndim, L, nitems, settings) bytes */
typedef struct {
    long phi_off; /* offset of the density in phi_all, in doubles */
    long row_off; /* first table row */
    int nsteps;   /* rows (steps) */
    int masks;    /* frozen_mask | nomut_mask << 8 */
} dgb_itemnd;
size_t dgb_batchnd_workspace_bytes(int ndim, int L, int nitems, const dgb_settings *settings);
int dgb_batchnd_integrate(const dgb_itemnd *items, const int *nsteps, int nitems, int ndim,
                          int L, const double *xx, double *phi_all, const double *table,
                          const dgb_settings *settings, void *ws, size_t ws_bytes,
                          void *stream);

/* The discrete adjoint of many N-dimensional integrations at once: the
 * batched forms of dgb_integrate_table_states and dgb_adjoint_table_nd
 * (the same per-step records, recomputation and transposed sweeps, every
 * sweep launch over the lines of every integration still running; each
 * integration's states, lambda and gpart are bitwise those of the
 * one-at-a-time calls).  Items are HOST arrays here, nitems of them sorted
 * longest first; each names its density (phi_all + phi_off: the initial
 * density on entry of the forward, dJ/dphi_final on entry of the adjoint,
 * dJ/dphi_initial on its exit), its table rows, its nsteps + 1 recorded
 * densities (states_all + state_off) and its nsteps x
 * dgb_adjoint_table_nd_gpart_doubles(ndim, L) partial rows (gpart_all +
 * gpart_off, laid out as dgb_adjoint_table_nd's, each step's rows by axis).
 * Thomas line solver; without the delj trick (DGB_ERR_UNSUPPORTED).
 * ws: dgb_batchnd_adjoint_workspace_bytes (records, Thomas scratch, the
 * recomputed sweep outputs: (ndim - 1) L^ndim doubles per item). */
typedef struct {
    long phi_off, row_off, state_off, gpart_off; /* in doubles / rows */
    int nsteps;
    int masks; /* frozen_mask | nomut_mask << 8 */
} dgb_itemnd_adj;
size_t dgb_batchnd_adjoint_workspace_bytes(int ndim, int L, int nitems,
                                           const dgb_settings *settings);
int dgb_batchnd_integrate_states(const dgb_itemnd_adj *items, int nitems, int ndim, int L,
                                 const double *xx, double *phi_all, const double *table,
                                 double *states_all, const dgb_settings *settings, void *ws,
                                 size_t ws_bytes, void *stream);
int dgb_batchnd_adjoint(const dgb_itemnd_adj *items, int nitems, int ndim, int L,
                        const double *xx, double *lam_all, const double *table,
                        const double *states_all, double *gpart_all,
                        const dgb_settings *settings, void *ws, size_t ws_bytes, void *stream);

/* One P-population integration (P = 1-5) in parametric form: the arguments
 * of Integration.one_pop .. five_pops (dadi/Integration.py:178-937) with
 * every parameter a dgb_pform; mig[k][j] is the rate into population k from
 * j (the diagonal is ignored). */
typedef struct {
    double T, initial_t;
    dgb_pform nu[DGB_MAX_DIM], gamma[DGB_MAX_DIM], h[DGB_MAX_DIM];
    dgb_pform mig[DGB_MAX_DIM][DGB_MAX_DIM];
    dgb_pform theta0;
    int ndim, pad_;
} dgb_instnd;

/* Parameter rows of parametric integrations, evaluated in C on the HOST
 * (all arrays host): the loop of dadi/Integration.py:504-553 (three_pops),
 * 672-726 (four_pops), 884-935 (five_pops), 224-257 (one_pop): dt from the
 * current parameters by _compute_dt (:147-176, the minimum over
 * populations), the parameters at the next time, the same validation
 * (reported as DGB_ST_* bits in status[i], which the caller zeroes).
 * table == NULL counts rows into row_cnt; otherwise row_cnt[i] bounds the
 * rows written at table + row_off[i] * DGB_ROW_STRIDE(ndim) and is replaced
 * by their number.  dx0 is the grid's first spacing (old-timestep mode). */
int dgb_schednd_host(const dgb_instnd *insts, int ninst, const dgb_settings *settings,
                     long max_steps, double dx0, int *row_cnt, const long *row_off,
                     double *table, int *status);

/* Derivative seeds of a dgb_instnd with respect to npar <= DGB_ND_MAXPAR
 * model parameters: d(a, b, c)/dtheta of every form (index 0, 1, 2 of the
 * middle dimension), dT and d(initial_t).  Unused entries are zero. */
#define DGB_ND_MAXPAR 16
typedef struct {
    double dT[DGB_ND_MAXPAR], dt0[DGB_ND_MAXPAR];
    double dnu[DGB_MAX_DIM][3][DGB_ND_MAXPAR];
    double dgamma[DGB_MAX_DIM][3][DGB_ND_MAXPAR];
    double dh[DGB_MAX_DIM][3][DGB_ND_MAXPAR];
    double dmig[DGB_MAX_DIM][DGB_MAX_DIM][3][DGB_ND_MAXPAR];
    double dtheta0[3][DGB_ND_MAXPAR];
} dgb_seednd;

/* The schedule walk of dgb_schednd_host for one integration in forward-mode
 * dual numbers (HOST arrays): the same rows, bit for bit, and their
 * derivatives with respect to the seeded parameters, drows[n][c][p] =
 * d table[n][c] / d theta_p (rows x DGB_ROW_STRIDE(ndim) x npar), along
 * the branch each max/min of the walk takes (_compute_dt,
 * dadi/Integration.py:147-176; the final partial step T - t).  The rows
 * feed the discrete adjoint's chain rule dJ/dtheta = sum dJ/drow drow/dtheta.
 * table == NULL counts into *nrows; otherwise *nrows bounds the rows
 * written and is replaced by their number.  status as dgb_schednd_host. */
int dgb_schednd_dual_host(const dgb_instnd *inst, const dgb_seednd *seed, int npar,
                          const dgb_settings *settings, long max_steps, double dx0,
                          int *nrows, double *table, double *drows, int *status);

/* Spectrum epilogue of 2-D integrations (device-resident inputs, one launch
 * per list).  dgb_from_phi2d: raw spectrum of each density,
 * out[a][b] (n1+1 x n2+1) = the piecewise-linear integral of phi against
 * binomial sampling (dadi/Spectrum_mod.py:1509-1547, _from_phi_2D_linalg),
 * given the weight tables d1 = dbeta1, d2 = dbeta2 of cached_dbeta(n, xx)
 * (:25-40), each (n+1) x (L-1) C-ordered.  The item array itself is in device
 * memory; Lmax / nmax bound every item's L and n2 (they size the shared
 * memory: dgb_from_phi2d_smem_bytes), items outside them are skipped.  The
 * reference computes these on the host with numpy after copying phi back. */
typedef struct {
    const double *phi;        /* L x L density */
    const double *xx;         /* the grid */
    const double *d1x, *d2x;  /* weight tables for n1 */
    const double *d1y, *d2y;  /* weight tables for n2 */
    double *out;              /* (n1+1) x (n2+1) */
    int L, n1, n2, pad_;
} dgb_fs_item2d;
size_t dgb_from_phi2d_smem_bytes(int Lmax, int nmax);
int dgb_from_phi2d(const dgb_fs_item2d *items, int nitems, int Lmax, int nmax, void *stream);

/* Raw spectra of nbatch densities of ndim populations (1-5), each L^ndim
 * doubles (C order, all axes on the grid xx of L points), stored one after
 * another in phi: out receives nbatch spectra of prod(ns[a]+1) doubles.
 * The linear-algebra form of Spectrum.from_phi (dadi/Spectrum_mod.py:
 * 1509-1547 for 2-D, 1774-1810 for 3-D, 1841-1870 for 4-D, 1938-2061):
 * each axis, last first, is contracted against its weight tables d1[a] =
 * dbeta1 and d2[a] = dbeta2 of cached_dbeta(ns[a], xx) (:25-40), device
 * pointers to (ns[a]+1) x (L-1) doubles; ns, d1 and d2 are HOST arrays of
 * ndim entries.  ws: dgb_from_phi_nd_workspace_bytes (the tensors between
 * contractions).  The reference computes these on the host with numpy. */
size_t dgb_from_phi_nd_workspace_bytes(int ndim, int L, const int *ns, int nbatch);
int dgb_from_phi_nd(const double *phi, int nbatch, int ndim, int L, const double *xx,
                    const int *ns, const double *const *d1, const double *const *d2,
                    double *out, void *ws, size_t ws_bytes, void *stream);

/* Extrapolation of 1-3 grids' spectra to zero grid spacing at x = 0
 * (linear_extrap / quadratic_extrap, dadi/Numerics.py:644-669; x = each
 * grid's xx[1], the Spectrum's extrap_x) with entries more than fail_mag
 * orders of magnitude from the smallest-x grid's replaced by it
 * (dadi/Numerics.py:449-464), written to out; with data and ll set, also the
 * Poisson log-likelihood sum(-m + d log m - lgamma(d + 1)), m = scale * out,
 * over entries with m > 0, excluding the first and last entry when
 * mask_corners (dadi/Inference.py:466-509); with data and ll_multinom set,
 * the multinomial log-likelihood: the same sum with scale = sum(d) / sum(out)
 * over the entries not excluded (ll_multinom with optimal_sfs_scaling,
 * dadi/Inference.py:559-575, 668-685). */
typedef struct {
    const double *fs[3];
    double x[3];
    double *out;
    const double *data;       /* NULL: no likelihood */
    double *ll;               /* one double (NULL: no Poisson likelihood) */
    double *ll_multinom;      /* one double (NULL: no multinomial likelihood) */
    double scale;
    int ngrids, size, mask_corners, pad_;
} dgb_extrap_item;
int dgb_extrap_ll(const dgb_extrap_item *items, int nitems, double fail_mag, void *stream);

/* Allocation-free 2-D integration; it has no counterpart in the reference.
 * The same computation as dgb_integrate_table for ndim == 2 (one integration
 * through a parameter table, phi updated in place), for callers that cannot
 * allocate device memory or pass a workspace -- e.g. code that runs where
 * cudaMalloc is not allowed or a caching allocator must not be entered, or
 * a host that embeds the library without a device allocator of its own.
 * Grids small enough for the Thomas scratch to sit in shared memory beside
 * the density (on GB300 up to L = 116, or 113 with the delj trick) keep it
 * there.  Larger grids use a file-scope device array of DGB_NOALLOC_MAX_L^2
 * doubles (128 KB) that every GPU which loads the library holds until the
 * process exits; grids with L > DGB_NOALLOC_MAX_L return DGB_ERR_TOO_LARGE.
 * The first such call on each device looks up the array's address
 * (cudaGetSymbolAddress) with that device current, so make that first call
 * before any stream capture; a failed lookup returns DGB_ERR_CUDA and is
 * retried by the next call.  Device ordinals 64 and up return
 * DGB_ERR_UNSUPPORTED.  Every call that uses the array shares it, and it
 * keeps the previous call's contents (nothing in it needs to start at
 * zero): such calls that overlap on the GPU -- on different streams or from
 * different host threads -- race on it, so serialise them.  The call
 * allocates nothing. */
#define DGB_NOALLOC_MAX_L 128
int dgb_integrate2d_noalloc(double *phi, int L, const double *xx, const double *table,
                            int nsteps, int frozen_mask, int nomut_mask, int use_delj_trick,
                            void *stream);

/* Measurement helpers with no counterpart in the reference.
 * dgb_probe_fp64_fma: blocks x threads threads, of which the first
 * active_lanes lanes of every warp run 8 independent chains of `iters` FP64
 * FMAs and store one double each to out[blocks*threads] (device).  Timing it
 * gives the FP64 pipe's FMA rate (the roofline of the sweeps) and shows
 * whether idle lanes cost issue slots.
 * dgb_probe_rcp: out[i] = the kernels' refined reciprocal of x[i] (device),
 * so tests can check it against correctly rounded division. */
int dgb_probe_fp64_fma(double *out, int blocks, int threads, int iters, int active_lanes,
                       void *stream);
int dgb_probe_rcp(const double *x, double *out, int n, void *stream);

#ifdef __cplusplus
}
#endif
#endif
