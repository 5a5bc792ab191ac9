// Discrete adjoint of the batched 2-population integrator.
//
// Forward (k_integrate2d with checkpoints): phi_{k+1} = Y_k^{-1} X_k^{-1}
// (phi_k + inj_k), with X_k, Y_k the dt-scaled tridiagonal operators
// A' = I + dt D of the x and y sweeps (dadi/integration2D.c:19-160) and inj_k
// the mutation mass of dadi/Integration.py:76-87.  Given lambda_n = dJ/dphi_n,
// each step backwards solves the transposed systems
//     mu = Y_k^{-T} lambda_{k+1},   nu = X_k^{-T} mu,   lambda_k = nu
// and contracts  dJ/dq = -mu^T (dY/dq) phi_{k+1} - nu^T (dX/dq) chi_k
// (chi_k = X_k^{-1} psi_k, psi_k = phi_k + inj_k) for every per-step scalar
// q of the parameter row: dt (through A' - I = dt D and the injection), nu,
// m, gamma, h of each axis, and theta0 (through the injection).  For dt the
// contraction is -(mu.r - mu.phi)/dt with r the sweep's right-hand side; for
// the others it is a sum over intervals of (f_i mu_i - f_{i+1} mu_{i+1})
// times the interval's coefficient derivatives (the a/b/c layout of
// compute_abc_nobc, dadi/integration_shared.c:72-93), plus the corner
// boundary terms.  The chain rule to the model parameters uses derivative
// rows dq_k/dtheta produced by a forward-mode (dual number) walk of the same
// schedule (k_sched2d_dual), which carries the schedule's own dependence on
// theta: dt from the parameters at the current time (_compute_dt,
// dadi/Integration.py:147-176), the final partial step T - t, and t/T inside
// the parametric sizes.
//
// Memory: phi is checkpointed every C steps by the forward pass; each segment
// of C steps is recomputed from its checkpoint into a per-CTA buffer, then
// walked backwards.  All per-item arrays live in global memory (per-CTA
// slices), so any grid size runs.
#include <algorithm>

#include <cooperative_groups.h>

#include "dgb_cluster.cuh"
#include "dgb_common.cuh"
#include "dgb_internal.h"

namespace dgb {

constexpr int AD_THREADS = 128;
constexpr int AD_MAXG = DGB_B2_MAXG;
constexpr int NPAR = DGB_AD_NPAR; // parameters differentiated
constexpr int NQ = 10;            // per-step scalars of a 2-D parameter row
enum { Q_DT, Q_NU0, Q_NU1, Q_M01, Q_M10, Q_G0, Q_G1, Q_H0, Q_H1, Q_TH };

// ------------------------------------------------------- dual numbers
//
// The derivative walk runs one thread per (schedule, parameter): each thread
// carries the value and one derivative component.  The FP64 pipe takes a
// warp instruction in the same time whether one lane or six are active, so
// six lanes that each repeat the value chain and carry their own component
// issue about a sixth of the FP64 instructions of one lane carrying all six
// components.

struct D1 {
    double v, d;
};

// Per-instance constants of one parametric form for one derivative
// component k: the reciprocals, logarithms and seed combinations that do not
// change along the walk.
struct PfK {
    int kind;
    double a, inv_a, inv_c, da, dc, s1, s2;
};

__device__ PfK pf_prepare(const dgb_pform &f, const double *da, const double *db,
                          const double *dc, int k)
{
    PfK c;
    c.kind = f.kind;
    c.a = f.a;
    c.inv_a = 1.0 / f.a;
    c.inv_c = 1.0 / f.c;
    c.da = da[k];
    c.dc = dc[k];
    c.s1 = 0;
    c.s2 = 0;
    switch (f.kind) {
    case DGB_PF_EXPGROW: {
        // a q^(t/c), q = b/a: s1 = (dq/dtheta)/q, s2 = log q
        const double q = f.b / f.a;
        c.s1 = (db[k] - q * da[k]) / f.a / q;
        c.s2 = log(q);
        break;
    }
    case DGB_PF_EXPLOG:
        // a exp(log(b/a) t / c): s1 = d log(b/a) / dtheta, s2 = log(b/a)
        c.s1 = db[k] / f.b - da[k] / f.a;
        c.s2 = log(f.b / f.a);
        break;
    case DGB_PF_LINEAR:
        // a + b t: s1 = db/dtheta, s2 = b
        c.s1 = db[k];
        c.s2 = f.b;
        break;
    default:
        break;
    }
    return c;
}

// A parametric form's value at t (as pform_eval gives it) and its derivative
// along component k, with t's own derivative t.d.
__device__ __forceinline__ D1 pform_d1(const dgb_pform &f, const PfK &c, const D1 &t)
{
    D1 r;
    r.v = pform_eval(f, t.v);
    switch (c.kind) {
    case DGB_PF_EXPGROW: {
        // p = q^y = value / a, y = t / c
        const double p = r.v * c.inv_a, y = t.v * c.inv_c;
        const double dy = (t.d - y * c.dc) * c.inv_c;
        r.d = p * (c.da + c.a * (y * c.s1 + c.s2 * dy));
        break;
    }
    case DGB_PF_EXPLOG: {
        // e = exp(z) = value / a, z = log(b/a) t / c
        const double e = r.v * c.inv_a, z = c.s2 * t.v * c.inv_c;
        const double dz = (c.s1 * t.v + c.s2 * t.d) * c.inv_c - z * c.dc * c.inv_c;
        r.d = e * (c.da + c.a * dz);
        break;
    }
    case DGB_PF_LINEAR:
        r.d = c.da + c.s1 * t.v + c.s2 * t.d;
        break;
    default:
        r.d = c.da;
    }
    return r;
}

// Derivative of compute_dt (dadi/Integration.py:147-176) along the branch the
// value takes; the value itself is compute_dt's.
__device__ D1 compute_dt_d1(const D1 &nu, const D1 &msum, const D1 &gamma, const D1 &h,
                            const dgb_settings &s, double dx0)
{
    D1 r;
    r.v = compute_dt(nu.v, msum.v, gamma.v, h.v, s, dx0);
    r.d = 0;
    if (s.use_old_timestep)
        return r;
    const double v1 = 0.25 / nu.v;
    const double t1 = fabs(h.v + (1 - 2 * h.v) * 0.5) * 0.5 * (1 - 0.5);
    const double u2 = h.v + (1 - 2 * h.v) * 0.25;
    const double t2 = fabs(u2) * 0.25 * (1 - 0.25);
    const bool use_t2 = t2 > t1;
    const double tm = use_t2 ? t2 : t1;
    const double v3 = fabs(gamma.v) * 2 * tm;
    int branch = 0;
    double mx = v1;
    if (msum.v > mx) {
        mx = msum.v;
        branch = 1;
    }
    if (v3 > mx) {
        mx = v3;
        branch = 2;
    }
    if (!(mx > 0))
        return r;
    double dmx;
    if (branch == 0)
        dmx = -0.25 * nu.d / (nu.v * nu.v);
    else if (branch == 1)
        dmx = msum.d;
    else {
        const double sg = gamma.v >= 0 ? 1.0 : -1.0, su = u2 >= 0 ? 1.0 : -1.0;
        const double dtm = use_t2 ? su * 0.5 * h.d * 0.25 * (1 - 0.25) : 0.0;
        dmx = sg * gamma.d * 2 * tm + fabs(gamma.v) * 2 * dtm;
    }
    r.d = -s.timescale_factor * dmx / (mx * mx);
    return r;
}

// The schedule walk of sched2d (dgb_integrate2d.cu) with component k of the
// derivatives, for exactly nrows steps: writes d(q)/dtheta_k of the NQ row
// quantities per step (stride NPAR, interleaved with the other components).
__device__ void sched2d_walk_d1(const dgb_inst2d &I, const dgb_seed2d &S,
                                const dgb_settings &st, double dx0, int nrows, int k,
                                double *drows)
{
    const dgb_pform *F[9] = {&I.nu[0], &I.nu[1], &I.m12, &I.m21, &I.gamma[0],
                             &I.gamma[1], &I.h[0], &I.h[1], &I.theta0};
    PfK c[9];
#pragma unroll
    for (int f = 0; f < 9; f++)
        c[f] = pf_prepare(*F[f], S.dform[f][0], S.dform[f][1], S.dform[f][2], k);
    D1 cur = {I.initial_t, S.dt0[k]};
    const D1 T = {I.T, S.dT[k]};
    D1 P[9];
#pragma unroll
    for (int f = 0; f < 8; f++)
        P[f] = pform_d1(*F[f], c[f], cur);
    for (int n = 0; n < nrows; n++) {
        const D1 d0 = compute_dt_d1(P[0], P[2], P[4], P[6], st, dx0);
        const D1 d1 = compute_dt_d1(P[1], P[3], P[5], P[7], st, dx0);
        const D1 dtm = (d1.v < d0.v) ? d1 : d0;
        const D1 rem = {T.v - cur.v, T.d - cur.d};
        const D1 dt = (rem.v < dtm.v) ? rem : dtm;
        const D1 next = {cur.v + dt.v, cur.d + dt.d};
#pragma unroll
        for (int f = 0; f < 9; f++)
            P[f] = pform_d1(*F[f], c[f], next);
        double *o = drows + (size_t)n * NQ * NPAR + k;
        o[0] = dt.d;
#pragma unroll
        for (int f = 0; f < 9; f++)
            o[(f + 1) * NPAR] = P[f].d;
        cur = next;
    }
}

// Eight lanes per schedule (instance, or instance x grid with
// use_old_timestep), the first NPAR of them each carrying one derivative
// component.
constexpr int SD_LANES = 8;

__global__ void k_sched2d_dual(const dgb_inst2d *insts, const dgb_seed2d *seeds, int nsched,
                               int ngrids, int per_grid, const double *dx0s, dgb_settings st,
                               const int *row_cnt, const long *row_off, double *drows)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = t / SD_LANES, k = t % SD_LANES;
    if (s >= nsched || k >= NPAR)
        return;
    const int inst = per_grid ? s / ngrids : s;
    const double dx0 = dx0s[per_grid ? s % ngrids : 0];
    sched2d_walk_d1(insts[inst], seeds[inst], st, dx0, row_cnt[s], k,
                    drows + row_off[s] * NQ * NPAR);
}

// ------------------------------------------------------- adjoint kernel

struct ADArgs {
    int ngrids;
    int L[AD_MAXG];
    long xx_off[AD_MAXG];
    long out_off[AD_MAXG];
    const double *xx_all;
    const double *table;  // value rows (11 per step)
    const double *drows;  // derivative rows (NQ*NPAR per step), same row offsets
    const long *row_off;
    const int *row_cnt;
    int sched_per_grid;
    const int *masks;
    const double *ckpt;
    const long *ckpt_off;
    int ckpt_every;
    double *lam;          // dJ/dphi_final in the phi_out layout (overwritten)
    double *grad;         // ninst x NPAR, accumulated (caller zeroes)
    const int *order;
    int nwork;
    int *counter;
    double *scratch;      // per CTA: (2 * ckpt_every + 3) * Lmax^2 doubles
    int lam_smem;         // the item's adjoint held in shared memory (odd pitch)
    int Lmax;
    // trajectory mode (null: segments recomputed by each work item's CTA):
    // for work item w, traj + traj_off[w] holds phi_0..phi_n then
    // chi_0..chi_{n-1}, (2n + 1) L^2 doubles, filled by k_adjoint2d_traj
    double *traj;
    const long *traj_off;
};

// Per-interval factors of the contraction for one axis and step:
// P_i = V_i/(2 dx_i), Q_i = V_{i+1}/(2 dx_i) (with 1/nu), and the
// derivatives of the selection term with respect to gamma (FG) and h (FH).
struct ADCVecs {
    double *P, *Q, *FG, *FH;
};

struct ADVecs {
    AxisVecs f[2]; // forward coefficient vectors
    AxisVecs t[2]; // transposed (sub/super swapped)
    ADCVecs c[2];  // contraction factors
};

// Doubles of shared memory the carve takes (grid constants, the forward,
// transposed and contraction vectors of both axes).
constexpr int AD_VEC_DOUBLES = 6 + 2 * 10 + 2 * 4;

struct ADShared {
    AxisScalars ax[2];
    double inj, dinj_dt, dinj_th;
    double D[NQ * NPAR];
    int item;
};

__device__ __forceinline__ void ad_axis_scalars(AxisScalars &s, int a, const double *row,
                                                const GridVecs &g, int L)
{
    double dt = row[0];
    s.dt = dt;
    s.nu = row[row_nu(2, a)];
    s.inv_nu = 1.0 / s.nu;
    s.gamma = row[row_gamma(2, a)];
    s.h = row[row_h(2, a)];
    double m = row[row_mig(2, a, 1 - a)];
    s.msum = m;
    s.mig[a] = 0;
    s.mig[1 - a] = m;
    s.B1s = 0.5 * (dt * g.dfac[0]);
    s.B1e = -0.5 * (dt * g.dfac[L - 1]);
    corner_bc(2, a, s.mig, s.nu, s.gamma, s.h, g.x[0], g.x[L - 1], g.dx[0], g.dx[L - 2], dt,
              s.bcs, s.bce);
}

// Per-step setup shared by the recomputation and the backward step: axis
// scalars, injection value and (with transposed) the derivative row.
__device__ void ad_step_setup(ADShared &S, ADVecs &V, const GridVecs &g, int L, const double *row,
                              const double *drow, bool transposed)
{
    const int tid = threadIdx.x;
    if (tid < 2)
        ad_axis_scalars(S.ax[tid], tid, row, g, L);
    else if (tid == 2) {
        S.inj = inject_value(2, row[0], row[1], g.x[0], g.x[1], g.x[2]);
        S.dinj_dt = inject_value(2, 1.0, row[1], g.x[0], g.x[1], g.x[2]);
        S.dinj_th = inject_value(2, row[0], 1.0, g.x[0], g.x[1], g.x[2]);
    }
    if (transposed)
        for (int j = tid; j < NQ * NPAR; j += blockDim.x)
            S.D[j] = drow[j];
    __syncthreads();
    for (int t = tid; t < 2 * L; t += blockDim.x) {
        int a = t >= L, i = t - a * L;
        build_axis_entry(i, L, g, S.ax[a], 1.0, false, V.f[a]);
    }
    __syncthreads();
    if (transposed) {
        for (int t = tid; t < 2 * L; t += blockDim.x) {
            int a = t >= L, i = t - a * L;
            if (i < L - 1) {
                const double inu = S.ax[a].inv_nu, hh = S.ax[a].h, gam = S.ax[a].gamma;
                const double xi = g.xInt[i];
                const double xx1 = xi * (1. - xi);
                V.c[a].P[i] = inu * g.xv[i] * g.ih[i];
                V.c[a].Q[i] = inu * g.xv[i + 1] * g.ih[i];
                V.c[a].FG[i] = 2 * (hh + (1. - 2 * hh) * xi) * xx1;
                V.c[a].FH[i] = gam * 2 * (1. - 2 * xi) * xx1;
            }
            V.t[a].A1[i] = (i > 0) ? V.f[a].C1[i - 1] : 0.0;
            V.t[a].A0[i] = (i > 0) ? V.f[a].C0[i - 1] : 0.0;
            V.t[a].C1[i] = (i < L - 1) ? V.f[a].A1[i + 1] : 0.0;
            V.t[a].C0[i] = (i < L - 1) ? V.f[a].A0[i + 1] : 0.0;
            V.t[a].B0[i] = V.f[a].B0[i];
        }
        __syncthreads();
    }
}

// Solve all lines of axis a of the L x L row-major array u (in place), with
// the forward or transposed vectors.
__device__ void ad_sweep(double *u, double *gam, int L, int a, const AxisVecs &v,
                         const AxisScalars &s, const GridVecs &g, int j0, int j1, int pu = 0)
{
    // u has row pitch pu (L when 0): global arrays are row-major, the
    // shared-memory adjoint uses an odd pitch (conflict-free both ways)
    const int P = pu ? pu : L;
    const int sp = (a == 0) ? P : 1, sl = (a == 0) ? 1 : P;
    for (int line = threadIdx.x; line < L; line += blockDim.x) {
        double W = s.mig[1 - a] * g.x[line];
        double bs = (line == j0) ? s.bcs : 0.0;
        double be = (line == j1) ? s.bce : 0.0;
        solve_line(u + (size_t)line * sl, sp, gam + line, L, L, W, bs, be, v, s);
    }
}

// Sensitivities of -mu^T (dA'/dq) phi for the lines of axis a handled by this
// thread, added into G[Q_DT], G[nu], G[m], G[gamma], G[h] of that axis.
__device__ void ad_contract(const double *mu, const double *phi, const double *rhs,
                            const double *inj_pts, double inj, int L, int a,
                            const AxisScalars &s, const GridVecs &g, const ADCVecs &cv, int j0,
                            int j1, double *G, int pm = 0)
{
    // mu has row pitch pm (L when 0); phi and rhs are row-major
    const int sp = (a == 0) ? L : 1, sl = (a == 0) ? 1 : L;
    const int PM = pm ? pm : L;
    const int msp = (a == 0) ? PM : 1, msl = (a == 0) ? 1 : PM;
    const int qn = a ? Q_NU1 : Q_NU0, qm = a ? Q_M10 : Q_M01, qg = a ? Q_G1 : Q_G0,
              qh = a ? Q_H1 : Q_H0;
    const double dt = s.dt, inu = s.inv_nu, gam = s.gamma, hh = s.h;
    for (int line = threadIdx.x; line < L; line += blockDim.x) {
        const double *m = mu + (size_t)line * msl, *p = phi + (size_t)line * sl,
                     *r = rhs + (size_t)line * sl;
        const double o = g.x[line];
        double smr = 0, smp = 0, snu = 0, sm = 0, sg = 0, sh = 0;
        double mi = m[0], pi = p[0];
        for (int i = 0; i < L; i++) {
            double ri = r[i * sp];
            if (inj_pts) {
                // psi = phi + injection at (1,0) / (0,1), which lie on lines 0 / 1
                int row = (a == 0) ? i : line, col = (a == 0) ? line : i;
                if ((row == 1 && col == 0) && inj_pts[0] != 0.0)
                    ri += inj;
                if ((row == 0 && col == 1) && inj_pts[1] != 0.0)
                    ri += inj;
            }
            smr = fma(mi, ri, smr);
            smp = fma(mi, pi, smp);
            if (i < L - 1) {
                double mn = m[(i + 1) * msp], pn = p[(i + 1) * sp];
                double Di = g.dfac[i] * mi - g.dfac[i + 1] * mn;
                double hp = 0.5 * (pi + pn);
                snu = fma(Di, (cv.Q[i] * pn - cv.P[i] * pi) * inu, snu);
                sm = fma(Di * (o - g.xInt[i]), hp, sm);
                sg = fma(Di * cv.FG[i], hp, sg);
                sh = fma(Di * cv.FH[i], hp, sh);
                mi = mn;
                pi = pn;
            }
        }
        double bnu = 0, bm = 0, bg = 0, bh = 0;
        if (line == j0 && s.bcs != 0.0) {
            double x0 = g.x[0], f = dt * 2. / g.dx[0], w = m[0] * p[0];
            bnu += w * f * (-0.5 * inu * inu);
            bm += w * f * x0;
            bg -= w * f * (2 * (hh + (1. - 2 * hh) * x0) * x0 * (1. - x0));
            bh -= w * f * (gam * 2 * (1. - 2 * x0) * x0 * (1. - x0));
        }
        if (line == j1 && s.bce != 0.0) {
            double xl = g.x[L - 1], f = dt * 2. / g.dx[L - 2];
            double w = m[(L - 1) * msp] * p[(L - 1) * sp];
            bnu += w * f * (-0.5 * inu * inu);
            bm += w * f * (1. - xl);
            bg += w * f * (2 * (hh + (1. - 2 * hh) * xl) * xl * (1. - xl));
            bh += w * f * (gam * 2 * (1. - 2 * xl) * xl * (1. - xl));
        }
        G[Q_DT] -= (smr - smp) / dt;
        G[qn] -= dt * snu + bnu;
        G[qm] -= dt * sm + bm;
        G[qg] -= dt * sg + bg;
        G[qh] -= dt * sh + bh;
    }
}

__device__ __forceinline__ void ad_carve(double *smem, int L, GridVecs &g, ADVecs &V)
{
    double *p = smem;
    g.x = p; p += L;
    g.xv = p; p += L;
    g.dfac = p; p += L;
    g.xInt = p; p += L;
    g.ih = p; p += L;
    g.dx = p; p += L;
    for (int a = 0; a < 2; a++) {
        V.f[a].A1 = p; p += L;
        V.f[a].A0 = p; p += L;
        V.f[a].C1 = p; p += L;
        V.f[a].C0 = p; p += L;
        V.f[a].B0 = p; p += L;
        V.t[a].A1 = p; p += L;
        V.t[a].A0 = p; p += L;
        V.t[a].C1 = p; p += L;
        V.t[a].C0 = p; p += L;
        V.t[a].B0 = p; p += L;
    }
    for (int a = 0; a < 2; a++) {
        V.c[a].P = p; p += L;
        V.c[a].Q = p; p += L;
        V.c[a].FG = p; p += L;
        V.c[a].FH = p; p += L;
    }
}

template <bool TRAJ>
__global__ void __launch_bounds__(AD_THREADS) k_adjoint2d(ADArgs A)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ ADShared S;
    __shared__ double red[AD_THREADS / 32][NPAR];
    const int tid = threadIdx.x;
    GridVecs g;
    ADVecs V;
    ad_carve(smem, A.Lmax, g, V);
    // the adjoint of the item in shared memory, after the vectors (26 Lmax)
    const int lpitch = (A.Lmax % 2) ? A.Lmax : A.Lmax + 1;
    double *lam_s = smem + (size_t)AD_VEC_DOUBLES * A.Lmax;
    const size_t L2max = (size_t)A.Lmax * A.Lmax;
    // per CTA: the segment's densities (C + 1 slots), the x-sweep outputs
    // chi of its steps (C slots), one spare array and the Thomas scratch;
    // in trajectory mode only the Thomas scratch (L^2 doubles)
    double *seg = nullptr, *chis = nullptr, *W1 = nullptr, *gam;
    if (TRAJ) {
        gam = A.scratch + (size_t)blockIdx.x * L2max;
    } else {
        seg = A.scratch + (size_t)blockIdx.x * (2 * A.ckpt_every + 3) * L2max;
        chis = seg + (size_t)(A.ckpt_every + 1) * L2max;
        W1 = chis + (size_t)A.ckpt_every * L2max;
        gam = W1 + L2max;
    }

    for (;;) {
        if (tid == 0)
            S.item = atomicAdd(A.counter, 1);
        __syncthreads();
        const int w = S.item;
        if (w >= A.nwork)
            break;
        const int wid = A.order[w];
        const int inst = wid / A.ngrids;
        const int gi = wid - inst * A.ngrids;
        const int L = A.L[gi];
        const size_t LL = (size_t)L * L;
        const double *xx = A.xx_all + A.xx_off[gi];
        double *lam_g = A.lam + A.out_off[gi] + (size_t)inst * LL;
        // work on the adjoint in shared memory when it fits (lp = its pitch),
        // else in place in global memory (lp = 0: row-major)
        double *lam = A.lam_smem ? lam_s : lam_g;
        const int lp = A.lam_smem ? lpitch : 0;
        const int LP = lp ? lp : L;
        if (A.lam_smem) {
            for (size_t idx = threadIdx.x; idx < LL; idx += blockDim.x) {
                const int r = (int)(idx / L), c = (int)(idx - (size_t)r * L);
                lam_s[r * lpitch + c] = lam_g[idx];
            }
            __syncthreads();
        }
        const int sidx = A.sched_per_grid ? wid : inst;
        const double *rows = A.table + A.row_off[sidx] * 11;
        const double *drows = A.drows + A.row_off[sidx] * NQ * NPAR;
        const int n = A.row_cnt[sidx];
        const double *ck = A.ckpt + A.ckpt_off[wid];
        const int frozen = A.masks ? (A.masks[inst] & 0xff) : 0;
        const int nomut = A.masks ? (A.masks[inst] >> 8 & 0xff) : 0;
        const bool injx = !(frozen & 1) && !(nomut & 1), injy = !(frozen & 2) && !(nomut & 2);
        const int C = A.ckpt_every;

        for (int i = tid; i < L; i += blockDim.x) {
            double x = xx[i];
            g.x[i] = x;
            g.xv[i] = x * (1. - x);
            if (i < L - 1) {
                double d = xx[i + 1] - x;
                g.dx[i] = d;
                g.ih[i] = 1.0 / (2 * d);
                g.xInt[i] = 0.5 * (xx[i + 1] + x);
            }
        }
        __syncthreads();
        for (int i = tid; i < L; i += blockDim.x) {
            if (i == 0)
                g.dfac[i] = 2. / g.dx[0];
            else if (i == L - 1)
                g.dfac[i] = 2. / g.dx[L - 2];
            else
                g.dfac[i] = 2. / (g.dx[i] + g.dx[i - 1]);
        }
        __syncthreads();
        const int j0 = (g.x[0] == 0.0) ? 0 : -1;
        const int j1 = (g.x[L - 1] == 1.0) ? L - 1 : -1;
        double acc[NPAR];
#pragma unroll
        for (int p = 0; p < NPAR; p++)
            acc[p] = 0;
        const double inj_on[2] = {injx ? 1.0 : 0.0, injy ? 1.0 : 0.0};

        // trajectory mode: the whole walk is one segment whose densities and
        // chi were recomputed beforehand (k_adjoint2d_traj)
        constexpr bool traj = TRAJ;
        double *tphi = traj ? A.traj + A.traj_off[wid] : nullptr;
        double *tchi = traj ? tphi + (size_t)(n + 1) * LL : nullptr;
        const int nseg = traj ? (n > 0 ? 1 : 0) : (n + C - 1) / C;
        for (int sgi = nseg - 1; sgi >= 0; sgi--) {
            const int k0 = traj ? 0 : sgi * C, k1 = traj ? n : min(k0 + C, n);
            double *sphi = traj ? tphi : seg, *schi = traj ? tchi : chis;
            if (!traj) {
                for (size_t idx = tid; idx < LL; idx += blockDim.x)
                    seg[idx] = ck[(size_t)sgi * LL + idx];
            }
            __syncthreads();
            // recompute phi_{k0+1} .. phi_{k1} into seg slots 1 .. k1-k0
            for (int k = k0; k < (traj ? k0 : k1 - 1); k++) {
                ad_step_setup(S, V, g, L, rows + (size_t)k * 11, nullptr, false);
                double *src = seg + (size_t)(k - k0) * LL, *dst = src + LL;
                for (size_t idx = tid; idx < LL; idx += blockDim.x)
                    dst[idx] = src[idx];
                __syncthreads();
                if (tid == 0) {
                    if (injx)
                        dst[1 * L + 0] += S.inj;
                    if (injy)
                        dst[0 * L + 1] += S.inj;
                }
                __syncthreads();
                if (!(frozen & 1)) {
                    ad_sweep(dst, gam, L, 0, V.f[0], S.ax[0], g, j0, j1);
                    __syncthreads();
                }
                // chi_k = X^{-1}(phi_k + inj), kept for the backward step
                double *chik = chis + (size_t)(k - k0) * LL;
                for (size_t idx = tid; idx < LL; idx += blockDim.x)
                    chik[idx] = dst[idx];
                __syncthreads();
                if (!(frozen & 2)) {
                    ad_sweep(dst, gam, L, 1, V.f[1], S.ax[1], g, j0, j1);
                    __syncthreads();
                }
            }
            // backward through the segment
            for (int k = k1 - 1; k >= k0; k--) {
                ad_step_setup(S, V, g, L, rows + (size_t)k * 11,
                              drows + (size_t)k * NQ * NPAR, true);
                const double *phik = sphi + (size_t)(k - k0) * LL;
                // chi_k = X^{-1}(phi_k + inj): kept by the recomputation,
                // except for the segment's last step, formed here in W1
                const double *chi = schi + (size_t)(k - k0) * LL;
                if (k == k1 - 1 && !traj) {
                    for (size_t idx = tid; idx < LL; idx += blockDim.x)
                        W1[idx] = phik[idx];
                    __syncthreads();
                    if (tid == 0) {
                        if (injx)
                            W1[1 * L + 0] += S.inj;
                        if (injy)
                            W1[0 * L + 1] += S.inj;
                    }
                    __syncthreads();
                    if (!(frozen & 1)) {
                        ad_sweep(W1, gam, L, 0, V.f[0], S.ax[0], g, j0, j1);
                        __syncthreads();
                    }
                    chi = W1;
                }
                double G[NQ];
#pragma unroll
                for (int q = 0; q < NQ; q++)
                    G[q] = 0;
                // phi_{k+1} = Y^{-1} chi: slot k-k0+1 holds it unless k is the
                // segment's last step; then recompute it in the spare slot.
                double *phin = sphi + (size_t)(k - k0 + 1) * LL;
                if (k == k1 - 1 && !traj) {
                    for (size_t idx = tid; idx < LL; idx += blockDim.x)
                        phin[idx] = W1[idx];
                    __syncthreads();
                    if (!(frozen & 2)) {
                        ad_sweep(phin, gam, L, 1, V.f[1], S.ax[1], g, j0, j1);
                        __syncthreads();
                    }
                }
                // y: mu = Y^{-T} lambda, contract with phi_{k+1}, rhs chi
                if (!(frozen & 2)) {
                    ad_sweep(lam, gam, L, 1, V.t[1], S.ax[1], g, j0, j1, lp);
                    __syncthreads();
                    ad_contract(lam, phin, chi, nullptr, 0.0, L, 1, S.ax[1], g, V.c[1], j0, j1,
                                G, lp);
                    __syncthreads();
                }
                // x: nu = X^{-T} mu, contract with chi, rhs psi
                if (!(frozen & 1)) {
                    ad_sweep(lam, gam, L, 0, V.t[0], S.ax[0], g, j0, j1, lp);
                    __syncthreads();
                    ad_contract(lam, chi, phik, inj_on, S.inj, L, 0, S.ax[0], g, V.c[0], j0, j1,
                                G, lp);
                }
                // injection: d psi(1,0), psi(0,1) / d(dt, theta0)
                if (tid == 0) {
                    double lin = (injx ? lam[1 * LP + 0] : 0.0) + (injy ? lam[0 * LP + 1] : 0.0);
                    G[Q_DT] += lin * S.dinj_dt;
                    G[Q_TH] += lin * S.dinj_th;
                }
#pragma unroll
                for (int p = 0; p < NPAR; p++) {
                    double sacc = acc[p];
#pragma unroll
                    for (int q = 0; q < NQ; q++)
                        sacc = fma(G[q], S.D[q * NPAR + p], sacc);
                    acc[p] = sacc;
                }
                __syncthreads();
            }
        }
        if (A.lam_smem) {
            // dJ/dphi_initial back to the caller's array
            for (size_t idx = threadIdx.x; idx < LL; idx += blockDim.x) {
                const int r = (int)(idx / L), c = (int)(idx - (size_t)r * L);
                lam_g[idx] = lam_s[r * lpitch + c];
            }
        }
        // block reduction of acc into this work item's row of grad
#pragma unroll
        for (int p = 0; p < NPAR; p++) {
            double v = acc[p];
            for (int off = 16; off > 0; off >>= 1)
                v += __shfl_down_sync(0xffffffffu, v, off);
            if ((tid & 31) == 0)
                red[tid >> 5][p] = v;
        }
        __syncthreads();
        if (tid < NPAR) {
            double v = 0;
            for (int wv = 0; wv < (int)(blockDim.x >> 5); wv++)
                v += red[wv][tid];
            A.grad[((size_t)inst * A.ngrids + gi) * NPAR + tid] = v;
        }
        __syncthreads();
    }
}


// Trajectory recomputation for the adjoint: one CTA per (work item,
// checkpoint segment), all segments at once in a grid-stride loop, instead
// of each work item's CTA recomputing its segments one after another before
// walking them back.  Segment s of item w starts from its checkpoint
// (phi_{sC}) and writes phi_{k+1} and chi_k = X^{-1}(phi_k + inj) for its
// steps into the item's trajectory; phi at a segment boundary is written by
// the next segment's CTA (its checkpoint), so no slot has two writers.  The
// steps use ad_step_setup and ad_sweep as k_adjoint2d's own recomputation
// does, so the trajectory is bitwise what it would recompute.
__global__ void __launch_bounds__(AD_THREADS) k_adjoint2d_traj(ADArgs A, const long *seg_off)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ ADShared S;
    const int tid = threadIdx.x;
    GridVecs g;
    ADVecs V;
    ad_carve(smem, A.Lmax, g, V);
    const size_t L2max = (size_t)A.Lmax * A.Lmax;
    double *gam = A.scratch + (size_t)blockIdx.x * L2max;
    const long total = seg_off[A.nwork];
    const int C = A.ckpt_every;
    for (long gs = blockIdx.x; gs < total; gs += gridDim.x) {
        int lo = 0, hi = A.nwork; // seg_off[lo] <= gs < seg_off[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (seg_off[mid] <= gs)
                lo = mid;
            else
                hi = mid;
        }
        const int wid = lo;
        const int sgi = (int)(gs - seg_off[wid]);
        const int inst = wid / A.ngrids;
        const int gi = wid - inst * A.ngrids;
        const int L = A.L[gi];
        const size_t LL = (size_t)L * L;
        const double *xx = A.xx_all + A.xx_off[gi];
        const int sidx = A.sched_per_grid ? wid : inst;
        const double *rows = A.table + A.row_off[sidx] * 11;
        const int n = A.row_cnt[sidx];
        const double *ck = A.ckpt + A.ckpt_off[wid];
        const int frozen = A.masks ? (A.masks[inst] & 0xff) : 0;
        const int nomut = A.masks ? (A.masks[inst] >> 8 & 0xff) : 0;
        const bool injx = !(frozen & 1) && !(nomut & 1), injy = !(frozen & 2) && !(nomut & 2);
        double *tphi = A.traj + A.traj_off[wid];
        double *tchi = tphi + (size_t)(n + 1) * LL;
        for (int i = tid; i < L; i += blockDim.x) {
            double x = xx[i];
            g.x[i] = x;
            g.xv[i] = x * (1. - x);
            if (i < L - 1) {
                double d = xx[i + 1] - x;
                g.dx[i] = d;
                g.ih[i] = 1.0 / (2 * d);
                g.xInt[i] = 0.5 * (xx[i + 1] + x);
            }
        }
        __syncthreads();
        for (int i = tid; i < L; i += blockDim.x) {
            if (i == 0)
                g.dfac[i] = 2. / g.dx[0];
            else if (i == L - 1)
                g.dfac[i] = 2. / g.dx[L - 2];
            else
                g.dfac[i] = 2. / (g.dx[i] + g.dx[i - 1]);
        }
        __syncthreads();
        const int j0 = (g.x[0] == 0.0) ? 0 : -1;
        const int j1 = (g.x[L - 1] == 1.0) ? L - 1 : -1;
        const int k0 = sgi * C, k1 = min(k0 + C, n);
        for (size_t idx = tid; idx < LL; idx += blockDim.x)
            tphi[(size_t)k0 * LL + idx] = ck[(size_t)sgi * LL + idx];
        __syncthreads();
        for (int k = k0; k < k1; k++) {
            ad_step_setup(S, V, g, L, rows + (size_t)k * 11, nullptr, false);
            const double *src = tphi + (size_t)k * LL;
            double *chik = tchi + (size_t)k * LL;
            for (size_t idx = tid; idx < LL; idx += blockDim.x)
                chik[idx] = src[idx];
            __syncthreads();
            if (tid == 0) {
                if (injx)
                    chik[1 * L + 0] += S.inj;
                if (injy)
                    chik[0 * L + 1] += S.inj;
            }
            __syncthreads();
            if (!(frozen & 1)) {
                ad_sweep(chik, gam, L, 0, V.f[0], S.ax[0], g, j0, j1);
                __syncthreads();
            }
            // phi_{k+1}, except at a segment boundary (the next CTA's checkpoint)
            if (k < k1 - 1 || k1 == n) {
                double *dst = tphi + (size_t)(k + 1) * LL;
                for (size_t idx = tid; idx < LL; idx += blockDim.x)
                    dst[idx] = chik[idx];
                __syncthreads();
                if (!(frozen & 2)) {
                    ad_sweep(dst, gam, L, 1, V.f[1], S.ax[1], g, j0, j1);
                    __syncthreads();
                }
            }
        }
        __syncthreads();
    }
}

} // namespace dgb

// ------------------------------------------------------------------ C ABI

extern "C" int dgb_sched2d_deriv(const dgb_inst2d *insts, const dgb_seed2d *seeds, int ninst,
                                 int ngrids, const double *dx0s, const dgb_settings *settings,
                                 const int *row_cnt, const long *row_off, double *drows,
                                 void *stream)
{
    if (!insts || !seeds || ninst < 1 || ngrids < 1 || !dx0s || !settings || !row_cnt ||
        !row_off || !drows)
        return DGB_ERR_ARG;
    int per_grid = settings->use_old_timestep ? 1 : 0;
    int nsched = per_grid ? ninst * ngrids : ninst;
    const long nthreads = (long)nsched * dgb::SD_LANES;
    dgb::k_sched2d_dual<<<(unsigned)((nthreads + 63) / 64), 64, 0, (cudaStream_t)stream>>>(
        insts, seeds, nsched, ngrids, per_grid, dx0s, *settings, row_cnt, row_off, drows);
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

extern "C" size_t dgb_adjoint2d_scratch_bytes(int Lmax, int ckpt_every, int nblocks)
{
    return (size_t)nblocks * (2 * ckpt_every + 3) * Lmax * Lmax * sizeof(double);
}

namespace dgb {

// The backward walk of one work item on a thread-block cluster (trajectory
// mode: phi_k and chi_k read from the stored trajectory): the transposed
// solves of k_adjoint2d partitioned as k_integrate2d_cluster partitions the
// forward (c2_sweep_x / c2_sweep_y with the transposed vectors), CTA r
// holding rows R0 .. R0+m-1 of the adjoint.  The contraction of each sweep
// is split over the threads that hold the points: its sums run over points
// and over the intervals (i, i+1) whose lower point a thread holds, so they
// add up; an interval across two CTAs' row blocks reads the next CTA's first
// adjoint row (exported after the x solve).  Per-CTA partial gradients are
// summed through distributed shared memory.  Cluster b walks order[b].
constexpr int AC_THREADS = C2_THREADS;

__host__ __device__ inline size_t adc_smem_doubles(int L)
{
    return (size_t)AD_VEC_DOUBLES * L + (size_t)C2_ROWS * c2_pitch(L) +
           2 * (size_t)C2_ROWS * L + (size_t)C2_XROW * L + 3 * (size_t)L +
           (size_t)C2_YSLOT * C2_YSEG * C2_ROWS + NPAR;
}

__global__ void __launch_bounds__(AC_THREADS) k_adjoint2d_cluster(ADArgs A)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ ADShared S;
    __shared__ double red[AC_THREADS / 32][NPAR];
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int NS = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int tid = threadIdx.x;
    const int w = blockIdx.x / NS;
    if (w >= A.nwork)
        return; // the whole cluster
    const int wid = A.order[w];
    const int inst = wid / A.ngrids;
    const int gi = wid - inst * A.ngrids;
    const int L = A.L[gi];
    const size_t LL = (size_t)L * L;
    const int pitch = c2_pitch(L);
    int R0, m;
    c2_rows(L, NS, rank, &R0, &m);
    GridVecs g;
    ADVecs V;
    ad_carve(smem, L, g, V);
    double *blk = smem + (size_t)AD_VEC_DOUBLES * L; // this CTA's rows of lambda
    double *al = blk + (size_t)C2_ROWS * pitch;
    double *ga = al + (size_t)C2_ROWS * L;
    double *xr = ga + (size_t)C2_ROWS * L;
    double *zin = xr + (size_t)C2_XROW * L;
    double *hx = zin + 2 * (size_t)L;                // exported first row of lambda
    double *yr = hx + L;
    double *part = yr + (size_t)C2_YSLOT * C2_YSEG * C2_ROWS; // this CTA's gradient

    const double *xx = A.xx_all + A.xx_off[gi];
    double *lam_g = A.lam + A.out_off[gi] + (size_t)inst * LL;
    const int sidx = A.sched_per_grid ? wid : inst;
    const double *rows = A.table + A.row_off[sidx] * 11;
    const double *drows = A.drows + A.row_off[sidx] * NQ * NPAR;
    const int n = A.row_cnt[sidx];
    const int frozen = A.masks ? (A.masks[inst] & 0xff) : 0;
    const int nomut = A.masks ? (A.masks[inst] >> 8 & 0xff) : 0;
    const bool injx = !(frozen & 1) && !(nomut & 1), injy = !(frozen & 2) && !(nomut & 2);
    const double *tphi = A.traj + A.traj_off[wid];
    const double *tchi = tphi + (size_t)(n + 1) * LL;

    for (int i = tid; i < L; i += AC_THREADS) {
        const double x = xx[i];
        g.x[i] = x;
        g.xv[i] = x * (1. - x);
        if (i < L - 1) {
            const double d = xx[i + 1] - x;
            g.dx[i] = d;
            g.ih[i] = 1.0 / (2 * d);
            g.xInt[i] = 0.5 * (xx[i + 1] + x);
        }
    }
    for (int idx = tid; idx < m * L; idx += AC_THREADS) {
        const int p = idx / L, c = idx - p * L;
        blk[p * pitch + c] = lam_g[(size_t)(R0 + p) * L + c];
    }
    __syncthreads();
    for (int i = tid; i < L; i += AC_THREADS)
        g.dfac[i] = (i == 0)       ? 2. / g.dx[0]
                    : (i == L - 1) ? 2. / g.dx[L - 2]
                                   : 2. / (g.dx[i] + g.dx[i - 1]);
    __syncthreads();
    const int j0 = (g.x[0] == 0.0) ? 0 : -1;
    const int j1 = (g.x[L - 1] == 1.0) ? L - 1 : -1;
    double acc[NPAR];
#pragma unroll
    for (int p = 0; p < NPAR; p++)
        acc[p] = 0;

    for (int k = n - 1; k >= 0; k--) {
        ad_step_setup(S, V, g, L, rows + (size_t)k * 11, drows + (size_t)k * NQ * NPAR, true);
        const double *phin = tphi + (size_t)(k + 1) * LL; // Y^{-1} chi_k
        const double *chi = tchi + (size_t)k * LL;        // X^{-1} psi_k
        const double *phik = tphi + (size_t)k * LL;       // psi_k - injection
        double G[NQ];
#pragma unroll
        for (int q = 0; q < NQ; q++)
            G[q] = 0;
        // ---- y: mu = Y^{-T} lambda on the CTA's rows, contracted with
        // phi_{k+1} (the sweep's output) and chi_k (its input)
        if (!(frozen & 2)) {
            c2_sweep_y(blk, pitch, L, R0, m, al, ga, yr, V.t[1], S.ax[1], g, j0, j1);
            const int p = tid % C2_ROWS, q = tid / C2_ROWS;
            if (p < m) {
                const int mlen = L / C2_YSEG, extra = L % C2_YSEG;
                const int s0 = q * mlen + min(q, extra);
                const int e0 = s0 + mlen + (q < extra ? 1 : 0); // points [s0, e0)
                const int line = R0 + p;
                const AxisScalars &s = S.ax[1];
                const ADCVecs &cv = V.c[1];
                const double *mr = blk + (size_t)p * pitch;
                const double *pr = phin + (size_t)line * L, *rr = chi + (size_t)line * L;
                const double o = g.x[line], inu = s.inv_nu, dt = s.dt;
                double smr = 0, smp = 0, snu = 0, sm = 0, sg = 0, sh = 0;
                double mi = mr[s0], pi = pr[s0];
                for (int i = s0; i < e0; i++) {
                    smr = fma(mi, rr[i], smr);
                    smp = fma(mi, pi, smp);
                    if (i < L - 1) {
                        const double mn = mr[i + 1], pn = pr[i + 1];
                        const double Di = g.dfac[i] * mi - g.dfac[i + 1] * mn;
                        const double hp = 0.5 * (pi + pn);
                        snu = fma(Di, (cv.Q[i] * pn - cv.P[i] * pi) * inu, snu);
                        sm = fma(Di * (o - g.xInt[i]), hp, sm);
                        sg = fma(Di * cv.FG[i], hp, sg);
                        sh = fma(Di * cv.FH[i], hp, sh);
                        mi = mn;
                        pi = pn;
                    }
                }
                double bnu = 0, bm = 0, bg = 0, bh = 0;
                const double hh = s.h, gam = s.gamma;
                if (s0 == 0 && line == j0 && s.bcs != 0.0) {
                    const double x0 = g.x[0], f = dt * 2. / g.dx[0], w0 = mr[0] * pr[0];
                    bnu += w0 * f * (-0.5 * inu * inu);
                    bm += w0 * f * x0;
                    bg -= w0 * f * (2 * (hh + (1. - 2 * hh) * x0) * x0 * (1. - x0));
                    bh -= w0 * f * (gam * 2 * (1. - 2 * x0) * x0 * (1. - x0));
                }
                if (e0 == L && line == j1 && s.bce != 0.0) {
                    const double xl = g.x[L - 1], f = dt * 2. / g.dx[L - 2];
                    const double w1 = mr[L - 1] * pr[L - 1];
                    bnu += w1 * f * (-0.5 * inu * inu);
                    bm += w1 * f * (1. - xl);
                    bg += w1 * f * (2 * (hh + (1. - 2 * hh) * xl) * xl * (1. - xl));
                    bh += w1 * f * (gam * 2 * (1. - 2 * xl) * xl * (1. - xl));
                }
                G[Q_DT] -= (smr - smp) / dt;
                G[Q_NU1] -= dt * snu + bnu;
                G[Q_M10] -= dt * sm + bm;
                G[Q_G1] -= dt * sg + bg;
                G[Q_H1] -= dt * sh + bh;
            }
            __syncthreads();
        }
        // ---- x: nu = X^{-T} mu across the cluster, contracted with chi_k
        // (the sweep's output) and psi_k (its input)
        if (!(frozen & 1)) {
            c2_sweep_x(cluster, NS, rank, blk, pitch, L, R0, m, al, ga, xr, zin, V.t[0],
                       S.ax[0], g, j0, j1);
            for (int j = tid; j < L; j += AC_THREADS)
                hx[j] = blk[j];
            cluster.sync();
            const int j = tid;
            if (j < L) {
                // nu at row R0 + m, the next CTA's first row
                const double mnext =
                    (rank + 1 < NS) ? cluster.map_shared_rank(hx, rank + 1)[j] : 0.0;
                const AxisScalars &s = S.ax[0];
                const ADCVecs &cv = V.c[0];
                const double o = g.x[j], inu = s.inv_nu, dt = s.dt;
                double smr = 0, smp = 0, snu = 0, sm = 0, sg = 0, sh = 0;
                double mi = blk[j], pi = chi[(size_t)R0 * L + j];
                for (int p = 0; p < m; p++) {
                    const int i = R0 + p;
                    double ri = phik[(size_t)i * L + j];
                    if (i == 1 && j == 0 && injx)
                        ri += S.inj;
                    if (i == 0 && j == 1 && injy)
                        ri += S.inj;
                    smr = fma(mi, ri, smr);
                    smp = fma(mi, pi, smp);
                    if (i < L - 1) {
                        const double mn = (p + 1 < m) ? blk[(p + 1) * pitch + j] : mnext;
                        const double pn = chi[(size_t)(i + 1) * L + j];
                        const double Di = g.dfac[i] * mi - g.dfac[i + 1] * mn;
                        const double hp = 0.5 * (pi + pn);
                        snu = fma(Di, (cv.Q[i] * pn - cv.P[i] * pi) * inu, snu);
                        sm = fma(Di * (o - g.xInt[i]), hp, sm);
                        sg = fma(Di * cv.FG[i], hp, sg);
                        sh = fma(Di * cv.FH[i], hp, sh);
                        mi = mn;
                        pi = pn;
                    }
                }
                double bnu = 0, bm = 0, bg = 0, bh = 0;
                const double hh = s.h, gam = s.gamma;
                if (R0 == 0 && j == j0 && s.bcs != 0.0) {
                    const double x0 = g.x[0], f = dt * 2. / g.dx[0], w0 = blk[j] * chi[j];
                    bnu += w0 * f * (-0.5 * inu * inu);
                    bm += w0 * f * x0;
                    bg -= w0 * f * (2 * (hh + (1. - 2 * hh) * x0) * x0 * (1. - x0));
                    bh -= w0 * f * (gam * 2 * (1. - 2 * x0) * x0 * (1. - x0));
                }
                if (R0 + m == L && j == j1 && s.bce != 0.0) {
                    const double xl = g.x[L - 1], f = dt * 2. / g.dx[L - 2];
                    const double w1 = blk[(m - 1) * pitch + j] * chi[(size_t)(L - 1) * L + j];
                    bnu += w1 * f * (-0.5 * inu * inu);
                    bm += w1 * f * (1. - xl);
                    bg += w1 * f * (2 * (hh + (1. - 2 * hh) * xl) * xl * (1. - xl));
                    bh += w1 * f * (gam * 2 * (1. - 2 * xl) * xl * (1. - xl));
                }
                G[Q_DT] -= (smr - smp) / dt;
                G[Q_NU0] -= dt * snu + bnu;
                G[Q_M01] -= dt * sm + bm;
                G[Q_G0] -= dt * sg + bg;
                G[Q_H0] -= dt * sh + bh;
            }
        }
        // injection: d psi(1,0), psi(0,1) / d(dt, theta0), rows 0 and 1 of
        // the first CTA
        if (rank == 0 && tid == 0) {
            const double lin = (injx ? blk[1 * pitch + 0] : 0.0) + (injy ? blk[0 * pitch + 1] : 0.0);
            G[Q_DT] += lin * S.dinj_dt;
            G[Q_TH] += lin * S.dinj_th;
        }
#pragma unroll
        for (int p = 0; p < NPAR; p++) {
            double sacc = acc[p];
#pragma unroll
            for (int q = 0; q < NQ; q++)
                sacc = fma(G[q], S.D[q * NPAR + p], sacc);
            acc[p] = sacc;
        }
        __syncthreads();
    }
    for (int idx = tid; idx < m * L; idx += AC_THREADS) {
        const int p = idx / L, c = idx - p * L;
        lam_g[(size_t)(R0 + p) * L + c] = blk[p * pitch + c];
    }
#pragma unroll
    for (int p = 0; p < NPAR; p++) {
        double v = acc[p];
        for (int off = 16; off > 0; off >>= 1)
            v += __shfl_down_sync(0xffffffffu, v, off);
        if ((tid & 31) == 0)
            red[tid >> 5][p] = v;
    }
    __syncthreads();
    if (tid < NPAR) {
        double v = 0;
        for (int wv = 0; wv < AC_THREADS / 32; wv++)
            v += red[wv][tid];
        part[tid] = v;
    }
    cluster.sync();
    if (rank == 0 && tid < NPAR) {
        double v = 0;
        for (int q = 0; q < NS; q++)
            v += cluster.map_shared_rank(part, q)[tid];
        A.grad[((size_t)inst * A.ngrids + gi) * NPAR + tid] = v;
    }
    // no CTA may leave while the first still reads its partial gradient
    cluster.sync();
}

} // namespace dgb

// norder: the work items of `order` to walk (<= 0: all ninst x ngrids);
// max_blocks: most CTAs of the backward walk (<= 0: as many as the workspace
// and the items allow); cluster: in trajectory mode, walk each item on a
// thread-block cluster of that many CTAs (k_adjoint2d_cluster; 0: one CTA
// per item).
static int adjoint2d_run(const int *masks, int ninst, const int *Ls, int ngrids,
                         const double *xx_all, const double *table, const double *drows,
                         const long *row_off, const int *row_cnt, const double *ckpt,
                         const long *ckpt_off, int ckpt_every, double *lam, double *grad,
                         const int *order, int norder, int max_blocks, int cluster,
                         const dgb_settings *settings, double *traj, const long *traj_off,
                         const long *seg_off, void *ws, size_t ws_bytes, void *stream)
{
    using namespace dgb;
    if (!Ls || !xx_all || !table || !drows || !row_off || !row_cnt || !ckpt || !ckpt_off ||
        ckpt_every < 1 || !lam || !grad || !order || !settings || ngrids < 1 ||
        ngrids > AD_MAXG || ninst < 1 || norder > ninst * ngrids)
        return DGB_ERR_ARG;
    if (settings->use_delj_trick)
        return DGB_ERR_UNSUPPORTED;
    if (cluster) {
        // every grid within the partitioned sweeps' range, in trajectory mode
        if (!traj || (cluster != 2 && cluster != 4 && cluster != 8 && cluster != 16))
            return DGB_ERR_ARG;
        for (int gi = 0; gi < ngrids; gi++)
            if (Ls[gi] < 3 * C2_YSEG || Ls[gi] > C2_THREADS || Ls[gi] < 3 * cluster ||
                Ls[gi] > C2_ROWS * cluster)
                return DGB_ERR_UNSUPPORTED;
    }
    ADArgs A = {};
    A.ngrids = ngrids;
    long xo = 0, oo = 0;
    int Lmax = 0;
    for (int gi = 0; gi < ngrids; gi++) {
        if (Ls[gi] < 3)
            return DGB_ERR_ARG;
        A.L[gi] = Ls[gi];
        A.xx_off[gi] = xo;
        A.out_off[gi] = oo;
        xo += Ls[gi];
        oo += (long)ninst * Ls[gi] * Ls[gi];
        Lmax = std::max(Lmax, Ls[gi]);
    }
    A.xx_all = xx_all;
    A.table = table;
    A.drows = drows;
    A.row_off = row_off;
    A.row_cnt = row_cnt;
    A.sched_per_grid = settings->use_old_timestep ? 1 : 0;
    A.masks = masks;
    A.ckpt = ckpt;
    A.ckpt_off = ckpt_off;
    A.ckpt_every = ckpt_every;
    A.lam = lam;
    A.grad = grad;
    A.order = order;
    A.nwork = ninst * ngrids;
    A.Lmax = Lmax;
    if (!ws || ws_bytes < 256)
        return DGB_ERR_WORKSPACE;
    A.counter = (int *)ws;
    A.traj = traj;
    A.traj_off = traj_off;
    // per CTA: the segment buffers, or in trajectory mode the Thomas scratch
    const size_t per_cta = traj ? (size_t)Lmax * Lmax * sizeof(double)
                                : dgb_adjoint2d_scratch_bytes(Lmax, ckpt_every, 1);
    long nblocks = (long)((ws_bytes - 256) / per_cta);
    if (nblocks < 1)
        return DGB_ERR_WORKSPACE;
    // the walk covers the first norder entries of `order`; the trajectory's
    // recomputation (every work id with segments in seg_off) sees them all
    const int nwalk = norder > 0 ? norder : A.nwork;
    nblocks = std::min<long>(nblocks, nwalk);
    if (max_blocks > 0)
        nblocks = std::min<long>(nblocks, max_blocks);
    A.scratch = (double *)((char *)ws + 256);
    size_t smem = (size_t)AD_VEC_DOUBLES * Lmax * sizeof(double);
    {
        // the adjoint in shared memory when vectors + Lmax x odd pitch fit
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        const int lpitch = (Lmax % 2) ? Lmax : Lmax + 1;
        size_t with_lam = smem + (size_t)Lmax * lpitch * sizeof(double);
        if (with_lam + sizeof(ADShared) + 4096 <= (size_t)optin) {
            A.lam_smem = 1;
            smem = with_lam;
        }
    }
    if (traj ? raise_smem_limit(k_adjoint2d<true>) : raise_smem_limit(k_adjoint2d<false>))
        return DGB_ERR_CUDA;
    if (traj) {
        // every checkpoint segment at once, on as many CTAs as the
        // workspace holds Thomas scratch for (at most two per SM)
        const size_t rsmem = (size_t)AD_VEC_DOUBLES * Lmax * sizeof(double);
        if (raise_smem_limit(k_adjoint2d_traj))
            return DGB_ERR_CUDA;
        int dev = 0, nsm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        const long rblocks = std::min<long>((long)((ws_bytes - 256) / per_cta), 2L * nsm);
        k_adjoint2d_traj<<<(unsigned)rblocks, AD_THREADS, rsmem, (cudaStream_t)stream>>>(
            A, seg_off);
        if (cudaGetLastError() != cudaSuccess)
            return DGB_ERR_CUDA;
    }
    if (cudaMemsetAsync(A.counter, 0, sizeof(int), (cudaStream_t)stream) != cudaSuccess)
        return DGB_ERR_CUDA;
    A.nwork = nwalk;
    if (traj && cluster > 0) {
        const size_t csmem =
            std::max(adc_smem_doubles(Lmax) * sizeof(double), (size_t)116 << 10);
        if (raise_smem_limit(k_adjoint2d_cluster))
            return DGB_ERR_CUDA;
        if (cluster > 8 && cudaFuncSetAttribute(k_adjoint2d_cluster,
                                                cudaFuncAttributeNonPortableClusterSizeAllowed,
                                                1) != cudaSuccess) {
            cudaGetLastError();
            return DGB_ERR_UNSUPPORTED;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)(cluster * nwalk), 1, 1);
        cfg.blockDim = dim3(AC_THREADS, 1, 1);
        cfg.dynamicSmemBytes = csmem;
        cfg.stream = (cudaStream_t)stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)cluster;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        if (cudaLaunchKernelEx(&cfg, k_adjoint2d_cluster, A) != cudaSuccess) {
            cudaGetLastError();
            return DGB_ERR_CUDA;
        }
        return DGB_OK;
    }
    if (traj)
        k_adjoint2d<true><<<(unsigned)nblocks, AD_THREADS, smem, (cudaStream_t)stream>>>(A);
    else
        k_adjoint2d<false><<<(unsigned)nblocks, AD_THREADS, smem, (cudaStream_t)stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

extern "C" int dgb_adjoint2d(const int *masks, int ninst, const int *Ls, int ngrids,
                             const double *xx_all, const double *table, const double *drows,
                             const long *row_off, const int *row_cnt, const double *ckpt,
                             const long *ckpt_off, int ckpt_every, double *lam, double *grad,
                             const int *order, const dgb_settings *settings, void *ws,
                             size_t ws_bytes, void *stream)
{
    return adjoint2d_run(masks, ninst, Ls, ngrids, xx_all, table, drows, row_off, row_cnt, ckpt,
                         ckpt_off, ckpt_every, lam, grad, order, 0, 0, 0, settings, nullptr,
                         nullptr, nullptr, ws, ws_bytes, stream);
}

extern "C" size_t dgb_adjoint2d_traj_ws_bytes(int Lmax, int nblocks)
{
    return 256 + (size_t)nblocks * Lmax * Lmax * sizeof(double);
}

extern "C" int dgb_adjoint2d_traj(const int *masks, int ninst, const int *Ls, int ngrids,
                                  const double *xx_all, const double *table,
                                  const double *drows, const long *row_off, const int *row_cnt,
                                  const double *ckpt, const long *ckpt_off, int ckpt_every,
                                  double *traj, const long *traj_off, const long *seg_off,
                                  double *lam, double *grad, const int *order,
                                  const dgb_settings *settings, void *ws, size_t ws_bytes,
                                  void *stream)
{
    if (!traj || !traj_off || !seg_off)
        return DGB_ERR_ARG;
    return adjoint2d_run(masks, ninst, Ls, ngrids, xx_all, table, drows, row_off, row_cnt, ckpt,
                         ckpt_off, ckpt_every, lam, grad, order, 0, 0, 0, settings, traj,
                         traj_off, seg_off, ws, ws_bytes, stream);
}

extern "C" int dgb_adjoint2d_part(const int *masks, int ninst, const int *Ls, int ngrids,
                                  const double *xx_all, const double *table,
                                  const double *drows, const long *row_off, const int *row_cnt,
                                  const double *ckpt, const long *ckpt_off, int ckpt_every,
                                  double *traj, const long *traj_off, const long *seg_off,
                                  double *lam, double *grad, const int *order, int norder,
                                  int max_blocks, int cluster, const dgb_settings *settings,
                                  void *ws, size_t ws_bytes, void *stream)
{
    if (norder < 1 || (traj && (!traj_off || !seg_off)))
        return DGB_ERR_ARG;
    return adjoint2d_run(masks, ninst, Ls, ngrids, xx_all, table, drows, row_off, row_cnt, ckpt,
                         ckpt_off, ckpt_every, lam, grad, order, norder, max_blocks, cluster,
                         settings, traj, traj_off, seg_off, ws, ws_bytes, stream);
}

namespace dgb {
int preload_adjoint2d()
{
    return preload(k_sched2d_dual) + preload(k_adjoint2d<false>) + preload(k_adjoint2d<true>) +
           preload(k_adjoint2d_traj) + preload(k_adjoint2d_cluster);
}
} // namespace dgb
