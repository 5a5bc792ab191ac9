// Shared-memory-resident 2-D integrator and the batched 2-population engine.
//
// One CTA owns one (instance, grid) work item for its whole time loop: phi
// (L x L doubles, odd row pitch so both sweep directions are bank-conflict
// free) is loaded once into shared memory; every step injects mutations,
// rebuilds the per-axis coefficient vectors and runs the x sweep (lines are
// columns) and the y sweep (lines are rows) with one thread per line; phi is
// written back once at the end.  The Thomas gam scratch lives in shared
// memory when it fits next to phi, otherwise in a per-CTA slice of a global
// workspace (L2-resident).
//
// The integrator only reads per-step parameter rows (see dadi_gb300.h).  For
// the drop-in path the host evaluates them from Python callables; for the
// batched engine a separate pass (k_sched2d, one thread per instance, so the
// scalar pow/exp/divide chain of the schedule runs on full warps instead of
// serialising inside every integrating CTA) evaluates the parametric forms
// with the reference's operation order: one fill pass into room reserved
// from host bounds on the rows, or count rows, scan, fill rows.
// The batched integration is a persistent launch whose CTAs pull work items
// longest-first from an atomic counter (one launch over all grids, or one
// per grid size with a CTA shaped for it, two items per CTA where that fills
// the warps better: k_integrate2d_pair), or one CTA per item.
//
// Reference: the time loop of Integration.two_pops (dadi/Integration.py:
// 340-386) with implicit_2Dx / implicit_2Dy (dadi/integration2D.c:19-160).
#include <algorithm>
#include <mutex>
#include <vector>

#include "dgb_common.cuh"
#include "dgb_internal.h"

namespace dgb {

constexpr int K2_THREADS = 128;
constexpr int K2_MAXG = DGB_B2_MAXG;
constexpr int K2_ROW = 11; // DGB_ROW_STRIDE(2)

struct K2Args {
    int ngrids;
    int L[K2_MAXG];
    long xx_off[K2_MAXG];
    long phi0_off[K2_MAXG];
    long out_off[K2_MAXG];
    const double *xx_all;
    const double *phi0_all; // null: phi_out holds the initial density
    double *phi_out;
    const double *table;   // parameter rows
    const long *row_off;   // first row of each schedule (null: one schedule at row 0)
    const int *row_cnt;    // rows of each schedule
    int fixed_cnt;         // rows of the single schedule when row_off is null
    int sched_per_grid;    // schedule index = inst*ngrids+g (1) or inst (0)
    const int *masks;      // per instance: frozen | nomut << 8 (null: use fixed)
    int frozen_mask, nomut_mask;
    const int *order;      // null: work id = position
    int nwork;
    int *counter;          // null: one item per CTA (blockIdx.x)
    int Lmax;
    int gam_smem;          // 1: gam in shared memory
    double *gam_glob;      // per-CTA slices of Lmax*Lmax doubles
    int use_delj;
    double *ckpt;          // optional: phi before every ckpt_every-th step
    const long *ckpt_off;  // first checkpoint double of each work id
    int ckpt_every;
    const dgb_item2d *items; // optional explicit work items (grid, slot, schedule each)
};

__host__ __device__ inline int odd_pitch(int L) { return (L % 2) ? L : L + 1; }

struct K2Layout {
    int pitch;
    size_t total;
};

static K2Layout k2_layout(int Lmax, bool gam_smem, bool delj)
{
    K2Layout l;
    l.pitch = odd_pitch(Lmax);
    size_t d = (size_t)Lmax * l.pitch + (gam_smem ? (size_t)Lmax * Lmax : 0) + 6 * (size_t)Lmax +
               2 * (size_t)(delj ? 10 : 5) * Lmax;
    l.total = d * sizeof(double);
    return l;
}

struct K2Shared {
    AxisScalars ax[2];
    double inj;
    int item;
};

__device__ __forceinline__ void k2_carve(double *smem, int Lmax, int pitch, bool gam_smem,
                                         bool delj, double *&phi, double *&gam, GridVecs &g,
                                         AxisVecs (&v)[2])
{
    double *p = smem;
    phi = p;
    p += (size_t)Lmax * pitch;
    gam = nullptr;
    if (gam_smem) {
        gam = p;
        p += (size_t)Lmax * Lmax;
    }
    g.x = p; p += Lmax;
    g.xv = p; p += Lmax;
    g.dfac = p; p += Lmax;
    g.xInt = p; p += Lmax;
    g.ih = p; p += Lmax;
    g.dx = p; p += Lmax;
    for (int a = 0; a < 2; a++) {
        v[a].A1 = p; p += Lmax;
        v[a].A0 = p; p += Lmax;
        v[a].C1 = p; p += Lmax;
        v[a].C0 = p; p += Lmax;
        v[a].B0 = p; p += Lmax;
        if (delj) {
            v[a].G = p; p += Lmax;
            v[a].Pv = p; p += Lmax;
            v[a].Qv = p; p += Lmax;
            v[a].VI = p; p += Lmax;
            v[a].DF = p; p += Lmax;
        }
    }
}

// Scalars of axis a for one step from a parameter row (called by one lane
// per axis so both axes cost one warp-wide instruction stream).
__device__ __forceinline__ void k2_axis_scalars(AxisScalars &s, int a, const double *row,
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

template <bool DELJ>
__global__ void __launch_bounds__(K2_THREADS) k_integrate2d(K2Args A)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ K2Shared S;
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int nwarps = blockDim.x >> 5;
    const int pitch = odd_pitch(A.Lmax);
    double *phi, *gam_s;
    GridVecs g;
    AxisVecs v[2];
    k2_carve(smem, A.Lmax, pitch, A.gam_smem, DELJ, phi, gam_s, g, v);
    double *gam_g = A.gam_glob ? A.gam_glob + (size_t)blockIdx.x * A.Lmax * A.Lmax : nullptr;

    // S.item is written by thread 0 and read by all between the barrier that
    // follows the write and the next barrier thread 0 must pass to write again.
    for (int iter = 0;; iter++) {
        if (tid == 0)
            S.item = A.counter ? atomicAdd(A.counter, 1) : (iter == 0 ? (int)blockIdx.x : A.nwork);
        __syncthreads();
        const int w = S.item;
        if (w >= A.nwork)
            break;
        const int wid = A.order ? A.order[w] : w;
        int inst, L, sidx, frozen, nomut;
        const double *xx, *src;
        double *out;
        if (A.items) {
            // explicit item: its own grid, output slot (holding the initial
            // density) and schedule
            const dgb_item2d &it = A.items[wid];
            inst = wid;
            L = it.L;
            xx = A.xx_all + it.xx_off;
            out = A.phi_out + it.out_off;
            src = out;
            sidx = (int)it.sched;
            frozen = it.masks & 0xff;
            nomut = it.masks >> 8 & 0xff;
        } else {
            inst = wid / A.ngrids;
            const int gi = wid - inst * A.ngrids;
            L = A.L[gi];
            xx = A.xx_all + A.xx_off[gi];
            out = A.phi_out + A.out_off[gi] + (size_t)inst * L * L;
            src = A.phi0_all ? A.phi0_all + A.phi0_off[gi] : out;
            sidx = A.sched_per_grid ? wid : inst;
            frozen = A.masks ? (A.masks[inst] & 0xff) : A.frozen_mask;
            nomut = A.masks ? (A.masks[inst] >> 8 & 0xff) : A.nomut_mask;
        }
        const double *rows = A.row_off ? A.table + A.row_off[sidx] * K2_ROW : A.table;
        const int nsteps = A.row_off ? A.row_cnt[sidx] : A.fixed_cnt;

        // grid constants and initial density
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
        for (int idx = tid; idx < L * L; idx += blockDim.x) {
            int r = idx / L, c = idx - r * L;
            phi[r * pitch + c] = src[idx];
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
        // grid index of the corner lines (other coordinate exactly 0 / 1)
        const int j0 = (g.x[0] == 0.0) ? 0 : -1;
        const int j1 = (g.x[L - 1] == 1.0) ? L - 1 : -1;
        const int lpw = (L + nwarps - 1) / nwarps;

        for (int step = 0; step < nsteps; step++) {
            const double *row = rows + (size_t)step * K2_ROW;
            if (A.ckpt && step % A.ckpt_every == 0) {
                // checkpoint for the adjoint: phi before this step, row-major
                double *c = A.ckpt + A.ckpt_off[wid] + (size_t)(step / A.ckpt_every) * L * L;
                for (int idx = tid; idx < L * L; idx += blockDim.x) {
                    int r = idx / L, q = idx - r * L;
                    c[idx] = phi[r * pitch + q];
                }
            }
            // ---- step scalars: lane a of warp 0 handles axis a, lane 2 the injection
            if (warp == 0) {
                if (lane < 2)
                    k2_axis_scalars(S.ax[lane], lane, row, g, L);
                else if (lane == 2)
                    S.inj = inject_value(2, row[0], row[1], g.x[0], g.x[1], g.x[2]);
            }
            __syncthreads();
            // ---- per-axis vectors (both axes) and mutation injection
            for (int t = tid; t < 2 * L; t += blockDim.x) {
                int a = t >= L, i = t - a * L;
                build_axis_entry(i, L, g, S.ax[a], 1.0, DELJ, v[a]);
            }
            if (tid == 0) {
                if (!(frozen & 1) && !(nomut & 1))
                    phi[1 * pitch + 0] += S.inj;
                if (!(frozen & 2) && !(nomut & 2))
                    phi[0 * pitch + 1] += S.inj;
            }
            __syncthreads();
            // ---- x sweep (axis 0): line = column j, element i at phi[i*pitch + j]
            // ---- y sweep (axis 1): line = row i, element j at phi[i*pitch + j]
            for (int a = 0; a < 2; a++) {
                if (frozen & (1 << a))
                    continue;
                const AxisScalars &s = S.ax[a];
                const int sp = (a == 0) ? pitch : 1;
                const int sl = (a == 0) ? 1 : pitch;
                const double mo = s.mig[1 - a];
                for (int k = lane; k < lpw; k += 32) {
                    int line = warp * lpw + k;
                    if (line >= L)
                        break;
                    double W = mo * g.x[line];
                    double bs = (line == j0) ? s.bcs : 0.0;
                    double be = (line == j1) ? s.bce : 0.0;
                    double *ph = phi + (size_t)line * sl;
                    if (A.gam_smem) {
                        double *gm = gam_s + line;
                        if (DELJ)
                            solve_line_delj(ph, sp, gm, L, L, &s.mig[1 - a], &g.x[line], 1,
                                            line == j0, line == j1, g, v[a], s);
                        else
                            solve_line(ph, sp, gm, L, L, W, bs, be, v[a], s);
                    } else {
                        double *gm = gam_g + line;
                        if (DELJ)
                            solve_line_delj(ph, sp, gm, L, L, &s.mig[1 - a], &g.x[line], 1,
                                            line == j0, line == j1, g, v[a], s);
                        else
                            solve_line(ph, sp, gm, L, L, W, bs, be, v[a], s);
                    }
                }
                __syncthreads();
            }
        }
        for (int idx = tid; idx < L * L; idx += blockDim.x) {
            int r = idx / L, c = idx - r * L;
            out[idx] = phi[r * pitch + c];
        }
        __syncthreads();
    }
}

// ------------------------------------------------ two items per CTA

// k_integrate2d for a launch over one grid of L points with two work items
// per CTA, stepped together: the 2L lines of a sweep (L of each item) are
// spread over ceil(2L/32) warps, so a grid whose L lines would leave a
// fourth warp mostly empty (L = 100: 25 of 32 lanes busy on four warps)
// fills its warps better (200 lines on seven warps: 29 of 32).  Each item
// keeps its own density, schedule, masks and coefficient vectors; the grid
// constants are shared.  The two items are neighbours in the longest-first
// order, so their step counts are close; the shorter one's lanes idle for
// the difference.  Per line the arithmetic is k_integrate2d's (default
// delta_j only), so the results are bitwise the same.  Thomas scratch: a 2L x L slice of the
// workspace per CTA (element p of line q at gam[p*2L + q]).
constexpr int K2P_MAXTHREADS = 256;
// dgb_settings.threads value: two work items per CTA at any grid size where
// that fills the warps better (the automatic choice keeps it to L > 96)
constexpr int K2_PAIR_ANY_L = -2;

struct K2PairShared {
    AxisScalars ax[2][2]; // [item slot][axis]
    double inj[2];
    int item[2];
};

__host__ __device__ inline size_t k2_pair_doubles(int L)
{
    return 2 * (size_t)L * odd_pitch(L) + 6 * (size_t)L + 4 * 5 * (size_t)L;
}

// Coefficient vectors of (slot, axis) index sa = 2*slot + axis.
__device__ __forceinline__ AxisVecs k2p_vecs(double *vbase, int sa, int L)
{
    double *p = vbase + (size_t)sa * 5 * L;
    AxisVecs v;
    v.A1 = p;
    v.A0 = p + L;
    v.C1 = p + 2 * L;
    v.C0 = p + 3 * L;
    v.B0 = p + 4 * L;
    v.G = v.Pv = v.Qv = v.VI = v.DF = nullptr;
    return v;
}

__global__ void __launch_bounds__(K2P_MAXTHREADS, 1) k_integrate2d_pair(K2Args A)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ K2PairShared S;
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int nwarps = blockDim.x >> 5;
    const int L = A.L[0];
    const int pitch = odd_pitch(L);
    const size_t psz = (size_t)L * pitch;
    double *phi0 = smem; // slot s at phi0 + s * psz
    GridVecs g;
    double *p = smem + 2 * psz;
    g.x = p; p += L;
    g.xv = p; p += L;
    g.dfac = p; p += L;
    g.xInt = p; p += L;
    g.ih = p; p += L;
    g.dx = p; p += L;
    double *vbase = p; // 4 x 5 x L doubles
    double *gam = A.gam_glob + (size_t)blockIdx.x * 2 * L * L;
    const double *xx = A.xx_all + A.xx_off[0];

    // grid constants, once for every item of the launch
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

    // S.item is written by thread 0 and read by all between the barrier that
    // follows the write and the next barrier thread 0 must pass to write again.
    for (int iter = 0;; iter++) {
        if (tid == 0) {
            const int base =
                A.counter ? atomicAdd(A.counter, 2) : (iter == 0 ? 2 * (int)blockIdx.x : A.nwork);
            S.item[0] = base;
            S.item[1] = base + 1;
        }
        __syncthreads();
        if (S.item[0] >= A.nwork)
            break;
        const int ns = (S.item[1] < A.nwork) ? 2 : 1; // item slots in use
        int nst0 = 0, nst1 = 0, fr0 = 0, fr1 = 0, nm0 = 0, nm1 = 0;
        const double *rows0 = nullptr, *rows1 = nullptr;
        double *out0 = nullptr, *out1 = nullptr;
        for (int s = 0; s < ns; s++) {
            const int wid = A.order ? A.order[S.item[s]] : S.item[s];
            double *out = A.phi_out + A.out_off[0] + (size_t)wid * L * L;
            const double *src = A.phi0_all ? A.phi0_all + A.phi0_off[0] : out;
            const int fr = A.masks ? (A.masks[wid] & 0xff) : A.frozen_mask;
            const int nm = A.masks ? (A.masks[wid] >> 8 & 0xff) : A.nomut_mask;
            const double *rows = A.row_off ? A.table + A.row_off[wid] * K2_ROW : A.table;
            const int nst = A.row_off ? A.row_cnt[wid] : A.fixed_cnt;
            if (s == 0) {
                out0 = out; fr0 = fr; nm0 = nm; rows0 = rows; nst0 = nst;
            } else {
                out1 = out; fr1 = fr; nm1 = nm; rows1 = rows; nst1 = nst;
            }
            double *ph = phi0 + s * psz;
            for (int idx = tid; idx < L * L; idx += blockDim.x) {
                int r = idx / L, c = idx - r * L;
                ph[r * pitch + c] = src[idx];
            }
        }
        __syncthreads();
        const int nmax = max(nst0, nst1);
        const int nl = ns * L; // lines of one sweep over the slots in use
        const int lpw = (nl + nwarps - 1) / nwarps;

        for (int step = 0; step < nmax; step++) {
            const bool act0 = step < nst0, act1 = step < nst1;
            // ---- step scalars: lane 2s+a of warp 0 for (slot s, axis a),
            // lane 4+s the injection of slot s
            if (warp == 0 && lane < 6) {
                const int s = (lane < 4) ? (lane >> 1) : lane - 4;
                if (s ? act1 : act0) {
                    const double *row = (s ? rows1 : rows0) + (size_t)step * K2_ROW;
                    if (lane < 4)
                        k2_axis_scalars(S.ax[s][lane & 1], lane & 1, row, g, L);
                    else
                        S.inj[s] = inject_value(2, row[0], row[1], g.x[0], g.x[1], g.x[2]);
                }
            }
            __syncthreads();
            // ---- per-axis vectors of both slots and mutation injection
            for (int t = tid; t < ns * 2 * L; t += blockDim.x) {
                const int sa = t / L, i = t - sa * L; // sa = 2*slot + axis
                if ((sa >> 1) ? act1 : act0) {
                    AxisVecs v = k2p_vecs(vbase, sa, L);
                    build_axis_entry(i, L, g, S.ax[sa >> 1][sa & 1], 1.0, false, v);
                }
            }
            if (tid == 0) {
                for (int s = 0; s < ns; s++) {
                    if (!(s ? act1 : act0))
                        continue;
                    const int fr = s ? fr1 : fr0, nm = s ? nm1 : nm0;
                    double *ph = phi0 + s * psz;
                    if (!(fr & 1) && !(nm & 1))
                        ph[1 * pitch + 0] += S.inj[s];
                    if (!(fr & 2) && !(nm & 2))
                        ph[0 * pitch + 1] += S.inj[s];
                }
            }
            __syncthreads();
            // ---- x sweep (axis 0) then y sweep (axis 1) over both slots' lines
            for (int a = 0; a < 2; a++) {
                const int sp = (a == 0) ? pitch : 1;
                const int sl = (a == 0) ? 1 : pitch;
                for (int k = lane; k < lpw; k += 32) {
                    const int q = warp * lpw + k;
                    if (q >= nl)
                        break;
                    const int s = (q >= L) ? 1 : 0;
                    const int line = q - s * L;
                    if (!(s ? act1 : act0) || ((s ? fr1 : fr0) & (1 << a)))
                        continue;
                    const AxisScalars &sc = S.ax[s][a];
                    const AxisVecs v = k2p_vecs(vbase, 2 * s + a, L);
                    const double W = sc.mig[1 - a] * g.x[line];
                    const double bs = (line == j0) ? sc.bcs : 0.0;
                    const double be = (line == j1) ? sc.bce : 0.0;
                    double *ph = phi0 + s * psz + (size_t)line * sl;
                    solve_line(ph, sp, gam + q, 2 * L, L, W, bs, be, v, sc);
                }
                __syncthreads();
            }
        }
        for (int s = 0; s < ns; s++) {
            const double *ph = phi0 + s * psz;
            double *out = s ? out1 : out0;
            for (int idx = tid; idx < L * L; idx += blockDim.x) {
                int r = idx / L, c = idx - r * L;
                out[idx] = ph[r * pitch + c];
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------- schedule pass

// Walk the reference time loop of two_pops (dadi/Integration.py:346-386) for
// one instance with parametric parameters.  Emits one row per step (when
// rows != null) and returns the number of rows; *status gets DGB_ST_* bits.
// dx0 is the grid's first spacing (only used with use_old_timestep).
__host__ __device__ inline long sched2d_walk(const dgb_inst2d &I, const dgb_settings &st,
                                             double dx0, long max_steps, double *rows,
                                             int *status)
{
    double cur = I.initial_t;
    double nu0 = pform_eval(I.nu[0], cur), nu1 = pform_eval(I.nu[1], cur);
    double m0 = pform_eval(I.m12, cur), m1 = pform_eval(I.m21, cur);
    double g0 = pform_eval(I.gamma[0], cur), g1 = pform_eval(I.gamma[1], cur);
    double h0 = pform_eval(I.h[0], cur), h1 = pform_eval(I.h[1], cur);
    long n = 0;
    int err = 0;
    while (cur < I.T) {
        if (n >= max_steps) {
            err |= DGB_ST_STEPCAP;
            break;
        }
        double d0 = compute_dt(nu0, m0, g0, h0, st, dx0);
        double d1 = compute_dt(nu1, m1, g1, h1, st, dx0);
        double dtm = pymin(d0, d1);
        if (dtm == 0) {
            err |= DGB_ST_ZERODT;
            break;
        }
        double dt = pymin(dtm, I.T - cur);
        double next = cur + dt;
        if (!(dt > 0) || !isfinite(next)) {
            err |= DGB_ST_NONFINITE;
            break;
        }
        nu0 = pform_eval(I.nu[0], next);
        nu1 = pform_eval(I.nu[1], next);
        m0 = pform_eval(I.m12, next);
        m1 = pform_eval(I.m21, next);
        g0 = pform_eval(I.gamma[0], next);
        g1 = pform_eval(I.gamma[1], next);
        h0 = pform_eval(I.h[0], next);
        h1 = pform_eval(I.h[1], next);
        double theta0 = pform_eval(I.theta0, next);
        if (I.T < 0 || nu0 < 0 || nu1 < 0 || m0 < 0 || m1 < 0 || theta0 < 0 || nu0 == 0 ||
            nu1 == 0) {
            err |= DGB_ST_BADPARAM;
            break;
        }
        if (rows) {
            double *r = rows + n * K2_ROW;
            r[0] = dt;
            r[1] = theta0;
            r[2] = nu0;
            r[3] = nu1;
            r[4] = g0;
            r[5] = g1;
            r[6] = h0;
            r[7] = h1;
            r[8] = 1.0;
            r[9] = m0;  // into pop 1 from pop 2 (m12)
            r[10] = m1; // into pop 2 from pop 1 (m21)
        }
        n++;
        cur = next;
    }
    if (status)
        *status |= err;
    return n;
}

// sched2d_walk on two lanes of a warp: lane p evaluates population p's
// forms and timestep (lane 0 also theta0), the two exchange their timesteps
// by shuffle and so take the same steps, and each writes its population's
// entries of the rows.  The FP64 pipe takes a warp instruction in the same
// time whatever the number of active lanes, so the per-step chain (one
// pow and one timestep per population) issues half the FP64 instructions of
// one lane doing both.  The same functions give the same rows and status as
// sched2d_walk.
__device__ long sched2d_walk_pair(const dgb_inst2d &I, const dgb_settings &st, double dx0,
                                  long max_steps, double *rows, int *status, int p)
{
    const unsigned pair = 3u << (threadIdx.x & 30);
    const dgb_pform &fnu = I.nu[p], &fm = p ? I.m21 : I.m12, &fg = I.gamma[p], &fh = I.h[p];
    double cur = I.initial_t;
    double nu = pform_eval(fnu, cur), m = pform_eval(fm, cur);
    double g = pform_eval(fg, cur), h = pform_eval(fh, cur);
    long n = 0;
    int err = 0;
    while (cur < I.T) {
        if (n >= max_steps) {
            err |= DGB_ST_STEPCAP;
            break;
        }
        const double mine = compute_dt(nu, m, g, h, st, dx0);
        const double other = __shfl_xor_sync(pair, mine, 1);
        const double dtm = p ? pymin(other, mine) : pymin(mine, other);
        if (dtm == 0) {
            err |= DGB_ST_ZERODT;
            break;
        }
        const double dt = pymin(dtm, I.T - cur);
        const double next = cur + dt;
        if (!(dt > 0) || !isfinite(next)) {
            err |= DGB_ST_NONFINITE;
            break;
        }
        nu = pform_eval(fnu, next);
        m = pform_eval(fm, next);
        g = pform_eval(fg, next);
        h = pform_eval(fh, next);
        const double theta0 = p ? 0.0 : pform_eval(I.theta0, next);
        const bool bad = nu < 0 || m < 0 || nu == 0 || theta0 < 0;
        if (I.T < 0 || __any_sync(pair, bad)) {
            err |= DGB_ST_BADPARAM;
            break;
        }
        if (rows) {
            double *r = rows + n * K2_ROW;
            if (p == 0) {
                r[0] = dt;
                r[1] = theta0;
                r[2] = nu;
                r[4] = g;
                r[6] = h;
                r[8] = 1.0;
                r[9] = m; // into pop 1 from pop 2 (m12)
            } else {
                r[3] = nu;
                r[5] = g;
                r[7] = h;
                r[10] = m; // into pop 2 from pop 1 (m21)
            }
        }
        n++;
        cur = next;
    }
    *status |= err;
    return n;
}

// Two lanes per schedule (instance, or instance x grid with
// use_old_timestep; sched2d_walk_pair).  fill == 0: count rows; fill == 1:
// write rows at row_off[s] and the status bits.
__global__ void k_sched2d(const dgb_inst2d *insts, int nsched, int ngrids, int per_grid,
                          const double *dx0s, dgb_settings st, long max_steps, int fill,
                          int *row_cnt, const long *row_off, double *table, int *status)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = t >> 1, p = t & 1;
    if (s >= nsched)
        return; // both lanes of the pair
    int inst = per_grid ? s / ngrids : s;
    double dx0 = dx0s[per_grid ? s % ngrids : 0];
    int err = 0;
    // fill == 2: row_cnt holds the room reserved at row_off (an upper bound
    // on the rows); a walk that would exceed it stops with DGB_ST_STEPCAP
    const long cap = (fill == 2) ? std::min<long>(max_steps, row_cnt[s]) : max_steps;
    long n = sched2d_walk_pair(insts[inst], st, dx0, cap,
                               fill ? table + row_off[s] * K2_ROW : nullptr, &err, p);
    if (p)
        return;
    if (fill != 1)
        row_cnt[s] = (int)n;
    if (fill && err)
        atomicOr(status + inst, err);
}

// ------------------------------------------------------------ host side

int k2_smem_fits(int Lmax, bool gam_smem, bool delj, size_t *bytes)
{
    K2Layout l = k2_layout(Lmax, gam_smem, delj);
    if (bytes)
        *bytes = l.total;
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return 0;
    return l.total + sizeof(K2Shared) + 1024 <= (size_t)optin;
}

static int k2_launch(K2Args &A, int nblocks, size_t smem, cudaStream_t st,
                     int threads = K2_THREADS)
{
    if (A.use_delj) {
        if (raise_smem_limit(k_integrate2d<true>))
            return DGB_ERR_CUDA;
        k_integrate2d<true><<<nblocks, threads, smem, st>>>(A);
    } else {
        if (raise_smem_limit(k_integrate2d<false>))
            return DGB_ERR_CUDA;
        k_integrate2d<false><<<nblocks, threads, smem, st>>>(A);
    }
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

// Resident CTAs per SM for a dynamic shared-memory size.  The kernel's
// dynamic-smem limit is raised to the opt-in maximum first: the occupancy
// query honours the current limit, so without this its answer would depend on
// the previous launch.
static int k2_occupancy(bool delj, size_t smem, int threads = K2_THREADS)
{
    int nb = 0;
    cudaError_t e;
    if (delj) {
        raise_smem_limit(k_integrate2d<true>);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_integrate2d<true>, threads,
                                                          smem);
    } else {
        raise_smem_limit(k_integrate2d<false>);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_integrate2d<false>, threads,
                                                          smem);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return nb > 0 ? nb : 1;
}

// Resident two-item CTAs per SM (k_integrate2d_pair), as k2_occupancy.
static int k2_pair_occupancy(size_t smem, int threads)
{
    int nb = 0;
    raise_smem_limit(k_integrate2d_pair);
    cudaError_t e =
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_integrate2d_pair, threads, smem);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return nb;
}

// Threads of a two-item CTA for grids of L points when pairing pays: one
// grid of 97-128 points (a single item needs four warps there) whose 2L
// lines fill their warps at least 5 % better than L lines fill four; else 0.
// Threads of a two-item CTA for grids of L points, or 0 where one item per
// CTA is kept: pairs only when they fill the warps' lanes at least 5 points
// better, and (unless any_L) only for L > 72.  Measured on the 4096-instance
// IM batch: at L = 100 (200 lines on 7 warps against 100 on 4) the launch
// went from 4977 to 4590 ms, at L = 80 (160 lines on 5 warps against 80 on
// 3, one CTA per SM instead of three) the step's integration from 11.30 to
// 11.00 s; at L = 90 pairs fill the lanes no better (180 of 192).
static int k2_pair_threads(int L, bool any_L = false)
{
    if ((!any_L && L <= 72) || L > K2P_MAXTHREADS / 2)
        return 0;
    const int w1 = (L + 31) / 32, w2 = (2 * L + 31) / 32;
    const double f1 = (double)L / (32 * w1), f2 = (double)(2 * L) / (32 * w2);
    return (f2 >= f1 + 0.05) ? 32 * w2 : 0;
}

static int k2_num_sms()
{
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    return nsm > 0 ? nsm : 1;
}

// Threads per CTA of a batched launch whose grids are at most Lmax points:
// the fewest warps (two to four) that give every line of the largest grid
// its own lane.  A sweep of one line is one lane's dependency chain and the
// FP64 pipe charges a warp instruction whatever its active lanes, so lines
// packed into fewer warps cost fewer pipe cycles per step.  Measured on the
// 4096-instance IM batch at pts 80/90/100, one launch per grid: three warps
// at L = 80 and 90 (27 and 30 of 32 lanes busy, instead of 20 and 23 with
// four) 11.72 s, four warps for every grid 13.39 s, bitwise the same
// densities.  settings->threads = 64, 96 or 128 asks for that size where it
// holds the lines (else the automatic choice applies); 0 is automatic.
// occ gets the CTAs per SM.  Returns 0 for an unsupported setting.
static int k2_pick_threads(const dgb_settings *settings, bool delj, size_t smem, int Lmax,
                           int &occ)
{
    const int want = (settings->threads == K2_PAIR_ANY_L) ? 0 : settings->threads;
    if (want != 0 && want != 64 && want != 96 && want != 128)
        return 0;
    int warps = std::min(4, std::max(2, (Lmax + 31) / 32));
    if (want != 0 && Lmax <= want)
        warps = want / 32;
    occ = k2_occupancy(delj, smem + sizeof(K2Shared), 32 * warps);
    return 32 * warps;
}

int k2_integrate_table(double *phi, int L, const double *xx, const double *table, int nsteps,
                       int frozen_mask, int nomut_mask, int use_delj, void *ws, size_t ws_bytes,
                       cudaStream_t st)
{
    // one schedule: rows 0 .. nsteps-1 of the table
    K2Args A = {};
    A.ngrids = 1;
    A.L[0] = L;
    A.xx_all = xx;
    A.phi_out = phi;
    A.table = table;
    A.fixed_cnt = nsteps;
    A.frozen_mask = frozen_mask;
    A.nomut_mask = nomut_mask;
    A.nwork = 1;
    A.Lmax = L;
    A.use_delj = use_delj;
    size_t bytes;
    A.gam_smem = k2_smem_fits(L, true, use_delj, &bytes);
    if (!A.gam_smem) {
        if (!k2_smem_fits(L, false, use_delj, &bytes))
            return DGB_ERR_UNSUPPORTED;
        if (!ws || ws_bytes < (size_t)L * L * sizeof(double))
            return DGB_ERR_WORKSPACE;
        A.gam_glob = (double *)ws;
    }
    return k2_launch(A, 1, bytes, st);
}

size_t k2_table_ws_bytes(int L) { return (size_t)L * L * sizeof(double); }

size_t k2_batch_ws_bytes(int Lmax, long nwork)
{
    (void)nwork;
    return 256 + (size_t)k2_num_sms() * 4 * Lmax * Lmax * sizeof(double);
}

// norder: integrate only the work items order[0 .. norder) (<= 0: all);
// reserve_sms: SMs to leave to launches running at the same time (the CTAs
// are capped at (SMs - reserve_sms) x CTAs per SM).
int k2_batch(int ninst, const int *masks, const int *Ls, int ngrids, const double *xx_all,
             const double *phi0_all, double *phi_out, const double *table, const long *row_off,
             const int *row_cnt, int sched_per_grid, const int *order,
             const dgb_settings *settings, void *ws, size_t ws_bytes, cudaStream_t st,
             double *ckpt = nullptr, const long *ckpt_off = nullptr, int ckpt_every = 0,
             int norder = 0, int reserve_sms = 0)
{
    if (ngrids < 1 || ngrids > K2_MAXG || ninst < 1)
        return DGB_ERR_ARG;
    K2Args A = {};
    A.ngrids = ngrids;
    long xo = 0, po = 0, oo = 0;
    int Lmax = 0;
    for (int gi = 0; gi < ngrids; gi++) {
        if (Ls[gi] < 3)
            return DGB_ERR_ARG;
        A.L[gi] = Ls[gi];
        A.xx_off[gi] = xo;
        A.phi0_off[gi] = po;
        A.out_off[gi] = oo;
        xo += Ls[gi];
        po += (long)Ls[gi] * Ls[gi];
        oo += (long)ninst * Ls[gi] * Ls[gi];
        Lmax = std::max(Lmax, Ls[gi]);
    }
    A.xx_all = xx_all;
    A.phi0_all = phi0_all;
    A.phi_out = phi_out;
    A.table = table;
    A.row_off = row_off;
    A.row_cnt = row_cnt;
    A.sched_per_grid = sched_per_grid;
    A.masks = masks;
    A.order = order;
    A.nwork = (norder > 0 && norder < ninst * ngrids) ? norder : ninst * ngrids;
    A.Lmax = Lmax;
    A.use_delj = settings->use_delj_trick;
    A.ckpt = ckpt;
    A.ckpt_off = ckpt_off;
    A.ckpt_every = ckpt_every > 0 ? ckpt_every : 1;
    if (!ws || ws_bytes < 256)
        return DGB_ERR_WORKSPACE;
    A.counter = (int *)ws;
    size_t bytes_s = 0, bytes_g = 0;
    bool fit_s = k2_smem_fits(Lmax, true, A.use_delj, &bytes_s);
    bool fit_g = k2_smem_fits(Lmax, false, A.use_delj, &bytes_g);
    if (!fit_g)
        return DGB_ERR_UNSUPPORTED;
    int nsm = k2_num_sms();
    int occ_s = fit_s ? k2_occupancy(A.use_delj, bytes_s + sizeof(K2Shared)) : 0;
    int occ_g = k2_occupancy(A.use_delj, bytes_g + sizeof(K2Shared));
    size_t slice = (size_t)Lmax * Lmax * sizeof(double);
    // auto: gam in shared memory only when that does not cost CTAs per SM.
    // Measured on the 4096-instance IM batch at pts 80/90/100: gam in the
    // workspace (two CTAs per SM at L = 100, two warps per SMSP) 13.44 s,
    // gam in shared memory (one CTA per SM) 17.11 s; the back substitution
    // prefetches its L2 operands, and the second warp per SMSP fills the FP64
    // pipe's dependency gaps.
    bool use_s = fit_s && occ_s >= occ_g;
    if (settings->gam_placement == 1) {
        if (!fit_s)
            return DGB_ERR_UNSUPPORTED;
        use_s = true;
    } else if (settings->gam_placement == 2) {
        use_s = false;
    }
    int nblocks;
    size_t smem;
    int threads;
    if (use_s) {
        A.gam_smem = 1;
        smem = bytes_s;
        threads = k2_pick_threads(settings, A.use_delj, smem, A.Lmax, occ_s);
        nblocks = nsm * occ_s;
    } else {
        A.gam_smem = 0;
        A.gam_glob = (double *)((char *)ws + 256);
        smem = bytes_g;
        threads = k2_pick_threads(settings, A.use_delj, smem, A.Lmax, occ_g);
        nblocks = (int)std::min<size_t>((ws_bytes - 256) / slice, (size_t)nsm * occ_g);
    }
    if (threads == 0)
        return DGB_ERR_ARG;
    // two work items per CTA where that fills the warps better (one grid,
    // automatic thread count, no checkpoints, scratch in the workspace; the
    // two-item kernel implements the default delta_j only, so the delj
    // trick keeps one item per CTA)
    const bool any_L = settings->threads == K2_PAIR_ANY_L;
    const int pthreads = (ngrids == 1 && !ckpt && !use_s && (settings->threads == 0 || any_L) &&
                          !A.use_delj)
                             ? k2_pair_threads(Lmax, any_L)
                             : 0;
    if (pthreads) {
        const size_t pbytes = k2_pair_doubles(Lmax) * sizeof(double);
        int dev = 0, optin = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
                cudaSuccess)
            return DGB_ERR_CUDA;
        const int pocc = (pbytes + sizeof(K2PairShared) + 1024 <= (size_t)optin)
                             ? k2_pair_occupancy(pbytes, pthreads)
                             : 0;
        long pblocks = std::min<long>((long)((ws_bytes - 256) / (2 * slice)), (long)nsm * pocc);
        pblocks = std::min<long>(pblocks, (A.nwork + 1) / 2);
        if (pblocks >= 1) {
            A.gam_smem = 0;
            A.gam_glob = (double *)((char *)ws + 256);
            if (cudaMemsetAsync(A.counter, 0, sizeof(int), st) != cudaSuccess)
                return DGB_ERR_CUDA;
            k_integrate2d_pair<<<(unsigned)pblocks, pthreads, pbytes, st>>>(A);
            return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
        }
    }
    if (nblocks < 1)
        return DGB_ERR_WORKSPACE;
    nblocks = std::min(nblocks, A.nwork);
    if (reserve_sms > 0) {
        const int occ = use_s ? occ_s : occ_g;
        nblocks = std::min(nblocks, std::max(1, (nsm - reserve_sms) * occ));
    }
    if (cudaMemsetAsync(A.counter, 0, sizeof(int), st) != cudaSuccess)
        return DGB_ERR_CUDA;
    return k2_launch(A, nblocks, smem, st, threads);
}

// ------------------------------------------- allocation-free entry point

// Thomas scratch of dgb_integrate2d_noalloc: one L x L array for L up to
// DGB_NOALLOC_MAX_L (128 KB), resident on every GPU that loads the library.
static __device__ __align__(256) double g_noalloc_gam[DGB_NOALLOC_MAX_L * DGB_NOALLOC_MAX_L];

// Device address of g_noalloc_gam per device, looked up with that device
// current (host code must not use the symbol itself).  Only a successful
// lookup is kept: a failed one (e.g. made during stream capture) is retried
// by the next call.
constexpr int NOALLOC_MAXDEV = 64;
static std::mutex g_noalloc_mu;
static double *g_noalloc_ptr[NOALLOC_MAXDEV];

static int noalloc_scratch(double **ptr)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0)
        return DGB_ERR_CUDA;
    if (dev >= NOALLOC_MAXDEV)
        return DGB_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_gam) != cudaSuccess || !p) {
            cudaGetLastError();
            return DGB_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = (double *)p;
    }
    *ptr = g_noalloc_ptr[dev];
    return DGB_OK;
}

} // namespace dgb

// ------------------------------------------------------------------ C ABI

extern "C" int dgb_sched2d(const dgb_inst2d *insts, int ninst, int ngrids, const double *dx0s,
                           const dgb_settings *settings, long max_steps, int fill, int *row_cnt,
                           const long *row_off, double *table, int *status, void *stream)
{
    if (!insts || ninst < 1 || ngrids < 1 || !dx0s || !settings || max_steps < 1 ||
        fill < 0 || fill > 2 || (fill != 1 && !row_cnt) ||
        (fill && (!row_off || !table || !status)))
        return DGB_ERR_ARG;
    int per_grid = settings->use_old_timestep ? 1 : 0;
    int nsched = per_grid ? ninst * ngrids : ninst;
    // one warp per block (16 schedules, two lanes each): schedules are long
    // serial chains, spread over the SMs
    const long nthreads = 2L * nsched;
    const int nt = 32;
    dgb::k_sched2d<<<(unsigned)((nthreads + nt - 1) / nt), nt, 0, (cudaStream_t)stream>>>(
        insts, nsched, ngrids, per_grid, dx0s, *settings, max_steps, fill, row_cnt, row_off,
        table, status);
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

extern "C" int dgb_batch2d_integrate(const int *masks, int ninst, const int *Ls, int ngrids,
                                     const double *xx_all, const double *phi0_all,
                                     double *phi_out, const double *table, const long *row_off,
                                     const int *row_cnt, const int *order,
                                     const dgb_settings *settings, void *ws, size_t ws_bytes,
                                     void *stream)
{
    if (!Ls || !xx_all || !phi0_all || !phi_out || !table || !row_off || !row_cnt || !order ||
        !settings)
        return DGB_ERR_ARG;
    return dgb::k2_batch(ninst, masks, Ls, ngrids, xx_all, phi0_all, phi_out, table, row_off,
                         row_cnt, settings->use_old_timestep ? 1 : 0, order, settings, ws,
                         ws_bytes, (cudaStream_t)stream);
}

extern "C" int dgb_batch2d_count_steps(const dgb_inst2d *insts, int ninst,
                                       const dgb_settings *settings, long max_steps,
                                       long *steps_out)
{
    if (!insts || !settings || !steps_out || ninst < 0)
        return DGB_ERR_ARG;
    for (int n = 0; n < ninst; n++)
        steps_out[n] = dgb::sched2d_walk(insts[n], *settings, 1e-3, max_steps, nullptr, nullptr);
    return DGB_OK;
}

extern "C" int dgb_integrate2d_noalloc(double *phi, int L, const double *xx, const double *table,
                                       int nsteps, int frozen_mask, int nomut_mask,
                                       int use_delj_trick, void *stream)
{
    if (!phi || !xx || !table || nsteps < 0 || L < 3)
        return DGB_ERR_ARG;
    if (L > DGB_NOALLOC_MAX_L)
        return DGB_ERR_TOO_LARGE;
    if (nsteps == 0)
        return DGB_OK;
    dgb::K2Args A = {};
    size_t bytes = 0;
    // the Thomas scratch in shared memory where it fits beside phi (as
    // dgb_integrate_table does); only larger grids use the static array
    A.gam_smem = dgb::k2_smem_fits(L, true, use_delj_trick != 0, &bytes);
    if (!A.gam_smem) {
        if (!dgb::k2_smem_fits(L, false, use_delj_trick != 0, &bytes))
            return DGB_ERR_UNSUPPORTED;
        int rc = dgb::noalloc_scratch(&A.gam_glob);
        if (rc)
            return rc;
    }
    A.ngrids = 1;
    A.L[0] = L;
    A.xx_all = xx;
    A.phi_out = phi;
    A.table = table;
    A.fixed_cnt = nsteps;
    A.frozen_mask = frozen_mask;
    A.nomut_mask = nomut_mask;
    A.nwork = 1;
    A.Lmax = L;
    A.use_delj = use_delj_trick;
    return dgb::k2_launch(A, 1, bytes, (cudaStream_t)stream);
}

extern "C" int dgb_batch2d_integrate_ckpt(const int *masks, int ninst, const int *Ls, int ngrids,
                                          const double *xx_all, const double *phi0_all,
                                          double *phi_out, const double *table,
                                          const long *row_off, const int *row_cnt,
                                          const int *order, const dgb_settings *settings,
                                          double *ckpt, const long *ckpt_off, int ckpt_every,
                                          void *ws, size_t ws_bytes, void *stream)
{
    if (!Ls || !xx_all || !phi0_all || !phi_out || !table || !row_off || !row_cnt || !order ||
        !settings || !ckpt || !ckpt_off || ckpt_every < 1)
        return DGB_ERR_ARG;
    return dgb::k2_batch(ninst, masks, Ls, ngrids, xx_all, phi0_all, phi_out, table, row_off,
                         row_cnt, settings->use_old_timestep ? 1 : 0, order, settings, ws,
                         ws_bytes, (cudaStream_t)stream, ckpt, ckpt_off, ckpt_every);
}

extern "C" int dgb_batch2d_integrate_ckpt_part(
    const int *masks, int ninst, const int *Ls, int ngrids, const double *xx_all,
    const double *phi0_all, double *phi_out, const double *table, const long *row_off,
    const int *row_cnt, const int *order, int norder, int reserve_sms,
    const dgb_settings *settings, double *ckpt, const long *ckpt_off, int ckpt_every, void *ws,
    size_t ws_bytes, void *stream)
{
    if (!Ls || !xx_all || !phi0_all || !phi_out || !table || !row_off || !row_cnt || !order ||
        !settings || !ckpt || !ckpt_off || ckpt_every < 1 || norder < 1 ||
        norder > ninst * ngrids)
        return DGB_ERR_ARG;
    return dgb::k2_batch(ninst, masks, Ls, ngrids, xx_all, phi0_all, phi_out, table, row_off,
                         row_cnt, settings->use_old_timestep ? 1 : 0, order, settings, ws,
                         ws_bytes, (cudaStream_t)stream, ckpt, ckpt_off, ckpt_every, norder,
                         reserve_sms);
}

extern "C" int dgb_items2d_integrate(const dgb_item2d *items, int nitems, int Lmax,
                                     const double *xx_all, double *phi_out, const double *table,
                                     const long *row_off, const int *row_cnt, const int *order,
                                     const dgb_settings *settings, int one_per_cta, void *ws,
                                     size_t ws_bytes, void *stream)
{
    using namespace dgb;
    if (!items || nitems < 1 || Lmax < 3 || !xx_all || !phi_out || !table || !row_off ||
        !row_cnt || !settings)
        return DGB_ERR_ARG;
    K2Args A = {};
    A.ngrids = 1;
    A.L[0] = Lmax;
    A.xx_all = xx_all;
    A.phi_out = phi_out;
    A.table = table;
    A.row_off = row_off;
    A.row_cnt = row_cnt;
    A.order = order;
    A.nwork = nitems;
    A.Lmax = Lmax;
    A.use_delj = settings->use_delj_trick;
    A.items = items;
    if (!ws || ws_bytes < 256)
        return DGB_ERR_WORKSPACE;
    A.counter = (int *)ws;
    size_t bytes_s = 0, bytes_g = 0;
    bool fit_s = k2_smem_fits(Lmax, true, A.use_delj, &bytes_s);
    if (!k2_smem_fits(Lmax, false, A.use_delj, &bytes_g))
        return DGB_ERR_UNSUPPORTED;
    // gam placement: 0 shared memory when it fits, 1 shared (must fit),
    // 2 the workspace
    if (settings->gam_placement == 1 && !fit_s)
        return DGB_ERR_UNSUPPORTED;
    if (settings->gam_placement == 2)
        fit_s = false;
    else if (settings->gam_placement == 0 && fit_s &&
             k2_occupancy(A.use_delj, bytes_s + sizeof(K2Shared)) <
                 k2_occupancy(A.use_delj, bytes_g + sizeof(K2Shared)))
        fit_s = false; // as in k2_batch: shared memory only if it costs no CTAs per SM
    int nsm = k2_num_sms();
    int nblocks;
    size_t smem = fit_s ? bytes_s : bytes_g;
    size_t slice = (size_t)Lmax * Lmax * sizeof(double);
    int occ = 1;
    const int threads = k2_pick_threads(settings, A.use_delj, smem, Lmax, occ);
    if (threads == 0)
        return DGB_ERR_ARG;
    if (one_per_cta) {
        // CTA b integrates item order[b] (or b) and retires: no queue
        A.counter = nullptr;
        nblocks = nitems;
        A.gam_smem = fit_s ? 1 : 0;
        if (!fit_s) {
            if ((ws_bytes - 256) / slice < (size_t)nitems)
                return DGB_ERR_WORKSPACE;
            A.gam_glob = (double *)((char *)ws + 256);
        }
        return k2_launch(A, nblocks, smem, (cudaStream_t)stream, threads);
    }
    if (fit_s) {
        A.gam_smem = 1;
        nblocks = nsm * occ;
    } else {
        A.gam_smem = 0;
        nblocks = (int)std::min<size_t>((ws_bytes - 256) / slice, (size_t)nsm * occ);
        A.gam_glob = (double *)((char *)ws + 256);
    }
    if (nblocks < 1)
        return DGB_ERR_WORKSPACE;
    nblocks = std::min(nblocks, nitems);
    if (cudaMemsetAsync(A.counter, 0, sizeof(int), (cudaStream_t)stream) != cudaSuccess)
        return DGB_ERR_CUDA;
    return k2_launch(A, nblocks, smem, (cudaStream_t)stream, threads);
}

extern "C" int dgb_sched2d_host(const dgb_inst2d *insts, int ninst,
                                const dgb_settings *settings, long max_steps, double dx0,
                                int *row_cnt, const long *row_off, double *table, int *status)
{
    if (!insts || ninst < 0 || !settings || max_steps < 1 || (!table && !row_cnt) ||
        (table && (!row_off || !status)))
        return DGB_ERR_ARG;
    for (int n = 0; n < ninst; n++) {
        int err = 0;
        long c = dgb::sched2d_walk(insts[n], *settings, dx0, max_steps,
                                   table ? table + row_off[n] * dgb::K2_ROW : nullptr, &err);
        if (!table)
            row_cnt[n] = (int)c;
        else
            status[n] |= err;
    }
    return DGB_OK;
}

namespace dgb {
int preload_integrate2d()
{
    return preload(k_integrate2d<false>) + preload(k_integrate2d<true>) +
           preload(k_integrate2d_pair) + preload(k_sched2d);
}
} // namespace dgb
