// Shared pieces of the per-axis N-dimensional sweep kernels: launch
// arguments, shared-memory carving, per-step parameter loading and the tile
// staging of lines (see dgb_sweepnd.cu), used by the forward sweeps and by
// the discrete adjoint of the N-dimensional time loop (dgb_adjointnd.cu).
#pragma once
#include <algorithm>

#include "dgb_common.cuh"
#include "dgb_internal.h"

namespace dgb {

struct NDArgs {
    double *phi;
    const double *xx;
    int ndim, L, axis;
    long nlines, S, LS; // lines, stride of the axis, L*S
    // parameters: from table row `step` when table != null, else explicit
    const double *table;
    long step;
    double nu, gamma, h, beta, dt, theta0;
    double mig[DGB_MAX_DIM];
    int inject_mask; // populations whose mutations are injected by this sweep
    // constant-coefficient mode
    const double *ca, *cb, *cc;
    const double *dts;
};

__host__ __device__ inline size_t nd_smem_doubles(int L, int nt, bool delj)
{
    return (size_t)L * (nt + 1) + (size_t)L * nt + (size_t)(delj ? 10 : 5) * L + 6 * (size_t)L;
}

struct NDShared {
    AxisScalars s;
    double vscale;
    double beta1; // the breeding ratio for one population, else 0
    double inj[DGB_MAX_DIM];
};

// Per-step coefficient records (k_coef_nd -> k_sweep_nd_rec, dgb_sweepnd.cu).
// A coefficient buffer holds the grid constants (x, xv, dfac, xInt, ih, dx:
// 6 L doubles, the GridVecs order) followed by one record per (step of the
// chunk, axis): the head (the axis scalars and the injection amounts), then
// the per-axis vectors A1, A0, C1, C0, B0 and, with the delj trick, G, Pv,
// Qv, VI, DF (L doubles each).
struct NDRecHead {
    AxisScalars s;
    double inj[DGB_MAX_DIM];
};
constexpr int ND_HEAD = (int)(sizeof(NDRecHead) / sizeof(double));
static_assert(sizeof(NDRecHead) == ND_HEAD * sizeof(double), "record head is whole doubles");

__host__ __device__ inline int nd_grid_doubles(int L) { return 6 * L; }

__host__ __device__ inline size_t nd_rec_doubles(int L, bool delj)
{
    return (size_t)ND_HEAD + (size_t)(delj ? 10 : 5) * L;
}

// The per-axis vectors laid out from p on (a record's vectors start at
// rec + ND_HEAD).
__host__ __device__ inline void nd_vecs_at(double *p, int L, bool delj, AxisVecs &v)
{
    v.A1 = p;
    v.A0 = p + L;
    v.C1 = p + 2 * L;
    v.C0 = p + 3 * L;
    v.B0 = p + 4 * L;
    v.G = v.Pv = v.Qv = v.VI = v.DF = nullptr;
    if (delj) {
        v.G = p + 5 * L;
        v.Pv = p + 6 * L;
        v.Qv = p + 7 * L;
        v.VI = p + 8 * L;
        v.DF = p + 9 * L;
    }
}

// Shared memory of k_sweep_nd_rec: the tile, gam, x/xInt/dx and the vectors.
__host__ __device__ inline size_t nd_rec_smem_doubles(int L, int nt, bool delj)
{
    return (size_t)L * (nt + 1) + (size_t)L * nt + 3 * (size_t)L + (size_t)(delj ? 10 : 5) * L;
}

// Steps per coefficient chunk: up to 256, with the records of a chunk kept
// under 8 MB (sized for the delj layout, so one chunk length serves both).
__host__ __device__ inline int nd_chunk_steps(int ndim, int L)
{
    const size_t per_step = (size_t)ndim * nd_rec_doubles(L, true) * sizeof(double);
    size_t c = ((size_t)8 << 20) / per_step;
    return (int)(c < 1 ? 1 : (c > 256 ? 256 : c));
}

// Bytes of a coefficient buffer for chunks of nd_chunk_steps steps.
inline size_t nd_coef_bytes(int ndim, int L)
{
    return ((size_t)nd_grid_doubles(L) +
            (size_t)nd_chunk_steps(ndim, L) * ndim * nd_rec_doubles(L, true)) *
           sizeof(double);
}

// Coordinates (all axes) of the first point of line `line` along `axis`.
__device__ __forceinline__ long nd_line_base(const NDArgs &A, long line, int *coord)
{
    long outer = line / A.S, inner = line - outer * A.S;
    long base = outer * A.LS + inner;
    long rem = base;
    for (int k = A.ndim - 1; k >= 0; k--) {
        coord[k] = (int)(rem % A.L);
        rem /= A.L;
    }
    return base;
}

static __device__ void nd_load_params(const NDArgs &A, NDShared &Sh, const GridVecs &g)
{
    const int P = A.ndim, ax = A.axis;
    AxisScalars &s = Sh.s;
    double beta = A.beta;
    if (A.table) {
        const double *row = A.table + A.step * row_stride(P);
        s.dt = row[0];
        Sh.inj[0] = row[1]; // theta0, used below
        s.nu = row[row_nu(P, ax)];
        s.gamma = row[row_gamma(P, ax)];
        s.h = row[row_h(P, ax)];
        beta = row[row_beta(P)];
        for (int j = 0; j < P; j++)
            s.mig[j] = (j == ax) ? 0.0 : row[row_mig(P, ax, j)];
    } else {
        s.dt = A.dt;
        Sh.inj[0] = A.theta0;
        s.nu = A.nu;
        s.gamma = A.gamma;
        s.h = A.h;
        for (int j = 0; j < P; j++)
            s.mig[j] = (j == ax) ? 0.0 : A.mig[j];
    }
    double theta0 = Sh.inj[0];
    s.inv_nu = 1.0 / s.nu;
    double msum = 0;
    for (int j = 0; j < P; j++)
        if (j != ax)
            msum = msum + s.mig[j];
    s.msum = msum;
    const int L = A.L;
    s.B1s = 0.5 * (s.dt * g.dfac[0]);
    s.B1e = -0.5 * (s.dt * g.dfac[L - 1]);
    corner_bc(P, ax, s.mig, s.nu, s.gamma, s.h, g.x[0], g.x[L - 1], g.dx[0], g.dx[L - 2], s.dt,
              s.bcs, s.bce);
    // Vfunc_beta's factor in 1-D (dadi/integration_shared.c:8-10)
    Sh.vscale = (P == 1) ? pow(beta + 1, 2) / (4 * beta) : 1.0;
    Sh.beta1 = (P == 1) ? beta : 0.0;
    double val = inject_value(P, s.dt, theta0, g.x[0], g.x[1], g.x[2]);
    for (int k = 0; k < DGB_MAX_DIM; k++)
        Sh.inj[k] = (A.inject_mask >> k & 1) ? val : 0.0;
}

static __device__ void nd_grid_consts(const NDArgs &A, GridVecs &g)
{
    const int L = A.L;
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
        double x = A.xx[i];
        g.x[i] = x;
        g.xv[i] = x * (1. - x);
        if (i < L - 1) {
            double d = A.xx[i + 1] - x;
            g.dx[i] = d;
            g.ih[i] = 1.0 / (2 * d);
            g.xInt[i] = 0.5 * (A.xx[i + 1] + x);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
        if (i == 0)
            g.dfac[i] = 2. / g.dx[0];
        else if (i == L - 1)
            g.dfac[i] = 2. / g.dx[L - 2];
        else
            g.dfac[i] = 2. / (g.dx[i] + g.dx[i - 1]);
    }
    __syncthreads();
}

__device__ __forceinline__ void nd_carve(double *smem, int L, int nt, bool delj, double *&tile,
                                         double *&gam, GridVecs &g, AxisVecs &v)
{
    double *p = smem;
    tile = p;
    p += (size_t)L * (nt + 1);
    gam = p;
    p += (size_t)L * nt;
    g.x = p; p += L;
    g.xv = p; p += L;
    g.dfac = p; p += L;
    g.xInt = p; p += L;
    g.ih = p; p += L;
    g.dx = p; p += L;
    v.A1 = p; p += L;
    v.A0 = p; p += L;
    v.C1 = p; p += L;
    v.C0 = p; p += L;
    v.B0 = p; p += L;
    if (delj) {
        v.G = p; p += L;
        v.Pv = p; p += L;
        v.Qv = p; p += L;
        v.VI = p; p += L;
        v.DF = p; p += L;
    }
}

// Load (dir=0) or store (dir=1) the CTA's tile of lines [l0, l0+n).  (Moving
// each thread's elements in batches of 8 loads in flight measured no faster
// on 3-D grids of L = 70-90: the sweep's time is its solve.)
__device__ __forceinline__ void nd_tile_io(const NDArgs &A, double *tile, int nt, long l0, int n,
                                           bool store)
{
    const int L = A.L, tp = nt + 1;
    if (A.S == 1) {
        // contiguous axis: the n lines are n*L consecutive doubles; each
        // warp copies whole lines with its lanes along the line (coalesced,
        // and no division by L per element)
        double *g0 = A.phi + l0 * L;
        const int lane = threadIdx.x & 31, nw = (int)(blockDim.x >> 5);
        for (int t = (int)(threadIdx.x >> 5); t < n; t += nw) {
            double *gl = g0 + (size_t)t * L;
            for (int p = lane; p < L; p += 32) {
                if (store)
                    gl[p] = tile[p * tp + t];
                else
                    tile[p * tp + t] = gl[p];
            }
        }
    } else {
        int t = threadIdx.x;
        if (t < n) {
            long line = l0 + t;
            long outer = line / A.S, inner = line - outer * A.S;
            double *g0 = A.phi + outer * A.LS + inner;
            for (int p = 0; p < L; p++) {
                if (store)
                    g0[p * A.S] = tile[p * tp + t];
                else
                    tile[p * tp + t] = g0[p * A.S];
            }
        }
    }
}

// Solve the CTA's tile of lines [l0, l0+n) in shared memory: per line the
// migration weight W and the corner flags from its other coordinates, the
// fused mutation injection (dadi/Integration.py:70-122) when this is the
// step's first sweep, then the Thomas solve.
template <bool DELJ>
__device__ __forceinline__ void nd_solve_tile(const NDArgs &A, double *tile, double *gam, int nt,
                                              long l0, int n, const GridVecs &g,
                                              const AxisVecs &v, const AxisScalars &s,
                                              const double *inj)
{
    const int L = A.L, P = A.ndim, ax = A.axis;
    // grid index of the corner coordinates (value exactly 0 / 1)
    const int j0 = (g.x[0] == 0.0) ? 0 : -1;
    const int j1 = (g.x[L - 1] == 1.0) ? L - 1 : -1;
    const int t = threadIdx.x;
    if (t >= n)
        return;
    int coord[DGB_MAX_DIM];
    nd_line_base(A, l0 + t, coord);
    double W = 0;
    double mo[DGB_MAX_DIM], oo[DGB_MAX_DIM];
    int no = 0;
    bool all0 = true, all1 = true;
    int n1 = 0, k1 = -1;
    for (int k = 0; k < P; k++) {
        if (k == ax)
            continue;
        W = fma(s.mig[k], g.x[coord[k]], W);
        mo[no] = s.mig[k];
        oo[no] = g.x[coord[k]];
        no++;
        all0 = all0 && coord[k] == j0;
        all1 = all1 && coord[k] == j1;
        if (coord[k] == 1) {
            n1++;
            k1 = k;
        } else if (coord[k] != 0) {
            n1 = 99;
        }
    }
    if (P == 1)
        all0 = all1 = true; // 1-D applies both boundary terms unconditionally
    const int tp = nt + 1;
    if (A.inject_mask) {
        if (n1 == 0 && inj[ax] != 0.0)
            tile[1 * tp + t] += inj[ax];
        if (n1 == 1 && inj[k1] != 0.0)
            tile[0 * tp + t] += inj[k1];
    }
    double bs = all0 ? s.bcs : 0.0;
    double be = all1 ? s.bce : 0.0;
    if (DELJ)
        solve_line_delj(tile + t, tp, gam + t, nt, L, mo, oo, no, all0, all1, g, v, s);
    else
        solve_line(tile + t, tp, gam + t, nt, L, W, bs, be, v, s);
}

// ------------------------------------------------------------ host side

static long ipow(int L, int p)
{
    long r = 1;
    for (int i = 0; i < p; i++)
        r *= L;
    return r;
}

// Lines per CTA of a sweep launch.  (Halving it to one warp so that small
// launches reach every SM was measured slower for 3-D grids of L = 70-90: the
// per-CTA setup of grid constants and coefficient vectors grows with fewer
// threads.)
static int nd_threads(int L, long nlines)
{
    int nt = (L <= 48) ? 128 : 64;
    if (nlines < nt)
        nt = (int)std::max<long>(32, (nlines + 31) / 32 * 32);
    return nt;
}

static void nd_fill(NDArgs &A, double *phi, int ndim, int L, int axis, const double *xx)
{
    A.phi = phi;
    A.xx = xx;
    A.ndim = ndim;
    A.L = L;
    A.axis = axis;
    A.S = ipow(L, ndim - 1 - axis);
    A.LS = A.S * L;
    A.nlines = ipow(L, ndim - 1);
}

static bool shape_ok(int ndim, int L) { return ndim >= 1 && ndim <= DGB_MAX_DIM && L >= 3; }

// One launch of the forward per-axis sweep (k_sweep_nd, dgb_sweepnd.cu).
int nd_sweep(NDArgs &A, bool delj, cudaStream_t st);

// Coefficient records of steps step0 .. step0+n-1 of A's table (every
// unfrozen axis; the step's first swept axis injects `active`) into coef,
// a buffer of nd_coef_bytes; n <= nd_chunk_steps.
int nd_coef_chunk(const NDArgs &A, bool delj, long step0, int n, int frozen_mask, int active,
                  double *coef, cudaStream_t st);

// One sweep (A.axis, A.step, A.inject_mask) reading the records that
// nd_coef_chunk wrote for the chunk starting at step0.
int nd_sweep_rec(NDArgs &A, bool delj, const double *coef, long step0, cudaStream_t st);

} // namespace dgb
