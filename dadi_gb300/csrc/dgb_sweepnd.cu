// Fused per-axis ADI sweep for 1-D, 3-D and 4-D densities (and 2-D grids too
// large for the shared-memory-resident kernel), the constant-coefficient
// sweep, a batched tridiagonal solver, and the C ABI entry points that drive
// them.
//
// A sweep kernel launch handles every line of one axis.  Each CTA stages a
// tile of NT lines x L points in shared memory ([point][line] layout, pitch
// NT+1, so line-parallel accesses are bank-conflict free): strided axes load
// with one coalesced row of NT lines per point, the contiguous axis with a
// linear cooperative copy of its NT*L contiguous doubles.  Coefficients are
// rebuilt from per-axis vectors (see dgb_common.cuh), mutation injection is
// fused into the first sweep of a step, and the Thomas gam scratch stays in
// shared memory, so a sweep reads and writes phi exactly once.
//
// Reference: implicit_1Dx / implicit_3D{x,y,z} / implicit_4D{x,y,z,a}
// (dadi/integration1D.c:7-66, integration3D.c:13-239, integration4D.c:13-321),
// implicit_precalc_* (integration2D.c:162-217, integration3D.c:241-345),
// tridiag_premalloc (dadi/tridiag.c:14-34).
#include <algorithm>
#include <cstring>

#include "dgb_nd.cuh"

namespace dgb {

// Sweep that builds its own step's coefficients: grid constants, the
// parameter row (one thread) and the per-axis vectors, every CTA.
template <bool DELJ>
__global__ void k_sweep_nd(NDArgs A)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ NDShared Sh;
    const int nt = blockDim.x, L = A.L;
    double *tile, *gam;
    GridVecs g;
    AxisVecs v;
    nd_carve(smem, L, nt, DELJ, tile, gam, g, v);
    nd_grid_consts(A, g);
    if (threadIdx.x == 0)
        nd_load_params(A, Sh, g);
    __syncthreads();
    for (int i = threadIdx.x; i < L; i += blockDim.x)
        build_axis_entry(i, L, g, Sh.s, Sh.vscale, DELJ, v, Sh.beta1);
    const long l0 = (long)blockIdx.x * nt;
    const int n = (int)min((long)nt, A.nlines - l0);
    nd_tile_io(A, tile, nt, l0, n, false);
    __syncthreads();
    nd_solve_tile<DELJ>(A, tile, gam, nt, l0, n, g, v, Sh.s, Sh.inj);
    __syncthreads();
    nd_tile_io(A, tile, nt, l0, n, true);
}

// Per-step coefficient records of a chunk of steps: one CTA per (step,
// axis) runs the setup k_sweep_nd repeats in every CTA -- grid constants,
// the parameter row, the per-axis vectors -- once, and stores it (layout in
// dgb_nd.cuh).  The CTA of the chunk's first step and first swept axis also
// stores the grid constants.  Same functions, same arithmetic: the sweeps
// that read the records compute what k_sweep_nd computes.
template <bool DELJ>
__global__ void k_coef_nd(NDArgs A, long step0, int frozen_mask, int active, double *coef)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ NDShared Sh;
    const int P = A.ndim, L = A.L;
    const int ax = (int)(blockIdx.x % P);
    const long sl = blockIdx.x / P;
    if (frozen_mask >> ax & 1)
        return; // the whole CTA: no barrier is skipped by part of it
    int first = 0;
    while (frozen_mask >> first & 1)
        first++;
    GridVecs g;
    g.x = smem;
    g.xv = smem + L;
    g.dfac = smem + 2 * L;
    g.xInt = smem + 3 * L;
    g.ih = smem + 4 * L;
    g.dx = smem + 5 * L;
    NDArgs B = A;
    B.axis = ax;
    B.step = step0 + sl;
    B.inject_mask = (ax == first) ? active : 0;
    nd_grid_consts(B, g);
    if (threadIdx.x == 0)
        nd_load_params(B, Sh, g);
    __syncthreads();
    double *rec = coef + nd_grid_doubles(L) + ((size_t)sl * P + ax) * nd_rec_doubles(L, DELJ);
    AxisVecs v;
    nd_vecs_at(rec + ND_HEAD, L, DELJ, v);
    for (int i = threadIdx.x; i < L; i += blockDim.x)
        build_axis_entry(i, L, g, Sh.s, Sh.vscale, DELJ, v, Sh.beta1);
    if (threadIdx.x == 0) {
        NDRecHead h;
        h.s = Sh.s;
        for (int k = 0; k < DGB_MAX_DIM; k++)
            h.inj[k] = Sh.inj[k];
        const double *hp = reinterpret_cast<const double *>(&h);
        for (int k = 0; k < ND_HEAD; k++)
            rec[k] = hp[k];
    }
    if (sl == 0 && ax == first)
        for (int i = threadIdx.x; i < nd_grid_doubles(L); i += blockDim.x)
            coef[i] = smem[i];
}

// Sweep that reads its step's coefficients from the records of k_coef_nd:
// one coalesced copy of O(L) doubles per CTA instead of the FP64 setup.
template <bool DELJ>
__global__ void k_sweep_nd_rec(NDArgs A, const double *coef, long step0)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ NDRecHead H;
    const int nt = blockDim.x, L = A.L, P = A.ndim;
    constexpr int NV = DELJ ? 10 : 5;
    double *tile = smem;
    double *gam = tile + (size_t)L * (nt + 1);
    double *gx = gam + (size_t)L * nt; // x, xInt, dx
    double *vv = gx + 3 * (size_t)L;
    const double *rec =
        coef + nd_grid_doubles(L) + ((size_t)(A.step - step0) * P + A.axis) * nd_rec_doubles(L, DELJ);
    double *hp = reinterpret_cast<double *>(&H);
    for (int i = threadIdx.x; i < ND_HEAD; i += nt)
        hp[i] = rec[i];
    for (int i = threadIdx.x; i < NV * L; i += nt)
        vv[i] = rec[ND_HEAD + i];
    for (int i = threadIdx.x; i < L; i += nt) {
        gx[i] = coef[i];
        if (DELJ) {
            gx[L + i] = coef[3 * L + i];
            gx[2 * L + i] = coef[5 * L + i];
        }
    }
    GridVecs g = {};
    g.x = gx;
    g.xInt = gx + L;
    g.dx = gx + 2 * L;
    AxisVecs v;
    nd_vecs_at(vv, L, DELJ, v);
    const long l0 = (long)blockIdx.x * nt;
    const int n = (int)min((long)nt, A.nlines - l0);
    nd_tile_io(A, tile, nt, l0, n, false);
    __syncthreads();
    nd_solve_tile<DELJ>(A, tile, gam, nt, l0, n, g, v, H.s, H.inj);
    __syncthreads();
    nd_tile_io(A, tile, nt, l0, n, true);
}

// Constant-coefficient sweep (reference arithmetic: b = bx + 1/dt,
// r = (1/dt)*phi), coefficients read straight from the a/b/c arrays.
__global__ void k_precalc_nd(NDArgs A)
{
    extern __shared__ __align__(16) double smem[];
    const int nt = blockDim.x, L = A.L, P = A.ndim, ax = A.axis;
    double *tile = smem, *gam = smem + (size_t)L * (nt + 1);
    const int tp = nt + 1;
    const long l0 = (long)blockIdx.x * nt;
    const int n = (int)min((long)nt, A.nlines - l0);
    const double dt = A.dts ? A.dts[A.step] : A.dt;
    const double idt = 1 / dt;
    nd_tile_io(A, tile, nt, l0, n, false);
    __syncthreads();
    const int t = threadIdx.x;
    if (t < n) {
        int coord[DGB_MAX_DIM];
        long base = nd_line_base(A, l0 + t, coord);
        if (A.inject_mask) {
            int n1 = 0, k1 = -1;
            for (int k = 0; k < P; k++) {
                if (k == ax)
                    continue;
                if (coord[k] == 1) {
                    n1++;
                    k1 = k;
                } else if (coord[k] != 0) {
                    n1 = 99;
                }
            }
            double val = inject_value(P, dt, A.theta0, A.xx[0], A.xx[1], A.xx[2]);
            if (n1 == 0 && (A.inject_mask >> ax & 1))
                tile[1 * tp + t] += val;
            if (n1 == 1 && (A.inject_mask >> k1 & 1))
                tile[0 * tp + t] += val;
        }
        double *ph = tile + t;
        double *gm = gam + t;
        const double *a = A.ca + base, *b = A.cb + base, *c = A.cc + base;
        const long S = A.S;
        double bet = b[0] + idt;
        double inv = rcp_full(bet);
        double u = (idt * ph[0]) * inv;
        ph[0] = u;
        for (int i = 1; i < L; i++) {
            double gg = c[(i - 1) * S] * inv;
            gm[i * nt] = gg;
            double ai = a[i * S];
            bet = fma(-ai, gg, b[i * S] + idt);
            inv = rcp_full(bet);
            u = fma(-ai, u, idt * ph[i * tp]) * inv;
            ph[i * tp] = u;
        }
        for (int i = L - 2; i >= 0; i--) {
            u = fma(-gm[(i + 1) * nt], u, ph[i * tp]);
            ph[i * tp] = u;
        }
    }
    __syncthreads();
    nd_tile_io(A, tile, nt, l0, n, true);
}

__global__ void k_tridiag_batch(const double *a, const double *b, const double *c,
                                const double *r, double *u, double *gam, int n, int batch)
{
    long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= batch)
        return;
    const double *as = a + s * n, *bs = b + s * n, *cs = c + s * n, *rs = r + s * n;
    double *us = u + s * n, *gs = gam + s * n;
    double bet = bs[0];
    double inv = rcp_full(bet);
    us[0] = rs[0] * inv;
    for (int j = 1; j < n; j++) {
        gs[j] = cs[j - 1] * inv;
        bet = fma(-as[j], gs[j], bs[j]);
        inv = rcp_full(bet);
        us[j] = fma(-as[j], us[j - 1], rs[j]) * inv;
    }
    for (int j = n - 2; j >= 0; j--)
        us[j] = fma(-gs[j + 1], us[j + 1], us[j]);
}

static int nd_launch_sweep(NDArgs &A, bool delj, cudaStream_t st)
{
    int nt = nd_threads(A.L, A.nlines);
    size_t smem = nd_smem_doubles(A.L, nt, delj) * sizeof(double);
    long nblocks = (A.nlines + nt - 1) / nt;
    cudaError_t e;
    (void)e;
    if (delj) {
        if (raise_smem_limit(k_sweep_nd<true>))
            return DGB_ERR_CUDA;
        k_sweep_nd<true><<<(unsigned)nblocks, nt, smem, st>>>(A);
    } else {
        if (raise_smem_limit(k_sweep_nd<false>))
            return DGB_ERR_CUDA;
        k_sweep_nd<false><<<(unsigned)nblocks, nt, smem, st>>>(A);
    }
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

static int nd_launch_precalc(NDArgs &A, cudaStream_t st)
{
    int nt = nd_threads(A.L, A.nlines);
    size_t smem = ((size_t)A.L * (nt + 1) + (size_t)A.L * nt) * sizeof(double);
    long nblocks = (A.nlines + nt - 1) / nt;
    if (raise_smem_limit(k_precalc_nd))
        return DGB_ERR_CUDA;
    k_precalc_nd<<<(unsigned)nblocks, nt, smem, st>>>(A);
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}


int nd_sweep(NDArgs &A, bool delj, cudaStream_t st) { return nd_launch_sweep(A, delj, st); }

int nd_coef_chunk(const NDArgs &A, bool delj, long step0, int n, int frozen_mask, int active,
                  double *coef, cudaStream_t st)
{
    if (n < 1 || n > nd_chunk_steps(A.ndim, A.L) || !A.table)
        return DGB_ERR_ARG;
    const size_t smem = (size_t)nd_grid_doubles(A.L) * sizeof(double);
    const unsigned grid = (unsigned)(n * A.ndim);
    if (delj) {
        if (raise_smem_limit(k_coef_nd<true>))
            return DGB_ERR_CUDA;
        k_coef_nd<true><<<grid, 128, smem, st>>>(A, step0, frozen_mask, active, coef);
    } else {
        if (raise_smem_limit(k_coef_nd<false>))
            return DGB_ERR_CUDA;
        k_coef_nd<false><<<grid, 128, smem, st>>>(A, step0, frozen_mask, active, coef);
    }
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

int nd_sweep_rec(NDArgs &A, bool delj, const double *coef, long step0, cudaStream_t st)
{
    const int nt = nd_threads(A.L, A.nlines);
    const size_t smem = nd_rec_smem_doubles(A.L, nt, delj) * sizeof(double);
    const long nblocks = (A.nlines + nt - 1) / nt;
    if (delj) {
        if (raise_smem_limit(k_sweep_nd_rec<true>))
            return DGB_ERR_CUDA;
        k_sweep_nd_rec<true><<<(unsigned)nblocks, nt, smem, st>>>(A, coef, step0);
    } else {
        if (raise_smem_limit(k_sweep_nd_rec<false>))
            return DGB_ERR_CUDA;
        k_sweep_nd_rec<false><<<(unsigned)nblocks, nt, smem, st>>>(A, coef, step0);
    }
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

} // namespace dgb

using namespace dgb;

// ------------------------------------------------------------------ C ABI

extern "C" int dgb_abi_version(void) { return 1; }

extern "C" const char *dgb_status_string(int status)
{
    switch (status) {
    case DGB_OK:
        return "ok";
    case DGB_ERR_ARG:
        return "invalid argument";
    case DGB_ERR_CUDA:
        return "CUDA error";
    case DGB_ERR_UNSUPPORTED:
        return "unsupported size or mode";
    case DGB_ERR_WORKSPACE:
        return "workspace missing or too small";
    case DGB_ERR_TOO_LARGE:
        return "grid larger than the allocation-free entry point's static scratch "
               "(L > DGB_NOALLOC_MAX_L)";
    default:
        return "unknown status";
    }
}

extern "C" size_t dgb_workspace_bytes(int kind, int ndim, int L, long n)
{
    if (kind == 0) {
        // the shared-memory 2-D integrator's scratch, or the coefficient
        // records of the per-axis sweeps
        if (ndim == 2 && k2_smem_fits(L, false, true, nullptr))
            return k2_table_ws_bytes(L);
        return std::max(ndim == 2 ? k2_table_ws_bytes(L) : (size_t)0, nd_coef_bytes(ndim, L));
    }
    if (kind == 1)
        return k2_batch_ws_bytes(L, n);
    if (kind == 2)
        return (size_t)n * L * sizeof(double);
    if (kind == 3) // any gam placement: a slice per work item
        return 256 + (size_t)n * L * L * sizeof(double);
    if (kind == 4) // recomputed intermediate densities + coefficient records
        return (size_t)std::max(ndim - 1, 1) * ipow(L, ndim) * sizeof(double) +
               nd_coef_bytes(ndim, L);
    return 0;
}

extern "C" int dgb_tridiag_batch(const double *a, const double *b, const double *c,
                                 const double *r, double *u, int n, int batch, void *ws,
                                 size_t ws_bytes, void *stream)
{
    if (!a || !b || !c || !r || !u || n < 1 || batch < 0)
        return DGB_ERR_ARG;
    if (batch == 0)
        return DGB_OK;
    if (!ws || ws_bytes < (size_t)n * batch * sizeof(double))
        return DGB_ERR_WORKSPACE;
    int nt = 128;
    k_tridiag_batch<<<(batch + nt - 1) / nt, nt, 0, (cudaStream_t)stream>>>(a, b, c, r, u,
                                                                          (double *)ws, n, batch);
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

extern "C" int dgb_implicit_sweep(double *phi, int ndim, int L, int axis, const double *xx,
                                  double nu, const double *mig, double gamma, double h,
                                  double beta, double dt, int use_delj_trick, void *ws,
                                  size_t ws_bytes, void *stream)
{
    (void)ws;
    (void)ws_bytes;
    if (!phi || !xx || !shape_ok(ndim, L) || axis < 0 || axis >= ndim || (ndim > 1 && !mig))
        return DGB_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    NDArgs A = {};
    nd_fill(A, phi, ndim, L, axis, xx);
    A.nu = nu;
    A.gamma = gamma;
    A.h = h;
    A.beta = beta;
    A.dt = dt;
    for (int k = 0; k < ndim; k++)
        A.mig[k] = (ndim > 1) ? mig[k] : 0.0;
    return nd_launch_sweep(A, use_delj_trick != 0, st);
}

extern "C" int dgb_implicit_precalc_sweep(double *phi, int ndim, int L, int axis,
                                          const double *a, const double *b, const double *c,
                                          double dt, void *ws, size_t ws_bytes, void *stream)
{
    (void)ws;
    (void)ws_bytes;
    if (!phi || !a || !b || !c || !shape_ok(ndim, L) || axis < 0 || axis >= ndim)
        return DGB_ERR_ARG;
    NDArgs A = {};
    nd_fill(A, phi, ndim, L, axis, nullptr);
    A.ca = a;
    A.cb = b;
    A.cc = c;
    A.dt = dt;
    return nd_launch_precalc(A, (cudaStream_t)stream);
}

extern "C" int dgb_integrate_table(double *phi, int ndim, int L, const double *xx,
                                   const double *table, int nsteps, int frozen_mask,
                                   int nomut_mask, int use_delj_trick, void *ws,
                                   size_t ws_bytes, void *stream)
{
    if (!phi || !xx || !table || !shape_ok(ndim, L) || nsteps < 0)
        return DGB_ERR_ARG;
    if (nsteps == 0)
        return DGB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (ndim == 2 && k2_smem_fits(L, false, use_delj_trick != 0, nullptr))
        return k2_integrate_table(phi, L, xx, table, nsteps, frozen_mask, nomut_mask,
                                  use_delj_trick, ws, ws_bytes, st);
    const int active = ((1 << ndim) - 1) & ~frozen_mask & ~nomut_mask;
    const bool delj = use_delj_trick != 0;
    NDArgs A = {};
    nd_fill(A, phi, ndim, L, 0, xx);
    int rc = DGB_OK;
    A.table = table;
    // with room for them in the workspace, each chunk of steps gets its
    // coefficient records from one launch, and the sweeps only read them
    double *coef = (ws && ws_bytes >= nd_coef_bytes(ndim, L)) ? (double *)ws : nullptr;
    const int chunk = nd_chunk_steps(ndim, L);
    long step0 = 0;
    for (long s = 0; s < nsteps; s++) {
        if (coef && s % chunk == 0) {
            step0 = s;
            rc = nd_coef_chunk(A, delj, s, (int)std::min<long>(chunk, nsteps - s), frozen_mask,
                               active, coef, st);
            if (rc)
                return rc;
        }
        bool first = true;
        for (int ax = 0; ax < ndim; ax++) {
            if (frozen_mask >> ax & 1)
                continue;
            A.axis = ax;
            A.S = ipow(L, ndim - 1 - ax);
            A.LS = A.S * L;
            A.step = s;
            A.inject_mask = first ? active : 0;
            first = false;
            rc = coef ? nd_sweep_rec(A, delj, coef, step0, st) : nd_launch_sweep(A, delj, st);
            if (rc)
                return rc;
        }
    }
    return DGB_OK;
}

extern "C" int dgb_integrate_precalc(double *phi, int ndim, int L, const double *xx,
                                     const double *abc, const double *dts, int nsteps,
                                     double theta0, int frozen_mask, int nomut_mask, void *ws,
                                     size_t ws_bytes, void *stream)
{
    (void)ws;
    (void)ws_bytes;
    if (!phi || !xx || !abc || !dts || !shape_ok(ndim, L) || nsteps < 0)
        return DGB_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const int active = ((1 << ndim) - 1) & ~frozen_mask & ~nomut_mask;
    const long n = ipow(L, ndim);
    NDArgs A = {};
    nd_fill(A, phi, ndim, L, 0, xx);
    A.dts = dts;
    A.theta0 = theta0;
    for (long s = 0; s < nsteps; s++) {
        bool first = true;
        for (int ax = 0; ax < ndim; ax++) {
            if (frozen_mask >> ax & 1)
                continue;
            A.axis = ax;
            A.S = ipow(L, ndim - 1 - ax);
            A.LS = A.S * L;
            A.step = s;
            A.ca = abc + (3 * ax + 0) * n;
            A.cb = abc + (3 * ax + 1) * n;
            A.cc = abc + (3 * ax + 2) * n;
            A.inject_mask = first ? active : 0;
            first = false;
            int rc = nd_launch_precalc(A, st);
            if (rc)
                return rc;
        }
    }
    return DGB_OK;
}

namespace dgb {
int preload_sweepnd()
{
    return preload(k_sweep_nd<false>) + preload(k_sweep_nd<true>) + preload(k_coef_nd<false>) +
           preload(k_coef_nd<true>) + preload(k_sweep_nd_rec<false>) +
           preload(k_sweep_nd_rec<true>) + preload(k_precalc_nd) + preload(k_tridiag_batch);
}
} // namespace dgb
