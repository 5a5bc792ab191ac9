// Shared-memory-resident 2-D integrator.
//
// One CTA owns one (instance, grid) work item for the whole time loop: phi
// (L x L doubles, row pitch L|1 so both sweep directions are bank-conflict
// free) is loaded once into shared memory, every step injects mutations,
// rebuilds the per-axis coefficient vectors and runs the x sweep (lines are
// columns) and the y sweep (lines are rows) with one thread per line, and
// phi is written back once at the end.  The Thomas gam scratch lives in
// shared memory when it fits next to phi, otherwise in a per-CTA slice of a
// global workspace (L2-resident).
//
// Two schedules feed the same kernel: a host-evaluated parameter table (the
// drop-in path for arbitrary Python callables) or the parametric forms of
// dgb_inst2d evaluated on the device (the batched engine, a persistent launch
// that pulls work items from an atomic counter in longest-first order).
//
// Reference: the time loop of Integration.two_pops (dadi/Integration.py:
// 340-386) with implicit_2Dx / implicit_2Dy (dadi/integration2D.c:19-160).
#include <algorithm>
#include <vector>

#include "dgb_common.cuh"
#include "dgb_internal.h"

namespace dgb {

constexpr int K2_THREADS = 128;
constexpr int K2_MAXG = DGB_B2_MAXG;

struct K2Args {
    // work description
    const dgb_inst2d *insts; // parametric mode (null in table mode)
    const double *table;     // table mode: nsteps rows of stride 11
    int nsteps;
    int frozen_mask, nomut_mask; // table mode
    int ngrids;
    int L[K2_MAXG];
    long xx_off[K2_MAXG];
    long phi0_off[K2_MAXG];
    long out_off[K2_MAXG];
    const double *xx_all;
    const double *phi0_all; // null: phi_out holds the initial density
    double *phi_out;
    const int *order;
    int nwork;
    int *counter;
    int *status;
    long max_steps;
    dgb_settings settings;
    int Lmax;
    int gam_smem;     // 1: gam in shared memory
    double *gam_glob; // per-CTA slices of Lmax*Lmax doubles
    int use_delj;
};

// Shared-memory layout for a given Lmax.
struct K2Layout {
    int pitch;     // row pitch of phi (odd)
    size_t phi, gam, grid, vec, total;
};

__host__ __device__ inline int odd_pitch(int L) { return (L % 2) ? L : L + 1; }

static K2Layout k2_layout(int Lmax, bool gam_smem, bool delj)
{
    K2Layout l;
    l.pitch = odd_pitch(Lmax);
    l.phi = (size_t)Lmax * l.pitch;
    l.gam = gam_smem ? (size_t)Lmax * Lmax : 0;
    l.grid = 6 * (size_t)Lmax;
    l.vec = 2 * (size_t)(delj ? 10 : 5) * Lmax;
    l.total = (l.phi + l.gam + l.grid + l.vec) * sizeof(double);
    return l;
}

struct K2Shared {
    AxisScalars ax[2];
    double theta0;
    double cur_t, T;
    double p_nu[2], p_m[2], p_g[2], p_h[2]; // params at the current time
    int item, last, err;
    long step;
};

__device__ __forceinline__ void k2_carve(double *smem, int Lmax, int pitch, bool gam_smem,
                                         bool delj, double *&phi, double *&gam,
                                         GridVecs &g, AxisVecs (&v)[2])
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

// One step's scalars for both axes from (dt, theta0, nu, m, gamma, h).
__device__ void k2_set_axes(K2Shared &S, const GridVecs &g, int L, double dt, double theta0,
                            const double *nu, const double *m, const double *gam,
                            const double *h)
{
    S.theta0 = theta0;
    for (int a = 0; a < 2; a++) {
        AxisScalars &s = S.ax[a];
        s.dt = dt;
        s.nu = nu[a];
        s.inv_nu = 1.0 / nu[a];
        s.msum = m[a];
        s.gamma = gam[a];
        s.h = h[a];
        s.mig[0] = s.mig[1] = 0;
        s.mig[1 - a] = m[a];
        s.B1s = 0.5 * (dt * g.dfac[0]);
        s.B1e = -0.5 * (dt * g.dfac[L - 1]);
        corner_bc(2, a, s.mig, s.nu, s.gamma, s.h, g.x[0], g.x[L - 1], g.dx[0], g.dx[L - 2],
                  dt, s.bcs, s.bce);
    }
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
    const bool table_mode = (A.insts == nullptr);

    // Shared flags written by thread 0 are only read between the barrier
    // that follows the write and the next barrier thread 0 must pass before
    // writing again.
    for (int iter = 0;; iter++) {
        if (tid == 0)
            S.item = table_mode ? (iter == 0 ? 0 : A.nwork) : atomicAdd(A.counter, 1);
        __syncthreads();
        const int w = S.item;
        if (w >= A.nwork)
            break;
        const int wid = table_mode ? 0 : A.order[w];
        const int inst = table_mode ? 0 : wid / A.ngrids;
        const int gi = table_mode ? 0 : wid % A.ngrids;
        const int L = A.L[gi];
        const double *xx = A.xx_all + A.xx_off[gi];
        double *out = A.phi_out + A.out_off[gi] + (size_t)inst * L * L;
        const double *src = A.phi0_all ? A.phi0_all + A.phi0_off[gi] : out;

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
        const int frozen = table_mode ? A.frozen_mask : A.insts[inst].frozen_mask;
        const int nomut = table_mode ? A.nomut_mask : A.insts[inst].nomut_mask;
        if (tid == 0) {
            S.last = 0;
            S.err = 0;
            S.step = 0;
            if (!table_mode) {
                const dgb_inst2d &I = A.insts[inst];
                S.cur_t = I.initial_t;
                S.T = I.T;
                for (int k = 0; k < 2; k++) {
                    S.p_nu[k] = pform_eval(I.nu[k], S.cur_t);
                    S.p_g[k] = pform_eval(I.gamma[k], S.cur_t);
                    S.p_h[k] = pform_eval(I.h[k], S.cur_t);
                }
                S.p_m[0] = pform_eval(I.m12, S.cur_t);
                S.p_m[1] = pform_eval(I.m21, S.cur_t);
                S.last = !(S.cur_t < S.T);
            } else {
                S.last = (A.nsteps <= 0);
            }
        }
        __syncthreads();
        bool more = !S.last;
        // grid index of the corner lines (other coordinate exactly 0 / 1)
        const int j0 = (g.x[0] == 0.0) ? 0 : -1;
        const int j1 = (g.x[L - 1] == 1.0) ? L - 1 : -1;
        __syncthreads();

        while (more) {
            // ---- schedule: this step's parameters (one thread)
            if (tid == 0) {
                double dt, theta0, nu[2], m[2], ga[2], hh[2];
                if (table_mode) {
                    const double *row = A.table + (size_t)S.step * 11;
                    dt = row[0];
                    theta0 = row[1];
                    for (int k = 0; k < 2; k++) {
                        nu[k] = row[row_nu(2, k)];
                        ga[k] = row[row_gamma(2, k)];
                        hh[k] = row[row_h(2, k)];
                    }
                    m[0] = row[row_mig(2, 0, 1)];
                    m[1] = row[row_mig(2, 1, 0)];
                    S.last = (S.step + 1 >= A.nsteps);
                } else {
                    const dgb_inst2d &I = A.insts[inst];
                    double dx0 = g.dx[0];
                    double d0 = compute_dt(S.p_nu[0], S.p_m[0], S.p_g[0], S.p_h[0], A.settings, dx0);
                    double d1 = compute_dt(S.p_nu[1], S.p_m[1], S.p_g[1], S.p_h[1], A.settings, dx0);
                    double dtm = pymin(d0, d1);
                    dt = pymin(dtm, S.T - S.cur_t);
                    double next_t = S.cur_t + dt;
                    for (int k = 0; k < 2; k++) {
                        nu[k] = pform_eval(I.nu[k], next_t);
                        ga[k] = pform_eval(I.gamma[k], next_t);
                        hh[k] = pform_eval(I.h[k], next_t);
                        S.p_nu[k] = nu[k];
                        S.p_g[k] = ga[k];
                        S.p_h[k] = hh[k];
                    }
                    m[0] = pform_eval(I.m12, next_t);
                    m[1] = pform_eval(I.m21, next_t);
                    S.p_m[0] = m[0];
                    S.p_m[1] = m[1];
                    theta0 = pform_eval(I.theta0, next_t);
                    int err = 0;
                    if (dtm == 0)
                        err |= DGB_ST_ZERODT;
                    if (S.T < 0 || nu[0] < 0 || nu[1] < 0 || m[0] < 0 || m[1] < 0 || theta0 < 0 ||
                        nu[0] == 0 || nu[1] == 0)
                        err |= DGB_ST_BADPARAM;
                    if (!isfinite(dt) || !isfinite(next_t))
                        err |= DGB_ST_NONFINITE;
                    S.cur_t = next_t;
                    S.last = !(S.cur_t < S.T);
                    if (S.step + 1 >= A.max_steps && !S.last)
                        err |= DGB_ST_STEPCAP;
                    S.err = err;
                }
                k2_set_axes(S, g, L, dt, theta0, nu, m, ga, hh);
            }
            __syncthreads();
            const bool last = S.last;
            if (S.err)
                break; // uniform: every thread read the same S.err
            // ---- per-axis vectors (both axes) and mutation injection
            for (int t = tid; t < 2 * L; t += blockDim.x) {
                int a = t >= L, i = t - a * L;
                build_axis_entry(i, L, g, S.ax[a], 1.0, DELJ, v[a]);
            }
            if (tid == 0) {
                double val = inject_value(2, S.ax[0].dt, S.theta0, g.x[0], g.x[1], g.x[2]);
                if (!(frozen & 1) && !(nomut & 1))
                    phi[1 * pitch + 0] += val;
                if (!(frozen & 2) && !(nomut & 2))
                    phi[0 * pitch + 1] += val;
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
                const int lpw = (L + nwarps - 1) / nwarps;
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
                            solve_line_delj(ph, sp, gm, L, L, &s.mig[1 - a], &g.x[line], 1, bs, be, g, v[a]);
                        else
                            solve_line(ph, sp, gm, L, L, W, bs, be, v[a], s);
                    } else {
                        double *gm = gam_g + line;
                        if (DELJ)
                            solve_line_delj(ph, sp, gm, L, L, &s.mig[1 - a], &g.x[line], 1, bs, be, g, v[a]);
                        else
                            solve_line(ph, sp, gm, L, L, W, bs, be, v[a], s);
                    }
                }
                __syncthreads();
            }
            if (tid == 0)
                S.step++;
            more = !last;
        }
        __syncthreads();
        // ---- write back (also on error, so callers can inspect)
        if (!table_mode && tid == 0 && S.err)
            atomicOr(A.status + inst, S.err);
        for (int idx = tid; idx < L * L; idx += blockDim.x) {
            int r = idx / L, c = idx - r * L;
            out[idx] = phi[r * pitch + c];
        }
        __syncthreads();
    }
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

static int k2_launch(K2Args &A, int nblocks, size_t smem, cudaStream_t st)
{
    cudaError_t e;
    if (A.use_delj) {
        e = cudaFuncSetAttribute(k_integrate2d<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess)
            return DGB_ERR_CUDA;
        k_integrate2d<true><<<nblocks, K2_THREADS, smem, st>>>(A);
    } else {
        e = cudaFuncSetAttribute(k_integrate2d<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess)
            return DGB_ERR_CUDA;
        k_integrate2d<false><<<nblocks, K2_THREADS, smem, st>>>(A);
    }
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

// Blocks per SM the kernel can keep resident with this dynamic smem.
static int k2_occupancy(bool delj, size_t smem)
{
    int nb = 0;
    cudaError_t e = delj ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                               &nb, k_integrate2d<true>, K2_THREADS, smem)
                         : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                               &nb, k_integrate2d<false>, K2_THREADS, smem);
    return (e == cudaSuccess && nb > 0) ? nb : 1;
}

int k2_integrate_table(double *phi, int L, const double *xx, const double *table, int nsteps,
                       int frozen_mask, int nomut_mask, int use_delj, void *ws, size_t ws_bytes,
                       cudaStream_t st)
{
    K2Args A = {};
    A.table = table;
    A.nsteps = nsteps;
    A.frozen_mask = frozen_mask;
    A.nomut_mask = nomut_mask;
    A.ngrids = 1;
    A.L[0] = L;
    A.xx_all = xx;
    A.phi_out = phi;
    A.nwork = 1;
    A.Lmax = L;
    A.use_delj = use_delj;
    size_t bytes;
    A.gam_smem = k2_smem_fits(L, true, use_delj, &bytes);
    if (!A.gam_smem) {
        if (!k2_smem_fits(L, false, use_delj, &bytes))
            return DGB_ERR_UNSUPPORTED;
        size_t need = (size_t)L * L * sizeof(double);
        if (!ws || ws_bytes < need)
            return DGB_ERR_WORKSPACE;
        A.gam_glob = (double *)ws;
    }
    cudaFuncAttributes fa;
    (void)fa;
    return k2_launch(A, 1, bytes, st);
}

size_t k2_table_ws_bytes(int L) { return (size_t)L * L * sizeof(double); }

size_t k2_batch_ws_bytes(int Lmax, long nwork)
{
    // counter (256 B) + per-CTA gam slices for the worst case
    int dev = 0, nsm = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    (void)nwork;
    return 256 + (size_t)nsm * 4 * Lmax * Lmax * sizeof(double);
}

int k2_batch(const dgb_inst2d *insts, int ninst, const int *Ls, int ngrids, const double *xx_all,
             const double *phi0_all, double *phi_out, const int *order, int *status,
             long max_steps, const dgb_settings *settings, void *ws, size_t ws_bytes,
             cudaStream_t st)
{
    if (ngrids < 1 || ngrids > K2_MAXG || ninst < 1)
        return DGB_ERR_ARG;
    K2Args A = {};
    A.insts = insts;
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
    A.order = order;
    A.nwork = ninst * ngrids;
    A.status = status;
    A.max_steps = max_steps;
    A.settings = *settings;
    A.Lmax = Lmax;
    A.use_delj = settings->use_delj_trick;
    if (!ws || ws_bytes < 256)
        return DGB_ERR_WORKSPACE;
    A.counter = (int *)ws;
    size_t bytes_s = 0, bytes_g = 0;
    bool fit_s = k2_smem_fits(Lmax, true, A.use_delj, &bytes_s);
    bool fit_g = k2_smem_fits(Lmax, false, A.use_delj, &bytes_g);
    if (!fit_g)
        return DGB_ERR_UNSUPPORTED;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    // Choose gam placement: shared if it keeps at least as many CTAs per SM
    // resident as the global variant would (the workspace bounds the latter).
    int occ_s = fit_s ? k2_occupancy(A.use_delj, bytes_s + sizeof(K2Shared)) : 0;
    int occ_g = k2_occupancy(A.use_delj, bytes_g + sizeof(K2Shared));
    size_t slice = (size_t)Lmax * Lmax * sizeof(double);
    int max_g_blocks = (int)std::min<size_t>((ws_bytes - 256) / slice, (size_t)nsm * occ_g);
    int nblocks;
    size_t smem;
    bool use_s = fit_s && (occ_s * nsm >= max_g_blocks || max_g_blocks < nsm);
    if (settings->gam_placement == 1) {
        if (!fit_s)
            return DGB_ERR_UNSUPPORTED;
        use_s = true;
    } else if (settings->gam_placement == 2) {
        use_s = false;
    }
    if (use_s) {
        A.gam_smem = 1;
        nblocks = nsm * occ_s;
        smem = bytes_s;
    } else {
        A.gam_smem = 0;
        A.gam_glob = (double *)((char *)ws + 256);
        nblocks = max_g_blocks;
        smem = bytes_g;
    }
    if (nblocks < 1)
        return DGB_ERR_WORKSPACE;
    nblocks = std::min(nblocks, A.nwork);
    if (cudaMemsetAsync(A.counter, 0, sizeof(int), st) != cudaSuccess)
        return DGB_ERR_CUDA;
    return k2_launch(A, nblocks, smem, st);
}

} // namespace dgb

// ------------------------------------------------------------------ C ABI

extern "C" int dgb_batch2d_integrate(const dgb_inst2d *insts, int ninst, const int *Ls,
                                     int ngrids, const double *xx_all, const double *phi0_all,
                                     double *phi_out, const int *order, int *status,
                                     long max_steps, const dgb_settings *settings, void *ws,
                                     size_t ws_bytes, void *stream)
{
    if (!insts || !Ls || !xx_all || !phi0_all || !phi_out || !order || !status || !settings ||
        max_steps < 1)
        return DGB_ERR_ARG;
    return dgb::k2_batch(insts, ninst, Ls, ngrids, xx_all, phi0_all, phi_out, order, status,
                         max_steps, settings, ws, ws_bytes, (cudaStream_t)stream);
}

extern "C" int dgb_batch2d_count_steps(const dgb_inst2d *insts, int ninst,
                                       const dgb_settings *settings, long max_steps,
                                       long *steps_out)
{
    if (!insts || !settings || !steps_out || ninst < 0)
        return DGB_ERR_ARG;
    for (int n = 0; n < ninst; n++) {
        const dgb_inst2d &I = insts[n];
        double t = I.initial_t;
        double nu0 = dgb::pform_eval(I.nu[0], t), nu1 = dgb::pform_eval(I.nu[1], t);
        double m0 = dgb::pform_eval(I.m12, t), m1 = dgb::pform_eval(I.m21, t);
        double g0 = dgb::pform_eval(I.gamma[0], t), g1 = dgb::pform_eval(I.gamma[1], t);
        double h0 = dgb::pform_eval(I.h[0], t), h1 = dgb::pform_eval(I.h[1], t);
        long steps = 0;
        while (t < I.T && steps < max_steps) {
            double d = dgb::pymin(dgb::compute_dt(nu0, m0, g0, h0, *settings, 1e-3),
                                  dgb::compute_dt(nu1, m1, g1, h1, *settings, 1e-3));
            double dt = dgb::pymin(d, I.T - t);
            if (!(dt > 0) || !std::isfinite(dt))
                break;
            t = t + dt;
            nu0 = dgb::pform_eval(I.nu[0], t);
            nu1 = dgb::pform_eval(I.nu[1], t);
            m0 = dgb::pform_eval(I.m12, t);
            m1 = dgb::pform_eval(I.m21, t);
            g0 = dgb::pform_eval(I.gamma[0], t);
            g1 = dgb::pform_eval(I.gamma[1], t);
            h0 = dgb::pform_eval(I.h[0], t);
            h1 = dgb::pform_eval(I.h[1], t);
            steps++;
        }
        steps_out[n] = steps;
    }
    return DGB_OK;
}
