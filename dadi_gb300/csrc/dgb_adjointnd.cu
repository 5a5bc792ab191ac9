// Discrete adjoint of the N-dimensional table-driven time loop (1 to 4
// populations; the per-axis ADI steps of dadi/Integration.py:178-727 with
// the sweeps of dadi/integration{1,2,3,4}D.c).
//
// One forward step is psi = phi_k + inj_k (dadi/Integration.py:70-122),
// s_1 = X_1^{-1} psi, s_2 = X_2^{-1} s_1, ..., phi_{k+1} = s_P, where X_j is
// the dt-scaled operator I + dt D_j of the j-th active axis' sweep.  Given
// lambda = dJ/dphi_{k+1}, the step backwards solves the transposed systems in
// reverse axis order, mu_j = X_j^{-T} mu_{j+1} (mu_{P+1} = lambda), and
// contracts each with the derivative of its matrix:
//     dJ/dq += -mu_j^T (dX_j/dq) s_j          (s_0 = psi)
// for every entry q of the step's parameter-table row (dt, nu, m, gamma, h
// of that axis), plus the injection's dependence on dt and theta0.  The
// result is dJ/d(table row) for every step; the caller maps it to model
// parameters with derivatives of the table (the schedule).  The forward
// states phi_k are recorded by dgb_integrate_table_states; the intermediate
// s_j of a step are recomputed from phi_k by the forward sweeps.
//
// The contraction per line follows the coefficient layout of
// compute_abc_nobc (dadi/integration_shared.c:72-93): for the interval
// (i, i+1) with D_i = dfactor_i mu_i - dfactor_{i+1} mu_{i+1} and
// hp = (u_i + u_{i+1})/2, d/dnu contributes D_i (Q_i u_{i+1} - P_i u_i)/nu,
// d/dm_k (the rate into this axis' population from population k)
// D_i (x_k - xInt_i) hp, d/dgamma and d/dh the selection term's
// derivatives times D_i hp; d/ddt is -(mu.r - mu.u)/dt; the corner boundary
// terms of the first/last point of the corner lines add their own.
#include "dgb_nd.cuh"

namespace dgb {

constexpr int ADN_MAXQ = 3 + 3 * DGB_MAX_DIM + DGB_MAX_DIM * (DGB_MAX_DIM - 1);

struct ADNArgs {
    NDArgs nd;          // lam as nd.phi; axis, strides, table row
    const double *out;  // this sweep's forward output s_j
    const double *rhs;  // this sweep's forward input s_{j-1} (psi without injection)
    double *gpart;      // per CTA: row_stride(P) doubles
    const double *coef; // coefficient records of the chunk from step0 (null: build inline)
    long step0;
};

__host__ __device__ inline size_t adn_smem_doubles(int L, int nt)
{
    return nd_smem_doubles(L, nt, false) + 5 * (size_t)L;
}

__global__ void k_adjoint_sweep_nd(ADNArgs A)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ NDShared Sh;
    __shared__ double red[ADN_MAXQ][8];
    const NDArgs &N = A.nd;
    const int nt = blockDim.x, L = N.L, P = N.ndim, ax = N.axis, tid = threadIdx.x;
    const int stride = row_stride(P);
    double *tile, *gam;
    GridVecs g;
    AxisVecs v, vt;
    nd_carve(smem, L, nt, false, tile, gam, g, v);
    double *p = v.B0 + L;
    vt.A1 = p; p += L;
    vt.A0 = p; p += L;
    vt.C1 = p; p += L;
    vt.C0 = p; p += L;
    vt.B0 = p;
    if (A.coef) {
        // the grid constants and this step's record, in the carve order
        const double *rec = A.coef + nd_grid_doubles(L) +
                            ((size_t)(N.step - A.step0) * P + ax) * nd_rec_doubles(L, false);
        constexpr int NS = (int)(sizeof(AxisScalars) / sizeof(double));
        double *sp = reinterpret_cast<double *>(&Sh.s);
        for (int i = tid; i < nd_grid_doubles(L); i += nt)
            g.x[i] = A.coef[i];
        for (int i = tid; i < 5 * L; i += nt)
            v.A1[i] = rec[ND_HEAD + i];
        for (int i = tid; i < ND_HEAD; i += nt) {
            if (i < NS)
                sp[i] = rec[i];
            else
                Sh.inj[i - NS] = rec[i];
        }
    } else {
        nd_grid_consts(N, g);
        if (tid == 0)
            nd_load_params(N, Sh, g);
        __syncthreads();
        for (int i = tid; i < L; i += nt)
            build_axis_entry(i, L, g, Sh.s, Sh.vscale, false, v);
    }
    __syncthreads();
    for (int i = tid; i < L; i += nt) {
        vt.A1[i] = (i > 0) ? v.C1[i - 1] : 0.0;
        vt.A0[i] = (i > 0) ? v.C0[i - 1] : 0.0;
        vt.C1[i] = (i < L - 1) ? v.A1[i + 1] : 0.0;
        vt.C0[i] = (i < L - 1) ? v.A0[i + 1] : 0.0;
        vt.B0[i] = v.B0[i];
    }
    const long l0 = (long)blockIdx.x * nt;
    const int n = (int)min((long)nt, N.nlines - l0);
    nd_tile_io(N, tile, nt, l0, n, false);
    __syncthreads();
    const int j0 = (g.x[0] == 0.0) ? 0 : -1;
    const int j1 = (g.x[L - 1] == 1.0) ? L - 1 : -1;
    const AxisScalars &s = Sh.s;
    double G[ADN_MAXQ];
    for (int q = 0; q < stride; q++)
        G[q] = 0;
    if (tid < n) {
        int coord[DGB_MAX_DIM];
        const long base = nd_line_base(N, l0 + tid, coord);
        double W = 0, oo[DGB_MAX_DIM];
        bool all0 = true, all1 = true;
        int n1 = 0, k1 = -1;
        for (int k = 0; k < P; k++) {
            oo[k] = g.x[coord[k]];
            if (k == ax)
                continue;
            W = fma(s.mig[k], g.x[coord[k]], W);
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
            all0 = all1 = true;
        const double bs = all0 ? s.bcs : 0.0, be = all1 ? s.bce : 0.0;
        const int tp = nt + 1;
        // mu = X^{-T} lambda on this line, in place in the tile
        solve_line(tile + tid, tp, gam + tid, nt, L, W, bs, be, vt, s);
        // contraction with u (forward output) and r (forward input)
        const double *u = A.out + base, *r = A.rhs + base;
        const long S = N.S;
        const double dt = s.dt, inu = s.inv_nu, gm = s.gamma, hh = s.h;
        const double inj0 = (n1 == 1 && k1 >= 0) ? Sh.inj[k1] : 0.0; // point 0 of this line
        const double inj1 = (n1 == 0) ? Sh.inj[ax] : 0.0;             // point 1 of this line
        double smr = 0, smp = 0, snu = 0, sg = 0, sh = 0, sm[DGB_MAX_DIM];
        for (int k = 0; k < P; k++)
            sm[k] = 0;
        double mi = tile[tid], ui = u[0];
        for (int i = 0; i < L; i++) {
            double ri = r[i * S];
            if (i == 0)
                ri += inj0;
            if (i == 1)
                ri += inj1;
            smr = fma(mi, ri, smr);
            smp = fma(mi, ui, smp);
            if (i < L - 1) {
                const double mn = tile[(i + 1) * tp + tid], un = u[(i + 1) * S];
                const double xi = g.xInt[i];
                const double Pi = inu * g.xv[i] * g.ih[i];
                const double Qi = inu * g.xv[i + 1] * g.ih[i];
                const double Di = g.dfac[i] * mi - g.dfac[i + 1] * mn;
                const double hp = 0.5 * (ui + un);
                const double xx1 = xi * (1. - xi);
                snu = fma(Di, (Qi * un - Pi * ui) * inu, snu);
                for (int k = 0; k < P; k++)
                    if (k != ax)
                        sm[k] = fma(Di * (oo[k] - xi), hp, sm[k]);
                sg = fma(Di * (2 * (hh + (1. - 2 * hh) * xi) * xx1), hp, sg);
                sh = fma(Di * (gm * 2 * (1. - 2 * xi) * xx1), hp, sh);
                mi = mn;
                ui = un;
            }
        }
        double bnu = 0, bg = 0, bh = 0, bmf = 0, bml = 0;
        if (bs != 0.0) {
            const double x0 = g.x[0], f = dt * 2. / g.dx[0], w = tile[tid] * u[0];
            bnu += w * f * (-0.5 * inu * inu);
            bmf = w * f * x0;
            bg -= w * f * (2 * (hh + (1. - 2 * hh) * x0) * x0 * (1. - x0));
            bh -= w * f * (gm * 2 * (1. - 2 * x0) * x0 * (1. - x0));
        }
        if (be != 0.0) {
            const double xl = g.x[L - 1], f = dt * 2. / g.dx[L - 2];
            const double w = tile[(L - 1) * tp + tid] * u[(L - 1) * S];
            bnu += w * f * (-0.5 * inu * inu);
            bml = w * f * (1. - xl);
            bg += w * f * (2 * (hh + (1. - 2 * hh) * xl) * xl * (1. - xl));
            bh += w * f * (gm * 2 * (1. - 2 * xl) * xl * (1. - xl));
        }
        G[0] -= (smr - smp) / dt;
        G[row_nu(P, ax)] -= dt * snu + bnu;
        G[row_gamma(P, ax)] -= dt * sg + bg;
        G[row_h(P, ax)] -= dt * sh + bh;
        for (int k = 0; k < P; k++)
            if (k != ax)
                G[row_mig(P, ax, k)] -= dt * sm[k] + bmf + bml;
    }
    __syncthreads();
    nd_tile_io(N, tile, nt, l0, n, true);
    // fixed-order block reduction of G into this CTA's partial row
    const int nw = nt >> 5;
    for (int q = 0; q < stride; q++) {
        double x = G[q];
        for (int off = 16; off > 0; off >>= 1)
            x += __shfl_down_sync(0xffffffffu, x, off);
        if ((tid & 31) == 0)
            red[q][tid >> 5] = x;
    }
    __syncthreads();
    if (tid < stride) {
        double x = 0;
        for (int w = 0; w < nw; w++)
            x += red[tid][w];
        A.gpart[(size_t)blockIdx.x * stride + tid] = x;
    }
}

// Injection's part of dJ/d(dt) and dJ/d(theta0) for one step: lambda (the
// adjoint at the start of the step) at the injected points.
__global__ void k_adjoint_inject_nd(const double *lam, const double *xx, const double *row,
                                    int P, int L, int active, double *gout)
{
    if (threadIdx.x != 0)
        return;
    double lin = 0;
    for (int k = 0; k < P; k++) {
        if (!(active >> k & 1))
            continue;
        long idx = 0;
        for (int j = 0; j < P; j++)
            idx = idx * L + (j == k ? 1 : 0);
        lin += lam[idx];
    }
    const double dt = row[0], th = row[1];
    gout[0] = lin * inject_value(P, 1.0, th, xx[0], xx[1], xx[2]);
    gout[1] = lin * inject_value(P, dt, 1.0, xx[0], xx[1], xx[2]);
}

static int adn_launch(ADNArgs &A, cudaStream_t st)
{
    const int L = A.nd.L;
    int nt = nd_threads(L, A.nd.nlines);
    size_t smem = adn_smem_doubles(L, nt) * sizeof(double);
    long nblocks = (A.nd.nlines + nt - 1) / nt;
    if (raise_smem_limit(k_adjoint_sweep_nd))
        return DGB_ERR_CUDA;
    k_adjoint_sweep_nd<<<(unsigned)nblocks, nt, smem, st>>>(A);
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

static void nd_set_axis(NDArgs &A, int ax)
{
    A.axis = ax;
    A.S = ipow(A.L, A.ndim - 1 - ax);
    A.LS = A.S * A.L;
}

} // namespace dgb

using namespace dgb;

extern "C" int dgb_integrate_table_states(double *phi, int ndim, int L, const double *xx,
                                          const double *table, int nsteps, int frozen_mask,
                                          int nomut_mask, double *states, void *ws,
                                          size_t ws_bytes, void *stream)
{
    if (!phi || !xx || !table || !states || !shape_ok(ndim, L) || nsteps < 0)
        return DGB_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const long N = ipow(L, ndim);
    const int active = ((1 << ndim) - 1) & ~frozen_mask & ~nomut_mask;
    NDArgs A = {};
    nd_fill(A, phi, ndim, L, 0, xx);
    A.table = table;
    double *coef = (ws && ws_bytes >= nd_coef_bytes(ndim, L)) ? (double *)ws : nullptr;
    const int chunk = nd_chunk_steps(ndim, L);
    long step0 = 0;
    for (long s = 0; s <= nsteps; s++) {
        if (cudaMemcpyAsync(states + s * N, phi, N * sizeof(double), cudaMemcpyDeviceToDevice,
                            st) != cudaSuccess)
            return DGB_ERR_CUDA;
        if (s == nsteps)
            break;
        if (coef && s % chunk == 0) {
            step0 = s;
            int rc = nd_coef_chunk(A, false, s, (int)std::min<long>(chunk, nsteps - s),
                                   frozen_mask, active, coef, st);
            if (rc)
                return rc;
        }
        bool first = true;
        for (int ax = 0; ax < ndim; ax++) {
            if (frozen_mask >> ax & 1)
                continue;
            nd_set_axis(A, ax);
            A.step = s;
            A.inject_mask = first ? active : 0;
            first = false;
            int rc = coef ? nd_sweep_rec(A, false, coef, step0, st) : nd_sweep(A, false, st);
            if (rc)
                return rc;
        }
    }
    return DGB_OK;
}

extern "C" size_t dgb_adjoint_table_nd_gpart_doubles(int ndim, int L)
{
    // per step: for each axis, one partial row per CTA of its sweep, plus the
    // injection's two entries
    const long nlines = ipow(L, ndim - 1);
    const int nt = nd_threads(L, nlines);
    const long nb = (nlines + nt - 1) / nt;
    return (size_t)ndim * nb * row_stride(ndim) + 2;
}

extern "C" int dgb_adjoint_table_nd(double *lam, int ndim, int L, const double *xx,
                                    const double *table, int nsteps, int frozen_mask,
                                    int nomut_mask, const double *states, double *gpart,
                                    double *ws, size_t ws_bytes, void *stream)
{
    if (!lam || !xx || !table || !states || !gpart || !shape_ok(ndim, L) || nsteps < 0)
        return DGB_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const long N = ipow(L, ndim);
    int axes[DGB_MAX_DIM], na = 0;
    for (int ax = 0; ax < ndim; ax++)
        if (!(frozen_mask >> ax & 1))
            axes[na++] = ax;
    if (na == 0)
        return DGB_OK;
    if (!ws || ws_bytes < (size_t)(na - 1) * N * sizeof(double))
        return DGB_ERR_WORKSPACE;
    const int active = ((1 << ndim) - 1) & ~frozen_mask & ~nomut_mask;
    const size_t per_step = dgb_adjoint_table_nd_gpart_doubles(ndim, L);
    const long nlines = ipow(L, ndim - 1);
    const long nb = (nlines + nd_threads(L, nlines) - 1) / nd_threads(L, nlines);
    const int stride = row_stride(ndim);
    if (cudaMemsetAsync(gpart, 0, (size_t)nsteps * per_step * sizeof(double), st) !=
        cudaSuccess)
        return DGB_ERR_CUDA;
    NDArgs F = {};
    nd_fill(F, nullptr, ndim, L, 0, xx);
    F.table = table;
    // coefficient records of the step's sweeps (recomputed forward and
    // adjoint), after the intermediate densities when the workspace holds
    // them; chunks walk backwards
    const size_t inter = (size_t)(na - 1) * N * sizeof(double);
    double *coef =
        (ws_bytes >= inter + nd_coef_bytes(ndim, L)) ? ws + (size_t)(na - 1) * N : nullptr;
    const int chunk = nd_chunk_steps(ndim, L);
    long lo = -1;
    for (long k = nsteps - 1; k >= 0; k--) {
        const double *phik = states + k * N, *phin = states + (k + 1) * N;
        if (coef && (lo < 0 || k < lo)) {
            lo = std::max(0L, k - chunk + 1);
            int rc = nd_coef_chunk(F, false, lo, (int)(k - lo + 1), frozen_mask, active, coef, st);
            if (rc)
                return rc;
        }
        // recompute s_1 .. s_{na-1} into ws
        for (int j = 0; j < na - 1; j++) {
            double *dst = ws + (size_t)j * N;
            const double *src = j ? ws + (size_t)(j - 1) * N : phik;
            if (cudaMemcpyAsync(dst, src, N * sizeof(double), cudaMemcpyDeviceToDevice, st) !=
                cudaSuccess)
                return DGB_ERR_CUDA;
            F.phi = dst;
            nd_set_axis(F, axes[j]);
            F.step = k;
            F.inject_mask = j ? 0 : active;
            int rc = coef ? nd_sweep_rec(F, false, coef, lo, st) : nd_sweep(F, false, st);
            if (rc)
                return rc;
        }
        double *gk = gpart + (size_t)k * per_step;
        for (int j = na - 1; j >= 0; j--) {
            ADNArgs A = {};
            A.nd = F;
            A.nd.phi = lam;
            nd_set_axis(A.nd, axes[j]);
            A.nd.step = k;
            A.nd.inject_mask = j ? 0 : active; // the first sweep's input is psi
            A.out = (j == na - 1) ? phin : ws + (size_t)j * N;
            A.rhs = j ? ws + (size_t)(j - 1) * N : phik;
            A.gpart = gk + (size_t)j * nb * stride;
            A.coef = coef;
            A.step0 = lo;
            int rc = adn_launch(A, st);
            if (rc)
                return rc;
        }
        if (active) {
            k_adjoint_inject_nd<<<1, 32, 0, st>>>(lam, xx, table + k * stride, ndim, L, active,
                                                  gk + (size_t)ndim * nb * stride);
            if (cudaGetLastError() != cudaSuccess)
                return DGB_ERR_CUDA;
        }
    }
    return DGB_OK;
}
