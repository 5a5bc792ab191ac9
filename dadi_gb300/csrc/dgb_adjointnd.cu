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
#include "dgb_adjnd.cuh"

namespace dgb {

__global__ void k_adjoint_sweep_nd(ADNArgs A)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ NDShared Sh;
    __shared__ double red[ADN_MAXQ][8];
    adn_tile(A, blockIdx.x, smem, Sh, red);
}

// Injection's part of dJ/d(dt) and dJ/d(theta0) for one step: lambda (the
// adjoint at the start of the step) at the injected points.
__global__ void k_adjoint_inject_nd(const double *lam, const double *xx, const double *row,
                                    int P, int L, int active, double *gout)
{
    if (threadIdx.x == 0)
        adn_inject_terms(lam, xx, row, P, L, active, gout);
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

namespace dgb {
int preload_adjointnd() { return preload(k_adjoint_sweep_nd) + preload(k_adjoint_inject_nd); }
} // namespace dgb
