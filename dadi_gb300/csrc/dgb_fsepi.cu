// Spectrum epilogue of 2-D integrations, on the device and for a list of work
// items per launch:
//
//  * k_from_phi2d: the sampling contraction of Spectrum.from_phi for two
//    populations (dadi/Spectrum_mod.py:1509-1547): phi is piecewise linear on
//    the grid, and each sample count's probability is its integral against
//    the binomial weights, i.e. differences of regularised incomplete beta
//    functions (cached_dbeta, dadi/Spectrum_mod.py:25-40) supplied as tables.
//    Along y: s = dphi/dx per interval, c1 = (phi - s x)/(n+1), then
//    over_y[i][b] = sum_j dbeta1[b][j] c1[i][j]
//                 + (b+1)/((n+1)(n+2)) sum_j dbeta2[b][j] s[i][j];
//    then the same along x on over_y.
//  * k_extrap_ll: Richardson extrapolation of 1-3 grids' spectra to zero
//    grid spacing (linear_extrap / quadratic_extrap, dadi/Numerics.py:644-669)
//    with the fail_mag guard (dadi/Numerics.py:449-464), and optionally the
//    Poisson log-likelihood of scale * model against data over entries that
//    are not masked corners and have a positive model
//    (dadi/Inference.py:466-509).
//
// One CTA per item.  The contraction is ~3 MFLOP per grid at L = 120, n =
// 40: small next to the integration; the point of doing it here is one launch
// per batch instead of dozens of library calls per spectrum, and results that
// do not depend on which other items share the launch.
#include <algorithm>

#include "dgb_internal.h"

namespace dgb {

constexpr int FS_THREADS = 256;
constexpr int FS_ROWS = 16; // rows of phi staged at a time for the y contraction

__host__ __device__ inline size_t fs_smem_doubles(int Lmax, int nmax)
{
    // x, dx | over_y (Lmax x (nmax+1)) | s_x ((Lmax-1) x (nmax+1)) |
    // staged rows: s and c1, FS_ROWS x (Lmax-1) each
    return 2 * (size_t)Lmax + 2 * (size_t)Lmax * (nmax + 1) + 2 * (size_t)FS_ROWS * Lmax;
}

__global__ void __launch_bounds__(FS_THREADS) k_from_phi2d(const dgb_fs_item2d *items,
                                                           int Lmax, int nmax)
{
    extern __shared__ __align__(16) double sm[];
    const dgb_fs_item2d it = items[blockIdx.x];
    const int L = it.L, n1 = it.n1, n2 = it.n2, M = L - 1;
    if (L < 2 || L > Lmax || n1 < 1 || n2 < 1 || n2 > nmax)
        return; // outside the launch's shared-memory sizing: left unwritten
    const int tid = threadIdx.x, nt = blockDim.x;
    double *x = sm;
    double *dx = x + Lmax;
    double *over = dx + Lmax;                     // [i][b], pitch n2+1
    double *sx = over + (size_t)Lmax * (nmax + 1); // [i][b], pitch n2+1
    double *rs = sx + (size_t)Lmax * (nmax + 1);   // staged s rows [r][j], pitch M
    double *rc = rs + (size_t)FS_ROWS * Lmax;      // staged c1 rows
    const int P2 = n2 + 1;

    for (int i = tid; i < L; i += nt)
        x[i] = it.xx[i];
    __syncthreads();
    for (int j = tid; j < M; j += nt)
        dx[j] = x[j + 1] - x[j];
    __syncthreads();

    // ---- contraction along y, FS_ROWS rows of phi at a time
    const double inv_n2 = 1.0 / (n2 + 1);
    for (int i0 = 0; i0 < L; i0 += FS_ROWS) {
        const int nr = min(FS_ROWS, L - i0);
        for (int e = tid; e < nr * M; e += nt) {
            const int r = e / M, j = e - r * M;
            const double *row = it.phi + (size_t)(i0 + r) * L;
            const double p0 = row[j], p1 = row[j + 1];
            const double s = (p1 - p0) / dx[j];
            rs[r * M + j] = s;
            rc[r * M + j] = (p0 - s * x[j]) * inv_n2;
        }
        __syncthreads();
        for (int e = tid; e < nr * P2; e += nt) {
            const int r = e / P2, b = e - r * P2;
            const double *d1 = it.d1y + (size_t)b * M, *d2 = it.d2y + (size_t)b * M;
            const double *cr = rc + r * M, *sr = rs + r * M;
            double t1 = 0, t2 = 0;
            for (int j = 0; j < M; j++) {
                t1 = fma(d1[j], cr[j], t1);
                t2 = fma(d2[j], sr[j], t2);
            }
            const double w = (double)(b + 1) / ((double)(n2 + 1) * (n2 + 2));
            over[(size_t)(i0 + r) * P2 + b] = t1 + t2 * w;
        }
        __syncthreads();
    }

    // ---- slopes and intercepts along x (intercepts overwrite over_y)
    const double inv_n1 = 1.0 / (n1 + 1);
    for (int e = tid; e < M * P2; e += nt) {
        const int i = e / P2, b = e - i * P2;
        sx[e] = (over[(size_t)(i + 1) * P2 + b] - over[e]) / dx[i];
    }
    __syncthreads();
    for (int e = tid; e < M * P2; e += nt) {
        const int i = e / P2;
        over[e] = (over[e] - sx[e] * x[i]) * inv_n1;
    }
    __syncthreads();

    // ---- contraction along x
    const int P1 = n1 + 1;
    for (int e = tid; e < P1 * P2; e += nt) {
        const int a = e / P2, b = e - a * P2;
        const double *d1 = it.d1x + (size_t)a * M, *d2 = it.d2x + (size_t)a * M;
        double t1 = 0, t2 = 0;
        for (int i = 0; i < M; i++) {
            t1 = fma(d1[i], over[(size_t)i * P2 + b], t1);
            t2 = fma(d2[i], sx[(size_t)i * P2 + b], t2);
        }
        const double w = (double)(a + 1) / ((double)(n1 + 1) * (n1 + 2));
        it.out[e] = t1 + t2 * w;
    }
}

// Fixed-order block sum of v over FS_THREADS threads (all threads get it).
__device__ __forceinline__ double block_sum(double *red, double v)
{
    const int tid = threadIdx.x;
    __syncthreads(); // red free: earlier readers are done
    red[tid] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (tid < s)
            red[tid] += red[tid + s];
        __syncthreads();
    }
    return red[0];
}

// Poisson term of one entry (dadi/Inference.py:482-509: entries with a
// nonpositive model are masked by model.log()).
__device__ __forceinline__ double poisson_term(double model, double d)
{
    return (model > 0) ? -model + d * log(model) - lgamma(d + 1.0) : 0.0;
}

__global__ void __launch_bounds__(FS_THREADS) k_extrap_ll(const dgb_extrap_item *items,
                                                          double fail_mag)
{
    __shared__ double red[FS_THREADS];
    const dgb_extrap_item it = items[blockIdx.x];
    const int tid = threadIdx.x;
    const int g = it.ngrids;
    if (g < 1 || g > 3)
        return;
    // Lagrange weights of the extrapolation to x = 0, in the reference's
    // order of operations
    double w0 = 0, w1 = 0, w2 = 0;
    const double x1 = it.x[0], x2 = it.x[1], x3 = it.x[2];
    if (g == 3) {
        w0 = x2 * x3 / ((x1 - x2) * (x1 - x3));
        w1 = x1 * x3 / ((x2 - x1) * (x2 - x3));
        w2 = x1 * x2 / ((x3 - x1) * (x3 - x2));
    }
    int best = 0;
    for (int k = 1; k < g; k++)
        if (it.x[k] < it.x[best])
            best = k;
    const bool pois = it.data && it.ll;
    const bool mult = it.data && it.ll_multinom;
    double acc = 0, sd = 0, sm = 0;
    for (int e = tid; e < it.size; e += blockDim.x) {
        const double y1 = it.fs[0][e];
        double ex;
        if (g == 1) {
            ex = y1;
        } else if (g == 2) {
            const double y2 = it.fs[1][e];
            ex = (x2 * y1 - x1 * y2) / (x2 - x1);
        } else {
            ex = w0 * y1 + w1 * it.fs[1][e] + w2 * it.fs[2][e];
        }
        if (g > 1) {
            const double bv = it.fs[best][e];
            if (fabs(log10(ex / bv)) > fail_mag)
                ex = bv;
        }
        it.out[e] = ex;
        const bool masked = it.mask_corners && (e == 0 || e == it.size - 1);
        if ((pois || mult) && !masked) {
            const double d = it.data[e];
            if (pois)
                acc += poisson_term(it.scale * ex, d);
            if (mult) {
                sd += d;
                sm += ex;
            }
        }
    }
    if (!(pois || mult))
        return;
    if (pois) {
        const double tot = block_sum(red, acc);
        if (tid == 0)
            *it.ll = tot;
    }
    if (!mult)
        return;
    // optimal scaling over the unmasked entries, then the Poisson sum at it;
    // each thread re-reads the entries it wrote above
    const double sdata = block_sum(red, sd);
    const double smodel = block_sum(red, sm);
    const double theta = sdata / smodel;
    double acc2 = 0;
    for (int e = tid; e < it.size; e += blockDim.x) {
        const bool masked = it.mask_corners && (e == 0 || e == it.size - 1);
        if (!masked)
            acc2 += poisson_term(theta * it.out[e], it.data[e]);
    }
    const double tot2 = block_sum(red, acc2);
    if (tid == 0)
        *it.ll_multinom = tot2;
}


// ---------------------------------------------- from_phi, any dimension

// One contraction of Spectrum.from_phi's linear-algebra form
// (dadi/Spectrum_mod.py:1509-1547, 1774-1810, 1841-1870): every row of L
// values along the last axis of the current tensor (M rows, row m at m*L) is
// integrated against the binomial sampling weights of n samples,
//   out[k][m] = sum_j d1[k][j] c1[m][j] + (k+1)/((n+1)(n+2)) sum_j d2[k][j] s[m][j],
//   s = (p[j+1] - p[j]) / (x[j+1] - x[j]),  c1 = (p[j] - s x[j]) / (n+1),
// and the new axis of n+1 entries comes first: out is (n+1) x M.  Applied
// once per axis, last axis first, this rotates the axes back into order and
// gives the spectrum (the reference's 3-D/4-D code contracts the last axis
// first as well).  A CTA takes CT_ROWS rows of one density: a coalesced copy
// into shared memory ([j][r], odd pitch), the slopes and intercepts in
// place, then each of its CT_KG warps accumulates every CT_KG-th output entry
// for its 32 rows from the weight tables (warp-uniform reads), KC entries at
// a time in registers.
constexpr int CT_ROWS = 32;
constexpr int CT_KG = 4;
constexpr int CT_KC = 6;

__host__ __device__ inline size_t ct_smem_doubles(int L)
{
    return 2 * (size_t)L + 2 * (size_t)L * (CT_ROWS + 1);
}

__global__ void __launch_bounds__(CT_ROWS *CT_KG)
    k_contract_last(const double *in, long in_bs, double *out, long out_bs, long M, int L, int n,
                    const double *xx, const double *d1, const double *d2)
{
    extern __shared__ __align__(16) double sm[];
    const int tid = threadIdx.x, nth = blockDim.x;
    const int r = tid % CT_ROWS, g = tid / CT_ROWS;
    const long m0 = (long)blockIdx.x * CT_ROWS;
    const int nr = (int)min((long)CT_ROWS, M - m0);
    const double *src = in + (long)blockIdx.y * in_bs + m0 * L;
    double *dst = out + (long)blockIdx.y * out_bs;
    constexpr int PT = CT_ROWS + 1;
    double *x = sm, *dx = sm + L;
    double *P = dx + L;                 // phi, then the intercepts c1: [j][r]
    double *S = P + (size_t)L * PT;     // slopes: [j][r]
    for (int i = tid; i < L; i += nth)
        x[i] = xx[i];
    for (int e = tid; e < nr * L; e += nth) {
        const int rr = e / L, j = e - rr * L;
        P[j * PT + rr] = src[e];
    }
    __syncthreads();
    for (int j = tid; j < L - 1; j += nth)
        dx[j] = x[j + 1] - x[j];
    __syncthreads();
    const double inv_n = 1.0 / (n + 1);
    for (int e = tid; e < (L - 1) * CT_ROWS; e += nth) {
        const int j = e / CT_ROWS, rr = e - j * CT_ROWS;
        S[j * PT + rr] = (P[(j + 1) * PT + rr] - P[j * PT + rr]) / dx[j];
    }
    __syncthreads();
    for (int e = tid; e < (L - 1) * CT_ROWS; e += nth) {
        const int j = e / CT_ROWS, rr = e - j * CT_ROWS;
        P[j * PT + rr] = (P[j * PT + rr] - S[j * PT + rr] * x[j]) * inv_n;
    }
    __syncthreads();
    const int Mj = L - 1;
    for (int k0 = g; k0 <= n; k0 += CT_KG * CT_KC) {
        double a1[CT_KC], a2[CT_KC];
#pragma unroll
        for (int q = 0; q < CT_KC; q++)
            a1[q] = a2[q] = 0;
        for (int j = 0; j < Mj; j++) {
            const double c = P[j * PT + r], sv = S[j * PT + r];
#pragma unroll
            for (int q = 0; q < CT_KC; q++) {
                const int k = k0 + q * CT_KG;
                if (k <= n) {
                    a1[q] = fma(d1[(size_t)k * Mj + j], c, a1[q]);
                    a2[q] = fma(d2[(size_t)k * Mj + j], sv, a2[q]);
                }
            }
        }
        if (r < nr) {
#pragma unroll
            for (int q = 0; q < CT_KC; q++) {
                const int k = k0 + q * CT_KG;
                if (k <= n) {
                    const double w = (double)(k + 1) / ((double)(n + 1) * (n + 2));
                    dst[(long)k * M + m0 + r] = a1[q] + a2[q] * w;
                }
            }
        }
    }
}

// Sizes (doubles per density) of the tensors between contractions: after
// contracting axes ndim-1 .. ndim-t the tensor has
// prod_{a >= ndim-t} (ns[a]+1) x L^(ndim-t) entries.
static long ct_size_after(int ndim, int L, const int *ns, int t)
{
    long s = 1;
    for (int a = ndim - t; a < ndim; a++)
        s *= ns[a] + 1;
    for (int a = 0; a < ndim - t; a++)
        s *= L;
    return s;
}

} // namespace dgb

using namespace dgb;

extern "C" size_t dgb_from_phi_nd_workspace_bytes(int ndim, int L, const int *ns, int nbatch)
{
    if (ndim < 1 || ndim > DGB_MAX_DIM || L < 2 || !ns || nbatch < 1)
        return 0;
    long mx = 0;
    for (int t = 1; t < ndim; t++)
        mx = std::max(mx, ct_size_after(ndim, L, ns, t));
    return (size_t)(2 * mx * (long)nbatch + 1) * sizeof(double);
}

extern "C" int dgb_from_phi_nd(const double *phi, int nbatch, int ndim, int L, const double *xx,
                               const int *ns, const double *const *d1, const double *const *d2,
                               double *out, void *ws, size_t ws_bytes, void *stream)
{
    if (!phi || nbatch < 0 || ndim < 1 || ndim > DGB_MAX_DIM || L < 2 || !xx || !ns || !d1 ||
        !d2 || !out)
        return DGB_ERR_ARG;
    for (int a = 0; a < ndim; a++)
        if (ns[a] < 1 || !d1[a] || !d2[a])
            return DGB_ERR_ARG;
    if (nbatch == 0)
        return DGB_OK;
    const size_t smem = ct_smem_doubles(L) * sizeof(double);
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
            cudaSuccess)
        return DGB_ERR_CUDA;
    if (smem > (size_t)optin)
        return DGB_ERR_UNSUPPORTED;
    if (ndim > 1 && (!ws || ws_bytes < dgb_from_phi_nd_workspace_bytes(ndim, L, ns, nbatch)))
        return DGB_ERR_WORKSPACE;
    if (raise_smem_limit(k_contract_last))
        return DGB_ERR_CUDA;
    long mx = 0;
    for (int t = 1; t < ndim; t++)
        mx = std::max(mx, ct_size_after(ndim, L, ns, t));
    double *buf[2] = {(double *)ws, (double *)ws + mx * (long)nbatch};
    const double *cur = phi;
    long cur_bs = ct_size_after(ndim, L, ns, 0);
    for (int t = 1; t <= ndim; t++) {
        const int a = ndim - t; // the axis contracted now
        const long M = ct_size_after(ndim, L, ns, t - 1) / L;
        const long nxt_bs = ct_size_after(ndim, L, ns, t);
        double *dst = (t == ndim) ? out : buf[t % 2];
        dim3 grid((unsigned)((M + CT_ROWS - 1) / CT_ROWS), (unsigned)nbatch);
        k_contract_last<<<grid, CT_ROWS * CT_KG, smem, (cudaStream_t)stream>>>(
            cur, cur_bs, dst, nxt_bs, M, L, ns[a], xx, d1[a], d2[a]);
        if (cudaGetLastError() != cudaSuccess)
            return DGB_ERR_CUDA;
        cur = dst;
        cur_bs = nxt_bs;
    }
    return DGB_OK;
}

extern "C" size_t dgb_from_phi2d_smem_bytes(int Lmax, int nmax)
{
    return fs_smem_doubles(Lmax, nmax) * sizeof(double);
}

extern "C" int dgb_from_phi2d(const dgb_fs_item2d *items, int nitems, int Lmax, int nmax,
                              void *stream)
{
    if (!items || nitems < 0 || Lmax < 2 || nmax < 1)
        return DGB_ERR_ARG;
    if (nitems == 0)
        return DGB_OK;
    size_t smem = fs_smem_doubles(Lmax, nmax) * sizeof(double);
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
            cudaSuccess)
        return DGB_ERR_CUDA;
    if (smem > (size_t)optin)
        return DGB_ERR_UNSUPPORTED;
    if (raise_smem_limit(k_from_phi2d))
        return DGB_ERR_CUDA;
    k_from_phi2d<<<(unsigned)nitems, FS_THREADS, smem, (cudaStream_t)stream>>>(items, Lmax, nmax);
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

extern "C" int dgb_extrap_ll(const dgb_extrap_item *items, int nitems, double fail_mag,
                             void *stream)
{
    if (!items || nitems < 0)
        return DGB_ERR_ARG;
    if (nitems == 0)
        return DGB_OK;
    k_extrap_ll<<<(unsigned)nitems, FS_THREADS, 0, (cudaStream_t)stream>>>(items, fail_mag);
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

namespace dgb {
int preload_fsepi()
{
    return preload(k_from_phi2d) + preload(k_extrap_ll) + preload(k_contract_last);
}
} // namespace dgb
