// One 2-D integration spread over a thread-block cluster.
//
// GB300's FP64 pipe retires about 1.7 FMA lanes per clock per SM, so a lone
// 2-D integration on one CTA (k_integrate2d) is bound by its one SM's pipe
// (L = 120: about 88,000 clocks per sweep).  Here the S CTAs of a cluster
// (S SMs) share the grid: CTA r holds rows R0 .. R0+m-1 of phi (all L
// columns) in shared memory for the whole time loop, and every sweep is a
// partitioned Thomas solve (the modified-Thomas form of the partition method,
// as in k_sweep_batch_part):
//
// * x sweep (lines = columns, points = rows): each column is cut into the S
//   CTAs' row blocks.  Each CTA's thread j runs the downward and upward
//   passes over its rows and exports the two end rows of its segment
//   (x_first = D' - A' z_prev - C' z, and al x_first + z + ga x_next = de);
//   after a cluster barrier, the thread of column j in CTA j mod S reads the
//   S segments' rows through distributed shared memory, solves the
//   tridiagonal system in the segments' last points z_0 .. z_{S-1} and
//   writes z_q, z_{q-1} into CTA q; after a second barrier each CTA
//   finishes its interior points.
// * y sweep (lines = rows, points = columns): the rows are local; each is
//   cut into 8 segments on 8 threads of the CTA (so 16 rows fill its 128
//   lanes) and solved the same way with CTA barriers.
//
// The rows, corner terms, injection and parameter rows are those of
// k_integrate2d (Integration.two_pops, dadi/Integration.py:340-386, with
// implicit_2Dx / implicit_2Dy, dadi/integration2D.c:19-160); the solves
// agree with Thomas to rounding.  Default delta_j only; L <= 16 S and
// segments of at least 3 rows (L >= 24, L >= 3 S).
#include <algorithm>

#include <cooperative_groups.h>

#include "dgb_cluster.cuh"
#include "dgb_internal.h"

namespace cg = cooperative_groups;

namespace dgb {


struct C2Args {
    double *phi;
    const double *xx;
    const double *table;
    int L, nsteps, frozen, nomut;
    // a list of work items, one cluster each (null: the one integration above)
    const dgb_item2d *items;
    const long *row_off; // first table row of each schedule
    const int *row_cnt;  // rows of each schedule
    int Lmin, Lmax;      // the grid sizes the launch was checked for
    // optional: phi before every ckpt_every-th step, row-major, item i's
    // checkpoints from ckpt + ckpt_off[i] (the forward of the adjoint)
    double *ckpt;
    const long *ckpt_off;
    int ckpt_every;
};

struct C2Shared {
    AxisScalars ax[2];
    double inj;
};


// Shared memory (doubles) of one CTA for grids of up to L points.
__host__ __device__ inline size_t c2_smem_doubles(int L)
{
    return (size_t)C2_ROWS * c2_pitch(L) + 2 * (size_t)C2_ROWS * L + 16 * (size_t)L +
           (size_t)C2_XROW * L + 2 * (size_t)L + (size_t)C2_YSLOT * C2_YSEG * C2_ROWS;
}


__global__ void __launch_bounds__(C2_THREADS) k_integrate2d_cluster(C2Args A)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ C2Shared Sh;
    cg::cluster_group cluster = cg::this_cluster();
    const int S = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    double *phi_g = A.phi;
    const double *xx = A.xx, *table = A.table;
    int L = A.L, nsteps = A.nsteps, frozen = A.frozen, nomut = A.nomut;
    double *ck = nullptr;
    if (A.items) {
        // this cluster's work item; every CTA of the cluster reads the same
        // one, so a skipped item is skipped by the whole cluster
        const dgb_item2d it = A.items[blockIdx.x / S];
        if (it.L < A.Lmin || it.L > A.Lmax)
            return;
        L = it.L;
        xx = A.xx + it.xx_off;
        phi_g = A.phi + it.out_off;
        table = A.table + A.row_off[it.sched] * 11;
        nsteps = A.row_cnt[it.sched];
        frozen = it.masks & 0xff;
        nomut = it.masks >> 8 & 0xff;
        if (A.ckpt)
            ck = A.ckpt + A.ckpt_off[blockIdx.x / S];
    }
    const int tid = threadIdx.x, pitch = c2_pitch(L);
    int R0, m;
    c2_rows(L, S, rank, &R0, &m);
    double *blk = smem;                                  // m x pitch: rows R0 ..
    double *al = blk + (size_t)C2_ROWS * pitch;          // x: [p][j]; y: [j][p]
    double *ga = al + (size_t)C2_ROWS * L;
    GridVecs g;
    double *q0 = ga + (size_t)C2_ROWS * L;
    g.x = q0;
    g.xv = q0 + L;
    g.dfac = q0 + 2 * L;
    g.xInt = q0 + 3 * L;
    g.ih = q0 + 4 * L;
    g.dx = q0 + 5 * L;
    AxisVecs v[2];
    v[0].A1 = q0 + 6 * L;
    v[0].A0 = q0 + 7 * L;
    v[0].C1 = q0 + 8 * L;
    v[0].C0 = q0 + 9 * L;
    v[0].B0 = q0 + 10 * L;
    v[1].A1 = q0 + 11 * L;
    v[1].A0 = q0 + 12 * L;
    v[1].C1 = q0 + 13 * L;
    v[1].C0 = q0 + 14 * L;
    v[1].B0 = q0 + 15 * L;
    for (int a = 0; a < 2; a++)
        v[a].G = v[a].Pv = v[a].Qv = v[a].VI = v[a].DF = nullptr;
    double *xr = q0 + 16 * L;             // exported rows of the x segments, [k][j]
    double *zin = xr + C2_XROW * L;       // z of this segment and of the one above, [2][j]
    double *yr = zin + 2 * L;             // y sweep slots, [(q * C2_YSLOT + k) * C2_ROWS + p]

    // grid constants and this CTA's rows of the initial density
    for (int i = tid; i < L; i += C2_THREADS) {
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
    for (int idx = tid; idx < m * L; idx += C2_THREADS) {
        const int p = idx / L, c = idx - p * L;
        blk[p * pitch + c] = phi_g[(size_t)(R0 + p) * L + c];
    }
    __syncthreads();
    for (int i = tid; i < L; i += C2_THREADS)
        g.dfac[i] = (i == 0)       ? 2. / g.dx[0]
                    : (i == L - 1) ? 2. / g.dx[L - 2]
                                   : 2. / (g.dx[i] + g.dx[i - 1]);
    __syncthreads();
    const int j0 = (g.x[0] == 0.0) ? 0 : -1;
    const int j1 = (g.x[L - 1] == 1.0) ? L - 1 : -1;

    for (int step = 0; step < nsteps; step++) {
        const double *row = table + (size_t)step * 11;
        if (ck && step % A.ckpt_every == 0) {
            // this CTA's rows of phi before the step
            double *c = ck + (size_t)(step / A.ckpt_every) * L * L + (size_t)R0 * L;
            for (int idx = tid; idx < m * L; idx += C2_THREADS) {
                const int p = idx / L, q = idx - p * L;
                c[idx] = blk[p * pitch + q];
            }
        }
        if (tid < 2) {
            AxisScalars &s = Sh.ax[tid];
            const int a = tid;
            const double dt = row[0];
            s.dt = dt;
            s.nu = row[row_nu(2, a)];
            s.inv_nu = 1.0 / s.nu;
            s.gamma = row[row_gamma(2, a)];
            s.h = row[row_h(2, a)];
            const double mg = row[row_mig(2, a, 1 - a)];
            s.msum = mg;
            s.mig[a] = 0;
            s.mig[1 - a] = mg;
            s.B1s = 0.5 * (dt * g.dfac[0]);
            s.B1e = -0.5 * (dt * g.dfac[L - 1]);
            corner_bc(2, a, s.mig, s.nu, s.gamma, s.h, g.x[0], g.x[L - 1], g.dx[0], g.dx[L - 2],
                      dt, s.bcs, s.bce);
        } else if (tid == 2) {
            Sh.inj = inject_value(2, row[0], row[1], g.x[0], g.x[1], g.x[2]);
        }
        __syncthreads();
        for (int t = tid; t < 2 * L; t += C2_THREADS) {
            const int a = t >= L, i = t - a * L;
            build_axis_entry(i, L, g, Sh.ax[a], 1.0, false, v[a]);
        }
        if (tid == 0 && rank == 0) {
            // rows 0 and 1 are this CTA's (m >= 3)
            if (!(frozen & 1) && !(nomut & 1))
                blk[1 * pitch + 0] += Sh.inj;
            if (!(frozen & 2) && !(nomut & 2))
                blk[0 * pitch + 1] += Sh.inj;
        }
        __syncthreads();

        if (!(frozen & 1))
            c2_sweep_x(cluster, S, rank, blk, pitch, L, R0, m, al, ga, xr, zin, v[0], Sh.ax[0],
                       g, j0, j1);
        if (!(frozen & 2))
            c2_sweep_y(blk, pitch, L, R0, m, al, ga, yr, v[1], Sh.ax[1], g, j0, j1);
    }
    for (int idx = tid; idx < m * L; idx += C2_THREADS) {
        const int p = idx / L, c = idx - p * L;
        phi_g[(size_t)(R0 + p) * L + c] = blk[p * pitch + c];
    }
    // no CTA may leave while another may still read its shared memory
    cluster.sync();
}

} // namespace dgb

using namespace dgb;

namespace dgb {

static bool c2_fits(int L, int cluster)
{
    return L >= 3 * C2_YSEG && L <= C2_THREADS && L >= 3 * cluster && L <= C2_ROWS * cluster;
}

static int c2_launch(const C2Args &A, int nclusters, int cluster, int Lmax, cudaStream_t st)
{
    // at least 116 KB per CTA, so that no two CTAs of a cluster share an SM
    // (and its FP64 pipe)
    const size_t smem = std::max(c2_smem_doubles(Lmax) * sizeof(double), (size_t)116 << 10);
    if (raise_smem_limit(k_integrate2d_cluster))
        return DGB_ERR_CUDA;
    if (cluster > 8 && cudaFuncSetAttribute(k_integrate2d_cluster,
                                            cudaFuncAttributeNonPortableClusterSizeAllowed,
                                            1) != cudaSuccess) {
        cudaGetLastError();
        return DGB_ERR_UNSUPPORTED;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(cluster * nclusters), 1, 1);
    cfg.blockDim = dim3(C2_THREADS, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, k_integrate2d_cluster, A) != cudaSuccess) {
        cudaGetLastError();
        return DGB_ERR_CUDA;
    }
    return DGB_OK;
}

} // namespace dgb

extern "C" int dgb_integrate2d_cluster(double *phi, int L, const double *xx, const double *table,
                                       int nsteps, int frozen_mask, int nomut_mask, int cluster,
                                       void *stream)
{
    if (!phi || !xx || !table || nsteps < 0 || L < 3)
        return DGB_ERR_ARG;
    if (cluster != 2 && cluster != 4 && cluster != 8 && cluster != 16)
        return DGB_ERR_ARG;
    if (!c2_fits(L, cluster))
        return DGB_ERR_UNSUPPORTED;
    if (nsteps == 0)
        return DGB_OK;
    C2Args A = {};
    A.phi = phi;
    A.xx = xx;
    A.table = table;
    A.L = L;
    A.nsteps = nsteps;
    A.frozen = frozen_mask;
    A.nomut = nomut_mask;
    return c2_launch(A, 1, cluster, L, (cudaStream_t)stream);
}

extern "C" int dgb_items2d_integrate_cluster(const dgb_item2d *items, int nitems, int Lmin,
                                             int Lmax, const double *xx_all, double *phi_out,
                                             const double *table, const long *row_off,
                                             const int *row_cnt, int cluster, double *ckpt,
                                             const long *ckpt_off, int ckpt_every, void *stream)
{
    if (!items || nitems < 0 || !xx_all || !phi_out || !table || !row_off || !row_cnt ||
        Lmin > Lmax || (ckpt && (!ckpt_off || ckpt_every < 1)))
        return DGB_ERR_ARG;
    if (cluster != 2 && cluster != 4 && cluster != 8 && cluster != 16)
        return DGB_ERR_ARG;
    if (!c2_fits(Lmin, cluster) || !c2_fits(Lmax, cluster))
        return DGB_ERR_UNSUPPORTED;
    if (nitems == 0)
        return DGB_OK;
    C2Args A = {};
    A.phi = phi_out;
    A.xx = xx_all;
    A.table = table;
    A.items = items;
    A.row_off = row_off;
    A.row_cnt = row_cnt;
    A.Lmin = Lmin;
    A.Lmax = Lmax;
    A.ckpt = ckpt;
    A.ckpt_off = ckpt_off;
    A.ckpt_every = ckpt_every;
    return c2_launch(A, nitems, cluster, Lmax, (cudaStream_t)stream);
}

namespace dgb {
int preload_cluster2d() { return preload(k_integrate2d_cluster); }
} // namespace dgb

extern "C" int dgb_preload(void)
{
    const int bad = preload_integrate2d() + preload_sweepnd() + preload_probe() +
                    preload_adjoint2d() + preload_fsepi() + preload_adjointnd() +
                    preload_batchnd() + preload_cluster2d();
    if (bad) {
        cudaGetLastError();
        return DGB_ERR_CUDA;
    }
    return DGB_OK;
}
