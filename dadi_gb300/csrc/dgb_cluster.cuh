// The partitioned sweeps of a 2-D density whose rows are spread over the
// CTAs of a thread-block cluster (the modified-Thomas form of the partition
// method): used by the forward (dgb_cluster2d.cu) and by the adjoint's
// backward walk (dgb_adjoint2d.cu), which solve the same kind of system --
// the forward with the sweep's vectors, the adjoint with the transposed
// ones.  The CTA holds rows R0 .. R0+m-1 of the density (m <= C2_ROWS) in
// `blk` at row pitch `pitch`.
//
// * c2_sweep_x (lines = columns): each column is cut into the CTAs' row
//   blocks; thread j runs the downward and upward passes over the CTA's
//   rows and exports the two end rows of its segment (x_first = D' - A'
//   z_prev - C' z and al x_first + z + ga x_next = de) into xr; after a
//   cluster barrier the thread of column j in CTA j mod S reads the S
//   segments' rows through distributed shared memory, solves the
//   tridiagonal system in the segments' last points z_0 .. z_{S-1} and
//   writes z_q, z_{q-1} into CTA q's zin; after a second barrier each CTA
//   finishes its interior points.
// * c2_sweep_y (lines = rows): the rows are the CTA's own; each is cut into
//   C2_YSEG segments on C2_YSEG threads (16 rows fill 128 lanes) and solved
//   the same way with CTA barriers.
//
// Both are called by every thread of the CTA (and, for x, of every CTA of
// the cluster): they contain the barriers.  Default delta_j rows only.
#pragma once
#include <cooperative_groups.h>

#include "dgb_common.cuh"

namespace dgb {

constexpr int C2_THREADS = 128;
constexpr int C2_ROWS = 16; // rows per CTA at most
constexpr int C2_YSEG = 8;  // segments per row in the y sweep
constexpr int C2_XROW = 6;  // exported values per column: A' C' D' al ga de
constexpr int C2_YSLOT = 8; // per (row, segment): A' C' D', al ga de / z row, z

__host__ __device__ inline int c2_pitch(int L) { return (L % 2) ? L : L + 1; }

// Rows of CTA r of S over L points: [*r0, *r0 + *m).
__host__ __device__ inline void c2_rows(int L, int S, int r, int *r0, int *m)
{
    const int base = L / S, extra = L % S;
    *r0 = r * base + (r < extra ? r : extra);
    *m = base + (r < extra ? 1 : 0);
}

// The x sweep of the CTA's rows; al, ga: C2_ROWS x L scratch ([p][j]); xr:
// C2_XROW x L doubles read by the other CTAs; zin: 2 L doubles they write.
__device__ __forceinline__ void c2_sweep_x(cooperative_groups::cluster_group &cluster, int S,
                                           int rank, double *blk, int pitch, int L, int R0,
                                           int m, double *al, double *ga, double *xr,
                                           double *zin, const AxisVecs &vv,
                                           const AxisScalars &s, const GridVecs &g, int j0,
                                           int j1)
{
    const int j = threadIdx.x;
    if (j < L) {
        const double W = s.mig[1] * g.x[j];
        auto arow = [&](int i) { return (i > 0) ? fma(W, vv.A1[i], vv.A0[i]) : 0.0; };
        auto crow = [&](int i) { return (i < L - 1) ? fma(W, vv.C1[i], vv.C0[i]) : 0.0; };
        auto brow = [&](int i) {
            if (i == 0)
                return fma(W, s.B1s, vv.B0[0]) + (j == j0 ? s.bcs : 0.0);
            if (i == L - 1)
                return fma(W, s.B1e, vv.B0[L - 1]) + (j == j1 ? s.bce : 0.0);
            return vv.B0[i];
        };
        int p = 1;
        double aa = arow(R0 + p);
        double inv = rcp_full(brow(R0 + p));
        double alp = aa * inv, gap = crow(R0 + p) * inv, dep = blk[p * pitch + j] * inv;
        al[p * L + j] = alp;
        ga[p * L + j] = gap;
        blk[p * pitch + j] = dep;
        for (p = 2; p < m; p++) {
            aa = arow(R0 + p);
            inv = rcp_full(fma(-aa, gap, brow(R0 + p)));
            alp = -aa * alp * inv;
            gap = crow(R0 + p) * inv;
            dep = fma(-aa, dep, blk[p * pitch + j]) * inv;
            al[p * L + j] = alp;
            ga[p * L + j] = gap;
            blk[p * pitch + j] = dep;
        }
        xr[3 * L + j] = alp;
        xr[4 * L + j] = gap;
        xr[5 * L + j] = dep;
        p = m - 2;
        double deu = blk[p * pitch + j], alu = al[p * L + j], gau = ga[p * L + j];
        for (p = m - 3; p >= 1; p--) {
            const double gg = ga[p * L + j];
            deu = fma(-gg, deu, blk[p * pitch + j]);
            alu = fma(-gg, alu, al[p * L + j]);
            gau = -gg * gau;
            blk[p * pitch + j] = deu;
            al[p * L + j] = alu;
            ga[p * L + j] = gau;
        }
        const double c0 = crow(R0);
        const double iB = rcp_full(fma(-c0, alu, brow(R0)));
        xr[0 * L + j] = arow(R0) * iB;
        xr[1 * L + j] = (-c0 * gau) * iB;
        xr[2 * L + j] = fma(-c0, deu, blk[j]) * iB;
    }
    cluster.sync();
    if (j < L && j % S == rank) {
        // column j's system in the segments' last points
        double gm[C2_ROWS], z[C2_ROWS];
        double gq = 0, u = 0;
        for (int q = 0; q < S; q++) {
            const double *rq = cluster.map_shared_rank(xr, q);
            const double Ap = rq[j], Cp = rq[L + j], Dp = rq[2 * L + j];
            const double alq = rq[3 * L + j], gaq = rq[4 * L + j], deq = rq[5 * L + j];
            double An = 0, Cn = 0, Dn = 0;
            if (q + 1 < S) {
                const double *rn = cluster.map_shared_rank(xr, q + 1);
                An = rn[j];
                Cn = rn[L + j];
                Dn = rn[2 * L + j];
            }
            const double ra = -alq * Ap;
            const double rb = fma(-gaq, An, fma(-alq, Cp, 1.0));
            const double rc = -gaq * Cn;
            const double rd = fma(-gaq, Dn, fma(-alq, Dp, deq));
            const double bet = (q == 0) ? rb : fma(-ra, gq, rb);
            const double iv = rcp_full(bet);
            u = ((q == 0) ? rd : fma(-ra, u, rd)) * iv;
            gq = rc * iv;
            gm[q] = gq;
            z[q] = u;
        }
        for (int q = S - 2; q >= 0; q--)
            z[q] = fma(-gm[q], z[q + 1], z[q]);
        for (int q = 0; q < S; q++) {
            double *zq = cluster.map_shared_rank(zin, q);
            zq[j] = z[q];
            zq[L + j] = q ? z[q - 1] : 0.0;
        }
    }
    cluster.sync();
    if (j < L) {
        const double xl = zin[j], zp = zin[L + j];
        const double xf = fma(-xr[L + j], xl, fma(-xr[j], zp, xr[2 * L + j]));
        blk[j] = xf;
        blk[(m - 1) * pitch + j] = xl;
        for (int p = 1; p < m - 1; p++)
            blk[p * pitch + j] =
                fma(-ga[p * L + j], xl, fma(-al[p * L + j], xf, blk[p * pitch + j]));
    }
    __syncthreads();
}

// The y sweep of the CTA's rows; al, ga: L x C2_ROWS scratch ([c][p]); yr:
// C2_YSLOT x C2_YSEG x C2_ROWS doubles of the segments' systems.
__device__ __forceinline__ void c2_sweep_y(double *blk, int pitch, int L, int R0, int m,
                                           double *al, double *ga, double *yr,
                                           const AxisVecs &vv, const AxisScalars &s,
                                           const GridVecs &g, int j0, int j1)
{
    const int tid = threadIdx.x;
    const int p = tid % C2_ROWS, q = tid / C2_ROWS;
    const int mlen = L / C2_YSEG, extra = L % C2_YSEG;
    const int s0 = q * mlen + min(q, extra);
    const int ml = mlen + (q < extra ? 1 : 0);
    double *r8 = yr + (size_t)q * C2_YSLOT * C2_ROWS + p;
    double *ph = blk + (size_t)p * pitch;
    const bool live = p < m;
    if (live) {
        const int i = R0 + p;
        const double W = s.mig[0] * g.x[i];
        auto arow = [&](int c) { return (c > 0) ? fma(W, vv.A1[c], vv.A0[c]) : 0.0; };
        auto crow = [&](int c) { return (c < L - 1) ? fma(W, vv.C1[c], vv.C0[c]) : 0.0; };
        auto brow = [&](int c) {
            if (c == 0)
                return fma(W, s.B1s, vv.B0[0]) + (i == j0 ? s.bcs : 0.0);
            if (c == L - 1)
                return fma(W, s.B1e, vv.B0[L - 1]) + (i == j1 ? s.bce : 0.0);
            return vv.B0[c];
        };
        int c = s0 + 1;
        double aa = arow(c);
        double inv = rcp_full(brow(c));
        double alp = aa * inv, gap = crow(c) * inv, dep = ph[c] * inv;
        al[c * C2_ROWS + p] = alp;
        ga[c * C2_ROWS + p] = gap;
        ph[c] = dep;
        for (c = s0 + 2; c < s0 + ml; c++) {
            aa = arow(c);
            inv = rcp_full(fma(-aa, gap, brow(c)));
            alp = -aa * alp * inv;
            gap = crow(c) * inv;
            dep = fma(-aa, dep, ph[c]) * inv;
            al[c * C2_ROWS + p] = alp;
            ga[c * C2_ROWS + p] = gap;
            ph[c] = dep;
        }
        r8[3 * C2_ROWS] = alp;
        r8[4 * C2_ROWS] = gap;
        r8[5 * C2_ROWS] = dep;
        c = s0 + ml - 2;
        double deu = ph[c], alu = al[c * C2_ROWS + p], gau = ga[c * C2_ROWS + p];
        for (c = s0 + ml - 3; c >= s0 + 1; c--) {
            const double gg = ga[c * C2_ROWS + p];
            deu = fma(-gg, deu, ph[c]);
            alu = fma(-gg, alu, al[c * C2_ROWS + p]);
            gau = -gg * gau;
            ph[c] = deu;
            al[c * C2_ROWS + p] = alu;
            ga[c * C2_ROWS + p] = gau;
        }
        const double c0 = crow(s0);
        const double iB = rcp_full(fma(-c0, alu, brow(s0)));
        r8[0] = arow(s0) * iB;
        r8[1 * C2_ROWS] = (-c0 * gau) * iB;
        r8[2 * C2_ROWS] = fma(-c0, deu, ph[s0]) * iB;
    }
    __syncthreads();
    if (live) {
        const double Ap = r8[0], Cp = r8[C2_ROWS], Dp = r8[2 * C2_ROWS];
        const double alq = r8[3 * C2_ROWS], gaq = r8[4 * C2_ROWS], deq = r8[5 * C2_ROWS];
        double An = 0, Cn = 0, Dn = 0;
        if (q + 1 < C2_YSEG) {
            const double *rn = r8 + C2_YSLOT * C2_ROWS;
            An = rn[0];
            Cn = rn[C2_ROWS];
            Dn = rn[2 * C2_ROWS];
        }
        r8[3 * C2_ROWS] = -alq * Ap;
        r8[4 * C2_ROWS] = fma(-gaq, An, fma(-alq, Cp, 1.0));
        r8[5 * C2_ROWS] = -gaq * Cn;
        r8[6 * C2_ROWS] = fma(-gaq, Dn, fma(-alq, Dp, deq));
    }
    __syncthreads();
    if (live && q == 0) {
        double gm[C2_YSEG], z[C2_YSEG];
        double gq = 0, u = 0;
#pragma unroll
        for (int k = 0; k < C2_YSEG; k++) {
            const double *rr = yr + (size_t)k * C2_YSLOT * C2_ROWS + p;
            const double ra = rr[3 * C2_ROWS], rb = rr[4 * C2_ROWS];
            const double rc = rr[5 * C2_ROWS], rd = rr[6 * C2_ROWS];
            const double bet = (k == 0) ? rb : fma(-ra, gq, rb);
            const double iv = rcp_full(bet);
            u = ((k == 0) ? rd : fma(-ra, u, rd)) * iv;
            gq = rc * iv;
            gm[k] = gq;
            z[k] = u;
        }
#pragma unroll
        for (int k = C2_YSEG - 2; k >= 0; k--)
            z[k] = fma(-gm[k], z[k + 1], z[k]);
#pragma unroll
        for (int k = 0; k < C2_YSEG; k++)
            yr[((size_t)k * C2_YSLOT + 7) * C2_ROWS + p] = z[k];
    }
    __syncthreads();
    if (live) {
        const double xl = r8[7 * C2_ROWS];
        const double zp = q ? r8[7 * C2_ROWS - C2_YSLOT * C2_ROWS] : 0.0;
        const double xf = fma(-r8[C2_ROWS], xl, fma(-r8[0], zp, r8[2 * C2_ROWS]));
        ph[s0] = xf;
        ph[s0 + ml - 1] = xl;
        for (int c = s0 + 1; c < s0 + ml - 1; c++)
            ph[c] = fma(-ga[c * C2_ROWS + p], xl, fma(-al[c * C2_ROWS + p], xf, ph[c]));
    }
    __syncthreads();
}

} // namespace dgb
