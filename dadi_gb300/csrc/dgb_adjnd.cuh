// The transposed per-axis sweep of the N-dimensional adjoint and its
// contraction with the derivatives of the sweep's matrix (the method is
// described in dgb_adjointnd.cu): shared by the one-integration kernel there
// and the batched one in dgb_batchnd.cu.
#pragma once
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
    long rec_off;       // offset of this integration's records after the grid constants
};

// Shared memory of an adjoint sweep CTA: the forward sweep's (tile, gam
// unless it sits in a workspace slice, grid constants, vectors), the
// transposed vectors and four per-interval contraction factors.
__host__ __device__ inline size_t adn_smem_doubles(int L, int nt, bool gsmem = true)
{
    return (size_t)L * (nt + 1) + (gsmem ? (size_t)L * nt : 0) + 20 * (size_t)L;
}

// The transposed sweep and contraction of tile `tile_idx` (nt lines from
// tile_idx * nt) of one integration: the body of k_adjoint_sweep_nd and of the
// batched k_adjoint_sweep_batch.  Called by the whole CTA.
__device__ __forceinline__ void adn_tile(const ADNArgs &A, long tile_idx, double *smem,
                                         NDShared &Sh, double (*red)[8],
                                         double *gam_slice = nullptr)
{
    const NDArgs &N = A.nd;
    const int nt = blockDim.x, L = N.L, P = N.ndim, ax = N.axis, tid = threadIdx.x;
    const int stride = row_stride(P);
    double *tile, *gam;
    GridVecs g;
    AxisVecs v, vt;
    if (gam_slice) {
        // the Thomas scratch in this CTA's workspace slice: the shared
        // memory holds the tile and the vectors only
        tile = smem;
        gam = gam_slice;
        double *q = smem + (size_t)L * (nt + 1);
        g.x = q; q += L;
        g.xv = q; q += L;
        g.dfac = q; q += L;
        g.xInt = q; q += L;
        g.ih = q; q += L;
        g.dx = q; q += L;
        nd_vecs_at(q, L, false, v);
    } else {
        nd_carve(smem, L, nt, false, tile, gam, g, v);
    }
    double *p = v.B0 + L;
    vt.A1 = p; p += L;
    vt.A0 = p; p += L;
    vt.C1 = p; p += L;
    vt.C0 = p; p += L;
    vt.B0 = p; p += L;
    // per interval i, for the contraction below: cP, cQ (the nu terms), gS,
    // hS (the selection terms' gamma and h factors)
    double *cP = p, *cQ = p + L, *gS = p + 2 * L, *hS = p + 3 * L;
    if (A.coef) {
        // the grid constants and this step's record, in the carve order
        const double *rec = A.coef + nd_grid_doubles(L) + A.rec_off +
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
        if (i < L - 1) {
            // with w = D_i (u_i + u_{i+1}) (twice D_i times the mean density):
            // d/dnu: D_i (Q_i u_{i+1} - P_i u_i) / nu = D_i (cQ u_{i+1} - cP u_i);
            // d/dgamma, d/dh of the selection term times D_i hp: w gS, w hS
            const double inu = Sh.s.inv_nu, hh = Sh.s.h, gm = Sh.s.gamma;
            const double xi = g.xInt[i], xx1 = xi * (1. - xi);
            cP[i] = inu * inu * g.xv[i] * g.ih[i];
            cQ[i] = inu * inu * g.xv[i + 1] * g.ih[i];
            gS[i] = (hh + (1. - 2 * hh) * xi) * xx1;
            hS[i] = gm * (1. - 2 * xi) * xx1;
        }
    }
    const long l0 = tile_idx * nt;
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
        // the migration terms D_i (x_k - xInt_i) hp of every other population
        // k from two sums: s1 = sum w, s2 = sum w xInt_i
        double smr = 0, smp = 0, snu = 0, sg = 0, sh = 0, s1 = 0, s2 = 0;
        double mi = tile[tid], ui = u[0];
        double dmi = g.dfac[0] * mi;
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
                const double dmn = g.dfac[i + 1] * mn;
                const double Di = dmi - dmn;
                const double w = Di * (ui + un);
                snu = fma(Di, fma(-cP[i], ui, cQ[i] * un), snu);
                s1 += w;
                s2 = fma(w, g.xInt[i], s2);
                sg = fma(w, gS[i], sg);
                sh = fma(w, hS[i], sh);
                mi = mn;
                ui = un;
                dmi = dmn;
            }
        }
        double sm[DGB_MAX_DIM];
        for (int k = 0; k < P; k++)
            sm[k] = 0.5 * fma(oo[k], s1, -s2);
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
        A.gpart[(size_t)tile_idx * stride + tid] = x;
    }
}

// The injection's part of dJ/d(dt) and dJ/d(theta0) for one step (one
// thread): lambda (the adjoint at the start of the step) at the injected
// points times d(injected amount)/d(dt, theta0).
__device__ __forceinline__ void adn_inject_terms(const double *lam, const double *xx,
                                                 const double *row, int P, int L, int active,
                                                 double *gout)
{
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

} // namespace dgb
