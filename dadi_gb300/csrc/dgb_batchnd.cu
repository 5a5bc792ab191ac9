// Batched N-dimensional engine: many integrations of the same number of
// populations on the same grid advance together, so that a 3-D or 4-D sweep
// launch carries the lines of every integration instead of one (a single
// 3-D grid of 70-90 points has 4,900-8,100 lines: 150-250 warps, a quarter
// of the warps the FP64 pipe of 152 SMs needs).
//
// Per chunk of steps one launch writes the coefficient records of every
// (integration, step, swept axis) -- the grid constants, the parameter row,
// the per-axis vectors, as k_coef_nd does for one integration -- and then
// per step and axis one launch sweeps the lines of every integration still
// running (integrations are ordered longest first, so the running ones are a
// prefix).  Each CTA stages its lines in shared memory as k_sweep_nd_rec
// does; the Thomas gam scratch sits in shared memory or in a per-CTA slice
// of the workspace (L2), which leaves room for twice the CTAs per SM.
// Per line the arithmetic is that of k_sweep_nd_rec, so every integration's
// density is bitwise the one dgb_integrate_table computes alone.  Two other
// line solvers are selectable (dgb_settings.line_solver): warp-level
// parallel cyclic reduction and the partitioned Thomas solve; they agree
// with Thomas to rounding, and the partition is the faster one for a lone
// grid whose few lines leave the FP64 pipes idle.
//
// Replaces many calls of Integration.three_pops / four_pops / five_pops
// (dadi/Integration.py:389-554, 556-727, 729-937), which the reference runs
// one at a time, or as host processes (dadi/DFE/Cache2D_mod.py:117-167).
#include <algorithm>
#include <cmath>

#include <vector>

#include "dgb_adjnd.cuh"

namespace dgb {

struct NDBatch {
    NDArgs A; // shared shape: ndim, L, axis, nlines, S, LS, xx
    const dgb_itemnd *items;
    double *phi_all;
    const double *table;
    double *coef;      // grid constants, then one block of records per integration
    long item_coef;    // doubles of one integration's block (chunk x ndim records)
    long step0;        // first step of the current chunk
    int chunk;         // steps per chunk
    int bpi;           // CTAs per integration in a sweep launch
    double *gam_glob;  // per-CTA gam slices (null: shared memory)
};

__device__ __forceinline__ int first_swept(int frozen)
{
    int f = 0;
    while (f < DGB_MAX_DIM && (frozen >> f & 1))
        f++;
    return f;
}

// One CTA per (integration, step of the chunk, axis): the record of
// k_coef_nd for that integration's table row.
template <bool DELJ>
__global__ void k_coef_batch(NDBatch B, int nsl)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ NDShared Sh;
    const int P = B.A.ndim, L = B.A.L;
    const long b = blockIdx.x;
    const int ax = (int)(b % P);
    const long sl = (b / P) % nsl;
    const long it = b / ((long)P * nsl);
    const dgb_itemnd I = B.items[it];
    const int frozen = I.masks & 0xff, nomut = (I.masks >> 8) & 0xff;
    GridVecs g;
    g.x = smem;
    g.xv = smem + L;
    g.dfac = smem + 2 * L;
    g.xInt = smem + 3 * L;
    g.ih = smem + 4 * L;
    g.dx = smem + 5 * L;
    NDArgs A = B.A;
    A.axis = ax;
    A.table = B.table + I.row_off * row_stride(P);
    A.step = B.step0 + sl;
    A.inject_mask = (ax == first_swept(frozen)) ? (((1 << P) - 1) & ~frozen & ~nomut) : 0;
    nd_grid_consts(A, g);
    if (b == 0)
        for (int i = threadIdx.x; i < nd_grid_doubles(L); i += blockDim.x)
            B.coef[i] = smem[i];
    if (A.step >= I.nsteps || (frozen >> ax & 1))
        return; // the whole CTA: no barrier is skipped by part of it
    if (threadIdx.x == 0)
        nd_load_params(A, Sh, g);
    __syncthreads();
    double *rec = B.coef + nd_grid_doubles(L) + it * B.item_coef +
                  ((size_t)sl * P + ax) * nd_rec_doubles(L, DELJ);
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
}

// One sweep along B.A.axis at `step` over the lines of every running
// integration: CTA b handles tile b % bpi of integration b / bpi.
template <bool DELJ, bool GSMEM>
__global__ void k_sweep_batch(NDBatch B, long step)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ NDRecHead H;
    const int nt = blockDim.x, L = B.A.L, P = B.A.ndim;
    constexpr int NV = DELJ ? 10 : 5;
    const long it = blockIdx.x / B.bpi;
    const long tl = blockIdx.x - it * B.bpi;
    const dgb_itemnd I = B.items[it];
    const int frozen = I.masks & 0xff, nomut = (I.masks >> 8) & 0xff;
    if (step >= I.nsteps || (frozen >> B.A.axis & 1))
        return;
    NDArgs A = B.A;
    A.phi = B.phi_all + I.phi_off;
    A.inject_mask =
        (A.axis == first_swept(frozen)) ? (((1 << P) - 1) & ~frozen & ~nomut) : 0;
    double *tile = smem;
    double *gam, *gx;
    if (GSMEM) {
        gam = tile + (size_t)L * (nt + 1);
        gx = gam + (size_t)L * nt;
    } else {
        gam = B.gam_glob + (size_t)blockIdx.x * L * nt;
        gx = tile + (size_t)L * (nt + 1);
    }
    double *vv = gx + 3 * (size_t)L;
    const double *rec = B.coef + nd_grid_doubles(L) + it * B.item_coef +
                        ((size_t)(step - B.step0) * P + A.axis) * nd_rec_doubles(L, DELJ);
    double *hp = reinterpret_cast<double *>(&H);
    for (int i = threadIdx.x; i < ND_HEAD; i += nt)
        hp[i] = rec[i];
    for (int i = threadIdx.x; i < NV * L; i += nt)
        vv[i] = rec[ND_HEAD + i];
    for (int i = threadIdx.x; i < L; i += nt) {
        gx[i] = B.coef[i];
        if (DELJ) {
            gx[L + i] = B.coef[3 * L + i];
            gx[2 * L + i] = B.coef[5 * L + i];
        }
    }
    GridVecs g = {};
    g.x = gx;
    g.xInt = gx + L;
    g.dx = gx + 2 * L;
    AxisVecs v;
    nd_vecs_at(vv, L, DELJ, v);
    const long l0 = tl * nt;
    const int n = (int)min((long)nt, A.nlines - l0);
    nd_tile_io(A, tile, nt, l0, n, false);
    __syncthreads();
    nd_solve_tile<DELJ>(A, tile, gam, nt, l0, n, g, v, H.s, H.inj);
    __syncthreads();
    nd_tile_io(A, tile, nt, l0, n, true);
}


// The alternative line solver: parallel cyclic reduction (Hockney's odd-even
// reduction in its parallel form), one warp per line, PCR_LINES lines per
// CTA.  The rows are those of the Thomas path (dt-scaled, affine in the
// line's migration weight W, corner terms); level s combines row p with rows
// p - s and p + s,
//     k1 = a_p / b_{p-s},  k2 = c_p / b_{p+s},
//     a'_p = -a_{p-s} k1,  c'_p = -c_{p+s} k2,
//     b'_p = b_p - c_{p-s} k1 - a_{p+s} k2,  d'_p = d_p - d_{p-s} k1 - d_{p+s} k2,
// until every row stands alone (ceil(log2 L) levels) and x_p = d_p / b_p.
// About 11 FP64 instructions per row and level against 10 per row for the
// whole Thomas solve, in exchange for 32 lanes per line.  L <= 128 (four rows
// per lane); the default delta_j only.
constexpr int PCR_LINES = 4;

__global__ void __launch_bounds__(32 * PCR_LINES) k_sweep_batch_pcr(NDBatch B, long step)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ NDRecHead H;
    const int L = B.A.L, P = B.A.ndim;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long it = blockIdx.x / B.bpi;
    const long tl = blockIdx.x - it * B.bpi;
    const dgb_itemnd I = B.items[it];
    const int frozen = I.masks & 0xff, nomut = (I.masks >> 8) & 0xff;
    if (step >= I.nsteps || (frozen >> B.A.axis & 1))
        return;
    NDArgs A = B.A;
    A.phi = B.phi_all + I.phi_off;
    const int inject =
        (A.axis == first_swept(frozen)) ? (((1 << P) - 1) & ~frozen & ~nomut) : 0;
    double *vv = smem;          // A1, A0, C1, C0, B0
    double *gx = vv + 5 * L;    // x
    const double *rec = B.coef + nd_grid_doubles(L) + it * B.item_coef +
                        ((size_t)(step - B.step0) * P + A.axis) * nd_rec_doubles(L, false);
    double *hp = reinterpret_cast<double *>(&H);
    for (int i = tid; i < ND_HEAD; i += blockDim.x)
        hp[i] = rec[i];
    for (int i = tid; i < 5 * L; i += blockDim.x)
        vv[i] = rec[ND_HEAD + i];
    for (int i = tid; i < L; i += blockDim.x)
        gx[i] = B.coef[i];
    __syncthreads();
    AxisVecs v;
    nd_vecs_at(vv, L, false, v);
    const AxisScalars &s = H.s;
    const long line = tl * PCR_LINES + warp;
    if (line >= A.nlines)
        return; // the warp alone: no CTA barrier follows
    int coord[DGB_MAX_DIM];
    const long base = nd_line_base(A, line, coord);
    const int j0 = (gx[0] == 0.0) ? 0 : -1;
    const int j1 = (gx[L - 1] == 1.0) ? L - 1 : -1;
    double W = 0;
    bool all0 = true, all1 = true;
    int n1 = 0, k1 = -1;
    for (int k = 0; k < P; k++) {
        if (k == A.axis)
            continue;
        W = fma(s.mig[k], gx[coord[k]], W);
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
    double *a = gx + L + (size_t)warp * 5 * L;
    double *b = a + L, *c = b + L, *d = c + L, *ib = d + L;
    for (int p = lane; p < L; p += 32) {
        double dv = A.phi[base + p * A.S];
        if (inject) {
            if (p == 1 && n1 == 0)
                dv += H.inj[A.axis];
            if (p == 0 && n1 == 1)
                dv += H.inj[k1];
        }
        d[p] = dv;
        a[p] = (p > 0) ? fma(W, v.A1[p], v.A0[p]) : 0.0;
        c[p] = (p < L - 1) ? fma(W, v.C1[p], v.C0[p]) : 0.0;
        double bv = v.B0[p];
        if (p == 0)
            bv = fma(W, s.B1s, v.B0[0]) + bs;
        else if (p == L - 1)
            bv = fma(W, s.B1e, v.B0[L - 1]) + be;
        b[p] = bv;
    }
    __syncwarp();
    for (int sh = 1; sh < L; sh <<= 1) {
        for (int p = lane; p < L; p += 32)
            ib[p] = rcp_full(b[p]);
        __syncwarp();
        double na[4], nb[4], nc[4], nd[4];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int p = lane + 32 * r;
            if (p >= L)
                break;
            const int pm = p - sh, pp = p + sh;
            double bb = b[p], dd = d[p], aa = 0.0, cc = 0.0;
            if (pm >= 0) {
                const double q = a[p] * ib[pm];
                aa = -a[pm] * q;
                bb = fma(-c[pm], q, bb);
                dd = fma(-d[pm], q, dd);
            }
            if (pp < L) {
                const double q = c[p] * ib[pp];
                cc = -c[pp] * q;
                bb = fma(-a[pp], q, bb);
                dd = fma(-d[pp], q, dd);
            }
            na[r] = aa;
            nb[r] = bb;
            nc[r] = cc;
            nd[r] = dd;
        }
        __syncwarp();
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int p = lane + 32 * r;
            if (p >= L)
                break;
            a[p] = na[r];
            b[p] = nb[r];
            c[p] = nc[r];
            d[p] = nd[r];
        }
        __syncwarp();
    }
    for (int p = lane; p < L; p += 32)
        A.phi[base + p * A.S] = d[p] * rcp_full(b[p]);
}

// The second alternative: partitioned Thomas (the partition method of
// H. H. Wang, ACM TOMS 7 (1981) 170-183, in the two-sweep "modified Thomas"
// form used for batched GPU solvers by Laszlo, Giles and Appleyard, ACM TOMS
// 42 (2016) 31).  Each line is cut into SEG segments, one thread each (warp
// q of the CTA holds segment q of the CTA's 32 lines), so a launch over one
// grid carries SEG times the threads of the Thomas sweep.  Per segment of
// rows s0 .. s0+m-1 (local j = 0 .. m-1, rows as in the Thomas path):
//   downward, j >= 1: every row becomes  al_j x_0 + x_j + ga_j x_{j+1} = de_j
//     (j = 1: al = a/b, ga = c/b, de = d/b; then with r = 1/(b_j - a_j ga_{j-1}):
//      al_j = -a_j al_{j-1} r, ga_j = c_j r, de_j = (d_j - a_j de_{j-1}) r);
//   upward, j <= m-3: x_j = de_j - al_j x_0 - ga_j x_{m-1}
//     (de_j -= ga_j de_{j+1}, al_j -= ga_j al_{j+1}, ga_j = -ga_j ga_{j+1});
//   row 0 with x_1 substituted:  a_0 x_prev + (b_0 - c_0 al_1) x_0
//                                - c_0 ga_1 x_{m-1} = d_0 - c_0 de_1,
//     i.e. x_0 = D' - A' z_{q-1} - C' z_q with z_q = x_{m-1} of segment q;
//   row m-1 as it stands:        al x_0 + x_{m-1} + ga x_next = de.
// Putting x_0 of segments q and q+1 into row m-1 of segment q leaves a
// tridiagonal system in the segments' last points z_0 .. z_{SEG-1},
//     -al A'_q z_{q-1} + (1 - al C'_q - ga A'_{q+1}) z_q - ga C'_{q+1} z_{q+1}
//         = de - al D'_q - ga D'_{q+1},
// each row formed by its segment's thread, the SEG rows solved by one
// thread per line; then x_0 and x_j = de_j - al_j x_0 - ga_j x_{m-1}
// inside.  About 17 FP64 instructions per row against 10 for Thomas.
// Default delta_j only; segments of at least three rows.
constexpr int PART_LINES = 32;
// Per (segment, line): A' C' D', then al ga de (replaced by the row of the
// system in the last points, read only by the segment's own thread), then z.
constexpr int PART_SLOTS = 8;

__host__ __device__ inline size_t part_smem_doubles(int L, int seg)
{
    return (size_t)6 * L + (size_t)L * (PART_LINES + 1) + (size_t)2 * L * PART_LINES +
           (size_t)PART_SLOTS * seg * PART_LINES;
}

template <int SEG>
__global__ void __launch_bounds__(32 * SEG) k_sweep_batch_part(NDBatch B, long step)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ NDRecHead H;
    const int L = B.A.L, P = B.A.ndim;
    constexpr int nt = PART_LINES, tp = PART_LINES + 1;
    const int tid = threadIdx.x, q = tid >> 5, t = tid & 31;
    const long it = blockIdx.x / B.bpi;
    const long tl = blockIdx.x - it * B.bpi;
    const dgb_itemnd I = B.items[it];
    const int frozen = I.masks & 0xff, nomut = (I.masks >> 8) & 0xff;
    if (step >= I.nsteps || (frozen >> B.A.axis & 1))
        return;
    NDArgs A = B.A;
    A.phi = B.phi_all + I.phi_off;
    const int inject =
        (A.axis == first_swept(frozen)) ? (((1 << P) - 1) & ~frozen & ~nomut) : 0;
    double *vv = smem;                        // A1, A0, C1, C0, B0
    double *gx = vv + 5 * L;                  // x
    double *tile = gx + L;                    // d, then de, then x
    double *al = tile + (size_t)L * tp;       // al_j
    double *ga = al + (size_t)L * nt;         // ga_j
    double *red = ga + (size_t)L * nt;        // PART_SLOTS per (segment, line)
    const double *rec = B.coef + nd_grid_doubles(L) + it * B.item_coef +
                        ((size_t)(step - B.step0) * P + A.axis) * nd_rec_doubles(L, false);
    double *hp = reinterpret_cast<double *>(&H);
    for (int i = tid; i < ND_HEAD; i += blockDim.x)
        hp[i] = rec[i];
    for (int i = tid; i < 5 * L; i += blockDim.x)
        vv[i] = rec[ND_HEAD + i];
    for (int i = tid; i < L; i += blockDim.x)
        gx[i] = B.coef[i];
    // this thread's segment
    const int mlen = L / SEG, extra = L % SEG;
    const int s0 = q * mlen + min(q, extra);
    const int m = mlen + (q < extra ? 1 : 0);
    const long l0 = tl * nt;
    const int n = (int)min((long)nt, A.nlines - l0);
    if (A.S == 1) {
        // contiguous lines: each warp copies whole lines, lanes along the line
        const double *g0 = A.phi + l0 * L;
        for (int w = q; w < n; w += SEG)
            for (int p = t; p < L; p += 32)
                tile[p * tp + w] = g0[(size_t)w * L + p];
    } else if (t < n) {
        const long line = l0 + t;
        const long outer = line / A.S, inner = line - outer * A.S;
        const double *g0 = A.phi + outer * A.LS + inner;
        for (int p = s0; p < s0 + m; p++)
            tile[p * tp + t] = g0[p * A.S];
    }
    __syncthreads();
    AxisVecs v;
    nd_vecs_at(vv, L, false, v);
    const AxisScalars &s = H.s;
    double *r8 = red + (size_t)q * PART_SLOTS * nt + t; // this segment's slots, stride nt
    if (t < n) {
        int coord[DGB_MAX_DIM];
        nd_line_base(A, l0 + t, coord);
        const int j0 = (gx[0] == 0.0) ? 0 : -1;
        const int j1 = (gx[L - 1] == 1.0) ? L - 1 : -1;
        double W = 0;
        bool all0 = true, all1 = true;
        int n1 = 0, k1 = -1;
        for (int k = 0; k < P; k++) {
            if (k == A.axis)
                continue;
            W = fma(s.mig[k], gx[coord[k]], W);
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
        if (inject && q == 0) {
            if (n1 == 0 && H.inj[A.axis] != 0.0)
                tile[1 * tp + t] += H.inj[A.axis];
            if (n1 == 1 && H.inj[k1] != 0.0)
                tile[0 * tp + t] += H.inj[k1];
        }
        auto arow = [&](int p) { return (p > 0) ? fma(W, v.A1[p], v.A0[p]) : 0.0; };
        auto crow = [&](int p) { return (p < L - 1) ? fma(W, v.C1[p], v.C0[p]) : 0.0; };
        auto brow = [&](int p) {
            if (p == 0)
                return fma(W, s.B1s, v.B0[0]) + (all0 ? s.bcs : 0.0);
            if (p == L - 1)
                return fma(W, s.B1e, v.B0[L - 1]) + (all1 ? s.bce : 0.0);
            return v.B0[p];
        };
        // downward
        int p = s0 + 1;
        double inv = rcp_full(brow(p));
        double a = arow(p);
        double alp = a * inv, gap = crow(p) * inv, dep = tile[p * tp + t] * inv;
        al[p * nt + t] = alp;
        ga[p * nt + t] = gap;
        tile[p * tp + t] = dep;
        for (p = s0 + 2; p < s0 + m; p++) {
            a = arow(p);
            inv = rcp_full(fma(-a, gap, brow(p)));
            alp = -a * alp * inv;
            gap = crow(p) * inv;
            dep = fma(-a, dep, tile[p * tp + t]) * inv;
            al[p * nt + t] = alp;
            ga[p * nt + t] = gap;
            tile[p * tp + t] = dep;
        }
        // the segment's last row, as it stands
        r8[3 * nt] = alp;
        r8[4 * nt] = gap;
        r8[5 * nt] = dep;
        // upward, from row m-3: ga_j now couples to x_{m-1}
        p = s0 + m - 2;
        double deu = tile[p * tp + t], alu = al[p * nt + t], gau = ga[p * nt + t];
        for (p = s0 + m - 3; p >= s0 + 1; p--) {
            const double g = ga[p * nt + t];
            deu = fma(-g, deu, tile[p * tp + t]);
            alu = fma(-g, alu, al[p * nt + t]);
            gau = -g * gau;
            tile[p * tp + t] = deu;
            al[p * nt + t] = alu;
            ga[p * nt + t] = gau;
        }
        // row 0 with x_1 substituted, solved for x_0
        const double c0 = crow(s0);
        const double iB = rcp_full(fma(-c0, alu, brow(s0)));
        r8[0] = arow(s0) * iB;
        r8[1 * nt] = (-c0 * gau) * iB;
        r8[2 * nt] = fma(-c0, deu, tile[s0 * tp + t]) * iB;
    }
    __syncthreads();
    if (t < n) {
        // this segment's row of the system in the last points
        const double Ap = r8[0], Cp = r8[nt], Dp = r8[2 * nt];
        const double alq = r8[3 * nt], gaq = r8[4 * nt], deq = r8[5 * nt];
        double An = 0, Cn = 0, Dn = 0;
        if (q + 1 < SEG) {
            const double *rn = r8 + PART_SLOTS * nt;
            An = rn[0];
            Cn = rn[nt];
            Dn = rn[2 * nt];
        }
        r8[3 * nt] = -alq * Ap;
        r8[4 * nt] = fma(-gaq, An, fma(-alq, Cp, 1.0));
        r8[5 * nt] = -gaq * Cn;
        r8[6 * nt] = fma(-gaq, Dn, fma(-alq, Dp, deq));
    }
    __syncthreads();
    if (q == 0 && t < n) {
        // Thomas on the SEG rows: z_k = the last point of segment k
        double gm[SEG], z[SEG];
        double g = 0, u = 0;
#pragma unroll
        for (int k = 0; k < SEG; k++) {
            const double *rr = red + (size_t)k * PART_SLOTS * nt + t;
            const double ra = rr[3 * nt], rb = rr[4 * nt], rc = rr[5 * nt], rd = rr[6 * nt];
            const double bet = (k == 0) ? rb : fma(-ra, g, rb);
            const double iv = rcp_full(bet);
            u = ((k == 0) ? rd : fma(-ra, u, rd)) * iv;
            g = rc * iv;
            gm[k] = g;
            z[k] = u;
        }
#pragma unroll
        for (int k = SEG - 2; k >= 0; k--)
            z[k] = fma(-gm[k], z[k + 1], z[k]);
#pragma unroll
        for (int k = 0; k < SEG; k++)
            red[(size_t)k * PART_SLOTS * nt + 7 * nt + t] = z[k];
    }
    __syncthreads();
    if (t < n) {
        const double xl = r8[7 * nt];
        const double zp = q ? r8[7 * nt - PART_SLOTS * nt] : 0.0;
        const double xf = fma(-r8[nt], xl, fma(-r8[0], zp, r8[2 * nt]));
        tile[s0 * tp + t] = xf;
        tile[(s0 + m - 1) * tp + t] = xl;
        for (int p = s0 + 1; p < s0 + m - 1; p++)
            tile[p * tp + t] = fma(-ga[p * nt + t], xl,
                                   fma(-al[p * nt + t], xf, tile[p * tp + t]));
    }
    __syncthreads();
    if (A.S == 1) {
        double *g0 = A.phi + l0 * L;
        for (int w = q; w < n; w += SEG)
            for (int p = t; p < L; p += 32)
                g0[(size_t)w * L + p] = tile[p * tp + w];
    } else if (t < n) {
        const long line = l0 + t;
        const long outer = line / A.S, inner = line - outer * A.S;
        double *g0 = A.phi + outer * A.LS + inner;
        for (int p = s0; p < s0 + m; p++)
            g0[p * A.S] = tile[p * tp + t];
    }
}

// ------------------------------------------------------------ host side

struct BatchPlan {
    int pcr;       // parallel cyclic reduction (one warp per line)
    int seg;       // partitioned Thomas: segments per line (0: not used)
    int nt;        // lines per CTA
    int gsmem;     // gam in shared memory
    int chunk;     // steps per record chunk
    int bpi;       // CTAs per integration
    size_t smem;   // dynamic shared memory of a sweep CTA
    size_t coef_doubles;
    size_t gam_doubles;
};

static size_t batch_sweep_smem(int L, int nt, bool delj, bool gsmem)
{
    return ((size_t)L * (nt + 1) + (gsmem ? (size_t)L * nt : 0) + 3 * (size_t)L +
            (size_t)(delj ? 10 : 5) * L) *
           sizeof(double);
}

// Records of at most ~64 MB per chunk, 1..64 steps.
static int batch_chunk(int ndim, int L, int nitems)
{
    const size_t per = (size_t)nitems * ndim * nd_rec_doubles(L, true) * sizeof(double);
    size_t c = ((size_t)64 << 20) / std::max<size_t>(per, 1);
    return (int)std::max<size_t>(1, std::min<size_t>(64, c));
}

static int batch_plan(int ndim, int L, int nitems, const dgb_settings *st, BatchPlan &p)
{
    const long nlines = ipow(L, ndim - 1);
    p.pcr = st && st->line_solver == 1;
    p.seg = 0;
    if (p.pcr) {
        if (L > 128 || st->use_delj_trick)
            return DGB_ERR_UNSUPPORTED;
        p.gsmem = 0;
        p.nt = PCR_LINES;
        p.bpi = (int)((nlines + PCR_LINES - 1) / PCR_LINES);
        p.chunk = batch_chunk(ndim, L, nitems);
        p.smem = (6 + 5 * PCR_LINES) * (size_t)L * sizeof(double);
        p.coef_doubles = (size_t)nd_grid_doubles(L) +
                         (size_t)nitems * p.chunk * ndim * nd_rec_doubles(L, false);
        p.gam_doubles = 0;
        return DGB_OK;
    }
    if (st && st->line_solver == 2) {
        const int seg = st->segments ? st->segments : 4;
        if (seg != 2 && seg != 4 && seg != 8)
            return DGB_ERR_ARG;
        if (L < 3 * seg || st->use_delj_trick)
            return DGB_ERR_UNSUPPORTED;
        int optin = 0, dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
                cudaSuccess)
            return DGB_ERR_CUDA;
        p.seg = seg;
        p.gsmem = 0;
        p.nt = PART_LINES;
        p.bpi = (int)((nlines + PART_LINES - 1) / PART_LINES);
        p.chunk = batch_chunk(ndim, L, nitems);
        p.smem = part_smem_doubles(L, seg) * sizeof(double);
        if (p.smem + sizeof(NDRecHead) + 1024 > (size_t)optin)
            return DGB_ERR_UNSUPPORTED;
        p.coef_doubles = (size_t)nd_grid_doubles(L) +
                         (size_t)nitems * p.chunk * ndim * nd_rec_doubles(L, false);
        p.gam_doubles = 0;
        return DGB_OK;
    }
    if (st && st->line_solver != 0)
        return DGB_ERR_ARG;
    int nt = st ? st->threads : 0;
    if (nt != 32 && nt != 64 && nt != 128)
        nt = (L <= 48) ? 128 : 64;
    if (nlines < nt)
        nt = (int)std::max<long>(32, (nlines + 31) / 32 * 32);
    const bool delj = st && st->use_delj_trick;
    int gp = st ? st->gam_placement : 0;
    int optin = 0, dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return DGB_ERR_CUDA;
    const size_t need_s = batch_sweep_smem(L, nt, delj, true) + sizeof(NDRecHead) + 1024;
    const size_t need_g = batch_sweep_smem(L, nt, delj, false) + sizeof(NDRecHead) + 1024;
    if (need_g > (size_t)optin)
        return DGB_ERR_UNSUPPORTED;
    if (gp == 1 && need_s > (size_t)optin)
        return DGB_ERR_UNSUPPORTED;
    p.gsmem = (gp == 1) ? 1 : 0; // auto: the workspace (twice the CTAs per SM)
    p.nt = nt;
    p.bpi = (int)((nlines + nt - 1) / nt);
    p.chunk = batch_chunk(ndim, L, nitems);
    p.smem = batch_sweep_smem(L, nt, delj, p.gsmem);
    p.coef_doubles = (size_t)nd_grid_doubles(L) +
                     (size_t)nitems * p.chunk * ndim * nd_rec_doubles(L, delj);
    p.gam_doubles = p.gsmem ? 0 : (size_t)nitems * p.bpi * nt * L;
    return DGB_OK;
}

template <int SEG>
static int batch_part_launch(NDBatch &B, long nact, size_t smem, long step, cudaStream_t st)
{
    if (raise_smem_limit(k_sweep_batch_part<SEG>))
        return DGB_ERR_CUDA;
    k_sweep_batch_part<SEG><<<(unsigned)(nact * B.bpi), 32 * SEG, smem, st>>>(B, step);
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

template <bool DELJ, bool GSMEM>
static int batch_sweep_launch(NDBatch &B, long nact, size_t smem, int nt, long step,
                              cudaStream_t st)
{
    if (raise_smem_limit(k_sweep_batch<DELJ, GSMEM>))
        return DGB_ERR_CUDA;
    k_sweep_batch<DELJ, GSMEM><<<(unsigned)(nact * B.bpi), nt, smem, st>>>(B, step);
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

} // namespace dgb

using namespace dgb;

extern "C" size_t dgb_batchnd_workspace_bytes(int ndim, int L, int nitems,
                                              const dgb_settings *settings)
{
    if (!shape_ok(ndim, L) || nitems < 1)
        return 0;
    BatchPlan p;
    if (batch_plan(ndim, L, nitems, settings, p))
        return 0;
    return (p.coef_doubles + p.gam_doubles) * sizeof(double) + 256;
}

namespace dgb {

// The records kernel's shared memory (the grid constants).
static int batch_coef_prepare(bool delj, size_t &csmem, int L)
{
    csmem = (size_t)nd_grid_doubles(L) * sizeof(double);
    return (delj ? raise_smem_limit(k_coef_batch<true>) : raise_smem_limit(k_coef_batch<false>))
               ? DGB_ERR_CUDA
               : DGB_OK;
}

// One sweep along B.A.axis at step s over the first nact items, with the
// plan's line solver.
static int batch_sweep(NDBatch &B, const BatchPlan &p, long nact, long s, bool delj,
                       cudaStream_t st)
{
    if (p.pcr) {
        k_sweep_batch_pcr<<<(unsigned)(nact * B.bpi), 32 * PCR_LINES, p.smem, st>>>(B, s);
        return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
    }
    if (p.seg)
        return (p.seg == 2)   ? batch_part_launch<2>(B, nact, p.smem, s, st)
               : (p.seg == 4) ? batch_part_launch<4>(B, nact, p.smem, s, st)
                              : batch_part_launch<8>(B, nact, p.smem, s, st);
    if (delj)
        return p.gsmem ? batch_sweep_launch<true, true>(B, nact, p.smem, p.nt, s, st)
                       : batch_sweep_launch<true, false>(B, nact, p.smem, p.nt, s, st);
    return p.gsmem ? batch_sweep_launch<false, true>(B, nact, p.smem, p.nt, s, st)
                   : batch_sweep_launch<false, false>(B, nact, p.smem, p.nt, s, st);
}

static void batch_set_axis(NDBatch &B, int ax)
{
    B.A.axis = ax;
    B.A.S = ipow(B.A.L, B.A.ndim - 1 - ax);
    B.A.LS = B.A.S * B.A.L;
}

// Densities recorded by the batched forward of the adjoint: before step s
// of every item with s <= nsteps (s == nsteps: its final density),
// states[state_off + s N] = phi_all[phi_off].  blockIdx.y = item.
__global__ void k_store_states(const dgb_itemnd_adj *items, const double *phi_all,
                               double *states_all, long s, long N)
{
    const dgb_itemnd_adj I = items[blockIdx.y];
    if (s > I.nsteps)
        return;
    const double *src = phi_all + I.phi_off;
    double *dst = states_all + I.state_off + s * N;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += (long)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// The time loop of a batch: records per chunk of steps, one sweep launch per
// step and axis over the items still running; with `adj` (the same items as
// adjoint records, device) every density is recorded as k_store_states
// says.
static int batch_loop(NDBatch &B, const BatchPlan &p, const int *nsteps, int nitems, bool delj,
                      const dgb_itemnd_adj *adj, double *states_all, cudaStream_t st)
{
    const int ndim = B.A.ndim, L = B.A.L;
    const long N = ipow(L, ndim);
    size_t csmem;
    if (batch_coef_prepare(delj, csmem, L))
        return DGB_ERR_CUDA;
    long nact = nitems;
    const long total = nsteps[0];
    for (long s = 0; s <= total; s++) {
        if (adj) {
            long nrec = nitems; // items with s <= nsteps: a prefix
            while (nrec > 0 && nsteps[nrec - 1] < s)
                nrec--;
            const dim3 grid((unsigned)std::min<long>((N + 255) / 256, 64), (unsigned)nrec);
            k_store_states<<<grid, 256, 0, st>>>(adj, B.phi_all, states_all, s, N);
            if (cudaGetLastError() != cudaSuccess)
                return DGB_ERR_CUDA;
        }
        if (s == total)
            break;
        while (nact > 0 && nsteps[nact - 1] <= s)
            nact--;
        if (s % p.chunk == 0) {
            B.step0 = s;
            const int nsl = (int)std::min<long>(p.chunk, total - s);
            const unsigned grid = (unsigned)(nact * nsl * ndim);
            if (delj)
                k_coef_batch<true><<<grid, 128, csmem, st>>>(B, nsl);
            else
                k_coef_batch<false><<<grid, 128, csmem, st>>>(B, nsl);
            if (cudaGetLastError() != cudaSuccess)
                return DGB_ERR_CUDA;
        }
        for (int ax = 0; ax < ndim; ax++) {
            batch_set_axis(B, ax);
            int rc = batch_sweep(B, p, nact, s, delj, st);
            if (rc)
                return rc;
        }
    }
    return DGB_OK;
}

} // namespace dgb

extern "C" int dgb_batchnd_integrate(const dgb_itemnd *items, const int *nsteps, int nitems,
                                     int ndim, int L, const double *xx, double *phi_all,
                                     const double *table, const dgb_settings *settings,
                                     void *ws, size_t ws_bytes, void *stream)
{
    if (!items || !nsteps || nitems < 1 || !xx || !phi_all || !table || !settings ||
        !shape_ok(ndim, L))
        return DGB_ERR_ARG;
    for (int i = 0; i < nitems; i++)
        if (nsteps[i] < 0 || (i > 0 && nsteps[i] > nsteps[i - 1]))
            return DGB_ERR_ARG; // longest first
    if (nsteps[0] == 0)
        return DGB_OK;
    BatchPlan p;
    int rc = batch_plan(ndim, L, nitems, settings, p);
    if (rc)
        return rc;
    if (!ws || ws_bytes < (p.coef_doubles + p.gam_doubles) * sizeof(double))
        return DGB_ERR_WORKSPACE;
    const bool delj = settings->use_delj_trick != 0;
    NDBatch B = {};
    nd_fill(B.A, phi_all, ndim, L, 0, xx);
    B.items = items;
    B.phi_all = phi_all;
    B.table = table;
    B.coef = (double *)ws;
    B.chunk = p.chunk;
    B.item_coef = (long)p.chunk * ndim * (long)nd_rec_doubles(L, delj);
    B.bpi = p.bpi;
    B.gam_glob = p.gsmem ? nullptr : (double *)ws + p.coef_doubles;
    return batch_loop(B, p, nsteps, nitems, delj, nullptr, nullptr, (cudaStream_t)stream);
}

// ------------------------------------------------- the batched adjoint

namespace dgb {

// First and last unfrozen axis of an integration.
__host__ __device__ inline int first_active(int frozen, int P)
{
    for (int a = 0; a < P; a++)
        if (!(frozen >> a & 1))
            return a;
    return P;
}
__host__ __device__ inline int last_active(int frozen, int P)
{
    for (int a = P - 1; a >= 0; a--)
        if (!(frozen >> a & 1))
            return a;
    return -1;
}

// The recomputation of step k's intermediate sweep outputs, per item in
// its scratch slots (slot a = the density after the step's sweep of axis
// a): slot[ax] = (ax == 0 ? states[k] : slot[ax - 1]) before the sweep of
// axis ax is run on it in place (a frozen axis leaves the copy, so slot[a]
// is always the output of the last unfrozen axis <= a).  blockIdx.y = item.
__global__ void k_slot_copy(const dgb_itemnd_adj *items, const double *states_all,
                            double *scratch, long slot_stride, long k, int ax, long N)
{
    const dgb_itemnd_adj I = items[blockIdx.y];
    if (k >= I.nsteps)
        return;
    double *base = scratch + (long)blockIdx.y * slot_stride;
    const double *src = ax ? base + (long)(ax - 1) * N : states_all + I.state_off + k * N;
    double *dst = base + (long)ax * N;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += (long)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

struct ADNBatch {
    ADNArgs a; // shape, axis, step, records (coef, step0); per item below
    const dgb_itemnd_adj *items;
    double *lam_all;
    const double *states_all, *scratch;
    double *gpart_all;
    double *gam; // per-CTA Thomas scratch slices of L x nt doubles
    long N, slot_stride, item_coef, per_step;
    int bpi, nb;
};

// The transposed sweep of axis a.nd.axis at step a.nd.step for the tiles of
// every running integration: CTA b handles tile b % bpi of item b / bpi,
// the per-line work of k_adjoint_sweep_nd on that item's lambda, recorded
// and recomputed densities, records and partial rows.
__global__ void k_adjoint_sweep_batch(ADNBatch B)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ NDShared Sh;
    __shared__ double red[ADN_MAXQ][8];
    const long it = blockIdx.x / B.bpi;
    const long tl = blockIdx.x - it * B.bpi;
    const dgb_itemnd_adj I = B.items[it];
    const int P = B.a.nd.ndim, ax = B.a.nd.axis;
    const long k = B.a.nd.step;
    const int frozen = I.masks & 0xff;
    if (k >= I.nsteps || (frozen >> ax & 1))
        return;
    ADNArgs A = B.a;
    A.nd.phi = B.lam_all + I.phi_off;
    const double *slots = B.scratch + it * B.slot_stride;
    A.out = (ax == last_active(frozen, P)) ? B.states_all + I.state_off + (k + 1) * B.N
                                           : slots + (long)ax * B.N;
    A.rhs = (ax == first_active(frozen, P)) ? B.states_all + I.state_off + k * B.N
                                            : slots + (long)(ax - 1) * B.N;
    int j = 0; // this axis' place among the item's swept axes
    for (int a = 0; a < ax; a++)
        j += !(frozen >> a & 1);
    A.gpart = B.gpart_all + I.gpart_off + k * B.per_step + (long)j * B.nb * row_stride(P);
    A.rec_off = it * B.item_coef;
    adn_tile(A, tl, smem, Sh, red,
             B.gam + (size_t)blockIdx.x * B.a.nd.L * blockDim.x);
}

// The injection's terms of step k, one thread per running item.
__global__ void k_adjoint_inject_batch(const dgb_itemnd_adj *items, int nact,
                                       const double *lam_all, const double *xx,
                                       const double *table, int P, int L, long k,
                                       long per_step, long inj_at, double *gpart_all)
{
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= nact)
        return;
    const dgb_itemnd_adj I = items[it];
    const int active = ((1 << P) - 1) & ~(I.masks & 0xff) & ~((I.masks >> 8) & 0xff);
    if (k >= I.nsteps || !active)
        return;
    adn_inject_terms(lam_all + I.phi_off, xx, table + (I.row_off + k) * row_stride(P), P, L,
                     active, gpart_all + I.gpart_off + k * per_step + inj_at);
}

// The Thomas plan of the batched forward and recomputation, and where the
// pieces of the workspace sit: records, Thomas scratch, recomputed slots,
// the device copies of the items (adjoint records, then plain items for the
// forward and for each recomputed axis).
struct AdjLayout {
    BatchPlan p;
    int nt, nb; // the transposed sweeps' lines per CTA and CTAs per item
    size_t coef, gam, slots, gam_adj, items_adj, items_nd, total; // offsets in bytes
};

static int adj_layout(int ndim, int L, int nitems, const dgb_settings *settings, AdjLayout &w)
{
    dgb_settings st = *settings;
    st.line_solver = 0;
    if (st.use_delj_trick)
        return DGB_ERR_UNSUPPORTED;
    int rc = batch_plan(ndim, L, nitems, &st, w.p);
    if (rc)
        return rc;
    const size_t N = (size_t)ipow(L, ndim);
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    w.coef = 0;
    w.gam = up(w.p.coef_doubles * sizeof(double));
    w.slots = w.gam + up(w.p.gam_doubles * sizeof(double));
    const long nlines = ipow(L, ndim - 1);
    w.nt = nd_threads(L, nlines);
    w.nb = (int)((nlines + w.nt - 1) / w.nt);
    w.gam_adj = w.slots + up((size_t)nitems * (ndim > 1 ? ndim - 1 : 0) * N * sizeof(double));
    w.items_adj = w.gam_adj + up((size_t)nitems * w.nb * w.nt * L * sizeof(double));
    w.items_nd = w.items_adj + up((size_t)nitems * sizeof(dgb_itemnd_adj));
    w.total = w.items_nd + up((size_t)(ndim + 1) * nitems * sizeof(dgb_itemnd));
    return DGB_OK;
}

static bool adj_items_ok(const dgb_itemnd_adj *items, int nitems)
{
    for (int i = 0; i < nitems; i++)
        if (items[i].nsteps < 0 || (i > 0 && items[i].nsteps > items[i - 1].nsteps) ||
            items[i].phi_off < 0 || items[i].row_off < 0 || items[i].state_off < 0 ||
            items[i].gpart_off < 0)
            return false;
    return true;
}

// The device copies of the items: the adjoint records, the plain items of
// the forward (phi in phi_all) and, per axis a < ndim - 1, the plain items
// whose density is the item's recomputation slot a.
static int adj_upload(const dgb_itemnd_adj *items, int nitems, int ndim, long N,
                      const AdjLayout &w, char *ws, cudaStream_t st)
{
    std::vector<dgb_itemnd> nd((size_t)(ndim + 1) * nitems);
    const long slot_stride = (long)(ndim - 1) * N;
    for (int i = 0; i < nitems; i++) {
        for (int a = 0; a <= ndim; a++) {
            dgb_itemnd &d = nd[(size_t)a * nitems + i];
            d.phi_off = a == 0 ? items[i].phi_off : (long)i * slot_stride + (long)(a - 1) * N;
            d.row_off = items[i].row_off;
            d.nsteps = items[i].nsteps;
            d.masks = items[i].masks;
        }
    }
    // pageable sources: each copy returns once its source has been staged
    if (cudaMemcpyAsync(ws + w.items_adj, items, (size_t)nitems * sizeof(dgb_itemnd_adj),
                        cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(ws + w.items_nd, nd.data(), nd.size() * sizeof(dgb_itemnd),
                        cudaMemcpyHostToDevice, st) != cudaSuccess)
        return DGB_ERR_CUDA;
    return DGB_OK;
}

static void adj_batch(NDBatch &B, const AdjLayout &w, int ndim, int L, const double *xx,
                      double *phi_all, const double *table, char *ws)
{
    B = NDBatch{};
    nd_fill(B.A, phi_all, ndim, L, 0, xx);
    B.phi_all = phi_all;
    B.table = table;
    B.coef = (double *)(ws + w.coef);
    B.chunk = w.p.chunk;
    B.item_coef = (long)w.p.chunk * ndim * (long)nd_rec_doubles(L, false);
    B.bpi = w.p.bpi;
    B.gam_glob = w.p.gsmem ? nullptr : (double *)(ws + w.gam);
}

} // namespace dgb

extern "C" size_t dgb_batchnd_adjoint_workspace_bytes(int ndim, int L, int nitems,
                                                      const dgb_settings *settings)
{
    if (!shape_ok(ndim, L) || nitems < 1 || !settings)
        return 0;
    AdjLayout w;
    if (adj_layout(ndim, L, nitems, settings, w))
        return 0;
    return w.total + 256;
}

extern "C" int dgb_batchnd_integrate_states(const dgb_itemnd_adj *items, int nitems, int ndim,
                                            int L, const double *xx, double *phi_all,
                                            const double *table, double *states_all,
                                            const dgb_settings *settings, void *ws,
                                            size_t ws_bytes, void *stream)
{
    if (!items || nitems < 1 || !xx || !phi_all || !table || !states_all || !settings ||
        !shape_ok(ndim, L) || !adj_items_ok(items, nitems))
        return DGB_ERR_ARG;
    AdjLayout w;
    int rc = adj_layout(ndim, L, nitems, settings, w);
    if (rc)
        return rc;
    if (!ws || ws_bytes < w.total)
        return DGB_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *wb = (char *)ws;
    const long N = ipow(L, ndim);
    rc = adj_upload(items, nitems, ndim, N, w, wb, st);
    if (rc)
        return rc;
    std::vector<int> nsteps(nitems);
    for (int i = 0; i < nitems; i++)
        nsteps[i] = items[i].nsteps;
    NDBatch B;
    adj_batch(B, w, ndim, L, xx, phi_all, table, wb);
    B.items = (const dgb_itemnd *)(wb + w.items_nd);
    return batch_loop(B, w.p, nsteps.data(), nitems, false,
                      (const dgb_itemnd_adj *)(wb + w.items_adj), states_all, st);
}

extern "C" int dgb_batchnd_adjoint(const dgb_itemnd_adj *items, int nitems, int ndim, int L,
                                   const double *xx, double *lam_all, const double *table,
                                   const double *states_all, double *gpart_all,
                                   const dgb_settings *settings, void *ws, size_t ws_bytes,
                                   void *stream)
{
    if (!items || nitems < 1 || !xx || !lam_all || !table || !states_all || !gpart_all ||
        !settings || !shape_ok(ndim, L) || !adj_items_ok(items, nitems))
        return DGB_ERR_ARG;
    AdjLayout w;
    int rc = adj_layout(ndim, L, nitems, settings, w);
    if (rc)
        return rc;
    if (!ws || ws_bytes < w.total)
        return DGB_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *wb = (char *)ws;
    const long N = ipow(L, ndim);
    const long total = items[0].nsteps;
    if (total == 0)
        return DGB_OK;
    rc = adj_upload(items, nitems, ndim, N, w, wb, st);
    if (rc)
        return rc;
    const long per_step = (long)dgb_adjoint_table_nd_gpart_doubles(ndim, L);
    for (int i = 0; i < nitems; i++)
        if (items[i].nsteps &&
            cudaMemsetAsync(gpart_all + items[i].gpart_off, 0,
                            (size_t)items[i].nsteps * per_step * sizeof(double),
                            st) != cudaSuccess)
            return DGB_ERR_CUDA;
    const dgb_itemnd *d_nd = (const dgb_itemnd *)(wb + w.items_nd);
    const dgb_itemnd_adj *d_adj = (const dgb_itemnd_adj *)(wb + w.items_adj);
    double *slots = (double *)(wb + w.slots);
    const long slot_stride = (long)(ndim - 1) * N;
    // the records (and the item list they are indexed by) and the
    // recomputation sweeps: slot a of item i is phi_all' = slots, items
    // d_nd + (a + 1) * nitems
    NDBatch B;
    adj_batch(B, w, ndim, L, xx, slots, table, wb);
    B.items = d_nd;
    size_t csmem;
    if (batch_coef_prepare(false, csmem, L))
        return DGB_ERR_CUDA;
    // the transposed sweeps: the tiles of dgb_adjoint_table_nd, with the
    // Thomas scratch in workspace slices (twice the CTAs per SM)
    const int nt = w.nt, nb = w.nb;
    ADNBatch AB = {};
    nd_fill(AB.a.nd, nullptr, ndim, L, 0, xx);
    AB.a.nd.table = table;
    AB.a.coef = B.coef;
    AB.items = d_adj;
    AB.lam_all = lam_all;
    AB.states_all = states_all;
    AB.scratch = slots;
    AB.gpart_all = gpart_all;
    AB.gam = (double *)(wb + w.gam_adj);
    AB.N = N;
    AB.slot_stride = slot_stride;
    AB.item_coef = B.item_coef;
    AB.per_step = per_step;
    AB.bpi = nb;
    AB.nb = nb;
    const size_t asmem = adn_smem_doubles(L, nt, false) * sizeof(double);
    if (raise_smem_limit(k_adjoint_sweep_batch))
        return DGB_ERR_CUDA;
    const long inj_at = (long)ndim * nb * row_stride(ndim);
    const unsigned cpx = (unsigned)std::min<long>((N + 255) / 256, 64);
    long nact = 0, lo = -1;
    for (long k = total - 1; k >= 0; k--) {
        while (nact < nitems && items[nact].nsteps > k)
            nact++;
        if (lo < 0 || k < lo) {
            lo = std::max(0L, k - w.p.chunk + 1);
            long nrec = 0; // every item running at some step of the chunk
            while (nrec < nitems && items[nrec].nsteps > lo)
                nrec++;
            B.step0 = lo;
            const int nsl = (int)(k - lo + 1);
            k_coef_batch<false><<<(unsigned)(nrec * nsl * ndim), 128, csmem, st>>>(B, nsl);
            if (cudaGetLastError() != cudaSuccess)
                return DGB_ERR_CUDA;
        }
        for (int ax = 0; ax < ndim - 1; ax++) {
            k_slot_copy<<<dim3(cpx, (unsigned)nact), 256, 0, st>>>(d_adj, states_all, slots,
                                                                 slot_stride, k, ax, N);
            if (cudaGetLastError() != cudaSuccess)
                return DGB_ERR_CUDA;
            B.items = d_nd + (size_t)(ax + 1) * nitems;
            batch_set_axis(B, ax);
            rc = batch_sweep(B, w.p, nact, k, false, st);
            if (rc)
                return rc;
        }
        B.items = d_nd;
        AB.a.step0 = lo;
        for (int ax = ndim - 1; ax >= 0; ax--) {
            AB.a.nd.axis = ax;
            AB.a.nd.S = ipow(L, ndim - 1 - ax);
            AB.a.nd.LS = AB.a.nd.S * L;
            AB.a.nd.step = k;
            k_adjoint_sweep_batch<<<(unsigned)(nact * nb), nt, asmem, st>>>(AB);
            if (cudaGetLastError() != cudaSuccess)
                return DGB_ERR_CUDA;
        }
        k_adjoint_inject_batch<<<(unsigned)((nact + 127) / 128), 128, 0, st>>>(
            d_adj, (int)nact, lam_all, xx, table, ndim, L, k, per_step, inj_at, gpart_all);
        if (cudaGetLastError() != cudaSuccess)
            return DGB_ERR_CUDA;
    }
    return DGB_OK;
}

// ------------------------------------------- parametric schedules (host)

// Value of a parametric form at t (dgb_pform; the same evaluation as the
// device's pform_eval).
static double pf_host(const dgb_pform &f, double t) { return pform_eval(f, t); }

// The table rows of one parametric P-population integration: the loop of
// Integration.three_pops / four_pops / five_pops (dadi/Integration.py:
// 504-553, 672-726, 884-935): dt from the current parameters (the minimum
// over populations of _compute_dt, :147-176, with each population's
// migration rates into it summed in increasing order), the parameters at
// the next time, the reference's validation.  rows == null counts; rows
// are written while fewer than `room` have been.
static long schednd_walk(const dgb_instnd &I, const dgb_settings &st, double dx0,
                         long max_steps, double *rows, long room, int *status)
{
    const int P = I.ndim;
    double nu[DGB_MAX_DIM], g[DGB_MAX_DIM], h[DGB_MAX_DIM], m[DGB_MAX_DIM][DGB_MAX_DIM];
    auto eval = [&](double t) {
        for (int k = 0; k < P; k++) {
            nu[k] = pf_host(I.nu[k], t);
            g[k] = pf_host(I.gamma[k], t);
            h[k] = pf_host(I.h[k], t);
            for (int j = 0; j < P; j++)
                m[k][j] = (j == k) ? 0.0 : pf_host(I.mig[k][j], t);
        }
    };
    double cur = I.initial_t;
    eval(cur);
    long n = 0;
    int err = 0;
    const int stride = row_stride(P);
    while (cur < I.T) {
        if (n >= max_steps) {
            err |= DGB_ST_STEPCAP;
            break;
        }
        double dtm = 0;
        for (int k = 0; k < P; k++) {
            double msum = 0;
            for (int j = 0; j < P; j++)
                if (j != k)
                    msum = msum + m[k][j];
            double d = compute_dt(nu[k], (P == 1) ? 0.0 : msum, g[k], h[k], st, dx0);
            dtm = (k == 0) ? d : pymin(dtm, d);
        }
        if (dtm == 0) {
            err |= DGB_ST_ZERODT;
            break;
        }
        double dt = pymin(dtm, I.T - cur);
        double next = cur + dt;
        if (!(dt > 0) || !std::isfinite(next)) {
            err |= DGB_ST_NONFINITE;
            break;
        }
        eval(next);
        double theta0 = pf_host(I.theta0, next);
        bool bad = I.T < 0 || theta0 < 0;
        for (int k = 0; k < P; k++) {
            bad = bad || nu[k] < 0 || nu[k] == 0;
            for (int j = 0; j < P; j++)
                bad = bad || (j != k && m[k][j] < 0);
        }
        if (bad) {
            err |= DGB_ST_BADPARAM;
            break;
        }
        if (rows && n >= room) {
            err |= DGB_ST_STEPCAP;
            break;
        }
        if (rows) {
            double *r = rows + n * stride;
            r[0] = dt;
            r[1] = theta0;
            for (int k = 0; k < P; k++) {
                r[row_nu(P, k)] = nu[k];
                r[row_gamma(P, k)] = g[k];
                r[row_h(P, k)] = h[k];
                for (int j = 0; j < P; j++)
                    if (j != k)
                        r[row_mig(P, k, j)] = m[k][j];
            }
            r[row_beta(P)] = 1.0;
        }
        n++;
        cur = next;
    }
    if (status)
        *status |= err;
    return n;
}

extern "C" int dgb_schednd_host(const dgb_instnd *insts, int ninst,
                                const dgb_settings *settings, long max_steps, double dx0,
                                int *row_cnt, const long *row_off, double *table, int *status)
{
    if (!insts || ninst < 0 || !settings || !row_cnt || max_steps < 1 || (table && !row_off))
        return DGB_ERR_ARG;
    for (int i = 0; i < ninst; i++)
        if (insts[i].ndim < 1 || insts[i].ndim > DGB_MAX_DIM)
            return DGB_ERR_ARG;
    for (int i = 0; i < ninst; i++) {
        const dgb_instnd &I = insts[i];
        const int P = I.ndim;
        if (!table) {
            row_cnt[i] = (int)schednd_walk(I, *settings, dx0, max_steps, nullptr, 0, nullptr);
        } else {
            int err = 0;
            long n = schednd_walk(I, *settings, dx0, max_steps,
                                  table + row_off[i] * row_stride(P), row_cnt[i], &err);
            row_cnt[i] = (int)n;
            if (status)
                status[i] |= err;
        }
    }
    return DGB_OK;
}

// ------------------------------------- parametric schedules in dual numbers

// A value and its derivatives with respect to the seeded model parameters.
struct DualN {
    double v;
    double d[DGB_ND_MAXPAR];
};

// A form at time t (dt/dtheta = dtd) with its derivative: the value exactly
// as pform_eval gives it, the derivative by differentiating the form.
static DualN pf_dual(const dgb_pform &f, const double (*dabc)[DGB_ND_MAXPAR], double t,
                     const double *dtd, int npar)
{
    DualN r;
    r.v = pform_eval(f, t);
    const double *da = dabc[0], *db = dabc[1], *dc = dabc[2];
    const double a = f.a, b = f.b, c = f.c;
    switch (f.kind) {
    case DGB_PF_EXPGROW:
    case DGB_PF_EXPLOG: {
        // v = a exp(lq t / c), lq = log(b / a)
        const double lq = log(b / a);
        const double e = r.v / a;
        for (int p = 0; p < npar; p++) {
            double dlq = db[p] / b - da[p] / a;
            double dz = (dlq * t + lq * dtd[p]) / c - (lq * t / c) * dc[p] / c;
            r.d[p] = da[p] * e + a * e * dz;
        }
        break;
    }
    case DGB_PF_LINEAR:
        for (int p = 0; p < npar; p++)
            r.d[p] = da[p] + db[p] * t + b * dtd[p];
        break;
    default:
        for (int p = 0; p < npar; p++)
            r.d[p] = da[p];
    }
    return r;
}

// compute_dt with its derivative along the branch its max takes (ties go to
// the first candidate, as Python's max does).
static DualN dt_dual(const DualN &nu, const DualN &ms, const DualN &g, const DualN &h,
                     const dgb_settings &st, double dx0, int npar)
{
    DualN r;
    r.v = compute_dt(nu.v, ms.v, g.v, h.v, st, dx0);
    for (int p = 0; p < npar; p++)
        r.d[p] = 0;
    if (st.use_old_timestep)
        return r;
    const double v1 = 0.25 / nu.v;
    const double t1 = fabs(h.v + (1 - 2 * h.v) * 0.5) * 0.5 * (1 - 0.5);
    const double u2 = h.v + (1 - 2 * h.v) * 0.25;
    const double t2 = fabs(u2) * 0.25 * (1 - 0.25);
    const double tm = (t2 > t1) ? t2 : t1;
    const double v3 = fabs(g.v) * 2 * tm;
    int br = 0;
    double mx = v1;
    if (ms.v > mx) {
        mx = ms.v;
        br = 1;
    }
    if (v3 > mx) {
        mx = v3;
        br = 2;
    }
    if (!(mx > 0))
        return r;
    const double sg = (g.v > 0) ? 1.0 : ((g.v < 0) ? -1.0 : 0.0);
    const double su = (u2 > 0) ? 1.0 : ((u2 < 0) ? -1.0 : 0.0);
    for (int p = 0; p < npar; p++) {
        double dmx;
        if (br == 0) {
            dmx = -0.25 * nu.d[p] / (nu.v * nu.v);
        } else if (br == 1) {
            dmx = ms.d[p];
        } else {
            // t1 does not depend on h; t2 = |u2| 3/16 with du2/dh = 1/2
            double dtm = (t2 > t1) ? su * 0.5 * h.d[p] * 0.25 * (1 - 0.25) : 0.0;
            dmx = sg * g.d[p] * 2 * tm + fabs(g.v) * 2 * dtm;
        }
        r.d[p] = -st.timescale_factor * dmx / (mx * mx);
    }
    return r;
}

extern "C" int dgb_schednd_dual_host(const dgb_instnd *inst, const dgb_seednd *seed, int npar,
                                     const dgb_settings *settings, long max_steps, double dx0,
                                     int *nrows, double *table, double *drows, int *status)
{
    if (!inst || !seed || !settings || !nrows || npar < 0 || npar > DGB_ND_MAXPAR ||
        max_steps < 1 || (table && !drows) || inst->ndim < 1 || inst->ndim > DGB_MAX_DIM)
        return DGB_ERR_ARG;
    const dgb_instnd &I = *inst;
    const dgb_seednd &S = *seed;
    const dgb_settings &st = *settings;
    const int P = I.ndim;
    const int stride = row_stride(P);
    const long room = table ? *nrows : 0;
    DualN nu[DGB_MAX_DIM], g[DGB_MAX_DIM], h[DGB_MAX_DIM], m[DGB_MAX_DIM][DGB_MAX_DIM];
    double dtd[DGB_ND_MAXPAR];
    auto eval = [&](double t) {
        for (int k = 0; k < P; k++) {
            nu[k] = pf_dual(I.nu[k], S.dnu[k], t, dtd, npar);
            g[k] = pf_dual(I.gamma[k], S.dgamma[k], t, dtd, npar);
            h[k] = pf_dual(I.h[k], S.dh[k], t, dtd, npar);
            for (int j = 0; j < P; j++)
                if (j != k)
                    m[k][j] = pf_dual(I.mig[k][j], S.dmig[k][j], t, dtd, npar);
        }
    };
    for (int p = 0; p < npar; p++)
        dtd[p] = S.dt0[p];
    double cur = I.initial_t;
    eval(cur);
    long n = 0;
    int err = 0;
    while (cur < I.T) {
        if (n >= max_steps) {
            err |= DGB_ST_STEPCAP;
            break;
        }
        DualN best;
        for (int k = 0; k < P; k++) {
            DualN ms;
            ms.v = 0;
            for (int p = 0; p < npar; p++)
                ms.d[p] = 0;
            for (int j = 0; j < P; j++)
                if (j != k) {
                    ms.v = ms.v + m[k][j].v;
                    for (int p = 0; p < npar; p++)
                        ms.d[p] += m[k][j].d[p];
                }
            DualN d = dt_dual(nu[k], ms, g[k], h[k], st, dx0, npar);
            if (k == 0 || d.v < best.v)
                best = d;
        }
        if (best.v == 0) {
            err |= DGB_ST_ZERODT;
            break;
        }
        const double rem = I.T - cur;
        DualN step;
        if (rem < best.v) {
            step.v = rem;
            for (int p = 0; p < npar; p++)
                step.d[p] = S.dT[p] - dtd[p];
        } else {
            step = best;
        }
        const double next = cur + step.v;
        if (!(step.v > 0) || !std::isfinite(next)) {
            err |= DGB_ST_NONFINITE;
            break;
        }
        for (int p = 0; p < npar; p++)
            dtd[p] += step.d[p];
        eval(next);
        const DualN th0 = pf_dual(I.theta0, S.dtheta0, next, dtd, npar);
        bool bad = I.T < 0 || th0.v < 0;
        for (int k = 0; k < P; k++) {
            bad = bad || nu[k].v < 0 || nu[k].v == 0;
            for (int j = 0; j < P; j++)
                bad = bad || (j != k && m[k][j].v < 0);
        }
        if (bad) {
            err |= DGB_ST_BADPARAM;
            break;
        }
        if (table && n >= room) {
            err |= DGB_ST_STEPCAP;
            break;
        }
        if (table) {
            double *r = table + n * stride;
            double *dr = drows + n * stride * npar;
            for (int c = 0; c < stride * npar; c++)
                dr[c] = 0;
            auto put = [&](int c, const DualN &x) {
                r[c] = x.v;
                for (int p = 0; p < npar; p++)
                    dr[c * npar + p] = x.d[p];
            };
            put(0, step);
            put(1, th0);
            for (int k = 0; k < P; k++) {
                put(row_nu(P, k), nu[k]);
                put(row_gamma(P, k), g[k]);
                put(row_h(P, k), h[k]);
                for (int j = 0; j < P; j++)
                    if (j != k)
                        put(row_mig(P, k, j), m[k][j]);
            }
            r[row_beta(P)] = 1.0;
        }
        n++;
        cur = next;
    }
    *nrows = (int)n;
    if (status)
        *status |= err;
    return DGB_OK;
}

namespace dgb {
int preload_batchnd()
{
    return preload(k_coef_batch<false>) + preload(k_coef_batch<true>) +
           preload(k_sweep_batch<false, false>) + preload(k_sweep_batch<false, true>) +
           preload(k_sweep_batch<true, false>) + preload(k_sweep_batch<true, true>) +
           preload(k_sweep_batch_pcr) + preload(k_sweep_batch_part<2>) +
           preload(k_sweep_batch_part<4>) + preload(k_sweep_batch_part<8>) +
           preload(k_store_states) + preload(k_slot_copy) + preload(k_adjoint_sweep_batch) +
           preload(k_adjoint_inject_batch);
}
} // namespace dgb
