// Shared device/host helpers of the dadi_gb300 kernels.
//
// The implicit ADI sweep of dadi (dadi/integration_shared.c:4-93,
// dadi/tridiag.c:14-34) is restated here in a form that costs ~10 FP64
// pipe instructions per grid point per sweep:
//
//  * Every tridiagonal row is multiplied by dt, so r = phi and the diagonal
//    is 1 + dt*(...); no per-point division by dt.
//  * With delta_j = 0.5 (dadi's default, use_delj_trick False), the
//    coefficients of a line are affine in W = sum_k m_k o_k, the only
//    quantity that depends on the line's other coordinates o_k:
//        a'_i = W*A1_i + A0_i,  c'_i = W*C1_i + C0_i,
//        b'_i = B0_i  (interior rows; W cancels),  b'_0 and b'_{L-1} carry W*B1.
//    A1..B0 are per-axis vectors rebuilt once per step (O(L) work) from
//    dx, dfactor, xInt, V = x(1-x)/nu and the selection term, following
//    compute_abc_nobc (dadi/integration_shared.c:72-93).
//  * 1/bet uses the hardware reciprocal seed (rcp.approx.ftz.f64) refined by
//    one third-order Newton-Raphson step r(1 + e + e^2), e = 1 - x r, which
//    is accurate to about one ulp; quotients become products.
// These reassociations move results by a few ulps per step relative to the
// reference C, far inside the 1e-9 relative bar on extrapolated spectra.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/dadi_gb300.h"

namespace dgb {

#define DGB_HD __host__ __device__ __forceinline__

// ---------------------------------------------------------------- arithmetic

__device__ __forceinline__ double rcp_seed(double x)
{
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    return r;
}

// Reciprocal to ~1 ulp: seed refined by one cubic Newton-Raphson step.
__device__ __forceinline__ double rcp_full(double x)
{
    double r = rcp_seed(x);
    double e = fma(-x, r, 1.0);
    return fma(r, fma(e, e, e), r);
}

// ------------------------------------------------------- parameter schedule

// Parametric time dependence (see dgb_pform in dadi_gb300.h).
DGB_HD double pform_eval(const dgb_pform &f, double t)
{
    switch (f.kind) {
    case DGB_PF_EXPGROW:
        return f.a * pow(f.b / f.a, t / f.c);
    case DGB_PF_EXPLOG:
        return f.a * exp(log(f.b / f.a) * t / f.c);
    case DGB_PF_LINEAR:
        return f.a + f.b * t;
    default:
        return f.a;
    }
}

// Timestep from one population's current parameters, as
// dadi/Integration.py:147-176 (Python max/min keep the first extreme).
DGB_HD double compute_dt(double nu, double msum, double gamma, double h,
                         const dgb_settings &s, double dx0)
{
    if (s.use_old_timestep)
        return s.old_timescale_factor * dx0;
    double v1 = 0.25 / nu;
    double t1 = fabs(h + (1 - 2 * h) * 0.5) * 0.5 * (1 - 0.5);
    double t2 = fabs(h + (1 - 2 * h) * 0.25) * 0.25 * (1 - 0.25);
    double tm = t1;
    if (t2 > tm)
        tm = t2;
    double v3 = fabs(gamma) * 2 * tm;
    double mx = v1;
    if (msum > mx)
        mx = msum;
    if (v3 > mx)
        mx = v3;
    if (mx > 0)
        return s.timescale_factor / mx;
    return INFINITY;
}

// Python min(a, b): a unless b < a.
DGB_HD double pymin(double a, double b) { return (b < a) ? b : a; }

// Selection part of M (dadi/integration_shared.c:12-14).
DGB_HD double msel(double x, double gamma, double h)
{
    return gamma * 2 * (h + (1. - 2 * h) * x) * x * (1. - x);
}

// Table-row layout (see dadi_gb300.h).
DGB_HD int row_stride(int P) { return 3 + 3 * P + P * (P - 1); }
DGB_HD int row_nu(int P, int k) { return 2 + k; }
DGB_HD int row_gamma(int P, int k) { return 2 + P + k; }
DGB_HD int row_h(int P, int k) { return 2 + 2 * P + k; }
DGB_HD int row_beta(int P) { return 2 + 3 * P; }
DGB_HD int row_mig(int P, int k, int j)
{
    return 3 + 3 * P + k * (P - 1) + (j < k ? j : j - 1);
}

// Mutation mass added at the unit corner of population k: the value of
// dadi/Integration.py:70-122 with the common grid xx (x0, x1, x2 = xx[0..2]).
DGB_HD double inject_value(int P, double dt, double theta0, double x0,
                           double x1, double x2)
{
    double denom = x2 - x0;
    for (int j = 1; j < P; j++)
        denom = denom * x1;
    double num = dt / x1 * theta0 / 2;
    return num * (double)(1 << P) / denom;
}

// ------------------------------------------------------ per-axis vectors

// Per-grid constants of one axis held in shared memory.
struct GridVecs {
    double *x;    // xx[i]
    double *xv;   // x(1-x)
    double *dfac; // dfactor[i]
    double *xInt; // midpoints
    double *ih;   // 1/(2 dx[i])
    double *dx;   // dx[i]
};

// Per-step coefficient vectors of one axis (see the header comment).
struct AxisVecs {
    double *A1, *A0, *C1, *C0, *B0;
    // delj-trick path only: per-interval G, P, Q, VInt and per-row dt*dfac
    double *G, *Pv, *Qv, *VI, *DF;
};

// Scalars of one axis for one step (written by one thread, read by all).
struct AxisScalars {
    double dt, nu, inv_nu, msum, gamma, h;
    double B1s, B1e; // W multipliers of b'_0 and b'_{L-1}
    double bcs, bce; // dt-scaled corner boundary terms (0 if not applied)
    double mig[DGB_MAX_DIM];
};

// Corner boundary terms of dadi/integration2D.c:67-70 (and the 3-D/4-D
// equivalents): M at x = xx[0] with every other coordinate 0, and at
// x = xx[L-1] with every other coordinate 1, summed in increasing axis order.
DGB_HD void corner_bc(int P, int axis, const double *mig, double nu, double gamma,
                      double h, double x0, double xl, double dx0, double dxl,
                      double dt, double &bcs, double &bce)
{
    double mf = 0, ml = 0;
    bool first = true;
    for (int k = 0; k < P; k++) {
        if (k == axis)
            continue;
        double tf = mig[k] * (0.0 - x0), tl = mig[k] * (1.0 - xl);
        mf = first ? tf : mf + tf;
        ml = first ? tl : ml + tl;
        first = false;
    }
    mf = first ? msel(x0, gamma, h) : mf + msel(x0, gamma, h);
    ml = first ? msel(xl, gamma, h) : ml + msel(xl, gamma, h);
    bcs = (mf <= 0) ? dt * ((0.5 / nu - mf) * 2. / dx0) : 0.0;
    bce = (ml >= 0) ? dt * (-(-0.5 / nu - ml) * 2. / dxl) : 0.0;
}

// Build entry i of the per-step vectors of one axis (called for i = 0..L-1
// by different threads).  vscale multiplies V (the breeding-ratio factor of
// Vfunc_beta in 1-D, 1 otherwise).
__device__ __forceinline__ void build_axis_entry(int i, int L, const GridVecs &g,
                                                 const AxisScalars &s, double vscale,
                                                 bool delj, AxisVecs &v)
{
    const double dt = s.dt;
    const double iv = s.inv_nu * vscale;
    auto Gk = [&](int k) { return msel(g.xInt[k], s.gamma, s.h) - s.msum * g.xInt[k]; };
    double dfi = dt * g.dfac[i];
    double p_i = 0, q_im1 = 0;
    if (i < L - 1) {
        double G = Gk(i);
        double P = iv * g.xv[i] * g.ih[i];
        double Q = iv * g.xv[i + 1] * g.ih[i];
        p_i = fma(0.5, G, P);
        v.C1[i] = 0.5 * dfi;
        v.C0[i] = -dfi * fma(-0.5, G, Q);
        if (delj) {
            // the delj path rebuilds MInt per point in the reference order,
            // so only the selection term and VInt are stored
            // (dadi/integration2D.c:47-49: VInt = Vfunc(xInt, nu))
            v.G[i] = msel(g.xInt[i], s.gamma, s.h);
            v.Pv[i] = P;
            v.Qv[i] = Q;
            v.VI[i] = (s.inv_nu * g.xInt[i]) * (1. - g.xInt[i]) * vscale;
        }
    } else {
        v.C1[i] = 0;
        v.C0[i] = 0;
    }
    if (i > 0) {
        double G = Gk(i - 1);
        double P = iv * g.xv[i - 1] * g.ih[i - 1];
        double Q = iv * g.xv[i] * g.ih[i - 1];
        q_im1 = fma(-0.5, G, Q);
        v.A1[i] = -0.5 * dfi;
        v.A0[i] = -dfi * fma(0.5, G, P);
    } else {
        v.A1[i] = 0;
        v.A0[i] = 0;
    }
    v.B0[i] = fma(dfi, p_i + q_im1, 1.0);
    if (delj)
        v.DF[i] = dfi;
}

// ------------------------------------------------------------ line solvers

// Back substitution u_i = u'_i - gam_{i+1} u_{i+1} for i = L-2..0, where
// u holds u_{L-1}.  The gam and u' of 16 rows are loaded before their
// dependent FMA chain runs, so scratch that lives in global memory (L2) does
// not stall the chain on every row.
template <typename TP, typename TG>
__device__ __forceinline__ void back_substitute(TP *__restrict__ ph, int sp,
                                                TG *__restrict__ gm, int gs, int L, double u)
{
    constexpr int B = 16;
    int i = L - 2;
    for (; i >= B - 1; i -= B) {
        double gv[B], pv[B];
#pragma unroll
        for (int k = 0; k < B; k++) {
            gv[k] = gm[(i - k + 1) * gs];
            pv[k] = ph[(i - k) * sp];
        }
#pragma unroll
        for (int k = 0; k < B; k++) {
            u = fma(-gv[k], u, pv[k]);
            ph[(i - k) * sp] = u;
        }
    }
    for (; i >= 0; i--) {
        u = fma(-(double)gm[(i + 1) * gs], u, ph[i * sp]);
        ph[i * sp] = u;
    }
}

// Thomas solve of one line, delta_j = 0.5.  Element p of the line is
// ph[p*sp]; gam scratch element p is gm[p*gs].  W is the line's migration
// weight, bs/be the corner boundary terms for this line (0 if none).
template <typename TP, typename TG>
__device__ __forceinline__ void solve_line(TP *__restrict__ ph, int sp, TG *__restrict__ gm,
                                           int gs, int L, double W, double bs, double be,
                                           const AxisVecs &v, const AxisScalars &s)
{
    double b = fma(W, s.B1s, v.B0[0]) + bs;
    double inv = rcp_full(b);
    double u = ph[0] * inv;
    ph[0] = u;
    double g = fma(W, v.C1[0], v.C0[0]) * inv;
    gm[gs] = g;
    int i = 1;
#pragma unroll 2
    for (; i < L - 1; i++) {
        double a = fma(W, v.A1[i], v.A0[i]);
        double bet = fma(-a, g, v.B0[i]);
        inv = rcp_full(bet);
        u = fma(-a, u, ph[i * sp]) * inv;
        ph[i * sp] = u;
        g = fma(W, v.C1[i], v.C0[i]) * inv;
        gm[(i + 1) * gs] = g;
    }
    {
        double a = fma(W, v.A1[i], v.A0[i]);
        double bl = fma(W, s.B1e, v.B0[i]) + be;
        double bet = fma(-a, g, bl);
        inv = rcp_full(bet);
        u = fma(-a, u, ph[i * sp]) * inv;
        ph[i * sp] = u;
    }
    back_substitute(ph, sp, gm, gs, L, u);
}

// Chang-Cooper delta_j (dadi/integration_shared.c:52-70) for one interval.
__device__ __forceinline__ double delj_of(double MInt, double VInt, double dx)
{
    double wj = 2 * MInt * dx;
    double epsj = exp(wj / VInt);
    if ((epsj != 1.0) && (wj != 0))
        return (-epsj * wj + epsj * VInt - VInt) / (wj - epsj * wj);
    return 0.5;
}

// Thomas solve of one line with the delj trick.  MInt is rebuilt per
// interval exactly as Mfunc{2,3,4}D computes it (dadi/integration_shared.c:
// 15-25: sum over the other axes of m_k (o_k - x), then the selection term),
// because exp(wj/VInt) amplifies any rounding difference in MInt; the
// coefficients then follow compute_abc_nobc, scaled by dt.
template <typename TP, typename TG>
__device__ __forceinline__ void solve_line_delj(TP *__restrict__ ph, int sp, TG *__restrict__ gm,
                                                int gs, int L, const double *mo,
                                                const double *oo, int nother, double bs,
                                                double be, const GridVecs &gv,
                                                const AxisVecs &v)
{
    auto mint = [&](int k) {
        double x = gv.xInt[k];
        if (nother == 0)
            return v.G[k];
        double acc = mo[0] * (oo[0] - x);
        for (int j = 1; j < nother; j++)
            acc = acc + mo[j] * (oo[j] - x);
        return acc + v.G[k];
    };
    // interval k quantities: at_k = MInt d + P, ct_k = -MInt (1-d) + Q
    double Mk = mint(0);
    double d = delj_of(Mk, v.VI[0], gv.dx[0]);
    double at = Mk * d + v.Pv[0];
    double ct = -Mk * (1 - d) + v.Qv[0];
    double b = fma(v.DF[0], at, 1.0) + bs;
    double inv = rcp_full(b);
    double u = ph[0] * inv;
    ph[0] = u;
    double g = (-v.DF[0] * ct) * inv;
    gm[gs] = g;
    for (int i = 1; i < L; i++) {
        double a = -v.DF[i] * at;
        double bsum = ct;
        if (i < L - 1) {
            Mk = mint(i);
            d = delj_of(Mk, v.VI[i], gv.dx[i]);
            at = Mk * d + v.Pv[i];
            bsum = bsum + at;
            ct = -Mk * (1 - d) + v.Qv[i];
        }
        double bb = fma(v.DF[i], bsum, 1.0) + (i == L - 1 ? be : 0.0);
        double bet = fma(-a, g, bb);
        inv = rcp_full(bet);
        u = fma(-a, u, ph[i * sp]) * inv;
        ph[i * sp] = u;
        if (i < L - 1) {
            g = (-v.DF[i] * ct) * inv;
            gm[(i + 1) * gs] = g;
        }
    }
    back_substitute(ph, sp, gm, gs, L, u);
}

} // namespace dgb
