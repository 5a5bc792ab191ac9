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
//
// Under the delj trick (Chang-Cooper delta_j, dadi/integration_shared.c:
// 52-70) none of this is done.  delta_j = (-e w + e V - V) / (w - e w),
// e = exp(w / V), cancels catastrophically as w / V -> 0, so any rounding
// of MInt or of delta_j's own terms is amplified; the delj path therefore
// follows the reference operation by operation: unscaled rows (b starts at
// 1/dt, r = phi/dt), every product and sum rounded on its own (the __d*_rn
// intrinsics, which the compiler never fuses into a multiply-add, where C
// compiled for x86-64 has no fused multiply-add either), IEEE division, and
// the Numerical-Recipes recurrence as written.  Only exp is CUDA's (an
// error bound of one ulp rather than the C library's half ulp).
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
    // delj-trick path only: per-interval selection term, V[i]/(2dx),
    // V[i+1]/(2dx), VInt, and per-row dfactor
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

// ------------------------------------------- the delj path's exact operations

__device__ __forceinline__ double xm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xa(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xs(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double xd(double a, double b) { return __ddiv_rn(a, b); }

// Selection part of Mfunc (dadi/integration_shared.c:12-14) in the
// reference's order: gamma * 2*(h + (1.-2*h)*x) * x*(1.-x).
__device__ __forceinline__ double msel_ref(double x, double gamma, double h)
{
    return xm(xm(xm(xm(gamma, 2.0), xa(h, xm(xs(1.0, xm(2.0, h)), x))), x), xs(1.0, x));
}

// Vfunc (dadi/integration_shared.c:4-6), or Vfunc_beta (:8-10) when beta > 0
// (one population): 1./nu * x*(1.-x) [* pow(beta+1, 2)/(4*beta)].
__device__ __forceinline__ double vfunc_ref(double x, double nu, double beta)
{
    double v = xm(xm(xd(1.0, nu), x), xs(1.0, x));
    if (beta > 0) {
        const double b1 = xa(beta, 1.0);
        v = xd(xm(v, xm(b1, b1)), xm(4.0, beta));
    }
    return v;
}

// Build entry i of the per-step vectors of one axis (called for i = 0..L-1
// by different threads).  vscale multiplies V (the breeding-ratio factor of
// Vfunc_beta in 1-D, 1 otherwise); beta1 is the breeding ratio itself for one
// population and 0 otherwise (the delj path evaluates Vfunc_beta as written).
__device__ __forceinline__ void build_axis_entry(int i, int L, const GridVecs &g,
                                                 const AxisScalars &s, double vscale,
                                                 bool delj, AxisVecs &v, double beta1 = 0.0)
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
            // the delj path rebuilds MInt per point in the reference order;
            // per interval it needs the selection term, V[i]/(2 dx[i]),
            // V[i+1]/(2 dx[i]) and VInt (dadi/integration2D.c:42-49,
            // integration_shared.c:72-93), each rounded as the reference does
            const double d2 = xm(2.0, g.dx[i]);
            v.G[i] = msel_ref(g.xInt[i], s.gamma, s.h);
            v.Pv[i] = xd(vfunc_ref(g.x[i], s.nu, beta1), d2);
            v.Qv[i] = xd(vfunc_ref(g.x[i + 1], s.nu, beta1), d2);
            v.VI[i] = vfunc_ref(g.xInt[i], s.nu, beta1);
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
        v.DF[i] = g.dfac[i]; // unscaled: the delj rows are the reference's
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

// Chang-Cooper delta_j (dadi/integration_shared.c:52-70) for one interval,
// in the reference's order.
__device__ __forceinline__ double delj_of(double MInt, double VInt, double dx)
{
    const double wj = xm(xm(2.0, MInt), dx);
    const double epsj = exp(xd(wj, VInt));
    if ((epsj != 1.0) && (wj != 0))
        return xd(xs(xa(xm(-epsj, wj), xm(epsj, VInt)), VInt), xs(wj, xm(epsj, wj)));
    return 0.5;
}

// Thomas solve of one line with the delj trick, as the reference computes
// it: MInt per interval as Mfunc{1..5}D (dadi/integration_shared.c:12-30:
// the migration terms m_k (o_k - x) summed in increasing axis order, then
// the selection term), delta_j, the unscaled rows of compute_abc_nobc
// (:72-93, b = 1/dt + ...), the corner terms of dadi/integration2D.c:67-70
// when c0 / c1 (this line's other coordinates are all 0 / all 1; always in
// one dimension, integration1D.c:47-51), r = phi/dt, and tridiag_premalloc
// (dadi/tridiag.c:14-34).  The gam scratch holds element p at gm[p*gs].
template <typename TP, typename TG>
__device__ __forceinline__ void solve_line_delj(TP *__restrict__ ph, int sp, TG *__restrict__ gm,
                                                int gs, int L, const double *mo,
                                                const double *oo, int nother, bool c0, bool c1,
                                                const GridVecs &gv, const AxisVecs &v,
                                                const AxisScalars &s)
{
    auto mfun = [&](double x, double sel) {
        if (nother == 0)
            return sel;
        double acc = xm(mo[0], xs(oo[0], x));
        for (int j = 1; j < nother; j++)
            acc = xa(acc, xm(mo[j], xs(oo[j], x)));
        return xa(acc, sel);
    };
    const double dt = s.dt;
    const double idt = xd(1.0, dt);
    // interval 0: atemp, ctemp (compute_abc_nobc)
    double Mk = mfun(gv.xInt[0], v.G[0]);
    double d = delj_of(Mk, v.VI[0], gv.dx[0]);
    double at = xa(xm(Mk, d), v.Pv[0]);
    double ct = xa(xm(-Mk, xs(1.0, d)), v.Qv[0]);
    double b = xa(idt, xm(v.DF[0], at));
    if (c0) {
        const double mf = mfun(gv.x[0], msel_ref(gv.x[0], s.gamma, s.h));
        if (mf <= 0)
            b = xa(b, xd(xm(xs(xd(0.5, s.nu), mf), 2.0), gv.dx[0]));
    }
    double bet = b;
    double u = xd(xd((double)ph[0], dt), bet);
    ph[0] = u;
    double cprev = -xm(v.DF[0], ct);
    for (int i = 1; i < L; i++) {
        const double a = -xm(v.DF[i], at);
        double bb = xa(idt, xm(v.DF[i], ct));
        double cnext = 0;
        if (i < L - 1) {
            Mk = mfun(gv.xInt[i], v.G[i]);
            d = delj_of(Mk, v.VI[i], gv.dx[i]);
            at = xa(xm(Mk, d), v.Pv[i]);
            ct = xa(xm(-Mk, xs(1.0, d)), v.Qv[i]);
            bb = xa(bb, xm(v.DF[i], at));
            cnext = -xm(v.DF[i], ct);
        } else if (c1) {
            const double ml = mfun(gv.x[L - 1], msel_ref(gv.x[L - 1], s.gamma, s.h));
            if (ml >= 0)
                bb = xa(bb, xd(xm(-xs(-xd(0.5, s.nu), ml), 2.0), gv.dx[L - 2]));
        }
        const double g = xd(cprev, bet);
        gm[i * gs] = g;
        bet = xs(bb, xm(a, g));
        u = xd(xs(xd((double)ph[i * sp], dt), xm(a, u)), bet);
        ph[i * sp] = u;
        cprev = cnext;
    }
    for (int i = L - 2; i >= 0; i--) {
        u = xs((double)ph[i * sp], xm((double)gm[(i + 1) * gs], u));
        ph[i * sp] = u;
    }
}

} // namespace dgb
