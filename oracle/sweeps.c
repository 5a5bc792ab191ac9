/*
 * ORACLE -- test infrastructure only.
 *
 * A plain-C CPU restatement of dadi's implicit ADI sweep (the per-axis
 * coefficient build plus the Numerical-Recipes Thomas solve) for 1..4
 * populations, written generically over the number of dimensions and the
 * swept axis.  It exists so that tests/, the smoke check and bench.py's CPU
 * baseline can compare the CUDA kernels against the reference arithmetic.
 * Nothing in the shipped package links, imports or calls this file.
 *
 * Every function follows the reference operation order (same association of
 * + and *, same divisions) so that, compiled with -ffp-contract=off, its
 * output is bit-identical to the reference C integrator on the same inputs.
 * References are to dadi 2.4.3 (dadi/...).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MAXDIM 5

/* Numerical Recipes tridiagonal solve without pivoting
 * (dadi/tridiag.c:14-34).  gam is caller-provided scratch of n doubles. */
void orc_tridiag(const double *a, const double *b, const double *c,
                 const double *r, double *u, int n, double *gam)
{
    double bet = b[0];
    u[0] = r[0] / bet;
    for (int j = 1; j < n; j++) {
        gam[j] = c[j - 1] / bet;
        bet = b[j] - a[j] * gam[j];
        u[j] = (r[j] - a[j] * u[j - 1]) / bet;
    }
    for (int j = n - 2; j >= 0; j--)
        u[j] -= gam[j + 1] * u[j + 1];
}

/* V(x) = x(1-x)/nu (dadi/integration_shared.c:4-6). */
static double orc_V(double x, double nu) { return 1. / nu * x * (1. - x); }

/* V with breeding ratio beta (dadi/integration_shared.c:8-10). */
static double orc_Vbeta(double x, double nu, double beta)
{
    return 1. / nu * x * (1. - x) * pow(beta + 1, 2) / (4 * beta);
}

/* Selection part of M (dadi/integration_shared.c:12-14). */
static double orc_Msel(double x, double gamma, double h)
{
    return gamma * 2 * (h + (1. - 2 * h) * x) * x * (1. - x);
}

/* M(x; others) = sum_k m_k (o_k - x) + selection, summed left to right over
 * the other axes in increasing order (dadi/integration_shared.c:15-30). */
static double orc_M(double x, int nother, const double *o, const double *m,
                    double gamma, double h)
{
    if (nother == 0)
        return orc_Msel(x, gamma, h);
    double acc = m[0] * (o[0] - x);
    for (int k = 1; k < nother; k++)
        acc = acc + m[k] * (o[k] - x);
    return acc + orc_Msel(x, gamma, h);
}

/* exp(z), or (exp_mode != 0) the other neighbour of the true value for
 * about half of the arguments (picked by a hash of z's bits): the result of
 * another faithfully rounded exp, such as one with a 1-ulp error bound.
 * Used only to measure how far an equally valid exp moves the reference's
 * results under the delj trick (its noise floor). */
static double orc_exp(double z, int exp_mode)
{
    double e = exp(z);
    if (!exp_mode)
        return e;
    unsigned long long b;
    memcpy(&b, &z, sizeof b);
    b ^= b >> 29;
    b *= 0xbf58476d1ce4e5b9ull;
    b ^= b >> 32;
    if (b & 1)
        return nextafter(e, (b & 2) ? INFINITY : 0.0);
    return e;
}

/* Chang-Cooper delta_j, or 0.5 (dadi/integration_shared.c:52-70). */
static void orc_delj(const double *dx, const double *MInt, const double *VInt,
                     int n, double *delj, int use_delj_trick, int exp_mode)
{
    for (int i = 0; i < n - 1; i++) {
        delj[i] = 0.5;
        if (!use_delj_trick)
            continue;
        double wj = 2 * MInt[i] * dx[i];
        double epsj = orc_exp(wj / VInt[i], exp_mode);
        if ((epsj != 1.0) && (wj != 0))
            delj[i] = (-epsj * wj + epsj * VInt[i] - VInt[i]) / (wj - epsj * wj);
    }
}

/* Fully implicit a, b, c without boundary terms
 * (dadi/integration_shared.c:72-93). */
static void orc_abc(const double *dx, const double *dfac, const double *delj,
                    const double *MInt, const double *V, double dt, int n,
                    double *a, double *b, double *c)
{
    a[0] = 0;
    c[n - 1] = 0;
    for (int i = 0; i < n; i++)
        b[i] = 1. / dt;
    for (int i = 0; i < n - 1; i++) {
        double at = MInt[i] * delj[i] + V[i] / (2 * dx[i]);
        a[i + 1] = -dfac[i + 1] * at;
        b[i] += dfac[i] * at;
        double ct = -MInt[i] * (1 - delj[i]) + V[i + 1] / (2 * dx[i]);
        b[i + 1] += dfac[i + 1] * ct;
        c[i] = -dfac[i] * ct;
    }
}

/* Per-axis grid quantities: dx, dfactor, xInt
 * (dadi/integration_shared.c:32-50). */
static void orc_grid(const double *xx, int n, double *dx, double *dfac,
                     double *xInt)
{
    for (int i = 0; i < n - 1; i++)
        dx[i] = xx[i + 1] - xx[i];
    for (int i = 1; i < n - 1; i++)
        dfac[i] = 2. / (dx[i] + dx[i - 1]);
    dfac[0] = 2. / dx[0];
    dfac[n - 1] = 2. / dx[n - 2];
    for (int i = 0; i < n - 1; i++)
        xInt[i] = 0.5 * (xx[i + 1] + xx[i]);
}

/* Line enumeration helper: for a C-ordered array with ndim axes of length L,
 * the start offset of line number `line` along `axis` and the coordinates of
 * the other axes (in increasing axis order). */
static long orc_line_start(int ndim, int L, int axis, long line, int *coords)
{
    long start = 0, stride = 1;
    int nk = 0;
    int tmp[ORC_MAXDIM];
    for (int ax = ndim - 1; ax >= 0; ax--) {
        if (ax == axis) {
            stride *= L;
            continue;
        }
        int idx = (int)(line % L);
        line /= L;
        tmp[ax] = idx;
        start += idx * stride;
        stride *= L;
    }
    for (int ax = 0; ax < ndim; ax++)
        if (ax != axis)
            coords[nk++] = tmp[ax];
    return start;
}

static long orc_ipow(int L, int p)
{
    long r = 1;
    for (int i = 0; i < p; i++)
        r *= L;
    return r;
}

/*
 * One implicit sweep along `axis` of phi (ndim axes, each of length L, on the
 * common grid xx), with the population parameters of the swept axis.
 * mig[k] is the migration rate into the swept population from population k
 * (mig[axis] is ignored).  ndim == 1 uses V with beta and unconditional
 * no-flux boundary terms (dadi/integration1D.c:7-66); ndim >= 2 applies the
 * boundary terms only on the line whose other coordinates are all 0 (start)
 * or all 1 (end) (dadi/integration2D.c:19-160, integration3D.c:13-239,
 * integration4D.c:13-321).  r = phi/dt.
 */
static int orc_sweep_impl(double *phi, int ndim, int L, int axis, const double *xx,
                          double nu, const double *mig, double gamma, double h,
                          double beta, double dt, int use_delj_trick, int r_mode);

int orc_sweep(double *phi, int ndim, int L, int axis, const double *xx,
              double nu, const double *mig, double gamma, double h,
              double beta, double dt, int use_delj_trick)
{
    return orc_sweep_impl(phi, ndim, L, axis, xx, nu, mig, gamma, h, beta, dt,
                          use_delj_trick, 0);
}

/* The same sweep with the right-hand side formed as (1/dt)*phi -- the form the
 * reference's own constant-parameter sweeps use (dadi/integration2D.c:177) --
 * instead of phi/dt.  Used only to measure how far an equally valid rounding
 * of the reference moves its results (its noise floor). */
int orc_sweep_rhs_variant(double *phi, int ndim, int L, int axis, const double *xx,
                          double nu, const double *mig, double gamma, double h,
                          double beta, double dt, int use_delj_trick)
{
    return orc_sweep_impl(phi, ndim, L, axis, xx, nu, mig, gamma, h, beta, dt,
                          use_delj_trick, 1);
}

/* The same sweep with exp replaced by another faithfully rounded exp (see
 * orc_exp): the reference's noise floor under the delj trick. */
int orc_sweep_exp_variant(double *phi, int ndim, int L, int axis, const double *xx,
                          double nu, const double *mig, double gamma, double h,
                          double beta, double dt, int use_delj_trick)
{
    return orc_sweep_impl(phi, ndim, L, axis, xx, nu, mig, gamma, h, beta, dt,
                          use_delj_trick, 2);
}

static int orc_sweep_impl(double *phi, int ndim, int L, int axis, const double *xx,
                          double nu, const double *mig, double gamma, double h,
                          double beta, double dt, int use_delj_trick, int r_mode)
{
    if (ndim < 1 || ndim > ORC_MAXDIM || axis < 0 || axis >= ndim || L < 3)
        return -1;
    double *w = malloc(sizeof(double) * 13 * L);
    if (!w)
        return -2;
    double *dx = w, *dfac = w + L, *xInt = w + 2 * L, *MInt = w + 3 * L,
           *V = w + 4 * L, *VInt = w + 5 * L, *delj = w + 6 * L,
           *a = w + 7 * L, *b = w + 8 * L, *c = w + 9 * L, *r = w + 10 * L,
           *u = w + 11 * L, *gam = w + 12 * L;
    orc_grid(xx, L, dx, dfac, xInt);
    for (int i = 0; i < L; i++)
        V[i] = ndim == 1 ? orc_Vbeta(xx[i], nu, beta) : orc_V(xx[i], nu);
    for (int i = 0; i < L - 1; i++)
        VInt[i] = ndim == 1 ? orc_Vbeta(xInt[i], nu, beta) : orc_V(xInt[i], nu);

    int nother = ndim - 1;
    double mo[ORC_MAXDIM];
    for (int ax = 0, k = 0; ax < ndim; ax++)
        if (ax != axis)
            mo[k++] = mig[ax];
    long stride = orc_ipow(L, ndim - 1 - axis);
    long nlines = orc_ipow(L, ndim - 1);
    int coords[ORC_MAXDIM];
    double o[ORC_MAXDIM];
    for (long line = 0; line < nlines; line++) {
        long s0 = orc_line_start(ndim, L, axis, line, coords);
        int all0 = 1, all1 = 1;
        for (int k = 0; k < nother; k++) {
            o[k] = xx[coords[k]];
            all0 = all0 && (o[k] == 0);
            all1 = all1 && (o[k] == 1);
        }
        double Mfirst = orc_M(xx[0], nother, o, mo, gamma, h);
        double Mlast = orc_M(xx[L - 1], nother, o, mo, gamma, h);
        for (int i = 0; i < L - 1; i++)
            MInt[i] = orc_M(xInt[i], nother, o, mo, gamma, h);
        orc_delj(dx, MInt, VInt, L, delj, use_delj_trick, r_mode == 2);
        orc_abc(dx, dfac, delj, MInt, V, dt, L, a, b, c);
        for (int i = 0; i < L; i++)
            r[i] = (r_mode == 1) ? (1 / dt) * phi[s0 + i * stride] : phi[s0 + i * stride] / dt;
        if (all0 && Mfirst <= 0)
            b[0] += (0.5 / nu - Mfirst) * 2. / dx[0];
        if (all1 && Mlast >= 0)
            b[L - 1] += -(-0.5 / nu - Mlast) * 2. / dx[L - 2];
        orc_tridiag(a, b, c, r, u, L, gam);
        for (int i = 0; i < L; i++)
            phi[s0 + i * stride] = u[i];
    }
    free(w);
    return 0;
}

/*
 * Constant-coefficient sweep: a, b, c are full arrays shaped like phi, with b
 * excluding the 1/dt term; b + 1/dt and r = (1/dt) * phi per element
 * (dadi/integration2D.c:162-217, integration3D.c:241-345).
 */
int orc_sweep_precalc(double *phi, int ndim, int L, int axis, const double *ax,
                      const double *bx, const double *cx, double dt)
{
    if (ndim < 1 || ndim > ORC_MAXDIM || axis < 0 || axis >= ndim || L < 2)
        return -1;
    double *w = malloc(sizeof(double) * 6 * L);
    if (!w)
        return -2;
    double *a = w, *b = w + L, *c = w + 2 * L, *r = w + 3 * L, *u = w + 4 * L,
           *gam = w + 5 * L;
    long stride = orc_ipow(L, ndim - 1 - axis);
    long nlines = orc_ipow(L, ndim - 1);
    int coords[ORC_MAXDIM];
    for (long line = 0; line < nlines; line++) {
        long s0 = orc_line_start(ndim, L, axis, line, coords);
        for (int i = 0; i < L; i++) {
            long idx = s0 + i * stride;
            a[i] = ax[idx];
            b[i] = bx[idx] + 1 / dt;
            c[i] = cx[idx];
            r[i] = 1 / dt * phi[idx];
        }
        orc_tridiag(a, b, c, r, u, L, gam);
        for (int i = 0; i < L; i++)
            phi[s0 + i * stride] = u[i];
    }
    free(w);
    return 0;
}

/* Plain tridiagonal solve entry point for tests (dadi/tridiag.c:36-40). */
int orc_tridiag_solve(const double *a, const double *b, const double *c,
                      const double *r, double *u, int n)
{
    double *gam = malloc(sizeof(double) * (n > 0 ? n : 1));
    if (!gam)
        return -2;
    orc_tridiag(a, b, c, r, u, n, gam);
    free(gam);
    return 0;
}

/* Steps taken by the two_pops time loop (dadi/Integration.py:346-386, dt by
 * _compute_dt, :147-176) of Demographics2D.IM (dadi/Demographics2D.py:
 * 297-307) for each parameter row (s, nu1, nu2, T, m12, m21):
 * nu1(t) = s (nu1/s)^(t/T), nu2(t) = (1-s) (nu2/(1-s))^(t/T), constant
 * migration, no selection.  The walk uses the reference's operations in
 * its order (libm pow, Python's max/min keeping the first extreme), so the
 * counts equal the reference loop's.  A walk that passes max_steps stops
 * there and reports max_steps + 1. */
static double orc_im_dt(double nu, double m, double tsf)
{
    double mx = 0.25 / nu;
    if (m > mx)
        mx = m;
    if (0.0 > mx) /* |gamma| * 2 * ... with gamma = 0 */
        mx = 0.0;
    return mx > 0 ? tsf / mx : INFINITY;
}

int orc_im_steps(const double *params, long n, double tsf, long max_steps, long *steps)
{
    for (long i = 0; i < n; i++) {
        const double *p = params + 6 * i;
        const double s = p[0], nu1 = p[1], nu2 = p[2], T = p[3], m12 = p[4], m21 = p[5];
        double t = 0.0;
        double n1 = s * pow(nu1 / s, t / T), n2 = (1 - s) * pow(nu2 / (1 - s), t / T);
        long k = 0;
        while (t < T && k <= max_steps) {
            double d1 = orc_im_dt(n1, m12, tsf), d2 = orc_im_dt(n2, m21, tsf);
            double dt = (d2 < d1) ? d2 : d1;
            double rest = T - t;
            double this_dt = (rest < dt) ? rest : dt;
            t = t + this_dt;
            n1 = s * pow(nu1 / s, t / T);
            n2 = (1 - s) * pow(nu2 / (1 - s), t / T);
            k++;
        }
        steps[i] = k;
    }
    return 0;
}
