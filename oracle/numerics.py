"""ORACLE -- test infrastructure only.

numpy restatement of the host-side pieces around dadi's integrator: the default
grid, the equilibrium initial condition and population splits, the
piecewise-linear from_phi contraction, Richardson extrapolation and the Poisson
likelihood, each citing the dadi 2.4.3 file:line it follows.
"""
import numpy as np
from scipy.special import betainc, gammaln

from . import integration as oint


def default_grid(pts, crwd=8.):
    """dadi/Numerics.py:215-231 (exponential_grid = default_grid)."""
    unif = np.linspace(-1, 1, pts)
    grid = 1. / (1. + np.exp(-crwd * unif))
    return (grid - grid[0]) / (grid[-1] - grid[0])


def phi_1D(xx, nu=1.0, theta0=1.0, gamma=0, beta=1):
    """Equilibrium 1-D density for h == 0.5 (dadi/PhiManip.py:12-42, 110-190)."""
    if gamma == 0:
        phi = 0 * xx
        phi[1:] = nu * theta0 / xx[1:]
        phi[0] = phi[1]
        return phi * 4. * beta / (beta + 1.) ** 2
    gamma = gamma * 4. * beta / (beta + 1.) ** 2
    exp = np.exp
    phi = 0 * xx
    if gamma > -300:
        phi[1:-1] = 1. / (xx[1:-1] * (1 - xx[1:-1])) \
            * (1 - exp(-2 * gamma * (1 - xx[1:-1]))) / (1 - exp(-2 * gamma))
    else:
        phi[1:-1] = 1. / (xx[1:-1] * (1 - xx[1:-1])) * exp(2 * gamma * xx[1:-1])
    phi[0] = phi[1]
    if gamma < 300:
        limit = 2 * gamma * exp(2 * gamma) / (exp(2 * gamma) - 1)
    else:
        limit = 2 * gamma
    phi[-1] = limit
    return phi * nu * theta0 * 4. * beta / (beta + 1.) ** 2


def phi_1D_to_2D(xx, phi_1D):
    """dadi/PhiManip.py:214-234."""
    pts = len(xx)
    phi_2D = np.zeros((pts, pts))
    for ii in range(1, pts - 1):
        phi_2D[ii, ii] = phi_1D[ii] * 2 / (xx[ii + 1] - xx[ii - 1])
    return phi_2D


def _admix_place(phi, ad_z, zz):
    """dadi/PhiManip.py:268-301 (_admixture_intermediates)."""
    upper = np.searchsorted(zz, ad_z)
    upper = np.minimum(upper, len(zz) - 1)
    upper = np.maximum(upper, 1)
    lower = upper - 1
    uz, lz = zz[upper], zz[lower]
    delz0 = np.where(lower == 0, 0, zz[lower] - zz[lower - 1])
    delz1 = np.where(upper == 0, 0, zz[upper] - zz[lower])
    delz2 = np.where(upper == len(zz) - 1, 0, zz[(upper + 1) % len(zz)] - zz[upper])
    frac_lower = (uz - ad_z) / (uz - lz)
    frac_upper = (ad_z - lz) / (uz - lz)
    norm = 2 * phi / (frac_lower * delz0 + delz1 + frac_upper * delz2)
    return lower, upper, frac_lower, frac_upper, norm


def phi_2D_to_3D_admix(phi, f1, xx, yy, zz):
    """dadi/PhiManip.py:372-409; split_2 is f1 = 0 (:236-250)."""
    ad_z = f1 * xx[:, None] + (1 - f1) * yy[None, :]
    lo, up, fl, fu, norm = _admix_place(phi, ad_z, zz)
    ii = np.arange(len(xx))[:, None]
    jj = np.arange(len(yy))[None, :]
    out = np.zeros((len(xx), len(yy), len(zz)))
    out[ii, jj, lo] = fl * norm
    out[ii, jj, up] += fu * norm
    return out


def phi_3D_to_4D(phi, f1, f2, xx, yy, zz, aa):
    """dadi/PhiManip.py:412-450."""
    ad_w = f1 * xx[:, None, None] + f2 * yy[None, :, None] + (1 - f1 - f2) * zz[None, None, :]
    lo, up, fl, fu, norm = _admix_place(phi, ad_w, aa)
    ii = np.arange(len(xx))[:, None, None]
    jj = np.arange(len(yy))[None, :, None]
    kk = np.arange(len(zz))[None, None, :]
    out = np.zeros((len(xx), len(yy), len(zz), len(aa)))
    out[ii, jj, kk, lo] = fl * norm
    out[ii, jj, kk, up] += fu * norm
    return out


def dbeta_tables(n, xx):
    """dadi/Spectrum_mod.py:25-40 (cached_dbeta)."""
    xx = np.minimum(np.maximum(xx, 0), 1.0)
    d1 = np.empty((n + 1, len(xx) - 1))
    d2 = np.empty((n + 1, len(xx) - 1))
    for i in range(n + 1):
        b = betainc(i + 1, n - i + 1, xx)
        d1[i] = b[1:] - b[:-1]
        b = betainc(i + 2, n - i + 1, xx)
        d2[i] = b[1:] - b[:-1]
    return d1, d2


def from_phi_1D(n, xx, phi):
    """dadi/Spectrum_mod.py:1307-1345 (analytic, divergent=False)."""
    data = np.zeros(n + 1)
    xx = np.minimum(np.maximum(xx, 0), 1.0)
    s = (phi[1:] - phi[:-1]) / (xx[1:] - xx[:-1])
    c1 = (phi[:-1] - s * xx[:-1]) / (n + 1)
    for d in range(n + 1):
        c2 = s * (d + 1) / ((n + 1) * (n + 2))
        b1 = betainc(d + 1, n - d + 1, xx)
        b2 = betainc(d + 2, n - d + 1, xx)
        data[d] = np.sum(c1 * (b1[1:] - b1[:-1]) + c2 * (b2[1:] - b2[:-1]))
    return data


def from_phi_2D(nx, ny, xx, yy, phi):
    """dadi/Spectrum_mod.py:1509-1547 (_from_phi_2D_linalg, raw data)."""
    d1x, d2x = dbeta_tables(nx, xx)
    d1y, d2y = dbeta_tables(ny, yy)
    s_yy = (phi[:, 1:] - phi[:, :-1]) / (yy[None, 1:] - yy[None, :-1])
    c1_yy = (phi[:, :-1] - s_yy * yy[None, :-1]) / (ny + 1)
    t1 = np.dot(d1y, c1_yy.T)
    t2 = np.dot(d2y, s_yy.T)
    t2 *= np.arange(1, ny + 2)[:, None] / ((ny + 1) * (ny + 2))
    over_y = t1 + t2
    s_xx = (over_y[:, 1:] - over_y[:, :-1]) / (xx[1:] - xx[:-1])
    c1_xx = (over_y[:, :-1] - s_xx * xx[:-1]) / (nx + 1)
    t1 = np.dot(d1x, c1_xx.T)
    t2 = np.dot(d2x, s_xx.T)
    t2 *= np.arange(1, nx + 2)[:, None] / ((nx + 1) * (nx + 2))
    return t1 + t2


def from_phi_3D(nx, ny, nz, xx, yy, zz, phi):
    """dadi/Spectrum_mod.py:1774-1810 (_from_phi_3D_linalg, raw data)."""
    data = np.zeros((nx + 1, ny + 1, nz + 1))
    d1z, d2z = dbeta_tables(nz, zz)
    s_zz = (phi[:, :, 1:] - phi[:, :, :-1]) / (zz[None, None, 1:] - zz[None, None, :-1])
    c1_zz = (phi[:, :, :-1] - s_zz * zz[None, None, :-1]) / (nz + 1)
    for kk in range(nz + 1):
        t1 = np.dot(c1_zz, d1z[kk])
        t2 = np.dot(s_zz, d2z[kk])
        t2 *= (kk + 1) / ((nz + 1) * (nz + 2))
        data[:, :, kk] = from_phi_2D(nx, ny, xx, yy, t1 + t2)
    return data


def from_phi_4D(nx, ny, nz, na, xx, yy, zz, aa, phi):
    """dadi/Spectrum_mod.py:1841-1870 (_from_phi_4D_linalg, raw data)."""
    data = np.zeros((nx + 1, ny + 1, nz + 1, na + 1))
    d1a, d2a = dbeta_tables(na, aa)
    s_aa = (phi[:, :, :, 1:] - phi[:, :, :, :-1]) / (aa[1:] - aa[:-1])
    c1_aa = (phi[:, :, :, :-1] - s_aa * aa[:-1]) / (na + 1)
    for ll in range(na + 1):
        t1 = np.dot(c1_aa, d1a[ll])
        t2 = np.dot(s_aa, d2a[ll])
        t2 *= (ll + 1) / ((na + 1) * (na + 2))
        data[:, :, :, ll] = from_phi_3D(nx, ny, nz, xx, yy, zz, t1 + t2)
    return data


def from_phi(phi, ns, xx):
    """Dispatch on dimension (dadi/Spectrum_mod.py:1938-2061), square grids."""
    P = phi.ndim
    if P == 1:
        return from_phi_1D(ns[0], xx, phi)
    if P == 2:
        return from_phi_2D(ns[0], ns[1], xx, xx, phi)
    if P == 3:
        return from_phi_3D(ns[0], ns[1], ns[2], xx, xx, xx, phi)
    if P == 4:
        return from_phi_4D(*ns, xx, xx, xx, xx, phi)
    raise ValueError(P)


def corner_mask(shape):
    """Masked 'absent' and 'fixed' entries (dadi/Spectrum_mod.py:178-182)."""
    m = np.zeros(shape, dtype=bool)
    m.flat[0] = m.flat[-1] = True
    return m


def linear_extrap(ys, xs):
    """dadi/Numerics.py:644-654."""
    y1, y2 = ys
    x1, x2 = xs
    return (x2 * y1 - x1 * y2) / (x2 - x1)


def quadratic_extrap(ys, xs):
    """dadi/Numerics.py:657-669."""
    y1, y2, y3 = ys
    x1, x2, x3 = xs
    return x2 * x3 / ((x1 - x2) * (x1 - x3)) * y1 + x1 * x3 / ((x2 - x1) * (x2 - x3)) * y2 \
        + x1 * x2 / ((x3 - x1) * (x3 - x2)) * y3


def extrapolate(results, x_l, fail_mag=10):
    """Richardson extrapolation with the fail_mag guard (dadi/Numerics.py:425-464)."""
    if len(results) == 1:
        return results[0].copy()
    ex = linear_extrap(results, x_l) if len(results) == 2 else quadratic_extrap(results, x_l)
    best = results[int(np.argmin(x_l))]
    with np.errstate(all='ignore'):
        failed = abs(np.log10(ex / best)) > fail_mag
    ex = np.array(ex, copy=True)
    ex[failed] = best[failed]
    return ex


def ll(model, data, mask):
    """Poisson log-likelihood over entries unmasked and with model > 0
    (dadi/Inference.py:466-509; numpy.ma.log masks model <= 0)."""
    ok = ~mask & (model > 0)
    return float(np.sum(-model[ok] + data[ok] * np.log(model[ok]) - gammaln(data[ok] + 1.)))


def ll_multinom(model, data, mask):
    """dadi/Inference.py:559-575 with optimal_sfs_scaling (:668-685)."""
    theta = data[~mask].sum() / model[~mask].sum()
    return ll(theta * model, data, mask)


# ---- the workloads' demographic models (dadi/Demographics2D.py:133-167, 268-309) ----

def split_mig(params, ns, pts):
    nu1, nu2, T, m = params
    xx = default_grid(pts)
    phi = phi_1D_to_2D(xx, phi_1D(xx))
    phi = oint.two_pops(phi, xx, T, nu1, nu2, m12=m, m21=m)
    return from_phi(phi, ns, xx), xx


def IM(params, ns, pts):
    s, nu1, nu2, T, m12, m21 = params
    xx = default_grid(pts)
    phi = phi_1D_to_2D(xx, phi_1D(xx))
    nu1_func = lambda t: s * (nu1 / s) ** (t / T)
    nu2_func = lambda t: (1 - s) * (nu2 / (1 - s)) ** (t / T)
    phi = oint.two_pops(phi, xx, T, nu1_func, nu2_func, m12=m12, m21=m21)
    return from_phi(phi, ns, xx), xx


def growth3(params, ns, pts):
    """Three populations split from one, each growing exponentially:
    nu_i(t) = nu0_i exp(log(nuF_i/nu0_i) t/T), symmetric migration."""
    (nu0, nuF, (m12, m13, m23), gammas, T) = params
    xx = default_grid(pts)
    phi = phi_1D_to_2D(xx, phi_1D(xx))
    phi = phi_2D_to_3D_admix(phi, 0, xx, xx, xx)
    nus = [(lambda a, b: (lambda t: a * np.exp(np.log(b / a) * t / T)))(a, b)
           for a, b in zip(nu0, nuF)]
    phi = oint.three_pops(phi, xx, T, nus[0], nus[1], nus[2],
                          m12=m12, m13=m13, m21=m12, m23=m23, m31=m13, m32=m23,
                          gamma1=gammas[0], gamma2=gammas[1], gamma3=gammas[2])
    return from_phi(phi, ns, xx), xx


def IM_sel(params, ns, pts):
    """DFE.DemogSelModels.IM_sel (dadi/DFE/DemogSelModels.py:162-197): IM_pre_sel
    (:64-121) with nuPre = 1 and TPre = 0, so the ancestral density is
    phi_1D with gamma1 (one_pop over T = 0 returns it unchanged)."""
    s, nu1, nu2, T, m12, m21, gamma1, gamma2 = params
    xx = default_grid(pts)
    phi = phi_1D_to_2D(xx, phi_1D(xx, gamma=gamma1))
    nu1_0, nu2_0 = 1 * s, 1 * (1 - s)
    nu1_func = lambda t: nu1_0 * (nu1 / nu1_0) ** (t / T)
    nu2_func = lambda t: nu2_0 * (nu2 / nu2_0) ** (t / T)
    phi = oint.two_pops(phi, xx, T, nu1_func, nu2_func, m12=m12, m21=m21,
                        gamma1=gamma1, gamma2=gamma2)
    return from_phi(phi, ns, xx), xx


def four_split(params, ns, pts):
    """Four populations split successively from one (dadi/PhiManip.py:
    214-250, 412-450), then four_pops for T with constant sizes and symmetric
    migration m."""
    nu1, nu2, nu3, nu4, m, T = params
    xx = default_grid(pts)
    phi = phi_1D_to_2D(xx, phi_1D(xx))
    phi = phi_2D_to_3D_admix(phi, 0, xx, xx, xx)
    phi = phi_3D_to_4D(phi, 0.0, 0.0, xx, xx, xx, xx)
    phi = oint.four_pops(phi, xx, T, nu1, nu2, nu3, nu4,
                         m12=m, m13=m, m14=m, m21=m, m23=m, m24=m,
                         m31=m, m32=m, m34=m, m41=m, m42=m, m43=m)
    return from_phi(phi, ns, xx), xx


def extrap_model(model, params, ns, pts_l):
    """make_extrap_func(model)(params, ns, pts_l) with extrap_x = xx[1]."""
    res, xs = [], []
    for pts in pts_l:
        fs, xx = model(params, ns, pts)
        res.append(fs)
        xs.append(xx[1])
    return extrapolate(res, xs)
