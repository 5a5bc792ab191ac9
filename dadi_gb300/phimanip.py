"""Initial densities and population splits (dadi/PhiManip.py)."""
import numpy as np
import scipy.integrate


def phi_1D_snm(xx, nu=1.0, theta0=1.0, beta=1):
    """Standard neutral density (dadi/PhiManip.py:166-196)."""
    if xx[0] == 0:
        phi = 0 * xx
        phi[1:] = nu * theta0 / xx[1:]
        phi[0] = phi[1]
    else:
        phi = nu * theta0 / xx
    return phi * 4. * beta / (beta + 1.) ** 2


def phi_1D_genic(xx, nu=1.0, theta0=1.0, gamma=0, beta=1):
    """Equilibrium density under genic selection (dadi/PhiManip.py:110-164)."""
    if gamma == 0:
        return phi_1D_snm(xx, nu, theta0, beta=beta)
    gamma = gamma * 4. * beta / (beta + 1.) ** 2
    exp = np.exp
    if xx[0] == 0 and xx[-1] == 1:
        phi = 0 * xx
        if gamma > -300:
            phi[1:-1] = 1. / (xx[1:-1] * (1 - xx[1:-1])) \
                * (1 - exp(-2 * gamma * (1 - xx[1:-1]))) / (1 - exp(-2 * gamma))
        else:
            phi[1:-1] = 1. / (xx[1:-1] * (1 - xx[1:-1])) * exp(2 * gamma * xx[1:-1])
    else:
        if gamma > -300:
            phi = 1. / (xx * (1 - xx)) * (1 - exp(-2 * gamma * (1 - xx))) / (1 - exp(-2 * gamma))
        else:
            phi = 1. / (xx * (1 - xx)) * exp(2 * gamma * xx)
    if xx[0] == 0:
        phi[0] = phi[1]
    if xx[-1] == 1:
        limit = 2 * gamma * exp(2 * gamma) / (exp(2 * gamma) - 1) if gamma < 300 else 2 * gamma
        phi[-1] = limit
    return phi * nu * theta0 * 4. * beta / (beta + 1.) ** 2


def phi_1D(xx, nu=1.0, theta0=1.0, gamma=0, h=0.5, theta=None, beta=1, deme_ids=None):
    """Equilibrium 1-D density (dadi/PhiManip.py:12-108)."""
    if theta is not None:
        raise ValueError('The parameter theta has been deprecated in favor of parameters nu '
                         'and theta0, for consistency with the Integration functions.')
    if h == 0.5:
        return phi_1D_genic(xx, nu, theta0, gamma, beta=beta)
    # Williamson et al. (2004) eqn 1 with dominance, integrated numerically.
    gamma = gamma * 4. * beta / (beta + 1.) ** 2
    Qadjust = 0
    if gamma < 0 and np.isinf(np.exp(-2 * gamma)):
        Qadjust = -2 * gamma
    integrand = lambda xi: np.exp(-4 * gamma * h * xi - 2 * gamma * (1 - 2 * h) * xi ** 2
                                  - Qadjust)
    int0, _ = scipy.integrate.quad(integrand, 0, 1, epsabs=0, points=np.linspace(0, 1, 41))
    ints = np.empty(len(xx))
    if gamma < 0:
        for ii, q in enumerate(xx):
            ints[ii], _ = scipy.integrate.quad(integrand, q, 1, epsabs=0,
                                               points=np.linspace(q, 1, 41))
        phi = np.exp(4 * gamma * h * xx + 2 * gamma * (1 - 2 * h) * xx ** 2) * ints / int0
    else:
        integrand2 = lambda xi, q: np.exp(-4 * gamma * h * (xi - q)
                                          - 2 * gamma * (1 - 2 * h) * (xi ** 2 - q ** 2))
        for ii, q in enumerate(xx):
            ints[ii], _ = scipy.integrate.quad(integrand2, q, 1, args=(q,))
        phi = ints / int0
    phi[1:-1] *= 1. / (xx[1:-1] * (1 - xx[1:-1]))
    phi[0] = phi[1]
    if Qadjust == 0:
        phi[-1] = 1. / int0
    else:
        phi[-1] = min(phi[-1], phi[-2])
    return phi * nu * theta0 * 4. * beta / (beta + 1.) ** 2


def check_xx(xx):
    """dadi/PhiManip.py:198-212."""
    if not xx[0] == 0 and xx[1] == 1:
        raise ValueError('Input xx argument does not run from 0 to 1.')
    if not np.all(np.diff(xx) >= 0):
        raise ValueError('Input xx argument is not monotonically increasing.')


def _is_cuda(a):
    return hasattr(a, "is_cuda") and bool(a.is_cuda)


def phi_1D_to_2D(xx, phi_1D, deme_ids=None):
    """One-to-two split: mass on the diagonal (dadi/PhiManip.py:214-234).
    A CUDA tensor phi_1D gives a CUDA tensor (the same arithmetic, on the
    device)."""
    check_xx(xx)
    pts = len(xx)
    idx = np.arange(1, pts - 1)
    if _is_cuda(phi_1D):
        import torch
        dev = phi_1D.device
        out = torch.zeros((pts, pts), dtype=torch.float64, device=dev)
        den = torch.from_numpy(np.ascontiguousarray(xx[2:] - xx[:-2])).to(dev)
        ti = torch.from_numpy(idx).to(dev)
        out[ti, ti] = phi_1D[1:-1].to(torch.float64) * 2 / den
        return out
    phi_2D = np.zeros((pts, pts))
    phi_2D[idx, idx] = phi_1D[1:-1] * 2 / (xx[2:] - xx[:-2])
    return phi_2D


def _admixture_intermediates(phi, ad_z, zz):
    """Linear placement of admixed frequencies on zz (dadi/PhiManip.py:268-301).
    The placement depends only on the grids; with a CUDA tensor phi the
    normalisation and the returned weights are device tensors."""
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
    den = frac_lower * delz0 + delz1 + frac_upper * delz2
    if _is_cuda(phi):
        import torch
        dev = phi.device
        t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev)
             for a in (lower, upper, frac_lower, frac_upper, den)]
        lower, upper, frac_lower, frac_upper, den = t
        return lower, upper, frac_lower, frac_upper, 2 * phi.to(torch.float64) / den
    norm = 2 * phi / den
    return lower, upper, frac_lower, frac_upper, norm


def _place(shape, lo, up, fl, fu, norm, like):
    """out[..., lo] = fl * norm; out[..., up] += fu * norm over the leading
    axes (host arrays or device tensors, as `like`)."""
    lead = [np.arange(n).reshape([-1 if k == j else 1 for k in range(len(shape) - 1)])
            for j, n in enumerate(shape[:-1])]
    if _is_cuda(like):
        import torch
        dev = like.device
        out = torch.zeros(shape, dtype=torch.float64, device=dev)
        lead = [torch.from_numpy(a).to(dev) for a in lead]
        out[(*lead, lo)] = fl * norm
        out[(*lead, up)] += fu * norm
        return out
    out = np.zeros(shape)
    out[(*lead, lo)] = fl * norm
    out[(*lead, up)] += fu * norm
    return out


def phi_2D_to_3D_admix(phi, f1, xx, yy, zz, deme_ids=None):
    """Population 3 admixed from 1 and 2 (dadi/PhiManip.py:372-409)."""
    ad_z = f1 * xx[:, None] + (1 - f1) * yy[None, :]
    lo, up, fl, fu, norm = _admixture_intermediates(phi, ad_z, zz)
    return _place((len(xx), len(yy), len(zz)), lo, up, fl, fu, norm, phi)


def phi_2D_to_3D_split_2(xx, phi_2D, deme_ids=None):
    """Split population 2 into 2 and 3 (dadi/PhiManip.py:236-250)."""
    check_xx(xx)
    return phi_2D_to_3D_admix(phi_2D, 0, xx, xx, xx)


def phi_2D_to_3D_split_1(xx, phi_2D, deme_ids=None):
    """Split population 1 into 1 and 3 (dadi/PhiManip.py:252-266)."""
    check_xx(xx)
    return phi_2D_to_3D_admix(phi_2D, 1, xx, xx, xx)


def phi_3D_to_4D(phi, f1, f2, xx, yy, zz, aa, deme_ids=None):
    """Population 4 from 1, 2 and 3 (dadi/PhiManip.py:412-450)."""
    ad_w = f1 * xx[:, None, None] + f2 * yy[None, :, None] + (1 - f1 - f2) * zz[None, None, :]
    lo, up, fl, fu, norm = _admixture_intermediates(phi, ad_w, aa)
    return _place((len(xx), len(yy), len(zz), len(aa)), lo, up, fl, fu, norm, phi)


def phi_4D_to_5D(phi, f1, f2, f3, xx, yy, zz, aa, bb, deme_ids=None):
    """Population 5 from populations 1-4 (dadi/PhiManip.py:453-490, with
    _four_pop_admixture_intermediates :333-352)."""
    if f1 + f2 + f3 > 1:
        raise ValueError('Admixture proportions (f1=%f, f2 = %f, f3=%f) are '
                         'non-sensible.' % (f1, f2, f3))
    ad_w = f1 * xx[:, None, None, None] + f2 * yy[None, :, None, None] \
        + f3 * zz[None, None, :, None] + (1 - f1 - f2 - f3) * aa[None, None, None, :]
    lo, up, fl, fu, norm = _admixture_intermediates(phi, ad_w, bb)
    return _place((len(xx), len(yy), len(zz), len(aa), len(bb)), lo, up, fl, fu, norm, phi)


#: dadi's name for phi_2D_to_3D_admix (dadi/PhiManip.py:410).
phi_2D_to_3D = phi_2D_to_3D_admix


def trapz(yy, xx, axis=-1):
    """Composite trapezoid rule of yy over the 1-D grid xx along `axis`
    (dadi/Numerics.py:303-332): sum of dx * (y_i + y_{i+1}) / 2."""
    yy = np.asanyarray(yy)
    nd = yy.ndim
    dx = np.diff(xx)
    s1 = [slice(None)] * nd
    s2 = [slice(None)] * nd
    sx = [None] * nd
    s1[axis], s2[axis], sx[axis] = slice(1, None), slice(None, -1), slice(None)
    return np.sum(dx[tuple(sx)] * (yy[tuple(s1)] + yy[tuple(s2)]) / 2.0, axis=axis)


def remove_pop(phi, xx, popnum):
    """Density with population popnum (numbered from 1) integrated out
    (dadi/PhiManip.py:1036-1051)."""
    return trapz(phi, xx, axis=popnum - 1)

