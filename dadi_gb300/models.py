"""The demographic models of the benchmark workloads, on the GPU integrator.

split_mig and IM follow dadi/Demographics2D.py:133-167 and 268-309; growth3
is three populations split from one (dadi/PhiManip.py:236-250) that each grow
exponentially, nu_i(t) = nu0_i exp(log(nuF_i/nu0_i) t/T), with symmetric
migration and per-population selection.
"""
import numpy as np

from . import integration, numerics, phimanip, spectrum


def snm_1d(notused, ns, pts):
    """Standard neutral model (dadi/Demographics1D.py:9-27): the equilibrium
    density, no integration."""
    xx = numerics.default_grid(pts)
    return spectrum.from_phi(phimanip.phi_1D(xx), ns, (xx,))


def two_epoch(params, ns, pts):
    """Instantaneous size change to nu, T ago (dadi/Demographics1D.py:29-50)."""
    nu, T = params
    xx = numerics.default_grid(pts)
    phi = integration.one_pop(phimanip.phi_1D(xx), xx, T, nu)
    return spectrum.from_phi(phi, ns, (xx,))


def split_mig(params, ns, pts):
    nu1, nu2, T, m = params
    xx = numerics.default_grid(pts)
    phi = phimanip.phi_1D_to_2D(xx, phimanip.phi_1D(xx))
    phi = integration.two_pops(phi, xx, T, nu1, nu2, m12=m, m21=m)
    return spectrum.from_phi(phi, ns, (xx, xx))


split_mig.__param_names__ = ['nu1', 'nu2', 'T', 'm']


def IM(params, ns, pts):
    s, nu1, nu2, T, m12, m21 = params
    xx = numerics.default_grid(pts)
    phi = phimanip.phi_1D_to_2D(xx, phimanip.phi_1D(xx))
    nu1_func = lambda t: s * (nu1 / s) ** (t / T)
    nu2_func = lambda t: (1 - s) * (nu2 / (1 - s)) ** (t / T)
    phi = integration.two_pops(phi, xx, T, nu1_func, nu2_func, m12=m12, m21=m21)
    return spectrum.from_phi(phi, ns, (xx, xx))


IM.__param_names__ = ['s', 'nu1', 'nu2', 'T', 'm12', 'm21']


def IM_sel(params, ns, pts):
    """IM with selection (dadi/DFE/DemogSelModels.py:162-197, via IM_pre_sel
    :64-121 with nuPre = 1, TPre = 0): the ancestral density is phi_1D with
    gamma1, then IM's growth with gamma1 / gamma2 in the two populations."""
    s, nu1, nu2, T, m12, m21, gamma1, gamma2 = params
    xx = numerics.default_grid(pts)
    phi = phimanip.phi_1D_to_2D(xx, phimanip.phi_1D(xx, gamma=gamma1))
    nu1_0, nu2_0 = 1.0 * s, 1.0 * (1 - s)
    nu1_func = lambda t: nu1_0 * (nu1 / nu1_0) ** (t / T)
    nu2_func = lambda t: nu2_0 * (nu2 / nu2_0) ** (t / T)
    phi = integration.two_pops(phi, xx, T, nu1_func, nu2_func, m12=m12, m21=m21,
                               gamma1=gamma1, gamma2=gamma2)
    return spectrum.from_phi(phi, ns, (xx, xx))


IM_sel.__param_names__ = ['s', 'nu1', 'nu2', 'T', 'm12', 'm21', 'gamma1', 'gamma2']


def growth3(params, ns, pts):
    """params = ((nu0_1..3), (nuF_1..3), (m12, m13, m23), (gamma1..3), T)."""
    (nu0, nuF, (m12, m13, m23), g, T) = params
    xx = numerics.default_grid(pts)
    phi = phimanip.phi_1D_to_2D(xx, phimanip.phi_1D(xx))
    phi = phimanip.phi_2D_to_3D_split_2(xx, phi)
    nus = [(lambda a, b: (lambda t: a * np.exp(np.log(b / a) * t / T)))(a, b)
           for a, b in zip(nu0, nuF)]
    phi = integration.three_pops(phi, xx, T, nus[0], nus[1], nus[2],
                                 m12=m12, m13=m13, m21=m12, m23=m23, m31=m13, m32=m23,
                                 gamma1=g[0], gamma2=g[1], gamma3=g[2])
    return spectrum.from_phi(phi, ns, (xx, xx, xx))


#: Parameters of the 3-population growth workload (nu0, nuF, m, gamma, T).
GROWTH3_DEFAULT = ((0.5, 1.0, 2.0), (5.0, 0.2, 10.0), (0.5, 1.5, 3.0), (-2.0, 0.0, 5.0), 0.15)


def four_split(params, ns, pts):
    """Four populations split successively from one (dadi/PhiManip.py:214-250,
    412-450: 1 -> 2, population 2 -> 2, 3, population 3 -> 3, 4), then
    four_pops for T with constant sizes nu1..nu4 and symmetric migration m."""
    nu1, nu2, nu3, nu4, m, T = params
    xx = numerics.default_grid(pts)
    phi = phimanip.phi_1D_to_2D(xx, phimanip.phi_1D(xx))
    phi = phimanip.phi_2D_to_3D_split_2(xx, phi)
    phi = phimanip.phi_3D_to_4D(phi, 0.0, 0.0, xx, xx, xx, xx)
    phi = integration.four_pops(phi, xx, T, nu1, nu2, nu3, nu4,
                                m12=m, m13=m, m14=m, m21=m, m23=m, m24=m,
                                m31=m, m32=m, m34=m, m41=m, m42=m, m43=m)
    return spectrum.from_phi(phi, ns, (xx, xx, xx, xx))


FOUR_DEFAULT = (1.5, 0.8, 2.0, 1.2, 0.5, 0.05)
