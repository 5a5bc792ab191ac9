"""Two-population DFE caches (dadi.DFE.Cache2D, dadi/DFE/Cache2D_mod.py:13-207)
generated by the batched GPU engine.

The reference fills its cache by calling the extrapolated demography +
selection model once per (gamma1, gamma2) pair, spread over worker
processes (`_single_process` / `_multiple_processes`, :93-207).  Here, for
the isolation-with-migration selection model (DemogSelModels.IM_sel,
dadi/DFE/DemogSelModels.py:162-197) every pair is one instance of one
persistent launch: per-instance selection coefficients in the parametric
records, per-instance initial densities (phi_1D with gamma1 on each grid,
shared by all pairs with the same gamma1), the device spectrum epilogue and
extrapolation.  Other models are evaluated pair by pair through the GPU
drop-in.  `integrate` and `merge` follow the reference's arithmetic.
"""
import numpy as np
import scipy.integrate

from . import _lib, batch, numerics, phimanip, spectrum

try:
    _trapz = np.trapezoid
except AttributeError:  # numpy < 2
    _trapz = np.trapz


class Cache2D:
    """Spectra of a 2-population demography + selection model over a grid
    of (gamma1, gamma2) pairs.  Arguments as dadi.DFE.Cache2D; cpus and gpus
    are accepted for compatibility (one GPU does the work)."""

    def __init__(self, params, ns, demo_sel_func, pts, gamma_bounds=(1e-4, 2000.),
                 gamma_pts=100, additional_gammas=[], cpus=None, gpus=0, verbose=False,
                 split_jobs=1, this_job_id=0):
        self.ns = ns
        self.pts = pts
        self.func_name = demo_sel_func.__name__
        self.params = params
        self.gammas = -np.logspace(np.log10(gamma_bounds[1]), np.log10(gamma_bounds[0]),
                                   gamma_pts)
        self.neg_gammas = self.gammas
        self.gammas = np.concatenate((self.gammas, additional_gammas))
        G = len(self.gammas)
        self.spectra = [[None] * G for _ in range(G)]
        pairs = [(ii, jj) for ii in range(G) for jj in range(G)
                 if (ii * G + jj) % split_jobs == this_job_id]
        if self.func_name == "IM_sel" and len(params) == 6:
            fs = im_sel_spectra(params, ns, pts,
                                [(self.gammas[ii], self.gammas[jj]) for ii, jj in pairs])
            for (ii, jj), f in zip(pairs, fs):
                self.spectra[ii][jj] = f
        else:
            func_ex = numerics.make_extrap_func(demo_sel_func)
            for ii, jj in pairs:
                self.spectra[ii][jj] = np.asarray(
                    func_ex(tuple(params) + (self.gammas[ii], self.gammas[jj]), ns, pts))
                if verbose:
                    print('{0},{1}: {2},{3}'.format(ii, jj, self.gammas[ii], self.gammas[jj]))
        if split_jobs == 1:
            self.spectra = np.array(self.spectra)

    def integrate(self, params, ns, sel_dist, theta, pts, exterior_int=True):
        """Spectrum integrated over a bivariate distribution of negative
        gammas (dadi/DFE/Cache2D_mod.py:209-310): trapezoid rule over the
        cached grid, plus, with exterior_int, the probability mass beyond the
        grid's strongly deleterious and neutral ends assigned to the edge
        spectra."""
        Nneg = len(self.neg_gammas)
        spectra = self.spectra[:Nneg, :Nneg]
        params = np.array(params)
        g = self.neg_gammas
        w = sel_dist(-g, -g, params)
        weighted = w[:, :, None, None] * spectra
        fs = _trapz(_trapz(weighted, g, axis=0), g, axis=0)
        if not exterior_int:
            return spectrum.Spectrum(theta * fs)
        tx = np.logspace(-2, 2, 3)
        tout = sel_dist(tx, tx, params)
        symmetric = np.allclose(tout, tout.T, atol=0, rtol=1e-12)
        gmax, gmin = -g[-1], -g[0]
        q = dict(epsabs=1e-4, epsrel=1e-3)
        w1lo, w1hi = np.zeros(Nneg), np.zeros(Nneg)
        w2lo, w2hi = np.zeros(Nneg), np.zeros(Nneg)
        for ii, gam in enumerate(-g):
            w1lo[ii] = scipy.integrate.quad(sel_dist, gmin, np.inf, args=(gam, params), **q)[0]
            w1hi[ii] = scipy.integrate.quad(sel_dist, 0, gmax, args=(gam, params), **q)[0]
            if symmetric:
                w2lo[ii], w2hi[ii] = w1lo[ii], w1hi[ii]
            else:
                def marg(g2, gam=gam):
                    return sel_dist(gam, g2, params)
                w2lo[ii] = scipy.integrate.quad(marg, gmin, np.inf, **q)[0]
                w2hi[ii] = scipy.integrate.quad(marg, 0, gmax, **q)[0]
        fs = fs + _trapz(spectra[:, 0] * w2lo[:, None, None], g, axis=0)
        fs = fs + _trapz(spectra[:, -1] * w2hi[:, None, None], g, axis=0)
        fs = fs + _trapz(spectra[0, :] * w1lo[:, None, None], g, axis=0)
        fs = fs + _trapz(spectra[-1, :] * w1hi[:, None, None], g, axis=0)
        both_neutral = scipy.integrate.dblquad(sel_dist, 0, gmax, lambda _: 0,
                                               lambda _: gmax, args=[params], **q)[0]
        fs = fs + spectra[-1, -1] * both_neutral
        wt = scipy.integrate.dblquad(sel_dist, 0, gmax, lambda _: gmin, lambda _: np.inf,
                                     args=[params], **q)[0]
        fs = fs + spectra[0, -1] * wt
        if not symmetric:
            wt = scipy.integrate.dblquad(sel_dist, gmin, np.inf, lambda _: 0,
                                         lambda _: gmax, args=[params], **q)[0]
        fs = fs + spectra[-1, 0] * wt
        return spectrum.Spectrum(theta * fs)

    @staticmethod
    def merge(caches):
        """Combine caches generated with split_jobs
        (dadi/DFE/Cache2D_mod.py:469-500)."""
        import copy
        new = copy.deepcopy(caches[0])
        for other in caches[1:]:
            for ii, row in enumerate(other.spectra):
                for jj, fs in enumerate(row):
                    if fs is None:
                        continue
                    if new.spectra[ii][jj] is not None and not np.all(new.spectra[ii][jj] == fs):
                        raise ValueError("Merged cached conflicts with current.")
                    new.spectra[ii][jj] = fs
        for ii, row in enumerate(new.spectra):
            for jj, fs in enumerate(row):
                if fs is None:
                    raise ValueError("Cache is incomplete after merging. "
                                     "First missing entry is {0},{1}.".format(ii, jj))
        new.spectra = np.array(new.spectra)
        return new


def im_sel_spectra(params, ns, pts_l, gamma_pairs, chunk=4096):
    """Extrapolated spectra of DemogSelModels.IM_sel (params s, nu1, nu2, T,
    m12, m21) for every (gamma1, gamma2) pair, on the batched engine.
    Returns a list of (n1+1, n2+1) arrays (masked corners hold the raw
    values, as the reference's cache arrays do)."""
    torch = _lib.require_cuda()
    pts_l = list(np.atleast_1d(pts_l))
    eng = batch.Batch2D(pts_l, ns)
    p = np.asarray(params, dtype=np.float64)
    pairs = np.asarray(gamma_pairs, dtype=np.float64).reshape(-1, 2)
    g1_vals, g1_idx = np.unique(pairs[:, 0], return_inverse=True)
    # initial densities: phi_1D with gamma1, split to 2-D (dadi/PhiManip.py:12-234)
    init = []
    for xx in eng.xxs:
        tab = np.stack([phimanip.phi_1D_to_2D(xx, phimanip.phi_1D(xx, gamma=g))
                        for g in g1_vals])
        init.append(_lib.to_device(torch, tab))
    out = []
    for a in range(0, len(pairs), chunk):
        sl = slice(a, min(a + chunk, len(pairs)))
        n = sl.stop - sl.start
        rec = batch.im_instances(np.repeat(p[None, :6], n, axis=0))
        for k in (0, 1):
            rec["gamma"][:, k] = batch._pf_array(_lib.PF_CONST, pairs[sl, k])
        idx = torch.from_numpy(g1_idx[sl].astype(np.int64)).cuda()
        phi0s = [t.index_select(0, idx).contiguous() for t in init]
        phis, status = eng.integrate_from(rec, phi0s)
        fs, _ = eng.spectra_ll(phis)
        st = _lib.to_host(torch, status)
        if np.any(st != 0):
            raise ValueError("integration failed for %d gamma pairs (status bits %s)"
                             % (int(np.sum(st != 0)), sorted(set(st[st != 0].tolist()))))
        out.extend(list(_lib.to_host(torch, fs)))
    return out


def biv_lognormal(xx, yy, params):
    """Bivariate lognormal density of (gamma1, gamma2) magnitudes
    (dadi/DFE/PDFs.py:41-76): params (mu, sigma, rho) with equal marginals
    or (mu1, mu2, sigma1, sigma2, rho); xx, yy scalars or vectors, the
    result over their outer grid, squeezed."""
    xx = np.atleast_1d(np.asarray(xx, dtype=float))
    yy = np.atleast_1d(np.asarray(yy, dtype=float))
    if len(params) == 3:
        mu1 = mu2 = params[0]
        s1 = s2 = params[1]
        rho = params[2]
    elif len(params) == 5:
        mu1, mu2, s1, s2, rho = params
    else:
        raise ValueError('Parameter array for bivariate lognormal must have '
                         'length 3 or 5.')
    u = (np.log(xx)[:, None] - mu1) / s1
    v = (np.log(yy)[None, :] - mu2) / s2
    q = (u * u - 2. * rho * u * v + v * v) / (1. - rho ** 2)
    norm = 2 * np.pi * s1 * s2 * np.sqrt(1. - rho ** 2) * np.outer(xx, yy)
    return np.squeeze(np.exp(-q / 2.) / norm)
