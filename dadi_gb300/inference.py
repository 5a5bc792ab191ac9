"""Poisson and multinomial composite likelihoods (dadi/Inference.py:466-575,
668-685) over entries masked in neither model nor data."""
import numpy as np
from scipy.special import gammaln


def _mask_of(a):
    m = np.ma.getmaskarray(a)
    return m


def ll_per_bin(model, data):
    """-model + data*log(model) - lgamma(data+1); masked where either input is
    masked or model <= 0 (numpy.ma.log's domain, dadi/Inference.py:505-509)."""
    mask = _mask_of(model) | _mask_of(data)
    m = np.ma.getdata(model).astype(np.float64)
    d = np.ma.getdata(data).astype(np.float64)
    with np.errstate(all="ignore"):
        res = -m + d * np.log(m) - gammaln(d + 1.)
    return np.ma.MaskedArray(res, mask=mask | ~(m > 0))


def ll(model, data):
    """dadi/Inference.py:466-480."""
    return ll_per_bin(model, data).sum()


def optimal_sfs_scaling(model, data):
    """dadi/Inference.py:668-685."""
    mask = _mask_of(model) | _mask_of(data)
    return np.ma.getdata(data)[~mask].sum() / np.ma.getdata(model)[~mask].sum()


def ll_multinom(model, data):
    """dadi/Inference.py:559-575."""
    theta = optimal_sfs_scaling(model, data)
    return ll(theta * model, data)


def Anscombe_Poisson_residual(model, data, mask=None):
    """Anscombe residuals of Poisson data given the model
    (dadi/Inference.py:612-659): 1.5 (d' - m') / model^(1/6) with
    x' = x^(2/3) - x^(-1/3) / 9, negated (positive where the model is high);
    with `mask`, entries where both are <= mask or the data are 0 are masked.
    (Folded spectra are not handled here.)"""
    d = np.ma.asarray(data, dtype=np.float64)
    m = np.ma.asarray(model, dtype=np.float64)
    dt = d ** (2. / 3) - np.ma.power(d, -1. / 3) / 9
    mt = m ** (2. / 3) - np.ma.power(m, -1. / 3) / 9
    resid = 1.5 * (dt - mt) / m ** (1. / 6)
    if mask is not None:
        tomask = np.logical_or(np.logical_and(m <= mask, d <= mask), d == 0)
        resid = np.ma.masked_where(tomask, resid)
    return -resid


# ------------------------------------------------------------ optimisation

def _project_down(p, fixed):
    if fixed is None:
        return np.asarray(p, dtype=float)
    return np.array([v for v, f in zip(p, fixed) if f is None], dtype=float)


def _project_up(p, fixed):
    if fixed is None:
        return np.asarray(p, dtype=float)
    out, it = [], iter(p)
    for f in fixed:
        out.append(next(it) if f is None else f)
    return np.array(out, dtype=float)


def _adjoint_engine(model_func, data, pts, func_args, func_kwargs):
    """A batched engine with a discrete adjoint for model_func, or None.
    Demographics2D.IM (dadi/Demographics2D.py:268-309; ours or dadi's) on
    2-D data qualifies."""
    if model_func.__name__ != "IM" or func_args or func_kwargs:
        return None
    ns = np.ma.getdata(data).shape
    if len(ns) != 2:
        return None
    from . import batch
    return batch.Batch2D(list(np.atleast_1d(pts)), (ns[0] - 1, ns[1] - 1))


def optimize_log_lbfgsb(p0, data, model_func, pts, lower_bound=None, upper_bound=None,
                        verbose=0, flush_delay=0.5, epsilon=1e-3, pgtol=1e-5, multinom=True,
                        maxiter=1e5, full_output=False, func_args=[], func_kwargs={},
                        fixed_params=None, ll_scale=1, output_file=None, gradient="auto"):
    """dadi.Inference.optimize_log_lbfgsb (dadi/Inference.py:337-455): L-BFGS-B
    over log(params), same arguments and return values.  The reference
    estimates the gradient by finite differences (step `epsilon`, one model
    evaluation per parameter per iteration); here, for models with a
    discrete adjoint on the GPU (the IM model), gradient="auto" or
    "adjoint" uses it: one forward with checkpoints and one adjoint per
    iteration give the exact gradient of the (multinomial or Poisson)
    log-likelihood.  gradient="fd" keeps the reference's finite differences
    over the GPU model."""
    import scipy.optimize
    data_arr = np.ma.getdata(data).astype(np.float64)
    dmask = np.ma.getmaskarray(data)
    eng = None if gradient == "fd" else _adjoint_engine(model_func, data, pts, func_args,
                                                        func_kwargs)
    if gradient == "adjoint" and eng is None:
        raise ValueError("no adjoint engine for %s" % model_func.__name__)
    out = open(output_file, 'w') if output_file else None
    counter = [0]

    def bounds_log(b):
        if b is None:
            return [None] * len(p0)
        with np.errstate(all="ignore"):
            lb = np.log(np.array([np.nan if v is None else v for v in b], dtype=float))
        lb = [None if np.isnan(v) else float(v) for v in lb]
        return [v for v, f in zip(lb, fixed_params or [None] * len(lb)) if f is None]

    bounds = list(zip(bounds_log(lower_bound), bounds_log(upper_bound)))
    x0 = np.log(_project_down(p0, fixed_params))

    def report(p, ll):
        counter[0] += 1
        if verbose > 0 and counter[0] % verbose == 0:
            line = '%-8i, %-12g, %s' % (counter[0], ll, ', '.join('%- 12g' % v for v in p))
            print(line, file=out) if out else print(line)

    if eng is not None:
        torch = eng.torch
        d_data = torch.from_numpy(np.where(dmask, 0.0, data_arr)).cuda()
        free = np.array([f is None for f in (fixed_params or [None] * len(p0))])

        def f_and_g(x):
            p = _project_up(np.exp(x), fixed_params)
            ll, g, st = eng.loglik_and_grad(p[None, :], d_data, scale=1.0, mask=dmask,
                                           multinom=multinom)
            ll = float(ll.cpu().numpy()[0])
            g = g.cpu().numpy()[0]
            report(p, ll)
            if int(st.cpu().numpy()[0]) != 0 or not np.isfinite(ll):
                return 1e10 / ll_scale, np.zeros_like(x)
            return -ll / ll_scale, -(p * g)[free] / ll_scale
        res = scipy.optimize.minimize(f_and_g, x0, jac=True, method="L-BFGS-B",
                                      bounds=bounds,
                                      options=dict(gtol=pgtol, maxfun=int(maxiter)))
    else:
        ns = tuple(s - 1 for s in data_arr.shape)

        def f(x):
            p = _project_up(np.exp(x), fixed_params)
            kw = dict(func_kwargs)
            kw['pts'] = pts
            sfs = model_func(p, ns, *func_args, **kw)
            res = ll_multinom(sfs, data) if multinom else ll(sfs, data)
            res = float(res)
            report(p, res)
            if not np.isfinite(res):
                return 1e10 / ll_scale
            return -res / ll_scale
        res = scipy.optimize.minimize(f, x0, jac="2-point", method="L-BFGS-B",
                                      bounds=bounds,
                                      options=dict(gtol=pgtol, maxfun=int(maxiter),
                                                   eps=epsilon))
    if out:
        out.close()
    xopt = _project_up(np.exp(res.x), fixed_params)
    if not full_output:
        return xopt
    # the information dictionary of scipy.optimize.fmin_l_bfgs_b
    info = {"grad": res.jac, "task": res.message, "funcalls": res.nfev, "nit": res.nit,
            "warnflag": res.status, "model_evaluations": counter[0]}
    return xopt, float(res.fun), info
