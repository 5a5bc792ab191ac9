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
