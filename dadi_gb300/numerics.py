"""Grid and Richardson extrapolation (dadi/Numerics.py:215-233, 334-475, 644-669)."""
import functools
import logging

import numpy as np

logger = logging.getLogger("dadi_gb300.numerics")


def exponential_grid(pts, crwd=8.):
    """Grid crowded toward 0 and 1 (dadi/Numerics.py:215-231)."""
    unif = np.linspace(-1, 1, pts)
    grid = 1. / (1. + np.exp(-crwd * unif))
    return (grid - grid[0]) / (grid[-1] - grid[0])


default_grid = exponential_grid


def linear_extrap(ys, xs):
    """Two-point extrapolation to x = 0 (dadi/Numerics.py:644-654)."""
    y1, y2 = ys
    x1, x2 = xs
    return (x2 * y1 - x1 * y2) / (x2 - x1)


def quadratic_extrap(ys, xs):
    """Three-point extrapolation to x = 0 (dadi/Numerics.py:657-669)."""
    y1, y2, y3 = ys
    x1, x2, x3 = xs
    return x2 * x3 / ((x1 - x2) * (x1 - x3)) * y1 + x1 * x3 / ((x2 - x1) * (x2 - x3)) * y2 \
        + x1 * x2 / ((x3 - x1) * (x3 - x2)) * y3


def extrapolate(result_l, x_l, fail_mag=10, extrap_log=False):
    """Extrapolate a list of results (1-3 grids) to infinitely many grid points,
    replacing entries more than fail_mag orders of magnitude away from the
    smallest-x result by that result (dadi/Numerics.py:418-464)."""
    if extrap_log:
        result_l = [np.log(r) for r in result_l]
    if len(result_l) == 1:
        ex = result_l[0]
    elif len(result_l) == 2:
        ex = linear_extrap(result_l, x_l)
    elif len(result_l) == 3:
        ex = quadratic_extrap(result_l, x_l)
    else:
        raise ValueError('Number of calculations to use for extrapolation must be between 1 '
                         'and 3 (the reference names cubic and higher orders without '
                         'defining them)')
    if extrap_log:
        ex = np.exp(ex)
    if len(result_l) > 1:
        best = result_l[int(np.argmin(x_l))]
        if extrap_log:
            best = np.exp(best)
        with np.errstate(all="ignore"):
            failed = abs(np.log10(ex / best)) > fail_mag
        if np.any(failed):
            logger.warning('Extrapolation may have failed. Check resulting frequency '
                           'spectrum for unexpected results.')
        ex[failed] = best[failed]
    return ex


def _map_grids(fn, pts_l):
    """fn over the grid sizes.  With a GPU, the grids run concurrently, each
    on its own thread and CUDA stream: one integration of a few grids leaves
    most SMs idle (a 3-D sweep at L = 70 is 77 CTAs), and the integrations of
    different grids are independent.  The results are the same as one at a
    time (to rounding where the drop-in would pick the partitioned solve
    for a lone 3-5 population grid)."""
    if len(pts_l) < 2:
        return [fn(p) for p in pts_l]
    try:
        import torch
        gpu = torch.cuda.is_available()
    except ImportError:
        gpu = False
    if not gpu:
        return [fn(p) for p in pts_l]
    from concurrent.futures import ThreadPoolExecutor
    from . import integration
    dev = torch.cuda.current_device()

    def one(p):
        # Thomas for 3-5 populations: the grids' sweeps together fill the pipes
        integration.local.sharing_gpu = True
        try:
            with torch.cuda.device(dev), torch.cuda.stream(torch.cuda.Stream()):
                return fn(p)
        finally:
            integration.local.sharing_gpu = False
    with ThreadPoolExecutor(max_workers=len(pts_l)) as ex:
        return list(ex.map(one, pts_l))


def make_extrap_func(func, extrap_x_l=None, extrap_log=False, fail_mag=10):
    """Version of func(params, ns, pts) taking a list of pts and returning the
    extrapolated result (dadi/Numerics.py:334-475).  x values come from the
    results' extrap_x attribute (xx[1]) unless extrap_x_l is given."""
    def extrap_func(*args, **kwargs):
        if 'pts' not in kwargs:
            other_args, pts_l = args[:-1], args[-1]
        else:
            other_args = args
            pts_l = kwargs.pop('pts')
        no_extrap = kwargs.pop('no_extrap', False)
        if np.isscalar(pts_l):
            pts_l = [pts_l]
        partial = functools.partial(func, *other_args, **kwargs)
        result_l = _map_grids(partial, pts_l)
        if no_extrap:
            return result_l
        if extrap_x_l is None:
            try:
                x_l = [r.extrap_x for r in result_l]
            except AttributeError:
                raise ValueError("Extrapolation function error: No explicit extrapolation x_l "
                                 "provided, and results do not have 'extrap_x' attributes.")
        else:
            x_l = extrap_x_l
        ex = extrapolate(result_l, x_l, fail_mag=fail_mag, extrap_log=extrap_log)
        try:
            ex.pop_ids = result_l[0].pop_ids
        except AttributeError:
            pass
        return ex
    extrap_func.__name__ = func.__name__
    extrap_func.__doc__ = func.__doc__
    return extrap_func


def make_extrap_log_func(func, extrap_x_l=None):
    """dadi/Numerics.py:477-501."""
    return make_extrap_func(func, extrap_x_l=extrap_x_l, extrap_log=True)
