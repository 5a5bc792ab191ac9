"""ORACLE -- test infrastructure only.

Restatement of dadi's host-side integration loop (dadi/Integration.py) on top of
the C sweep restatement in oracle/sweeps.c.  The time stepping, parameter
evaluation order, validation, mutation injection and the constant-parameter
"precalc" coefficient builders follow the reference expression by expression,
so the CPU path reproduces the reference bit for bit on the same inputs.
"""
import numpy as np

from . import clib

#: Module-level settings read at call time, as dadi/Integration.py:25,39,42-44.
use_delj_trick = False
timescale_factor = 1e-3
use_old_timestep = False
old_timescale_factor = 0.1


def ensure_1arg_func(var):
    """Scalar -> constant function returning float64 (dadi/Misc.py:45-68)."""
    if np.isscalar(var):
        f0 = lambda t: var
    else:
        f0 = var
    f = lambda t: np.float64(f0(t))
    if not callable(f0):
        raise ValueError('Argument is not a constant or a function.')
    f(0.0)
    return f


def compute_dt(dx, nu, ms, gamma, h):
    """Timestep from the current parameters (dadi/Integration.py:147-176)."""
    if use_old_timestep:
        return old_timescale_factor * dx[0]
    maxVM = max(0.25 / nu, sum(ms),
                abs(gamma) * 2 * max(np.abs(h + (1 - 2 * h) * 0.5) * 0.5 * (1 - 0.5),
                                     np.abs(h + (1 - 2 * h) * 0.25) * 0.25 * (1 - 0.25)))
    if maxVM > 0:
        dt = timescale_factor / maxVM
    else:
        dt = np.inf
    if dt == 0:
        raise ValueError('Timestep is zero.')
    return dt


def inject_mutations(phi, dt, xx, theta0, active):
    """Add new-mutation mass at the unit corners
    (dadi/Integration.py:70-122); active[k] is False for frozen/nomut pops."""
    P = phi.ndim
    for k in range(P):
        if not active[k]:
            continue
        denom = xx[2] - xx[0]
        for j in range(P):
            if j != k:
                denom = denom * xx[1]
        idx = [0] * P
        idx[k] = 1
        phi[tuple(idx)] += dt / xx[1] * theta0 / 2 * 2 ** P / denom
    return phi


def _mig_lists(P, mig):
    """mig[k][j] = rate into k from j; returns per-pop ordered lists."""
    return [[mig[k][j] for j in range(P) if j != k] for k in range(P)]


def integrate_temporal(phi, xx, T, initial_t, nu_f, mig_f, gamma_f, h_f, theta0_f,
                       frozen, nomut=None, beta_f=None):
    """Generic P-population temporal loop: dadi/Integration.py:178-258 (P=1),
    :260-387 (P=2), :389-554 (P=3), :556-727 (P=4).  nu_f/gamma_f/h_f are lists
    of callables, mig_f[k][j] callables (rate into k from j), phi is modified
    in place and returned."""
    P = phi.ndim
    if nomut is None:
        nomut = [False] * P
    current_t = initial_t
    nu = [f(current_t) for f in nu_f]
    gamma = [f(current_t) for f in gamma_f]
    h = [f(current_t) for f in h_f]
    mig = [[mig_f[k][j](current_t) if j != k else 0.0 for j in range(P)] for k in range(P)]
    beta = beta_f(current_t) if beta_f is not None else 1.0
    dx = np.diff(xx)
    while current_t < T:
        ml = _mig_lists(P, mig) if P > 1 else [[0]]
        dt = min(compute_dt(dx, nu[k], ml[k], gamma[k], h[k]) for k in range(P))
        this_dt = min(dt, T - current_t)
        next_t = current_t + this_dt
        nu = [f(next_t) for f in nu_f]
        gamma = [f(next_t) for f in gamma_f]
        h = [f(next_t) for f in h_f]
        mig = [[mig_f[k][j](next_t) if j != k else 0.0 for j in range(P)]
               for k in range(P)]
        if beta_f is not None:
            beta = beta_f(next_t)
        theta0 = theta0_f(next_t)
        flat_m = [mig[k][j] for k in range(P) for j in range(P) if j != k]
        if np.any(np.less([T] + nu + flat_m + [theta0], 0)):
            raise ValueError('A time, population size, migration rate, or '
                             'theta0 is < 0. Has the model been mis-specified?')
        if np.any(np.equal(nu, 0)):
            raise ValueError('A population size is 0. Has the model been '
                             'mis-specified?')
        active = [not frozen[k] and not nomut[k] for k in range(P)]
        inject_mutations(phi, this_dt, xx, theta0, active)
        for k in range(P):
            if not frozen[k]:
                clib.sweep(phi, xx, k, nu[k], mig[k], gamma[k], h[k], this_dt,
                           beta=beta, use_delj_trick=use_delj_trick)
        current_t = next_t
    return phi


def _Vfunc(x, nu, beta=1):
    return 1. / nu * x * (1 - x) * (beta + 1.) ** 2 / (4. * beta)


def _Msel(x, gamma, h):
    return gamma * 2 * (h + (1 - 2 * h) * x) * x * (1 - x)


def _Mfull(xk, others, ms, gamma, h):
    """Python M (dadi/Integration.py:951-956) with others in increasing axis order."""
    if not others:
        return _Msel(xk, gamma, h)
    acc = ms[0] * (others[0] - xk)
    for o, m in zip(others[1:], ms[1:]):
        acc = acc + m * (o - xk)
    return acc + _Msel(xk, gamma, h)


def _compute_dfactor(dx):
    """dadi/Integration.py:958-971."""
    dfactor = np.zeros(len(dx) + 1)
    dfactor[1:-1] = 2 / (dx[:-1] + dx[1:])
    dfactor[0] = 2 / dx[0]
    dfactor[-1] = 2 / dx[-1]
    return dfactor


def _compute_delj(dx, MInt, VInt):
    """dadi/Integration.py:973-984 (arrays already broadcast by the caller)."""
    if use_delj_trick:
        wj = 2 * MInt * dx
        epsj = np.exp(wj / VInt)
        delj = (-epsj * wj + epsj * VInt - VInt) / (wj - epsj * wj)
        delj = np.where(np.isnan(delj), 0.5, delj)
        delj = np.where(np.isinf(delj), 0.5, delj)
        return delj
    return 0.5


def precalc_coefficients(xx, P, axis, nu, ms, gamma, h):
    """Full a, b, c arrays (b without 1/dt) of one axis for constant parameters
    (dadi/Integration.py:1057-1095 for P=2, :1145-1222 for P=3).  ms are the
    migration rates into this population, others in increasing axis order."""
    L = len(xx)
    sh = lambda k: tuple(slice(None) if j == k else None for j in range(P))
    others_ax = [j for j in range(P) if j != axis]
    xInt = (xx[:-1] + xx[1:]) / 2
    V = _Vfunc(xx, nu)
    VInt = _Vfunc(xInt, nu)
    M = _Mfull(xx[sh(axis)], [xx[sh(j)] for j in others_ax], ms, gamma, h)
    MInt = _Mfull(xInt[sh(axis)], [xx[sh(j)] for j in others_ax], ms, gamma, h)
    dx = np.diff(xx)
    dfact = _compute_dfactor(dx)
    delj = _compute_delj(dx[sh(axis)], MInt, VInt[sh(axis)])
    a, b, c = [np.zeros((L,) * P) for _ in range(3)]

    def sl(lo, hi):
        return tuple(slice(lo, hi) if j == axis else slice(None) for j in range(P))
    up = lambda v: v[sh(axis)]
    a[sl(1, None)] += up(dfact[1:]) * (-MInt * delj - up(V[:-1]) / (2 * up(dx)))
    c[sl(None, -1)] += up(dfact[:-1]) * (MInt * (1 - delj) - up(V[1:]) / (2 * up(dx)))
    b[sl(None, -1)] += up(dfact[:-1]) * (MInt * delj + up(V[:-1]) / (2 * up(dx)))
    b[sl(1, None)] += up(dfact[1:]) * (-MInt * (1 - delj) + up(V[1:]) / (2 * up(dx)))
    z, e = (0,) * P, (-1,) * P
    if M[z] <= 0:
        b[z] += (0.5 / nu - M[z]) * 2 / dx[0]
    if M[e] >= 0:
        b[e] += -(-0.5 / nu - M[e]) * 2 / dx[-1]
    return a, b, c


def integrate_const(phi, xx, T, initial_t, nu, mig, gamma, h, theta0, frozen, nomut=None):
    """Constant-parameter precalc path for P=2,3 (dadi/Integration.py:1037-1118,
    1120-1242); mig[k][j] = rate into k from j.  phi modified in place."""
    P = phi.ndim
    if nomut is None:
        nomut = [False] * P
    flat_m = [mig[k][j] for k in range(P) for j in range(P) if j != k]
    if np.any(np.less([T] + list(nu) + flat_m + [theta0], 0)):
        raise ValueError('A time, population size, migration rate, or theta0 '
                         'is < 0. Has the model been mis-specified?')
    if np.any(np.equal(nu, 0)):
        raise ValueError('A population size is 0. Has the model been '
                         'mis-specified?')
    ml = _mig_lists(P, mig)
    coefs = [precalc_coefficients(xx, P, k, nu[k], ml[k], gamma[k], h[k]) for k in range(P)]
    dx = np.diff(xx)
    dt = min(compute_dt(dx, nu[k], ml[k], gamma[k], h[k]) for k in range(P))
    current_t = initial_t
    active = [not frozen[k] and not nomut[k] for k in range(P)]
    while current_t < T:
        this_dt = min(dt, T - current_t)
        inject_mutations(phi, this_dt, xx, theta0, active)
        for k in range(P):
            if not frozen[k]:
                clib.sweep_precalc(phi, k, *coefs[k], this_dt)
        current_t += this_dt
    return phi


def one_pop_const(phi, xx, T, nu=1, gamma=0, h=0.5, theta0=1, initial_t=0, beta=1):
    """dadi/Integration.py:986-1035."""
    if np.any(np.less([T, nu, theta0], 0)):
        raise ValueError('A time, population size, migration rate, or theta0 '
                         'is < 0. Has the model been mis-specified?')
    if np.any(np.equal([nu], 0)):
        raise ValueError('A population size is 0. Has the model been '
                         'mis-specified?')
    M = _Msel(xx, gamma, h)
    MInt = _Msel((xx[:-1] + xx[1:]) / 2, gamma, h)
    V = _Vfunc(xx, nu, beta=beta)
    VInt = _Vfunc((xx[:-1] + xx[1:]) / 2, nu, beta=beta)
    dx = np.diff(xx)
    dfactor = _compute_dfactor(dx)
    delj = _compute_delj(dx, MInt, VInt)
    a = np.zeros(phi.shape)
    a[1:] += dfactor[1:] * (-MInt * delj - V[:-1] / (2 * dx))
    c = np.zeros(phi.shape)
    c[:-1] += -dfactor[:-1] * (-MInt * (1 - delj) + V[1:] / (2 * dx))
    b = np.zeros(phi.shape)
    b[:-1] += -dfactor[:-1] * (-MInt * delj - V[:-1] / (2 * dx))
    b[1:] += dfactor[1:] * (-MInt * (1 - delj) + V[1:] / (2 * dx))
    if M[0] <= 0:
        b[0] += (0.5 / nu - M[0]) * 2 / dx[0]
    if M[-1] >= 0:
        b[-1] += -(-0.5 / nu - M[-1]) * 2 / dx[-1]
    dt = compute_dt(dx, nu, [0], gamma, h)
    current_t = initial_t
    while current_t < T:
        this_dt = min(dt, T - current_t)
        inject_mutations(phi, this_dt, xx, theta0, [True])
        r = phi / this_dt
        phi = clib.tridiag(a, b + 1 / this_dt, c, r)
        current_t += this_dt
    return phi


# ---- reference-signature wrappers (dadi/Integration.py:178, 260, 389, 556) ----

def _all_scalar(vals):
    return np.all([np.isscalar(v) for v in vals])


def one_pop(phi, xx, T, nu=1, gamma=0, h=0.5, theta0=1.0, initial_t=0, frozen=False, beta=1):
    phi = phi.copy()
    if frozen or T - initial_t == 0:
        return phi
    if T - initial_t < 0:
        raise ValueError('Final integration time T is less than intial_time.')
    if _all_scalar((nu, gamma, h, theta0, beta)):
        return one_pop_const(phi, xx, T, nu, gamma, h, theta0, initial_t, beta)
    f = ensure_1arg_func
    return integrate_temporal(phi, xx, T, initial_t, [f(nu)], [[None]], [f(gamma)],
                              [f(h)], f(theta0), [False], beta_f=f(beta))


def two_pops(phi, xx, T, nu1=1, nu2=1, m12=0, m21=0, gamma1=0, gamma2=0,
             h1=0.5, h2=0.5, theta0=1, initial_t=0, frozen1=False, frozen2=False,
             nomut1=False, nomut2=False):
    phi = phi.copy()
    if T - initial_t == 0:
        return phi
    if T - initial_t < 0:
        raise ValueError('Final integration time T is less than intial_time.')
    if (frozen1 or frozen2) and (m12 != 0 or m21 != 0):
        raise ValueError('Population cannot be frozen and have non-zero '
                         'migration to or from it.')
    vals = [nu1, nu2, m12, m21, gamma1, gamma2, h1, h2, theta0]
    if _all_scalar(vals):
        return integrate_const(phi, xx, T, initial_t, [nu1, nu2], [[0, m12], [m21, 0]],
                               [gamma1, gamma2], [h1, h2], theta0, [frozen1, frozen2],
                               [nomut1, nomut2])
    f = ensure_1arg_func
    return integrate_temporal(phi, xx, T, initial_t, [f(nu1), f(nu2)],
                              [[None, f(m12)], [f(m21), None]], [f(gamma1), f(gamma2)],
                              [f(h1), f(h2)], f(theta0), [frozen1, frozen2], [nomut1, nomut2])


def three_pops(phi, xx, T, nu1=1, nu2=1, nu3=1, m12=0, m13=0, m21=0, m23=0, m31=0, m32=0,
               gamma1=0, gamma2=0, gamma3=0, h1=0.5, h2=0.5, h3=0.5, theta0=1, initial_t=0,
               frozen1=False, frozen2=False, frozen3=False):
    phi = phi.copy()
    if T - initial_t == 0:
        return phi
    if T - initial_t < 0:
        raise ValueError('Final integration time T is less than intial_time.')
    if (frozen1 and (m12 != 0 or m21 != 0 or m13 != 0 or m31 != 0)) \
            or (frozen2 and (m12 != 0 or m21 != 0 or m23 != 0 or m32 != 0)) \
            or (frozen3 and (m13 != 0 or m31 != 0 or m23 != 0 or m32 != 0)):
        raise ValueError('Population cannot be frozen and have non-zero '
                         'migration to or from it.')
    vals = [nu1, nu2, nu3, m12, m13, m21, m23, m31, m32, gamma1, gamma2, gamma3,
            h1, h2, h3, theta0]
    mig = [[0, m12, m13], [m21, 0, m23], [m31, m32, 0]]
    if _all_scalar(vals):
        return integrate_const(phi, xx, T, initial_t, [nu1, nu2, nu3], mig,
                               [gamma1, gamma2, gamma3], [h1, h2, h3], theta0,
                               [frozen1, frozen2, frozen3])
    f = ensure_1arg_func
    mig_f = [[None if j == k else f(mig[k][j]) for j in range(3)] for k in range(3)]
    return integrate_temporal(phi, xx, T, initial_t, [f(nu1), f(nu2), f(nu3)], mig_f,
                              [f(gamma1), f(gamma2), f(gamma3)], [f(h1), f(h2), f(h3)],
                              f(theta0), [frozen1, frozen2, frozen3])


def five_pops(phi, xx, T, nu1=1, nu2=1, nu3=1, nu4=1, nu5=1,
              m12=0, m13=0, m14=0, m15=0, m21=0, m23=0, m24=0, m25=0,
              m31=0, m32=0, m34=0, m35=0, m41=0, m42=0, m43=0, m45=0,
              m51=0, m52=0, m53=0, m54=0,
              gamma1=0, gamma2=0, gamma3=0, gamma4=0, gamma5=0,
              h1=0.5, h2=0.5, h3=0.5, h4=0.5, h5=0.5,
              theta0=1, initial_t=0, frozen1=False, frozen2=False, frozen3=False,
              frozen4=False, frozen5=False):
    """Like dadi/Integration.py:729-937 this integrates phi in place (no copy)."""
    if T - initial_t == 0:
        return phi
    if T - initial_t < 0:
        raise ValueError('Final integration time T is less than intial_time.')
    mig = [[0, m12, m13, m14, m15], [m21, 0, m23, m24, m25], [m31, m32, 0, m34, m35],
           [m41, m42, m43, 0, m45], [m51, m52, m53, m54, 0]]
    fr = [frozen1, frozen2, frozen3, frozen4, frozen5]
    for k in range(5):
        if fr[k] and any(mig[k][j] != 0 or mig[j][k] != 0 for j in range(5) if j != k):
            raise ValueError('Population cannot be frozen and have non-zero '
                             'migration to or from it.')
    f = ensure_1arg_func
    mig_f = [[None if j == k else f(mig[k][j]) for j in range(5)] for k in range(5)]
    return integrate_temporal(phi, xx, T, initial_t,
                              [f(v) for v in (nu1, nu2, nu3, nu4, nu5)], mig_f,
                              [f(v) for v in (gamma1, gamma2, gamma3, gamma4, gamma5)],
                              [f(v) for v in (h1, h2, h3, h4, h5)], f(theta0), fr)


def four_pops(phi, xx, T, nu1=1, nu2=1, nu3=1, nu4=1,
              m12=0, m13=0, m14=0, m21=0, m23=0, m24=0,
              m31=0, m32=0, m34=0, m41=0, m42=0, m43=0,
              gamma1=0, gamma2=0, gamma3=0, gamma4=0, h1=0.5, h2=0.5, h3=0.5, h4=0.5,
              theta0=1, initial_t=0, frozen1=False, frozen2=False, frozen3=False,
              frozen4=False):
    """Like dadi/Integration.py:556-727 this integrates phi in place (no copy)."""
    if T - initial_t == 0:
        return phi
    if T - initial_t < 0:
        raise ValueError('Final integration time T is less than intial_time.')
    mig = [[0, m12, m13, m14], [m21, 0, m23, m24], [m31, m32, 0, m34], [m41, m42, m43, 0]]
    fr = [frozen1, frozen2, frozen3, frozen4]
    for k in range(4):
        if fr[k] and any(mig[k][j] != 0 or mig[j][k] != 0 for j in range(4) if j != k):
            raise ValueError('Population cannot be frozen and have non-zero '
                             'migration to or from it.')
    f = ensure_1arg_func
    mig_f = [[None if j == k else f(mig[k][j]) for j in range(4)] for k in range(4)]
    return integrate_temporal(phi, xx, T, initial_t, [f(v) for v in (nu1, nu2, nu3, nu4)],
                              mig_f, [f(v) for v in (gamma1, gamma2, gamma3, gamma4)],
                              [f(v) for v in (h1, h2, h3, h4)], f(theta0), fr)
