"""Parity cases shared by the golden-vector generator (make_golden.py) and the
tests.  Each case is a plain description (grid, seeded initial density, the
integrator arguments); time-dependent parameters are named entries of TFUNCS
so both sides build identical callables.

The cases mirror the reference's own integrator tests: arbitrary linspace grids
and non-physical random densities (dadi tests/test_CUDA.py:23-255), frozen and
nomut populations, initial_t != 0, time-dependent theta0, gamma and h, plus the
default grid.
"""
import numpy as np

#: Time-dependent parameter forms used by the cases (t -> value).
TFUNCS = {
    "lin_nu": lambda t: 0.1 + 10 * t,          # tests/test_CUDA.py:42
    "lin_m": lambda t: 3 - 20 * t,             # tests/test_CUDA.py:43
    "lin_nu3": lambda t: 0.1 + 4 * t,          # tests/test_CUDA.py:118
    "lin_m23": lambda t: 9 - 10 * t,           # tests/test_CUDA.py:120
    "ident": lambda t: t,                       # tests/test_CUDA.py:122
    "h_t": lambda t: 0.2 + t,
    "theta_t": lambda t: 1 + 2 * t,            # tests/test_CUDA.py:190
    "exp_grow": lambda t: 0.5 * (4.0 / 0.5) ** (t / 0.3),
}


def resolve(v):
    """Map a case argument to a value or a callable."""
    if isinstance(v, str):
        return TFUNCS[v]
    return v


def grid(kind, pts):
    if kind == "lin":
        return np.linspace(0, 1, pts)
    unif = np.linspace(-1, 1, pts)
    g = 1. / (1. + np.exp(-8. * unif))
    return (g - g[0]) / (g[-1] - g[0])


def initial_phi(seed, shape):
    return np.random.default_rng(seed).uniform(size=shape)


# two_pops(phi, xx, T, nu1, nu2, m12, m21, gamma1, gamma2, h1, h2, theta0,
#          initial_t, frozen1, frozen2, nomut1, nomut2)
TWO_POPS = [
    dict(name="2d_const_lin20", grid="lin", pts=20, seed=1,
         args=[0.1, 0.1, 2, 0.3, 0.5, -0.2, 2, 0.1, 0.9, 2]),
    dict(name="2d_temporal_lin20", grid="lin", pts=20, seed=2,
         args=[0.1, "lin_nu", 2, 0.3, "lin_m", -0.2, 2, 0.1, 0.9, 2]),
    dict(name="2d_temporal_default31", grid="default", pts=31, seed=3,
         args=[0.25, "exp_grow", 1.5, 0.7, 1.1, 0.5, -1.0, 0.5, "h_t", "theta_t"],
         kw=dict(initial_t=0.05)),
    dict(name="2d_frozen1_nomut2", grid="default", pts=24, seed=4,
         args=[0.2, 1.0, 2.0, 0, 0, 0.5, 0.5, 0.5, 0.5, 1.0],
         kw=dict(frozen1=True, nomut2=True)),
    dict(name="2d_nomut1_temporal", grid="default", pts=26, seed=5,
         args=[0.15, "exp_grow", 0.4, 1.0, 0.2, 0, 3.0, 0.5, 0.5, 1.0],
         kw=dict(nomut1=True)),
]

# three_pops(phi, xx, T, nu1, nu2, nu3, m12, m13, m21, m23, m31, m32,
#            gamma1, gamma2, gamma3, h1, h2, h3, theta0, initial_t, frozen1..3)
THREE_POPS = [
    dict(name="3d_const_lin13", grid="lin", pts=13, seed=213,
         args=[0.2, 2, 1, 0.1, 0.1, 3, 10, 0, 0.3, 0.1, -1, 2.0, 0.1, 0.2, 0.3, 0.9,
               10.2, 0.1]),
    dict(name="3d_temporal_lin17", grid="lin", pts=17, seed=17,
         args=[0.2, "lin_nu3", 1, 0.1, 0.1, 3, 10, "lin_m23", 0.3, 0.1, -1, 2.0,
               "ident", 0.2, 0.3, "h_t", 10.2, 0.1]),
    dict(name="3d_temporal_default15", grid="default", pts=15, seed=15,
         args=[0.1, "exp_grow", 1, 2, 0.5, 0.5, 1.5, 1.5, 3.0, 3.0, -2, 0, 5,
               0.5, 0.5, 0.5, "theta_t", 0.0]),
]
# all eight frozen combinations with zero migration (tests/test_CUDA.py:88-108)
for _f in range(8):
    THREE_POPS.append(dict(
        name="3d_frozen%d" % _f, grid="lin", pts=11, seed=300 + _f,
        args=[0.2, 2, 1, 0.1, 0, 0, 0, 0, 0, 0, -1, 2.0, 0.1, 0.2, 0.3, 0.9, 10.2, 0.1,
              bool(_f & 1), bool(_f & 2), bool(_f & 4)]))
    THREE_POPS.append(dict(
        name="3d_frozen%d_temporal" % _f, grid="lin", pts=11, seed=310 + _f,
        args=[0.2, "lin_nu3", 1, 0.1, 0, 0, 0, 0, 0, 0, -1, 2.0, "ident", 0.2, 0.3, 0.9,
              10.2, 0.1, bool(_f & 1), bool(_f & 2), bool(_f & 4)]))

# four_pops(phi, xx, T, nu1..nu4, m12, m13, m14, m21, m23, m24, m31, m32, m34,
#           m41, m42, m43, gamma1..4, h1..4, theta0, initial_t, frozen1..4)
FOUR_POPS = [
    dict(name="4d_default10", grid="default", pts=10, seed=44,
         args=[0.1, 1, 2, 0.5, 1.5, 0.5, 1, 0.2, 0.3, 0.4, 1, 0.6, 0.7, 0.2, 0.9,
               1, 0.1, -1, 2, 0.5, 0.3, 0.4, 0.5, 0.6, 0.7, "theta_t", 0.02]),
    dict(name="4d_temporal_lin9", grid="lin", pts=9, seed=45,
         args=[0.1, "lin_nu3", 2, 0.5, 1.5, 0.5, 1, 0.2, "lin_m23", 0.4, 1, 0.6, 0.7,
               0.2, 0.9, 1, 0.1, -1, 2, 0.5, 0.3, 0.4, 0.5, 0.6, 0.7, 1.0, 0.0]),
]
for _f in range(16):
    FOUR_POPS.append(dict(
        name="4d_frozen%d" % _f, grid="default", pts=8, seed=400 + _f,
        args=[0.1, 1, 2, 0.5, 1.5] + [0] * 12 + [0.1, -1, 2, 0.5, 0.3, 0.4, 0.5, 0.6,
                                                  "theta_t", 0.0] +
             [bool(_f & 1), bool(_f & 2), bool(_f & 4), bool(_f & 8)]))

# five_pops(phi, xx, T, nu1..nu5, m12, m13, m14, m15, m21, m23, m24, m25, m31, m32,
#           m34, m35, m41, m42, m43, m45, m51, m52, m53, m54, gamma1..5, h1..5,
#           theta0, initial_t, frozen1..5)
FIVE_POPS = [
    dict(name="5d_default7", grid="default", pts=7, seed=55,
         args=[0.05, 1, 2, 0.5, 1.5, 0.8] + [0.3, 0.2, 0.1, 0.4, 1, 0.6, 0.2, 0.3, 0.7,
                                             0.2, 0.5, 0.1, 0.9, 1, 0.4, 0.3, 0.2, 0.6,
                                             0.5, 0.1] +
              [-1, 2, 0.5, 0, 1.5, 0.3, 0.4, 0.5, 0.6, 0.7, "theta_t", 0.01]),
    dict(name="5d_temporal_lin6", grid="lin", pts=6, seed=56,
         args=[0.05, "lin_nu3", 2, 0.5, 1.5, 0.8] + [0.3, 0.2, 0.1, 0.4, "lin_m23", 0.6, 0.2,
                                                     0.3, 0.7, 0.2, 0.5, 0.1, 0.9, 1, 0.4,
                                                     0.3, 0.2, 0.6, 0.5, 0.1] +
              [-1, 2, "ident", 0, 1.5, 0.3, 0.4, 0.5, "h_t", 0.7, 1.0, 0.0]),
]
for _f in (1, 6, 21, 31):
    FIVE_POPS.append(dict(
        name="5d_frozen%d" % _f, grid="default", pts=6, seed=500 + _f,
        args=[0.05, 1, 2, 0.5, 1.5, 0.8] + [0] * 20 + [-1, 2, 0.5, 0, 1.5, 0.3, 0.4, 0.5,
                                                      0.6, 0.7, "theta_t", 0.0] +
             [bool(_f & 1), bool(_f & 2), bool(_f & 4), bool(_f & 8), bool(_f & 16)]))

# one_pop(phi, xx, T, nu, gamma, h, theta0, initial_t, frozen, beta)
ONE_POP = [
    dict(name="1d_const", grid="default", pts=40, seed=10,
         args=[0.3, 2.0, -1.0, 0.3, 1.5], kw=dict(beta=1.2)),
    dict(name="1d_temporal", grid="default", pts=33, seed=11,
         args=[0.3, "exp_grow", 1.0, "h_t", "theta_t"], kw=dict(initial_t=0.01)),
    dict(name="1d_temporal_lin", grid="lin", pts=21, seed=12,
         args=[0.2, "lin_nu", 0.0, 0.5, 1.0]),
]

# Single sweeps: name -> (ndim, axis, pts, grid, params for the swept population)
SWEEPS = [
    ("1Dx", 1, 0, 30, "default"),
    ("2Dx", 2, 0, 25, "default"), ("2Dy", 2, 1, 25, "default"),
    ("3Dx", 3, 0, 12, "lin"), ("3Dy", 3, 1, 12, "default"), ("3Dz", 3, 2, 12, "default"),
    ("4Dx", 4, 0, 7, "default"), ("4Dy", 4, 1, 7, "lin"), ("4Dz", 4, 2, 7, "default"),
    ("4Da", 4, 3, 7, "default"),
    ("5Dx", 5, 0, 6, "default"), ("5Dy", 5, 1, 6, "lin"), ("5Dz", 5, 2, 6, "default"),
    ("5Da", 5, 3, 6, "default"), ("5Db", 5, 4, 6, "default"),
]
SWEEP_PARAMS = dict(nu=0.7, mig=[0.3, 1.2, 0.5, 2.0, 0.8], gamma=-1.5, h=0.3, beta=1.3,
                    dt=0.004)

#: Config-1 workload (split_mig) and the IM parameter draws of the batched workload.
SPLIT_MIG = dict(params=(2.0, 0.5, 0.2, 1.0), ns=(20, 20), pts_l=[40, 50, 60])


def im_draws(n=4096, seed=0):
    """Seed-0 IM parameter sets: s~U(.05,.95); nu1, nu2 log-U[.01,100];
    T log-U[.01,2]; m12, m21 ~ U(0,10), drawn in that order as n-vectors."""
    rng = np.random.default_rng(seed)
    s = rng.uniform(0.05, 0.95, n)
    nu1 = np.exp(rng.uniform(np.log(0.01), np.log(100), n))
    nu2 = np.exp(rng.uniform(np.log(0.01), np.log(100), n))
    T = np.exp(rng.uniform(np.log(0.01), np.log(2), n))
    m12 = rng.uniform(0, 10, n)
    m21 = rng.uniform(0, 10, n)
    return np.stack([s, nu1, nu2, T, m12, m21], axis=1)


def im_parity_sample(draws, steps, n=64):
    """Indices (sorted) of a stratified sample of the 4096-draw IM workload for
    parity at scale: draws 0-5; the longest and shortest schedules; the
    extremes of each parameter (smallest and largest nu1, nu2, T, m12, m21 and
    s); then instances at evenly spaced quantiles of the step counts until
    there are n.  steps[i] is instance i's step count."""
    steps = np.asarray(steps)
    picks = list(range(6))
    picks += [int(np.argmax(steps)), int(np.argmin(steps))]
    for col in range(6):
        picks += [int(np.argmin(draws[:, col])), int(np.argmax(draws[:, col]))]
    chosen = []
    for i in picks:
        if i not in chosen:
            chosen.append(i)
    order = np.argsort(steps, kind="stable")
    q = 0
    nq = n - len(chosen)
    while len(chosen) < n:
        # quantile ranks in (0, 1): skip the extremes already taken
        r = order[int(round((q + 0.5) / max(nq, 1) * (len(order) - 1)))]
        q += 1
        if int(r) not in chosen:
            chosen.append(int(r))
        if q > 4 * len(order):
            break
    return np.array(sorted(chosen[:n]), dtype=np.int64)


#: Dadi golden spectra at the batched workload's grids: this many of the
#: parity sample, the longest schedules first.
IM_SCALE_GOLDEN = 16


#: Config-2 workload: 3 populations with exponential growth (see oracle growth3).
GROWTH3 = dict(params=((0.5, 1.0, 2.0), (5.0, 0.2, 10.0), (0.5, 1.5, 3.0), (-2.0, 0.0, 5.0),
                       0.15),
               ns=(20, 20, 20), pts_l=[70, 80, 90])


#: A small two-population DFE cache (dadi.DFE.Cache2D with DemogSelModels.IM_sel)
#: and its integration over a bivariate lognormal (dadi.DFE.PDFs.biv_lognormal).
DFE = dict(params=(0.4, 1.5, 0.6, 0.1, 1.0, 0.5), ns=(6, 6), pts=[12, 16, 20], gamma_pts=3,
           sel_params=(1.0, 2.0, 0.5), theta=1000.0)


#: dadi's module-level integration settings (dadi/Integration.py:25-44)
#: other than the defaults: each entry runs an IM model pipeline under one
#: of them.  The IM parameters give a time-dependent nu, so dt varies.
SETTINGS = [
    ("old_timestep", dict(use_old_timestep=True, old_timescale_factor=0.1)),
    ("delj", dict(use_delj_trick=True)),
    ("timescale5e-3", dict(timescale_factor=5e-3)),
]
SETTINGS_IM = dict(params=(0.4, 1.5, 0.6, 0.05, 1.0, 0.5), ns=(8, 8), pts_l=[20, 25, 30])

