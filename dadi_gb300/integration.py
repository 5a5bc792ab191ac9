"""Host side of the GPU integrator: dadi's Integration API on sm_103a kernels.

one_pop / two_pops / three_pops / four_pops keep the reference signatures and
semantics (dadi/Integration.py:178-727).  The host evaluates the parameter
functions step by step exactly as the reference loop does -- dt from the
parameters at the current time (`_compute_dt`), every parameter at the next
time, the same validation errors -- and records one table row per step.  The
whole table then runs in one call of the C ABI (dgb_integrate_table): a
shared-memory-resident single-CTA kernel for 2-D grids, one fused sweep kernel
per axis per step for 1-D/3-D/4-D.  A 3-5 population grid whose lines are too
few to fill the FP64 pipes (fewer than two warps per SM sub-partition with one
line per thread) runs instead through dgb_batchnd_integrate as a batch of one
with the partitioned Thomas solve (nd_line_solver).  phi crosses the
host/device boundary once in each direction per call.

Constant-parameter 2-D/3-D calls take the temporal path, as the reference
does when CUDA is enabled (dadi/Integration.py:324, 468); with
enable_cuda_cached=True they take the constant-coefficient path instead
(dgb_integrate_precalc with the a/b/c arrays of dadi/Integration.py:1037-1242).
"""
import sys
import threading

import numpy as np

from . import _lib

#: Settings read at call time, as the module globals of dadi/Integration.py:25-44.
#: When dadi itself is loaded (drop-in mode) its values take precedence.
use_delj_trick = False
timescale_factor = 1e-3
use_old_timestep = False
old_timescale_factor = 0.1

#: Line solver of the 3-5 population integrations: "thomas" (one line per
#: thread, dgb_integrate_table), "partition" (the partitioned Thomas solve of
#: dgb_batchnd_integrate, segments per line from nd_segments or by grid size)
#: or "auto" (autotune.tune_nd_line_solver times both on this GPU once per
#: grid shape).  The results agree to rounding (1e-12); "thomas" keeps them
#: bitwise those of the batched engine.
nd_line_solver = "auto"
nd_segments = 0

#: Solver of the lone 2-population integrations: "thomas" (one CTA,
#: dgb_integrate_table), "cluster" (dgb_integrate2d_cluster over
#: cluster_ctas CTAs, or by the autotuner when 0) or "auto" (the autotuner
#: times both once per grid size).  The results agree to rounding; "thomas"
#: keeps them bitwise those of the batched engine.
line_solver_2d = "auto"
cluster_ctas = 0


def current_settings():
    """(timescale_factor, old_timescale_factor, use_old_timestep, use_delj_trick)."""
    src = sys.modules.get("dadi.Integration") or sys.modules[__name__]
    return (float(getattr(src, "timescale_factor", timescale_factor)),
            float(getattr(src, "old_timescale_factor", old_timescale_factor)),
            bool(getattr(src, "use_old_timestep", use_old_timestep)),
            bool(getattr(src, "use_delj_trick", use_delj_trick)))


def ensure_1arg_func(var):
    """Scalar -> constant function of t returning float64 (dadi/Misc.py:45-68)."""
    if np.isscalar(var):
        f0 = lambda t: var
    else:
        f0 = var
    f = lambda t: np.float64(f0(t))
    if not callable(f0):
        raise ValueError('Argument is not a constant or a function.')
    try:
        f(0.0)
    except TypeError:
        raise ValueError('Argument is not a constant or a one-argument function.')
    return f


def _compute_dt(dx, nu, ms, gamma, h):
    """Timestep from the current parameters (dadi/Integration.py:147-176)."""
    return _dt_with(current_settings(), dx[0], nu, ms, gamma, h)


def _dt_with(settings, dx0, nu, ms, gamma, h):
    """_compute_dt with the settings read once by the caller (the same
    arithmetic; abs of a float64 is exact, as numpy's is)."""
    tsf, otsf, old, _ = settings
    if old:
        return otsf * dx0
    maxVM = max(0.25 / nu, sum(ms),
                abs(gamma) * 2 * max(abs(h + (1 - 2 * h) * 0.5) * 0.5 * (1 - 0.5),
                                     abs(h + (1 - 2 * h) * 0.25) * 0.25 * (1 - 0.25)))
    dt = tsf / maxVM if maxVM > 0 else np.inf
    if dt == 0:
        raise ValueError('Timestep is zero. Values passed in are nu=%f, ms=%s,'
                         'gamma=%f, h=%f.' % (nu, str(ms), gamma, h))
    return dt


def row_stride(P):
    return 3 + 3 * P + P * (P - 1)


def build_table(P, xx, T, initial_t, nu_f, mig_f, gamma_f, h_f, theta0_f, beta_f=None):
    """Per-step parameter table of a P-population time loop.

    nu_f, gamma_f, h_f: P callables; mig_f[k][j]: callable for the rate into k
    from j (ignored for j == k); theta0_f, beta_f callables.  Follows the loop
    of dadi/Integration.py:224-257 (P=1), 346-386 (P=2), 504-553 (P=3),
    672-726 (P=4), raising the same ValueErrors.  Returns (table, history)
    where history lists [t, [nu...], [m...]] like the Demes records.
    """
    current_t = initial_t
    nu = [f(current_t) for f in nu_f]
    gamma = [f(current_t) for f in gamma_f]
    h = [f(current_t) for f in h_f]
    offd = [(k, j) for k in range(P) for j in range(P) if j != k]
    mig = {kj: mig_f[kj[0]][kj[1]](current_t) for kj in offd}
    dx0 = xx[1] - xx[0]
    settings = current_settings()
    rows = []
    hist = [[0, list(nu), [mig[kj] for kj in offd]]]
    stride = row_stride(P)
    into = [[kj for kj in offd if kj[0] == k] for k in range(P)]
    while current_t < T:
        if P == 1:
            dt = _dt_with(settings, dx0, nu[0], [0], gamma[0], h[0])
        else:
            dt = min(_dt_with(settings, dx0, nu[k], [mig[kj] for kj in into[k]], gamma[k], h[k])
                     for k in range(P))
        this_dt = min(dt, T - current_t)
        next_t = current_t + this_dt
        nu = [f(next_t) for f in nu_f]
        gamma = [f(next_t) for f in gamma_f]
        h = [f(next_t) for f in h_f]
        mig = {kj: mig_f[kj[0]][kj[1]](next_t) for kj in offd}
        beta = beta_f(next_t) if beta_f is not None else 1.0
        theta0 = theta0_f(next_t)
        ms = [mig[kj] for kj in offd]
        hist.append([next_t, list(nu), ms])
        if T < 0 or theta0 < 0 or any(v < 0 for v in nu) or any(v < 0 for v in ms):
            raise ValueError('A time, population size, migration rate, or '
                             'theta0 is < 0. Has the model been mis-specified?')
        if any(v == 0 for v in nu):
            raise ValueError('A population size is 0. Has the model been '
                             'mis-specified?')
        rows.append([this_dt, theta0] + nu + gamma + h + [beta] + ms)
        current_t = next_t
    table = np.array(rows, dtype=np.float64).reshape(len(rows), stride)
    return table, hist


def on_device(phi):
    """True for a CUDA torch tensor: the integrators then keep the density on
    the device (a new CUDA tensor is returned), so models chaining epochs and
    splits never copy it to the host in between."""
    return hasattr(phi, "is_cuda") and bool(phi.is_cuda)


def _copy_in(phi):
    """A new array to integrate: a host copy, or a device copy of a CUDA
    tensor (float64, contiguous)."""
    if on_device(phi):
        import torch
        return phi.detach().to(torch.float64).contiguous().clone()
    return np.array(phi, dtype=np.float64, copy=True)


def _device_phi(torch, phi):
    """(device tensor to integrate in place, whether the caller gave one)."""
    if on_device(phi):
        return phi.detach().to(torch.float64).contiguous().clone(), True
    return _lib.to_device(torch, np.ascontiguousarray(phi, dtype=np.float64)), False


#: Per-thread state: `sharing_gpu` is set on the threads of
#: numerics.make_extrap_func that integrate several grids at once, whose
#: Thomas sweeps together already fill the pipes.
local = threading.local()


def partition_segments(P, L, delj=False):
    """Segments per line of the partitioned solve for a lone P-population
    grid of L points under nd_line_solver, or 0 for Thomas.  "partition":
    nd_segments, or as many as keep 8 rows per segment (8 from L = 64, 4
    from 32, 2 from 16); "auto": the autotuner's choice for the shape, and
    Thomas on threads that share the GPU with other grids' integrations
    (measured on the growth model at pts 70/80/90 run concurrently: 0.184 s
    with Thomas, 0.189 s with the partition; one grid after another 0.372 s
    and 0.295 s)."""
    mode = nd_line_solver
    if mode not in ("auto", "thomas", "partition"):
        raise ValueError("nd_line_solver must be 'auto', 'thomas' or 'partition'")
    if P < 3 or delj or mode == "thomas":
        return 0
    if mode == "auto":
        if getattr(local, "sharing_gpu", False):
            return 0
        from . import autotune
        return autotune.tune_nd_line_solver(P, L)["segments"]
    seg = int(nd_segments) or next((s for s in (8, 4, 2) if L >= 8 * s), 0)
    return seg if seg and L >= 3 * seg else 0


def cluster_size_2d(L, delj=False):
    """CTAs of the cluster for a lone 2-population grid of L points under
    line_solver_2d, or 0 for the one-CTA Thomas path."""
    mode = line_solver_2d
    if mode not in ("auto", "thomas", "cluster"):
        raise ValueError("line_solver_2d must be 'auto', 'thomas' or 'cluster'")
    if delj or mode == "thomas" or not 24 <= L <= 128:
        return 0
    if mode == "cluster" and cluster_ctas:
        return int(cluster_ctas)
    from . import autotune
    return autotune.tune_2d_cluster(L)["ctas"]


_engines = {}


def _partition_engine(P, L, xx, seg):
    """A batch-of-one engine with the partitioned solve, kept per (P, grid,
    segments) for the life of the process: its grid stays on the device,
    and is never freed under a launch still in flight on another stream."""
    from . import batchnd
    xx = np.ascontiguousarray(xx, dtype=np.float64)
    key = (P, seg, xx.tobytes())
    eng = _engines.get(key)
    if eng is None:
        eng = _engines.setdefault(key, batchnd.BatchND(P, L, xx=xx, line_solver=2,
                                                       segments=seg))
    return eng


def run_table(phi, xx, table, frozen_mask=0, nomut_mask=0):
    """Integrate phi (host ndarray, or CUDA tensor kept on the device)
    through a parameter table on the GPU; returns a new array of the same
    kind."""
    torch = _lib.require_cuda()
    P, L = phi.ndim, phi.shape[0]
    if any(s != L for s in phi.shape) or len(xx) != L:
        raise ValueError("phi must be square with len(xx) points per axis")
    if len(table) == 0:
        return _copy_in(phi)
    d_phi, dev = _device_phi(torch, phi)
    delj = current_settings()[3]
    ctas = cluster_size_2d(L, delj) if P == 2 else 0
    if ctas:
        d_xx, d_tab = _lib.to_device(torch, xx), _lib.to_device(torch, table)
        _lib.check(_lib.lib().dgb_integrate2d_cluster(
            _lib.dptr(d_phi), L, _lib.dptr(d_xx), _lib.dptr(d_tab), len(table),
            int(frozen_mask), int(nomut_mask), ctas, _lib.stream_handle(torch)),
            "dgb_integrate2d_cluster")
        return d_phi if dev else _lib.to_host(torch, d_phi)
    seg = partition_segments(P, L, delj)
    if seg:
        out = _partition_engine(P, L, xx, seg).integrate(
            d_phi, [np.asarray(table, dtype=np.float64)],
            [int(frozen_mask) | int(nomut_mask) << 8])[0]
        return out if dev else _lib.to_host(torch, out)
    d_xx = _lib.to_device(torch, xx)
    d_tab = _lib.to_device(torch, table)
    ws, nws = _lib.workspace(torch, _lib.lib().dgb_workspace_bytes(0, P, L, 0))
    delj = current_settings()[3]
    rc = _lib.lib().dgb_integrate_table(_lib.dptr(d_phi), P, L, _lib.dptr(d_xx), _lib.dptr(d_tab),
                                        len(table), int(frozen_mask), int(nomut_mask), int(delj),
                                        _lib.dptr(ws), nws, _lib.stream_handle(torch))
    _lib.check(rc, "dgb_integrate_table")
    return d_phi if dev else _lib.to_host(torch, d_phi)


def step_lengths(dt, T, initial_t):
    """The step lengths of the constant-parameter loops
    (dadi/Integration.py:1108-1117): min(dt, T - t) until t reaches T."""
    dts = []
    t = initial_t
    while t < T:
        this_dt = min(dt, T - t)
        dts.append(this_dt)
        t += this_dt
    return np.array(dts, dtype=np.float64)


def run_precalc(phi, xx, abc, dts, theta0, frozen_mask=0, nomut_mask=0):
    """Constant-coefficient loop on the GPU (abc: 3*P arrays shaped like phi);
    phi a host ndarray or a CUDA tensor (kept on the device)."""
    torch = _lib.require_cuda()
    P, L = phi.ndim, phi.shape[0]
    if len(dts) == 0:
        return _copy_in(phi)
    d_phi, dev = _device_phi(torch, phi)
    d_xx = _lib.to_device(torch, xx)
    d_abc = _lib.to_device(torch, np.stack([np.asarray(v, dtype=np.float64) for v in abc]))
    d_dts = _lib.to_device(torch, dts)
    ws, nws = _lib.workspace(torch, 0)
    rc = _lib.lib().dgb_integrate_precalc(_lib.dptr(d_phi), P, L, _lib.dptr(d_xx), _lib.dptr(d_abc),
                                          _lib.dptr(d_dts), len(dts), float(theta0),
                                          int(frozen_mask), int(nomut_mask), _lib.dptr(ws), nws,
                                          _lib.stream_handle(torch))
    _lib.check(rc, "dgb_integrate_precalc")
    return d_phi if dev else _lib.to_host(torch, d_phi)


# -------------------------------------------------- constant-coefficient build

def _Vfunc(x, nu, beta=1):
    return 1. / nu * x * (1 - x) * (beta + 1.) ** 2 / (4. * beta)


def _Msel(x, gamma, h):
    return gamma * 2 * (h + (1 - 2 * h) * x) * x * (1 - x)


def _Mfull(xk, others, ms, gamma, h):
    if not others:
        return _Msel(xk, gamma, h)
    acc = ms[0] * (others[0] - xk)
    for o, m in zip(others[1:], ms[1:]):
        acc = acc + m * (o - xk)
    return acc + _Msel(xk, gamma, h)


def _compute_dfactor(dx):
    dfactor = np.zeros(len(dx) + 1)
    dfactor[1:-1] = 2 / (dx[:-1] + dx[1:])
    dfactor[0] = 2 / dx[0]
    dfactor[-1] = 2 / dx[-1]
    return dfactor


def const_coefficients(xx, P, axis, nu, ms, gamma, h):
    """a, b, c of one axis for constant parameters, b without 1/dt, with the
    corner boundary terms (dadi/Integration.py:1057-1095, 1145-1222).  ms are
    the migration rates into this population, other axes in increasing order."""
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
    up = lambda v: v[sh(axis)]
    if current_settings()[3]:
        wj = 2 * MInt * up(dx)
        with np.errstate(all="ignore"):
            epsj = np.exp(wj / up(VInt))
            delj = (-epsj * wj + epsj * up(VInt) - up(VInt)) / (wj - epsj * wj)
        delj = np.where(np.isnan(delj), 0.5, delj)
        delj = np.where(np.isinf(delj), 0.5, delj)
    else:
        delj = 0.5
    a, b, c = [np.zeros((L,) * P) for _ in range(3)]

    def sl(lo, hi):
        return tuple(slice(lo, hi) if j == axis else slice(None) for j in range(P))
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


# ------------------------------------------------- reference-signature API

def _check_T(T, initial_t):
    if T - initial_t < 0:
        raise ValueError('Final integration time T (%f) is less than '
                         'intial_time (%f). Integration cannot be run '
                         'backwards.' % (T, initial_t))


def _masks(flags):
    return sum(1 << k for k, f in enumerate(flags) if f)


def one_pop(phi, xx, T, nu=1, gamma=0, h=0.5, theta0=1.0, initial_t=0, frozen=False, beta=1,
            deme_ids=None):
    """dadi/Integration.py:178-258 on the GPU (temporal loop for all inputs)."""
    phi = _copy_in(phi)
    if frozen or T - initial_t == 0:
        return phi
    _check_T(T, initial_t)
    f = ensure_1arg_func
    table, _ = build_table(1, xx, T, initial_t, [f(nu)], [[None]], [f(gamma)], [f(h)],
                           f(theta0), beta_f=f(beta))
    return run_table(phi, xx, table)


def _frozen_mig_check(P, frozen, mig):
    for k in range(P):
        if frozen[k] and any(mig[k][j] != 0 or mig[j][k] != 0 for j in range(P) if j != k):
            raise ValueError('Population cannot be frozen and have non-zero '
                             'migration to or from it.')


def _integrate(P, phi, xx, T, initial_t, nus, mig, gammas, hs, theta0, frozen, nomut,
               enable_cuda_cached):
    _frozen_mig_check(P, frozen, mig)
    vals = list(nus) + [mig[k][j] for k in range(P) for j in range(P) if j != k] + \
        list(gammas) + list(hs) + [theta0]
    if P in (2, 3) and enable_cuda_cached and np.all([np.isscalar(v) for v in vals]):
        flat_m = [mig[k][j] for k in range(P) for j in range(P) if j != k]
        if np.any(np.less([T] + list(nus) + flat_m + [theta0], 0)):
            raise ValueError('A time, population size, migration rate, or theta0 '
                             'is < 0. Has the model been mis-specified?')
        if np.any(np.equal(nus, 0)):
            raise ValueError('A population size is 0. Has the model been '
                             'mis-specified?')
        ms = [[mig[k][j] for j in range(P) if j != k] for k in range(P)]
        abc = []
        for k in range(P):
            abc.extend(const_coefficients(xx, P, k, nus[k], ms[k], gammas[k], hs[k]))
        dx = np.diff(xx)
        dt = min(_compute_dt(dx, nus[k], ms[k], gammas[k], hs[k]) for k in range(P))
        return run_precalc(phi, xx, abc, step_lengths(dt, T, initial_t), theta0,
                           _masks(frozen), _masks(nomut))
    f = ensure_1arg_func
    mig_f = [[None if j == k else f(mig[k][j]) for j in range(P)] for k in range(P)]
    table, _ = build_table(P, xx, T, initial_t, [f(v) for v in nus], mig_f,
                           [f(v) for v in gammas], [f(v) for v in hs], f(theta0))
    return run_table(phi, xx, table, _masks(frozen), _masks(nomut))


def two_pops(phi, xx, T, nu1=1, nu2=1, m12=0, m21=0, gamma1=0, gamma2=0, h1=0.5, h2=0.5,
             theta0=1, initial_t=0, frozen1=False, frozen2=False, nomut1=False, nomut2=False,
             enable_cuda_cached=False, deme_ids=None):
    """dadi/Integration.py:260-387 on the GPU; returns a new array."""
    phi = _copy_in(phi)
    if T - initial_t == 0:
        return phi
    _check_T(T, initial_t)
    return _integrate(2, phi, xx, T, initial_t, [nu1, nu2], [[0, m12], [m21, 0]],
                      [gamma1, gamma2], [h1, h2], theta0, [frozen1, frozen2], [nomut1, nomut2],
                      enable_cuda_cached)


def three_pops(phi, xx, T, nu1=1, nu2=1, nu3=1, m12=0, m13=0, m21=0, m23=0, m31=0, m32=0,
               gamma1=0, gamma2=0, gamma3=0, h1=0.5, h2=0.5, h3=0.5, theta0=1, initial_t=0,
               frozen1=False, frozen2=False, frozen3=False, enable_cuda_cached=False,
               deme_ids=None):
    """dadi/Integration.py:389-554 on the GPU; returns a new array."""
    phi = _copy_in(phi)
    if T - initial_t == 0:
        return phi
    _check_T(T, initial_t)
    mig = [[0, m12, m13], [m21, 0, m23], [m31, m32, 0]]
    return _integrate(3, phi, xx, T, initial_t, [nu1, nu2, nu3], mig, [gamma1, gamma2, gamma3],
                      [h1, h2, h3], theta0, [frozen1, frozen2, frozen3], [False] * 3,
                      enable_cuda_cached)


def five_pops(phi, xx, T, nu1=1, nu2=1, nu3=1, nu4=1, nu5=1,
              m12=0, m13=0, m14=0, m15=0, m21=0, m23=0, m24=0, m25=0,
              m31=0, m32=0, m34=0, m35=0, m41=0, m42=0, m43=0, m45=0,
              m51=0, m52=0, m53=0, m54=0,
              gamma1=0, gamma2=0, gamma3=0, gamma4=0, gamma5=0,
              h1=0.5, h2=0.5, h3=0.5, h4=0.5, h5=0.5,
              theta0=1, initial_t=0, frozen1=False, frozen2=False,
              frozen3=False, frozen4=False, frozen5=False, deme_ids=None):
    """dadi/Integration.py:729-937 on the GPU; returns a new array (the
    reference's CPU path updates phi in place)."""
    phi = _copy_in(phi)
    if T - initial_t == 0:
        return phi
    _check_T(T, initial_t)
    mig = [[0, m12, m13, m14, m15], [m21, 0, m23, m24, m25], [m31, m32, 0, m34, m35],
           [m41, m42, m43, 0, m45], [m51, m52, m53, m54, 0]]
    return _integrate(5, phi, xx, T, initial_t, [nu1, nu2, nu3, nu4, nu5], mig,
                      [gamma1, gamma2, gamma3, gamma4, gamma5], [h1, h2, h3, h4, h5], theta0,
                      [frozen1, frozen2, frozen3, frozen4, frozen5], [False] * 5, False)


def four_pops(phi, xx, T, nu1=1, nu2=1, nu3=1, nu4=1, m12=0, m13=0, m14=0, m21=0, m23=0,
              m24=0, m31=0, m32=0, m34=0, m41=0, m42=0, m43=0, gamma1=0, gamma2=0, gamma3=0,
              gamma4=0, h1=0.5, h2=0.5, h3=0.5, h4=0.5, theta0=1, initial_t=0, frozen1=False,
              frozen2=False, frozen3=False, frozen4=False, deme_ids=None):
    """dadi/Integration.py:556-727 on the GPU.  Like the reference's CUDA path
    this returns a new array (the reference's CPU path updates phi in place)."""
    phi = _copy_in(phi)
    if T - initial_t == 0:
        return phi
    _check_T(T, initial_t)
    mig = [[0, m12, m13, m14], [m21, 0, m23, m24], [m31, m32, 0, m34], [m41, m42, m43, 0]]
    return _integrate(4, phi, xx, T, initial_t, [nu1, nu2, nu3, nu4], mig,
                      [gamma1, gamma2, gamma3, gamma4], [h1, h2, h3, h4], theta0,
                      [frozen1, frozen2, frozen3, frozen4], [False] * 4, False)
