"""Batched N-dimensional engine: many integrations of 1-5 populations that
share a grid advance together (dgb_batchnd_integrate), so a 3-D or 4-D sweep
launch carries the lines of every integration instead of the 4,900-8,100
lines of one grid -- enough warps to keep every SM's FP64 pipe busy.

Schedules come from parameter tables: either built by the caller (any
parameter callables, integration.build_table, the reference loop of
dadi/Integration.py:389-937) or walked in C from parametric records
(dgb_schednd_host: constant, exponential-growth and linear parameters, the
same loop).  Each integration's density is bitwise the one the one-at-a-time
drop-in (dgb_integrate_table) computes.

This is the GPU form of evaluating make_extrap_func(model) of a three- or
four-population model for many parameter sets (dadi/Numerics.py:334-475;
the reference runs them one at a time, or in worker processes as
dadi/DFE/Cache2D_mod.py:117-167 does for two populations).
"""
import ctypes

import numpy as np

from . import _lib, epilogue, integration, numerics, phimanip, spectrum

PF_CONST, PF_EXPLOG = _lib.PF_CONST, _lib.PF_EXPLOG


def _pf(kind, a, b=0.0, c=1.0):
    f = _lib.PForm()
    f.kind, f.a, f.b, f.c = kind, float(a), float(b), float(c)
    return f


def instance(ndim, T, nu, mig=None, gamma=None, h=None, theta0=1.0, initial_t=0.0):
    """A dgb_instnd record.  nu, gamma, h: per population, each a number
    (constant) or a dgb_pform built with form(); mig[k][j]: the rate into
    population k from j (numbers or forms; the diagonal is ignored)."""
    rec = _lib.InstND()
    rec.T, rec.initial_t, rec.ndim = float(T), float(initial_t), int(ndim)

    def asf(v):
        return v if isinstance(v, _lib.PForm) else _pf(PF_CONST, v)
    gamma = [0.0] * ndim if gamma is None else gamma
    h = [0.5] * ndim if h is None else h
    for k in range(ndim):
        rec.nu[k] = asf(nu[k])
        rec.gamma[k] = asf(gamma[k])
        rec.h[k] = asf(h[k])
        for j in range(ndim):
            rec.mig[k][j] = asf(0.0 if (mig is None or j == k) else mig[k][j])
    rec.theta0 = asf(theta0)
    return rec


def form_explog(a, b, c):
    """a * exp(log(b / a) * t / c): exponential growth from a to b over c."""
    return _pf(PF_EXPLOG, a, b, c)


def growth3_instance(params):
    """The three-population growth model (models.growth3): sizes
    nu0_i exp(log(nuF_i / nu0_i) t / T), symmetric migration m12, m13, m23,
    per-population selection."""
    (nu0, nuF, (m12, m13, m23), g, T) = params
    nu = [form_explog(a, b, T) for a, b in zip(nu0, nuF)]
    mig = [[0, m12, m13], [m12, 0, m23], [m13, m23, 0]]
    return instance(3, T, nu, mig, gamma=list(g))


def four_split_instance(params):
    """The four-population model (models.four_split): constant sizes and
    symmetric migration m between every pair."""
    nu1, nu2, nu3, nu4, m, T = params
    mig = [[0 if j == k else m for j in range(4)] for k in range(4)]
    return instance(4, T, [nu1, nu2, nu3, nu4], mig)


def schedules(insts, settings=None, dx0=None, max_steps=10 ** 7):
    """Parameter tables of dgb_instnd records (all the same ndim), walked in C
    on the host: (list of (nsteps, stride) tables, status per record)."""
    n = len(insts)
    arr = (_lib.InstND * n)(*insts)
    st = settings or integration_settings()
    lib = _lib.lib()
    cnt = np.zeros(n, dtype=np.int32)
    d0 = float(dx0) if dx0 is not None else 0.0
    _lib.check(lib.dgb_schednd_host(ctypes.cast(arr, ctypes.c_void_p), n, ctypes.byref(st),
                                    int(max_steps), d0, cnt.ctypes.data_as(ctypes.c_void_p),
                                    None, None, None), "dgb_schednd_host(count)")
    P = insts[0].ndim
    stride = integration.row_stride(P)
    off = np.zeros(n, dtype=np.int64)
    off[1:] = np.cumsum(cnt.astype(np.int64))[:-1]
    table = np.zeros((max(int(cnt.sum()), 1), stride))
    status = np.zeros(n, dtype=np.int32)
    _lib.check(lib.dgb_schednd_host(ctypes.cast(arr, ctypes.c_void_p), n, ctypes.byref(st),
                                    int(max_steps), d0, cnt.ctypes.data_as(ctypes.c_void_p),
                                    off.ctypes.data_as(ctypes.c_void_p),
                                    table.ctypes.data_as(ctypes.c_void_p),
                                    status.ctypes.data_as(ctypes.c_void_p)),
               "dgb_schednd_host(fill)")
    tabs = [table[o:o + c] for o, c in zip(off, cnt)]
    return tabs, status


def integration_settings(gam_placement=0, threads=0, line_solver=0, segments=0):
    tsf, otsf, old, delj = integration.current_settings()
    return _lib.settings_struct(tsf, otsf, old, delj, gam_placement, threads, line_solver,
                                segments)


class BatchND:
    """Integrations of `ndim` populations on one grid xx (default grid of L
    points unless given).  gam_placement / threads: the launch knobs of
    dgb_batchnd_integrate (0 = auto); line_solver: 0 Thomas (one line per
    thread), 1 parallel cyclic reduction (one warp per line), 2 partitioned
    Thomas (`segments` threads per line: 2, 4 or 8, 0 = 4)."""

    def __init__(self, ndim, L, xx=None, gam_placement=0, threads=0, line_solver=0,
                 segments=0):
        self.torch = _lib.require_cuda()
        self.ndim, self.L = int(ndim), int(L)
        self.xx = numerics.default_grid(L) if xx is None else np.asarray(xx, dtype=np.float64)
        self.d_xx = _lib.upload_resident(self.torch, self.xx)
        self.gam_placement, self.threads = gam_placement, threads
        self.line_solver, self.segments = line_solver, segments

    def integrate(self, phi0, tables, masks=None, timer=None):
        """Integrate n densities through their tables.  phi0: a CUDA tensor
        (n, L, ..., L) of initial densities, or one (L, ..., L) density
        shared by all; tables: n parameter tables (rows of
        integration.build_table); masks: n values frozen_mask | nomut_mask
        << 8.  Returns the (n, L, ..., L) CUDA tensor of results."""
        torch = self.torch
        lib = _lib.lib()
        P, L = self.ndim, self.L
        n = len(tables)
        per = L ** P
        if phi0.dim() == P:
            phi = phi0.to(torch.float64).reshape(1, per).expand(n, per).contiguous()
        else:
            phi = phi0.to(torch.float64).reshape(n, per).contiguous().clone()
        if n == 0:
            return phi.view((0,) + (L,) * P)
        steps = np.array([len(t) for t in tables], dtype=np.int32)
        order = np.argsort(-steps, kind="stable")
        stride = integration.row_stride(P)
        tab = np.concatenate([np.asarray(tables[i], dtype=np.float64).reshape(-1, stride)
                              for i in order] + [np.zeros((1, stride))])
        row_off = np.zeros(n, dtype=np.int64)
        row_off[1:] = np.cumsum(steps[order].astype(np.int64))[:-1]
        items = np.zeros(n, dtype=[("phi_off", "i8"), ("row_off", "i8"), ("nsteps", "i4"),
                                   ("masks", "i4")])
        items["phi_off"] = order.astype(np.int64) * per
        items["row_off"] = row_off
        items["nsteps"] = steps[order]
        items["masks"] = 0 if masks is None else np.asarray(masks, dtype=np.int32)[order]
        nsteps_h = np.ascontiguousarray(steps[order])
        st = integration_settings(self.gam_placement, self.threads, self.line_solver,
                                  self.segments)
        d_items = _lib.to_device(torch, items.view(np.uint8), np.uint8)
        d_tab = _lib.to_device(torch, tab)
        nws = lib.dgb_batchnd_workspace_bytes(P, L, n, ctypes.byref(st))
        if nws == 0:
            raise _lib.DgbError(_lib.DGB_ERR_UNSUPPORTED, "dgb_batchnd_workspace_bytes")
        ws, nws = _lib.workspace(torch, nws)
        if timer is not None:
            timer[0].record()
        rc = lib.dgb_batchnd_integrate(_lib.dptr(d_items),
                                       nsteps_h.ctypes.data_as(ctypes.c_void_p), n, P, L,
                                       _lib.dptr(self.d_xx), _lib.dptr(phi), _lib.dptr(d_tab),
                                       ctypes.byref(st), _lib.dptr(ws), nws,
                                       _lib.stream_handle(torch))
        if timer is not None:
            timer[1].record()
        _lib.check(rc, "dgb_batchnd_integrate")
        self._keep = (d_items, d_tab, ws)
        return phi.view((n,) + (L,) * P)


def initial_density(kind, L):
    """The initial density of the workload models on the default grid of L
    points: growth3 (phi_1D split to 2-D, population 2 split to 3) and four
    (then population 3 split to 4), dadi/PhiManip.py:12-250, 412-450."""
    xx = numerics.default_grid(L)
    phi = phimanip.phi_1D_to_2D(xx, phimanip.phi_1D(xx))
    phi = phimanip.phi_2D_to_3D_split_2(xx, phi)
    if kind == "four":
        phi = phimanip.phi_3D_to_4D(phi, 0.0, 0.0, xx, xx, xx, xx)
    return phi


#: The workload models with a batched form: (ndim, record builder).
MODELS = {"growth3": (3, growth3_instance), "four": (4, four_split_instance)}


class ModelBatch:
    """Extrapolated spectra of many parameter sets of a three- or
    four-population workload model ("growth3": models.growth3, "four":
    models.four_split) on grids pts_l with sample sizes ns: the GPU form of
    make_extrap_func(model)(params, ns, pts_l) for each set
    (dadi/Numerics.py:334-475).  Per grid one batched integration (all sets
    advance together; the grids on their own streams), the N-dimensional
    from_phi kernel, then extrapolation with the fail_mag guard and the
    Poisson likelihood in one launch: densities never leave the device."""

    def __init__(self, kind, pts_l, ns, gam_placement=0, threads=0):
        self.torch = _lib.require_cuda()
        self.kind = kind
        self.ndim, self.make = MODELS[kind]
        self.pts_l = list(pts_l)
        self.ns = tuple(ns)
        self.engines = [BatchND(self.ndim, L, gam_placement=gam_placement, threads=threads)
                        for L in self.pts_l]
        self.phi0 = [_lib.upload_resident(self.torch, initial_density(kind, L))
                     for L in self.pts_l]
        self.x_l = [e.xx[1] for e in self.engines]
        self._side = None

    def tables(self, params_list):
        """Per grid, the parameter tables of every set (one list shared by
        all grids unless old-timestep mode makes dt depend on the grid), and
        the status bits per set."""
        insts = [self.make(p) for p in params_list]
        if integration.current_settings()[2]:
            per, status = [], np.zeros(len(insts), dtype=np.int32)
            for e in self.engines:
                t, st = schedules(insts, dx0=e.xx[1] - e.xx[0])
                per.append(t)
                status |= st
            return per, status
        t, status = schedules(insts)
        return [t] * len(self.engines), status

    def run(self, params_list, data=None, scale=1.0, timer=None):
        """(extrapolated spectra (n, n1+1, ...), Poisson ll (n,) or None,
        status (n,) numpy) for the parameter sets; CUDA tensors."""
        torch = self.torch
        tabs, status = self.tables(params_list)
        cur = torch.cuda.current_stream()
        if self._side is None:
            self._side = [torch.cuda.Stream() for _ in self.engines]
        fork = torch.cuda.Event()
        fork.record(cur)
        if timer is not None:
            timer[0].record(cur)
        raws = []
        for e, p0, t, side in zip(self.engines, self.phi0, tabs, self._side):
            side.wait_event(fork)
            with torch.cuda.stream(side):
                phi = e.integrate(p0, t)
                raws.append(spectrum.from_phi_nd_batch(torch, phi, self.ns, e.xx))
                phi.record_stream(side)
            cur.wait_stream(side)
        for r, side in zip(raws, self._side):
            r.record_stream(cur)
        if timer is not None:
            timer[1].record(cur)
        fs, ll = epilogue.extrapolate_batch(torch, raws, self.x_l, data, scale)
        return fs, ll, status
