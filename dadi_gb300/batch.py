"""Batched 2-population engine: thousands of integrations in one launch.

Each (instance, grid) pair is one work item of a persistent kernel
(dgb_batch2d_integrate): the parametric schedule is evaluated on the device
with the reference's operation order (dadi/Integration.py:147-176, 355-386),
phi stays in shared memory for the whole loop, and CTAs pull items
longest-first from an atomic counter, so instances with 11 or 20,000 steps
balance across the SMs.  The launch shape — one launch over all grids or one
per grid size (CTA size fitted to each L, two items per CTA where that fills
the warps better), the Thomas scratch placement — is what
autotune.tune_batch2d chooses; every shape gives the same bits.  The spectra, their Richardson extrapolation and the
Poisson likelihood are computed on the device afterwards, so only parameters
go in and spectra / likelihoods come out.

This is the GPU form of evaluating dadi.Numerics.make_extrap_func(model) for
many parameter sets (dadi/Numerics.py:334-475; the reference parallelises such
work with host processes, dadi/DFE/Cache2D_mod.py:117-167).
"""
import ctypes

import numpy as np

from . import _lib, epilogue, integration, numerics, phimanip, spectrum

INST_DTYPE = np.dtype({
    "names": ["T", "initial_t", "nu", "m12", "m21", "gamma", "h", "theta0", "frozen", "nomut"],
    "formats": ["f8", "f8", ("f8", (2, 4)), ("f8", 4), ("f8", 4), ("f8", (2, 4)),
                ("f8", (2, 4)), ("f8", 4), "i4", "i4"],
    "offsets": [0, 8, 16, 80, 112, 144, 208, 272, 304, 308],
    "itemsize": 312})


def _pf(kind, a=0.0, b=0.0, c=0.0):
    """A dgb_pform packed as 4 doubles (kind stored in the first int)."""
    v = np.zeros(4)
    v.view(np.int32)[0] = kind
    v[1], v[2], v[3] = a, b, c
    return v


def _pf_array(kind, a, b=None, c=None):
    n = len(a)
    out = np.zeros((n, 4))
    out.view(np.int32)[:, 0] = kind
    out[:, 1] = a
    if b is not None:
        out[:, 2] = b
    if c is not None:
        out[:, 3] = c
    return out


def im_instances(params, initial_t=0.0, theta0=1.0):
    """dgb_inst2d records of Demographics2D.IM (dadi/Demographics2D.py:297-307)
    for rows (s, nu1, nu2, T, m12, m21): nu1(t) = s (nu1/s)**(t/T),
    nu2(t) = (1-s) (nu2/(1-s))**(t/T), constant migration."""
    p = np.asarray(params, dtype=np.float64).reshape(-1, 6)
    n = len(p)
    s, nu1, nu2, T, m12, m21 = p.T
    rec = np.zeros(n, dtype=INST_DTYPE)
    rec["T"] = T
    rec["initial_t"] = initial_t
    rec["nu"][:, 0] = _pf_array(_lib.PF_EXPGROW, s, nu1, T)
    rec["nu"][:, 1] = _pf_array(_lib.PF_EXPGROW, 1 - s, nu2, T)
    rec["m12"] = _pf_array(_lib.PF_CONST, m12)
    rec["m21"] = _pf_array(_lib.PF_CONST, m21)
    rec["gamma"][:, 0] = _pf_array(_lib.PF_CONST, np.zeros(n))
    rec["gamma"][:, 1] = _pf_array(_lib.PF_CONST, np.zeros(n))
    rec["h"][:, 0] = _pf_array(_lib.PF_CONST, np.full(n, 0.5))
    rec["h"][:, 1] = _pf_array(_lib.PF_CONST, np.full(n, 0.5))
    rec["theta0"] = _pf_array(_lib.PF_CONST, np.full(n, theta0))
    return rec


#: dgb_seed2d: dT[6], dt0[6], dform[9 forms][a, b, c][6]
SEED_DTYPE = np.dtype([("dT", "f8", 6), ("dt0", "f8", 6), ("dform", "f8", (9, 3, 6))])
IM_PARAMS = ("s", "nu1", "nu2", "T", "m12", "m21")


def im_seeds(n):
    """Derivative seeds of im_instances' coefficients with respect to
    (s, nu1, nu2, T, m12, m21): nu1(t) = s (nu1/s)**(t/T) has a = s, b = nu1,
    c = T; nu2(t) = (1-s) (nu2/(1-s))**(t/T) has a = 1-s, b = nu2, c = T."""
    sd = np.zeros(n, dtype=SEED_DTYPE)
    S, N1, N2, T, M12, M21 = range(6)
    sd["dT"][:, T] = 1
    sd["dform"][:, 0, 0, S] = 1
    sd["dform"][:, 0, 1, N1] = 1
    sd["dform"][:, 0, 2, T] = 1
    sd["dform"][:, 1, 0, S] = -1
    sd["dform"][:, 1, 1, N2] = 1
    sd["dform"][:, 1, 2, T] = 1
    sd["dform"][:, 2, 0, M12] = 1
    sd["dform"][:, 3, 0, M21] = 1
    return sd


def hybrid_plan(steps, Lsq, limit, ctas, cluster_items, nsm, per_sm):
    """How the hybrid adjoint splits work items (steps and L^2 per item):
    order, longest (steps x L^2) first; size, each item's trajectory in
    bytes ((2 steps + 1) L^2 doubles); k, the longest items whose
    trajectories fit `limit` bytes (at least one, and at least one item
    left for the segment mode); j, how many of those walk on clusters of
    `ctas` CTAs (at most cluster_items, within a quarter of the nsm SMs; 0
    when ctas is 0); rest, the segment-mode walk's CTAs: the SMs the
    clusters and the other trajectory items leave at per_sm CTAs each, never
    fewer than a quarter of the device's CTAs nor more than its items."""
    steps = np.asarray(steps, dtype=np.int64)
    Lsq = np.asarray(Lsq, dtype=np.int64)
    order = np.argsort(-(steps * Lsq), kind="stable").astype(np.int32)
    size = (2 * steps + 1) * Lsq * 8
    k = int(np.searchsorted(np.cumsum(size[order]), limit, side="right"))
    k = max(1, min(k, len(order) - 1))
    j = min(k, cluster_items, nsm // (4 * ctas)) if ctas else 0
    rest = min(len(order) - k, max(nsm * per_sm // 4, (nsm - j * ctas) * per_sm - (k - j)))
    return order, size, k, j, max(1, rest)


def settings_from_globals(gam_placement=0, threads=0):
    tsf, otsf, old, delj = integration.current_settings()
    return _lib.settings_struct(tsf, otsf, old, delj, gam_placement, threads)


def _pform_at(f, t):
    """Values of dgb_pform records f ((n, 4) float64, the kind in the first
    int) at times t (n,), as pform_eval computes them."""
    kind = np.ascontiguousarray(f).view(np.int32)[:, 0]
    a, b, c = f[:, 1], f[:, 2], f[:, 3]
    with np.errstate(all="ignore"):
        return np.where(kind == _lib.PF_EXPGROW, a * (b / a) ** (t / c),
                        np.where(kind == _lib.PF_EXPLOG, a * np.exp(np.log(b / a) * t / c),
                                 np.where(kind == _lib.PF_LINEAR, a + b * t, a)))


#: Reserve at most this many schedule rows from host bounds (else count them).
ROW_BOUND_LIMIT = 2 * 10 ** 8


def row_bounds(rec, settings, dx0s, max_steps):
    """Upper bounds on the rows of each schedule of dgb_inst2d records (one
    per instance, or per (instance, grid) under use_old_timestep), so that
    dgb_sched2d can fill them in one pass; None when no useful bound exists
    (non-finite or nonpositive sizes at an end of the interval, or more than
    ROW_BOUND_LIMIT rows in all).

    Every parametric form is monotone in t (constant, exponential, linear),
    so over [initial_t, T] a size is at least its smaller end value, a
    migration rate at most its larger one, and |gamma| and the dominance
    factor of _compute_dt (dadi/Integration.py:147-176) at most their larger
    ends.  Each step is then at least dt_min = timescale_factor / max(0.25 /
    nu_min, m_max, 2 |gamma|_max tm_max) over both populations (division and
    max are monotone in floating point), so a schedule has at most
    (T - initial_t) / dt_min rows; the reserve adds 1e-9 relative and two
    rows for the rounding of the sums of steps."""
    rec = np.ascontiguousarray(rec)
    t0, T = rec["initial_t"], rec["T"]
    span = T - t0
    if settings.use_old_timestep:
        # one schedule per (instance, grid): dt = old_timescale_factor * dx0
        dts = settings.old_timescale_factor * np.asarray(dx0s, dtype=np.float64)
        span = np.repeat(span[:, None], len(dts), axis=1)
        per = span / dts[None, :]
    else:
        live = span > 0  # the others take no step (NaN included)

        def ends(f):
            return _pform_at(f, t0), _pform_at(f, T)
        vm = []
        for k, mig in ((0, rec["m12"]), (1, rec["m21"])):
            nu = np.minimum(*ends(rec["nu"][:, k]))
            m = np.maximum(*ends(mig))
            g = np.maximum(*[np.abs(v) for v in ends(rec["gamma"][:, k])])
            tm = np.maximum(*[np.maximum(np.abs(h + (1 - 2 * h) * 0.5) * 0.5 * (1 - 0.5),
                                         np.abs(h + (1 - 2 * h) * 0.25) * 0.25 * (1 - 0.25))
                              for h in ends(rec["h"][:, k])])
            if not np.all((np.isfinite(nu) & (nu > 0))[live]):
                return None
            with np.errstate(all="ignore"):
                vm.append(np.maximum(np.maximum(0.25 / nu, m), g * 2 * tm))
        with np.errstate(all="ignore"):
            per = np.where(live, span * np.maximum(vm[0], vm[1]) / settings.timescale_factor,
                           0.0)
    per = np.where(span > 0, per, 0.0)
    if not np.all(np.isfinite(per)):
        return None
    caps = np.where(per > 0, np.floor(per * (1 + 1e-9)) + 2, 0.0)
    caps = np.minimum(caps, float(max_steps)).reshape(-1)
    if caps.sum() > ROW_BOUND_LIMIT:
        return None
    return caps.astype(np.int64)


#: dgb_item2d (dadi_gb300.h): one (integration, grid) work item.
ITEM2D_DTYPE = np.dtype([("L", "i4"), ("masks", "i4"), ("xx_off", "i8"), ("out_off", "i8"),
                         ("sched", "i8")])


def count_steps(rec, settings=None, max_steps=10 ** 8):
    """Steps each instance takes (host C, used to order work longest-first)."""
    rec = np.ascontiguousarray(rec, dtype=INST_DTYPE)
    out = np.zeros(len(rec), dtype=np.int64)
    st = settings or settings_from_globals()
    rc = _lib.lib().dgb_batch2d_count_steps(
        rec.ctypes.data_as(ctypes.POINTER(_lib.Inst2D)), len(rec), ctypes.byref(st),
        int(max_steps), out.ctypes.data_as(ctypes.POINTER(ctypes.c_long)))
    _lib.check(rc, "dgb_batch2d_count_steps")
    return out


class Batch2D:
    """Fixed grids and sample sizes; `run` integrates a batch of instances.

    pts_l: grid sizes (default grids, dadi/Numerics.py:215-233) used for the
    Richardson extrapolation; ns: sample sizes of the spectra.  The initial
    density is the equilibrium phi_1D split to 2-D (dadi/PhiManip.py:12-234),
    shared by every instance.
    """

    def __init__(self, pts_l=(80, 90, 100), ns=(40, 40), max_steps=10 ** 7, gam_placement=0):
        self.torch = _lib.require_cuda()
        torch = self.torch
        self.pts_l = list(pts_l)
        self.ns = tuple(ns)
        self.max_steps = int(max_steps)
        self.gam_placement = gam_placement
        self.threads = 0  # threads per CTA: 0 auto, 64, 96 or 128 (dgb_settings.threads)
        self.schedule_passes = 2
        self.launch_mode = "persistent"
        self.adjoint_ctas_per_sm = None  # None: sized to L2 (see adjoint)
        self.xxs = [numerics.default_grid(p) for p in self.pts_l]
        phi0 = [phimanip.phi_1D_to_2D(xx, phimanip.phi_1D(xx)) for xx in self.xxs]
        self.d_xx = _lib.to_device(torch, np.concatenate(self.xxs))
        self.d_phi0 = _lib.to_device(torch, np.concatenate([p.ravel() for p in phi0]))
        self.dx0s = np.array([xx[1] - xx[0] for xx in self.xxs])
        self.d_dx0 = _lib.to_device(torch, self.dx0s)
        self.Ls = (ctypes.c_int * len(self.pts_l))(*self.pts_l)
        self.x_l = [xx[1] for xx in self.xxs]
        self.mask = np.zeros((ns[0] + 1, ns[1] + 1), dtype=bool)
        self.mask.flat[0] = self.mask.flat[-1] = True

    def launches_per_integrate(self):
        """Kernel launches of ours in the last integrate(): the schedule
        passes (one within host bounds, or count and fill) and the
        integration, one launch per grid size with launch_mode "per_grid"."""
        per_grid = self.launch_mode == "per_grid" and len(set(self.pts_l)) > 1 \
            and not integration.current_settings()[2]
        return self.schedule_passes + (len(self.pts_l) if per_grid else 1)

    def schedule(self, d_rec, n, rec=None):
        """Device schedules of n dgb_inst2d records already on the device:
        (table, row_off, row_cnt, status).  With the host records `rec`, one
        fill pass into room reserved from host-side upper bounds on each
        schedule's rows (row_bounds); else (or when no useful bound exists)
        a count pass, a scan and a fill pass."""
        torch = self.torch
        lib = _lib.lib()
        st = settings_from_globals(self.gam_placement, self.threads)
        ng = len(self.pts_l)
        nsched = n * ng if st.use_old_timestep else n
        sh = _lib.stream_handle(torch)
        caps = row_bounds(rec, st, self.dx0s, self.max_steps) if rec is not None else None
        if caps is not None:
            self.schedule_passes = 1
            off_h = np.zeros(nsched, dtype=np.int64)
            np.cumsum(caps[:-1], out=off_h[1:])
            cnt = _lib.to_device(torch, caps.astype(np.int32), np.int32)
            off = _lib.to_device(torch, off_h, np.int64)
            table = torch.empty(max(int(caps.sum()), 1) * 11, dtype=torch.float64, device="cuda")
            status = torch.zeros(n, dtype=torch.int32, device="cuda")
            _lib.check(lib.dgb_sched2d(_lib.dptr(d_rec), n, ng, _lib.dptr(self.d_dx0),
                                       ctypes.byref(st), self.max_steps, 2, _lib.dptr(cnt),
                                       _lib.dptr(off), _lib.dptr(table), _lib.dptr(status), sh),
                       "dgb_sched2d(fill within bounds)")
            return table, off, cnt, status
        self.schedule_passes = 2
        cnt = torch.zeros(nsched, dtype=torch.int32, device="cuda")
        _lib.check(lib.dgb_sched2d(_lib.dptr(d_rec), n, ng, _lib.dptr(self.d_dx0), ctypes.byref(st),
                                   self.max_steps, 0, _lib.dptr(cnt), None, None, None, sh),
                   "dgb_sched2d(count)")
        ends = torch.cumsum(cnt.to(torch.int64), 0)
        total = int(_lib.to_host(torch, ends[-1:])[0])
        off = (ends - cnt.to(torch.int64)).contiguous()
        table = torch.empty(max(total, 1) * 11, dtype=torch.float64, device="cuda")
        status = torch.zeros(n, dtype=torch.int32, device="cuda")
        _lib.check(lib.dgb_sched2d(_lib.dptr(d_rec), n, ng, _lib.dptr(self.d_dx0), ctypes.byref(st),
                                   self.max_steps, 1, _lib.dptr(cnt), _lib.dptr(off),
                                   _lib.dptr(table), _lib.dptr(status), sh),
                   "dgb_sched2d(fill)")
        return table, off, cnt, status

    def integrate(self, rec, order=None, timer=None):
        """Run the integrations of dgb_inst2d records `rec` (host structured
        array).  Returns (list of per-grid phi tensors (n, L, L), status).
        timer: optional pair of CUDA events recorded around the integration
        kernel alone.  The launch follows self.launch_mode ("persistent": a
        device-sized grid pulling work items from a queue; "one_per_cta": one
        CTA per item) and self.gam_placement (0 auto, 1 shared memory, 2
        workspace), the knobs autotune.tune_batch2d chooses."""
        torch = self.torch
        if self.launch_mode == "per_grid" and len(set(self.pts_l)) > 1:
            out = self._integrate_per_grid(rec, timer)
            if out is not None:
                return out
        if self.launch_mode == "one_per_cta":
            n = len(rec)
            phi0s = [self.d_phi0[o:o + L * L].view(1, L, L).expand(n, L, L)
                     for o, L in zip(np.cumsum([0] + [L * L for L in self.pts_l[:-1]]),
                                     self.pts_l)]
            return self.integrate_from(rec, phi0s, one_per_cta=True, timer=timer)
        n = len(rec)
        ng = len(self.pts_l)
        st = settings_from_globals(self.gam_placement, self.threads)
        rec = np.ascontiguousarray(rec)
        d_rec = _lib.to_device(torch, rec.view(np.uint8), np.uint8)
        table, off, cnt, status = self.schedule(d_rec, n, rec)
        Lsq = torch.tensor([L * L for L in self.pts_l], dtype=torch.int64, device="cuda")
        if order is None:
            steps = cnt.to(torch.int64).view(n, -1)
            cost = (steps * Lsq[None, :]).reshape(-1)
            d_order = torch.argsort(-cost, stable=True).to(torch.int32)
        else:
            d_order = _lib.to_device(torch, order, np.int32)
        masks = (rec["frozen"].astype(np.int32) & 0xff) | ((rec["nomut"].astype(np.int32) & 0xff) << 8)
        d_masks = _lib.to_device(torch, masks, np.int32)
        total = sum(n * L * L for L in self.pts_l)
        d_out = torch.empty(total, dtype=torch.float64, device="cuda")
        nws = _lib.lib().dgb_workspace_bytes(1, 2, max(self.pts_l), n * ng)
        ws, nws = _lib.workspace(torch, nws)
        if timer is not None:
            timer[0].record()
        rc = _lib.lib().dgb_batch2d_integrate(
            _lib.dptr(d_masks), n, self.Ls, ng, _lib.dptr(self.d_xx), _lib.dptr(self.d_phi0),
            _lib.dptr(d_out), _lib.dptr(table), _lib.dptr(off), _lib.dptr(cnt), _lib.dptr(d_order),
            ctypes.byref(st), _lib.dptr(ws), nws, _lib.stream_handle(torch))
        if timer is not None:
            timer[1].record()
        _lib.check(rc, "dgb_batch2d_integrate")
        phis, o = [], 0
        for L in self.pts_l:
            phis.append(d_out[o:o + n * L * L].view(n, L, L))
            o += n * L * L
        return phis, status

    def _integrate_per_grid(self, rec, timer):
        """One persistent launch per grid size, each shaped for its own L
        (CTAs per SM, threads per CTA) instead of the largest, on side
        streams so that one launch's tail overlaps the next's start.  None
        when schedules are per grid (use_old_timestep)."""
        torch = self.torch
        lib = _lib.lib()
        st = settings_from_globals(self.gam_placement, self.threads)
        if st.use_old_timestep:
            return None
        n = len(rec)
        rec = np.ascontiguousarray(rec)
        d_rec = _lib.to_device(torch, rec.view(np.uint8), np.uint8)
        table, off, cnt, status = self.schedule(d_rec, n, rec)
        d_order = torch.argsort(-cnt.to(torch.int64), stable=True).to(torch.int32)
        masks = (rec["frozen"].astype(np.int32) & 0xff) | ((rec["nomut"].astype(np.int32) & 0xff) << 8)
        d_masks = _lib.to_device(torch, masks, np.int32)
        total = sum(n * L * L for L in self.pts_l)
        d_out = torch.empty(total, dtype=torch.float64, device="cuda")
        cur = torch.cuda.current_stream()
        if not hasattr(self, "_side"):
            self._side = [torch.cuda.Stream() for _ in self.pts_l]
        # workspaces first, so that allocation stays outside the timed launches
        wss = [_lib.workspace(torch, lib.dgb_workspace_bytes(1, 2, L, n)) for L in self.pts_l]
        fork = torch.cuda.Event()
        if timer is not None:
            timer[0].record()
        fork.record(cur)
        xo = po = oo = 0
        # largest grids first: their longest items set the end
        for g in sorted(range(len(self.pts_l)), key=lambda k: -self.pts_l[k]):
            L = self.pts_l[g]
            xo = sum(self.pts_l[:g])
            po = sum(l * l for l in self.pts_l[:g])
            oo = sum(n * l * l for l in self.pts_l[:g])
            side = self._side[g]
            with torch.cuda.stream(side):
                side.wait_event(fork)
                ws, nws = wss[g]
                Ls = (ctypes.c_int * 1)(L)
                _lib.check(lib.dgb_batch2d_integrate(
                    _lib.dptr(d_masks), n, Ls, 1, _lib.dptr(self.d_xx[xo:xo + L]),
                    _lib.dptr(self.d_phi0[po:po + L * L]), _lib.dptr(d_out[oo:oo + n * L * L]),
                    _lib.dptr(table), _lib.dptr(off), _lib.dptr(cnt), _lib.dptr(d_order),
                    ctypes.byref(st), _lib.dptr(ws), nws, _lib.stream_handle(torch)),
                    "dgb_batch2d_integrate")
            cur.wait_stream(side)
        if timer is not None:
            timer[1].record()
        phis, o = [], 0
        for L in self.pts_l:
            phis.append(d_out[o:o + n * L * L].view(n, L, L))
            o += n * L * L
        return phis, status

    def integrate_from(self, rec, phi0s, one_per_cta=False, timer=None):
        """integrate() with per-instance initial densities: phi0s[g] is an
        (n, L_g, L_g) float64 CUDA tensor for grid g (e.g. phi_1D with each
        instance's own selection, as the DFE models start from).  One launch
        over explicit work items (dgb_items2d_integrate): persistent, or with
        one_per_cta one CTA per item.  Returns (per-grid phi tensors (n, L,
        L), status)."""
        torch = self.torch
        lib = _lib.lib()
        n = len(rec)
        ng = len(self.pts_l)
        st = settings_from_globals(self.gam_placement, self.threads)
        rec = np.ascontiguousarray(rec)
        d_rec = _lib.to_device(torch, rec.view(np.uint8), np.uint8)
        table, off, cnt, status = self.schedule(d_rec, n, rec)
        blocks, o = [], 0
        for L in self.pts_l:
            blocks.append(o)
            o += n * L * L
        d_out = torch.empty(o, dtype=torch.float64, device="cuda")
        for g, L in enumerate(self.pts_l):
            assert tuple(phi0s[g].shape) == (n, L, L)
            d_out[blocks[g]:blocks[g] + n * L * L].view(n, L, L).copy_(phi0s[g])
        masks = (rec["frozen"].astype(np.int32) & 0xff) | ((rec["nomut"].astype(np.int32) & 0xff) << 8)
        items = np.zeros((n, ng), dtype=ITEM2D_DTYPE)
        xo = np.cumsum([0] + self.pts_l[:-1])
        idx = np.arange(n, dtype=np.int64)
        for g, L in enumerate(self.pts_l):
            items["L"][:, g] = L
            items["masks"][:, g] = masks
            items["xx_off"][:, g] = xo[g]
            items["out_off"][:, g] = blocks[g] + idx * L * L
            items["sched"][:, g] = idx * ng + g if st.use_old_timestep else idx
        Lsq = torch.tensor([L * L for L in self.pts_l], dtype=torch.int64, device="cuda")
        steps = cnt.to(torch.int64).view(n, -1)
        cost = (steps * Lsq[None, :]).reshape(-1)
        d_order = torch.argsort(-cost, stable=True).to(torch.int32)
        d_items = _lib.to_device(torch, items.reshape(-1).view(np.uint8), np.uint8)
        Lmax = max(self.pts_l)
        if one_per_cta:
            nws = lib.dgb_workspace_bytes(3, 2, Lmax, n * ng)
        else:
            nws = lib.dgb_workspace_bytes(1, 2, Lmax, n * ng)
        ws, nws = _lib.workspace(torch, nws)
        if timer is not None:
            timer[0].record()
        rc = lib.dgb_items2d_integrate(
            _lib.dptr(d_items), n * ng, Lmax, _lib.dptr(self.d_xx), _lib.dptr(d_out),
            _lib.dptr(table), _lib.dptr(off), _lib.dptr(cnt), _lib.dptr(d_order),
            ctypes.byref(st), int(bool(one_per_cta)), _lib.dptr(ws), nws,
            _lib.stream_handle(torch))
        if timer is not None:
            timer[1].record()
        _lib.check(rc, "dgb_items2d_integrate")
        phis = [d_out[b:b + n * L * L].view(n, L, L) for b, L in zip(blocks, self.pts_l)]
        return phis, status

    def loglik_and_grad(self, params, data, scale=1.0, ckpt_every=None, seeds=None, rec=None,
                        mask=None, multinom=False, trajectory=None):
        """Poisson log-likelihood of scale * (extrapolated IM spectrum) against
        data for each parameter row (or its multinomial form, see loglik), and
        its gradient with respect to (s, nu1, nu2, T, m12, m21) by the
        discrete adjoint.  Returns CUDA tensors (ll (n,), grad (n, 6),
        status (n,))."""
        ll, ctx = self.forward_for_adjoint(params, data, scale, ckpt_every, seeds, rec,
                                           mask=mask, multinom=multinom)
        grad = self.adjoint(ctx, self.torch.ones_like(ll), trajectory=trajectory)
        return ll.detach(), grad, ctx["status"]

    def forward_for_adjoint(self, params, data, scale=1.0, ckpt_every=None, seeds=None,
                            rec=None, tail_per_set=False, mask=None, multinom=False):
        """Forward pass that keeps what the adjoint needs: schedules,
        derivative rows, checkpoints and the differentiable tail (from_phi,
        extrapolation, likelihood) as a torch graph.  tail_per_set evaluates
        the tail one parameter set at a time, so each set's spectrum,
        likelihood and gradient are bitwise independent of the other sets in
        the batch (batched matrix products may order sums by batch size)."""
        torch = self.torch
        lib = _lib.lib()
        if rec is None:
            rec = im_instances(params)
        rec = np.ascontiguousarray(rec)
        n = len(rec)
        ng = len(self.pts_l)
        st = settings_from_globals(self.gam_placement, self.threads)
        if st.use_delj_trick:
            raise NotImplementedError("the adjoint does not support the delj trick")
        sh = _lib.stream_handle(torch)
        d_rec = _lib.to_device(torch, rec.view(np.uint8), np.uint8)
        table, off, cnt, status = self.schedule(d_rec, n, rec)
        seeds = im_seeds(n) if seeds is None else np.ascontiguousarray(seeds)
        d_seed = _lib.to_device(torch, seeds.view(np.uint8), np.uint8)
        drows = torch.empty(max(int(table.numel() // 11), 1) * 60, dtype=torch.float64,
                            device="cuda")
        # the derivative rows are for the adjoint only: their walk (serial
        # per schedule, like the value walk) runs on a side stream beside
        # the forward integration, joined before this returns
        main = torch.cuda.current_stream()
        dual = torch.cuda.Stream()
        dual.wait_stream(main)
        with torch.cuda.stream(dual):
            _lib.check(lib.dgb_sched2d_deriv(_lib.dptr(d_rec), _lib.dptr(d_seed), n, ng,
                                             _lib.dptr(self.d_dx0), ctypes.byref(st),
                                             _lib.dptr(cnt), _lib.dptr(off), _lib.dptr(drows),
                                             _lib.stream_handle(torch)), "dgb_sched2d_deriv")
        for t in (d_rec, d_seed, cnt, off, drows):
            t.record_stream(dual)
        steps = cnt.to(torch.int64).view(n, -1)
        Lsq = torch.tensor([L * L for L in self.pts_l], dtype=torch.int64, device="cuda")
        cost = (steps * Lsq[None, :]).reshape(-1)
        d_order = torch.argsort(-cost, stable=True).to(torch.int32)
        smax = int(_lib.to_host(torch, steps.max().reshape(1))[0])
        C = int(ckpt_every) if ckpt_every else max(8, min(256, int(np.ceil(np.sqrt(max(smax, 1))))))
        per_item = ((steps + C - 1) // C).expand(n, ng) * Lsq[None, :]
        ends = torch.cumsum(per_item.reshape(-1), 0)
        ck_off = (ends - per_item.reshape(-1)).contiguous()
        ckpt = torch.empty(max(int(_lib.to_host(torch, ends[-1:])[0]), 1), dtype=torch.float64,
                           device="cuda")
        masks = (rec["frozen"].astype(np.int32) & 0xff) | ((rec["nomut"].astype(np.int32) & 0xff) << 8)
        d_masks = _lib.to_device(torch, masks, np.int32)
        total = sum(n * L * L for L in self.pts_l)
        d_out = torch.empty(total, dtype=torch.float64, device="cuda")
        nws = lib.dgb_workspace_bytes(1, 2, max(self.pts_l), n * ng)
        ws, nws = _lib.workspace(torch, nws)
        common = (_lib.dptr(d_masks), n, self.Ls, ng, _lib.dptr(self.d_xx),
                  _lib.dptr(self.d_phi0), _lib.dptr(d_out), _lib.dptr(table), _lib.dptr(off),
                  _lib.dptr(cnt))
        longest = self._cluster_work(cnt, masks, st) if self.cluster_forward else None
        if longest is None:
            _lib.check(lib.dgb_batch2d_integrate_ckpt(
                *common, _lib.dptr(d_order), ctypes.byref(st), _lib.dptr(ckpt), _lib.dptr(ck_off),
                C, _lib.dptr(ws), nws, sh), "dgb_batch2d_integrate_ckpt")
        else:
            self._forward_split(longest, common, d_out, ckpt, ck_off, C, table, off, cnt, st, ws,
                                nws)
        phis, o = [], 0
        for L in self.pts_l:
            phis.append(d_out[o:o + n * L * L].view(n, L, L).detach().requires_grad_(True))
            o += n * L * L
        d = data if torch.is_tensor(data) else _lib.to_device(torch, data)
        with torch.enable_grad():
            if tail_per_set:
                fss, lls = [], []
                for i in range(n):
                    fs_i = self.extrapolate(self.spectra([p[i:i + 1] for p in phis]))
                    fss.append(fs_i)
                    lls.append(self.loglik(fs_i, d, scale, mask, multinom))
                fs = torch.cat(fss)
                ll = torch.cat(lls)
            else:
                fs = self.extrapolate(self.spectra(phis))
                ll = self.loglik(fs, d, scale, mask, multinom)
        main.wait_stream(dual)
        ctx = dict(phis=phis, ll=ll, fs=fs.detach(), table=table, off=off, cnt=cnt, drows=drows, ckpt=ckpt,
                   ck_off=ck_off, C=C, masks=d_masks, order=d_order, status=status, n=n, st=st)
        return ll, ctx

    #: Run the forward of a few integrations on thread-block clusters (8
    #: CTAs each; see _cluster_work).
    cluster_forward = True

    def _cluster_work(self, cnt, masks, st):
        """The work items to run on clusters in the forward: all of them when
        each can have a cluster of 8 CTAs (a few integrations, each bound by
        one SM's FP64 pipe on one CTA: the longest seed-0 request's forward
        3.48 -> 2.14 s), else none -- a larger batch has a tail of long items
        too many for clusters, and SMs reserved for a few of them slow the
        rest (256 sets: 3.09 -> 3.36 s with its 9 longest items on
        clusters).  Grids of 24-128 points, default delta_j."""
        torch = self.torch
        if st.use_delj_trick or not all(24 <= L <= 128 for L in self.pts_l):
            return None
        ng = len(self.pts_l)
        steps = _lib.to_host(torch, cnt).astype(np.int64)
        steps = steps.reshape(-1, ng) if st.use_old_timestep else \
            np.repeat(steps.reshape(-1, 1), ng, axis=1)
        n = steps.shape[0]
        nsm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        if n * ng * 8 > nsm:
            return None
        Lsq = np.array([L * L for L in self.pts_l], dtype=np.int64)
        order = np.argsort(-(steps * Lsq[None, :]).reshape(-1), kind="stable")
        return dict(order=order.astype(np.int32), pick=[int(w) for w in order], steps=steps,
                    n=n, masks=np.asarray(masks, dtype=np.int32))

    def _forward_split(self, longest, common, d_out, ckpt, ck_off, C, table, off, cnt, st, ws,
                       nws):
        """The forward with checkpoints with its longest work items on
        clusters (dgb_items2d_integrate_cluster, the current stream) and the
        rest through dgb_batch2d_integrate_ckpt_part on a side stream,
        leaving the clusters their SMs."""
        torch = self.torch
        lib = _lib.lib()
        ng = len(self.pts_l)
        n, pick, order = longest["n"], longest["pick"], longest["order"]
        xo = np.concatenate([[0], np.cumsum(self.pts_l)[:-1]]).astype(np.int64)
        go = np.concatenate([[0], np.cumsum([n * L * L for L in self.pts_l])[:-1]])
        po = np.concatenate([[0], np.cumsum([L * L for L in self.pts_l])[:-1]])
        items = np.zeros(len(pick), dtype=ITEM2D_DTYPE)
        ck_h = _lib.to_host(torch, ck_off)
        for k, w in enumerate(pick):
            inst, g = divmod(w, ng)
            L = self.pts_l[g]
            items["L"][k], items["xx_off"][k] = L, xo[g]
            items["out_off"][k] = go[g] + inst * L * L
            items["sched"][k] = w if st.use_old_timestep else inst
            items["masks"][k] = longest["masks"][inst]
            # the initial density, integrated in place in its output slot
            d_out[items["out_off"][k]:items["out_off"][k] + L * L].copy_(
                self.d_phi0[po[g]:po[g] + L * L])
        d_items = _lib.to_device(torch, items.view(np.uint8), np.uint8)
        d_ckoff = _lib.to_device(torch, ck_h[pick].astype(np.int64), np.int64)
        picked = set(pick)
        rest = np.array([w for w in order if w not in picked], dtype=np.int32)
        d_rest = _lib.to_device(torch, rest, np.int32) if len(rest) else None
        main = torch.cuda.current_stream()
        side = torch.cuda.Stream()
        side.wait_stream(main)
        Ls = [self.pts_l[w % ng] for w in pick]
        _lib.check(lib.dgb_items2d_integrate_cluster(
            _lib.dptr(d_items), len(pick), min(Ls), max(Ls), _lib.dptr(self.d_xx),
            _lib.dptr(d_out), _lib.dptr(table), _lib.dptr(off), _lib.dptr(cnt), 8,
            _lib.dptr(ckpt), _lib.dptr(d_ckoff), C, _lib.stream_handle(torch)),
            "dgb_items2d_integrate_cluster")
        if d_rest is not None:
            with torch.cuda.stream(side):
                _lib.check(lib.dgb_batch2d_integrate_ckpt_part(
                    *common, _lib.dptr(d_rest), len(rest), 8 * len(pick), ctypes.byref(st),
                    _lib.dptr(ckpt), _lib.dptr(ck_off), C, _lib.dptr(ws), nws,
                    _lib.stream_handle(torch)), "dgb_batch2d_integrate_ckpt_part")
            main.wait_stream(side)
            for t in (d_rest, ws):
                t.record_stream(side)
        self._split_keep = (d_items, d_ckoff, d_rest)

    #: Largest trajectory (bytes) the adjoint stores so that every checkpoint
    #: segment is recomputed at once (dgb_adjoint2d_traj); beyond it the
    #: longest items that fit are walked from a stored trajectory and the
    #: rest recompute their segments in turn (the hybrid).  256 sets at pts
    #: 100/110/120: 7.13 s at 24 GB, 6.16 s at 48, 5.80 s at 64, 5.84 s at 80.
    traj_budget = 64 << 30

    def _traj_limit(self):
        """traj_budget, but at most half the device memory free now (the
        driver's free bytes plus what torch's allocator holds unused)."""
        torch = self.torch
        free, _ = torch.cuda.mem_get_info()
        idle = torch.cuda.memory_reserved() - torch.cuda.memory_allocated()
        return min(self.traj_budget, (free + idle) // 2)

    def trajectory_bytes(self, ctx):
        """Bytes of the adjoint's full trajectory for a forward context:
        per work item (2 n + 1) L^2 doubles (every density and x-sweep
        output of its n steps)."""
        steps = self._work_steps(ctx)
        Lsq = np.array([L * L for L in self.pts_l], dtype=np.int64)
        return int(8 * np.sum((2 * steps + 1) * Lsq[None, :]))

    def _work_steps(self, ctx):
        """Steps of each (instance, grid) work item, (n, ngrids), host."""
        n, ng = ctx["n"], len(self.pts_l)
        cnt = _lib.to_host(self.torch, ctx["cnt"]).astype(np.int64)
        if ctx["st"].use_old_timestep:      # one schedule per work item
            return cnt.reshape(n, ng)
        return np.repeat(cnt.reshape(n, 1), ng, axis=1)

    def adjoint(self, ctx, grad_ll, trajectory=None):
        """d(sum_i grad_ll[i] * ll_i)/d(params) by the discrete adjoint: (n, 6).
        trajectory: recompute every checkpoint segment at once into a stored
        trajectory first (True), each work item's segments in turn (False),
        or (None) the first for as many of the longest work items as
        traj_budget holds -- all of them when it holds the whole trajectory
        -- and the second for the rest, the two on their own streams at once:
        the longest items' serial backward walks lose their recomputation,
        which bounds a batch with a few long integrations.  The gradients are
        the same bit for bit whichever way."""
        torch = self.torch
        lib = _lib.lib()
        phis = ctx["phis"]
        lams = torch.autograd.grad(ctx["ll"], phis, grad_outputs=grad_ll, allow_unused=True)
        lam = torch.cat([(l if l is not None else torch.zeros_like(p)).reshape(-1)
                         for l, p in zip(lams, phis)]).contiguous()
        n = ctx["n"]
        ng = len(self.pts_l)
        part = torch.empty(n, ng, 6, dtype=torch.float64, device="cuda")
        C = ctx["C"]
        Lmax = max(self.pts_l)
        props = torch.cuda.get_device_properties(torch.cuda.current_device())
        nsm = props.multi_processor_count
        per_sm = self.adjoint_ctas_per_sm
        if per_sm is None:
            # each CTA streams ~5 L^2 arrays per step backwards through L2
            # (segment state, chi, the next state, lambda, gam): keep the CTAs'
            # per-step working set within 3/4 of L2.  Measured at pts
            # 100/110/120 (256 sets): 1 CTA per SM 11.9 s, 2: 16.9 s, 3: 21.8 s.
            l2 = getattr(props, "L2_cache_size", 0) or (96 << 20)
            per_sm = int(0.75 * l2 // (nsm * 5 * Lmax * Lmax * 8))
            per_sm = max(1, min(4, per_sm))
        nblocks = min(n * ng, nsm * per_sm)
        st = ctx["st"]
        common = (_lib.dptr(ctx["masks"]), n, self.Ls, ng, _lib.dptr(self.d_xx),
                  _lib.dptr(ctx["table"]), _lib.dptr(ctx["drows"]), _lib.dptr(ctx["off"]),
                  _lib.dptr(ctx["cnt"]), _lib.dptr(ctx["ckpt"]), _lib.dptr(ctx["ck_off"]), C)
        if trajectory is None:
            if self.trajectory_bytes(ctx) <= self._traj_limit():
                trajectory = True
            else:
                self._adjoint_hybrid(ctx, lam, part, common, nsm, per_sm, Lmax)
                trajectory = "hybrid"
        if trajectory == "hybrid":
            pass
        elif trajectory:
            ctas = self._cluster_adjoint_ctas(ctx, nsm)
            steps = self._work_steps(ctx).reshape(-1)
            Lsq = np.tile(np.array([L * L for L in self.pts_l], dtype=np.int64), n)
            size = (2 * steps + 1) * Lsq
            t_off = np.zeros(n * ng, dtype=np.int64)
            np.cumsum(size[:-1], out=t_off[1:])
            seg_off = np.zeros(n * ng + 1, dtype=np.int64)
            np.cumsum((steps + C - 1) // C, out=seg_off[1:])
            traj = torch.empty(max(int(size.sum()), 1), dtype=torch.float64, device="cuda")
            d_toff = _lib.to_device(torch, t_off, np.int64)
            d_soff = _lib.to_device(torch, seg_off, np.int64)
            ws, nws = _lib.workspace(torch, lib.dgb_adjoint2d_traj_ws_bytes(
                Lmax, max(nblocks, 2 * nsm)))
            if ctas:
                _lib.check(lib.dgb_adjoint2d_part(
                    *common, _lib.dptr(traj), _lib.dptr(d_toff), _lib.dptr(d_soff),
                    _lib.dptr(lam), _lib.dptr(part), _lib.dptr(ctx["order"]), n * ng, 0, ctas,
                    ctypes.byref(st), _lib.dptr(ws), nws, _lib.stream_handle(torch)),
                    "dgb_adjoint2d_part(cluster)")
            else:
                _lib.check(lib.dgb_adjoint2d_traj(
                    *common, _lib.dptr(traj), _lib.dptr(d_toff), _lib.dptr(d_soff),
                    _lib.dptr(lam), _lib.dptr(part), _lib.dptr(ctx["order"]), ctypes.byref(st),
                    _lib.dptr(ws), nws, _lib.stream_handle(torch)), "dgb_adjoint2d_traj")
        else:
            per_cta = lib.dgb_adjoint2d_scratch_bytes(Lmax, C, 1)
            ws, nws = _lib.workspace(torch, 256 + per_cta * nblocks)
            _lib.check(lib.dgb_adjoint2d(
                *common, _lib.dptr(lam), _lib.dptr(part), _lib.dptr(ctx["order"]),
                ctypes.byref(st), _lib.dptr(ws), nws, _lib.stream_handle(torch)),
                "dgb_adjoint2d")
        grad = part[:, 0].clone()
        for gi in range(1, ng):
            grad += part[:, gi]
        return grad

    #: CTAs of the thread-block cluster that walks each work item's adjoint
    #: in trajectory mode when there are few items (2, 4, 8 or 16; 0: one
    #: CTA per item always; see _cluster_adjoint_ctas).
    cluster_adjoint = 8

    def _cluster_adjoint_ctas(self, ctx, nsm):
        """CTAs per work item of the trajectory-mode backward walk:
        cluster_adjoint (a cluster per item, dgb_adjoint2d_part) when every
        item can have its cluster at once and every grid has 3-16 rows per
        CTA within 24-128 points, else 0 (one CTA per item).  A single
        item's walk on one CTA is bound by one SM's FP64 pipe."""
        c = self.cluster_adjoint
        if not c or ctx["st"].use_delj_trick:
            return 0
        if not all(max(24, 3 * c) <= L <= min(128, 16 * c) for L in self.pts_l):
            return 0
        return c if ctx["n"] * len(self.pts_l) * c <= nsm else 0

    #: In the hybrid adjoint, walk the longest (at most this many)
    #: trajectory-mode items on clusters of cluster_adjoint CTAs, within a
    #: quarter of the SMs (0: none).  Off by default: the hybrid's bound is
    #: the segment-mode walk of the other items, which the clusters' SMs
    #: slow (256 sets at pts 100/110/120: 5.81 s with none, 6.32 s with 2,
    #: 7.15 s with 4).
    hybrid_cluster_items = 0

    def _adjoint_hybrid(self, ctx, lam, part, common, nsm, per_sm, Lmax):
        """The longest work items (while their trajectory fits traj_budget)
        in trajectory mode -- the longest hybrid_cluster_items of them on
        clusters on the current stream, the others one CTA each on a side
        stream -- and the rest with per-CTA segment recomputation on another
        side stream on the remaining CTAs (dgb_adjoint2d_part up to three
        times, each trajectory call recomputing its own items' segments)."""
        torch = self.torch
        lib = _lib.lib()
        n, ng, C, st = ctx["n"], len(self.pts_l), ctx["C"], ctx["st"]
        steps = self._work_steps(ctx).reshape(-1)
        Lsq = np.tile(np.array([L * L for L in self.pts_l], dtype=np.int64), n)
        c = self.cluster_adjoint
        if not c or not all(max(24, 3 * c) <= L <= min(128, 16 * c) for L in self.pts_l):
            c = 0
        order, size, k, j, rest = hybrid_plan(steps, Lsq, self._traj_limit(), c,
                                              self.hybrid_cluster_items, nsm, per_sm)
        tset = order[:k]
        t_off = np.zeros(n * ng, dtype=np.int64)
        t_off[tset] = np.concatenate([[0], np.cumsum(size[tset] // 8)[:-1]])
        traj = torch.empty(max(int(size[tset].sum() // 8), 1), dtype=torch.float64,
                           device="cuda")
        d_toff = _lib.to_device(torch, t_off, np.int64)
        d_order = _lib.to_device(torch, order, np.int32)
        keep = [traj, d_toff, d_order]
        # (first, count, CTAs, cluster) of each trajectory-mode call
        calls = [(0, j, j, c), (j, k - j, k - j, 0)]
        ws_s, nws_s = _lib.workspace(torch, 256 + lib.dgb_adjoint2d_scratch_bytes(Lmax, C, 1)
                                     * rest)
        keep.append(ws_s)
        # every upload on the current stream before the side streams wait on it
        args = []
        for first, cnt, ctas, cl in calls:
            if cnt < 1:
                args.append(None)
                continue
            nseg = np.zeros(n * ng, dtype=np.int64)
            ids = order[first:first + cnt]
            nseg[ids] = (steps[ids] + C - 1) // C
            seg_off = np.zeros(n * ng + 1, dtype=np.int64)
            np.cumsum(nseg, out=seg_off[1:])
            d_soff = _lib.to_device(torch, seg_off, np.int64)
            ws_t, nws_t = _lib.workspace(torch, lib.dgb_adjoint2d_traj_ws_bytes(Lmax, 2 * nsm))
            keep += [d_soff, ws_t]
            args.append((d_soff, ws_t, nws_t))
        main = torch.cuda.current_stream()
        sides = [torch.cuda.Stream(), torch.cuda.Stream()]
        for sd in sides:
            sd.wait_stream(main)
        for (first, cnt, ctas, cl), a, strm in zip(calls, args, (main, sides[0])):
            if a is None:
                continue
            d_soff, ws_t, nws_t = a
            with torch.cuda.stream(strm):
                _lib.check(lib.dgb_adjoint2d_part(
                    *common, _lib.dptr(traj), _lib.dptr(d_toff), _lib.dptr(d_soff),
                    _lib.dptr(lam), _lib.dptr(part), _lib.dptr(d_order[first:]), cnt, ctas, cl,
                    ctypes.byref(st), _lib.dptr(ws_t), nws_t, _lib.stream_handle(torch)),
                    "dgb_adjoint2d_part(trajectory)")
        with torch.cuda.stream(sides[1]):
            _lib.check(lib.dgb_adjoint2d_part(
                *common, None, None, None, _lib.dptr(lam), _lib.dptr(part),
                _lib.dptr(d_order[k:]), len(order) - k, rest, 0, ctypes.byref(st),
                _lib.dptr(ws_s), nws_s, _lib.stream_handle(torch)), "dgb_adjoint2d_part")
        for sd in sides:
            main.wait_stream(sd)
            for t in keep:
                t.record_stream(sd)

    def spectra(self, phis):
        """Per-grid raw spectra (n, n1+1, n2+1) on the device."""
        return [spectrum.from_phi_2D_batch(self.torch, p, self.ns[0], self.ns[1], xx)
                for p, xx in zip(phis, self.xxs)]

    def extrapolate(self, fs_l, fail_mag=10):
        """Richardson extrapolation with the fail_mag guard
        (dadi/Numerics.py:425-464) on the device."""
        torch = self.torch
        x = self.x_l
        if len(fs_l) == 1:
            return fs_l[0].clone()
        if len(fs_l) == 2:
            ex = numerics.linear_extrap(fs_l, x)
        else:
            ex = numerics.quadratic_extrap(fs_l, x)
        best = fs_l[int(np.argmin(x))]
        failed = torch.abs(torch.log10(ex / best)) > fail_mag
        return torch.where(failed, best, ex)

    def loglik(self, fs, data, scale=1.0, mask=None, multinom=False):
        """Poisson log-likelihood of scale*fs against data over entries
        unmasked (the corners, or `mask`, a boolean array: True = masked) with
        positive model (dadi/Inference.py:466-509); shape (n,).  multinom:
        the multinomial form, scale = sum(data)/sum(fs) over unmasked entries
        for each spectrum (ll_multinom, :559-575 with optimal_sfs_scaling,
        :668-685), kept inside the autograd graph."""
        torch = self.torch
        d = data if torch.is_tensor(data) else _lib.to_device(torch, data)
        m = self.mask if mask is None else (np.asarray(mask, dtype=bool) | self.mask)
        um = ~torch.from_numpy(m).to(fs.device)
        if multinom:
            scale = (d * um).sum() / (fs * um).sum(dim=(1, 2))
            scale = scale[:, None, None]
        model = scale * fs
        ok = um & (model > 0)
        term = -model + d * torch.log(torch.where(ok, model, torch.ones_like(model))) \
            - torch.lgamma(d + 1.0)
        return torch.where(ok, term, torch.zeros_like(term)).sum(dim=(1, 2))

    def spectra_ll(self, phis, data=None, scale=1.0, multinom=False):
        """The device epilogue (dgb_from_phi2d + dgb_extrap_ll, two launches
        for the whole batch): extrapolated spectra (n, n1+1, n2+1) and, with
        data, Poisson log-likelihoods (n,); CUDA tensors.  multinom: also the
        multinomial log-likelihoods (n,), returned third."""
        torch = self.torch
        d = None
        if data is not None:
            d = data if torch.is_tensor(data) else _lib.to_device(torch, data)
            d = d.to(torch.float64).contiguous()
        res = epilogue.spectra_2d_batch(torch, [p.contiguous() for p in phis], self.xxs,
                                        self.ns, d, scale, multinom=multinom and d is not None)
        if multinom and d is None:
            return res[0], None, None
        return res

    def run(self, params, data=None, scale=1.0):
        """IM parameter rows -> (extrapolated spectra (n, n1+1, n2+1), ll or
        None, status), all CUDA tensors."""
        rec = im_instances(params)
        phis, status = self.integrate(rec)
        fs, ll = self.spectra_ll(phis, data, scale)
        return fs, ll, status


class IMLogLik:
    """torch.autograd.Function wrapper: ll = IMLogLik.apply(engine, params,
    data, scale) with params a (n, 6) float64 tensor of IM parameters
    (s, nu1, nu2, T, m12, m21); ll.backward() runs the discrete adjoint."""

    @staticmethod
    def _function():
        import torch

        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, params, engine, data, scale):
                p = params.detach().cpu().numpy()
                ll, actx = engine.forward_for_adjoint(p, data, scale)
                ctx.engine = engine
                ctx.actx = actx
                ctx.dev = params.device
                return ll.detach()

            @staticmethod
            def backward(ctx, grad_ll):
                g = ctx.engine.adjoint(ctx.actx, grad_ll.contiguous())
                return g.to(ctx.dev), None, None, None
        return _Fn

    @classmethod
    def apply(cls, engine, params, data, scale=1.0):
        return cls._function().apply(params, engine, data, scale)
