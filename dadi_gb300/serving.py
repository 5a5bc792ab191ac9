"""Continuous-batching request server for spectrum (and gradient) requests.

Requests arrive over time; each asks for the extrapolated spectrum of a
model at its own grid sizes and sample sizes, optionally its Poisson
log-likelihood against observed data and, for 2-D IM requests, its gradient.

Scheduling:

* Admission by HBM footprint: a request's device bytes (its densities on
  every grid, its schedule rows, checkpoints if it wants a gradient) are
  reserved from a budget when it is admitted and released when its results
  are read back; requests wait while the budget is exhausted.
* 2-D requests (IM, and IM with selection as used for DFE caches,
  dadi/DFE/DemogSelModels.py:162-197) are batched into *waves*: one wave is
  one persistent launch over an explicit work-item list
  (dgb_items2d_integrate), so requests with different grid sizes and sample
  sizes share a launch.  Each wave runs on its own CUDA stream; a wave formed
  while earlier ones are still running is launched immediately, and its CTAs
  take SMs as the earlier waves' CTAs retire, so arrivals join work already
  on the device instead of waiting for it to finish.  Densities stay on the
  device from the initial condition to the spectrum; only spectra,
  likelihoods and gradients come back.
* 3-D and 4-D requests, and gradient requests, run on worker threads with
  their own streams, overlapping the waves.

Every request records arrival, admission and completion times; latency is
completion minus arrival.
"""
import ctypes
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

from . import _lib, batch, integration, models, numerics, phimanip, spectrum

ITEM_DTYPE = np.dtype([("L", "i4"), ("masks", "i4"), ("xx_off", "i8"), ("out_off", "i8"),
                       ("sched", "i8")])


@dataclass
class Request:
    """kind: "im" (Demographics2D.IM params), "im_sel" (IM params + gamma1,
    gamma2), "growth3" (models.growth3 params), "four" (models.four_split
    params)."""
    rid: int
    kind: str
    params: tuple
    pts_l: tuple
    ns: tuple
    data: object = None
    scale: float = 1.0
    want_grad: bool = False
    arrival: float = 0.0
    fs: object = None
    ll: object = None
    grad: object = None
    status: int = 0
    t_admit: float = None
    t_done: float = None
    error: str = None

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival


def _inst_record(req):
    if req.kind == "im":
        return batch.im_instances(np.asarray(req.params, dtype=np.float64)[None, :])[0]
    if req.kind == "im_sel":
        p = np.asarray(req.params, dtype=np.float64)
        rec = batch.im_instances(p[None, :6])[0]
        rec["gamma"][0] = batch._pf_array(_lib.PF_CONST, np.array([p[6]]))[0]
        rec["gamma"][1] = batch._pf_array(_lib.PF_CONST, np.array([p[7]]))[0]
        return rec
    raise ValueError(req.kind)


class Server:
    """hbm_budget: bytes of device memory requests may hold at once;
    max_wave: most requests per 2-D wave; workers: threads for 3-D/4-D and
    gradient requests."""

    def __init__(self, hbm_budget=16 << 30, max_wave=512, workers=3, max_inflight=4):
        self.torch = _lib.require_cuda()
        self.budget = int(hbm_budget)
        self.max_wave = max_wave
        self.max_inflight = max_inflight
        self.workers = workers
        self._used = 0
        self._lock = threading.Lock()
        self._grids = {}
        self._phi0 = {}
        self._engines = {}

    # ----------------------------------------------------------- resources

    def footprint(self, req):
        """Device bytes the request holds while admitted."""
        P = 2 if req.kind in ("im", "im_sel") else (3 if req.kind == "growth3" else 4)
        dens = sum(8 * L ** P for L in req.pts_l)
        steps = self._steps(req)
        rows = steps * 11 * 8
        extra = 0
        if req.want_grad:
            C = max(8, int(np.ceil(np.sqrt(max(steps, 1)))))
            extra = sum(8 * L * L * ((steps + C - 1) // C) for L in req.pts_l) + steps * 60 * 8
        return dens * 2 + rows + extra

    def _steps(self, req):
        if getattr(req, "_steps", None) is None:
            if req.kind in ("im", "im_sel"):
                req._steps = int(batch.count_steps(_inst_record(req)[None])[0])
            else:
                req._steps = 2000
        return req._steps

    def _grid(self, L):
        torch = self.torch
        if L not in self._grids:
            xx = numerics.default_grid(L)
            self._grids[L] = (xx, torch.from_numpy(xx).cuda())
        return self._grids[L]

    def _initial(self, L, gamma1):
        """phi_1D(gamma1) split to 2-D (dadi/PhiManip.py:12-234), cached."""
        key = (L, float(gamma1))
        if key not in self._phi0:
            xx = self._grid(L)[0]
            phi = phimanip.phi_1D_to_2D(xx, phimanip.phi_1D(xx, gamma=gamma1))
            self._phi0[key] = self.torch.from_numpy(phi.ravel()).cuda()
        return self._phi0[key]

    # --------------------------------------------------------------- waves

    def _launch_wave(self, reqs, stream):
        """Enqueue one 2-D wave on `stream`; returns a finisher."""
        torch = self.torch
        lib = _lib.lib()
        n = len(reqs)
        with torch.cuda.stream(stream):
            sh = _lib.stream_handle(torch)
            recs = np.stack([_inst_record(r) for r in reqs])
            Ls = sorted({L for r in reqs for L in r.pts_l})
            xx_off, xs, o = {}, [], 0
            for L in Ls:
                xx_off[L] = o
                xs.append(self._grid(L)[1])
                o += L
            d_xx = torch.cat(xs)
            items, phi0s, off = [], [], 0
            slots = []
            for k, r in enumerate(reqs):
                g1 = r.params[6] if r.kind == "im_sel" else 0.0
                sl = []
                for L in r.pts_l:
                    items.append((L, 0, xx_off[L], off, k))
                    phi0s.append(self._initial(L, g1))
                    sl.append((off, L))
                    off += L * L
                slots.append(sl)
            d_phi = torch.cat(phi0s)
            d_items = torch.from_numpy(np.array(items, dtype=ITEM_DTYPE).view(np.uint8)).cuda()
            st = batch.settings_from_globals()
            table_h, roff_h, cnt_h, status_h = host_schedules(recs, st, self._grid(Ls[0])[0][1])
            table = torch.from_numpy(table_h).cuda()
            roff = torch.from_numpy(roff_h).cuda()
            cnt = torch.from_numpy(cnt_h).cuda()
            sched = torch.tensor([it[4] for it in items], dtype=torch.int64, device="cuda")
            Lsq = torch.tensor([it[0] ** 2 for it in items], dtype=torch.int64, device="cuda")
            order = torch.argsort(-(cnt.to(torch.int64)[sched] * Lsq), stable=True).to(torch.int32)
            Lmax = max(Ls)
            ws, nws = _lib.workspace(torch, lib.dgb_workspace_bytes(1, 2, Lmax, len(items)))
            _lib.check(lib.dgb_items2d_integrate(
                _lib.dptr(d_items), len(items), Lmax, _lib.dptr(d_xx), _lib.dptr(d_phi),
                _lib.dptr(table), _lib.dptr(roff), _lib.dptr(cnt), _lib.dptr(order),
                ctypes.byref(st), _lib.dptr(ws), nws, sh), "dgb_items2d_integrate")
            # spectra per (request): from_phi on each grid, extrapolate, ll
            outs = []
            for k, r in enumerate(reqs):
                fs_l = []
                for (o2, L) in slots[k]:
                    phi = d_phi[o2:o2 + L * L].view(1, L, L)
                    fs_l.append(spectrum.from_phi_2D_batch(torch, phi, r.ns[0], r.ns[1],
                                                           self._grid(L)[0])[0])
                x_l = [self._grid(L)[0][1] for L in r.pts_l]
                fs = _extrap_torch(torch, fs_l, x_l)
                ll = None
                if r.data is not None:
                    ll = _loglik_torch(torch, fs, r.data, r.scale)
                outs.append((fs, ll))
            done = torch.cuda.Event()
            done.record(stream)
        keep = (d_phi, d_items, table, ws, order, cnt, roff)

        def finish():
            done.synchronize()
            for k, r in enumerate(reqs):
                fs, ll = outs[k]
                r.fs = fs.cpu().numpy()
                r.ll = None if ll is None else float(ll.item())
                r.status = int(status_h[k])
            return keep
        return done, finish

    # ------------------------------------------------------------- workers

    def _run_other(self, req):
        torch = self.torch
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            if req.kind == "growth3":
                f = numerics.make_extrap_func(models.growth3)
                fs = f(req.params, req.ns, list(req.pts_l))
            elif req.kind == "four":
                f = numerics.make_extrap_func(models.four_split)
                fs = f(req.params, req.ns, list(req.pts_l))
            elif req.kind == "im" and req.want_grad:
                key = (tuple(req.pts_l), tuple(req.ns))
                if key not in self._engines:
                    self._engines[key] = batch.Batch2D(req.pts_l, req.ns)
                eng = self._engines[key]
                ll, grad, st = eng.loglik_and_grad(np.asarray(req.params)[None, :], req.data,
                                                   scale=req.scale)
                fs_t, _, _ = eng.run(np.asarray(req.params)[None, :])
                req.fs = fs_t.cpu().numpy()[0]
                req.ll = float(ll.item())
                req.grad = grad.cpu().numpy()[0]
                req.status = int(st.abs().sum())
                return req
            else:
                raise ValueError(req.kind)
            req.fs = np.asarray(fs.data)
            if req.data is not None:
                from . import inference
                req.ll = float(inference.ll(req.scale * fs, spectrum.Spectrum(req.data)))
        return req

    # ----------------------------------------------------------------- run

    def run(self, requests, clock=time.perf_counter):
        """Serve `requests` (arrival in seconds from now); returns them with
        results and timings filled in."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        t0 = clock()
        pending, inflight, futures = [], [], []
        streams = [self.torch.cuda.Stream() for _ in range(self.max_inflight)]
        free_streams = list(streams)
        pool = ThreadPoolExecutor(max_workers=self.workers)
        nxt = 0
        remaining = len(reqs)
        while remaining:
            now = clock() - t0
            while nxt < len(reqs) and reqs[nxt].arrival <= now:
                pending.append(reqs[nxt])
                nxt += 1
            # admit 2-D spectrum requests into a wave; others to the workers
            wave, keep = [], []
            for r in pending:
                fp = self.footprint(r)
                if self._used + fp > self.budget and (inflight or futures or wave):
                    keep.append(r)
                    continue
                r._fp = fp
                self._used += fp
                r.t_admit = clock() - t0
                if r.kind in ("im", "im_sel") and not r.want_grad and len(wave) < self.max_wave:
                    wave.append(r)
                elif r.kind in ("im", "im_sel") and not r.want_grad:
                    self._used -= fp
                    keep.append(r)
                else:
                    futures.append((r, pool.submit(self._run_other, r)))
            pending = keep
            if wave:
                if free_streams:
                    s = free_streams.pop()
                    ev, fin = self._launch_wave(wave, s)
                    inflight.append((ev, fin, wave, s))
                else:
                    for r in wave:
                        self._used -= r._fp
                    pending = wave + pending
            # completions
            still = []
            for ev, fin, wv, s in inflight:
                if ev.query():
                    fin()
                    tdone = clock() - t0
                    for r in wv:
                        r.t_done = tdone
                        self._used -= r._fp
                        remaining -= 1
                    free_streams.append(s)
                else:
                    still.append((ev, fin, wv, s))
            inflight = still
            fst = []
            for r, fu in futures:
                if fu.done():
                    try:
                        fu.result()
                    except Exception as e:  # report per request, keep serving
                        r.error = repr(e)
                    r.t_done = clock() - t0
                    self._used -= r._fp
                    remaining -= 1
                else:
                    fst.append((r, fu))
            futures = fst
            if remaining:
                time.sleep(2e-4)
        pool.shutdown()
        return reqs


def host_schedules(recs, st, dx0, max_steps=10 ** 7):
    """Parameter rows of dgb_inst2d records evaluated on the host
    (dgb_sched2d_host): (table, row_off, row_cnt, status) numpy arrays."""
    lib = _lib.lib()
    recs = np.ascontiguousarray(recs)
    n = len(recs)
    cnt = np.zeros(n, dtype=np.int32)
    rp = recs.ctypes.data_as(ctypes.c_void_p)
    _lib.check(lib.dgb_sched2d_host(rp, n, ctypes.byref(st), max_steps, float(dx0),
                                    cnt.ctypes.data_as(ctypes.c_void_p), None, None, None),
               "dgb_sched2d_host(count)")
    off = np.zeros(n, dtype=np.int64)
    off[1:] = np.cumsum(cnt.astype(np.int64))[:-1]
    table = np.empty(max(int(cnt.sum()), 1) * 11)
    status = np.zeros(n, dtype=np.int32)
    _lib.check(lib.dgb_sched2d_host(rp, n, ctypes.byref(st), max_steps, float(dx0),
                                    cnt.ctypes.data_as(ctypes.c_void_p),
                                    off.ctypes.data_as(ctypes.c_void_p),
                                    table.ctypes.data_as(ctypes.c_void_p),
                                    status.ctypes.data_as(ctypes.c_void_p)),
               "dgb_sched2d_host(fill)")
    return table, off, cnt, status


def _extrap_torch(torch, fs_l, x_l, fail_mag=10):
    if len(fs_l) == 1:
        return fs_l[0]
    ex = numerics.linear_extrap(fs_l, x_l) if len(fs_l) == 2 else \
        numerics.quadratic_extrap(fs_l, x_l)
    best = fs_l[int(np.argmin(x_l))]
    failed = torch.abs(torch.log10(ex / best)) > fail_mag
    return torch.where(failed, best, ex)


def _loglik_torch(torch, fs, data, scale):
    model = scale * fs
    d = data if torch.is_tensor(data) else torch.from_numpy(np.asarray(data, np.float64)).cuda()
    mask = torch.zeros_like(model, dtype=torch.bool)
    mask.view(-1)[0] = True
    mask.view(-1)[-1] = True
    ok = (~mask) & (model > 0)
    term = -model + d * torch.log(torch.where(ok, model, torch.ones_like(model))) \
        - torch.lgamma(d + 1.0)
    return torch.where(ok, term, torch.zeros_like(term)).sum()


def config5_stream(n, seed=0, rate=2000.0, grad_frac=0.1, obs=None):
    """The mixed request stream of the serving workload: Poisson arrivals at
    `rate` per second; 70% 2-D IM (pts base uniform in 40..120, pts_l = base,
    base+10, base+20, ns (20,20) or (40,40)), 20% DFE cache entries (IM with
    selection, gamma1 and gamma2 from the 50-point log grid on
    [-2000, -1e-4]), 8% 3-D growth model (pts 60..90), 2% four populations
    (pts 30..40, ns (10,10,10,10)); grad_frac of the IM requests also ask for
    gradients (they need `obs`, an observed 41x41 spectrum)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n)
    cls = rng.choice(4, size=n, p=[0.70, 0.20, 0.08, 0.02])
    gammas = -np.logspace(np.log10(2000), np.log10(1e-4), 50)
    base = batch.IM_PARAMS
    im0 = (0.6233, 0.05171, 0.2775, 0.01061, 8.917, 7.671)
    draws = _im_draws(n, rng)
    reqs, t = [], 0.0
    for k in range(n):
        t += gaps[k]
        c = cls[k]
        if c == 0:
            p = int(rng.integers(40, 101))
            ns = (20, 20) if rng.random() < 0.5 else (40, 40)
            want = bool(rng.random() < grad_frac) and obs is not None and ns == (40, 40)
            reqs.append(Request(k, "im", tuple(draws[k]), (p, p + 10, p + 20), ns,
                                data=obs if want else None, scale=5e4, want_grad=want,
                                arrival=t))
        elif c == 1:
            g1, g2 = gammas[rng.integers(50)], gammas[rng.integers(50)]
            reqs.append(Request(k, "im_sel", im0 + (g1, g2), (40, 50, 60), (20, 20), arrival=t))
        elif c == 2:
            p = int(rng.integers(60, 71))
            reqs.append(Request(k, "growth3", models.GROWTH3_DEFAULT, (p, p + 10, p + 20),
                                (20, 20, 20), arrival=t))
        else:
            p = int(rng.integers(30, 37))
            reqs.append(Request(k, "four", models.FOUR_DEFAULT, (p, p + 2, p + 4),
                                (10, 10, 10, 10), arrival=t))
    del base
    return reqs


def _im_draws(n, rng):
    s = rng.uniform(0.05, 0.95, n)
    nu1 = np.exp(rng.uniform(np.log(0.01), np.log(100), n))
    nu2 = np.exp(rng.uniform(np.log(0.01), np.log(100), n))
    T = np.exp(rng.uniform(np.log(0.01), np.log(2), n))
    m12 = rng.uniform(0, 10, n)
    m21 = rng.uniform(0, 10, n)
    return np.stack([s, nu1, nu2, T, m12, m21], axis=1)


def latency_summary(reqs):
    lat = np.array([r.latency for r in reqs if r.latency is not None and r.error is None])
    span = max(r.t_done for r in reqs if r.t_done is not None) - min(r.arrival for r in reqs)
    return {"requests": len(reqs), "completed": int(lat.size),
            "p50_s": float(np.percentile(lat, 50)) if lat.size else None,
            "p99_s": float(np.percentile(lat, 99)) if lat.size else None,
            "spectra_per_s": float(lat.size / span) if span > 0 else None,
            "errors": sum(1 for r in reqs if r.error)}
