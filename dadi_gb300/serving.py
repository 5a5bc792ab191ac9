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
  one launch over an explicit work-item list (dgb_items2d_integrate) with one
  CTA per (request, grid) item, so requests with different grid sizes and
  sample sizes share a launch.  Each wave's integration runs on its own
  lowest-priority CUDA stream and its CTAs retire item by item, so a wave
  launched while earlier ones are still running takes SMs as soon as any CTA
  finishes: arrivals join work already on the device instead of waiting for
  it to drain.  Waiting requests stay on the host, cheapest first, and are
  launched while fewer than `slots` work items are in flight, so the host
  keeps the order and new work never queues behind a deep device backlog.
  When the host sees a wave's integration finish it queues the wave's
  spectra, extrapolation and likelihoods on one highest-priority stream.
  Densities stay on the device from the initial condition to the spectrum;
  only spectra and likelihoods come back, in one copy per wave.
* Gradient requests that share grid sizes, sample sizes and observed data
  are grouped the same way into one forward-with-checkpoints launch and one
  adjoint launch; they run on worker threads with their own streams,
  overlapping the waves.
* 3-D and 4-D requests wait on the host until a worker is free; the worker
  then takes every waiting request of the same model, grids, sample sizes
  and data and integrates them as one batch (batchnd.ModelBatch: all of
  them advance together in each sweep launch, densities stay on the device,
  only spectra and likelihoods come back).

Every request records arrival, admission and completion times; latency is
completion minus arrival.  The server uses up to max_inflight + 2 * workers
+ 2 streams at once; with CUDA_DEVICE_MAX_CONNECTIONS=32 in the environment
before CUDA starts, they do not share hardware queues.
"""
import ctypes
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass

import numpy as np

from . import _lib, batch, batchnd, epilogue, models, numerics, phimanip, spectrum

ITEM_DTYPE = batch.ITEM2D_DTYPE


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


class _Wave:
    """One 2-D wave: phase 0 while its integration runs on its own stream,
    phase 1 once its spectra are queued on the tail stream."""

    def __init__(self, reqs, stream):
        self.reqs = reqs
        self.stream = stream
        self.slots = []
        self.shapes = []
        self.phase = 0
        self.event = None
        self.nitems = 0

    def finish(self):
        """Copy results into the requests (the tail event has completed)."""
        h = self.host.numpy()
        lls = self.host_ll.numpy()
        o = 0
        for k, r in enumerate(self.reqs):
            m = int(np.prod(self.shapes[k]))
            r.fs = h[o:o + m].reshape(self.shapes[k]).copy()
            o += m
            if r.data is not None:
                r.ll = float(lls[k])
            r.status = int(self.status[k])
        self.keep = self.d_phi = self.host = self.host_ll = None


class Server:
    """hbm_budget: bytes of device memory requests may hold at once;
    max_wave / min_wave: most / fewest requests per 2-D wave (fewer when
    fewer are waiting); max_inflight: waves in flight at once (one CUDA
    stream each); slots: most 2-D work items in flight (default two per
    SM); workers: threads for 3-D/4-D request groups, and as many again for
    gradient groups; max_nd_group: most 3-D/4-D requests per group;
    cluster_items: a 2-D wave of at most this many work items (default one
    per 16 SMs) runs each on a cluster of 8 CTAs
    (dgb_items2d_integrate_cluster), which cuts a lone request's latency
    2-2.8x at the cost of 8 SMs per item; larger waves run one CTA per item.
    A request's 2-D spectrum is then the same alone and in the mix to
    rounding (1e-10 relative after extrapolation), not bitwise."""

    def __init__(self, hbm_budget=16 << 30, max_wave=512, workers=4, max_inflight=16,
                 min_wave=8, slots=None, max_nd_group=64, cluster_items=None):
        self.torch = _lib.require_cuda()
        self.budget = int(hbm_budget)
        self.max_wave = max_wave
        self.max_inflight = max_inflight
        self.min_wave = min_wave
        if slots is None:
            slots = 2 * self.torch.cuda.get_device_properties(
                self.torch.cuda.current_device()).multi_processor_count
        self.slots = int(slots)
        if cluster_items is None:
            cluster_items = self.torch.cuda.get_device_properties(
                self.torch.cuda.current_device()).multi_processor_count // 16
        self.cluster_items = int(cluster_items)
        self.workers = workers
        self.max_nd_group = int(max_nd_group)
        self._streams = None
        self._used = 0
        self._lock = threading.Lock()
        self._grids = {}
        self._phi0 = {}
        self._engines = {}
        self._batches = {}
        self._obs = {}

    # ----------------------------------------------------------- resources

    def footprint(self, req):
        """Device bytes the request holds while admitted."""
        P = 2 if req.kind in ("im", "im_sel") else (3 if req.kind == "growth3" else 4)
        dens = sum(8 * L ** P for L in req.pts_l)
        steps = self._steps(req)
        rows = steps * 11 * 8
        extra = 0
        if req.want_grad:
            # checkpoints, derivative rows and the adjoint's stored trajectory
            C = max(8, int(np.ceil(np.sqrt(max(steps, 1)))))
            extra = sum(8 * L * L * ((steps + C - 1) // C) for L in req.pts_l) + steps * 60 * 8
            extra += sum(8 * L * L * (2 * steps + 1) for L in req.pts_l)
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
            self._grids[L] = (xx, _lib.upload_resident(torch, xx))
        return self._grids[L]

    def _initial(self, L, gamma1):
        """phi_1D(gamma1) split to 2-D (dadi/PhiManip.py:12-234), cached."""
        key = (L, float(gamma1))
        if key not in self._phi0:
            xx = self._grid(L)[0]
            phi = phimanip.phi_1D_to_2D(xx, phimanip.phi_1D(xx, gamma=gamma1))
            self._phi0[key] = _lib.upload_resident(self.torch, phi.ravel())
        return self._phi0[key]

    # --------------------------------------------------------------- waves

    def _data(self, data):
        """Observed spectrum as a device tensor, uploaded once per array."""
        if self.torch.is_tensor(data):
            return data
        key = id(data)
        with self._lock:
            hit = self._obs.get(key)
            if hit is None or hit[0] is not data:
                hit = self._obs[key] = (data, _lib.upload_resident(self.torch, data))
        return hit[1]

    def prepare(self, pts, ns_list):
        """Upload ahead of time what 2-D requests at these grid sizes and
        sample sizes need (grids, sampling tables, initial densities), so
        the first requests of each size do not pay for it."""
        for L in pts:
            xx = self._grid(L)[0]
            self._initial(L, 0.0)
            for ns in ns_list:
                for n in set(ns):
                    spectrum._device_tables(self.torch, n, xx, self.torch.device("cuda"))

    def _launch_wave(self, reqs, stream):
        """Enqueue one 2-D wave's integration on `stream` (lowest priority)
        without waiting for the device; returns the _Wave."""
        torch = self.torch
        lib = _lib.lib()
        w = _Wave(reqs, stream)
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
            for k, r in enumerate(reqs):
                g1 = r.params[6] if r.kind == "im_sel" else 0.0
                sl = []
                for L in r.pts_l:
                    items.append((L, 0, xx_off[L], off, k))
                    phi0s.append(self._initial(L, g1))
                    sl.append((off, L))
                    off += L * L
                w.slots.append(sl)
            items = np.array(items, dtype=ITEM_DTYPE)
            w.nitems = len(items)
            w.d_phi = torch.cat(phi0s)
            st = batch.settings_from_globals()
            if st.use_old_timestep:
                # dt depends on the grid: one schedule per item
                req_of_item = items["sched"].copy()
                table_h, roff_h, cnt_h, status_i = _item_schedules(
                    recs, req_of_item, items["L"], st, {L: self._grid(L)[0][1] for L in Ls})
                items["sched"] = np.arange(len(items))
                w.status = np.zeros(len(reqs), np.int32)
                np.bitwise_or.at(w.status, req_of_item, status_i)
            else:
                table_h, roff_h, cnt_h, w.status = host_schedules(recs, st,
                                                                  self._grid(Ls[0])[0][1])
            cost = cnt_h[items["sched"]].astype(np.int64) * items["L"].astype(np.int64) ** 2
            order_h = np.argsort(-cost, kind="stable").astype(np.int32)
            d_items = _lib.to_device(torch, items.view(np.uint8), np.uint8)
            table = _lib.to_device(torch, table_h)
            roff = _lib.to_device(torch, roff_h, np.int64)
            cnt = _lib.to_device(torch, cnt_h, np.int32)
            order = _lib.to_device(torch, order_h, np.int32)
            Lmin, Lmax = min(Ls), max(Ls)
            ws = None
            if (len(items) <= self.cluster_items and not st.use_delj_trick
                    and Lmin >= 24 and Lmax <= 128):
                # few items: each on a cluster of 8 CTAs (8 SMs' FP64 pipes)
                _lib.check(lib.dgb_items2d_integrate_cluster(
                    _lib.dptr(d_items), len(items), Lmin, Lmax, _lib.dptr(d_xx),
                    _lib.dptr(w.d_phi), _lib.dptr(table), _lib.dptr(roff), _lib.dptr(cnt), 8,
                    None, None, 0, sh), "dgb_items2d_integrate_cluster")
            else:
                ws, nws = _lib.workspace(torch, lib.dgb_workspace_bytes(3, 2, Lmax, len(items)))
                _lib.check(lib.dgb_items2d_integrate(
                    _lib.dptr(d_items), len(items), Lmax, _lib.dptr(d_xx), _lib.dptr(w.d_phi),
                    _lib.dptr(table), _lib.dptr(roff), _lib.dptr(cnt), _lib.dptr(order),
                    ctypes.byref(st), 1, _lib.dptr(ws), nws, sh), "dgb_items2d_integrate")
            w.event = torch.cuda.Event()
            w.event.record(stream)
        w.keep = [d_items, table, ws, order, cnt, roff, d_xx]
        return w

    def _launch_tail(self, w, tail):
        """A wave whose integration has finished: its spectra, extrapolation
        and likelihoods (two launches, dgb_from_phi2d and dgb_extrap_ll) on
        the shared high-priority `tail` stream, copied into pinned host
        buffers."""
        torch = self.torch
        with torch.cuda.stream(tail):
            jobs = []
            for k, r in enumerate(w.reqs):
                phis = [w.d_phi[o2:o2 + L * L].view(L, L) for (o2, L) in w.slots[k]]
                xxs = [self._grid(L)[0] for L in r.pts_l]
                data = self._data(r.data) if r.data is not None else None
                jobs.append((phis, xxs, tuple(r.ns), data, r.scale))
                w.shapes.append((r.ns[0] + 1, r.ns[1] + 1))
            _, ll, flat = epilogue.spectra_2d(torch, jobs)
            w.host = torch.empty(flat.numel(), dtype=torch.float64, pin_memory=True)
            w.host.copy_(flat, non_blocking=True)
            w.host_ll = torch.empty(ll.numel(), dtype=torch.float64, pin_memory=True)
            w.host_ll.copy_(ll, non_blocking=True)
            w.event = torch.cuda.Event()
            w.event.record(tail)
        w.phase = 1

    # ------------------------------------------------------------- workers

    def _engine(self, pts_l, ns):
        key = (tuple(pts_l), tuple(ns))
        with self._lock:
            if key not in self._engines:
                self._engines[key] = batch.Batch2D(pts_l, ns)
            return self._engines[key]

    def _run_grad_group(self, reqs):
        """Gradient requests sharing grid sizes, sample sizes and data: one
        forward-with-checkpoints and one adjoint launch for the group."""
        torch = self.torch
        s = torch.cuda.Stream(priority=-1)
        with torch.cuda.stream(s):
            r0 = reqs[0]
            eng = self._engine(r0.pts_l, r0.ns)
            params = np.array([r.params for r in reqs], dtype=np.float64)
            ll, ctx = eng.forward_for_adjoint(params, r0.data, scale=r0.scale,
                                              tail_per_set=True)
            grad = eng.adjoint(ctx, torch.ones_like(ll))
            fs = _lib.to_host(torch, ctx["fs"])
            ll = _lib.to_host(torch, ll.detach())
            grad = _lib.to_host(torch, grad)
            st = _lib.to_host(torch, ctx["status"])
        for k, r in enumerate(reqs):
            r.fs, r.ll, r.grad, r.status = fs[k], float(ll[k]), grad[k], int(st[k])
        return reqs

    def _model_batch(self, kind, pts_l, ns):
        key = (kind, tuple(pts_l), tuple(ns))
        with self._lock:
            mb = self._batches.get(key)
            if mb is None:
                mb = self._batches[key] = batchnd.ModelBatch(kind, pts_l, ns)
                mb.lock = threading.Lock()
        return mb

    def _run_other(self, reqs):
        """3-D and 4-D requests sharing model, grids, sample sizes and data:
        one batched integration per grid on a worker stream."""
        torch = self.torch
        r0 = reqs[0]
        mb = self._model_batch(r0.kind, r0.pts_l, r0.ns)
        s = torch.cuda.Stream(priority=-1)
        with mb.lock, torch.cuda.stream(s):
            data = self._data(r0.data) if r0.data is not None else None
            fs, ll, status = mb.run([r.params for r in reqs], data=data, scale=r0.scale)
            fs = _lib.to_host(torch, fs)
            ll = _lib.to_host(torch, ll) if ll is not None else None
        for k, r in enumerate(reqs):
            r.fs = fs[k]
            if ll is not None:
                r.ll = float(ll[k])
            r.status = int(status[k])
        return reqs

    # ----------------------------------------------------------------- run

    def _cost(self, req):
        return self._steps(req) * sum(L * L for L in req.pts_l)

    def run(self, requests, clock=time.perf_counter):
        """Serve `requests` (arrival in seconds from now); returns them with
        results and timings filled in.

        2-D requests wait on the host, cheapest first (cost = steps x grid
        points), and are launched in waves while the device has CTA slots
        to spare: at most `slots` work items are in flight, so a new wave
        never queues behind a deep backlog of CTAs already submitted, and the
        host keeps the freedom to reorder what waits.  A wave takes an equal
        share of the waiting requests per free stream, between min_wave and
        max_wave, so waves hold requests of similar cost."""
        torch = self.torch
        reqs = sorted(requests, key=lambda r: r.arrival)
        t0 = clock()
        waiting2d, inflight, futures = [], [], []
        # integrations at the lowest priority, spectra at the highest (torch
        # clamps to the device's range)
        # the server's own streams, kept across runs: the caching allocator
        # keeps a memory pool per stream, and a burst on fresh streams pays
        # device allocations (which stall the device) in its first waves
        if self._streams is None:
            self._streams = ([torch.cuda.Stream(priority=0) for _ in range(self.max_inflight)],
                             torch.cuda.Stream(priority=-8))
        free_streams, tail = list(self._streams[0]), self._streams[1]
        pool = ThreadPoolExecutor(max_workers=self.workers)
        gpool = ThreadPoolExecutor(max_workers=self.workers)
        # the scheduling loop must get the interpreter back quickly from
        # worker threads that build tables in Python
        switch = sys.getswitchinterval()
        sys.setswitchinterval(min(switch, 5e-4))
        nxt = 0
        remaining = len(reqs)
        held = []   # non-wave requests waiting for budget
        waiting_nd = []  # admitted 3-D / 4-D requests waiting for a worker
        nd_busy = [0]

        def busy():
            return bool(inflight or futures or waiting_nd)

        try:
            while remaining:
                now = clock() - t0
                arrived = []
                while nxt < len(reqs) and reqs[nxt].arrival <= now:
                    arrived.append(reqs[nxt])
                    nxt += 1
                # gradient groups and 3-D/4-D requests go to the workers
                groups, keep = {}, []
                for r in held + arrived:
                    if r.kind in ("im", "im_sel") and not r.want_grad:
                        waiting2d.append(r)
                        continue
                    fp = self.footprint(r)
                    if self._used + fp > self.budget and (busy() or groups):
                        keep.append(r)
                        continue
                    r._fp = fp
                    self._used += fp
                    r.t_admit = clock() - t0
                    if r.kind == "im" and r.want_grad:
                        key = (tuple(r.pts_l), tuple(r.ns), id(r.data), r.scale)
                        groups.setdefault(key, []).append(r)
                    else:
                        waiting_nd.append(r)
                held = keep
                for grp in groups.values():
                    futures.append((grp, gpool.submit(self._run_grad_group, grp)))
                # 3-D / 4-D: a free worker takes every waiting request that
                # shares the oldest one's model, grids, sample sizes and data
                while waiting_nd and nd_busy[0] < self.workers:
                    r0 = waiting_nd[0]
                    key = (r0.kind, tuple(r0.pts_l), tuple(r0.ns), id(r0.data), r0.scale)
                    grp = [r for r in waiting_nd
                           if (r.kind, tuple(r.pts_l), tuple(r.ns), id(r.data), r.scale) == key]
                    grp = grp[:self.max_nd_group]
                    ids = set(id(r) for r in grp)
                    waiting_nd = [r for r in waiting_nd if id(r) not in ids]
                    nd_busy[0] += 1
                    futures.append((grp, pool.submit(self._run_other, grp), True))
                # 2-D waves, cheapest first, while streams and CTA slots are free
                if waiting2d and arrived:
                    waiting2d.sort(key=self._cost)
                in_items = sum(w.nitems for w in inflight if w.phase == 0)
                while waiting2d and free_streams and in_items < self.slots:
                    share = -(-len(waiting2d) // len(free_streams))
                    size = max(self.min_wave, min(self.max_wave, share))
                    wave, items = [], 0
                    for r in waiting2d:
                        if len(wave) >= size or (wave and in_items + items >= self.slots):
                            break
                        fp = self.footprint(r)
                        if self._used + fp > self.budget and (busy() or wave):
                            break
                        r._fp = fp
                        self._used += fp
                        r.t_admit = clock() - t0
                        wave.append(r)
                        items += len(r.pts_l)
                    if not wave:
                        break
                    del waiting2d[:len(wave)]
                    inflight.append(self._launch_wave(wave, free_streams.pop()))
                    in_items += items
                # completions
                still = []
                for w in inflight:
                    if not w.event.query():
                        still.append(w)
                    elif w.phase == 0:
                        # integration done: queue its spectra, free its stream
                        self._launch_tail(w, tail)
                        free_streams.append(w.stream)
                        still.append(w)
                    else:
                        w.finish()
                        tdone = clock() - t0
                        for r in w.reqs:
                            r.t_done = tdone
                            self._used -= r._fp
                            remaining -= 1
                inflight = still
                fst = []
                for item in futures:
                    grp, fu = item[0], item[1]
                    if fu.done():
                        if len(item) > 2:
                            nd_busy[0] -= 1
                        try:
                            fu.result()
                        except Exception as e:  # report per request, keep serving
                            for r in grp:
                                r.error = repr(e)
                        tdone = clock() - t0
                        for r in grp:
                            r.t_done = tdone
                            self._used -= r._fp
                            remaining -= 1
                    else:
                        fst.append(item)
                futures = fst
                if remaining:
                    time.sleep(2e-4)
        finally:
            pool.shutdown()
            gpool.shutdown()
            sys.setswitchinterval(switch)
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


def _item_schedules(recs, req_of_item, L_of_item, st, dx0_of_L):
    """One schedule per work item (with use_old_timestep the step depends on
    the grid spacing): item j's request evaluated with item j's grid."""
    tabs, cnts, stats = [], [], []
    for j in range(len(req_of_item)):
        q = int(req_of_item[j])
        t, _, c, sst = host_schedules(recs[q:q + 1], st, dx0_of_L[int(L_of_item[j])])
        tabs.append(t[:int(c[0]) * 11])
        cnts.append(int(c[0]))
        stats.append(int(sst[0]))
    cnt = np.array(cnts, dtype=np.int32)
    off = np.zeros(len(cnt), dtype=np.int64)
    off[1:] = np.cumsum(cnt.astype(np.int64))[:-1]
    table = np.concatenate(tabs) if tabs else np.zeros(11)
    return table, off, cnt, np.array(stats, dtype=np.int32)


def config5_stream(n, seed=0, rate=2000.0, grad_frac=0.1, obs=None):
    """The mixed request stream of the serving workload: Poisson arrivals at
    `rate` per second; 70% 2-D IM (pts_l = base, base+10, base+20 with the
    base uniform in 40..100, so every grid lies in 40..120; ns (20,20) or
    (40,40)), 20% DFE cache entries (IM with
    selection, gamma1 and gamma2 from the 50-point log grid on
    [-2000, -1e-4]), 8% 3-D growth model (grids in 60..90: base 60..70),
    2% four populations (grids in 30..40: base 30..36, ns (10,10,10,10));
    grad_frac of the IM requests also ask for
    gradients (they need `obs`, an observed 41x41 spectrum)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n)
    cls = rng.choice(4, size=n, p=[0.70, 0.20, 0.08, 0.02])
    gammas = -np.logspace(np.log10(2000), np.log10(1e-4), 50)
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
