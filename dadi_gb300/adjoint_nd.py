"""Gradients of spectrum log-likelihoods for N-population models
(1-4 populations) by the discrete adjoint of the table-driven time loop
(dgb_integrate_table_states, dgb_adjoint_table_nd).

The adjoint gives dJ/d(parameter-table entry) for every step.  The table is
a function of the model parameters through the schedule walk of the
reference loop (dadi/Integration.py:504-553 for three populations: dt from
the current parameters by _compute_dt, :147-176, the final partial step
T - t, and the sizes evaluated at the next time); `table_dual` walks that
schedule in forward-mode dual numbers, producing the table values exactly as
integration.build_table does and their derivatives, and the chain rule
dJ/dtheta = sum_k sum_j dJ/drow_kj drow_kj/dtheta finishes the gradient.

The loss tail (from_phi, extrapolation, Poisson likelihood) is tiny and is
differentiated by torch autograd; its gradient with respect to each grid's
final density seeds the adjoint.

`Growth3` is the three-population workload (three populations split from
one, each growing exponentially from nu0_i to nuF_i over T, symmetric
migration): parameters (nu0_1, nu0_2, nu0_3, nuF_1, nuF_2, nuF_3, m12, m13,
m23, T) with fixed selection gammas.
"""

import ctypes

import numpy as np

from . import _lib, integration, numerics, phimanip, spectrum

PF_CONST, PF_EXPLOG = 0, 2


class Form:
    """A parameter as a function of time with derivative seeds: kind
    PF_CONST (value a) or PF_EXPLOG (a * exp(log(b / a) * t / c), the
    exponential-growth lambda of the workloads); da, db, dc are
    d(a, b, c)/dtheta."""

    def __init__(self, kind, a, b=0.0, c=1.0, da=None, db=None, dc=None, npar=0):
        z = np.zeros(npar)
        self.kind, self.a, self.b, self.c = kind, float(a), float(b), float(c)
        self.da = z if da is None else np.asarray(da, float)
        self.db = z if db is None else np.asarray(db, float)
        self.dc = z if dc is None else np.asarray(dc, float)

    def at(self, t, dtd):
        """(value, d value/dtheta) at time t with dt/dtheta = dtd."""
        if self.kind == PF_CONST:
            return self.a, self.da.copy()
        a, b, c = self.a, self.b, self.c
        lq = np.log(b / a)
        v = a * np.exp(lq * t / c)
        e = v / a
        dlq = self.db / b - self.da / a
        dz = (dlq * t + lq * dtd) / c - (lq * t / c) * self.dc / c
        return v, self.da * e + a * e * dz


def _compute_dt_dual(nu, dnu, ms, dms, gamma, dgamma, h, dh, settings, dx0):
    """_compute_dt (dadi/Integration.py:147-176) with its derivative along the
    branch its max takes; the value is computed exactly as
    integration._compute_dt does."""
    tsf, otsf, old, _ = settings
    npar = len(dnu)
    if old:
        return otsf * dx0, np.zeros(npar)
    t1 = np.abs(h + (1 - 2 * h) * 0.5) * 0.5 * (1 - 0.5)
    u2 = h + (1 - 2 * h) * 0.25
    t2 = np.abs(u2) * 0.25 * (1 - 0.25)
    tm = max(t1, t2)
    cands = [0.25 / nu, sum(ms), abs(gamma) * 2 * tm]
    maxVM = max(cands)
    if not maxVM > 0:
        return np.inf, np.zeros(npar)
    br = cands.index(maxVM)
    if br == 0:
        dmx = -0.25 * dnu / (nu * nu)
    elif br == 1:
        dmx = np.sum(dms, axis=0) if len(dms) else np.zeros(npar)
    else:
        dtm = (np.sign(u2) * 0.5 * dh * 0.25 * (1 - 0.25)) if t2 > t1 else 0.0 * dh
        dmx = np.sign(gamma) * dgamma * 2 * tm + abs(gamma) * 2 * dtm
    dt = tsf / maxVM
    if dt == 0:
        raise ValueError('Timestep is zero.')
    return dt, -tsf * dmx / (maxVM * maxVM)


def table_dual(P, xx, T, dT, nu_forms, mig_forms, gamma_forms, h_forms, theta0_form,
               initial_t=0.0):
    """Parameter table of a P-population time loop (the layout of
    integration.build_table, DGB_ROW_STRIDE(P) doubles per step) and its
    derivative with respect to the npar model parameters: (table (n,
    stride), drows (n, stride, npar)).  mig_forms[k][j] is the rate into k
    from j; gamma, h and theta0 are Forms as well."""
    settings = integration.current_settings()
    npar = len(dT)
    dx0 = xx[1] - xx[0]
    stride = integration.row_stride(P)
    offd = [(k, j) for k in range(P) for j in range(P) if j != k]
    t, dtd = float(initial_t), np.zeros(npar)
    nu = [f.at(t, dtd) for f in nu_forms]
    gam = [f.at(t, dtd) for f in gamma_forms]
    hh = [f.at(t, dtd) for f in h_forms]
    mig = {kj: mig_forms[kj[0]][kj[1]].at(t, dtd) for kj in offd}
    rows, drows = [], []
    while t < T:
        best = None
        for k in range(P):
            ms = [mig[(k, j)][0] for j in range(P) if j != k]
            dms = [mig[(k, j)][1] for j in range(P) if j != k]
            if P == 1:
                ms, dms = [0], [np.zeros(npar)]
            c = _compute_dt_dual(nu[k][0], nu[k][1], ms, dms, gam[k][0], gam[k][1],
                                 hh[k][0], hh[k][1], settings, dx0)
            if best is None or c[0] < best[0]:
                best = c
        rem, drem = T - t, dT - dtd
        this, dthis = (best if best[0] <= rem else (rem, drem))
        t, dtd = t + this, dtd + dthis
        nu = [f.at(t, dtd) for f in nu_forms]
        gam = [f.at(t, dtd) for f in gamma_forms]
        hh = [f.at(t, dtd) for f in h_forms]
        mig = {kj: mig_forms[kj[0]][kj[1]].at(t, dtd) for kj in offd}
        th = theta0_form.at(t, dtd)
        row = np.empty(stride)
        drow = np.zeros((stride, npar))
        row[0], drow[0] = this, dthis
        row[1], drow[1] = th
        for k in range(P):
            row[2 + k], drow[2 + k] = nu[k]
            row[2 + P + k], drow[2 + P + k] = gam[k]
            row[2 + 2 * P + k], drow[2 + 2 * P + k] = hh[k]
        row[2 + 3 * P] = 1.0
        for q, kj in enumerate(offd):
            row[3 + 3 * P + q], drow[3 + 3 * P + q] = mig[kj]
        rows.append(row)
        drows.append(drow)
    return (np.array(rows, dtype=np.float64).reshape(len(rows), stride),
            np.array(drows, dtype=np.float64).reshape(len(rows), stride, npar))


def schedule_dual(rec, seed, npar, xx, max_steps=10 ** 7):
    """table_dual walked in C (dgb_schednd_dual_host) for a dgb_instnd record
    and its dgb_seednd derivative seeds: (table (n, stride), drows (n,
    stride, npar)), the rows bit for bit those of batchnd.schedules."""
    lib = _lib.lib()
    st = _lib.settings_struct(*integration.current_settings())
    dx0 = float(xx[1] - xx[0])
    n = ctypes.c_int(0)
    status = ctypes.c_int(0)
    args = (ctypes.byref(rec), ctypes.byref(seed), int(npar), ctypes.byref(st), int(max_steps),
            dx0)
    _lib.check(lib.dgb_schednd_dual_host(*args, ctypes.byref(n), None, None,
                                         ctypes.byref(status)), "dgb_schednd_dual_host(count)")
    stride = integration.row_stride(rec.ndim)
    table = np.zeros((max(n.value, 1), stride))
    drows = np.zeros((max(n.value, 1), stride, npar))
    status.value = 0
    _lib.check(lib.dgb_schednd_dual_host(*args, ctypes.byref(n),
                                         table.ctypes.data_as(ctypes.c_void_p),
                                         drows.ctypes.data_as(ctypes.c_void_p),
                                         ctypes.byref(status)), "dgb_schednd_dual_host")
    if status.value:
        raise ValueError("schedule walk failed: status %d" % status.value)
    return table[:n.value], drows[:n.value]


def _row_grads(torch, gpart, n, per, stride, drows):
    """d J / d theta from one integration's per-step partial rows (n steps of
    `per` doubles: the CTAs' rows, then the injection's dt and theta0 terms)
    and the table's derivatives drows (n, stride, npar)."""
    gp = gpart.view(n, per)
    G = gp[:, :per - 2].reshape(n, -1, stride).sum(dim=1)
    G[:, 0] += gp[:, per - 2]
    G[:, 1] += gp[:, per - 1]
    return torch.einsum("kj,kjp->p", G, _lib.to_device(torch, drows))


class TableModel:
    """An N-population model run through parameter tables on the GPU, with
    the gradient of its Poisson log-likelihood by the discrete adjoint.
    Subclasses give P, the initial density and the table with derivatives."""

    P = None
    npar = None

    def __init__(self, pts_l, ns):
        self.torch = _lib.require_cuda()
        self.pts_l = [int(p) for p in np.atleast_1d(pts_l)]
        self.ns = tuple(int(n) for n in ns)
        self.xxs = [numerics.default_grid(L) for L in self.pts_l]

    def initial(self, xx):
        raise NotImplementedError

    def table(self, params, xx):
        raise NotImplementedError

    def _forward(self, params, keep_states):
        torch, lib = self.torch, _lib.lib()
        P = self.P
        out = []
        for L, xx in zip(self.pts_l, self.xxs):
            table, drows = self.table(params, xx)
            d_phi = _lib.to_device(torch, self.initial(xx))
            d_xx = _lib.to_device(torch, xx)
            d_tab = _lib.to_device(torch, table)
            n = len(table)
            states = torch.empty(((n + 1) * L ** P if keep_states else L ** P),
                                 dtype=torch.float64, device="cuda")
            sh = _lib.stream_handle(torch)
            ws, nws = _lib.workspace(torch, lib.dgb_workspace_bytes(0, P, L, 0))
            if keep_states:
                _lib.check(lib.dgb_integrate_table_states(
                    _lib.dptr(d_phi), P, L, _lib.dptr(d_xx), _lib.dptr(d_tab), n, 0, 0,
                    _lib.dptr(states), _lib.dptr(ws), nws, sh), "dgb_integrate_table_states")
            else:
                _lib.check(lib.dgb_integrate_table(
                    _lib.dptr(d_phi), P, L, _lib.dptr(d_xx), _lib.dptr(d_tab), n, 0, 0, 0,
                    _lib.dptr(ws), nws, sh), "dgb_integrate_table")
            out.append(dict(L=L, xx=xx, d_xx=d_xx, d_tab=d_tab, n=n, drows=drows,
                            phi=d_phi.view(*([L] * P)), states=states))
        return out

    def _tail(self, phis, data, scale):
        """Extrapolated spectrum and Poisson log-likelihood (torch, so that
        autograd gives dJ/dphi)."""
        torch = self.torch
        fs_l = [from_phi_torch(torch, p, self.ns, xx) for p, xx in zip(phis, self.xxs)]
        x_l = [xx[1] for xx in self.xxs]
        if len(fs_l) == 1:
            fs = fs_l[0]
        else:
            ex = (numerics.linear_extrap(fs_l, x_l) if len(fs_l) == 2
                  else numerics.quadratic_extrap(fs_l, x_l))
            best = fs_l[int(np.argmin(x_l))]
            failed = torch.abs(torch.log10(ex / best)) > 10
            fs = torch.where(failed, best, ex)
        if data is None:
            return fs, None
        d = data if torch.is_tensor(data) else _lib.to_device(torch, data)
        model = scale * fs
        mask = torch.zeros(tuple(model.shape), dtype=torch.bool, device=model.device)
        mask.view(-1)[0] = True
        mask.view(-1)[-1] = True
        ok = (~mask) & (model > 0)
        term = -model + d * torch.log(torch.where(ok, model, torch.ones_like(model))) \
            - torch.lgamma(d + 1.0)
        return fs, torch.where(ok, term, torch.zeros_like(term)).sum()

    def spectrum_ll(self, params, data=None, scale=1.0):
        """(extrapolated spectrum, log-likelihood or None) as CUDA tensors."""
        runs = self._forward(params, keep_states=False)
        return self._tail([r["phi"] for r in runs], data, scale)

    def loglik_and_grad(self, params, data, scale=1.0):
        """(ll, dll/dparams (npar,), spectrum) for one parameter set."""
        torch, lib = self.torch, _lib.lib()
        P = self.P
        runs = self._forward(params, keep_states=True)
        phis = [r["phi"].detach().requires_grad_(True) for r in runs]
        with torch.enable_grad():
            fs, ll = self._tail(phis, data, scale)
        lams = torch.autograd.grad(ll, phis, allow_unused=True)
        grad = torch.zeros(self.npar, dtype=torch.float64, device="cuda")
        stride = integration.row_stride(P)
        for r, lam in zip(runs, lams):
            L, n = r["L"], r["n"]
            if n == 0:
                continue
            lam = (lam if lam is not None else torch.zeros_like(r["phi"])).contiguous().clone()
            per = lib.dgb_adjoint_table_nd_gpart_doubles(P, L)
            gpart = torch.empty(n * per, dtype=torch.float64, device="cuda")
            ws, nws = _lib.workspace(torch, lib.dgb_workspace_bytes(4, P, L, 0))
            _lib.check(lib.dgb_adjoint_table_nd(
                _lib.dptr(lam), P, L, _lib.dptr(r["d_xx"]), _lib.dptr(r["d_tab"]), n, 0, 0,
                _lib.dptr(r["states"]), _lib.dptr(gpart), _lib.dptr(ws), nws,
                _lib.stream_handle(torch)), "dgb_adjoint_table_nd")
            grad += _row_grads(torch, gpart, n, per, stride, r["drows"])
            r["states"] = None
        return ll.detach(), grad, fs.detach()


    #: Bytes of recorded densities one batched gradient pass may hold (None:
    #: half the device memory free at the call); more parameter sets are
    #: taken in groups of about equal size.
    states_budget = None

    def loglik_and_grad_batch(self, thetas, data, scale=1.0):
        """loglik_and_grad for many parameter sets at once: per grid one
        batched forward recording every step's density
        (dgb_batchnd_integrate_states), each set's loss tail by autograd, and
        one batched adjoint (dgb_batchnd_adjoint), so that every sweep launch
        carries the lines of all the sets.  Returns [(ll, grad, fs)] in the
        order of thetas, each bitwise the one-at-a-time result."""
        torch = self.torch
        thetas = [np.asarray(t, dtype=np.float64) for t in thetas]
        d = data if torch.is_tensor(data) else _lib.to_device(torch, data)
        tabs = [[self.table(th, xx) for xx in self.xxs] for th in thetas]
        nbytes = [sum(8 * (len(tabs[i][g][0]) + 1) * L ** self.P
                      for g, L in enumerate(self.pts_l)) for i in range(len(thetas))]
        budget = self.states_budget
        if budget is None:
            budget = torch.cuda.mem_get_info()[0] // 2
        ngroups = max(1, -(-sum(nbytes) // int(budget)))
        bounds = np.searchsorted(np.cumsum(nbytes), np.arange(1, ngroups) * sum(nbytes) / ngroups)
        out = [None] * len(thetas)
        for grp in np.split(np.arange(len(thetas)), bounds):
            if len(grp):
                self._grad_group([int(i) for i in grp], tabs, d, scale, out)
        return out

    def _grad_group(self, grp, tabs, d, scale, out):
        torch, lib = self.torch, _lib.lib()
        P, m = self.P, len(grp)
        st = _lib.settings_struct(*integration.current_settings())
        sh = _lib.stream_handle(torch)
        stride = integration.row_stride(P)
        runs = []
        for g, (L, xx) in enumerate(zip(self.pts_l, self.xxs)):
            N = L ** P
            steps = np.array([len(tabs[i][g][0]) for i in grp], dtype=np.int64)
            order = np.argsort(-steps, kind="stable")
            per = int(lib.dgb_adjoint_table_nd_gpart_doubles(P, L))
            items = (_lib.ItemNDAdj * m)()
            slot = np.empty(m, dtype=np.int64)   # set (position in grp) -> slot
            row = state = gp = 0
            for pos, j in enumerate(order):
                it = items[pos]
                it.phi_off, it.row_off, it.state_off, it.gpart_off = pos * N, row, state, gp
                it.nsteps, it.masks = int(steps[j]), 0
                slot[j] = pos
                row += int(steps[j])
                state += (int(steps[j]) + 1) * N
                gp += int(steps[j]) * per
            table = np.concatenate([tabs[grp[j]][g][0] for j in order] +
                                   [np.zeros((1, stride))])
            phi = _lib.to_device(torch, self.initial(xx)).reshape(1, N).expand(m, N).contiguous()
            states = torch.empty(max(state, 1), dtype=torch.float64, device="cuda")
            gpart = torch.empty(max(gp, 1), dtype=torch.float64, device="cuda")
            d_xx, d_tab = _lib.to_device(torch, xx), _lib.to_device(torch, table)
            ws, nws = _lib.workspace(torch, lib.dgb_batchnd_adjoint_workspace_bytes(
                P, L, m, ctypes.byref(st)))
            _lib.check(lib.dgb_batchnd_integrate_states(
                ctypes.byref(items), m, P, L, _lib.dptr(d_xx), _lib.dptr(phi), _lib.dptr(d_tab),
                _lib.dptr(states), ctypes.byref(st), _lib.dptr(ws), nws, sh),
                "dgb_batchnd_integrate_states")
            runs.append(dict(L=L, N=N, per=per, items=items, slot=slot, phi=phi, states=states,
                             gpart=gpart, d_xx=d_xx, d_tab=d_tab, ws=ws, nws=nws,
                             lam=torch.zeros_like(phi)))
        for k, i in enumerate(grp):
            phis = [r["phi"][r["slot"][k]].view((r["L"],) * P).detach().requires_grad_(True)
                    for r in runs]
            with torch.enable_grad():
                fs, ll = self._tail(phis, d, scale)
            lams = torch.autograd.grad(ll, phis, allow_unused=True)
            for r, lam in zip(runs, lams):
                if lam is not None:
                    r["lam"][r["slot"][k]] = lam.reshape(-1)
            out[i] = (ll.detach(), fs.detach())
        for r in runs:
            _lib.check(lib.dgb_batchnd_adjoint(
                ctypes.byref(r["items"]), m, P, r["L"], _lib.dptr(r["d_xx"]),
                _lib.dptr(r["lam"]), _lib.dptr(r["d_tab"]), _lib.dptr(r["states"]),
                _lib.dptr(r["gpart"]), ctypes.byref(st), _lib.dptr(r["ws"]), r["nws"], sh),
                "dgb_batchnd_adjoint")
            r["states"] = None
        for k, i in enumerate(grp):
            grad = torch.zeros(self.npar, dtype=torch.float64, device="cuda")
            for g, r in enumerate(runs):
                n = len(tabs[i][g][0])
                if n == 0:
                    continue
                it = r["items"][int(r["slot"][k])]
                gpart = r["gpart"][it.gpart_off:it.gpart_off + n * r["per"]]
                grad += _row_grads(torch, gpart, n, r["per"], stride, tabs[i][g][1])
            ll, fs = out[i]
            out[i] = (ll, grad, fs)

    def loglik_and_grad_many(self, thetas, data, scale=1.0, workers=4):
        """loglik_and_grad for several parameter sets, `workers` at a time on
        their own threads and CUDA streams (one set's sweeps leave most SMs
        idle).  Returns [(ll, grad, fs)] in the order of thetas."""
        torch = self.torch
        from concurrent.futures import ThreadPoolExecutor
        dev = torch.cuda.current_device()
        d = data if torch.is_tensor(data) else _lib.to_device(torch, data)

        def one(th):
            with torch.cuda.device(dev), torch.cuda.stream(torch.cuda.Stream()):
                ll, g, fs = self.loglik_and_grad(th, d, scale)
                torch.cuda.current_stream().synchronize()
                return ll, g, fs
        with ThreadPoolExecutor(max_workers=max(1, int(workers))) as ex:
            return list(ex.map(one, list(thetas)))


class Growth3(TableModel):
    """models.growth3 with parameters theta = (nu0_1, nu0_2, nu0_3, nuF_1,
    nuF_2, nuF_3, m12, m13, m23, T) and fixed gammas (default: the
    3-population workload's (-2, 0, 5)), h = 0.5, theta0 = 1."""

    P = 3
    npar = 10

    def __init__(self, pts_l, ns, gammas=(-2.0, 0.0, 5.0)):
        super().__init__(pts_l, ns)
        self.gammas = tuple(float(g) for g in gammas)

    @staticmethod
    def from_model_params(p):
        """models.growth3 parameters ((nu0..), (nuF..), (m12, m13, m23),
        gammas, T) -> theta."""
        nu0, nuF, m, _, T = p
        return np.array(list(nu0) + list(nuF) + list(m) + [T], dtype=np.float64)

    def model_params(self, theta):
        th = [float(v) for v in theta]
        return (tuple(th[0:3]), tuple(th[3:6]), tuple(th[6:9]), self.gammas, th[9])

    def initial(self, xx):
        phi = phimanip.phi_1D_to_2D(xx, phimanip.phi_1D(xx))
        return phimanip.phi_2D_to_3D_split_2(xx, phi)

    def table(self, theta, xx):
        """The parameter table and its derivatives, walked in C."""
        from . import batchnd
        th = [float(v) for v in theta]
        rec = batchnd.growth3_instance(self.model_params(th))
        seed = _lib.SeedND()
        for i in range(3):
            seed.dnu[i][0][i] = 1.0       # nu0_i
            seed.dnu[i][1][3 + i] = 1.0   # nuF_i
            seed.dnu[i][2][9] = 1.0       # the growth time is T
        for q, (k, j) in zip((6, 7, 8), ((0, 1), (0, 2), (1, 2))):
            seed.dmig[k][j][0][q] = seed.dmig[j][k][0][q] = 1.0
        seed.dT[9] = 1.0
        return schedule_dual(rec, seed, self.npar, xx)

    def table_python(self, theta, xx):
        """The same table walked in Python (table_dual)."""
        th = np.asarray(theta, dtype=np.float64)
        e = np.eye(self.npar)
        T = th[9]
        nus = [Form(PF_EXPLOG, th[i], th[3 + i], T, da=e[i], db=e[3 + i], dc=e[9],
                    npar=self.npar) for i in range(3)]
        mi = {(0, 1): 6, (0, 2): 7, (1, 2): 8}
        mig = [[None] * 3 for _ in range(3)]
        for k in range(3):
            for j in range(3):
                if j != k:
                    q = mi[(min(k, j), max(k, j))]
                    mig[k][j] = Form(PF_CONST, th[q], da=e[q], npar=self.npar)
        gam = [Form(PF_CONST, g, npar=self.npar) for g in self.gammas]
        hs = [Form(PF_CONST, 0.5, npar=self.npar) for _ in range(3)]
        th0 = Form(PF_CONST, 1.0, npar=self.npar)
        return table_dual(3, xx, T, e[9], nus, mig, gam, hs, th0)


def from_phi_torch(torch, phi, ns, xx):
    """Spectrum.from_phi for 1-3 populations as differentiable torch ops on
    the GPU (the contraction of dadi/Spectrum_mod.py:1509-1547, and for three
    populations the loop over the third axis of :1774-1810 as one batched
    product)."""
    P = phi.dim()
    if P == 2:
        return spectrum.from_phi_2D_batch(torch, phi[None], ns[0], ns[1], xx)[0]
    if P == 3:
        nz = ns[2]
        d1z, d2z, x = spectrum._device_tables(torch, nz, xx, phi.device)
        dxv = x[1:] - x[:-1]
        s_z = (phi[:, :, 1:] - phi[:, :, :-1]) / dxv
        c1_z = (phi[:, :, :-1] - s_z * x[:-1]) / (nz + 1)
        w = torch.arange(1, nz + 2, dtype=torch.float64, device=phi.device) / \
            ((nz + 1) * (nz + 2))
        over = torch.einsum("ijk,bk->bij", c1_z, d1z) + \
            w[:, None, None] * torch.einsum("ijk,bk->bij", s_z, d2z)
        fs = spectrum.from_phi_2D_batch(torch, over.contiguous(), ns[0], ns[1], xx)
        return fs.permute(1, 2, 0).contiguous()
    raise NotImplementedError("from_phi_torch handles 2 or 3 populations")
