"""Discrete adjoint of the N-dimensional time loop on the three-population
growth model (the 3-D part of the gradient workload): against central finite
differences of the same GPU forward, 1e-6 max-norm relative.

As for the 2-D adjoint, central differences carry an O(eps^2) truncation
error, so the bar is applied to the Richardson combination
(4 D(eps/2) - D(eps)) / 3.  The likelihood is strongly curved in m13, m23
and T here: measured against the adjoint, the Richardson error of those
components falls 16-fold per halving of eps (6e-4, 3e-5, 2e-6, 1.3e-7 of
the gradient's max norm for eps = 2e-4 ... 2.5e-5), the O(eps^4) of the
combination, while the other components sit at 1e-10..1e-9; so the pair
eps = 5e-5, 2.5e-5 is used.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-6


def _theta():
    """The workload's parameters with T moved off an integer number of steps
    (at exactly 675 steps of 1e-3 / 4.5 the likelihood has a kink in the
    parameters that set dt, and finite differences straddle it)."""
    from dadi_gb300 import adjoint_nd, models
    th = adjoint_nd.Growth3.from_model_params(models.GROWTH3_DEFAULT)
    th[9] = 0.1537
    return th


def _fd(model, theta, data, scale, eps):
    g = np.zeros(len(theta))
    for k in range(len(theta)):
        h = eps * theta[k]
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        lp = float(model.spectrum_ll(tp, data, scale)[1])
        lm = float(model.spectrum_ll(tm, data, scale)[1])
        g[k] = (lp - lm) / (2 * h)
    return g


@pytest.mark.parametrize("pts_l", [(16,), (16, 20)])
def test_growth3_gradient_matches_fd(cuda_lib, pts_l):
    from dadi_gb300 import adjoint_nd
    model = adjoint_nd.Growth3(pts_l, (6, 6, 6))
    theta = _theta()
    fs0, _ = model.spectrum_ll(theta)
    data = np.random.default_rng(0).poisson(1e3 * np.abs(fs0.cpu().numpy())).astype(float)
    ll, grad, fs = model.loglik_and_grad(theta, data, 1e3)
    grad = grad.cpu().numpy()
    d1 = _fd(model, theta, data, 1e3, 5e-5)
    d2 = _fd(model, theta, data, 1e3, 2.5e-5)
    rich = (4 * d2 - d1) / 3
    err = np.max(np.abs(grad - rich)) / np.max(np.abs(rich))
    assert err < GRAD_TOL, (grad, rich, err)


def test_growth3_spectrum_matches_dropin(cuda_lib):
    """The gradient engine's forward is the drop-in growth3 model's."""
    from dadi_gb300 import adjoint_nd, models, numerics
    from util import assert_fs_parity
    model = adjoint_nd.Growth3((16, 20, 24), (6, 6, 6))
    theta = _theta()
    fs, _ = model.spectrum_ll(theta)
    ref = numerics.make_extrap_func(models.growth3)(model.model_params(theta), (6, 6, 6),
                                                     [16, 20, 24])
    assert_fs_parity(fs.cpu().numpy(), np.asarray(ref.data))


def test_many_sets_concurrently_equal_one_at_a_time(cuda_lib):
    """Concurrent gradient evaluation (threads + streams) gives each set's
    own gradient, bitwise."""
    from dadi_gb300 import adjoint_nd
    model = adjoint_nd.Growth3((16,), (6, 6, 6))
    th = _theta()
    sets = [th * f for f in (1.0, 0.9, 1.1)]
    data = np.ones((7, 7, 7))
    many = model.loglik_and_grad_many(sets, data, 10.0, workers=3)
    for t, (ll, g, fs) in zip(sets, many):
        ll1, g1, _ = model.loglik_and_grad(t, data, 10.0)
        assert float(ll) == float(ll1)
        assert np.array_equal(g.cpu().numpy(), g1.cpu().numpy())


@pytest.mark.parametrize("P,L,frozen", [(3, 14, 0), (3, 12, 4), (4, 8, 0)])
def test_adjoint_records_match_inline_setup(cuda_lib, P, L, frozen):
    """dgb_integrate_table_states and dgb_adjoint_table_nd give bitwise the
    same states, dJ/dphi_initial and per-step row gradients whether the
    recomputed sweeps read coefficient records (workspace kind 4) or build
    their coefficients in every CTA (the minimal workspace), over 300 steps
    (more than one chunk of records, walked backwards)."""
    import torch
    from dadi_gb300 import _lib
    import cases
    from util import table_rows
    lib = cuda_lib
    xx = cases.grid("default", L)
    N = L ** P
    tab = table_rows(P, 300, seed=7 * P + L)
    n = len(tab)
    d_xx = torch.from_numpy(xx).cuda()
    d_tab = torch.from_numpy(tab).cuda()
    phi0 = np.abs(cases.initial_phi(5, (L,) * P)) + 1e-3
    lam0 = cases.initial_phi(6, (L,) * P) - 0.5
    na = P - bin(frozen).count("1")
    per = lib.dgb_adjoint_table_nd_gpart_doubles(P, L)
    sh = _lib.stream_handle(torch)
    res = []
    for fwd_ws, adj_ws in ((0, (na - 1) * N * 8), (lib.dgb_workspace_bytes(0, P, L, 0),
                                                    lib.dgb_workspace_bytes(4, P, L, 0))):
        d_phi = torch.from_numpy(phi0.copy()).cuda()
        states = torch.empty((n + 1) * N, dtype=torch.float64, device="cuda")
        ws, nws = _lib.workspace(torch, fwd_ws)
        _lib.check(lib.dgb_integrate_table_states(
            _lib.dptr(d_phi), P, L, _lib.dptr(d_xx), _lib.dptr(d_tab), n, frozen, 0,
            _lib.dptr(states), _lib.dptr(ws) if fwd_ws else None, fwd_ws, sh),
            "dgb_integrate_table_states")
        lam = torch.from_numpy(lam0.copy()).cuda()
        gpart = torch.empty(n * per, dtype=torch.float64, device="cuda")
        ws2, nws2 = _lib.workspace(torch, adj_ws)
        _lib.check(lib.dgb_adjoint_table_nd(
            _lib.dptr(lam), P, L, _lib.dptr(d_xx), _lib.dptr(d_tab), n, frozen, 0,
            _lib.dptr(states), _lib.dptr(gpart), _lib.dptr(ws2), nws2, sh),
            "dgb_adjoint_table_nd")
        res.append((states.cpu().numpy(), lam.cpu().numpy(), gpart.cpu().numpy()))
    for a, b in zip(res[0], res[1]):
        assert np.all(np.isfinite(a))
        assert np.array_equal(a, b)


@pytest.mark.parametrize("P,L,frozen", [(3, 12, [0, 0, 0, 0]), (3, 14, [0, 4, 0, 1]),
                                        (4, 7, [0, 0, 2, 0]), (2, 20, [0, 1, 0, 0]),
                                        (1, 30, [0, 0, 0, 0])])
def test_batched_adjoint_equals_one_at_a_time(cuda_lib, P, L, frozen):
    """dgb_batchnd_integrate_states + dgb_batchnd_adjoint over four
    integrations of different lengths (and frozen populations) give each one
    bitwise the recorded densities, dJ/dphi_initial and per-step partial rows
    of dgb_integrate_table_states + dgb_adjoint_table_nd run for it alone."""
    import ctypes
    import torch
    from dadi_gb300 import _lib, batchnd
    import cases
    from util import table_rows
    lib = cuda_lib
    xx = cases.grid("default", L)
    N = L ** P
    nst = [23, 23, 9, 0] if P > 1 else [30, 12, 5, 1]
    tabs = [table_rows(P, n, 500 + k) for k, n in enumerate(nst)]
    phi0 = [np.abs(cases.initial_phi(70 + k, (L,) * P)) + 1e-3 for k in range(4)]
    lam0 = [np.random.default_rng(80 + k).normal(size=(L,) * P) for k in range(4)]
    d_xx = torch.from_numpy(xx).cuda()
    sh = _lib.stream_handle(torch)
    per = lib.dgb_adjoint_table_nd_gpart_doubles(P, L)
    alone = []
    for k in range(4):
        n = nst[k]
        d_phi = torch.from_numpy(phi0[k].copy()).cuda()
        d_tab = torch.from_numpy(np.concatenate([tabs[k], np.zeros((1, tabs[k].shape[1]))])).cuda()
        states = torch.empty((n + 1) * N, dtype=torch.float64, device="cuda")
        ws, nws = _lib.workspace(torch, lib.dgb_workspace_bytes(0, P, L, 0))
        _lib.check(lib.dgb_integrate_table_states(
            _lib.dptr(d_phi), P, L, _lib.dptr(d_xx), _lib.dptr(d_tab), n, frozen[k], 0,
            _lib.dptr(states), _lib.dptr(ws), nws, sh), "dgb_integrate_table_states")
        lam = torch.from_numpy(lam0[k].copy()).cuda()
        gpart = torch.zeros(max(n * per, 1), dtype=torch.float64, device="cuda")
        ws2, nws2 = _lib.workspace(torch, lib.dgb_workspace_bytes(4, P, L, 0))
        if n:
            _lib.check(lib.dgb_adjoint_table_nd(
                _lib.dptr(lam), P, L, _lib.dptr(d_xx), _lib.dptr(d_tab), n, frozen[k], 0,
                _lib.dptr(states), _lib.dptr(gpart), _lib.dptr(ws2), nws2, sh),
                "dgb_adjoint_table_nd")
        alone.append((states.cpu().numpy(), lam.cpu().numpy(), gpart.cpu().numpy()[:n * per]))
    order = np.argsort(-np.array(nst), kind="stable")
    items = (_lib.ItemNDAdj * 4)()
    row = state = gp = 0
    for pos, k in enumerate(order):
        it = items[pos]
        it.phi_off, it.row_off, it.state_off, it.gpart_off = k * N, row, state, gp
        it.nsteps, it.masks = nst[k], frozen[k]
        row += nst[k]
        state += (nst[k] + 1) * N
        gp += nst[k] * per
    table = np.concatenate([tabs[k] for k in order] + [np.zeros((1, tabs[0].shape[1]))])
    d_tab = torch.from_numpy(table).cuda()
    phi = torch.from_numpy(np.concatenate([p.reshape(-1) for p in phi0])).cuda()
    lam = torch.from_numpy(np.concatenate([x.reshape(-1) for x in lam0])).cuda()
    states = torch.empty(state, dtype=torch.float64, device="cuda")
    gpart = torch.empty(max(gp, 1), dtype=torch.float64, device="cuda")
    st = batchnd.integration_settings()
    ws, nws = _lib.workspace(torch, lib.dgb_batchnd_adjoint_workspace_bytes(P, L, 4,
                                                                           ctypes.byref(st)))
    _lib.check(lib.dgb_batchnd_integrate_states(
        ctypes.byref(items), 4, P, L, _lib.dptr(d_xx), _lib.dptr(phi), _lib.dptr(d_tab),
        _lib.dptr(states), ctypes.byref(st), _lib.dptr(ws), nws, sh), "integrate_states")
    _lib.check(lib.dgb_batchnd_adjoint(
        ctypes.byref(items), 4, P, L, _lib.dptr(d_xx), _lib.dptr(lam), _lib.dptr(d_tab),
        _lib.dptr(states), _lib.dptr(gpart), ctypes.byref(st), _lib.dptr(ws), nws, sh),
        "dgb_batchnd_adjoint")
    states, lam, gpart = states.cpu().numpy(), lam.cpu().numpy(), gpart.cpu().numpy()
    for pos, k in enumerate(order):
        it = items[pos]
        s_ref, l_ref, g_ref = alone[k]
        assert np.array_equal(states[it.state_off:it.state_off + (nst[k] + 1) * N], s_ref), k
        assert np.array_equal(lam[k * N:(k + 1) * N], l_ref.reshape(-1)), k
        assert np.array_equal(gpart[it.gpart_off:it.gpart_off + nst[k] * per], g_ref), k


def test_growth3_batched_gradients_equal_one_at_a_time(cuda_lib):
    """loglik_and_grad_batch (every set's sweeps in the same launches, two
    groups by the states budget) gives each set bitwise its one-at-a-time
    likelihood, gradient and spectrum."""
    from dadi_gb300 import adjoint_nd
    model = adjoint_nd.Growth3((16, 20), (6, 6, 6))
    th = _theta()
    sets = [th * f for f in (1.0, 0.9, 1.1, 1.3, 0.7)]
    fs0, _ = model.spectrum_ll(th)
    data = np.random.default_rng(1).poisson(1e3 * np.abs(fs0.cpu().numpy())).astype(float)
    model.states_budget = 3 * 8 * 350 * (16 ** 3 + 20 ** 3)   # about two groups
    batch = model.loglik_and_grad_batch(sets, data, 1e3)
    for t, (ll, g, fs) in zip(sets, batch):
        ll1, g1, fs1 = model.loglik_and_grad(t, data, 1e3)
        assert float(ll) == float(ll1)
        assert np.array_equal(g.cpu().numpy(), g1.cpu().numpy())
        assert np.array_equal(fs.cpu().numpy(), fs1.cpu().numpy())
