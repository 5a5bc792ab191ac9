"""Discrete-adjoint gradients of the Poisson log-likelihood of extrapolated 2-D
IM spectra, against finite differences of the same GPU forward and against
dadi's own Godambe.get_grad on the CPU reference (golden vector).

Central differences with eps = 1e-4 (relative; the step Godambe.get_grad
uses, dadi/Godambe.py:131-185) carry an O(eps^2) truncation error that, for
the extrapolated likelihood, reaches ~1e-5 of the gradient's max norm in the
T component; halving eps divides it by 4.  So the adjoint is held to 1e-6
(max-norm relative) against the Richardson combination (4 D(eps/2) - D(eps))/3
of two central differences, and against Godambe.get_grad with that same
truncation estimate removed.
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-6
PTS = (20, 25, 30)
NS = (10, 10)


def _engine(pts=PTS):
    from dadi_gb300 import batch
    return batch.Batch2D(pts, NS)


def _ll(eng, params, data, scale):
    fs, ll, st = eng.run(np.atleast_2d(params), data=data, scale=scale)
    return ll.cpu().numpy()


def _central_fd(eng, p, data, scale, eps):
    g = np.zeros(6)
    for k in range(6):
        h = eps * p[k]
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        g[k] = (_ll(eng, pp, data, scale)[0] - _ll(eng, pm, data, scale)[0]) / (2 * h)
    return g


def _fd_pair(eng, p, data, scale, eps=1e-4):
    d1 = _central_fd(eng, p, data, scale, eps)
    d2 = _central_fd(eng, p, data, scale, eps / 2)
    return d1, (4 * d2 - d1) / 3


def _close(g, ref):
    return float(np.max(np.abs(g - ref)) / np.max(np.abs(ref)))


def test_adjoint_matches_finite_differences_and_godambe(cuda_lib, golden):
    g = golden["grad"]
    p0 = g["grad_p0"]
    data = g["grad_data"]
    eng = _engine()
    ll, grad, st = eng.loglik_and_grad(p0[None, :], data, scale=1e4)
    assert int(st.abs().sum()) == 0
    adj = grad.cpu().numpy()[0]
    fd, rich = _fd_pair(eng, p0, data, 1e4)
    assert _close(adj, rich) < GRAD_TOL, (adj, rich)
    # the reference's eps=1e-4 gradient equals ours at the same eps ...
    assert _close(fd, g["grad_godambe"]) < 1e-7
    # ... and, with the truncation error estimated from the eps pair removed,
    # the adjoint
    godambe_corrected = g["grad_godambe"] + (rich - fd)
    assert _close(adj, godambe_corrected) < GRAD_TOL, (adj, godambe_corrected)


def test_adjoint_single_grid_matches_fd(cuda_lib, golden):
    g = golden["grad"]
    eng = _engine((30,))
    ll, grad, st = eng.loglik_and_grad(g["grad_p0"][None, :], g["grad_data"], scale=1e4)
    fd, rich = _fd_pair(eng, g["grad_p0"], g["grad_data"], 1e4)
    assert _close(grad.cpu().numpy()[0], rich) < GRAD_TOL
    assert _close(grad.cpu().numpy()[0], fd) < GRAD_TOL


def test_adjoint_batch_matches_alone(cuda_lib, golden):
    """Several parameter sets in one adjoint launch give each set's own
    gradient (within 1e-10: the loss seeds pass through cuBLAS matrix
    products whose summation order depends on the batch size), and the
    gradient agrees with finite differences for sets with different step
    counts."""
    from dadi_gb300 import batch
    draws = cases.im_draws(4096)
    steps = batch.count_steps(batch.im_instances(draws))
    sel = [i for i in range(64) if 30 <= steps[i] <= 1500][:4]
    data = golden["grad"]["grad_data"]
    eng = _engine()
    ll, grad, st = eng.loglik_and_grad(draws[sel], data, scale=1e4)
    grad = grad.cpu().numpy()
    for k, i in enumerate(sel):
        _, g1, _ = eng.loglik_and_grad(draws[i][None, :], data, scale=1e4)
        assert _close(grad[k], g1.cpu().numpy()[0]) < 1e-10
    fd, rich = _fd_pair(eng, draws[sel[0]], data, 1e4)
    assert _close(grad[0], rich) < GRAD_TOL, (grad[0], rich)


def test_autograd_function(cuda_lib, golden):
    import torch
    from dadi_gb300 import batch
    g = golden["grad"]
    eng = _engine()
    p = torch.tensor(g["grad_p0"][None, :], dtype=torch.float64, requires_grad=True)
    ll = batch.IMLogLik.apply(eng, p, g["grad_data"], 1e4)
    ll.sum().backward()
    _, direct, _ = eng.loglik_and_grad(g["grad_p0"][None, :], g["grad_data"], scale=1e4)
    assert _close(p.grad.numpy()[0], direct.cpu().numpy()[0]) < 1e-12


def test_adjoint_trajectory_mode_is_bitwise(cuda_lib, golden):
    """Recomputing every checkpoint segment at once into a stored trajectory
    (dgb_adjoint2d_traj) gives the gradients of the segment-by-segment
    adjoint bit for bit, for sets with different step counts and a
    checkpoint interval that leaves a partial last segment."""
    from dadi_gb300 import batch
    draws = cases.im_draws(4096)
    steps = batch.count_steps(batch.im_instances(draws))
    sel = [i for i in range(64) if 30 <= steps[i] <= 1500][:5]
    data = golden["grad"]["grad_data"]
    eng = _engine()
    eng.cluster_adjoint = 0
    for C in (None, 7):
        _, g_seg, _ = eng.loglik_and_grad(draws[sel], data, scale=1e4, ckpt_every=C,
                                          trajectory=False)
        _, g_traj, _ = eng.loglik_and_grad(draws[sel], data, scale=1e4, ckpt_every=C,
                                           trajectory=True)
        assert np.array_equal(g_seg.cpu().numpy(), g_traj.cpu().numpy()), C


def test_adjoint_hybrid_mode_is_bitwise(cuda_lib, golden):
    """With a trajectory budget that holds only the longest work items, those
    walk back from a stored trajectory on the current stream while the rest
    recompute their segments on a side stream (dgb_adjoint2d_part twice);
    the gradients are the segment-by-segment adjoint's bit for bit."""
    from dadi_gb300 import batch
    draws = cases.im_draws(4096)
    steps = batch.count_steps(batch.im_instances(draws))
    sel = [i for i in range(64) if 30 <= steps[i] <= 1500][:6]
    data = golden["grad"]["grad_data"]
    eng = _engine()
    _, g_seg, _ = eng.loglik_and_grad(draws[sel], data, scale=1e4, ckpt_every=7,
                                      trajectory=False)
    ll, ctx = eng.forward_for_adjoint(draws[sel], data, scale=1e4, ckpt_every=7)
    eng.traj_budget = eng.trajectory_bytes(ctx) // 3   # about a third of the items
    try:
        _, g_hyb, _ = eng.loglik_and_grad(draws[sel], data, scale=1e4, ckpt_every=7)
    finally:
        eng.traj_budget = batch.Batch2D.traj_budget
    assert np.array_equal(g_seg.cpu().numpy(), g_hyb.cpu().numpy())


def test_forward_of_few_items_on_clusters(cuda_lib, golden):
    """The gradient's forward of a few integrations on thread-block clusters
    (with checkpoints) gives the one-CTA forward's likelihoods to 1e-12 and
    gradients to 1e-9 (the cluster's partitioned solves round
    differently)."""
    from dadi_gb300 import batch
    draws = cases.im_draws(4096)
    steps = batch.count_steps(batch.im_instances(draws))
    sel = [i for i in range(64) if 30 <= steps[i] <= 1500][:4]
    data = golden["grad"]["grad_data"]
    eng = batch.Batch2D((30, 40, 50), NS)
    eng.cluster_forward = False
    eng.cluster_adjoint = 0
    ll0, g0, _ = eng.loglik_and_grad(draws[sel], data, scale=1e4)
    eng.cluster_forward = True
    eng._split_keep = None
    ll1, g1, st = eng.loglik_and_grad(draws[sel], data, scale=1e4)
    assert eng._split_keep is not None and int(st.abs().sum()) == 0
    ll0, ll1 = ll0.cpu().numpy(), ll1.cpu().numpy()
    assert np.max(np.abs(ll1 - ll0) / np.abs(ll0)) < 1e-12
    g0, g1 = g0.cpu().numpy(), g1.cpu().numpy()
    assert float(np.max(np.abs(g1 - g0)) / np.max(np.abs(g0))) < 1e-9


@pytest.mark.parametrize("pts,ctas", [((30,), 2), ((30, 40, 50), 4), ((30, 40, 50), 8),
                                      ((50, 60), 16)])
def test_adjoint_on_clusters_matches_one_cta(cuda_lib, golden, pts, ctas):
    """The trajectory-mode backward walk on thread-block clusters of 2-16
    CTAs (dgb_adjoint2d_part with a cluster size) against the one-CTA walk
    on the same forward: gradients within 1e-10 (max-norm relative; the
    partitioned solves and the split contraction sums round differently),
    also with a frozen or a mutation-free population (the masks set on the
    context, the same for both walks)."""
    import torch
    from dadi_gb300 import batch
    draws = cases.im_draws(4096)
    steps = batch.count_steps(batch.im_instances(draws))
    sel = [i for i in range(64) if 30 <= steps[i] <= 1500][:2]
    data = golden["grad"]["grad_data"]
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    eng = batch.Batch2D(pts, NS)
    eng.cluster_forward = False
    for mask in (0, 1, 2, 1 << 8, 2 << 8):
        out = []
        for c in (0, ctas):
            eng.cluster_adjoint = c
            ll, ctx = eng.forward_for_adjoint(draws[sel], data, scale=1e4, ckpt_every=7)
            ctx["masks"].fill_(mask)
            assert eng._cluster_adjoint_ctas(ctx, nsm) == c
            out.append(eng.adjoint(ctx, torch.ones_like(ll), trajectory=True).cpu().numpy())
        assert np.all(np.isfinite(out[1]))
        assert _close(out[1], out[0]) < 1e-10, (mask, _close(out[1], out[0]))


def test_hybrid_adjoint_with_clusters(cuda_lib, golden):
    """The hybrid adjoint with its longest trajectory-mode items walked on
    clusters of 8 CTAs, the other trajectory items on one CTA each and the
    rest in segment mode, on three streams: the segment-mode gradients
    within 1e-10."""
    from dadi_gb300 import batch
    draws = cases.im_draws(4096)
    steps = batch.count_steps(batch.im_instances(draws))
    sel = [i for i in range(64) if 30 <= steps[i] <= 1500][:6]
    data = golden["grad"]["grad_data"]
    eng = batch.Batch2D((30, 40, 50), NS)
    eng.cluster_forward = False
    eng.hybrid_cluster_items = 4
    _, g_seg, _ = eng.loglik_and_grad(draws[sel], data, scale=1e4, ckpt_every=7,
                                      trajectory=False)
    ll, ctx = eng.forward_for_adjoint(draws[sel], data, scale=1e4, ckpt_every=7)
    eng.traj_budget = eng.trajectory_bytes(ctx) // 3
    try:
        _, g_hyb, st = eng.loglik_and_grad(draws[sel], data, scale=1e4, ckpt_every=7)
    finally:
        eng.traj_budget = batch.Batch2D.traj_budget
    g_seg, g_hyb = g_seg.cpu().numpy(), g_hyb.cpu().numpy()
    assert int(st.abs().sum()) == 0 and np.all(np.isfinite(g_hyb))
    assert _close(g_hyb, g_seg) < 1e-10


def test_cluster_walk_rejects_what_it_does_not_solve(cuda_lib):
    """dgb_adjoint2d_part with a cluster size: sizes other than 2, 4, 8, 16
    or no trajectory are DGB_ERR_ARG, grids outside 24-128 points or 3-16
    rows per CTA DGB_ERR_UNSUPPORTED, all before any launch."""
    import ctypes
    import torch
    from dadi_gb300 import _lib
    lib = cuda_lib
    buf = torch.zeros(1024, dtype=torch.float64, device="cuda")
    p = _lib.dptr(buf)
    st = _lib.settings_struct()
    ws, nws = _lib.workspace(torch, 4096)

    def call(Ls, cluster, traj=True):
        arr = (ctypes.c_int * len(Ls))(*Ls)
        t = p if traj else None
        return lib.dgb_adjoint2d_part(p, 1, arr, len(Ls), p, p, p, p, p, p, p, 1, t, t, t, p,
                                      p, p, 1, 0, cluster, ctypes.byref(st), _lib.dptr(ws), nws,
                                      _lib.stream_handle(torch))

    assert call([40], 3) == _lib.DGB_ERR_ARG
    assert call([40], 8, traj=False) == _lib.DGB_ERR_ARG
    for Ls, c in (([20], 8), ([130], 16), ([40], 2), ([30], 16), ([40, 20], 8)):
        assert call(Ls, c) == _lib.DGB_ERR_UNSUPPORTED, (Ls, c)
    torch.cuda.synchronize()


def test_device_schedules_match_host_schedules(cuda_lib):
    """The schedule pass on the device (dgb_sched2d: two lanes per schedule
    exchanging their timesteps) against the host walk (dgb_sched2d_host):
    the same row counts and status bits, NaN in the same places and rows
    within 1e-10 relative, for 512 seed-0 IM draws -- three of them with bad
    parameters -- under the default and the old timestep rule.  Device and
    host pow may round a size differently by an ulp; through the running
    time, over up to 19,546 steps of T down to 0.01, that reaches 5e-12 of
    a row's sizes."""
    import ctypes
    import torch
    from dadi_gb300 import _lib, batch, serving
    lib = cuda_lib
    draws = cases.im_draws(512).copy()
    draws[3, 1] = -1.0      # nu1 < 0
    draws[7, 2] = 0.0       # nu2 == 0
    draws[11, 4] = -2.0     # m12 < 0
    rec = np.ascontiguousarray(batch.im_instances(draws))
    n = len(rec)
    d_rec = _lib.to_device(torch, rec.view(np.uint8), np.uint8)
    dx0 = 0.01
    d_dx0 = torch.tensor([dx0], dtype=torch.float64, device="cuda")
    sh = _lib.stream_handle(torch)
    for old in (False, True):
        st = _lib.settings_struct(use_old_timestep=old)
        tab_h, off_h, cnt_h, stat_h = serving.host_schedules(rec, st, dx0)
        assert np.count_nonzero(stat_h) >= 3
        cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
        _lib.check(lib.dgb_sched2d(_lib.dptr(d_rec), n, 1, _lib.dptr(d_dx0), ctypes.byref(st),
                                   10 ** 7, 0, _lib.dptr(cnt), None, None, None, sh),
                   "dgb_sched2d(count)")
        assert np.array_equal(cnt.cpu().numpy(), cnt_h)
        d_off = torch.from_numpy(off_h).cuda()
        rows = int(cnt_h.sum())
        table = torch.zeros(max(rows, 1) * 11, dtype=torch.float64, device="cuda")
        status = torch.zeros(n, dtype=torch.int32, device="cuda")
        _lib.check(lib.dgb_sched2d(_lib.dptr(d_rec), n, 1, _lib.dptr(d_dx0), ctypes.byref(st),
                                   10 ** 7, 1, _lib.dptr(cnt), _lib.dptr(d_off),
                                   _lib.dptr(table), _lib.dptr(status), sh), "dgb_sched2d(fill)")
        assert np.array_equal(status.cpu().numpy(), stat_h)
        a, b = table.cpu().numpy()[:rows * 11], tab_h[:rows * 11]
        # a negative size gives NaN rows on both sides (not a status bit)
        assert np.array_equal(np.isnan(a), np.isnan(b))
        ok = ~np.isnan(b)
        assert np.max(np.abs(a[ok] - b[ok]) / np.maximum(np.abs(b[ok]), 1e-300)) <= 1e-10, old
