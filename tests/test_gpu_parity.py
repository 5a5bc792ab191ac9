"""CUDA path against the reference: every single sweep, the tridiagonal
solver, every integration case and the model pipelines, compared with golden
vectors produced by dadi 2.4.3 and with the oracle.

Tolerances: single sweeps and solves 1e-12 relative (a few ulps of
reassociation); whole integrations 1e-9 relative per entry (entries below
1e-12 of the array maximum compared absolutely); extrapolated spectra 1e-9
relative on every entry, the bar the work is held to.
"""
import ctypes

import numpy as np
import pytest

import cases
from util import ALL_CASES, assert_fs_parity, case_inputs, fs_parity, max_rel, table_rows

pytestmark = pytest.mark.gpu

SWEEP_TOL = 1e-12
# The delj trick's delta_j = (-e w + e V - V)/(w - e w), e = exp(w/V), loses
# digits by cancellation as w/V -> 0 (the reference notes the trick "seems to
# lower accuracy", dadi/Integration.py:24).  The kernels follow the
# reference's operations one by one on that path; only exp is CUDA's, and
# another faithfully rounded exp moves the reference's own sweeps by up to
# 6.9e-10 (test_oracle.py::test_reference_exp_noise_delj).
DELJ_SWEEP_TOL = 1e-9
INT_TOL = 1e-9
# Five populations: the kernels form the drift sum_k m_k (x_k - x) of four
# migration terms as W - msum * x with W = sum_k m_k x_k per line, which
# reassociates four partly cancelling terms (measured 2.8e-12 on the last
# axis, where the rates into population 5 sum to 4).
SWEEP_TOL_5D = 5e-12


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _rel(a, b):
    return max_rel(a, b, floor=1e-12 * np.max(np.abs(b)))


@pytest.mark.parametrize("name,nd,axis,pts,gk", cases.SWEEPS)
@pytest.mark.parametrize("delj", [0, 1])
def test_single_sweep(cuda_lib, golden, name, nd, axis, pts, gk, delj):
    import torch
    from dadi_gb300 import _lib
    g = golden["sweeps"]
    p = cases.SWEEP_PARAMS
    xx = cases.grid(gk, pts)
    phi = _dev(torch, g["sweep_%s_phi0" % name])
    mig = (ctypes.c_double * len(p["mig"]))(*p["mig"])
    rc = cuda_lib.dgb_implicit_sweep(_lib.dptr(phi), nd, pts, axis, _lib.dptr(_dev(torch, xx)),
                                     p["nu"], mig, p["gamma"], p["h"], p["beta"], p["dt"], delj,
                                     None, 0, _lib.stream_handle(torch))
    assert rc == 0
    out = phi.cpu().numpy()
    tol = DELJ_SWEEP_TOL if delj else (SWEEP_TOL_5D if nd == 5 else SWEEP_TOL)
    assert _rel(out, g["sweep_%s_delj%d" % (name, delj)]) < tol


@pytest.mark.parametrize("nd,axis", [(2, 0), (2, 1), (3, 0), (3, 1), (3, 2)])
def test_precalc_sweep(cuda_lib, golden, nd, axis):
    import torch
    from dadi_gb300 import _lib
    g = golden["sweeps"]
    k = "precalc_%dD%d" % (nd, axis)
    phi = _dev(torch, g[k + "_phi0"])
    a, b, c = [_dev(torch, v) for v in g[k + "_abc"]]
    rc = cuda_lib.dgb_implicit_precalc_sweep(_lib.dptr(phi), nd, 9, axis, _lib.dptr(a),
                                             _lib.dptr(b), _lib.dptr(c), 0.01, None, 0,
                                             _lib.stream_handle(torch))
    assert rc == 0
    assert _rel(phi.cpu().numpy(), g[k]) < SWEEP_TOL


def test_tridiag_batch(cuda_lib, golden):
    import torch
    from dadi_gb300 import _lib
    h = golden["host"]
    a, b, c, r = [np.tile(v, 3) for v in h["tridiag_abcr"]]
    d = [_dev(torch, v) for v in (a, b, c, r)]
    u = torch.empty_like(d[3])
    ws, nws = _lib.workspace(torch, cuda_lib.dgb_workspace_bytes(2, 1, 100, 3))
    rc = cuda_lib.dgb_tridiag_batch(*[_lib.dptr(v) for v in d], _lib.dptr(u), 100, 3,
                                    _lib.dptr(ws), nws, _lib.stream_handle(torch))
    assert rc == 0
    out = u.cpu().numpy().reshape(3, 100)
    for k in range(3):
        assert _rel(out[k], h["tridiag_u"]) < SWEEP_TOL


@pytest.mark.parametrize("group,case", ALL_CASES, ids=[c["name"] for _, c in ALL_CASES])
def test_integration_case(cuda_lib, golden, group, case):
    from dadi_gb300 import integration as gi
    fn = {"one": gi.one_pop, "two": gi.two_pops, "three": gi.three_pops,
          "four": gi.four_pops, "five": gi.five_pops}[group]
    xx, phi0, args, kw = case_inputs(group, case)
    out = fn(phi0.copy(), xx, *args, **kw)
    assert _rel(out, golden["integrate"]["int_" + case["name"]]) < INT_TOL


@pytest.mark.parametrize("group,case", [(g, c) for g, c in ALL_CASES
                                        if g in ("two", "three") and "const" in c["name"]
                                        or "frozen" in c["name"] and "temporal" not in c["name"]
                                        and g in ("two", "three")],
                         ids=lambda v: v["name"] if isinstance(v, dict) else v)
def test_integration_case_precalc(cuda_lib, golden, group, case):
    """Constant parameters through the constant-coefficient path
    (enable_cuda_cached=True), which the reference's CPU uses."""
    from dadi_gb300 import integration as gi
    fn = gi.two_pops if group == "two" else gi.three_pops
    xx, phi0, args, kw = case_inputs(group, case)
    out = fn(phi0.copy(), xx, *args, enable_cuda_cached=True, **kw)
    assert _rel(out, golden["integrate"]["int_" + case["name"]]) < INT_TOL


def test_dropin_signatures(cuda_lib, golden):
    """dadi.cuda.Integration's private drivers with the reference signatures."""
    from dadi_gb300.cuda import Integration as CI
    from dadi_gb300 import integration as gi
    f = gi.ensure_1arg_func
    case = cases.TWO_POPS[1]
    xx, phi0, a, kw = case_inputs("two", case)
    T, nu1, nu2, m12, m21, g1, g2, h1, h2, th = a
    out = CI._two_pops_temporal_params(phi0.copy(), xx, T, 0, f(nu1), f(nu2), f(m12), f(m21),
                                       f(g1), f(g2), f(h1), f(h2), f(th), False, False, False,
                                       False, None)
    assert _rel(out, golden["integrate"]["int_" + case["name"]]) < INT_TOL
    case = cases.TWO_POPS[0]
    xx, phi0, a, kw = case_inputs("two", case)
    T, nu1, nu2, m12, m21, g1, g2, h1, h2, th = a
    ms = [[m12], [m21]]
    abc = []
    for k, (nu, g, h) in enumerate([(nu1, g1, h1), (nu2, g2, h2)]):
        abc.extend(gi.const_coefficients(xx, 2, k, nu, ms[k], g, h))
    dx = np.diff(xx)
    dt = min(gi._compute_dt(dx, nu1, [m12], g1, h1), gi._compute_dt(dx, nu2, [m21], g2, h2))
    out = CI._two_pops_const_params(phi0.copy(), xx, th, False, False, False, False, *abc, 0, dt, T)
    assert _rel(out, golden["integrate"]["int_" + case["name"]]) < INT_TOL


def test_split_mig_extrapolated(cuda_lib, golden):
    """Config-1 workload: split_mig, pts [40,50,60], ns (20,20), all 441
    extrapolated entries within 1e-9 of the reference."""
    from dadi_gb300 import models, numerics
    sm = cases.SPLIT_MIG
    f = numerics.make_extrap_func(models.split_mig)
    fs = f(sm["params"], sm["ns"], sm["pts_l"])
    assert_fs_parity(fs.data, golden["models"]["splitmig_fs"])
    assert fs_parity(fs.data, golden["models"]["splitmig_fs"])[2] == 0


@pytest.mark.parametrize("i", [0, 1, 2, 3, 5])
def test_im_extrapolated(cuda_lib, golden, i):
    from dadi_gb300 import models, numerics
    d = cases.im_draws()[i]
    f = numerics.make_extrap_func(models.IM)
    fs = f(d, (40, 40), [80, 90, 100])
    assert_fs_parity(fs.data, golden["models"]["im_fs_%d" % i])


def test_growth3_extrapolated(cuda_lib, golden):
    """Config-2 workload: 3 populations with exponential growth, pts
    [70,80,90], ns (20,20,20), temporal path."""
    from dadi_gb300 import models, numerics
    g = cases.GROWTH3
    f = numerics.make_extrap_func(models.growth3)
    fs = f(g["params"], g["ns"], g["pts_l"])
    assert_fs_parity(fs.data, golden["models"]["growth3_fs"])


def test_batched_matches_reference(cuda_lib, golden):
    """The batched engine (device schedule, persistent launch, device
    from_phi/extrapolation/likelihood) on seed-0 IM draws."""
    from dadi_gb300 import batch
    sel = [0, 1, 2, 3, 5]
    draws = cases.im_draws()[sel]
    eng = batch.Batch2D((80, 90, 100), (40, 40))
    g = golden["models"]
    fs, ll, status = eng.run(draws, data=g["im_obs"], scale=5e4)
    assert int(status.abs().sum()) == 0
    fs = fs.cpu().numpy()
    for k, i in enumerate(sel):
        assert_fs_parity(fs[k], g["im_fs_%d" % i])
    assert np.allclose(ll.cpu().numpy(), g["im_ll"], rtol=1e-9, atol=0)


def test_batched_alone_equals_in_mix(cuda_lib):
    """Each instance's integrated densities and its spectrum are bitwise the
    same alone and inside a batch (one CTA per item in every launch)."""
    from dadi_gb300 import batch
    draws = cases.im_draws(24)
    eng = batch.Batch2D((30, 40), (10, 10))
    phis_mix, _ = eng.integrate(batch.im_instances(draws))
    fs_mix, _, _ = eng.run(draws)
    for i in (0, 7, 23):
        phis, _ = eng.integrate(batch.im_instances(draws[i:i + 1]))
        for pa, pm in zip(phis, phis_mix):
            assert np.array_equal(pa.cpu().numpy()[0], pm.cpu().numpy()[i])
        alone, _, _ = eng.run(draws[i:i + 1])
        assert np.array_equal(alone.cpu().numpy()[0], fs_mix.cpu().numpy()[i])


def test_dropin_five_pops_signature(cuda_lib, golden):
    """dadi.cuda.Integration._five_pops_temporal_params (the call
    dadi/Integration.py:864-872 makes under cuda_enabled) with the reference
    signature, against dadi's own five_pops."""
    from dadi_gb300.cuda import Integration as CI
    from dadi_gb300 import integration as gi
    f = gi.ensure_1arg_func
    case = cases.FIVE_POPS[0]
    xx, phi0, a, kw = case_inputs("five", case)
    T = a[0]
    nus, ms, gs, hs = a[1:6], a[6:26], a[26:31], a[31:36]
    th, t0 = a[36], a[37]
    out = CI._five_pops_temporal_params(phi0.copy(), xx, T, t0, *[f(v) for v in nus],
                                        *[f(v) for v in ms], *[f(v) for v in gs],
                                        *[f(v) for v in hs], f(th), False, False, False, False,
                                        False, None)
    assert _rel(out, golden["integrate"]["int_" + case["name"]]) < INT_TOL


def test_edges_large_grid_and_zero_time(cuda_lib):
    """A 2-D grid too large for the shared-memory-resident kernel (L = 180:
    its density alone is 254 KB) runs through the per-axis sweeps and still
    matches the oracle; T == initial_t returns an unchanged copy; frozen
    populations with migration raise the reference's ValueError."""
    from dadi_gb300 import integration as gi
    from oracle import integration as oint
    xx = cases.grid("default", 180)
    phi0 = cases.initial_phi(7, (180, 180))
    args = (0.002, 1.5, 0.7, 0.4, 0.9)
    out = gi.two_pops(phi0.copy(), xx, *args)
    ref = oint.two_pops(phi0.copy(), xx, *args)
    assert _rel(out, ref) < INT_TOL
    same = gi.two_pops(phi0, xx, 0.3, initial_t=0.3)
    assert np.array_equal(same, phi0) and same is not phi0
    with pytest.raises(ValueError):
        gi.two_pops(phi0, xx, 0.1, m12=1.0, frozen1=True)


def test_transpose_gpuarray(cuda_lib):
    """dadi.cuda.transpose_gpuarray's contract (tests/test_CUDA.py:11-21 of
    the reference) on device tensors."""
    import torch
    from dadi_gb300 import cuda as dcuda
    a = np.random.default_rng(0).uniform(size=(2, 3))
    a_gpu = torch.from_numpy(a).cuda()
    aT_gpu = torch.empty(a.shape[::-1], dtype=a_gpu.dtype, device="cuda")
    dcuda.transpose_gpuarray(a_gpu, aT_gpu)
    assert np.array_equal(aT_gpu.cpu().numpy(), a.T)
    with pytest.raises(ValueError):
        dcuda.transpose_gpuarray(a_gpu, torch.empty(2, 3, dtype=a_gpu.dtype, device="cuda"))


@pytest.mark.parametrize("name,kw", cases.SETTINGS, ids=[n for n, _ in cases.SETTINGS])
def test_dadi_settings(cuda_lib, golden, name, kw):
    """The drop-in integrators and the batched engine under each non-default
    setting of dadi.Integration (read at call time: use_old_timestep,
    use_delj_trick, timescale_factor) against dadi run with the same
    setting, within the integration and spectrum bars."""
    from dadi_gb300 import batch, integration as gi, models, numerics, phimanip
    g = golden["settings"]
    d = cases.SETTINGS_IM
    tol = INT_TOL
    saved = {k: getattr(gi, k) for k in kw}
    try:
        for k, v in kw.items():
            setattr(gi, k, v)
        xx = numerics.default_grid(18)
        phi = phimanip.phi_1D_to_2D(xx, phimanip.phi_1D(xx))
        p2 = gi.two_pops(phi, xx, 0.04, 2.0, lambda t: 0.5 + t, 1.0, 0.4, gamma1=-1.0,
                         gamma2=2.0, h1=0.3)
        assert _rel(p2, g["set_%s_2d" % name]) < tol
        p3 = gi.three_pops(phimanip.phi_2D_to_3D_split_2(xx, phi), xx, 0.02,
                           lambda t: 1.0 + t, 0.5, 2.0, m12=1.0, m21=0.5, m23=0.3, m32=0.6,
                           gamma3=1.5)
        assert _rel(p3, g["set_%s_3d" % name]) < tol
        ref = g["set_%s_im" % name]
        fs = numerics.make_extrap_func(models.IM)(d["params"], d["ns"], d["pts_l"])
        eng = batch.Batch2D(d["pts_l"], d["ns"])
        fsb, _, st = eng.run(np.array([d["params"]]))
        assert int(st.abs().sum()) == 0
        # one launch per grid size (CTA size per grid) gives the same bits
        eng.launch_mode = "per_grid"
        fsp, _, stp = eng.run(np.array([d["params"]]))
        assert int(stp.abs().sum()) == 0
        assert np.array_equal(fsp.cpu().numpy(), fsb.cpu().numpy())
        for f in (np.asarray(fs.data), fsb.cpu().numpy()[0]):
            assert_fs_parity(f, ref)
    finally:
        for k, v in saved.items():
            setattr(gi, k, v)


@pytest.mark.parametrize("P,L,delj,frozen", [(3, 20, 0, 0), (3, 20, 1, 0), (3, 16, 0, 1),
                                             (4, 10, 0, 0), (4, 10, 1, 2), (1, 60, 0, 0),
                                             (1, 60, 1, 0), (2, 180, 0, 0), (5, 7, 0, 0)])
def test_coefficient_records_match_inline_setup(cuda_lib, P, L, delj, frozen):
    """The per-axis sweeps that read per-step coefficient records (the
    workspace holds them) give bitwise the densities of the sweeps that build
    their coefficients in every CTA (no workspace), over 300 steps -- more
    than one chunk of records -- with and without the delj trick and frozen
    populations."""
    import torch
    from dadi_gb300 import _lib
    lib = cuda_lib
    xx = cases.grid("default", L)
    phi0 = np.abs(cases.initial_phi(11, (L,) * P)) + 1e-3
    tab = table_rows(P, 300, seed=P * 100 + L)
    d_xx, d_tab = _dev(torch, xx), _dev(torch, tab)
    outs = []
    for ws_bytes in (0, lib.dgb_workspace_bytes(0, P, L, 0)):
        d_phi = _dev(torch, phi0)
        ws, nws = _lib.workspace(torch, ws_bytes)
        _lib.check(lib.dgb_integrate_table(_lib.dptr(d_phi), P, L, _lib.dptr(d_xx),
                                           _lib.dptr(d_tab), len(tab), frozen, 0, delj,
                                           _lib.dptr(ws) if ws_bytes else None, ws_bytes,
                                           _lib.stream_handle(torch)), "dgb_integrate_table")
        outs.append(d_phi.cpu().numpy())
    assert np.all(np.isfinite(outs[0]))
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("pts_l,delj", [((100,), False), ((100, 110), False), ((100,), True)])
def test_two_items_per_cta_bitwise(cuda_lib, pts_l, delj):
    """A launch over one grid of 97-128 points runs two work items per CTA
    when the thread count is automatic; its densities are bitwise those of
    one item per CTA (threads forced to 128), with an odd number of
    instances (the last CTA holds one item).  With the delj trick the
    engine keeps one item per CTA, so the two settings agree as well."""
    from dadi_gb300 import batch, integration as gi
    saved = gi.use_delj_trick
    try:
        gi.use_delj_trick = bool(delj)
        eng = batch.Batch2D(pts_l, (10, 10))
        # five IM parameter sets around the settings case (the delj trick
        # overflows exp, and the reference gives NaN, at the workload's
        # extreme draws), with different step counts
        base = np.array(cases.SETTINGS_IM["params"], dtype=np.float64)
        params = np.repeat(base[None, :], 5, axis=0)
        params[:, 3] = (0.05, 0.03, 0.07, 0.02, 0.06)
        params[:, 4] = (1.0, 2.0, 0.5, 3.0, 1.5)
        rec = batch.im_instances(params)
        for mode in ("persistent", "per_grid"):
            eng.launch_mode = mode
            out = []
            for threads in (0, 128):
                eng.threads = threads
                phis, st = eng.integrate(rec)
                assert int(st.abs().sum()) == 0
                out.append([p.cpu().numpy() for p in phis])
            assert all(np.array_equal(a, b) for a, b in zip(out[0], out[1])), mode
            assert all(np.all(np.isfinite(a)) for a in out[0])
    finally:
        gi.use_delj_trick = saved


@pytest.mark.parametrize("old_timestep", [False, True])
def test_schedule_single_pass_matches_two_passes(cuda_lib, old_timestep):
    """Filling the device schedules in one pass, into room reserved from the
    host bounds, writes exactly the rows and counts of the count-scan-fill
    passes (IM draws and records with every parametric form)."""
    import torch
    from dadi_gb300 import _lib, batch, integration as gi
    from test_host import _random_records
    saved = gi.use_old_timestep
    try:
        gi.use_old_timestep = old_timestep
        eng = batch.Batch2D((20, 25, 30), (8, 8))
        rec = np.concatenate([batch.im_instances(cases.im_draws(200)),
                              _random_records(100, seed=9)])
        n = len(rec)
        d_rec = _lib.to_device(torch, rec.view(np.uint8), np.uint8)
        one = eng.schedule(d_rec, n, rec)
        assert eng.schedule_passes == 1
        two = eng.schedule(d_rec, n)
        assert eng.schedule_passes == 2
        (t1, o1, c1, s1), (t2, o2, c2, s2) = [[x.cpu().numpy() for x in r] for r in (one, two)]
        assert np.array_equal(c1, c2) and np.array_equal(s1, s2)
        t1, t2 = t1.reshape(-1, 11), t2.reshape(-1, 11)
        for s in range(len(c1)):
            a = t1[o1[s]:o1[s] + c1[s]]
            b = t2[o2[s]:o2[s] + c2[s]]
            assert np.array_equal(a, b), s
    finally:
        gi.use_old_timestep = saved
