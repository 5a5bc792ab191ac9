"""The oracle (CPU restatement) against the reference's own outputs: golden
vectors produced by running dadi 2.4.3 (tests/golden/make_golden.py), and the
reference C sweeps compiled from their sources when that build exists."""
import numpy as np
import pytest

import cases
from oracle import clib, integration as oint, numerics as onum
from util import ALL_CASES, case_inputs


@pytest.mark.parametrize("group,case", ALL_CASES, ids=[c["name"] for _, c in ALL_CASES])
def test_integration_bitwise(golden, group, case):
    fn = {"one": oint.one_pop, "two": oint.two_pops, "three": oint.three_pops,
          "four": oint.four_pops, "five": oint.five_pops}[group]
    xx, phi0, args, kw = case_inputs(group, case)
    out = fn(phi0.copy(), xx, *args, **kw)
    assert np.array_equal(out, golden["integrate"]["int_" + case["name"]])


@pytest.mark.parametrize("name,nd,axis,pts,gk", cases.SWEEPS)
@pytest.mark.parametrize("delj", [0, 1])
def test_sweep_bitwise(golden, name, nd, axis, pts, gk, delj):
    g = golden["sweeps"]
    p = cases.SWEEP_PARAMS
    phi = g["sweep_%s_phi0" % name].copy()
    clib.sweep(phi, cases.grid(gk, pts), axis, p["nu"], p["mig"][:nd], p["gamma"], p["h"],
               p["dt"], beta=p["beta"], use_delj_trick=delj)
    assert np.array_equal(phi, g["sweep_%s_delj%d" % (name, delj)])


@pytest.mark.parametrize("nd,axis", [(2, 0), (2, 1), (3, 0), (3, 1), (3, 2)])
def test_precalc_sweep_bitwise(golden, nd, axis):
    g = golden["sweeps"]
    k = "precalc_%dD%d" % (nd, axis)
    phi = g[k + "_phi0"].copy()
    a, b, c = g[k + "_abc"]
    clib.sweep_precalc(phi, axis, a, b, c, 0.01)
    assert np.array_equal(phi, g[k])


def test_tridiag(golden):
    h = golden["host"]
    a, b, c, r = h["tridiag_abcr"]
    assert np.array_equal(clib.tridiag(a, b, c, r), h["tridiag_u"])


def test_host_pieces(golden):
    h = golden["host"]
    for pts in (5, 10, 40, 80, 100, 120):
        assert np.array_equal(onum.default_grid(pts), h["grid_%d" % pts])
    xx = onum.default_grid(30)
    assert np.array_equal(onum.phi_1D(xx), h["phi1d_snm"])
    assert np.array_equal(onum.phi_1D(xx, nu=1.5, theta0=2.0, gamma=2.0), h["phi1d_g2"])
    assert np.array_equal(onum.phi_1D(xx, gamma=-5.0, beta=1.4), h["phi1d_gm5"])
    assert np.array_equal(onum.phi_1D_to_2D(xx, onum.phi_1D(xx)), h["phi2d_split"])
    xs = onum.default_grid(12)
    p3 = onum.phi_2D_to_3D_admix(onum.phi_1D_to_2D(xs, onum.phi_1D(xs)), 0, xs, xs, xs)
    assert np.array_equal(p3, h["phi3d_split2"])
    assert np.array_equal(onum.phi_3D_to_4D(p3, 0.3, 0.2, xs, xs, xs, xs), h["phi4d_from3d"])
    for nd, pts in [(1, 25), (2, 21), (3, 11), (4, 7)]:
        fs = onum.from_phi(h["fromphi_%dd_phi" % nd], tuple(h["fromphi_%dd_ns" % nd]),
                           onum.default_grid(pts))
        assert np.array_equal(fs, h["fromphi_%dd" % nd])
    ys = list(h["extrap_in"])
    assert np.array_equal(onum.quadratic_extrap(ys, [0.01, 0.008, 0.006]), h["extrap_q"])
    assert np.array_equal(onum.linear_extrap(ys[:2], [0.01, 0.008]), h["extrap_l"])
    m, d = h["ll_model"], h["ll_data"]
    mask = onum.corner_mask(m.shape)
    assert onum.ll(m, d, mask) == pytest.approx(float(h["ll"]), rel=1e-14)
    assert onum.ll_multinom(m, d, mask) == pytest.approx(float(h["ll_multinom"]), rel=1e-14)


def test_models_small(golden):
    """Full model pipelines (grid, initial condition, integration, from_phi,
    extrapolation) against dadi's own make_extrap_func output."""
    g = golden["models"]
    sm = cases.SPLIT_MIG
    fs = onum.extrap_model(onum.split_mig, sm["params"], sm["ns"], sm["pts_l"])
    assert np.array_equal(fs, g["splitmig_fs"])
    d0 = cases.im_draws()[0]
    assert np.array_equal(cases.im_draws()[:64], g["im_draws_head"])
    fs = onum.extrap_model(onum.IM, d0, (10, 10), [20, 25, 30])
    assert np.array_equal(fs, g["im_small_fs"])


def test_against_compiled_reference():
    """The C restatement equals the reference C sweeps compiled from their own
    sources (only where the reference tree was available to build them)."""
    import ctypes
    ref = clib.ref_lib()
    if ref is None:
        pytest.skip("reference C not built here (no reference tree)")
    dp = ctypes.POINTER(ctypes.c_double)
    rng = np.random.default_rng(3)
    L = 17
    xx = onum.default_grid(L)
    for delj in (0, 1):
        phi = rng.uniform(size=(L, L))
        a = phi.copy()
        ref.implicit_2Dx.argtypes = [dp, dp, dp] + [ctypes.c_double] * 5 + [ctypes.c_int] * 5
        ref.implicit_2Dx(a.ctypes.data_as(dp), xx.ctypes.data_as(dp), xx.ctypes.data_as(dp),
                         0.7, 1.3, -2.0, 0.3, 0.01, L, L, delj, 0, L)
        b = phi.copy()
        clib.sweep(b, xx, 0, 0.7, [0, 1.3], -2.0, 0.3, 0.01, use_delj_trick=delj)
        assert np.array_equal(a, b)
        ref.implicit_3Dz.argtypes = [dp, dp, dp, dp] + [ctypes.c_double] * 6 + [ctypes.c_int] * 6
        phi3 = rng.uniform(size=(9, 9, 9))
        x9 = onum.default_grid(9)
        a = phi3.copy()
        ref.implicit_3Dz(a.ctypes.data_as(dp), x9.ctypes.data_as(dp), x9.ctypes.data_as(dp),
                         x9.ctypes.data_as(dp), 1.1, 0.4, 2.2, 1.5, 0.8, 0.02, 9, 9, 9, delj, 0, 9)
        b = phi3.copy()
        clib.sweep(b, x9, 2, 1.1, [0.4, 2.2, 0], 1.5, 0.8, 0.02, use_delj_trick=delj)
        assert np.array_equal(a, b)


def test_reference_noise_floor_at_scale():
    """Forming the right-hand side as (1/dt)*phi instead of phi/dt -- the form
    the reference's own constant-parameter sweeps use -- moves entries of an
    at-scale IM spectrum (draw 2568 of the batched workload, pts [80,90,100],
    ns (40,40)) between 1e-12 and 1e-9 of the maximum by more than 1e-9
    relative (1.5e-8), while entries above 1e-9 of the maximum move by less
    than 1e-9 and every smaller entry by less than 1e-18 of the maximum.
    This is why spectrum parity is relative above 1e-9 of the maximum and
    absolute below it (util.fs_parity)."""
    import os
    from util import FS_REL, TINY_FRAC, fs_parity
    g = np.load(os.path.join(os.path.dirname(cases.__file__), "im_scale.npz"))
    k = list(g["golden_idx"]).index(2568)
    ref = g["golden_fs"][k]
    clib.rhs_variant = True
    try:
        fs = onum.extrap_model(onum.IM, g["golden_params"][k], (40, 40), [80, 90, 100])
    finally:
        clib.rhs_variant = False
    m = onum.corner_mask(ref.shape)
    mx = np.max(np.abs(ref[~m]))
    mid = (np.abs(ref) >= 1e-12 * mx) & (np.abs(ref) < TINY_FRAC * mx) & ~m
    with np.errstate(all="ignore"):
        rel = np.abs(fs - ref) / np.abs(ref)
    assert np.max(rel[mid]) > 1e-8          # the reference's own floor there
    rel_big, abs_small, n_small = fs_parity(fs, ref)
    assert n_small > 0
    assert rel_big < FS_REL                  # entries that matter move less
    assert abs_small < FS_REL * TINY_FRAC    # and small ones little in absolute terms


@pytest.mark.parametrize("name,kw", cases.SETTINGS, ids=[n for n, _ in cases.SETTINGS])
def test_oracle_under_dadi_settings(golden, name, kw):
    """The oracle under each non-default setting of dadi.Integration
    (use_old_timestep, use_delj_trick, timescale_factor) equals dadi run with
    the same setting, bit for bit."""
    g = golden["settings"]
    d = cases.SETTINGS_IM
    saved = {k: getattr(oint, k) for k in kw}
    try:
        for k, v in kw.items():
            setattr(oint, k, v)
        fs = onum.extrap_model(onum.IM, d["params"], d["ns"], d["pts_l"])
        assert np.array_equal(fs, g["set_%s_im" % name])
        xx = onum.default_grid(18)
        phi = onum.phi_1D_to_2D(xx, onum.phi_1D(xx))
        p2 = oint.two_pops(phi.copy(), xx, 0.04, 2.0, lambda t: 0.5 + t, 1.0, 0.4,
                           gamma1=-1.0, gamma2=2.0, h1=0.3)
        assert np.array_equal(p2, g["set_%s_2d" % name])
        phi3 = onum.phi_2D_to_3D_admix(phi, 0, xx, xx, xx)
        p3 = oint.three_pops(phi3, xx, 0.02, lambda t: 1.0 + t, 0.5, 2.0, m12=1.0, m21=0.5,
                             m23=0.3, m32=0.6, gamma3=1.5)
        assert np.array_equal(p3, g["set_%s_3d" % name])
    finally:
        for k, v in saved.items():
            setattr(oint, k, v)


# ---------------------------------------------- the batched workload at scale

def _reference_loop_steps(p, tsf=1e-3):
    """Steps of dadi's two_pops loop for Demographics2D.IM, walked in Python
    with the reference's expressions (dadi/Integration.py:346-386,
    dadi/Demographics2D.py:297-307)."""
    s, nu1, nu2, T, m12, m21 = p
    f1 = oint.ensure_1arg_func(lambda t: s * (nu1 / s) ** (t / T))
    f2 = oint.ensure_1arg_func(lambda t: (1 - s) * (nu2 / (1 - s)) ** (t / T))
    t, n = 0, 0
    a, b = f1(t), f2(t)
    dx = np.diff(onum.default_grid(10))
    while t < T:
        dt = min(oint.compute_dt(dx, a, [m12], 0, 0.5), oint.compute_dt(dx, b, [m21], 0, 0.5))
        t = t + min(dt, T - t)
        a, b = f1(t), f2(t)
        n += 1
    return n


def test_im_step_counter_matches_reference_loop():
    """The oracle's C walk of the IM schedule (used to pick and scale the CPU
    sample and by the reference arm of the benchmark) counts exactly the
    steps of the reference loop."""
    draws = cases.im_draws()
    steps = clib.im_steps(draws)
    sel = [i for i in range(200) if steps[i] < 2500][:40]
    for i in sel:
        assert _reference_loop_steps(draws[i]) == steps[i]
    assert steps.sum() == 10784487 and steps.max() == 19546


def test_im_step_counter_matches_library_host_walk():
    """... and the GPU package's host walk of the same schedules agrees on all
    4096 draws (the batched engine's device walk is tested against it on the
    GPU)."""
    from dadi_gb300 import batch
    draws = cases.im_draws()
    assert np.array_equal(clib.im_steps(draws), batch.count_steps(batch.im_instances(draws)))


def test_parity_sample_is_stratified(golden):
    import os
    g = np.load(os.path.join(os.path.dirname(cases.__file__), "im_scale.npz"))
    draws = cases.im_draws()
    steps = clib.im_steps(draws)
    idx = cases.im_parity_sample(draws, steps)
    assert np.array_equal(idx, g["sample_idx"])
    assert np.array_equal(steps[idx], g["sample_steps"])
    assert len(idx) == 64 and 4 in idx and steps[idx].max() == 19546
    for col in range(6):
        assert int(np.argmin(draws[:, col])) in idx and int(np.argmax(draws[:, col])) in idx
    # the goldens are the 16 longest schedules of the sample
    order = idx[np.argsort(-steps[idx], kind="stable")]
    assert np.array_equal(g["golden_idx"], order[:cases.IM_SCALE_GOLDEN])
    assert np.array_equal(g["golden_params"], draws[g["golden_idx"]])


def test_oracle_matches_dadi_at_scale():
    """The oracle equals dadi bit for bit on the cheapest at-scale golden
    spectrum (pts [80,90,100], ns (40,40), 3285 steps)."""
    import os
    g = np.load(os.path.join(os.path.dirname(cases.__file__), "im_scale.npz"))
    k = len(g["golden_idx"]) - 1
    fs = onum.extrap_model(onum.IM, g["golden_params"][k], (40, 40), [80, 90, 100])
    assert np.array_equal(fs, g["golden_fs"][k])


@pytest.mark.parametrize("name,nd,axis,pts,gk", cases.SWEEPS)
def test_reference_exp_noise_delj(golden, name, nd, axis, pts, gk):
    """Under the delj trick the reference's sweeps depend on exp's last
    ulp: with another faithfully rounded exp (oracle/sweeps.c orc_exp) they
    move by up to 6.9e-10 relative, which bounds what a GPU exp with a
    one-ulp error bound can do to an otherwise operation-for-operation
    restatement (the delj sweep bar is 1e-9)."""
    from util import max_rel
    g = golden["sweeps"]
    p = cases.SWEEP_PARAMS
    phi = g["sweep_%s_phi0" % name].copy()
    clib.exp_variant = True
    try:
        clib.sweep(phi, cases.grid(gk, pts), axis, p["nu"], p["mig"][:nd], p["gamma"], p["h"],
                   p["dt"], beta=p["beta"], use_delj_trick=1)
    finally:
        clib.exp_variant = False
    ref = g["sweep_%s_delj1" % name]
    assert max_rel(phi, ref, floor=1e-12 * np.max(np.abs(ref))) < 1e-9
