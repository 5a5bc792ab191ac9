"""Host-side pieces of the package against the reference's own outputs
(golden vectors from dadi 2.4.3) and the oracle: grid, initial conditions,
splits, from_phi, extrapolation, likelihoods, the per-step parameter table and
the constant-coefficient builder.  No GPU needed."""
import numpy as np
import pytest

import cases
from dadi_gb300 import inference, integration, numerics, phimanip, spectrum
from oracle import integration as oint
from util import max_rel


def test_grid_and_phi(golden):
    h = golden["host"]
    for pts in (5, 10, 40, 80, 100, 120):
        assert np.array_equal(numerics.default_grid(pts), h["grid_%d" % pts])
    xx = numerics.default_grid(30)
    assert np.array_equal(phimanip.phi_1D(xx), h["phi1d_snm"])
    assert np.array_equal(phimanip.phi_1D(xx, nu=1.5, theta0=2.0, gamma=2.0), h["phi1d_g2"])
    assert np.array_equal(phimanip.phi_1D(xx, gamma=-5.0, beta=1.4), h["phi1d_gm5"])
    assert max_rel(phimanip.phi_1D(xx, gamma=-3.0, h=0.3), h["phi1d_h03"]) < 1e-12
    assert np.array_equal(phimanip.phi_1D_to_2D(xx, phimanip.phi_1D(xx)), h["phi2d_split"])
    xs = numerics.default_grid(12)
    p3 = phimanip.phi_2D_to_3D_split_2(xs, phimanip.phi_1D_to_2D(xs, phimanip.phi_1D(xs)))
    assert np.array_equal(p3, h["phi3d_split2"])
    assert np.array_equal(phimanip.phi_3D_to_4D(p3, 0.3, 0.2, xs, xs, xs, xs),
                          h["phi4d_from3d"])


def test_phi_4D_to_5D(golden):
    h = golden["host"]
    x6 = numerics.default_grid(6)
    p4 = phimanip.phi_3D_to_4D(phimanip.phi_2D_to_3D_split_2(
        x6, phimanip.phi_1D_to_2D(x6, phimanip.phi_1D(x6))), 0.3, 0.2, x6, x6, x6, x6)
    assert np.array_equal(phimanip.phi_4D_to_5D(p4, 0.2, 0.3, 0.1, x6, x6, x6, x6, x6),
                          h["phi5d_from4d"])


@pytest.mark.parametrize("nd,pts", [(1, 25), (2, 21), (3, 11), (4, 7), (5, 6)])
def test_from_phi(golden, nd, pts):
    h = golden["host"]
    xx = numerics.default_grid(pts)
    fs = spectrum.from_phi(h["fromphi_%dd_phi" % nd], tuple(h["fromphi_%dd_ns" % nd]),
                           (xx,) * nd)
    assert np.array_equal(np.asarray(fs.data), h["fromphi_%dd" % nd])
    assert fs.mask.flat[0] and fs.mask.flat[-1] and fs.extrap_x == xx[1]


def test_extrap_and_ll(golden):
    h = golden["host"]
    ys = list(h["extrap_in"])
    assert np.array_equal(numerics.quadratic_extrap(ys, [0.01, 0.008, 0.006]), h["extrap_q"])
    assert np.array_equal(numerics.linear_extrap(ys[:2], [0.01, 0.008]), h["extrap_l"])
    model = spectrum.Spectrum(h["ll_model"])
    data = spectrum.Spectrum(h["ll_data"])
    assert inference.ll(model, data) == pytest.approx(float(h["ll"]), rel=1e-14)
    assert inference.ll_multinom(model, data) == pytest.approx(float(h["ll_multinom"]), rel=1e-14)


def test_extrap_fail_mag():
    """Entries extrapolated more than fail_mag decades away fall back to the
    smallest-x input (dadi/Numerics.py:449-464)."""
    a = np.array([1.0, 1e-5])
    b = np.array([1.0, 1e-20])
    c = np.array([1.0, 1e-30])
    ex = numerics.extrapolate([a, b, c], [0.3, 0.2, 0.1])
    assert ex[1] == c[1]
    assert ex[0] == pytest.approx(1.0)


@pytest.mark.parametrize("case", cases.TWO_POPS + cases.THREE_POPS[:3],
                         ids=lambda c: c["name"])
def test_table_matches_oracle_schedule(case):
    """The host-evaluated schedule (step count, dt sequence, final time) is the
    reference loop's: rebuilding the oracle's integration from the table's dts
    gives the same step count."""
    P = 2 if case["name"].startswith("2d") else 3
    xx = cases.grid(case["grid"], case["pts"])
    args = [cases.resolve(v) for v in case["args"]]
    kw = {k: cases.resolve(v) for k, v in case.get("kw", {}).items()}
    T = args[0]
    initial_t = kw.get("initial_t", args[12 if P == 2 else 18] if len(args) > (12 if P == 2 else 18) else 0)
    f = integration.ensure_1arg_func
    if P == 2:
        T, nu1, nu2, m12, m21, g1, g2, h1, h2, th = args[:10]
        table, hist = integration.build_table(2, xx, T, initial_t, [f(nu1), f(nu2)],
                                              [[None, f(m12)], [f(m21), None]],
                                              [f(g1), f(g2)], [f(h1), f(h2)], f(th))
    else:
        (T, n1, n2, n3, m12, m13, m21, m23, m31, m32, g1, g2, g3, h1, h2, h3, th) = args[:17]
        mig = [[None, f(m12), f(m13)], [f(m21), None, f(m23)], [f(m31), f(m32), None]]
        table, hist = integration.build_table(3, xx, T, initial_t, [f(n1), f(n2), f(n3)], mig,
                                              [f(g1), f(g2), f(g3)], [f(h1), f(h2), f(h3)],
                                              f(th))
    t = initial_t
    for row in table:
        t = t + row[0]
    assert t == pytest.approx(T, rel=1e-12)
    assert len(hist) == len(table) + 1
    assert table.shape[1] == integration.row_stride(P)


def test_table_validation():
    xx = numerics.default_grid(10)
    f = integration.ensure_1arg_func
    with pytest.raises(ValueError):
        integration.build_table(2, xx, 0.1, 0, [f(1.0), f(lambda t: 1.0 if t < 0.05 else -1.0)],
                                [[None, f(0)], [f(0), None]], [f(0), f(0)], [f(.5), f(.5)], f(1))
    with pytest.raises(ValueError):
        integration.build_table(2, xx, 0.1, 0, [f(1.0), f(1.0)],
                                [[None, f(-1.0)], [f(0), None]], [f(0), f(0)], [f(.5), f(.5)],
                                f(1))
    with pytest.raises(ValueError):
        integration.two_pops(np.zeros((10, 10)), xx, 0.1, 1, 1, m12=1, frozen1=True)
    with pytest.raises(ValueError):
        integration.two_pops(np.zeros((10, 10)), xx, 0.1, initial_t=0.2)


@pytest.mark.parametrize("P,axis", [(2, 0), (2, 1), (3, 0), (3, 2)])
def test_const_coefficients_match_oracle(P, axis):
    xx = cases.grid("lin", 9)
    ms = [0.3, 1.7][:P - 1]
    a1 = integration.const_coefficients(xx, P, axis, 0.7, ms, -1.2, 0.3)
    a2 = oint.precalc_coefficients(xx, P, axis, 0.7, ms, -1.2, 0.3)
    for u, v in zip(a1, a2):
        assert np.array_equal(u, v)


def test_table_dual_values_equal_build_table():
    """The dual-number schedule walk of the N-dimensional adjoint produces the
    parameter table exactly as the drop-in's build_table does from the model's
    own callables (dadi/Integration.py:504-553) -- bit for bit in Python
    (numpy's exp and log on both sides), to an ulp in C (the C library's) with
    the same step lengths -- and its derivative matches finite differences of
    the table."""
    from dadi_gb300 import adjoint_nd, integration, models, numerics
    xx = numerics.default_grid(20)
    (nu0, nuF, (m12, m13, m23), g, T) = models.GROWTH3_DEFAULT
    # T / dt must not be an integer, or a perturbation adds or drops a step
    # and the table has no elementwise derivative (the workload's default T
    # is exactly 675 steps of 1e-3 / 4.5)
    T = 0.1537
    nus = [(lambda a, b: (lambda t: a * np.exp(np.log(b / a) * t / T)))(a, b)
           for a, b in zip(nu0, nuF)]
    f = integration.ensure_1arg_func
    mig = [[None, f(m12), f(m13)], [f(m12), None, f(m23)], [f(m13), f(m23), None]]
    ref, _ = integration.build_table(3, xx, T, 0.0, [f(v) for v in nus], mig,
                                     [f(v) for v in g], [f(0.5)] * 3, f(1.0))
    model = adjoint_nd.Growth3.__new__(adjoint_nd.Growth3)
    model.gammas = tuple(g)
    theta = adjoint_nd.Growth3.from_model_params(models.GROWTH3_DEFAULT)
    theta[9] = T
    assert np.array_equal(model.table_python(theta, xx)[0], ref)
    tab, drows = model.table(theta, xx)
    assert tab.shape == ref.shape and np.array_equal(tab[:, 0], ref[:, 0])
    assert float((np.abs(tab - ref) / np.maximum(np.abs(ref), 1e-300)).max()) <= 5e-16
    for k in range(10):
        h = 1e-6 * theta[k]
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        a, _ = model.table(tp, xx)
        b, _ = model.table(tm, xx)
        assert a.shape == b.shape == tab.shape
        fd = (a - b) / (2 * h)
        # finite-difference noise: an ulp of a table entry over 2h (~1e-9)
        assert np.allclose(drows[:, :, k], fd, rtol=1e-6, atol=1e-8)


def _dfe_cache_from_golden(golden):
    """A Cache2D holding the reference's own cached spectra."""
    from dadi_gb300 import dfe
    g = golden["dfe"]
    c = dfe.Cache2D.__new__(dfe.Cache2D)
    c.gammas = c.neg_gammas = g["dfe_gammas"]
    c.spectra = g["dfe_spectra"]
    return c


def test_dfe_pdf_and_integrate_match_reference(golden):
    """Cache2D.integrate (trapezoid over the gamma grid plus the quadrature of
    the mass beyond it, dadi/DFE/Cache2D_mod.py:209-310) and the bivariate
    lognormal (dadi/DFE/PDFs.py:41-76), on the reference's cached spectra,
    against dadi's results."""
    import cases
    from dadi_gb300 import dfe
    g = golden["dfe"]
    d = cases.DFE
    x = np.array([0.5, 3.0, 40.0])
    assert np.allclose(dfe.biv_lognormal(x, x, np.array(d["sel_params"])), g["dfe_pdf"],
                       rtol=1e-13, atol=0)
    c = _dfe_cache_from_golden(golden)
    fs = c.integrate(d["sel_params"], None, dfe.biv_lognormal, d["theta"], None)
    assert np.allclose(np.asarray(fs.data), g["dfe_fs"], rtol=1e-12, atol=0)
    fs = c.integrate(d["sel_params"], None, dfe.biv_lognormal, d["theta"], None,
                     exterior_int=False)
    assert np.allclose(np.asarray(fs.data), g["dfe_fs_interior"], rtol=1e-12, atol=0)


def _phi1d_direct(xx, gamma, h, prec=None):
    """The stationary density with selection and dominance evaluated straight
    from its integral form, phi(x) = e^{S(x)} int_x^1 e^{-S} / int_0^1 e^{-S}
    / (x (1 - x)) with S(x) = 4 gamma h x + 2 gamma (1 - 2h) x^2 (end points
    as phi_1D sets them), by scipy quadrature or, with prec, by mpmath at
    that many digits.  The check the reference's test_phi1D.py makes."""
    S = lambda x: 4 * gamma * h * x + 2 * gamma * (1 - 2 * h) * x * x
    if prec:
        import mpmath
        mpmath.mp.dps = prec
        f = lambda x: mpmath.exp(-S(x))
        int0 = mpmath.quad(f, [0, 1])
        ints = [mpmath.quad(f, [q, 1]) for q in xx]
        phi = np.array([float(mpmath.exp(S(q)) * v / int0) for q, v in zip(xx, ints)])
        int0 = float(int0)
    else:
        import warnings
        import scipy.integrate
        f = lambda x: np.exp(-S(x))
        with np.errstate(all="ignore"), warnings.catch_warnings():
            warnings.simplefilter("ignore")  # the overflow this form is known for
            int0 = scipy.integrate.quad(f, 0, 1)[0]
            ints = np.array([scipy.integrate.quad(f, q, 1)[0] for q in xx])
            phi = np.exp(S(xx)) * ints / int0
    phi[1:-1] /= xx[1:-1] * (1 - xx[1:-1])
    phi[0] = phi[1]
    phi[-1] = 1. / int0
    return phi


def test_phi_1D_dominance_matches_integral_form():
    """phi_1D with dominance (dadi/PhiManip.py:12-108) against the integral
    form: close to direct quadrature where that converges (gamma = 50),
    finite where direct quadrature overflows (gamma = 500), and within
    5e-3 of arbitrary-precision quadrature for strongly negative gammas
    (the reference's tests/test_phi1D.py cases)."""
    xx = numerics.default_grid(20)
    for gamma, h in ([50, 0.14], [50, 0.84]):
        assert np.allclose(phimanip.phi_1D(xx, gamma=gamma, h=h), _phi1d_direct(xx, gamma, h))
    for gamma, h in ([500, 0.14], [500, 0.84]):
        assert np.any(np.isnan(_phi1d_direct(xx, gamma, h)))
        assert not np.any(np.isnan(phimanip.phi_1D(xx, gamma=gamma, h=h)))
    pytest.importorskip("mpmath")
    for gamma, h in [(-500, 0.14), (-500, 0.94), (-2000, 0.34), (-1429, 0.51), (-1e4, 0),
                     (-1e5, 0), (-1e6, 0)]:
        ours = phimanip.phi_1D(xx, gamma=gamma, h=h)
        ref = _phi1d_direct(xx, gamma, h, prec=5)
        assert np.max(2 * np.abs(ours - ref) / (ours + ref + 1e-12)) < 5e-3, (gamma, h)


def _random_records(n, seed):
    """dgb_inst2d records with every parametric form: exponential growth and
    decline, exp-log, linear and constant sizes, migration, selection and
    dominance that change over time."""
    from dadi_gb300 import _lib, batch
    rng = np.random.default_rng(seed)
    rec = np.zeros(n, dtype=batch.INST_DTYPE)
    rec["initial_t"] = rng.uniform(0, 0.05, n)
    rec["T"] = rec["initial_t"] + rng.uniform(0.001, 0.5, n)
    T = rec["T"]

    def forms(lo, hi, kinds=(0, 1, 2, 3)):
        a = rng.uniform(lo, hi, n)
        b = rng.uniform(lo, hi, n)
        kind = rng.choice(np.array(kinds), n)
        out = np.zeros((n, 4))
        out.view(np.int32)[:, 0] = kind
        out[:, 1] = a
        lin = kind == _lib.PF_LINEAR
        # linear: from a at t = 0 to b at T
        out[:, 2] = np.where(lin, (b - a) / T, b)
        out[:, 3] = np.where(lin, 0.0, T)
        return out

    for k in (0, 1):
        rec["nu"][:, k] = forms(0.01, 20)
        # exponential forms need ends of one sign
        rec["gamma"][:, k] = forms(-20, 20, kinds=(_lib.PF_CONST, _lib.PF_LINEAR))
        rec["h"][:, k] = forms(0.0, 1.0, kinds=(_lib.PF_CONST, _lib.PF_LINEAR))
    rec["m12"] = forms(0, 8)
    rec["m21"] = forms(0, 8)
    rec["theta0"] = forms(0.5, 2)
    return rec


def test_row_bounds_cover_the_schedules():
    """The host bounds that let the device schedule be filled in one pass
    are never below the rows the reference's time loop takes (the same walk
    in C on the host), for the 4096-draw IM workload, records with every
    parametric form, the old timestep and degenerate intervals; and they
    stay close (the workload reserves 1.26x its rows)."""
    from dadi_gb300 import batch
    st = batch.settings_from_globals()
    rec = batch.im_instances(cases.im_draws(4096))
    steps = batch.count_steps(rec, st)
    caps = batch.row_bounds(rec, st, [1e-3], 10 ** 8)
    assert np.all(caps >= steps)
    assert caps.sum() < 1.3 * steps.sum()
    mixed = _random_records(3000, seed=5)
    steps = batch.count_steps(mixed, st)
    caps = batch.row_bounds(mixed, st, [1e-3], 10 ** 8)
    assert caps is not None and np.all(caps >= steps)
    capped = batch.row_bounds(mixed, st, [1e-3], 50)
    assert np.all(capped <= 50) and np.all(capped >= np.minimum(steps, 50))
    old = batch.settings_from_globals()
    old.use_old_timestep = 1
    steps = batch.count_steps(mixed, old)
    caps = batch.row_bounds(mixed, old, [1e-3], 10 ** 8)
    assert np.all(caps >= steps)
    edge = mixed[:4].copy()
    edge["T"][0] = edge["initial_t"][0]        # no time to integrate
    edge["T"][1] = np.nan
    caps = batch.row_bounds(edge, st, [1e-3], 10 ** 8)
    assert caps[0] == 0 and caps[1] == 0
    bad = mixed[:2].copy()
    bad["nu"][0, 0] = batch._pf(0, 0.0)        # a zero size: no bound
    assert batch.row_bounds(bad, st, [1e-3], 10 ** 8) is None


def test_serving_stream_and_summary():
    """The serving workload's request stream (host side): seeded and
    reproducible, Poisson arrivals at the stated rate, the 70/20/8/2 class
    mix, gradients only on (40,40) IM requests with data, DFE entries on the
    50-point gamma grid; and the latency summary over finished requests."""
    from dadi_gb300 import serving
    obs = np.ones((41, 41))
    a = serving.config5_stream(2000, seed=3, rate=2000.0, obs=obs)
    b = serving.config5_stream(2000, seed=3, rate=2000.0, obs=obs)
    assert [(r.kind, r.params, r.pts_l, r.ns, r.arrival) for r in a] == \
        [(r.kind, r.params, r.pts_l, r.ns, r.arrival) for r in b]
    kinds = np.array([r.kind for r in a])
    frac = {k: float(np.mean(kinds == k)) for k in ("im", "im_sel", "growth3", "four")}
    for k, want in (("im", 0.70), ("im_sel", 0.20), ("growth3", 0.08), ("four", 0.02)):
        assert abs(frac[k] - want) < 0.03, frac
    arr = np.array([r.arrival for r in a])
    assert np.all(np.diff(arr) > 0) and abs(arr[-1] - 1.0) < 0.1  # 2000 at 2000/s
    gammas = -np.logspace(np.log10(2000), np.log10(1e-4), 50)
    for r in a:
        assert max(r.pts_l) <= 120
        if r.want_grad:
            assert r.kind == "im" and r.ns == (40, 40) and r.data is obs
        if r.kind == "im_sel":
            assert r.params[-2] in gammas and r.params[-1] in gammas
    assert any(r.want_grad for r in a)
    done = a[:10]
    for i, r in enumerate(done):
        r.t_done = r.arrival + 0.1 * (i + 1)
    done[3].error = "failed"
    summ = serving.latency_summary(done)
    lat = np.array([0.1 * (i + 1) for i in range(10) if i != 3])
    assert summ["completed"] == 9 and summ["errors"] == 1
    assert summ["p50_s"] == pytest.approx(np.percentile(lat, 50))
    assert summ["p99_s"] == pytest.approx(np.percentile(lat, 99))


def test_autotune_sample_spans_the_cost_quantiles():
    """The autotuner's sample: the requested number of instances, spread
    evenly over the 5-85 % quantiles of the batch's step counts, in batch
    order; the whole batch when it is smaller than the sample."""
    from dadi_gb300 import autotune, batch
    rec = batch.im_instances(cases.im_draws(1000))
    steps = batch.count_steps(rec)
    smp = autotune._sample(rec, 100)
    assert len(smp) == 100
    s = batch.count_steps(smp)
    lo, hi = np.sort(steps)[[int(0.05 * 999), int(0.85 * 999)]]
    assert s.min() >= lo and s.max() <= hi
    assert np.median(s) == pytest.approx(np.quantile(steps, 0.45), rel=0.25)
    idx = [int(np.nonzero(rec["T"] == t)[0][0]) for t in smp["T"]]
    assert idx == sorted(idx)
    assert len(autotune._sample(rec[:50], 100)) == 50


def test_cluster_adjoint_rule():
    """Batch2D's choice of a cluster per work item for the trajectory-mode
    backward walk: only when every item can have its cluster at once
    (instances x grids x CTAs <= SMs), every grid has 3-16 rows per CTA
    within 24-128 points, and the delj trick is off."""
    from dadi_gb300 import _lib, batch
    eng = batch.Batch2D.__new__(batch.Batch2D)
    st = _lib.settings_struct()
    ctx = lambda n, s=st: {"n": n, "st": s}
    eng.pts_l = (100, 110, 120)
    eng.cluster_adjoint = 8
    assert eng._cluster_adjoint_ctas(ctx(1), 152) == 8
    assert eng._cluster_adjoint_ctas(ctx(6), 152) == 8      # 144 CTAs
    assert eng._cluster_adjoint_ctas(ctx(7), 152) == 0      # 168 > 152
    assert eng._cluster_adjoint_ctas(ctx(1, _lib.settings_struct(use_delj_trick=True)),
                                     152) == 0
    eng.cluster_adjoint = 0
    assert eng._cluster_adjoint_ctas(ctx(1), 152) == 0
    eng.cluster_adjoint = 4                                  # 120 > 16 x 4 rows
    assert eng._cluster_adjoint_ctas(ctx(1), 152) == 0
    eng.cluster_adjoint = 16
    assert eng._cluster_adjoint_ctas(ctx(3), 152) == 16
    eng.pts_l = (20, 25, 30)                                 # below 24 points
    eng.cluster_adjoint = 8
    assert eng._cluster_adjoint_ctas(ctx(1), 152) == 0
    eng.pts_l = (30, 40, 50)
    assert eng._cluster_adjoint_ctas(ctx(1), 152) == 8
    eng.cluster_adjoint = 16                                 # 30 < 3 x 16 rows
    assert eng._cluster_adjoint_ctas(ctx(1), 152) == 0


def test_hybrid_plan():
    """The hybrid adjoint's split: longest items first into trajectory mode
    while their trajectories fit, at least one item each way, the clustered
    ones within a quarter of the SMs, and the segment-mode walk never on
    fewer than a quarter of the device's CTAs."""
    import numpy as np
    from dadi_gb300 import batch
    rng = np.random.default_rng(3)
    steps = rng.integers(10, 20000, 768)
    Lsq = np.tile(np.array([100 ** 2, 110 ** 2, 120 ** 2]), 256)
    size = (2 * steps + 1) * Lsq * 8
    for limit in (0, 4 << 30, 64 << 30, 1 << 50):
        for ctas, items in ((0, 0), (8, 4), (8, 100), (16, 2)):
            order, sz, k, j, rest = batch.hybrid_plan(steps, Lsq, limit, ctas, items, 152, 1)
            assert np.array_equal(sz, size)
            cost = (steps * Lsq)[order]
            assert np.all(cost[:-1] >= cost[1:])
            assert 1 <= k <= len(order) - 1
            if 1 < k < len(order) - 1:
                assert size[order[:k]].sum() <= limit < size[order[:k + 1]].sum()
            assert j <= min(k, items) and j * ctas <= 152 // 4
            assert (j == 0) == (ctas == 0 or items == 0)
            assert min(len(order) - k, 38) <= rest <= len(order) - k
    # few items: the segment mode keeps its items even when clusters and
    # trajectory items would take every SM
    order, sz, k, j, rest = batch.hybrid_plan([5000] * 12, [14400] * 12, 1 << 50, 8, 4, 152, 1)
    assert (k, j, rest) == (11, 4, 1)


def _partition_solve(a, b, c, d, bounds):
    """The partitioned tridiagonal solve of the cluster sweeps
    (csrc/dgb_cluster.cuh), restated in numpy: each segment [s, e) (at least
    three points) runs its downward pass over s+1 .. e-1, giving
    al x_s + x_i + ga x_(i+1) = de; its upward pass expresses every interior
    point by the segment's first point x_s and last point z; the first row
    then gives x_s = D' - A' z_prev - C' z; substituting both segments'
    first points into each last row leaves a tridiagonal system in the
    segments' last points, solved by Thomas; the interior points follow."""
    import numpy as np
    S = len(bounds)
    x = np.zeros_like(d)
    Ap, Cp, Dp, al_l, ga_l, de_l = (np.zeros(S) for _ in range(6))
    rel = []
    for q, (s, e) in enumerate(bounds):
        al, ga, de = {}, {}, {}
        i = s + 1
        al[i], ga[i], de[i] = a[i] / b[i], c[i] / b[i], d[i] / b[i]
        for i in range(s + 2, e):
            inv = 1.0 / (b[i] - a[i] * ga[i - 1])
            al[i], ga[i], de[i] = -a[i] * al[i - 1] * inv, c[i] * inv, (d[i] - a[i] * de[i - 1]) * inv
        al_l[q], ga_l[q], de_l[q] = al[e - 1], ga[e - 1], de[e - 1]
        deu, alu, gau = de[e - 2], al[e - 2], ga[e - 2]
        up = {e - 2: (deu, alu, gau)}
        for i in range(e - 3, s, -1):
            deu, alu, gau = de[i] - ga[i] * deu, al[i] - ga[i] * alu, -ga[i] * gau
            up[i] = (deu, alu, gau)
        B = b[s] - c[s] * alu
        Ap[q], Cp[q], Dp[q] = a[s] / B, -c[s] * gau / B, (d[s] - c[s] * deu) / B
        rel.append(up)
    # the system in the last points z_q
    ra = -al_l * Ap
    rb = 1.0 - al_l * Cp - ga_l * np.append(Ap[1:], 0.0)
    rc = -ga_l * np.append(Cp[1:], 0.0)
    rd = de_l - al_l * Dp - ga_l * np.append(Dp[1:], 0.0)
    z = np.linalg.solve(np.diag(rb) + np.diag(ra[1:], -1) + np.diag(rc[:-1], 1), rd)
    for q, (s, e) in enumerate(bounds):
        zp = z[q - 1] if q else 0.0
        xf = Dp[q] - Ap[q] * zp - Cp[q] * z[q]
        x[s], x[e - 1] = xf, z[q]
        for i, (deu, alu, gau) in rel[q].items():
            x[i] = deu - alu * xf - gau * z[q]
    return x


@pytest.mark.parametrize("L,S", [(24, 8), (37, 4), (100, 8), (128, 16), (48, 16), (30, 2)])
def test_partition_solve_matches_dense(L, S):
    """The partition method's algebra (as the cluster kernels apply it, rows
    of each CTA or segment as c2_rows splits them) solves random
    diagonally dominant tridiagonal systems and their transposes to 1e-12
    of a dense solve."""
    import numpy as np
    rng = np.random.default_rng(L * 100 + S)
    base, extra = L // S, L % S
    starts = [r * base + min(r, extra) for r in range(S)]
    bounds = [(s0, s0 + base + (1 if r < extra else 0)) for r, s0 in enumerate(starts)]
    assert all(e - s >= 3 for s, e in bounds)
    a, c = rng.uniform(-1, 0, L), rng.uniform(-1, 0, L)
    a[0], c[-1] = 0.0, 0.0
    b = 1.0 + np.abs(a) + np.abs(c) + rng.uniform(0, 1, L)
    d = rng.normal(size=L)
    M = np.diag(b) + np.diag(a[1:], -1) + np.diag(c[:-1], 1)
    for sub, diag, sup, mat in ((a, b, c, M), (np.append(0.0, c[:-1]), b, np.append(a[1:], 0.0), M.T)):
        x = _partition_solve(sub, diag, sup, d, bounds)
        ref = np.linalg.solve(mat, d)
        assert np.max(np.abs(x - ref)) <= 1e-12 * np.max(np.abs(ref))
