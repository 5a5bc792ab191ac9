"""Host side of the batched N-dimensional engine (no GPU): the parametric
schedules walked in C (dgb_schednd_host) equal the reference loop's tables
(integration.build_table, which follows dadi/Integration.py:389-937 step by
step): the same steps and step lengths bit for bit, and the sizes to within
an ulp or two (the C walk evaluates exp and log with the C library, the
Python callables with numpy's own routines)."""
import numpy as np
import pytest

from dadi_gb300 import _lib, batchnd, integration, models


def _table_of(ndim, T, nu_f, mig_f, gamma, h):
    f = integration.ensure_1arg_func
    xx = np.linspace(0, 1, 10)
    mf = [[None if j == k else f(mig_f[k][j]) for j in range(ndim)] for k in range(ndim)]
    tab, _ = integration.build_table(ndim, xx, T, 0.0, [f(v) for v in nu_f], mf,
                                     [f(v) for v in gamma], [f(v) for v in h], f(1.0))
    return tab


def _assert_same_table(tab, ref):
    assert tab.shape == ref.shape
    assert np.array_equal(tab[:, 0], ref[:, 0])       # step lengths
    rel = np.abs(tab - ref) / np.maximum(np.abs(ref), 1e-300)
    assert float(rel.max()) <= 5e-16, float(rel.max())


def _growth3_callables(params):
    (nu0, nuF, (m12, m13, m23), g, T) = params
    nus = [(lambda a, b: (lambda t: a * np.exp(np.log(b / a) * t / T)))(a, b)
           for a, b in zip(nu0, nuF)]
    mig = [[0, m12, m13], [m12, 0, m23], [m13, m23, 0]]
    return nus, mig, list(g), T


@pytest.mark.parametrize("scale", [1.0, 0.6, 1.7])
def test_growth3_schedule_equals_reference_loop(scale):
    nu0, nuF, m, g, T = models.GROWTH3_DEFAULT
    params = (tuple(v * scale for v in nu0), nuF, tuple(v / scale for v in m), g, T * scale)
    tabs, status = batchnd.schedules([batchnd.growth3_instance(params)])
    nus, mig, gam, T = _growth3_callables(params)
    ref = _table_of(3, T, nus, mig, gam, [0.5] * 3)
    assert status[0] == 0
    _assert_same_table(tabs[0], ref)


def test_four_split_schedule_equals_reference_loop():
    p = models.FOUR_DEFAULT
    tabs, status = batchnd.schedules([batchnd.four_split_instance(p)])
    nu1, nu2, nu3, nu4, m, T = p
    mig = [[0 if j == k else m for j in range(4)] for k in range(4)]
    ref = _table_of(4, T, [nu1, nu2, nu3, nu4], mig, [0.0] * 4, [0.5] * 4)
    assert status[0] == 0 and np.array_equal(tabs[0], ref)  # constants: exact


def test_schedule_reports_bad_parameters():
    """A negative migration rate sets DGB_ST_BADPARAM, where the reference
    raises ValueError (dadi/Integration.py:540-546)."""
    nu0, nuF, m, g, T = models.GROWTH3_DEFAULT
    bad = (nu0, nuF, (0.5, -1.0, 3.0), g, T)
    _, status = batchnd.schedules([batchnd.growth3_instance(bad),
                                   batchnd.growth3_instance(models.GROWTH3_DEFAULT)])
    assert status[0] & _lib.ST_BADPARAM and status[1] == 0


@pytest.mark.parametrize("theta_scale", [1.0, 0.7, 1.3])
def test_dual_schedule_in_c_equals_python(theta_scale):
    """The schedule walk in dual numbers (dgb_schednd_dual_host) gives the
    rows of dgb_schednd_host bit for bit, and rows and derivatives equal to
    the Python walk (adjoint_nd.table_dual) within an ulp or two (libm
    against numpy's exp and log)."""
    from dadi_gb300 import adjoint_nd, numerics
    g3 = adjoint_nd.Growth3.__new__(adjoint_nd.Growth3)  # the table needs no device
    g3.gammas = (-2.0, 0.0, 5.0)
    theta = g3.from_model_params(models.GROWTH3_DEFAULT) * theta_scale
    xx = numerics.default_grid(12)
    tab, drows = g3.table(theta, xx)
    plain, status = batchnd.schedules([batchnd.growth3_instance(g3.model_params(theta))])
    assert status[0] == 0 and np.array_equal(tab, plain[0])
    ref, dref = g3.table_python(theta, xx)
    _assert_same_table(tab, ref)
    assert drows.shape == dref.shape == tab.shape + (10,)
    scale = np.maximum(np.abs(dref).max(axis=0, keepdims=True), 1e-300)
    assert float((np.abs(drows - dref) / scale).max()) <= 1e-14


def test_dual_schedule_linear_and_power_forms_match_differences():
    """Derivatives of the forms the Python walk does not cover (a + b t and
    a (b / a)^(t / c)) against central differences of the rows."""
    from dadi_gb300 import adjoint_nd
    T = 0.05
    xx = np.linspace(0, 1, 12)

    def rec(v):
        nu = [batchnd._pf(_lib.PF_LINEAR, v[0], 2.0), batchnd._pf(_lib.PF_EXPGROW, 0.5, v[1], T)]
        return batchnd.instance(2, T, nu, [[0, 0.3], [0.2, 0]], gamma=[0.0, 1.0])
    v0 = np.array([1.0, 3.0])
    seed = _lib.SeedND()
    seed.dnu[0][0][0] = 1.0
    seed.dnu[1][1][1] = 1.0
    tab, drows = adjoint_nd.schedule_dual(rec(v0), seed, 2, xx)
    cols = [2, 3]  # nu1, nu2
    for p in range(2):
        e = np.zeros(2)
        e[p] = 1e-6 * v0[p]
        tp, _ = adjoint_nd.schedule_dual(rec(v0 + e), seed, 2, xx)
        tm, _ = adjoint_nd.schedule_dual(rec(v0 - e), seed, 2, xx)
        assert len(tp) == len(tm) == len(tab)
        fd = (tp[:, cols] - tm[:, cols]) / (2 * e[p])
        err = np.abs(fd - drows[:, cols, p]).max() / max(np.abs(fd).max(), 1e-300)
        assert err < 1e-6, (p, err)


def test_partition_segment_rule():
    """Segments per line of the drop-in's partitioned solve: at least 8 rows
    per segment, none for 1-2 populations, the delj trick or "thomas"; a
    fixed count when nd_segments is set (without a GPU: "partition" mode)."""
    saved = integration.nd_line_solver, integration.nd_segments
    try:
        integration.nd_line_solver = "partition"
        assert integration.partition_segments(3, 70) == 8
        assert integration.partition_segments(3, 40) == 4
        assert integration.partition_segments(4, 20) == 2
        assert integration.partition_segments(4, 12) == 0
        assert integration.partition_segments(2, 90) == 0
        assert integration.partition_segments(3, 90, delj=True) == 0
        integration.nd_segments = 4
        assert integration.partition_segments(3, 12) == 4
        assert integration.partition_segments(3, 11) == 0
        integration.nd_line_solver = "thomas"
        assert integration.partition_segments(3, 90) == 0
        integration.nd_line_solver = "fast"
        with pytest.raises(ValueError):
            integration.partition_segments(3, 90)
    finally:
        integration.nd_line_solver, integration.nd_segments = saved
