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
