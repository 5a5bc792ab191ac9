"""The batched N-dimensional engine (dgb_batchnd_integrate): every
integration of a batch gives bitwise the density the one-at-a-time path
(dgb_integrate_table) gives it alone -- 3-D, 4-D and 5-D, integrations of
different lengths, frozen and nomut populations, the delj trick, both
Thomas-scratch placements and every lines-per-CTA choice -- and config 2
through the batch matches dadi's golden spectrum."""
import numpy as np
import pytest

import cases
from util import assert_fs_parity, table_rows

pytestmark = pytest.mark.gpu


def _alone(phi0, xx, table, masks, delj=False):
    """The drop-in's one-at-a-time integration with the Thomas solve
    (dgb_integrate_table)."""
    from dadi_gb300 import integration
    saved = integration.use_delj_trick, integration.nd_line_solver, integration.line_solver_2d
    integration.use_delj_trick, integration.nd_line_solver = delj, "thomas"
    integration.line_solver_2d = "thomas"
    try:
        return integration.run_table(phi0, xx, table, masks & 0xff, masks >> 8)
    finally:
        (integration.use_delj_trick, integration.nd_line_solver,
         integration.line_solver_2d) = saved


@pytest.mark.parametrize("P,L,gam,threads,delj", [
    (3, 20, 0, 0, False), (3, 20, 1, 0, False), (3, 21, 2, 32, False), (3, 20, 2, 128, True),
    (4, 12, 0, 0, False), (4, 12, 1, 64, True), (5, 7, 0, 0, False), (2, 24, 0, 0, False),
])
def test_batch_equals_alone(cuda_lib, P, L, gam, threads, delj):
    import torch
    from dadi_gb300 import batchnd, integration
    xx = cases.grid("default", L)
    n = 6
    tables = [table_rows(P, nst, 100 + k) for k, nst in enumerate([7, 19, 3, 19, 11, 1])]
    masks = [0, 1, 2 << 8, 0, (1 << (P - 1)) | (1 << 8), 0]
    phi0 = np.stack([cases.initial_phi(40 + k, (L,) * P) for k in range(n)])
    saved = integration.use_delj_trick
    integration.use_delj_trick = delj
    try:
        eng = batchnd.BatchND(P, L, xx=xx, gam_placement=gam, threads=threads)
        out = eng.integrate(torch.from_numpy(phi0).cuda(), tables, masks).cpu().numpy()
    finally:
        integration.use_delj_trick = saved
    for k in range(n):
        ref = _alone(phi0[k], xx, tables[k], masks[k], delj)
        assert np.array_equal(out[k], ref), (k, float(np.max(np.abs(out[k] - ref))))


def test_batch_shared_initial_density(cuda_lib):
    """One initial density for every integration of the batch."""
    import torch
    from dadi_gb300 import batchnd
    P, L = 3, 16
    xx = cases.grid("default", L)
    phi0 = cases.initial_phi(5, (L,) * P)
    tables = [table_rows(P, 5 + k, 200 + k) for k in range(4)]
    out = batchnd.BatchND(P, L, xx=xx).integrate(torch.from_numpy(phi0).cuda(), tables)
    out = out.cpu().numpy()
    for k in range(4):
        assert np.array_equal(out[k], _alone(phi0, xx, tables[k], 0))


def test_growth3_batch_extrapolated_matches_dadi(cuda_lib, golden):
    """Config 2 (three populations, exponential growth, pts [70,80,90], ns
    (20,20,20)) with schedules walked in C and the grids integrated as
    batches: the extrapolated spectrum within the spectrum bar of dadi's."""
    import torch
    from dadi_gb300 import batchnd, numerics, spectrum
    g = cases.GROWTH3
    rec = batchnd.growth3_instance(g["params"])
    tabs, status = batchnd.schedules([rec])
    assert status[0] == 0 and len(tabs[0]) == 675
    res = []
    for L in g["pts_l"]:
        eng = batchnd.BatchND(3, L)
        phi0 = torch.from_numpy(batchnd.initial_density("growth3", L)).cuda()
        phi = eng.integrate(phi0, [tabs[0]])[0]
        xx = numerics.default_grid(L)
        res.append(spectrum.from_phi(phi, g["ns"], (xx, xx, xx)))
    fs = numerics.extrapolate(res, [r.extrap_x for r in res])
    assert_fs_parity(np.asarray(fs.data), golden["models"]["growth3_fs"])


@pytest.mark.parametrize("kind,pts_l,ns", [("growth3", [16, 20, 24], (6, 7, 8)),
                                           ("four", [10, 12, 14], (3, 4, 3, 5))])
def test_model_batch_equals_drop_in(cuda_lib, kind, pts_l, ns):
    """ModelBatch (schedules in C, batched integration per grid, N-D
    from_phi, device extrapolation and likelihood) gives each parameter set
    the spectrum and likelihood of the one-at-a-time drop-in."""
    from dadi_gb300 import batchnd, inference, models, numerics, spectrum
    base = models.GROWTH3_DEFAULT if kind == "growth3" else models.FOUR_DEFAULT
    if kind == "growth3":
        sets = [base, (base[0], base[1], (1.0, 0.7, 2.0), base[3], 0.07),
                ((1.0, 0.6, 3.0), (2.0, 0.3, 6.0), base[2], (0.0, 1.0, -3.0), 0.11)]
        fn = models.growth3
    else:
        sets = [base, (0.9, 1.4, 0.6, 2.5, 0.8, 0.03), (2.0, 2.0, 0.5, 0.5, 0.1, 0.04)]
        fn = models.four_split
    data = np.random.default_rng(3).poisson(50, size=tuple(n + 1 for n in ns)).astype(float)
    fs, ll, status = batchnd.ModelBatch(kind, pts_l, ns).run(sets, data=data, scale=1e3)
    assert not status.any()
    fs, ll = fs.cpu().numpy(), ll.cpu().numpy()
    f = numerics.make_extrap_func(fn)
    for k, p in enumerate(sets):
        ref = f(p, ns, pts_l)
        assert_fs_parity(fs[k], np.asarray(ref.data))
        ll_ref = inference.ll(1e3 * ref, spectrum.Spectrum(data))
        assert abs(ll[k] - ll_ref) <= 1e-9 * abs(ll_ref)


def test_model_batch_config2_matches_dadi(cuda_lib, golden):
    """Config 2 through ModelBatch (a batch of one) against dadi."""
    from dadi_gb300 import batchnd
    g = cases.GROWTH3
    fs, _, status = batchnd.ModelBatch("growth3", g["pts_l"], g["ns"]).run([g["params"]])
    assert not status.any()
    assert_fs_parity(fs.cpu().numpy()[0], golden["models"]["growth3_fs"])


@pytest.mark.parametrize("P,L", [(3, 20), (3, 33), (4, 12), (1, 100), (2, 128)])
def test_pcr_line_solver_matches_thomas(cuda_lib, P, L):
    """The alternative line solver (parallel cyclic reduction, one warp per
    line) solves the same systems as Thomas: the densities agree to 1e-12
    relative (a different order of the same arithmetic)."""
    import torch
    from dadi_gb300 import batchnd
    xx = cases.grid("default", L)
    tables = [table_rows(P, nst, 300 + k) for k, nst in enumerate([9, 4, 9])]
    masks = [0, 0, 1 << 8]
    phi0 = np.stack([np.abs(cases.initial_phi(50 + k, (L,) * P)) + 1e-3 for k in range(3)])
    d0 = torch.from_numpy(phi0).cuda()
    th = batchnd.BatchND(P, L, xx=xx).integrate(d0, tables, masks).cpu().numpy()
    pc = batchnd.BatchND(P, L, xx=xx, line_solver=1).integrate(d0, tables, masks)
    pc = pc.cpu().numpy()
    for k in range(3):
        rel = np.max(np.abs(pc[k] - th[k]) / np.maximum(np.abs(th[k]), 1e-12 * np.abs(th[k]).max()))
        assert rel < 1e-12, (k, rel)


def test_pcr_line_solver_config2_matches_dadi(cuda_lib, golden):
    """Config 2 with the PCR line solver, against dadi."""
    import torch
    from dadi_gb300 import batchnd, numerics, spectrum
    g = cases.GROWTH3
    tabs, _ = batchnd.schedules([batchnd.growth3_instance(g["params"])])
    res = []
    for L in g["pts_l"]:
        eng = batchnd.BatchND(3, L, line_solver=1)
        phi = eng.integrate(torch.from_numpy(batchnd.initial_density("growth3", L)).cuda(),
                            tabs)[0]
        xx = numerics.default_grid(L)
        res.append(spectrum.from_phi(phi, g["ns"], (xx, xx, xx)))
    fs = numerics.extrapolate(res, [r.extrap_x for r in res])
    assert_fs_parity(np.asarray(fs.data), golden["models"]["growth3_fs"])


@pytest.mark.parametrize("P,L,seg", [(3, 20, 4), (3, 33, 2), (3, 33, 8), (4, 12, 4),
                                     (1, 100, 8), (2, 128, 4), (3, 9, 2)])
def test_partition_line_solver_matches_thomas(cuda_lib, P, L, seg):
    """The partitioned Thomas solve (segments of a line on their own threads,
    the segments' end points from a small tridiagonal system) solves the same
    systems as Thomas: the densities agree to 1e-12 relative, every axis,
    contiguous and strided, uneven segment lengths, a frozen population."""
    import torch
    from dadi_gb300 import batchnd
    xx = cases.grid("default", L)
    tables = [table_rows(P, nst, 400 + k) for k, nst in enumerate([9, 4, 9])]
    masks = [0, 0, 1 << 8] if P == 1 else [0, 1, 1 << 8]
    phi0 = np.stack([np.abs(cases.initial_phi(60 + k, (L,) * P)) + 1e-3 for k in range(3)])
    d0 = torch.from_numpy(phi0).cuda()
    th = batchnd.BatchND(P, L, xx=xx).integrate(d0, tables, masks).cpu().numpy()
    pt = batchnd.BatchND(P, L, xx=xx, line_solver=2, segments=seg).integrate(d0, tables, masks)
    pt = pt.cpu().numpy()
    for k in range(3):
        rel = np.max(np.abs(pt[k] - th[k]) / np.maximum(np.abs(th[k]), 1e-12 * np.abs(th[k]).max()))
        assert rel < 1e-12, (k, rel)


def test_partition_line_solver_config2_matches_dadi(cuda_lib, golden):
    """Config 2 with the partitioned solver (4 segments), against dadi."""
    import torch
    from dadi_gb300 import batchnd, numerics, spectrum
    g = cases.GROWTH3
    tabs, _ = batchnd.schedules([batchnd.growth3_instance(g["params"])])
    res = []
    for L in g["pts_l"]:
        eng = batchnd.BatchND(3, L, line_solver=2, segments=4)
        phi = eng.integrate(torch.from_numpy(batchnd.initial_density("growth3", L)).cuda(),
                            tabs)[0]
        xx = numerics.default_grid(L)
        res.append(spectrum.from_phi(phi, g["ns"], (xx, xx, xx)))
    fs = numerics.extrapolate(res, [r.extrap_x for r in res])
    assert_fs_parity(np.asarray(fs.data), golden["models"]["growth3_fs"])


def test_partition_rejects_what_it_does_not_solve(cuda_lib):
    """Segments of fewer than three rows, an unknown segment count and the
    delj trick are refused with a status, not solved differently."""
    import torch
    from dadi_gb300 import _lib, batchnd, integration
    tab = [table_rows(3, 2, 7)]
    for L, seg in ((8, 4), (20, 3)):
        eng = batchnd.BatchND(3, L, line_solver=2, segments=seg)
        with pytest.raises(_lib.DgbError):
            eng.integrate(torch.ones((L,) * 3, dtype=torch.float64, device="cuda"), tab)
    saved = integration.use_delj_trick
    integration.use_delj_trick = True
    try:
        eng = batchnd.BatchND(3, 20, line_solver=2)
        with pytest.raises(_lib.DgbError):
            eng.integrate(torch.ones((20,) * 3, dtype=torch.float64, device="cuda"), tab)
    finally:
        integration.use_delj_trick = saved


@pytest.mark.parametrize("P,L,frozen", [(3, 70, 0), (3, 40, 2), (4, 20, 0)])
def test_dropin_partition_path_matches_thomas(cuda_lib, P, L, frozen):
    """The drop-in's partitioned path (a lone 3-D / 4-D grid as a batch of
    one) gives densities within 1e-12 relative of the Thomas path, masks
    included, from host and from device densities alike."""
    import torch
    from dadi_gb300 import integration
    xx = cases.grid("default", L)
    phi0 = np.abs(cases.initial_phi(3, (L,) * P)) + 1e-3
    tab = table_rows(P, 40, 77)
    saved = integration.nd_line_solver
    integration.nd_line_solver = "partition"
    try:
        assert integration.partition_segments(P, L) > 0
        part = integration.run_table(phi0, xx, tab, frozen, 0)
        dev = integration.run_table(torch.from_numpy(phi0).cuda(), xx, tab, frozen, 0)
    finally:
        integration.nd_line_solver = saved
    assert np.array_equal(dev.cpu().numpy(), part)
    th = _alone(phi0, xx, tab, frozen)
    rel = np.max(np.abs(part - th) / np.maximum(np.abs(th), 1e-12 * np.abs(th).max()))
    assert rel < 1e-12, rel


def test_dropin_auto_line_solver_is_tuned_per_shape(cuda_lib):
    """"auto" asks the autotuner once per shape: the partition for a 3-D
    grid of 60 points (few lines: measured 1.9x), a cached answer the second
    time; never for the delj trick or two populations."""
    from dadi_gb300 import autotune, integration
    assert integration.nd_line_solver == "auto"
    t = autotune.tune_nd_line_solver(3, 60)
    assert t["segments"] in (2, 4, 8) and set(t["ms"]) >= {0, 2, 4, 8}
    assert autotune.tune_nd_line_solver(3, 60) is t
    assert integration.partition_segments(3, 60) == t["segments"]
    assert integration.partition_segments(3, 70, delj=True) == 0
    assert integration.partition_segments(2, 100) == 0
