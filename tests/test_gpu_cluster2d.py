"""One 2-D integration spread over a thread-block cluster
(dgb_integrate2d_cluster): the partitioned solves across and within the
cluster's CTAs agree with the one-CTA Thomas path (dgb_integrate_table) to
1e-12 relative -- every cluster size, grids from 24 to 128 points, uneven row
blocks, frozen and nomut populations -- and the drop-in's IM model through
the cluster path matches dadi's golden spectrum."""
import numpy as np
import pytest

import cases
from util import assert_fs_parity, table_rows

pytestmark = pytest.mark.gpu


def _run(lib, torch, phi0, xx, tab, frozen, nomut, ctas):
    from dadi_gb300 import _lib
    L = len(xx)
    d_phi = torch.from_numpy(phi0.copy()).cuda()
    d_xx = torch.from_numpy(xx).cuda()
    d_tab = torch.from_numpy(tab).cuda()
    sh = _lib.stream_handle(torch)
    if ctas:
        _lib.check(lib.dgb_integrate2d_cluster(_lib.dptr(d_phi), L, _lib.dptr(d_xx),
                                               _lib.dptr(d_tab), len(tab), frozen, nomut, ctas,
                                               sh), "dgb_integrate2d_cluster")
    else:
        ws, nws = _lib.workspace(torch, lib.dgb_workspace_bytes(0, 2, L, 0))
        _lib.check(lib.dgb_integrate_table(_lib.dptr(d_phi), 2, L, _lib.dptr(d_xx),
                                           _lib.dptr(d_tab), len(tab), frozen, nomut, 0,
                                           _lib.dptr(ws), nws, sh), "dgb_integrate_table")
    return d_phi.cpu().numpy()


@pytest.mark.parametrize("L,ctas,frozen,nomut", [
    (24, 2, 0, 0), (24, 8, 0, 0), (40, 4, 1, 0), (64, 8, 0, 2), (100, 8, 0, 0),
    (101, 8, 2, 0), (120, 8, 0, 1), (128, 8, 0, 0), (128, 16, 0, 0), (48, 16, 0, 0)])
def test_cluster_matches_thomas(cuda_lib, L, ctas, frozen, nomut):
    import torch
    xx = cases.grid("default", L)
    phi0 = np.abs(cases.initial_phi(90 + L, (L, L))) + 1e-3
    tab = table_rows(2, 60, 600 + L)
    ref = _run(cuda_lib, torch, phi0, xx, tab, frozen, nomut, 0)
    out = _run(cuda_lib, torch, phi0, xx, tab, frozen, nomut, ctas)
    assert np.all(np.isfinite(out))
    rel = np.max(np.abs(out - ref) / np.maximum(np.abs(ref), 1e-12 * np.abs(ref).max()))
    assert rel < 1e-12, rel


def test_cluster_rejects_what_it_does_not_solve(cuda_lib):
    """Grids outside 24..128 points or 3..16 rows per CTA and cluster sizes
    other than 2, 4, 8, 16 are refused with a status before any launch."""
    import torch
    from dadi_gb300 import _lib
    lib = cuda_lib
    for L, ctas, want in ((20, 2, _lib.DGB_ERR_UNSUPPORTED), (130, 16, _lib.DGB_ERR_UNSUPPORTED),
                          (40, 2, _lib.DGB_ERR_UNSUPPORTED), (30, 16, _lib.DGB_ERR_UNSUPPORTED),
                          (40, 3, _lib.DGB_ERR_ARG)):
        phi = torch.ones((L, L), dtype=torch.float64, device="cuda")
        xx = torch.from_numpy(cases.grid("default", L)).cuda()
        tab = torch.from_numpy(table_rows(2, 2, 1)).cuda()
        rc = lib.dgb_integrate2d_cluster(_lib.dptr(phi), L, _lib.dptr(xx), _lib.dptr(tab), 2,
                                         0, 0, ctas, _lib.stream_handle(torch))
        assert rc == want, (L, ctas, rc)


@pytest.mark.parametrize("i", [1, 5])
def test_dropin_im_through_the_cluster_matches_dadi(cuda_lib, golden, i):
    """The drop-in's IM model (pts 80/90/100, ns (40,40)) and split_mig (pts
    40/50/60) with every grid on an 8-CTA cluster: the extrapolated spectra
    within the spectrum bar of dadi's golden ones."""
    from dadi_gb300 import integration, models, numerics
    saved = integration.line_solver_2d, integration.cluster_ctas
    integration.line_solver_2d, integration.cluster_ctas = "cluster", 8
    try:
        assert integration.cluster_size_2d(80) == 8
        fs = numerics.make_extrap_func(models.IM)(cases.im_draws()[i], (40, 40), [80, 90, 100])
        sm = cases.SPLIT_MIG
        fs2 = numerics.make_extrap_func(models.split_mig)(sm["params"], sm["ns"], sm["pts_l"])
    finally:
        integration.line_solver_2d, integration.cluster_ctas = saved
    assert_fs_parity(np.asarray(fs.data), golden["models"]["im_fs_%d" % i])
    assert_fs_parity(np.asarray(fs2.data), golden["models"]["splitmig_fs"])


def test_dropin_auto_2d_is_tuned_per_grid(cuda_lib):
    """"auto" asks the autotuner once per grid size; the answer is a size
    the kernel accepts (or 0, the one-CTA path) and is cached."""
    from dadi_gb300 import autotune, integration
    t = autotune.tune_2d_cluster(100)
    assert t["ctas"] in (0, 8, 16) and 0 in t["ms"]
    assert autotune.tune_2d_cluster(100) is t
    assert integration.cluster_size_2d(100) == t["ctas"]
    assert integration.cluster_size_2d(100, delj=True) == 0
    assert integration.cluster_size_2d(20) == 0


def test_items_on_clusters_match_one_cta_per_item(cuda_lib):
    """dgb_items2d_integrate_cluster (one cluster of 8 CTAs per work item,
    grids of 40-120 points, own schedules and masks) against
    dgb_items2d_integrate (one CTA per item): 1e-12 relative; an item
    outside the checked grid range is left untouched."""
    import ctypes
    import torch
    from dadi_gb300 import _lib, batch
    lib = cuda_lib
    Ls = [40, 64, 120, 100, 33]
    xx_h = [cases.grid("default", L) for L in Ls]
    xx_off = np.cumsum([0] + Ls[:-1])
    tabs = [table_rows(2, n, 700 + k) for k, n in enumerate([30, 12, 25, 1, 5])]
    roff = np.cumsum([0] + [len(t) for t in tabs[:-1]]).astype(np.int64)
    cnt = np.array([len(t) for t in tabs], dtype=np.int32)
    items = np.zeros(5, dtype=batch.ITEM2D_DTYPE)
    phi0, off = [], 0
    for k, L in enumerate(Ls):
        items["L"][k], items["xx_off"][k], items["out_off"][k] = L, xx_off[k], off
        items["sched"][k], items["masks"][k] = k, [0, 1, 0, 2 << 8, 0][k]
        phi0.append((np.abs(cases.initial_phi(30 + k, (L, L))) + 1e-3).reshape(-1))
        off += L * L
    d_items = _lib.to_device(torch, items.view(np.uint8), np.uint8)
    d_xx = torch.from_numpy(np.concatenate(xx_h)).cuda()
    d_tab = torch.from_numpy(np.concatenate(tabs)).cuda()
    d_roff = torch.from_numpy(roff).cuda()
    d_cnt = torch.from_numpy(cnt).cuda()
    sh = _lib.stream_handle(torch)
    ref = torch.from_numpy(np.concatenate(phi0)).cuda()
    st = _lib.settings_struct()
    ws, nws = _lib.workspace(torch, lib.dgb_workspace_bytes(3, 2, 120, 5))
    _lib.check(lib.dgb_items2d_integrate(_lib.dptr(d_items), 5, 120, _lib.dptr(d_xx),
                                         _lib.dptr(ref), _lib.dptr(d_tab), _lib.dptr(d_roff),
                                         _lib.dptr(d_cnt), None, ctypes.byref(st), 1,
                                         _lib.dptr(ws), nws, sh), "dgb_items2d_integrate")
    out = torch.from_numpy(np.concatenate(phi0)).cuda()
    _lib.check(lib.dgb_items2d_integrate_cluster(_lib.dptr(d_items), 5, 40, 120, _lib.dptr(d_xx),
                                                 _lib.dptr(out), _lib.dptr(d_tab),
                                                 _lib.dptr(d_roff), _lib.dptr(d_cnt), 8,
                                                 None, None, 0, sh),
               "dgb_items2d_integrate_cluster")
    ref, out = ref.cpu().numpy(), out.cpu().numpy()
    off = 0
    for k, L in enumerate(Ls):
        a, b = out[off:off + L * L], ref[off:off + L * L]
        if L < 40:   # outside [Lmin, Lmax]: skipped
            assert np.array_equal(a, phi0[k])
        else:
            rel = np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-12 * np.abs(b).max()))
            assert rel < 1e-12, (k, rel)
        off += L * L
