"""The allocation-free 2-D entry point (dgb_integrate2d_noalloc).

Some callers cannot allocate device memory or hand the library a workspace:
code running where cudaMalloc is not allowed, or a host embedding the library
without an allocator of its own.  For them the library keeps its Thomas
scratch in a static device array of at most DGB_NOALLOC_MAX_L^2 doubles.  This
test calls that entry point through the C ABI twice in a row (the array keeps
the previous call's contents) and checks each result against the workspace
entry point dgb_integrate_table on the same inputs, within the tolerance the
other single-integration tests use.  It lives in a file pytest collects last
so that a run stopping at the first failure has run everything else first.
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, entries below 1e-12 of the maximum compared absolutely


def _table_case(L, seed, T):
    from dadi_gb300 import integration as gi
    xx = cases.grid("default", L)
    phi0 = cases.initial_phi(seed, (L, L))
    f = gi.ensure_1arg_func
    nu1 = lambda t: 0.4 * (3.0 / 0.4) ** (t / T)
    table, _ = gi.build_table(2, xx, T, 0.0, [f(nu1), f(1.3)],
                              [[None, f(0.8)], [f(1.7), None]], [f(-0.5), f(0.0)],
                              [f(0.3), f(0.5)], f(1.0))
    return xx, phi0, table


def _run(lib, name, L, xx, phi0, table):
    import torch
    from dadi_gb300 import _lib
    d_phi = torch.from_numpy(phi0.copy()).cuda()
    d_xx = torch.from_numpy(xx).cuda()
    d_tab = torch.from_numpy(np.ascontiguousarray(table)).cuda()
    sh = _lib.stream_handle(torch)
    if name == "noalloc":
        rc = lib.dgb_integrate2d_noalloc(_lib.dptr(d_phi), L, _lib.dptr(d_xx), _lib.dptr(d_tab),
                                         len(table), 0, 0, 0, sh)
    else:
        nws = lib.dgb_workspace_bytes(0, 2, L, 0)
        ws, nws = _lib.workspace(torch, nws)
        rc = lib.dgb_integrate_table(_lib.dptr(d_phi), 2, L, _lib.dptr(d_xx), _lib.dptr(d_tab),
                                     len(table), 0, 0, 0, _lib.dptr(ws), nws, sh)
    assert rc == 0, _lib.status_string(rc)
    torch.cuda.synchronize()
    return d_phi.cpu().numpy()


def _close(a, b):
    floor = 1e-12 * np.max(np.abs(b))
    rel = np.abs(a - b) / np.maximum(np.abs(b), floor)
    return float(np.max(rel))


def test_noalloc_matches_workspace_entry_point_twice(cuda_lib):
    from dadi_gb300 import _lib
    for L, seed, T in [(120, 7, 0.05), (64, 8, 0.08)]:
        xx, phi0, table = _table_case(L, seed, T)
        ref = _run(cuda_lib, "table", L, xx, phi0, table)
        first = _run(cuda_lib, "noalloc", L, xx, phi0, table)
        second = _run(cuda_lib, "noalloc", L, xx, phi0, table)
        assert _close(first, ref) < TOL
        assert _close(second, ref) < TOL
    assert L <= _lib.NOALLOC_MAX_L


def test_noalloc_rejects_grids_beyond_its_scratch(cuda_lib):
    import torch
    from dadi_gb300 import _lib
    L = _lib.NOALLOC_MAX_L + 1
    d = torch.zeros(L * L, dtype=torch.float64, device="cuda")
    x = torch.linspace(0, 1, L, dtype=torch.float64, device="cuda")
    t = torch.zeros(11, dtype=torch.float64, device="cuda")
    rc = cuda_lib.dgb_integrate2d_noalloc(_lib.dptr(d), L, _lib.dptr(x), _lib.dptr(t), 1, 0, 0, 0,
                                          _lib.stream_handle(torch))
    assert rc == _lib.DGB_ERR_TOO_LARGE
    assert "DGB_NOALLOC_MAX_L" in _lib.status_string(rc)
