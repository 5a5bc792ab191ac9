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


def _table_case(L, seed, T, mig=(0.8, 1.7)):
    from dadi_gb300 import integration as gi
    xx = cases.grid("default", L)
    phi0 = cases.initial_phi(seed, (L, L))
    f = gi.ensure_1arg_func
    nu1 = lambda t: 0.4 * (3.0 / 0.4) ** (t / T)
    table, _ = gi.build_table(2, xx, T, 0.0, [f(nu1), f(1.3)],
                              [[None, f(mig[0])], [f(mig[1]), None]], [f(-0.5), f(0.0)],
                              [f(0.3), f(0.5)], f(1.0))
    return xx, phi0, table


def _run(lib, name, L, xx, phi0, table, frozen=0, nomut=0, delj=0):
    import torch
    from dadi_gb300 import _lib
    d_phi = torch.from_numpy(phi0.copy()).cuda()
    d_xx = torch.from_numpy(xx).cuda()
    d_tab = torch.from_numpy(np.ascontiguousarray(table)).cuda()
    sh = _lib.stream_handle(torch)
    if name == "noalloc":
        rc = lib.dgb_integrate2d_noalloc(_lib.dptr(d_phi), L, _lib.dptr(d_xx), _lib.dptr(d_tab),
                                         len(table), frozen, nomut, delj, sh)
    else:
        nws = lib.dgb_workspace_bytes(0, 2, L, 0)
        ws, nws = _lib.workspace(torch, nws)
        rc = lib.dgb_integrate_table(_lib.dptr(d_phi), 2, L, _lib.dptr(d_xx), _lib.dptr(d_tab),
                                     len(table), frozen, nomut, delj, _lib.dptr(ws), nws, sh)
    assert rc == 0, _lib.status_string(rc)
    torch.cuda.synchronize()
    return d_phi.cpu().numpy()


def _close(a, b):
    floor = 1e-12 * np.max(np.abs(b))
    rel = np.abs(a - b) / np.maximum(np.abs(b), floor)
    return float(np.max(rel))


# (L, seed, T, migration, frozen_mask, nomut_mask, use_delj_trick): L = 120
# and the delj case at L = 120 use the static array (their Thomas scratch
# does not fit in shared memory beside the density); the others keep it in
# shared memory
NOALLOC_CASES = [
    (120, 7, 0.05, (0.8, 1.7), 0, 0, 0),
    (64, 8, 0.08, (0.8, 1.7), 0, 0, 0),
    (120, 9, 0.03, (0.8, 1.7), 0, 0, 1),
    (72, 10, 0.04, (0.8, 1.7), 0, 0, 1),
    (100, 11, 0.05, (0.8, 1.7), 0, 2, 0),
    (124, 12, 0.05, (0.0, 0.0), 1, 0, 0),
]


@pytest.mark.parametrize("L,seed,T,mig,frozen,nomut,delj", NOALLOC_CASES)
def test_noalloc_matches_workspace_entry_point_twice(cuda_lib, L, seed, T, mig, frozen, nomut,
                                                     delj):
    from dadi_gb300 import _lib
    assert L <= _lib.NOALLOC_MAX_L
    xx, phi0, table = _table_case(L, seed, T, mig)
    ref = _run(cuda_lib, "table", L, xx, phi0, table, frozen, nomut, delj)
    first = _run(cuda_lib, "noalloc", L, xx, phi0, table, frozen, nomut, delj)
    second = _run(cuda_lib, "noalloc", L, xx, phi0, table, frozen, nomut, delj)
    assert _close(first, ref) < TOL
    assert _close(second, ref) < TOL


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
