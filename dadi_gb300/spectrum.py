"""Sample frequency spectra from phi: the piecewise-linear binomial-sampling
contraction of dadi's Spectrum.from_phi (dadi/Spectrum_mod.py:25-40,
1307-1345, 1509-1547, 1774-1810, 1841-1870, 1938-2061).

`Spectrum` is a numpy masked array with dadi's corner masking and the
`extrap_x` attribute used by extrapolation.  `dbeta_tables` are the
incomplete-beta weight tables; `from_phi_2D_batch` applies them on the GPU to
a whole batch of 2-D densities as two FP64 matrix products per axis.
"""
import numpy as np
from scipy.special import betainc


class Spectrum(np.ma.MaskedArray):
    """Masked frequency spectrum with dadi's 'absent'/'fixed' corners masked
    (dadi/Spectrum_mod.py:178-182) and an extrap_x attribute."""

    def __new__(cls, data, mask=np.ma.nomask, mask_corners=True, extrap_x=None, pop_ids=None):
        obj = np.ma.MaskedArray.__new__(cls, np.asarray(data, dtype=np.float64), mask=mask,
                                        keep_mask=True, shrink=False)
        if obj.mask is np.ma.nomask or np.ndim(obj.mask) == 0:
            obj.mask = np.zeros(obj.shape, dtype=bool)
        if mask_corners:
            obj.mask.flat[0] = obj.mask.flat[-1] = True
        obj.extrap_x = extrap_x
        obj.pop_ids = pop_ids
        return obj

    def __array_finalize__(self, obj):
        super().__array_finalize__(obj)
        self.extrap_x = getattr(obj, "extrap_x", None)
        self.pop_ids = getattr(obj, "pop_ids", None)

    def marginalize(self, over, mask_corners=True):
        """Spectrum of the populations not in `over`, summing over those
        (dadi/Spectrum_mod.py:444-490; masked entries are left out of the
        sums, as the masked-array sum does)."""
        out = np.ma.MaskedArray(self.data, mask=self.mask)
        for axis in sorted(over)[::-1]:
            out = out.sum(axis=axis)
        pop_ids = None
        if self.pop_ids is not None:
            pop_ids = [p for k, p in enumerate(self.pop_ids) if k not in over]
        return Spectrum(np.ma.getdata(out), mask=np.ma.getmaskarray(out),
                        mask_corners=mask_corners, extrap_x=self.extrap_x, pop_ids=pop_ids)


_dbeta_cache = {}


def dbeta_tables(n, xx):
    """dbeta1[i, k] = I(x_{k+1}; i+1, n-i+1) - I(x_k; i+1, n-i+1) and dbeta2
    likewise with i+2 (dadi/Spectrum_mod.py:25-40)."""
    key = n, tuple(xx)
    if key not in _dbeta_cache:
        x = np.minimum(np.maximum(xx, 0), 1.0)
        d1 = np.empty((n + 1, len(x) - 1))
        d2 = np.empty((n + 1, len(x) - 1))
        for i in range(n + 1):
            b = betainc(i + 1, n - i + 1, x)
            d1[i] = b[1:] - b[:-1]
            b = betainc(i + 2, n - i + 1, x)
            d2[i] = b[1:] - b[:-1]
        _dbeta_cache[key] = d1, d2
    return _dbeta_cache[key]


def _from_phi_1D(n, xx, phi):
    data = np.zeros(n + 1)
    xx = np.minimum(np.maximum(xx, 0), 1.0)
    s = (phi[1:] - phi[:-1]) / (xx[1:] - xx[:-1])
    c1 = (phi[:-1] - s * xx[:-1]) / (n + 1)
    for d in range(n + 1):
        c2 = s * (d + 1) / ((n + 1) * (n + 2))
        b1 = betainc(d + 1, n - d + 1, xx)
        b2 = betainc(d + 2, n - d + 1, xx)
        data[d] = np.sum(c1 * (b1[1:] - b1[:-1]) + c2 * (b2[1:] - b2[:-1]))
    return data


def _from_phi_2D(nx, ny, xx, yy, phi):
    d1x, d2x = dbeta_tables(nx, xx)
    d1y, d2y = dbeta_tables(ny, yy)
    s_yy = (phi[:, 1:] - phi[:, :-1]) / (yy[None, 1:] - yy[None, :-1])
    c1_yy = (phi[:, :-1] - s_yy * yy[None, :-1]) / (ny + 1)
    t1 = np.dot(d1y, c1_yy.T)
    t2 = np.dot(d2y, s_yy.T)
    t2 *= np.arange(1, ny + 2)[:, None] / ((ny + 1) * (ny + 2))
    over_y = t1 + t2
    s_xx = (over_y[:, 1:] - over_y[:, :-1]) / (xx[1:] - xx[:-1])
    c1_xx = (over_y[:, :-1] - s_xx * xx[:-1]) / (nx + 1)
    t1 = np.dot(d1x, c1_xx.T)
    t2 = np.dot(d2x, s_xx.T)
    t2 *= np.arange(1, nx + 2)[:, None] / ((nx + 1) * (nx + 2))
    return t1 + t2


def _from_phi_3D(nx, ny, nz, xx, yy, zz, phi):
    data = np.zeros((nx + 1, ny + 1, nz + 1))
    d1z, d2z = dbeta_tables(nz, zz)
    s_zz = (phi[:, :, 1:] - phi[:, :, :-1]) / (zz[None, None, 1:] - zz[None, None, :-1])
    c1_zz = (phi[:, :, :-1] - s_zz * zz[None, None, :-1]) / (nz + 1)
    for kk in range(nz + 1):
        t1 = np.dot(c1_zz, d1z[kk])
        t2 = np.dot(s_zz, d2z[kk])
        t2 *= (kk + 1) / ((nz + 1) * (nz + 2))
        data[:, :, kk] = _from_phi_2D(nx, ny, xx, yy, t1 + t2)
    return data


def _from_phi_4D(nx, ny, nz, na, xx, yy, zz, aa, phi):
    data = np.zeros((nx + 1, ny + 1, nz + 1, na + 1))
    d1a, d2a = dbeta_tables(na, aa)
    s_aa = (phi[:, :, :, 1:] - phi[:, :, :, :-1]) / (aa[1:] - aa[:-1])
    c1_aa = (phi[:, :, :, :-1] - s_aa * aa[:-1]) / (na + 1)
    for ll in range(na + 1):
        t1 = np.dot(c1_aa, d1a[ll])
        t2 = np.dot(s_aa, d2a[ll])
        t2 *= (ll + 1) / ((na + 1) * (na + 2))
        data[:, :, :, ll] = _from_phi_3D(nx, ny, nz, xx, yy, zz, t1 + t2)
    return data


def _from_phi_5D(nx, ny, nz, na, nb, xx, yy, zz, aa, bb, phi):
    data = np.zeros((nx + 1, ny + 1, nz + 1, na + 1, nb + 1))
    d1b, d2b = dbeta_tables(nb, bb)
    s_bb = (phi[..., 1:] - phi[..., :-1]) / (bb[1:] - bb[:-1])
    c1_bb = (phi[..., :-1] - s_bb * bb[:-1]) / (nb + 1)
    for mm in range(nb + 1):
        t1 = np.dot(c1_bb, d1b[mm])
        t2 = np.dot(s_bb, d2b[mm])
        t2 *= (mm + 1) / ((nb + 1) * (nb + 2))
        data[..., mm] = _from_phi_4D(nx, ny, nz, na, xx, yy, zz, aa, t1 + t2)
    return data


def from_phi_nd_batch(torch, phi_b, ns, xx):
    """Raw spectra of a batch of densities phi_b (B, L, ..., L) of 1-5
    populations resident on the GPU, all axes on grid xx: the hand-written
    contraction kernel (dgb_from_phi_nd), one launch per axis.  Returns a
    (B, n1+1, ..., nP+1) float64 CUDA tensor."""
    import ctypes
    from . import _lib
    lib = _lib.lib()
    B, P = phi_b.shape[0], phi_b.dim() - 1
    L = phi_b.shape[1]
    if any(s != L for s in phi_b.shape[1:]) or len(xx) != L or len(ns) != P:
        raise ValueError("phi_b must be (B, L, ..., L) with len(xx) == L and len(ns) axes")
    phi_b = phi_b.to(torch.float64).contiguous()
    dev = phi_b.device
    tabs = [_device_tables(torch, int(n), xx, dev) for n in ns]
    x = tabs[0][2]
    out = torch.empty((B,) + tuple(int(n) + 1 for n in ns), dtype=torch.float64, device=dev)
    if B == 0:
        return out
    ns_c = (ctypes.c_int * P)(*[int(n) for n in ns])
    d1 = (ctypes.c_void_p * P)(*[t[0].data_ptr() for t in tabs])
    d2 = (ctypes.c_void_p * P)(*[t[1].data_ptr() for t in tabs])
    nws = lib.dgb_from_phi_nd_workspace_bytes(P, L, ctypes.cast(ns_c, ctypes.c_void_p), B)
    ws, nws = _lib.workspace(torch, nws)
    _lib.check(lib.dgb_from_phi_nd(_lib.dptr(phi_b), B, P, L, _lib.dptr(x),
                                   ctypes.cast(ns_c, ctypes.c_void_p),
                                   ctypes.cast(d1, ctypes.c_void_p),
                                   ctypes.cast(d2, ctypes.c_void_p), _lib.dptr(out),
                                   _lib.dptr(ws), nws, _lib.stream_handle(torch)),
               "dgb_from_phi_nd")
    return out


def _from_phi_device(phi, ns, xxs):
    """Raw spectrum of a CUDA-tensor density on one grid for every axis:
    two populations through the device epilogue, three to five through the
    contraction kernel; the spectrum (not the density) comes back to the
    host."""
    import torch
    from . import _lib
    P = phi.dim()
    same = all(np.array_equal(xxs[0], x) for x in xxs[1:])
    if not same:
        return None
    if P == 2:
        from . import epilogue
        fs, _, _ = epilogue.spectra_2d(torch, [([phi.to(torch.float64).contiguous()],
                                                [np.asarray(xxs[0], dtype=np.float64)],
                                                tuple(ns), None, 1.0)])
        return _lib.to_host(torch, fs[0])
    fs = from_phi_nd_batch(torch, phi[None], ns, np.asarray(xxs[0], dtype=np.float64))
    return _lib.to_host(torch, fs[0])


def from_phi(phi, ns, xxs, mask_corners=True, pop_ids=None):
    """Spectrum of sample sizes ns from phi on grids xxs (1-5 populations,
    the linear-algebra paths of dadi/Spectrum_mod.py:1938-2061).  phi may be
    a CUDA tensor (a density kept on the device): its spectrum is then
    computed there (all axes on one grid, as dadi's models use) and only the
    spectrum is copied back."""
    if hasattr(phi, "is_cuda") and phi.is_cuda:
        if not phi.dim() == len(ns) == len(xxs):
            raise ValueError('Dimensionality of phi and lengths of ns and xxs do not all '
                             'agree.')
        data = _from_phi_device(phi, ns, xxs)
        if data is not None:
            return Spectrum(data, mask_corners=mask_corners, extrap_x=xxs[0][1],
                            pop_ids=pop_ids)
        phi = phi.detach().cpu().numpy()
    phi = np.asarray(phi)
    if not phi.ndim == len(ns) == len(xxs):
        raise ValueError('Dimensionality of phi and lengths of ns and xxs do not all agree.')
    P = phi.ndim
    if P == 1:
        data = _from_phi_1D(ns[0], xxs[0], phi)
    elif P == 2:
        data = _from_phi_2D(ns[0], ns[1], xxs[0], xxs[1], phi)
    elif P == 3:
        data = _from_phi_3D(*ns, *xxs, phi)
    elif P == 4:
        data = _from_phi_4D(*ns, *xxs, phi)
    elif P == 5:
        data = _from_phi_5D(*ns, *xxs, phi)
    else:
        raise ValueError('Only implemented for dimensions 1-5.')
    return Spectrum(data, mask_corners=mask_corners, extrap_x=xxs[0][1], pop_ids=pop_ids)


_device_cache = {}


def _device_tables(torch, n, xx, dev):
    """(dbeta1, dbeta2, xx) as device tensors, uploaded once per (n, grid,
    device) and kept: later calls enqueue no host-to-device copy, so they
    never wait for work already queued on their stream."""
    from . import _lib
    dev = torch.device(dev)
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    key = (n, np.asarray(xx, dtype=np.float64).tobytes(), dev.index)
    hit = _device_cache.get(key)
    if hit is None:
        d1, d2 = dbeta_tables(n, xx)
        with torch.cuda.device(dev):
            hit = tuple(_lib.upload_resident(torch, t) for t in (d1, d2, xx))
        _device_cache[key] = hit
    return hit


def from_phi_2D_batch(torch, phi_b, n1, n2, xx):
    """Raw 2-D spectra of a batch of densities phi_b (B, L, L) resident on
    the GPU: the same contraction as _from_phi_2D, batched as FP64 GEMMs.
    Returns a (B, n1+1, n2+1) float64 CUDA tensor."""
    dev = phi_b.device
    d1x, d2x, x = _device_tables(torch, n1, xx, dev)
    d1y, d2y, _ = _device_tables(torch, n2, xx, dev)
    dxv = x[1:] - x[:-1]
    s_y = (phi_b[:, :, 1:] - phi_b[:, :, :-1]) / dxv
    c1_y = (phi_b[:, :, :-1] - s_y * x[:-1]) / (n2 + 1)
    wy = torch.arange(1, n2 + 2, dtype=torch.float64, device=dev)[:, None] / ((n2 + 1) * (n2 + 2))
    over_y = torch.matmul(d1y, c1_y.transpose(1, 2)) + wy * torch.matmul(d2y, s_y.transpose(1, 2))
    s_x = (over_y[:, :, 1:] - over_y[:, :, :-1]) / dxv
    c1_x = (over_y[:, :, :-1] - s_x * x[:-1]) / (n1 + 1)
    wx = torch.arange(1, n1 + 2, dtype=torch.float64, device=dev)[:, None] / ((n1 + 1) * (n1 + 2))
    return torch.matmul(d1x, c1_x.transpose(1, 2)) + wx * torch.matmul(d2x, s_x.transpose(1, 2))
