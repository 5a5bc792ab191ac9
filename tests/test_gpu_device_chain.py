"""Multi-epoch models with the density kept on the device: the drop-in
integrators and the split functions accept CUDA tensors and return CUDA
tensors, so a model chains epochs and splits without copying the density to
the host; the results equal the host-array path (bitwise for densities, the
spectrum bar for spectra)."""
import numpy as np
import pytest

from util import assert_fs_parity

pytestmark = pytest.mark.gpu


def _model(phi1d, xx, dev):
    from dadi_gb300 import integration as gi, phimanip as pm
    T2 = 0.05
    p2 = pm.phi_1D_to_2D(xx, phi1d)
    p2 = gi.two_pops(p2, xx, 0.1, nu1=2.0, nu2=0.5, m12=1.0, m21=0.5)
    p2 = gi.two_pops(p2, xx, T2, nu1=lambda t: 2.0 * (3.0 / 2.0) ** (t / T2),
                     nu2=lambda t: 0.5 * (0.2 / 0.5) ** (t / T2), m12=0.3, m21=0.8,
                     gamma1=-1.0)
    p3 = pm.phi_2D_to_3D_split_2(xx, p2)
    p3 = gi.three_pops(p3, xx, 0.03, nu1=1.0, nu2=0.4, nu3=1.5, m12=0.5, m21=0.5, m13=0.2,
                       m31=0.2, m23=1.0, m32=1.0)
    p4 = pm.phi_3D_to_4D(p3, 0.3, 0.2, xx, xx, xx, xx)
    p4 = gi.four_pops(p4, xx, 0.01, nu1=1.0, nu2=0.5, nu3=1.0, nu4=2.0, m14=0.5, m41=0.5)
    return p2, p3, p4


def test_device_chain_equals_host(cuda_lib, monkeypatch):
    import torch
    from dadi_gb300 import _lib, numerics, phimanip, spectrum
    xx = numerics.default_grid(16)
    phi1d = phimanip.phi_1D(xx)
    host = _model(phi1d, xx, False)
    dev = _model(torch.from_numpy(phi1d).cuda(), xx, True)
    for h, d in zip(host, dev):
        assert torch.is_tensor(d) and d.is_cuda
        assert np.array_equal(d.cpu().numpy(), h)
    # spectra of device densities: 2-D through the device epilogue, 3-D and
    # 4-D through the contraction kernel; only spectra come back to the host
    copied = []
    real_to_host = _lib.to_host
    monkeypatch.setattr(_lib, "to_host", lambda t, x: copied.append(tuple(x.shape)) or
                        real_to_host(t, x))
    monkeypatch.setattr(torch.Tensor, "cpu", lambda *a, **k: pytest.fail("density copied"))
    spectra = []
    for d, ns in zip(dev, [(8, 8), (6, 6, 6), (3, 3, 3, 3)]):
        spectra.append(spectrum.from_phi(d, ns, (xx,) * len(ns)))
    monkeypatch.undo()
    assert all(np.prod(s) <= 9 ** 3 for s in copied), copied
    for h, fd, ns in zip(host, spectra, [(8, 8), (6, 6, 6), (3, 3, 3, 3)]):
        fh = spectrum.from_phi(h, ns, (xx,) * len(ns))
        assert fd.extrap_x == xx[1] and fd.mask.flat[0] and fd.mask.flat[-1]
        assert_fs_parity(np.asarray(fd.data), np.asarray(fh.data))
