"""Device spectrum epilogue for 2-D integrations: from_phi, extrapolation and
the Poisson (and multinomial) log-likelihoods for many densities in two
launches (dgb_from_phi2d, dgb_extrap_ll).

Each spectrum is computed by one CTA from its own density alone, so a
request's result does not depend on what else shares the launch.  The
incomplete-beta weight tables (dadi/Spectrum_mod.py:25-40) are evaluated on
the host with scipy, as the reference does, and kept on the device per
(sample size, grid).
"""
import numpy as np

from . import _lib, spectrum

FS_ITEM = np.dtype([("phi", "u8"), ("xx", "u8"), ("d1x", "u8"), ("d2x", "u8"), ("d1y", "u8"),
                    ("d2y", "u8"), ("out", "u8"), ("L", "i4"), ("n1", "i4"), ("n2", "i4"),
                    ("pad", "i4")])
EX_ITEM = np.dtype([("fs", "u8", 3), ("x", "f8", 3), ("out", "u8"), ("data", "u8"),
                    ("ll", "u8"), ("llm", "u8"), ("scale", "f8"), ("ngrids", "i4"),
                    ("size", "i4"), ("mask_corners", "i4"), ("pad", "i4")])


def spectra_2d(torch, jobs, fail_mag=10.0):
    """jobs: list of (phis, xxs, ns, data, scale) per spectrum, where phis
    are contiguous (L, L) float64 CUDA tensors (one per grid, 1-3 grids),
    xxs their host grids, ns = (n1, n2), data a (n1+1, n2+1) CUDA tensor or
    None.  Returns (fs list of CUDA tensors (n1+1, n2+1), ll CUDA tensor
    (njobs,), NaN where no data, flat: every fs back to back), all enqueued
    on the current stream."""
    lib = _lib.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    sizes = [(n[0] + 1) * (n[1] + 1) for (_, _, n, _, _) in jobs]
    ngr = sum(len(j[0]) for j in jobs)
    raw = torch.empty(max(sum(len(j[0]) * s for j, s in zip(jobs, sizes)), 1),
                      dtype=torch.float64, device=dev)
    out = torch.empty(max(sum(sizes), 1), dtype=torch.float64, device=dev)
    ll = torch.full((len(jobs),), float("nan"), dtype=torch.float64, device=dev)
    fs_items = np.zeros(ngr, dtype=FS_ITEM)
    ex_items = np.zeros(len(jobs), dtype=EX_ITEM)
    raw_p, out_p, ll_p = raw.data_ptr(), out.data_ptr(), ll.data_ptr()
    ro = oo = g = 0
    Lmax = nmax = 2
    for k, (phis, xxs, ns, data, scale) in enumerate(jobs):
        n1, n2 = ns
        ex = ex_items[k]
        for q, (phi, xx) in enumerate(zip(phis, xxs)):
            L = len(xx)
            assert phi.is_contiguous() and phi.numel() == L * L
            d1x, d2x, dxx = spectrum._device_tables(torch, n1, xx, dev)
            d1y, d2y, _ = spectrum._device_tables(torch, n2, xx, dev)
            it = fs_items[g]
            it["phi"], it["xx"] = phi.data_ptr(), dxx.data_ptr()
            it["d1x"], it["d2x"] = d1x.data_ptr(), d2x.data_ptr()
            it["d1y"], it["d2y"] = d1y.data_ptr(), d2y.data_ptr()
            it["out"] = raw_p + 8 * ro
            it["L"], it["n1"], it["n2"] = L, n1, n2
            ex["fs"][q] = raw_p + 8 * ro
            ex["x"][q] = xx[1]
            ro += sizes[k]
            g += 1
            Lmax, nmax = max(Lmax, L), max(nmax, n1, n2)
        ex["ngrids"] = len(phis)
        ex["size"] = sizes[k]
        ex["out"] = out_p + 8 * oo
        ex["mask_corners"] = 1
        if data is not None:
            ex["data"] = data.data_ptr()
            ex["ll"] = ll_p + 8 * k
            ex["scale"] = scale
        oo += sizes[k]
    d_fs = _lib.to_device(torch, fs_items.view(np.uint8), np.uint8)
    d_ex = _lib.to_device(torch, ex_items.view(np.uint8), np.uint8)
    sh = _lib.stream_handle(torch)
    _lib.check(lib.dgb_from_phi2d(_lib.dptr(d_fs), ngr, Lmax, nmax, sh), "dgb_from_phi2d")
    _lib.check(lib.dgb_extrap_ll(_lib.dptr(d_ex), len(jobs), float(fail_mag), sh),
               "dgb_extrap_ll")
    fs, o = [], 0
    for (_, _, ns, _, _), s in zip(jobs, sizes):
        fs.append(out[o:o + s].view(ns[0] + 1, ns[1] + 1))
        o += s
    return fs, ll, out


def spectra_2d_batch(torch, phis, xxs, ns, data=None, scale=1.0, fail_mag=10.0,
                     multinom=False):
    """A batch sharing grids and sample sizes: phis[g] is an (n, L_g, L_g)
    contiguous CUDA tensor per grid.  Returns (fs (n, n1+1, n2+1), ll (n,)
    or None), enqueued on the current stream; with multinom (and data),
    (fs, ll, ll_multinom): the multinomial log-likelihoods (n,) from the
    same launch (dadi/Inference.py:559-575)."""
    lib = _lib.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    n = int(phis[0].shape[0])
    ng = len(phis)
    n1, n2 = ns
    size = (n1 + 1) * (n2 + 1)
    raw = torch.empty(ng * n * size, dtype=torch.float64, device=dev)
    out = torch.empty(n * size, dtype=torch.float64, device=dev)
    ll = torch.empty(n, dtype=torch.float64, device=dev) if data is not None else None
    llm = torch.empty(n, dtype=torch.float64, device=dev) \
        if (data is not None and multinom) else None
    fs_items = np.zeros((ng, n), dtype=FS_ITEM)
    ex_items = np.zeros(n, dtype=EX_ITEM)
    idx = np.arange(n, dtype=np.uint64)
    Lmax = 2
    for q, (phi, xx) in enumerate(zip(phis, xxs)):
        L = len(xx)
        assert phi.is_contiguous() and tuple(phi.shape) == (n, L, L)
        d1x, d2x, dxx = spectrum._device_tables(torch, n1, xx, dev)
        d1y, d2y, _ = spectrum._device_tables(torch, n2, xx, dev)
        it = fs_items[q]
        it["phi"] = np.uint64(phi.data_ptr()) + idx * np.uint64(8 * L * L)
        it["xx"], it["d1x"], it["d2x"] = dxx.data_ptr(), d1x.data_ptr(), d2x.data_ptr()
        it["d1y"], it["d2y"] = d1y.data_ptr(), d2y.data_ptr()
        it["out"] = np.uint64(raw.data_ptr() + 8 * q * n * size) + idx * np.uint64(8 * size)
        it["L"], it["n1"], it["n2"] = L, n1, n2
        ex_items["fs"][:, q] = it["out"]
        ex_items["x"][:, q] = xx[1]
        Lmax = max(Lmax, L)
    ex_items["out"] = np.uint64(out.data_ptr()) + idx * np.uint64(8 * size)
    ex_items["ngrids"], ex_items["size"], ex_items["mask_corners"] = ng, size, 1
    if data is not None:
        ex_items["data"] = data.data_ptr()
        ex_items["ll"] = np.uint64(ll.data_ptr()) + idx * np.uint64(8)
        ex_items["scale"] = scale
        if llm is not None:
            ex_items["llm"] = np.uint64(llm.data_ptr()) + idx * np.uint64(8)
    d_fs = _lib.to_device(torch, fs_items.reshape(-1).view(np.uint8), np.uint8)
    d_ex = _lib.to_device(torch, ex_items.view(np.uint8), np.uint8)
    sh = _lib.stream_handle(torch)
    _lib.check(lib.dgb_from_phi2d(_lib.dptr(d_fs), ng * n, Lmax, max(n1, n2), sh),
               "dgb_from_phi2d")
    _lib.check(lib.dgb_extrap_ll(_lib.dptr(d_ex), n, float(fail_mag), sh), "dgb_extrap_ll")
    if multinom:
        return out.view(n, n1 + 1, n2 + 1), ll, llm
    return out.view(n, n1 + 1, n2 + 1), ll


def extrapolate_batch(torch, raws, x_l, data=None, scale=1.0, fail_mag=10.0, multinom=False):
    """Extrapolation (with the fail_mag guard) and likelihoods of n spectra of
    any dimension given on 1-3 grids: raws[g] is an (n, ...) contiguous CUDA
    tensor of raw spectra on grid g, x_l the grids' extrap_x (xx[1]).  One
    dgb_extrap_ll launch; the first and last entries are the masked corners
    (dadi/Spectrum_mod.py:178-182).  Returns (fs (n, ...), ll (n,) or None)
    and, with multinom, the multinomial likelihoods third."""
    lib = _lib.lib()
    dev = raws[0].device
    n = int(raws[0].shape[0])
    shape = tuple(raws[0].shape[1:])
    size = int(np.prod(shape))
    out = torch.empty((n,) + shape, dtype=torch.float64, device=dev)
    ll = torch.empty(n, dtype=torch.float64, device=dev) if data is not None else None
    llm = torch.empty(n, dtype=torch.float64, device=dev) \
        if (data is not None and multinom) else None
    ex = np.zeros(n, dtype=EX_ITEM)
    idx = np.arange(n, dtype=np.uint64)
    for q, (r, x) in enumerate(zip(raws, x_l)):
        assert r.is_contiguous() and tuple(r.shape) == (n,) + shape
        ex["fs"][:, q] = np.uint64(r.data_ptr()) + idx * np.uint64(8 * size)
        ex["x"][:, q] = x
    ex["out"] = np.uint64(out.data_ptr()) + idx * np.uint64(8 * size)
    ex["ngrids"], ex["size"], ex["mask_corners"] = len(raws), size, 1
    if data is not None:
        d = data if torch.is_tensor(data) else _lib.to_device(torch, data)
        d = d.to(torch.float64).contiguous()
        assert d.numel() == size
        ex["data"] = d.data_ptr()
        ex["ll"] = np.uint64(ll.data_ptr()) + idx * np.uint64(8)
        ex["scale"] = scale
        if llm is not None:
            ex["llm"] = np.uint64(llm.data_ptr()) + idx * np.uint64(8)
        keep = d
    d_ex = _lib.to_device(torch, ex.view(np.uint8), np.uint8)
    _lib.check(lib.dgb_extrap_ll(_lib.dptr(d_ex), n, float(fail_mag),
                                 _lib.stream_handle(torch)), "dgb_extrap_ll")
    if data is not None:
        del keep
    if multinom:
        return out, ll, llm
    return out, ll
