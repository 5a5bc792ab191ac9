"""ctypes binding of libdadi_gb300.so, the C ABI declared in include/dadi_gb300.h.

There is no CPU fallback: importing the package works without a GPU (so the
library and its symbols can be inspected), but every compute call requires
the compiled library and a CUDA device and raises otherwise.
"""
import ctypes
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libdadi_gb300.so")

DGB_OK = 0
DGB_ERR_ARG = -1
DGB_ERR_CUDA = -2
DGB_ERR_UNSUPPORTED = -3
DGB_ERR_WORKSPACE = -4
DGB_ERR_TOO_LARGE = -5
NOALLOC_MAX_L = 128

PF_CONST, PF_EXPGROW, PF_EXPLOG, PF_LINEAR = 0, 1, 2, 3
ST_BADPARAM, ST_STEPCAP, ST_NONFINITE, ST_ZERODT = 1, 2, 4, 8

#: Every entry point the header declares (checked by the test suite).
EXPORTS = ["dgb_abi_version", "dgb_status_string", "dgb_workspace_bytes",
           "dgb_tridiag_batch", "dgb_implicit_sweep", "dgb_implicit_precalc_sweep",
           "dgb_integrate_table", "dgb_integrate_precalc", "dgb_sched2d",
           "dgb_batch2d_integrate", "dgb_batch2d_count_steps", "dgb_probe_fp64_fma",
           "dgb_probe_rcp", "dgb_integrate2d_noalloc", "dgb_sched2d_deriv",
           "dgb_batch2d_integrate_ckpt", "dgb_adjoint2d_scratch_bytes", "dgb_adjoint2d",
           "dgb_items2d_integrate", "dgb_sched2d_host", "dgb_from_phi2d_smem_bytes",
           "dgb_from_phi2d", "dgb_extrap_ll", "dgb_integrate_table_states",
           "dgb_adjoint_table_nd_gpart_doubles", "dgb_adjoint_table_nd",
           "dgb_batchnd_workspace_bytes", "dgb_batchnd_integrate", "dgb_schednd_host",
           "dgb_from_phi_nd_workspace_bytes", "dgb_from_phi_nd", "dgb_adjoint2d_traj_ws_bytes",
           "dgb_adjoint2d_traj", "dgb_schednd_dual_host", "dgb_batchnd_adjoint_workspace_bytes",
           "dgb_batchnd_integrate_states", "dgb_batchnd_adjoint", "dgb_integrate2d_cluster",
           "dgb_items2d_integrate_cluster", "dgb_adjoint2d_part", "dgb_preload",
           "dgb_batch2d_integrate_ckpt_part"]


class PForm(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("pad_", ctypes.c_int),
                ("a", ctypes.c_double), ("b", ctypes.c_double), ("c", ctypes.c_double)]


class Inst2D(ctypes.Structure):
    _fields_ = [("T", ctypes.c_double), ("initial_t", ctypes.c_double),
                ("nu", PForm * 2), ("m12", PForm), ("m21", PForm), ("gamma", PForm * 2),
                ("h", PForm * 2), ("theta0", PForm),
                ("frozen_mask", ctypes.c_int), ("nomut_mask", ctypes.c_int)]


class InstND(ctypes.Structure):
    _fields_ = [("T", ctypes.c_double), ("initial_t", ctypes.c_double),
                ("nu", PForm * 5), ("gamma", PForm * 5), ("h", PForm * 5),
                ("mig", (PForm * 5) * 5), ("theta0", PForm),
                ("ndim", ctypes.c_int), ("pad_", ctypes.c_int)]


#: Model parameters a dgb_seednd can seed (DGB_ND_MAXPAR).
ND_MAXPAR = 16


class SeedND(ctypes.Structure):
    """dgb_seednd: d(a, b, c)/dtheta of every form of a dgb_instnd."""
    _V = ctypes.c_double * ND_MAXPAR
    _fields_ = [("dT", _V), ("dt0", _V), ("dnu", (_V * 3) * 5), ("dgamma", (_V * 3) * 5),
                ("dh", (_V * 3) * 5), ("dmig", ((_V * 3) * 5) * 5), ("dtheta0", _V * 3)]


class ItemND(ctypes.Structure):
    _fields_ = [("phi_off", ctypes.c_long), ("row_off", ctypes.c_long),
                ("nsteps", ctypes.c_int), ("masks", ctypes.c_int)]


class ItemNDAdj(ctypes.Structure):
    _fields_ = [("phi_off", ctypes.c_long), ("row_off", ctypes.c_long),
                ("state_off", ctypes.c_long), ("gpart_off", ctypes.c_long),
                ("nsteps", ctypes.c_int), ("masks", ctypes.c_int)]


class Settings(ctypes.Structure):
    _fields_ = [("timescale_factor", ctypes.c_double), ("old_timescale_factor", ctypes.c_double),
                ("use_old_timestep", ctypes.c_int), ("use_delj_trick", ctypes.c_int),
                ("gam_placement", ctypes.c_int), ("threads", ctypes.c_int),
                ("line_solver", ctypes.c_int), ("segments", ctypes.c_int)]


class DgbError(RuntimeError):
    """A libdadi_gb300 call returned a non-zero status."""

    def __init__(self, status, what):
        self.status = status
        super().__init__("%s failed: %s (status %d)" % (what, status_string(status), status))


_lib = None
_vp = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)


def _declare(L):
    i, d, sz, lg = ctypes.c_int, ctypes.c_double, ctypes.c_size_t, ctypes.c_long
    sig = {
        "dgb_abi_version": (i, []),
        "dgb_preload": (i, []),
        "dgb_status_string": (ctypes.c_char_p, [i]),
        "dgb_workspace_bytes": (sz, [i, i, i, lg]),
        "dgb_tridiag_batch": (i, [_vp, _vp, _vp, _vp, _vp, i, i, _vp, sz, _vp]),
        "dgb_implicit_sweep": (i, [_vp, i, i, i, _vp, d, _dp, d, d, d, d, i, _vp, sz, _vp]),
        "dgb_implicit_precalc_sweep": (i, [_vp, i, i, i, _vp, _vp, _vp, d, _vp, sz, _vp]),
        "dgb_integrate_table": (i, [_vp, i, i, _vp, _vp, i, i, i, i, _vp, sz, _vp]),
        "dgb_integrate_precalc": (i, [_vp, i, i, _vp, _vp, _vp, i, d, i, i, _vp, sz, _vp]),
        "dgb_sched2d": (i, [_vp, i, i, _vp, ctypes.POINTER(Settings), lg, i, _vp, _vp, _vp, _vp,
                            _vp]),
        "dgb_batch2d_integrate": (i, [_vp, i, ctypes.POINTER(ctypes.c_int), i, _vp, _vp, _vp, _vp,
                                      _vp, _vp, _vp, ctypes.POINTER(Settings), _vp, sz, _vp]),
        "dgb_batch2d_count_steps": (i, [ctypes.POINTER(Inst2D), i, ctypes.POINTER(Settings), lg,
                                        ctypes.POINTER(ctypes.c_long)]),
        "dgb_probe_fp64_fma": (i, [_vp, i, i, i, i, _vp]),
        "dgb_probe_rcp": (i, [_vp, _vp, i, _vp]),
        "dgb_integrate2d_noalloc": (i, [_vp, i, _vp, _vp, i, i, i, i, _vp]),
        "dgb_sched2d_deriv": (i, [_vp, _vp, i, i, _vp, ctypes.POINTER(Settings), _vp, _vp, _vp,
                                  _vp]),
        "dgb_batch2d_integrate_ckpt": (i, [_vp, i, ctypes.POINTER(ctypes.c_int), i, _vp, _vp,
                                           _vp, _vp, _vp, _vp, _vp, ctypes.POINTER(Settings),
                                           _vp, _vp, i, _vp, sz, _vp]),
        "dgb_adjoint2d_scratch_bytes": (sz, [i, i, i]),
        "dgb_items2d_integrate": (i, [_vp, i, i, _vp, _vp, _vp, _vp, _vp, _vp,
                                      ctypes.POINTER(Settings), i, _vp, sz, _vp]),
        "dgb_sched2d_host": (i, [_vp, i, ctypes.POINTER(Settings), lg, d, _vp, _vp, _vp, _vp]),
        "dgb_from_phi2d_smem_bytes": (sz, [i, i]),
        "dgb_from_phi2d": (i, [_vp, i, i, i, _vp]),
        "dgb_extrap_ll": (i, [_vp, i, d, _vp]),
        "dgb_integrate_table_states": (i, [_vp, i, i, _vp, _vp, i, i, i, _vp, _vp, sz, _vp]),
        "dgb_adjoint_table_nd_gpart_doubles": (sz, [i, i]),
        "dgb_adjoint_table_nd": (i, [_vp, i, i, _vp, _vp, i, i, i, _vp, _vp, _vp, sz, _vp]),
        "dgb_batchnd_workspace_bytes": (sz, [i, i, i, ctypes.POINTER(Settings)]),
        "dgb_batchnd_integrate": (i, [_vp, _vp, i, i, i, _vp, _vp, _vp,
                                      ctypes.POINTER(Settings), _vp, sz, _vp]),
        "dgb_schednd_host": (i, [_vp, i, ctypes.POINTER(Settings), lg, d, _vp, _vp, _vp, _vp]),
        "dgb_schednd_dual_host": (i, [_vp, _vp, i, ctypes.POINTER(Settings), lg, d, _vp, _vp,
                                      _vp, _vp]),
        "dgb_batchnd_adjoint_workspace_bytes": (sz, [i, i, i, ctypes.POINTER(Settings)]),
        "dgb_integrate2d_cluster": (i, [_vp, i, _vp, _vp, i, i, i, i, _vp]),
        "dgb_items2d_integrate_cluster": (i, [_vp, i, i, i, _vp, _vp, _vp, _vp, _vp, i, _vp,
                                              _vp, i, _vp]),
        "dgb_batch2d_integrate_ckpt_part": (i, [_vp, i, ctypes.POINTER(ctypes.c_int), i, _vp,
                                                _vp, _vp, _vp, _vp, _vp, _vp, i, i,
                                                ctypes.POINTER(Settings), _vp, _vp, i, _vp, sz,
                                                _vp]),
        "dgb_batchnd_integrate_states": (i, [_vp, i, i, i, _vp, _vp, _vp, _vp,
                                             ctypes.POINTER(Settings), _vp, sz, _vp]),
        "dgb_batchnd_adjoint": (i, [_vp, i, i, i, _vp, _vp, _vp, _vp, _vp,
                                    ctypes.POINTER(Settings), _vp, sz, _vp]),
        "dgb_from_phi_nd_workspace_bytes": (sz, [i, i, _vp, i]),
        "dgb_from_phi_nd": (i, [_vp, i, i, i, _vp, _vp, _vp, _vp, _vp, _vp, sz, _vp]),
        "dgb_adjoint2d_traj_ws_bytes": (sz, [i, i]),
        "dgb_adjoint2d_traj": (i, [_vp, i, ctypes.POINTER(ctypes.c_int), i, _vp, _vp, _vp, _vp,
                                   _vp, _vp, _vp, i, _vp, _vp, _vp, _vp, _vp, _vp,
                                   ctypes.POINTER(Settings), _vp, sz, _vp]),
        "dgb_adjoint2d_part": (i, [_vp, i, ctypes.POINTER(ctypes.c_int), i, _vp, _vp, _vp, _vp,
                                   _vp, _vp, _vp, i, _vp, _vp, _vp, _vp, _vp, _vp, i, i, i,
                                   ctypes.POINTER(Settings), _vp, sz, _vp]),
        "dgb_adjoint2d": (i, [_vp, i, ctypes.POINTER(ctypes.c_int), i, _vp, _vp, _vp, _vp, _vp,
                              _vp, _vp, i, _vp, _vp, _vp, ctypes.POINTER(Settings), _vp, sz,
                              _vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libdadi_gb300.so is not built (%s); run "
                              "`python -c 'import __graft_entry__ as g; g.build()'` or "
                              "`python dadi_gb300/build.py`" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def status_string(status):
    try:
        return lib().dgb_status_string(int(status)).decode()
    except ImportError:
        return "status %d" % status


def check(status, what):
    if status != DGB_OK:
        raise DgbError(status, what)


# ---------------------------------------------------------------- devices

_preloaded = set()


def require_cuda():
    """torch with a visible CUDA device, or a RuntimeError (no CPU fallback).
    The first call on a device loads every kernel of the library there
    (dgb_preload), so that no kernel's first launch waits for the device to
    go idle while other streams have work in flight."""
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("dadi_gb300 needs a CUDA device; none is visible")
    L = lib()
    dev = torch.cuda.current_device()
    if dev not in _preloaded:
        check(L.dgb_preload(), "dgb_preload")
        _preloaded.add(dev)
    return torch


def stream_handle(torch):
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def dptr(t):
    """Device pointer of a contiguous torch tensor."""
    assert t.is_contiguous()
    return ctypes.c_void_p(t.data_ptr())


def to_device(torch, arr, dtype=None):
    """Host array -> device tensor, staged through pinned memory and copied
    asynchronously on the current stream.  (A copy from pageable memory is
    synchronous and, in the driver, serialises with every other thread's
    pageable copies, so one thread waiting for its stream would stall the
    others.)"""
    a = np.ascontiguousarray(arr, dtype=dtype if dtype is not None else np.float64)
    return torch.from_numpy(a).pin_memory().to("cuda", non_blocking=True)


def to_host(torch, t):
    """Device tensor -> numpy array: copied into pinned memory on the
    current stream, which alone is then synchronised."""
    out = torch.empty(tuple(t.shape), dtype=t.dtype, pin_memory=True)
    out.copy_(t, non_blocking=True)
    torch.cuda.current_stream().synchronize()
    return out.numpy()


_upload_streams = {}
_upload_lock = threading.Lock()


def upload_resident(torch, arr, dtype=None):
    """Host array -> device tensor that is complete on return and may be
    read from any stream: copied on a private stream that is synchronised
    alone, so the call never waits for work queued on the caller's streams.
    For long-lived constants (grids, tables, initial densities)."""
    a = np.ascontiguousarray(arr, dtype=dtype if dtype is not None else np.float64)
    dev = torch.cuda.current_device()
    with _upload_lock:
        s = _upload_streams.get(dev)
        if s is None:
            s = _upload_streams[dev] = torch.cuda.Stream()
        with torch.cuda.stream(s):
            t = torch.from_numpy(a).pin_memory().to("cuda", non_blocking=True)
        s.synchronize()
    return t


def workspace(torch, nbytes):
    n = max(int(nbytes), 1)
    return torch.empty(n, dtype=torch.uint8, device="cuda"), n


def settings_struct(timescale_factor=1e-3, old_timescale_factor=0.1, use_old_timestep=False,
                    use_delj_trick=False, gam_placement=0, threads=0, line_solver=0,
                    segments=0):
    return Settings(float(timescale_factor), float(old_timescale_factor),
                    int(bool(use_old_timestep)), int(bool(use_delj_trick)), int(gam_placement),
                    int(threads), int(line_solver), int(segments))


def fp64_fma_peak_tflops(torch, active_lanes=32, target_s=0.1, repeats=5):
    """Measured FP64 FMA rate of this GPU in TFLOP/s (2 flops per FMA): 4 and
    8 warps per SM on every SM, 8 independent chains per thread, counting only
    the FMAs of the active lanes; each launch sized to last about target_s,
    the best of `repeats` launches per shape."""
    nsm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    sh = stream_handle(torch)
    best = 0.0
    for threads in (128, 256):
        blocks = nsm
        out = torch.empty(blocks * threads, dtype=torch.float64, device="cuda")

        def timed(iters):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            check(lib().dgb_probe_fp64_fma(dptr(out), blocks, threads, iters, active_lanes, sh),
                  "dgb_probe_fp64_fma")
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) * 1e-3
        timed(16)
        iters = 4096
        t = timed(iters)
        iters = int(min(2 ** 30 // 8, max(iters, iters * target_s / max(t, 1e-6))))
        for _ in range(repeats):
            t = timed(iters)
            fmas = blocks * (threads // 32) * active_lanes * iters * 8
            best = max(best, 2.0 * fmas / t / 1e12)
    return best
