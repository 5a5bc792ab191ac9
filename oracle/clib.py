"""ORACLE -- test infrastructure only.  ctypes bindings for oracle/_build/liboracle.so
(the C restatement in oracle/sweeps.c) and, when built, oracle/_ref/libdadi_ref.so
(the reference C sweeps compiled from their own sources)."""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_dp = ctypes.POINTER(ctypes.c_double)
_lib = None
_ref = None


def build():
    """Compile oracle/sweeps.c (and the reference C if its tree is present)."""
    subprocess.run(["make", "-s", "-C", _HERE, "oracle"], check=True)


def _ptr(a):
    return a.ctypes.data_as(_dp)


def lib():
    """The restatement library, built on first use."""
    global _lib
    if _lib is None:
        path = os.path.join(_HERE, "_build", "liboracle.so")
        if not os.path.exists(path):
            subprocess.run(["make", "-s", "-C", _HERE, "oracle"], check=True)
        L = ctypes.CDLL(path)
        L.orc_sweep.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp,
                                ctypes.c_double, _dp, ctypes.c_double, ctypes.c_double,
                                ctypes.c_double, ctypes.c_double, ctypes.c_int]
        L.orc_sweep.restype = ctypes.c_int
        L.orc_sweep_rhs_variant.argtypes = L.orc_sweep.argtypes
        L.orc_sweep_rhs_variant.restype = ctypes.c_int
        L.orc_sweep_exp_variant.argtypes = L.orc_sweep.argtypes
        L.orc_sweep_exp_variant.restype = ctypes.c_int
        L.orc_sweep_precalc.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        _dp, _dp, _dp, ctypes.c_double]
        L.orc_sweep_precalc.restype = ctypes.c_int
        L.orc_tridiag_solve.argtypes = [_dp, _dp, _dp, _dp, _dp, ctypes.c_int]
        L.orc_tridiag_solve.restype = ctypes.c_int
        L.orc_im_steps.argtypes = [_dp, ctypes.c_long, ctypes.c_double, ctypes.c_long,
                                   ctypes.POINTER(ctypes.c_long)]
        L.orc_im_steps.restype = ctypes.c_int
        _lib = L
    return _lib


def ref_lib():
    """The reference C sweeps compiled from their own sources, or None."""
    global _ref
    if _ref is None:
        path = os.path.join(_HERE, "_ref", "libdadi_ref.so")
        if not os.path.exists(path):
            return None
        _ref = ctypes.CDLL(path)
    return _ref


#: When True, sweep() uses orc_sweep_rhs_variant (noise-floor measurements).
rhs_variant = False
#: When True, sweep() uses orc_sweep_exp_variant (noise floor under the delj
#: trick: another faithfully rounded exp).
exp_variant = False


def sweep(phi, xx, axis, nu, mig, gamma, h, dt, beta=1.0, use_delj_trick=False):
    """In-place implicit sweep of phi along axis (see orc_sweep in sweeps.c)."""
    assert phi.dtype == np.float64 and phi.flags.c_contiguous
    xx = np.ascontiguousarray(xx, dtype=np.float64)
    mig = np.ascontiguousarray(np.broadcast_to(np.asarray(mig, dtype=np.float64),
                                               (phi.ndim,)))
    fn = lib().orc_sweep_rhs_variant if rhs_variant else lib().orc_sweep
    if exp_variant:
        fn = lib().orc_sweep_exp_variant
    rc = fn(_ptr(phi), phi.ndim, phi.shape[0], axis, _ptr(xx),
                         float(nu), _ptr(mig), float(gamma), float(h), float(beta),
                         float(dt), int(bool(use_delj_trick)))
    if rc != 0:
        raise RuntimeError("orc_sweep failed: %d" % rc)
    return phi


def sweep_precalc(phi, axis, a, b, c, dt):
    """In-place constant-coefficient sweep (see orc_sweep_precalc)."""
    arrs = [np.ascontiguousarray(v, dtype=np.float64) for v in (a, b, c)]
    rc = lib().orc_sweep_precalc(_ptr(phi), phi.ndim, phi.shape[0], axis,
                                 _ptr(arrs[0]), _ptr(arrs[1]), _ptr(arrs[2]), float(dt))
    if rc != 0:
        raise RuntimeError("orc_sweep_precalc failed: %d" % rc)
    return phi


def im_steps(params, timescale_factor=1e-3, max_steps=10 ** 8):
    """Steps of the reference two_pops loop of Demographics2D.IM for each row
    (s, nu1, nu2, T, m12, m21) of params (see orc_im_steps in sweeps.c)."""
    p = np.ascontiguousarray(np.asarray(params, dtype=np.float64).reshape(-1, 6))
    out = np.zeros(len(p), dtype=np.int64)
    lib().orc_im_steps(_ptr(p), len(p), float(timescale_factor), int(max_steps),
                       out.ctypes.data_as(ctypes.POINTER(ctypes.c_long)))
    return out


def tridiag(a, b, c, r):
    """Solve one tridiagonal system (dadi/tridiag_cython.pyx:14-18 semantics)."""
    a, b, c, r = [np.ascontiguousarray(v, dtype=np.float64) for v in (a, b, c, r)]
    u = np.empty_like(r)
    lib().orc_tridiag_solve(_ptr(a), _ptr(b), _ptr(c), _ptr(r), _ptr(u), len(r))
    return u
