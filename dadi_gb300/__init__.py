"""dadi_gb300: dadi's allele-frequency diffusion integrator on GB300 (sm_103a).

Two ways in:

* As dadi's CUDA backend.  With dadi importable, ``dadi_gb300.install()``
  registers ``dadi_gb300.cuda`` as ``dadi.cuda`` (and routes one_pop too);
  then ``dadi.cuda_enabled(True)`` sends dadi's own model code to the GPU.
* Standalone.  ``dadi_gb300.integration`` mirrors dadi.Integration's
  one_pop/two_pops/three_pops/four_pops; ``numerics``, ``phimanip``,
  ``spectrum`` and ``inference`` mirror the host pieces around them; and
  ``batch`` runs thousands of 2-D integrations in one persistent launch.

The kernels live in libdadi_gb300.so (C ABI: include/dadi_gb300.h), built by
``dadi_gb300.build.build()``.  There is no CPU fallback.
"""
import sys

__version__ = "0.1.0"


def install(dadi_module=None):
    """Register this package as ``dadi.cuda`` so that ``dadi.cuda_enabled(True)``
    uses it, and give ``dadi.Integration.one_pop`` a GPU branch while CUDA is
    enabled (the reference has none; this is an extension).  Returns the
    dadi module."""
    if dadi_module is None:
        import dadi as dadi_module
    from . import cuda
    sys.modules["dadi.cuda"] = cuda
    dadi_module.cuda = cuda
    integ = dadi_module.Integration
    if not getattr(integ.one_pop, "_dadi_gb300", False):
        cpu_one_pop = integ.one_pop

        def one_pop(phi, xx, T, nu=1, gamma=0, h=0.5, theta0=1.0, initial_t=0, frozen=False,
                    beta=1, deme_ids=None):
            if not integ.cuda_enabled:
                return cpu_one_pop(phi, xx, T, nu, gamma, h, theta0, initial_t, frozen, beta,
                                   deme_ids)
            import numpy as np
            phi = np.array(phi, dtype=np.float64, copy=True)
            if frozen or T - initial_t == 0:
                return phi
            if T - initial_t < 0:
                raise ValueError('Final integration time T (%f) is less than intial_time (%f). '
                                 'Integration cannot be run backwards.' % (T, initial_t))
            if np.all([np.isscalar(v) for v in (nu, gamma, h, theta0, beta)]):
                # recorded as dadi records it before its constant-parameter
                # loop (dadi/Integration.py:214-216); the GPU then takes the
                # temporal loop, as dadi's two_pops does under CUDA (:318-345)
                demes = dadi_module.Demes
                demes.cache.append(demes.IntegrationConst(duration=T - initial_t,
                                                          start_sizes=[nu], deme_ids=deme_ids))
            f = dadi_module.Misc.ensure_1arg_func
            return cuda.Integration._one_pop_temporal_params(
                phi, xx, T, initial_t, f(nu), f(gamma), f(h), f(theta0), f(beta), deme_ids)
        one_pop._dadi_gb300 = True
        one_pop.__doc__ = cpu_one_pop.__doc__
        integ.one_pop = one_pop
    return dadi_module
