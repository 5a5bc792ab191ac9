"""The private driver functions dadi's Integration module calls when CUDA is
enabled, with the reference signatures of dadi/cuda/Integration.py:89-994.

Each function evaluates the parameter callables on the host exactly as the
reference loop does (dadi/cuda/Integration.py:163-291, 376-545, 547-750),
runs the whole time loop in one call of the C ABI and returns a new host
array.  Differences from the reference backend: the delj trick is supported
instead of raising (dadi/cuda/Integration.py:171-172), and the 2-D driver
validates parameters like the CPU loop (dadi/Integration.py:369-374).
"""
import sys

import numpy as np

from .. import integration as _core


def _append_demes(record):
    demes = sys.modules.get("dadi.Demes")
    if demes is not None:
        demes.cache.append(record)


def _nonconst(hist, deme_ids):
    demes = sys.modules.get("dadi.Demes")
    if demes is not None:
        _append_demes(demes.IntegrationNonConst(history=hist, deme_ids=deme_ids))


def _masks(flags):
    return sum(1 << k for k, f in enumerate(flags) if f)


def _temporal(P, phi, xx, T, initial_t, nu_f, mig_f, gamma_f, h_f, theta0_f, frozen, nomut,
              deme_ids, beta_f=None):
    table, hist = _core.build_table(P, xx, T, initial_t, nu_f, mig_f, gamma_f, h_f, theta0_f,
                                    beta_f=beta_f)
    out = _core.run_table(phi, xx, table, _masks(frozen), _masks(nomut))
    _nonconst(hist, deme_ids)
    return out


def _one_pop_temporal_params(phi, xx, T, initial_t, nu_f, gamma_f, h_f, theta0_f, beta_f,
                             deme_ids=None):
    """GPU counterpart of the one_pop loop (dadi/Integration.py:224-257); the
    reference has no CUDA branch for one population, see install()."""
    return _temporal(1, phi, xx, T, initial_t, [nu_f], [[None]], [gamma_f], [h_f], theta0_f,
                     [False], [False], deme_ids, beta_f=beta_f)


def _two_pops_temporal_params(phi, xx, T, initial_t, nu1_f, nu2_f, m12_f, m21_f, gamma1_f,
                              gamma2_f, h1_f, h2_f, theta0_f, frozen1, frozen2, nomut1, nomut2,
                              deme_ids):
    """dadi/cuda/Integration.py:163-291."""
    return _temporal(2, phi, xx, T, initial_t, [nu1_f, nu2_f], [[None, m12_f], [m21_f, None]],
                     [gamma1_f, gamma2_f], [h1_f, h2_f], theta0_f, [frozen1, frozen2],
                     [nomut1, nomut2], deme_ids)


def _three_pops_temporal_params(phi, xx, T, initial_t, nu1_f, nu2_f, nu3_f, m12_f, m13_f,
                                m21_f, m23_f, m31_f, m32_f, gamma1_f, gamma2_f, gamma3_f, h1_f,
                                h2_f, h3_f, theta0_f, frozen1, frozen2, frozen3, deme_ids):
    """dadi/cuda/Integration.py:376-545."""
    mig_f = [[None, m12_f, m13_f], [m21_f, None, m23_f], [m31_f, m32_f, None]]
    return _temporal(3, phi, xx, T, initial_t, [nu1_f, nu2_f, nu3_f], mig_f,
                     [gamma1_f, gamma2_f, gamma3_f], [h1_f, h2_f, h3_f], theta0_f,
                     [frozen1, frozen2, frozen3], [False] * 3, deme_ids)


def _four_pops_temporal_params(phi, xx, T, initial_t, nu1_f, nu2_f, nu3_f, nu4_f, m12_f, m13_f,
                               m14_f, m21_f, m23_f, m24_f, m31_f, m32_f, m34_f, m41_f, m42_f,
                               m43_f, gamma1_f, gamma2_f, gamma3_f, gamma4_f, h1_f, h2_f, h3_f,
                               h4_f, theta0_f, frozen1, frozen2, frozen3, frozen4, deme_ids):
    """dadi/cuda/Integration.py:547-750."""
    mig_f = [[None, m12_f, m13_f, m14_f], [m21_f, None, m23_f, m24_f],
             [m31_f, m32_f, None, m34_f], [m41_f, m42_f, m43_f, None]]
    return _temporal(4, phi, xx, T, initial_t, [nu1_f, nu2_f, nu3_f, nu4_f], mig_f,
                     [gamma1_f, gamma2_f, gamma3_f, gamma4_f], [h1_f, h2_f, h3_f, h4_f],
                     theta0_f, [frozen1, frozen2, frozen3, frozen4], [False] * 4, deme_ids)


def _five_pops_temporal_params(phi, xx, T, initial_t, nu1_f, nu2_f, nu3_f, nu4_f, nu5_f,
                               m12_f, m13_f, m14_f, m15_f, m21_f, m23_f, m24_f, m25_f, m31_f,
                               m32_f, m34_f, m35_f, m41_f, m42_f, m43_f, m45_f, m51_f, m52_f,
                               m53_f, m54_f, gamma1_f, gamma2_f, gamma3_f, gamma4_f, gamma5_f,
                               h1_f, h2_f, h3_f, h4_f, h5_f, theta0_f, frozen1, frozen2,
                               frozen3, frozen4, frozen5, deme_ids):
    """dadi/cuda/Integration.py:753-994."""
    mig_f = [[None, m12_f, m13_f, m14_f, m15_f], [m21_f, None, m23_f, m24_f, m25_f],
             [m31_f, m32_f, None, m34_f, m35_f], [m41_f, m42_f, m43_f, None, m45_f],
             [m51_f, m52_f, m53_f, m54_f, None]]
    return _temporal(5, phi, xx, T, initial_t, [nu1_f, nu2_f, nu3_f, nu4_f, nu5_f], mig_f,
                     [gamma1_f, gamma2_f, gamma3_f, gamma4_f, gamma5_f],
                     [h1_f, h2_f, h3_f, h4_f, h5_f], theta0_f,
                     [frozen1, frozen2, frozen3, frozen4, frozen5], [False] * 5, deme_ids)


def _const(phi, xx, theta0, frozen, nomut, abc, current_t, dt, T):
    dts = _core.step_lengths(dt, T, current_t)
    out = _core.run_precalc(phi, xx, abc, dts, theta0, _masks(frozen), _masks(nomut))
    return out.reshape((len(xx),) * len(frozen))


def _two_pops_const_params(phi, xx, theta0, frozen1, frozen2, nomut1, nomut2, ax, bx, cx, ay,
                           by, cy, current_t, dt, T):
    """dadi/cuda/Integration.py:89-161 (a/b/c built by the caller,
    dadi/Integration.py:1055-1095)."""
    return _const(phi, xx, theta0, [frozen1, frozen2], [nomut1, nomut2],
                  [ax, bx, cx, ay, by, cy], current_t, dt, T)


def _three_pops_const_params(phi, xx, theta0, frozen1, frozen2, frozen3, ax, bx, cx, ay, by, cy,
                             az, bz, cz, current_t, dt, T):
    """dadi/cuda/Integration.py:293-374."""
    return _const(phi, xx, theta0, [frozen1, frozen2, frozen3], [False] * 3,
                  [ax, bx, cx, ay, by, cy, az, bz, cz], current_t, dt, T)
