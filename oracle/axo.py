"""ctypes wrapper of the CPU oracle (oracle/_build/libaxo.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
checker, and by bench.py for the CPU baseline / reference arm.  The product
(axion_grav_gb300) never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(_HERE))

from axion_grav_gb300 import Params  # noqa: E402  (shared struct layout only)

_lib = None


def lib():
    global _lib
    if _lib is None:
        sys.path.insert(0, _HERE)
        import build as _b  # oracle/build.py

        path = _b.build()
        _lib = ctypes.CDLL(path)
        L = _lib
        dp = ctypes.POINTER(ctypes.c_double)
        i64p = ctypes.POINTER(ctypes.c_int64)
        P = ctypes.POINTER(Params)
        spec = {
            "axo_msquared": ([ctypes.c_double], ctypes.c_double),
            "axo_maxion2": ([ctypes.c_double, ctypes.c_double], ctypes.c_double),
            "axo_kick_coeffs": ([P, ctypes.c_double, ctypes.c_double, dp, dp], None),
            "axo_get_dtau": ([P, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp, i64p], None),
            "axo_evolve_phi": ([P, dp, dp, dp, dp, ctypes.c_double], None),
            "axo_evolve_phidot": ([P, dp, dp, dp, dp, ctypes.c_double, ctypes.c_double], None),
            "axo_symplectic_integration": ([P, dp, dp, dp, dp, dp, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double], ctypes.c_int64),
            "axo_fft3d": ([ctypes.c_int64, dp, ctypes.c_int], None),
            "axo_data1_to_arr_dphi": ([P, dp, dp], None),
            "axo_data1_to_arr_dphi_degrade": ([P, dp, dp], None),
            "axo_grav_wave_integration": ([P, dp, dp, ctypes.c_double, ctypes.c_double], None),
            "axo_grav_spec_estimation": ([P, dp, dp, dp, dp, dp], None),
            "axo_uij_grav_spec": ([P, dp, dp, ctypes.c_double, dp, dp, dp, dp], None),
            "axo_grav_spec_log_green": ([P, dp, dp, dp, dp, dp], None),
            "axo_uij_grav_spec_log": ([P, dp, dp, ctypes.c_double, dp, dp, dp, dp], None),
            "axo_ic_gaussian_flat": ([P, ctypes.c_double, ctypes.c_uint32, dp, dp], None),
            "axo_ic_thermal": ([P, ctypes.c_double, ctypes.c_uint32, dp, dp], None),
            "axo_field_moments": ([P, dp, dp, ctypes.c_double, dp], None),
            "axo_det_atan2": ([ctypes.c_double, ctypes.c_double], ctypes.c_double),
            "axo_det_sincos": ([ctypes.c_double, dp, dp], None),
            "axo_philox": ([ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32),
                            ctypes.POINTER(ctypes.c_uint32)], None),
            "axo_num_threads": ([], ctypes.c_int),
        }
        optional = {
            "axo_classify_cells": ([P, dp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int8), i64p], None),
            "axo_string_winding": ([P, dp, i64p], None),
            "axo_id_defects": ([P, dp, dp, ctypes.c_double, dp, dp, dp, i64p, dp, ctypes.c_int64, dp,
                                ctypes.c_int64, ctypes.POINTER(ctypes.c_int8)], None),
            "axo_chi2_string_ff": ([dp, dp], ctypes.c_double),
            "axo_chi2_string_fp64": ([dp, dp], ctypes.c_double),
            "axo_fit_cells": ([P, dp, dp, i64p, ctypes.c_int64, dp, i64p, ctypes.c_int64, dp], None),
            "axo_position_string": ([dp, ctypes.c_uint64, ctypes.c_uint64, dp, dp, dp, dp], None),
            "axo_position_wall": ([dp, dp, dp, dp, dp], None),
            "axo_string_length": ([dp, dp], ctypes.c_double),
            "axo_init_spectrum": ([P, dp, dp, dp, dp], None),
            "axo_spectrum_estimation": ([P, dp, ctypes.POINTER(ctypes.c_int8), ctypes.c_double, dp, dp,
                                         dp, dp, dp], None),
            "axo_compute_crho": ([P, dp, dp, dp], None),
            "axo_pp_inverse": ([ctypes.c_int, dp], ctypes.c_int),
            "axo_estimate_covmat": ([P, ctypes.POINTER(ctypes.c_int8), dp, dp, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_double, dp, ctypes.POINTER(ctypes.c_int)], None),
            "axo_compute_crho_cov": ([P, dp, dp, dp, dp, dp], None),
            "axo_epsilon": ([ctypes.c_int, dp, dp, dp, dp, dp, ctypes.c_double, ctypes.c_double, dp, dp], None),
            "axo_gw_band_energy": ([P, dp, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double], ctypes.c_double),
            "axo_tl_run": ([P, dp, dp, dp, dp, dp, dp, dp, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                            ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, dp, dp], None),
        }
        for name, (a, r) in spec.items():
            f = getattr(L, name)
            f.argtypes = a
            f.restype = r
        for name, (a, r) in optional.items():
            if hasattr(L, name):
                f = getattr(L, name)
                f.argtypes = a
                f.restype = r
    return _lib


def dptr(a):
    if a is None:
        return None
    if a.dtype == np.complex128:
        a = a.view(np.float64)
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def kick_coeffs(p: Params, t: float, dt: float):
    f = np.zeros(4)
    pot = np.zeros(4)
    lib().axo_kick_coeffs(ctypes.byref(p), t, dt, dptr(f), dptr(pot))
    return f, pot


def get_dtau(p: Params, t1, t2, eps):
    dt = ctypes.c_double()
    n = ctypes.c_int64()
    lib().axo_get_dtau(ctypes.byref(p), t1, t2, eps, ctypes.byref(dt), ctypes.byref(n))
    return dt.value, n.value


def evolve_phi(p, phi, phid, u, ud, dt):
    lib().axo_evolve_phi(ctypes.byref(p), dptr(phi), dptr(phid), dptr(u), dptr(ud), dt)


def evolve_phidot(p, phi, phid, u, ud, t, dt):
    lib().axo_evolve_phidot(ctypes.byref(p), dptr(phi), dptr(phid), dptr(u), dptr(ud), t, dt)


def symplectic_integration(p, phi, phid, u, ud, acc, t1, t2, eps):
    return lib().axo_symplectic_integration(ctypes.byref(p), dptr(phi), dptr(phid), dptr(u), dptr(ud),
                                            dptr(acc), t1, t2, eps)


def leapfrog(p, phi, phid, u, ud, acc, t1, dt, nsteps, first_half=True, last_half=True):
    """Same step sequence as the library's axg_leapfrog, built from the
    restated drift / kick (evolve.f90:246-255)."""
    t = t1
    if first_half:
        evolve_phi(p, phi, phid, u, ud, dt / 2)
        t = t + dt / 2
    for it in range(1, nsteps + 1):
        evolve_phidot(p, phi, phid, u, ud, t, dt)
        if p.gw_mode == 1 and acc is not None:
            grav_wave_integration(p, phi, acc, t, dt)
        h = dt / 2 if (it == nsteps and last_half) else dt
        evolve_phi(p, phi, phid, u, ud, h)
        t = t + h
    return t


def fft3d(a: np.ndarray, sign: int):
    b = np.ascontiguousarray(a, dtype=np.complex128).copy()
    lib().axo_fft3d(b.shape[0], dptr(b), sign)
    return b


def default_params(**kw):
    """The defaults of axg_params_default (settings.f90 values), filled in
    Python so that a process that only runs the oracle maps no GPU library."""
    p = Params()
    p.ngrid, p.precision, p.gw_mode = 64, 0, 0
    p.num_bin, p.num_bin_grav, p.degrade_spec = 50, 25, 0
    p.flags, p.compat, p.potential, p.n_dw, p.gw_log_bins = 1 | 2 | 4, 1, 0, 1, 64
    p.dspa = p.sigma_cr = p.kappa = p.tau_cr = p.a_now = 1.0
    p.width_cr, p.thickness_cr = 1.0 / np.sqrt(2.0), 1.0
    p.lambda_, p.vev, p.ma2_power, p.seed = 1.0, 1.0, 2.0, 1
    return p.update(**kw)


def gw_grid(p):
    """(ngrid_grav, dspa_grav) of init_grav (grav_waves.f90:37-45)."""
    deg = 1 << p.degrade_spec
    return p.ngrid // deg, p.dspa * deg


def green_acc_zeros(p):
    """Zeroed Green's-function accumulators arr_grav: [4][ng][ng][ng] complex128."""
    ng = gw_grid(p)[0]
    return np.zeros((4, ng, ng, ng), dtype=np.complex128)


def data1_to_arr_dphi_degrade(p, phi):
    ng = gw_grid(p)[0]
    out = np.zeros((3, ng, ng, ng), dtype=np.complex128)
    lib().axo_data1_to_arr_dphi_degrade(ctypes.byref(p), dptr(phi), dptr(out))
    return out


def grav_wave_integration(p, phi, acc, tau, dtau):
    lib().axo_grav_wave_integration(ctypes.byref(p), dptr(phi), dptr(acc), tau, dtau)


def grav_spec_estimation(p, acc):
    nb = p.num_bin_grav
    w, pw, nu, de = (np.zeros(nb) for _ in range(4))
    lib().axo_grav_spec_estimation(ctypes.byref(p), dptr(acc), dptr(w), dptr(pw), dptr(nu), dptr(de))
    return w, pw, nu, de


def uij_grav_spec(p, u, ud, tau):
    nb = p.num_bin_grav
    w, pw, nu, de = (np.zeros(nb) for _ in range(4))
    lib().axo_uij_grav_spec(ctypes.byref(p), dptr(u), dptr(ud), tau, dptr(w), dptr(pw), dptr(nu), dptr(de))
    return w, pw, nu, de


def grav_spec_log_green(p, acc):
    nb = p.gw_log_bins
    e = np.zeros(nb + 1)
    pw, nu, de = (np.zeros(nb) for _ in range(3))
    lib().axo_grav_spec_log_green(ctypes.byref(p), dptr(acc), dptr(e), dptr(pw), dptr(nu), dptr(de))
    return e, pw, nu, de


def uij_grav_spec_log(p, u, ud, tau):
    nb = p.gw_log_bins
    e = np.zeros(nb + 1)
    pw, nu, de = (np.zeros(nb) for _ in range(3))
    lib().axo_uij_grav_spec_log(ctypes.byref(p), dptr(u), dptr(ud), tau, dptr(e), dptr(pw), dptr(nu), dptr(de))
    return e, pw, nu, de


def ic_gaussian_flat(p, kcut, realisation=0):
    n = p.ngrid
    phi = np.zeros((n, n, n), np.complex128)
    phid = np.zeros((n, n, n), np.complex128)
    lib().axo_ic_gaussian_flat(ctypes.byref(p), kcut, realisation, dptr(phi), dptr(phid))
    return phi, phid


def ic_thermal(p, tau_ini, realisation=0):
    n = p.ngrid
    phi = np.zeros((n, n, n), np.complex128)
    phid = np.zeros((n, n, n), np.complex128)
    lib().axo_ic_thermal(ctypes.byref(p), tau_ini, realisation, dptr(phi), dptr(phid))
    return phi, phid


def field_moments(p, phi, phid, tau):
    out = np.zeros(4)
    lib().axo_field_moments(ctypes.byref(p), dptr(phi), dptr(phid), tau, dptr(out))
    return out


def det_atan2(y, x):
    return lib().axo_det_atan2(y, x)


def det_sincos(x):
    s = ctypes.c_double()
    c = ctypes.c_double()
    lib().axo_det_sincos(x, ctypes.byref(s), ctypes.byref(c))
    return s.value, c.value


def philox(ctr, key):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib().axo_philox(c, k, o)
    return tuple(o)


def classify_cells(p, phi, which, phase_mode=0):
    n = p.ngrid
    flags = np.zeros((n, n, n), np.int8)
    c = (ctypes.c_int64 * 3)()
    lib().axo_classify_cells(ctypes.byref(p), dptr(phi), which, phase_mode,
                             flags.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)), c)
    return flags, np.array(c[:], np.int64)


def string_winding(p, phi):
    c = (ctypes.c_int64 * 3)()
    lib().axo_string_winding(ctypes.byref(p), dptr(phi), c)
    return np.array(c[:], np.int64)


def id_defects(p, phi, phid, tau, max_strings=None, max_walls=None):
    n = p.ngrid
    ms = n ** 3 if max_strings is None else max_strings
    mw = n ** 3 if max_walls is None else max_walls
    sl, wa, sv = np.zeros(3), np.zeros(3), np.zeros(3)
    c = (ctypes.c_int64 * 3)()
    s = np.zeros((max(ms, 1), 13))
    w = np.zeros((max(mw, 1), 10))
    flags = np.zeros((n, n, n), np.int8)
    lib().axo_id_defects(ctypes.byref(p), dptr(phi), dptr(phid), tau, dptr(sl), dptr(wa), dptr(sv), c,
                         dptr(s), ms, dptr(w), mw, flags.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)))
    cnt = np.array(c[:], np.int64)
    return sl, wa, sv, cnt, s[:cnt[0]], w[:cnt[1]], flags


def fit_cells(p, phi, phid, scells, wcells):
    """Rows of the id_defects fits (as id_defects returns them) for the given
    string and wall cell indices only."""
    sc = np.ascontiguousarray(scells, np.int64)
    wc = np.ascontiguousarray(wcells, np.int64)
    s = np.zeros((max(len(sc), 1), 13))
    w = np.zeros((max(len(wc), 1), 10))
    i64p = ctypes.POINTER(ctypes.c_int64)
    lib().axo_fit_cells(ctypes.byref(p), dptr(phi), dptr(phid), sc.ctypes.data_as(i64p), len(sc), dptr(s),
                        wc.ctypes.data_as(i64p), len(wc), dptr(w))
    return s[:len(sc)], w[:len(wc)]


def position_string(ph, seed, cell):
    ph = np.ascontiguousarray(ph, np.float64)
    pos, d = np.zeros(3), np.zeros(3)
    gof = ctypes.c_double()
    sl = ctypes.c_double()
    lib().axo_position_string(dptr(ph), seed, cell, dptr(pos), dptr(d), ctypes.byref(gof), ctypes.byref(sl))
    return pos, d, gof.value, sl.value


def position_wall(ph):
    ph = np.ascontiguousarray(ph, np.float64)
    pos, d = np.zeros(3), np.zeros(3)
    gof = ctypes.c_double()
    wa = ctypes.c_double()
    lib().axo_position_wall(dptr(ph), dptr(pos), dptr(d), ctypes.byref(gof), ctypes.byref(wa))
    return pos, d, gof.value, wa.value


def string_length(pos, d):
    pos = np.ascontiguousarray(pos, np.float64)
    d = np.ascontiguousarray(d, np.float64)
    return lib().axo_string_length(dptr(pos), dptr(d))


def spectrum_estimation(p, phid, flags, tau):
    nb = p.num_bin
    w, pw, cv, ct = (np.zeros(nb) for _ in range(4))
    md = np.zeros(nb * (nb + 1) // 2)
    fptr = flags.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)) if flags is not None else None
    lib().axo_spectrum_estimation(ctypes.byref(p), dptr(phid), fptr, tau, dptr(w), dptr(pw), dptr(cv),
                                  dptr(ct), dptr(md))
    return w, pw, cv, ct, md


def init_spectrum(p):
    nb = p.num_bin
    nc = nb * (nb + 1) // 2
    ms = np.zeros((nc, 501))
    lq = np.zeros((nc, 501))
    dq = np.zeros(nc)
    wav = np.zeros(nb + 1)
    lib().axo_init_spectrum(ctypes.byref(p), dptr(ms), dptr(lq), dptr(dq), dptr(wav))
    return ms, lq, dq, wav


def compute_crho(p, wav, power):
    r = ctypes.c_double()
    lib().axo_compute_crho(ctypes.byref(p), dptr(np.ascontiguousarray(wav)), dptr(np.ascontiguousarray(power)),
                           ctypes.byref(r))
    return r.value


def pp_inverse(ap: np.ndarray, n: int):
    a = np.ascontiguousarray(ap, np.float64).copy()
    info = lib().axo_pp_inverse(n, dptr(a))
    return a, info


def gw_band_energy(p, u, ud, tau, kmin, kmax):
    return lib().axo_gw_band_energy(ctypes.byref(p), dptr(u), dptr(ud), tau, kmin, kmax)


def tl_run(p, state, dstate, dlambda, t1, dt, nsteps, kmin, kmax, first_half=True, last_half=True):
    """Forward + tangent-linear run (copies its inputs); returns (J, dJ)."""
    phi, phid, u, ud = (np.ascontiguousarray(a).copy() for a in state)
    dphi, dphid, du, dud = (np.ascontiguousarray(a).copy() for a in dstate)
    J = ctypes.c_double()
    dJ = ctypes.c_double()
    lib().axo_tl_run(ctypes.byref(p), dptr(phi), dptr(phid), dptr(u), dptr(ud), dptr(dphi), dptr(dphid), dptr(du),
                     dptr(dud), dlambda, t1, dt, nsteps, int(first_half), int(last_half), kmin, kmax,
                     ctypes.byref(J), ctypes.byref(dJ))
    return J.value, dJ.value


def estimate_covmat(p, flags, power, mat_div, min_mc=10, max_mc=100, tol=0.1):
    nb = p.num_bin
    cov = np.zeros(nb * (nb + 1) // 2)
    it = ctypes.c_int()
    fptr = flags.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)) if flags is not None else None
    lib().axo_estimate_covmat(ctypes.byref(p), fptr, dptr(np.ascontiguousarray(power, np.float64)),
                              dptr(np.ascontiguousarray(mat_div, np.float64)), min_mc, max_mc, tol, dptr(cov),
                              ctypes.byref(it))
    return cov, it.value


def compute_crho_cov(p, wav, power, cov):
    r, d = ctypes.c_double(), ctypes.c_double()
    lib().axo_compute_crho_cov(ctypes.byref(p), dptr(np.ascontiguousarray(wav, np.float64)),
                               dptr(np.ascontiguousarray(power, np.float64)), dptr(np.ascontiguousarray(cov, np.float64)),
                               ctypes.byref(r), ctypes.byref(d))
    return r.value, d.value


def epsilon(nb, wav, p1, p2, c1, c2, tau1, tau2):
    e, d = ctypes.c_double(), ctypes.c_double()
    a = [np.ascontiguousarray(x, np.float64) for x in (wav, p1, p2, c1, c2)]
    lib().axo_epsilon(nb, *[dptr(x) for x in a], tau1, tau2, ctypes.byref(e), ctypes.byref(d))
    return e.value, d.value


def mat_divided(md, counts):
    """spectrum.f90:267-273: the deconvolution matrix divided by the mode counts."""
    nb = len(counts)
    out = np.array(md, dtype=np.float64).copy()
    for i in range(1, nb + 1):
        for j in range(1, i + 1):
            ij = i * (i - 1) // 2 + j
            out[ij - 1] = out[ij - 1] / counts[i - 1] / counts[j - 1]
    return out
