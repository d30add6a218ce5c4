"""axion_grav_gb300 -- GB300-native lattice hot path of axion_grav.

The compute lives in ``libaxgpu.so`` (hand-written CUDA for sm_103a plus
cuFFT), reached through the C-ABI of ``include/axgpu.h``.  This module is a
thin ctypes mirror of that C-ABI whose method names follow the reference's
Fortran module routines (evolve.f90, grav_waves.f90, defects_3d.f90,
spectrum.f90, initial.f90), so host code reads like the reference:

    lat = Lattice(params)                  # init_grav / init_spectrum / allocate_data
    lat.upload(phi, phidot)                # data1 / data2 in
    t = lat.evolve_phi(t, dt / 2)          # evolve.f90:259
    lat.evolve_phidot(t, dt)               # evolve.f90:283
    nt = lat.symplectic_integration(t1, t2, eps_dtau)   # evolve.f90:238
    counts = lat.classify_cells()          # defects_3d.f90:67-103
    wave, power, numer, denom = lat.grav_spec_estimation(tau)   # grav_waves.f90:257

There is no CPU fallback: importing works without a GPU (so the C-ABI can be
inspected), but creating a Lattice requires the compiled library and a CUDA
device and raises otherwise.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

__all__ = [
    "Params", "Lattice", "AxgError", "load_library", "library_path", "default_params",
    "PREC_FP64_PLAIN", "PREC_FP64_FUSED", "PREC_FP32_MIXED", "GW_NONE", "GW_GREEN", "GW_UIJ",
    "F_ID_STRINGS", "F_ID_WALLS", "F_SPEC_EST", "F_GRAV_SPEC", "F_INITIAL_LOOP", "F_GROUP_STRINGS",
    "F_GROUP_WALLS",
    "POT_REFERENCE", "POT_QUARTIC", "COMPAT_INTENDED", "COMPAT_REF", "EXPORTED_SYMBOLS",
    "field_moments_noalloc", "Ensemble", "epsilon", "tile_table",
]

_HERE = os.path.dirname(os.path.abspath(__file__))

PREC_FP64_PLAIN, PREC_FP64_FUSED, PREC_FP32_MIXED = 0, 1, 2
GW_NONE, GW_GREEN, GW_UIJ = 0, 1, 2
F_ID_STRINGS, F_ID_WALLS, F_SPEC_EST, F_GRAV_SPEC, F_INITIAL_LOOP = 1, 2, 4, 8, 16
F_GROUP_STRINGS, F_GROUP_WALLS = 32, 64
POT_REFERENCE, POT_QUARTIC = 0, 1
COMPAT_INTENDED, COMPAT_REF = 0, 1

_STATUS = {0: "OK", -1: "ERR_ARG", -2: "ERR_CUDA", -3: "ERR_NOMEM", -4: "ERR_STATE",
           -5: "ERR_IO", -6: "ERR_TIMEOUT", -7: "ERR_UNSUPPORTED", -8: "ERR_NUMERIC"}


class AxgError(RuntimeError):
    """Nonzero status of a C-ABI call (the reference calls MpiStop, utils.f90:44)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{_STATUS.get(code, code)}: {msg}")
        self.code = code


class Params(ctypes.Structure):
    """Mirror of ``axg_params`` (include/axgpu.h)."""

    _fields_ = [
        ("ngrid", ctypes.c_int32), ("precision", ctypes.c_int32), ("gw_mode", ctypes.c_int32),
        ("num_bin", ctypes.c_int32), ("degrade_spec", ctypes.c_int32), ("flags", ctypes.c_int32),
        ("compat", ctypes.c_int32), ("potential", ctypes.c_int32), ("n_dw", ctypes.c_int32),
        ("num_bin_grav", ctypes.c_int32), ("gw_log_bins", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("dspa", ctypes.c_double), ("sigma_cr", ctypes.c_double), ("kappa", ctypes.c_double),
        ("tau_cr", ctypes.c_double), ("a_now", ctypes.c_double), ("width_cr", ctypes.c_double),
        ("thickness_cr", ctypes.c_double), ("lambda_", ctypes.c_double), ("vev", ctypes.c_double),
        ("ma2_0", ctypes.c_double), ("tau_axion_on", ctypes.c_double),
        ("ma2_power", ctypes.c_double), ("seed", ctypes.c_uint64), ("reserved1", ctypes.c_uint64),
    ]

    def update(self, **kw) -> "Params":
        for k, v in kw.items():
            if k == "lambda":
                k = "lambda_"
            if not hasattr(self, k):
                raise KeyError(k)
            setattr(self, k, v)
        return self

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


# Every function include/axgpu.h declares (checked by the CPU test suite).
EXPORTED_SYMBOLS = (
    "axg_version", "axg_params_default", "axg_create", "axg_destroy", "axg_last_error",
    "axg_memory_bytes", "axg_upload", "axg_download", "axg_upload_uij", "axg_download_uij",
    "axg_upload_gw_green", "axg_download_gw_green", "axg_get_dtau", "axg_evolve_phi",
    "axg_evolve_phidot", "axg_symplectic_integration", "axg_leapfrog",
    "axg_grav_spec_estimation", "axg_grav_spec_log", "axg_classify_cells",
    "axg_download_defect_flags", "axg_string_winding", "axg_id_defects",
    "axg_download_defect_lists", "axg_spectrum_estimation", "axg_compute_crho",
    "axg_ic_gaussian_flat", "axg_ic_thermal", "axg_field_moments", "axg_write_chk",
    "axg_read_chk", "axg_write_param_chk", "axg_read_param_chk", "axg_synchronize",
    "axg_event_record", "axg_event_elapsed", "axg_set_kernel_timing", "axg_kernel_timing",
    "axg_launch_count", "axg_tile_count", "axg_tile_info", "axg_set_tile", "axg_autotune",
    "axg_field_moments_noalloc", "axg_ensemble_create", "axg_ensemble_destroy", "axg_ensemble_last_error",
    "axg_ensemble_size", "axg_ensemble_member", "axg_ensemble_leapfrog", "axg_ensemble_autotune",
    "axg_ensemble_launch_count", "axg_adjoint_gw_band", "axg_spectrum_covariance", "axg_compute_crho_cov",
    "axg_epsilon", "axg_ensemble_set_tile", "axg_ensemble_set_launch_mode", "axg_ensemble_launch_mode",
    "axg_selftest_wait_timeout", "axg_ensemble_grav_spec_mean", "axg_ensemble_defect_mean",
    "axg_write_spectrum", "axg_write_covariance", "axg_write_gravspec", "axg_append_string_wall_line",
    "axg_append_crho_line", "axg_append_eps_line",
)

_lib = None


def library_path() -> str:
    return os.environ.get("AXGPU_LIB", os.path.join(_HERE, "libaxgpu.so"))


def load_library():
    """Load libaxgpu.so (raises if it was not built: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(f"libaxgpu.so not built at {path}; run __graft_entry__.build()")
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    c_ctx = ctypes.c_void_p
    dp = P(ctypes.c_double)
    i64p = P(ctypes.c_int64)
    sig = {
        "axg_version": ([], ctypes.c_int),
        "axg_params_default": ([P(Params)], ctypes.c_int),
        "axg_create": ([P(Params), P(c_ctx)], ctypes.c_int),
        "axg_destroy": ([c_ctx], ctypes.c_int),
        "axg_last_error": ([c_ctx], ctypes.c_char_p),
        "axg_memory_bytes": ([c_ctx, i64p], ctypes.c_int),
        "axg_upload": ([c_ctx, dp, dp, ctypes.c_int64, ctypes.c_int64], ctypes.c_int),
        "axg_download": ([c_ctx, dp, dp, ctypes.c_int64, ctypes.c_int64], ctypes.c_int),
        "axg_upload_uij": ([c_ctx, dp, dp], ctypes.c_int),
        "axg_download_uij": ([c_ctx, dp, dp], ctypes.c_int),
        "axg_upload_gw_green": ([c_ctx, dp], ctypes.c_int),
        "axg_download_gw_green": ([c_ctx, dp], ctypes.c_int),
        "axg_get_dtau": ([P(Params), ctypes.c_double, ctypes.c_double, ctypes.c_double, dp, i64p],
                         ctypes.c_int),
        "axg_evolve_phi": ([c_ctx, dp, ctypes.c_double], ctypes.c_int),
        "axg_evolve_phidot": ([c_ctx, ctypes.c_double, ctypes.c_double], ctypes.c_int),
        "axg_symplectic_integration": ([c_ctx, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        i64p], ctypes.c_int),
        "axg_leapfrog": ([c_ctx, ctypes.c_double, ctypes.c_double, ctypes.c_int64, ctypes.c_int,
                          ctypes.c_int], ctypes.c_int),
        "axg_grav_spec_estimation": ([c_ctx, ctypes.c_double, dp, dp, dp, dp], ctypes.c_int),
        "axg_grav_spec_log": ([c_ctx, ctypes.c_double, dp, dp, dp, dp], ctypes.c_int),
        "axg_classify_cells": ([c_ctx, ctypes.c_int, i64p], ctypes.c_int),
        "axg_download_defect_flags": ([c_ctx, P(ctypes.c_int8)], ctypes.c_int),
        "axg_string_winding": ([c_ctx, i64p], ctypes.c_int),
        "axg_id_defects": ([c_ctx, ctypes.c_int64, ctypes.c_double, dp, dp, dp, i64p], ctypes.c_int),
        "axg_download_defect_lists": ([c_ctx, dp, ctypes.c_int64, dp, ctypes.c_int64], ctypes.c_int),
        "axg_spectrum_estimation": ([c_ctx, ctypes.c_double, dp, dp, dp, dp], ctypes.c_int),
        "axg_compute_crho": ([c_ctx, dp], ctypes.c_int),
        "axg_ic_gaussian_flat": ([c_ctx, ctypes.c_double, ctypes.c_uint32], ctypes.c_int),
        "axg_ic_thermal": ([c_ctx, ctypes.c_double, ctypes.c_uint32], ctypes.c_int),
        "axg_field_moments": ([c_ctx, ctypes.c_double, dp], ctypes.c_int),
        "axg_write_chk": ([c_ctx, ctypes.c_char_p], ctypes.c_int),
        "axg_read_chk": ([c_ctx, ctypes.c_char_p], ctypes.c_int),
        "axg_write_param_chk": ([ctypes.c_char_p, ctypes.c_int64, ctypes.c_double, ctypes.c_int],
                                ctypes.c_int),
        "axg_read_param_chk": ([ctypes.c_char_p, i64p, dp, P(ctypes.c_int)], ctypes.c_int),
        "axg_synchronize": ([c_ctx], ctypes.c_int),
        "axg_event_record": ([c_ctx, ctypes.c_int], ctypes.c_int),
        "axg_event_elapsed": ([c_ctx, ctypes.c_int, ctypes.c_int, P(ctypes.c_float)], ctypes.c_int),
        "axg_set_kernel_timing": ([c_ctx, ctypes.c_int], ctypes.c_int),
        "axg_kernel_timing": ([c_ctx, ctypes.c_int, ctypes.c_char_p, ctypes.c_int64, i64p, dp],
                              ctypes.c_int),
        "axg_launch_count": ([c_ctx, i64p], ctypes.c_int),
        "axg_selftest_wait_timeout": ([c_ctx, ctypes.c_int64], ctypes.c_int),
        "axg_tile_count": ([], ctypes.c_int),
        "axg_tile_info": ([ctypes.c_int, P(ctypes.c_int32), P(ctypes.c_int32), P(ctypes.c_int32),
                           P(ctypes.c_int32)], ctypes.c_int),
        "axg_set_tile": ([c_ctx, ctypes.c_int], ctypes.c_int),
        "axg_autotune": ([c_ctx, ctypes.c_int, P(ctypes.c_int), dp], ctypes.c_int),
        "axg_field_moments_noalloc": ([P(Params), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, dp,
                                       ctypes.c_void_p], ctypes.c_int),
        "axg_ensemble_create": ([P(Params), ctypes.c_int32, P(ctypes.c_void_p)], ctypes.c_int),
        "axg_ensemble_destroy": ([ctypes.c_void_p], ctypes.c_int),
        "axg_ensemble_set_tile": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
        "axg_ensemble_set_launch_mode": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
        "axg_ensemble_launch_mode": ([ctypes.c_void_p, P(ctypes.c_int)], ctypes.c_int),
        "axg_ensemble_last_error": ([ctypes.c_void_p], ctypes.c_char_p),
        "axg_ensemble_size": ([ctypes.c_void_p, P(ctypes.c_int32)], ctypes.c_int),
        "axg_ensemble_member": ([ctypes.c_void_p, ctypes.c_int32, P(ctypes.c_void_p)], ctypes.c_int),
        "axg_ensemble_leapfrog": ([ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int64, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "axg_ensemble_autotune": ([ctypes.c_void_p, ctypes.c_int, P(ctypes.c_int), dp], ctypes.c_int),
        "axg_ensemble_launch_count": ([ctypes.c_void_p, P(ctypes.c_int64)], ctypes.c_int),
        "axg_ensemble_grav_spec_mean": ([ctypes.c_void_p, ctypes.c_double, dp, dp, dp, dp], ctypes.c_int),
        "axg_ensemble_defect_mean": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, dp, dp, dp, dp],
                                     ctypes.c_int),
        "axg_write_spectrum": ([ctypes.c_char_p, ctypes.c_int32, dp, dp, dp, dp, ctypes.c_int32], ctypes.c_int),
        "axg_write_covariance": ([ctypes.c_char_p, ctypes.c_int32, dp, ctypes.c_int32], ctypes.c_int),
        "axg_write_gravspec": ([ctypes.c_char_p, ctypes.c_int32, ctypes.c_double, dp, dp, dp, ctypes.c_int32,
                                ctypes.c_double, ctypes.c_double], ctypes.c_int),
        "axg_append_string_wall_line": ([ctypes.c_char_p, ctypes.c_int32, ctypes.c_double, ctypes.c_double, dp, dp,
                                         dp], ctypes.c_int),
        "axg_append_crho_line": ([ctypes.c_char_p, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_double], ctypes.c_int),
        "axg_append_eps_line": ([ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, dp, dp], ctypes.c_int),
        "axg_spectrum_covariance": ([c_ctx, ctypes.c_int, ctypes.c_int, ctypes.c_double, dp, P(ctypes.c_int)],
                                    ctypes.c_int),
        "axg_compute_crho_cov": ([c_ctx, dp, dp], ctypes.c_int),
        "axg_epsilon": ([ctypes.c_int32, dp, dp, dp, dp, dp, ctypes.c_double, ctypes.c_double, dp, dp], ctypes.c_int),
        "axg_adjoint_gw_band": ([c_ctx, ctypes.c_double, ctypes.c_double, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_int64, ctypes.c_double, ctypes.c_double, dp, dp, dp, dp, dp, dp],
                                ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def default_params(**kw) -> Params:
    p = Params()
    load_library().axg_params_default(ctypes.byref(p))
    return p.update(**kw)


def field_moments_noalloc(params: Params, d_phi: int, d_phidot: int, tau: float,
                          stream: Optional[int] = None) -> np.ndarray:
    """axg_field_moments_noalloc: volume moments of caller-owned complex128
    device arrays (raw device addresses) without any device allocation, for
    callers that cannot allocate device memory; ngrid <= 2048."""
    lib = load_library()
    out = np.zeros(4)
    rc = lib.axg_field_moments_noalloc(ctypes.byref(params), ctypes.c_void_p(d_phi), ctypes.c_void_p(d_phidot),
                                       tau, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                       ctypes.c_void_p(stream) if stream else None)
    if rc != 0:
        raise AxgError(rc, lib.axg_last_error(None).decode())
    return out


def tile_table() -> list:
    """(tx, ty, zc, pointwise_tma) of every fused-kernel tile shape, by index."""
    lib = load_library()
    out = []
    for i in range(lib.axg_tile_count()):
        a, b, c, d = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        lib.axg_tile_info(i, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d))
        out.append((a.value, b.value, c.value, d.value))
    return out


def epsilon(wav, p1, p2, c1, c2, tau1, tau2):
    """get_epsilon (spectrum.f90:1002-1036) for one pair of output times."""
    lib = load_library()
    e, d = ctypes.c_double(), ctypes.c_double()
    arrs = [np.ascontiguousarray(a, np.float64) for a in (wav, p1, p2, c1, c2)]
    rc = lib.axg_epsilon(len(arrs[1]), *[_dptr(a) for a in arrs], tau1, tau2, ctypes.byref(e), ctypes.byref(d))
    if rc != 0:
        raise AxgError(rc, "axg_epsilon")
    return e.value, d.value


def _dptr(a: Optional[np.ndarray]):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Lattice:
    """One GPU lattice context (owns all device state of the hot path)."""

    def __init__(self, params: Params, _handle=None, _owner=None):
        self.lib = load_library()
        self.params = params
        self.n = int(params.ngrid)
        self._ctx = ctypes.c_void_p()
        self._owner = _owner  # a member of an Ensemble is destroyed with it
        if _handle is not None:
            self._ctx = _handle
            return
        rc = self.lib.axg_create(ctypes.byref(params), ctypes.byref(self._ctx))
        if rc != 0:
            raise AxgError(rc, self.lib.axg_last_error(None).decode())

    # -- housekeeping -----------------------------------------------------
    def _check(self, rc: int):
        if rc != 0:
            raise AxgError(rc, self.lib.axg_last_error(self._ctx).decode())

    def close(self):
        if self._ctx and self._owner is None:
            self.lib.axg_destroy(self._ctx)
        self._ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._ctx

    def memory_bytes(self) -> int:
        v = ctypes.c_int64()
        self._check(self.lib.axg_memory_bytes(self._ctx, ctypes.byref(v)))
        return v.value

    def synchronize(self):
        self._check(self.lib.axg_synchronize(self._ctx))

    # -- state ---------------------------------------------------------------
    def upload(self, phi: Optional[np.ndarray] = None, phidot: Optional[np.ndarray] = None):
        n = self.n
        for a in (phi, phidot):
            if a is not None:
                assert a.dtype == np.complex128 and a.flags.c_contiguous and a.size == n ** 3
        self._check(self.lib.axg_upload(self._ctx, _dptr(phi.view(np.float64) if phi is not None else None),
                                        _dptr(phidot.view(np.float64) if phidot is not None else None),
                                        n * n, 0))

    def download(self, phi: bool = True, phidot: bool = True):
        """(phi, phidot) as complex128 host arrays; a field not asked for is None."""
        n = self.n
        a = np.empty((n, n, n), np.complex128) if phi else None
        b = np.empty((n, n, n), np.complex128) if phidot else None
        self._check(self.lib.axg_download(self._ctx, _dptr(a.view(np.float64)) if phi else None,
                                          _dptr(b.view(np.float64)) if phidot else None, n * n, 0))
        return a, b

    def upload_uij(self, u: np.ndarray, udot: np.ndarray):
        for a in (u, udot):
            assert a.dtype == np.float64 and a.flags.c_contiguous and a.size == 6 * self.n ** 3
        self._check(self.lib.axg_upload_uij(self._ctx, _dptr(u), _dptr(udot)))

    def download_uij(self):
        n = self.n
        u = np.empty((6, n, n, n), np.float64)
        ud = np.empty((6, n, n, n), np.float64)
        self._check(self.lib.axg_download_uij(self._ctx, _dptr(u), _dptr(ud)))
        return u, ud

    @property
    def gw_n(self) -> int:
        """Side of the Green's-function GW grid: ngrid / 2**degrade_spec
        (init_grav, grav_waves.f90:37-45)."""
        return self.n >> int(self.params.degrade_spec)

    def upload_gw_green(self, acc: np.ndarray):
        assert acc.dtype == np.complex128 and acc.size == 4 * self.gw_n ** 3
        self._check(self.lib.axg_upload_gw_green(self._ctx, _dptr(acc.view(np.float64))))

    def download_gw_green(self) -> np.ndarray:
        n = self.gw_n
        acc = np.empty((4, n, n, n), np.complex128)
        self._check(self.lib.axg_download_gw_green(self._ctx, _dptr(acc.view(np.float64))))
        return acc

    # -- initial conditions (initial.f90) ---------------------------------------
    def ic_gaussian_flat(self, kcut: float, realisation: int = 0):
        self._check(self.lib.axg_ic_gaussian_flat(self._ctx, kcut, realisation))

    def ic_thermal(self, tau_ini: float, realisation: int = 0):
        self._check(self.lib.axg_ic_thermal(self._ctx, tau_ini, realisation))

    def field_moments(self, tau: float) -> np.ndarray:
        out = np.zeros(4)
        self._check(self.lib.axg_field_moments(self._ctx, tau, _dptr(out)))
        return out

    # -- evolution (evolve.f90) -------------------------------------------------
    def get_dtau(self, tau1: float, tau2: float, eps_dtau: float):
        dt = ctypes.c_double()
        nt = ctypes.c_int64()
        self._check(self.lib.axg_get_dtau(ctypes.byref(self.params), tau1, tau2, eps_dtau,
                                          ctypes.byref(dt), ctypes.byref(nt)))
        return dt.value, nt.value

    def evolve_phi(self, t: float, dt: float) -> float:
        tt = ctypes.c_double(t)
        self._check(self.lib.axg_evolve_phi(self._ctx, ctypes.byref(tt), dt))
        return tt.value

    def evolve_phidot(self, t: float, dt: float):
        self._check(self.lib.axg_evolve_phidot(self._ctx, t, dt))

    def symplectic_integration(self, t1: float, t2: float, eps_dtau: float) -> int:
        nt = ctypes.c_int64()
        self._check(self.lib.axg_symplectic_integration(self._ctx, t1, t2, eps_dtau, ctypes.byref(nt)))
        return nt.value

    def leapfrog(self, t1: float, dt: float, nsteps: int, first_half: bool = True,
                 last_half: bool = True):
        self._check(self.lib.axg_leapfrog(self._ctx, t1, dt, nsteps, int(first_half), int(last_half)))

    # -- gravitational waves (grav_waves.f90) -----------------------------------
    def grav_spec_estimation(self, tau: float):
        nb = int(self.params.num_bin_grav)
        w, p, nu, de = (np.zeros(nb) for _ in range(4))
        self._check(self.lib.axg_grav_spec_estimation(self._ctx, tau, _dptr(w), _dptr(p), _dptr(nu), _dptr(de)))
        return w, p, nu, de

    def grav_spec_log(self, tau: float):
        nb = int(self.params.gw_log_bins)
        e = np.zeros(nb + 1)
        p, nu, de = (np.zeros(nb) for _ in range(3))
        self._check(self.lib.axg_grav_spec_log(self._ctx, tau, _dptr(e), _dptr(p), _dptr(nu), _dptr(de)))
        return e, p, nu, de

    # -- defects (defects_3d.f90) -----------------------------------------------
    def classify_cells(self, which: Optional[int] = None) -> np.ndarray:
        if which is None:
            which = int(self.params.flags) & (F_ID_STRINGS | F_ID_WALLS | F_SPEC_EST)
        c = (ctypes.c_int64 * 3)()
        self._check(self.lib.axg_classify_cells(self._ctx, which, c))
        return np.array(c[:], dtype=np.int64)

    def defect_flags(self) -> np.ndarray:
        n = self.n
        f = np.empty((n, n, n), np.int8)
        self._check(self.lib.axg_download_defect_flags(self._ctx, f.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))))
        return f

    def string_winding(self) -> np.ndarray:
        c = (ctypes.c_int64 * 3)()
        self._check(self.lib.axg_string_winding(self._ctx, c))
        return np.array(c[:], dtype=np.int64)

    def id_defects(self, idx: int, tau: float):
        sl, wa, sv = np.zeros(3), np.zeros(3), np.zeros(3)
        c = (ctypes.c_int64 * 3)()
        self._check(self.lib.axg_id_defects(self._ctx, idx, tau, _dptr(sl), _dptr(wa), _dptr(sv), c))
        return sl, wa, sv, np.array(c[:], dtype=np.int64)

    def defect_lists(self, ns: int, nw: int):
        s = np.zeros((max(ns, 1), 13))
        w = np.zeros((max(nw, 1), 10))
        self._check(self.lib.axg_download_defect_lists(self._ctx, _dptr(s), ns, _dptr(w), nw))
        return s[:ns], w[:nw]

    # -- field spectrum (spectrum.f90) ------------------------------------------
    def spectrum_estimation(self, tau: float):
        nb = int(self.params.num_bin)
        w, p, cv, ct = (np.zeros(nb) for _ in range(4))
        self._check(self.lib.axg_spectrum_estimation(self._ctx, tau, _dptr(w), _dptr(p), _dptr(cv), _dptr(ct)))
        return w, p, cv, ct

    def spectrum_covariance(self, min_mc: int = 10, max_mc: int = 100, tol: float = 0.1):
        nb = int(self.params.num_bin)
        cov = np.zeros(nb * (nb + 1) // 2)
        it = ctypes.c_int()
        self._check(self.lib.axg_spectrum_covariance(self._ctx, min_mc, max_mc, tol, _dptr(cov), ctypes.byref(it)))
        return cov, it.value

    def compute_crho_cov(self):
        r, d = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.axg_compute_crho_cov(self._ctx, ctypes.byref(r), ctypes.byref(d)))
        return r.value, d.value

    def compute_crho(self) -> float:
        r = ctypes.c_double()
        self._check(self.lib.axg_compute_crho(self._ctx, ctypes.byref(r)))
        return r.value

    # -- adjoint ----------------------------------------------------------------
    def adjoint_gw_band(self, t1, dt, nsteps, stride, kmin, kmax, first_half=True, last_half=True,
                        want_grads=True):
        """J, dJ/dlambda, dJ/dphi0, dJ/dphidot0 (complex128 arrays) and the GPU
        ms of the forward and reverse sweeps (axg_adjoint_gw_band)."""
        n = self.n
        J, dl, mf, mr = (ctypes.c_double() for _ in range(4))
        g0 = np.zeros((n, n, n), np.complex128) if want_grads else None
        g1 = np.zeros((n, n, n), np.complex128) if want_grads else None
        self._check(self.lib.axg_adjoint_gw_band(
            self._ctx, t1, dt, nsteps, int(first_half), int(last_half), stride, kmin, kmax, ctypes.byref(J),
            ctypes.byref(dl), _dptr(g0.view(np.float64)) if want_grads else None,
            _dptr(g1.view(np.float64)) if want_grads else None, ctypes.byref(mf), ctypes.byref(mr)))
        return J.value, dl.value, g0, g1, mf.value, mr.value

    # -- checkpoint (evolve.f90:401-546) ----------------------------------------
    def write_chk(self, path: str):
        self._check(self.lib.axg_write_chk(self._ctx, path.encode()))

    def read_chk(self, path: str):
        self._check(self.lib.axg_read_chk(self._ctx, path.encode()))

    # -- timing -------------------------------------------------------------------
    def event_record(self, slot: int):
        self._check(self.lib.axg_event_record(self._ctx, slot))

    def event_elapsed(self, a: int, b: int) -> float:
        ms = ctypes.c_float()
        self._check(self.lib.axg_event_elapsed(self._ctx, a, b, ctypes.byref(ms)))
        return ms.value

    def set_kernel_timing(self, on: bool):
        self._check(self.lib.axg_set_kernel_timing(self._ctx, int(on)))

    def kernel_timings(self) -> list:
        out = []
        i = 0
        buf = ctypes.create_string_buffer(128)
        while True:
            nl = ctypes.c_int64()
            ms = ctypes.c_double()
            rc = self.lib.axg_kernel_timing(self._ctx, i, buf, 128, ctypes.byref(nl), ctypes.byref(ms))
            if rc != 0:
                break
            out.append((buf.value.decode(), nl.value, ms.value))
            i += 1
        return out

    # -- fused-kernel tiles / autotuner -------------------------------------------
    def tiles(self) -> list:
        return tile_table()

    def set_tile(self, cfg: int):
        self._check(self.lib.axg_set_tile(self._ctx, cfg))

    def autotune(self, steps: int = 3):
        best = ctypes.c_int()
        ms = ctypes.c_double()
        self._check(self.lib.axg_autotune(self._ctx, steps, ctypes.byref(best), ctypes.byref(ms)))
        return best.value, ms.value

    def launch_count(self) -> int:
        v = ctypes.c_int64()
        self._check(self.lib.axg_launch_count(self._ctx, ctypes.byref(v)))
        return v.value

    def selftest_wait_timeout(self, wait_cycles: int = 2_000_000):
        """Run the give-up path of the bounded stage wait (axg_selftest_wait_timeout);
        raises AxgError(ERR_TIMEOUT) when the path works."""
        self._check(self.lib.axg_selftest_wait_timeout(self._ctx, int(wait_cycles)))


class Ensemble:
    """Batched ensemble of lattices of uneven sizes stepped together
    (axg_ensemble_*); member(i) gives a Lattice view of one realisation."""

    def __init__(self, params_list):
        self.lib = load_library()
        arr = (Params * len(params_list))(*params_list)
        self._params = list(params_list)
        self._e = ctypes.c_void_p()
        rc = self.lib.axg_ensemble_create(arr, len(params_list), ctypes.byref(self._e))
        if rc != 0:
            raise AxgError(rc, self.lib.axg_last_error(None).decode())
        self.members = []
        for i, p in enumerate(self._params):
            h = ctypes.c_void_p()
            self._check(self.lib.axg_ensemble_member(self._e, i, ctypes.byref(h)))
            self.members.append(Lattice(p, _handle=h, _owner=self))

    def _check(self, rc):
        if rc != 0:
            raise AxgError(rc, self.lib.axg_ensemble_last_error(self._e).decode())

    def __len__(self):
        return len(self.members)

    def member(self, i) -> Lattice:
        return self.members[i]

    def leapfrog(self, t1, dt, nsteps, first_half=True, last_half=True, use_graph=True):
        self._check(self.lib.axg_ensemble_leapfrog(self._e, t1, dt, nsteps, int(first_half), int(last_half),
                                                   int(use_graph)))

    def set_tile(self, cfg: int):
        self._check(self.lib.axg_ensemble_set_tile(self._e, cfg))

    def set_launch_mode(self, persistent: bool):
        """True: resident CTAs walk the work items; False: one CTA per item."""
        self._check(self.lib.axg_ensemble_set_launch_mode(self._e, int(bool(persistent))))

    def launch_mode(self) -> bool:
        v = ctypes.c_int()
        self._check(self.lib.axg_ensemble_launch_mode(self._e, ctypes.byref(v)))
        return bool(v.value)

    def autotune(self, steps=3):
        best = ctypes.c_int()
        ms = ctypes.c_double()
        self._check(self.lib.axg_ensemble_autotune(self._e, steps, ctypes.byref(best), ctypes.byref(ms)))
        return best.value, ms.value

    def launch_count(self):
        v = ctypes.c_int64()
        self._check(self.lib.axg_ensemble_launch_count(self._e, ctypes.byref(v)))
        return v.value

    def grav_spec_mean(self, tau: float):
        """axg_ensemble_grav_spec_mean: (wave, power mean, power standard
        error, modes) over the members' GW spectra."""
        nb = int(self._params[0].num_bin_grav)
        w, m, s, d = (np.zeros(nb) for _ in range(4))
        self._check(self.lib.axg_ensemble_grav_spec_mean(self._e, tau, _dptr(w), _dptr(m), _dptr(s), _dptr(d)))
        return w, m, s, d

    def defect_mean(self, idx: int, tau: float):
        """axg_ensemble_defect_mean: (xi mean, xi standard error, A mean, A
        standard error), three components each."""
        xm, xs, am, as_ = (np.zeros(3) for _ in range(4))
        self._check(self.lib.axg_ensemble_defect_mean(self._e, idx, tau, _dptr(xm), _dptr(xs), _dptr(am), _dptr(as_)))
        return xm, xs, am, as_

    def close(self):
        if self._e:
            for m in self.members:
                m._ctx = ctypes.c_void_p()
            self.lib.axg_ensemble_destroy(self._e)
            self._e = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
