"""Text outputs in the reference program's file formats.

The reference writes its results from the host after each output time:

- ``<root>_string_wall_parameters.txt``: one ``(I,11E20.10e3)`` line per
  output, (idx, tau, tau^2 zeta, xi(1:3), A(1:3), v(1:3)) (evolve.f90:90,127,202);
- ``<root>_crho.txt``: ``(I,3E20.10e3)`` lines of the energy densities of
  analyze_energy (evolve.f90:91,128,215-235);
- ``<root>_spectrum_<idx>.dat``: ``(4E20.10e3)`` rows (q, P, conv/count, count)
  (spectrum.f90:278-285);
- ``<root>_covariance_<idx>.dat``: ``(2I,E20.10e3)`` rows (i, j, cov_ij)
  (spectrum.f90:294-302);
- ``<root>_gravspec_<idx>.dat``: ``(5E20.10e3)`` rows (tau, q, f, P_GW, modes)
  (grav_waves.f90:308-316);
- ``<root>_eps.txt``: ``(2I,7E20.10e3)`` rows of get_epsilon
  (spectrum.f90:996-1036).

A Fortran host keeps its own writers; these functions give a Python caller
of the library the same files.  Integers use the Intel compiler's default
``I`` width for 4-byte integers (12); reals follow the Fortran ``Ew.dEe``
edit descriptor (0.d...d mantissa, signed 3-digit exponent).
"""
from __future__ import annotations

import math
from decimal import ROUND_HALF_EVEN, Decimal
from typing import Iterable, Sequence

import numpy as np

# potential.f90:13-23 (reduced Planck mass, GeV -> Hz), the reference's pi
MSTAR_IN_GEV = 2.435e18
GEV_IN_HZ = 1.5192488833521e24
MSTAR_IN_HZ = MSTAR_IN_GEV * GEV_IN_HZ
REF_PI = 3.14159265359
REF_TWOPI = 2 * REF_PI
INT_WIDTH = 12


def fortran_e(x: float, w: int = 20, d: int = 10, e: int = 3) -> str:
    """``Ew.dEe``: x as 0.<d digits>E<sign><e digits>, right-justified in w."""
    x = float(x)
    if math.isnan(x):
        return "NaN".rjust(w)
    if math.isinf(x):
        return ("-Infinity" if x < 0 else "Infinity").rjust(w)
    sign = "-" if (x < 0 or (x == 0 and math.copysign(1.0, x) < 0)) else ""
    if x == 0:
        body = "0." + "0" * d + "E+" + "0" * e
    else:
        # d significant digits, rounded to nearest (exact decimal expansion of the double)
        q = Decimal(abs(x))
        exp10 = q.adjusted() + 1  # 0.d... x 10^exp10
        mant = q.scaleb(-exp10).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
        if mant >= 1:  # rounding carried into a new digit
            exp10 += 1
            mant = (mant / 10).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
        digits = str(mant)[2:].ljust(d, "0")
        body = "0." + digits + "E" + ("+" if exp10 >= 0 else "-") + str(abs(exp10)).rjust(e, "0")
    return (sign + body).rjust(w)


def fortran_i(n: int, w: int = INT_WIDTH) -> str:
    return str(int(n)).rjust(w)


def _line(ints: Iterable[int], reals: Iterable[float]) -> str:
    return "".join(fortran_i(i) for i in ints) + "".join(fortran_e(r) for r in reals)


def string_wall_line(idx: int, tau: float, zeta_tau2: float, xi: Sequence[float], area: Sequence[float],
                     vel: Sequence[float]) -> str:
    """One line of _string_wall_parameters.txt (evolve.f90:127, array_sw of :202)."""
    return _line([idx], [tau, zeta_tau2, *xi[:3], *area[:3], *vel[:3]])


def string_parameters(tau: float, dspa: float, ngrid: int, sl: Sequence[float], wa: Sequence[float]):
    """xi and A from the summed string length and wall area (evolve.f90:190-192)."""
    n3 = float(ngrid) ** 3
    xi = [(tau / dspa) ** 2 * s / n3 / 4 for s in sl[:3]]
    area = [(tau / dspa) * a / n3 / 2 for a in wa[:3]]
    return xi, area


def analyze_energy(tau: float, xi: Sequence[float], gamma: float, width_cr: float, crho_spec: float):
    """Conformal comoving energy densities of analyze_energy (evolve.f90:215-235):
    crho0 from the long strings xi(3), crho1 from the rest xi(1) - xi(3), crho2
    from the spectrum.  (array_sw(5) = xi(3), array_sw(3) = xi(1), array_sw(11) = v(3).)"""
    xi0 = xi[2]
    xi1 = xi[0] - xi[2]
    lg = math.log(0.5 * tau ** 2 / math.sqrt(xi0) / width_cr)
    crho0 = xi0 * REF_TWOPI * lg * 4 * gamma
    crho1 = xi1 * REF_TWOPI * lg * 4 * gamma
    return crho0, crho1, crho_spec


def crho_line(idx: int, crho0: float, crho1: float, crho2: float) -> str:
    """One line of _crho.txt (evolve.f90:128)."""
    return _line([idx], [crho0, crho1, crho2])


def spectrum_path(rootname: str, idx: int) -> str:
    return f"{rootname}_spectrum_{int(idx)}.dat"


def write_spectrum(rootname: str, idx: int, wave: Sequence[float], power: Sequence[float],
                   conv_per_mode: Sequence[float], count: Sequence[float]) -> str:
    """_spectrum_<idx>.dat (spectrum.f90:278-285): bin centre, deconvolved power,
    mean convolved power per mode, mode count."""
    path = spectrum_path(rootname, idx)
    with open(path, "w") as f:
        for q, p, c, n in zip(wave, power, conv_per_mode, count):
            f.write(_line([], [q, p, c, n]) + "\n")
    return path


def write_covariance(rootname: str, idx: int, cov: Sequence[float], num_bin: int) -> str:
    """_covariance_<idx>.dat (spectrum.f90:294-302), packed upper storage."""
    path = f"{rootname}_covariance_{int(idx)}.dat"
    with open(path, "w") as f:
        for i in range(1, num_bin + 1):
            for j in range(1, i + 1):
                f.write(_line([i, j], [cov[i * (i - 1) // 2 + j - 1]]) + "\n")
    return path


def freq_cr_in_hz(tau_cr: float, a_now: float) -> float:
    """grav_waves.f90:266."""
    return MSTAR_IN_HZ / tau_cr / a_now / REF_TWOPI


def write_gravspec(rootname: str, idx: int, tau: float, wave: Sequence[float], power: Sequence[float],
                   denom: Sequence[float], tau_cr: float, a_now: float) -> str:
    """_gravspec_<idx>.dat (grav_waves.f90:308-316): tau, bin centre q, q in Hz,
    P_GW, modes per bin."""
    path = f"{rootname}_gravspec_{int(idx)}.dat"
    fq = freq_cr_in_hz(tau_cr, a_now)
    with open(path, "w") as f:
        for q, p, dn in zip(wave, power, denom):
            f.write(_line([], [tau, q, q * fq, p, dn]) + "\n")
    return path


def eps_line(idx: int, idx2: int, tau1: float, tau2: float, eps: float, deps: float, crho1: Sequence[float],
             crho2: Sequence[float]) -> str:
    """One line of _eps.txt (spectrum.f90:1034-1035); crho = (rho, drho) at
    each output time."""
    tau = (tau2 + tau1) / 2
    return _line([idx, idx2], [tau1, tau2, tau, eps, deps, crho2[0] - crho1[0],
                               math.sqrt(crho2[1] ** 2 + crho1[1] ** 2)])


def read_columns(path: str) -> np.ndarray:
    """Numeric columns of a written file (Fortran E fields parse as floats)."""
    return np.loadtxt(path, ndmin=2)
