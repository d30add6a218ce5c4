"""Text outputs in the reference's formats (evolve.f90, spectrum.f90,
grav_waves.f90 writers): Fortran Ew.dEe / I edit descriptors and the files."""
import math

import numpy as np
import pytest

from axion_grav_gb300 import outputs as out


def test_fortran_e_edit_descriptor():
    # 0.<10 digits>E<sign><3 digits> is 17 characters, right-justified in 20
    assert out.fortran_e(1.0) == "   0.1000000000E+001"
    assert out.fortran_e(-1.23456789012345e-4) == "  -0.1234567890E-003"
    assert out.fortran_e(0.0) == "   0.0000000000E+000"
    assert out.fortran_e(9.99999999995) == "   0.1000000000E+002"  # rounding carries into a new digit
    assert out.fortran_e(1e-300) == "   0.1000000000E-299"
    assert out.fortran_e(123456.789) == "   0.1234567890E+006"
    assert len(out.fortran_e(-3.0e250)) == 20
    assert out.fortran_e(float("nan")).strip() == "NaN"
    assert out.fortran_i(7) == " " * 11 + "7" and len(out.fortran_i(-123)) == 12


def test_string_wall_and_crho_lines():
    xi, area = out.string_parameters(tau=4.0, dspa=0.5, ngrid=8, sl=[512.0, 256.0, 128.0], wa=[64.0, 32.0, 16.0])
    assert xi == [pytest.approx(64 * 512 / 512 / 4), pytest.approx(64 * 256 / 512 / 4), pytest.approx(64 * 128 / 512 / 4)]
    assert area[0] == pytest.approx(8 * 64 / 512 / 2)
    line = out.string_wall_line(3, 4.0, 1.5, xi, area, [0.1, 0.2, 1.1])
    assert len(line) == 12 + 11 * 20
    vals = [float(v) for v in line.split()]
    assert vals[0] == 3 and vals[1] == 4.0 and vals[3:6] == pytest.approx(xi, rel=1e-9)
    c0, c1, c2 = out.analyze_energy(4.0, xi, 1.1, 0.7, 2.5)
    assert c0 == pytest.approx(xi[2] * 2 * 3.14159265359 * math.log(0.5 * 16 / math.sqrt(xi[2]) / 0.7) * 4 * 1.1)
    assert c2 == 2.5
    assert [float(v) for v in out.crho_line(3, c0, c1, c2).split()] == pytest.approx([3, c0, c1, c2], rel=1e-9)


def test_spectrum_covariance_gravspec_files(tmp_path):
    root = str(tmp_path / "run")
    rng = np.random.default_rng(0)
    nb = 5
    w, p, c, n = rng.random(nb), rng.random(nb) * 1e-7, rng.random(nb), np.arange(1, nb + 1) * 6.0
    path = out.write_spectrum(root, 12, w, p, c, n)
    assert path.endswith("run_spectrum_12.dat")
    got = out.read_columns(path)
    assert got.shape == (nb, 4)
    np.testing.assert_allclose(got, np.stack([w, p, c, n], 1), rtol=1e-9)
    cov = rng.random(nb * (nb + 1) // 2)
    got = out.read_columns(out.write_covariance(root, 12, cov, nb))
    assert got.shape == (len(cov), 3) and list(got[:3, 0]) == [1, 2, 2] and list(got[:3, 1]) == [1, 1, 2]
    np.testing.assert_allclose(got[:, 2], cov, rtol=1e-9)
    got = out.read_columns(out.write_gravspec(root, 12, 7.5, w, p, n, tau_cr=1.0, a_now=1.0))
    assert got.shape == (nb, 5)
    np.testing.assert_allclose(got[:, 2], w * out.freq_cr_in_hz(1.0, 1.0), rtol=1e-9)


def test_eps_line():
    line = out.eps_line(4, 6, 10.0, 12.0, 0.25, 0.01, (1.0, 0.1), (1.5, 0.2))
    v = [float(x) for x in line.split()]
    assert v[:2] == [4, 6] and v[4] == 11.0 and v[7] == pytest.approx(0.5) and v[8] == pytest.approx(math.hypot(0.1, 0.2))
