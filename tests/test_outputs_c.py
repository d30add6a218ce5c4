"""The C-ABI text writers (axg_outputs.cu) against the Python writers
(axion_grav_gb300.outputs), byte for byte: the same files in the reference's
edit descriptors.  Host-only calls, no GPU."""
import ctypes

import numpy as np

import axion_grav_gb300 as ag
from axion_grav_gb300 import outputs as out


def _values(rng, n):
    v = rng.standard_normal(n) * 10.0 ** rng.integers(-300, 300, n)
    special = np.array([0.0, -0.0, 1.0, -1.0, 0.5, 2.0 ** -20, 9.9999999995, 9.99999999949, 1e-300, -1e300,
                        5e-324, np.pi, 0.1, 123456789012.0, np.inf, -np.inf, np.nan])
    return np.concatenate([special, v])[:n]


def _dp(a):
    a = np.ascontiguousarray(a, np.float64)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def test_c_writers_match_python(tmp_path, built):
    lib = ag.load_library()
    rng = np.random.default_rng(41)
    nb = 40
    w, pw, cv, ct = (_values(rng, nb) for _ in range(4))
    root_c, root_p = str(tmp_path / "c"), str(tmp_path / "p")
    a = [_dp(x) for x in (w, pw, cv, ct)]
    assert lib.axg_write_spectrum(root_c.encode(), 3, *(p for _, p in a), nb) == 0
    out.write_spectrum(root_p, 3, w, pw, cv, ct)
    assert open(root_c + "_spectrum_3.dat").read() == open(root_p + "_spectrum_3.dat").read()

    cov = _values(rng, nb * (nb + 1) // 2)
    assert lib.axg_write_covariance(root_c.encode(), 4, _dp(cov)[1], nb) == 0
    out.write_covariance(root_p, 4, cov, nb)
    assert open(root_c + "_covariance_4.dat").read() == open(root_p + "_covariance_4.dat").read()

    de = np.abs(_values(rng, nb))
    assert lib.axg_write_gravspec(root_c.encode(), 5, 7.25, a[0][1], a[1][1], _dp(de)[1], nb, 1.5, 0.75) == 0
    out.write_gravspec(root_p, 5, 7.25, w, pw, de, 1.5, 0.75)
    assert open(root_c + "_gravspec_5.dat").read() == open(root_p + "_gravspec_5.dat").read()

    sw_c, sw_p = str(tmp_path / "c_sw.txt"), str(tmp_path / "p_sw.txt")
    with open(sw_p, "w") as f:
        for idx in range(3):
            xi, ar, ve = (_values(rng, 3) for _ in range(3))
            assert lib.axg_append_string_wall_line(sw_c.encode(), idx, 2.5 + idx, -1e-5, _dp(xi)[1], _dp(ar)[1],
                                                   _dp(ve)[1]) == 0
            f.write(out.string_wall_line(idx, 2.5 + idx, -1e-5, xi, ar, ve) + "\n")
            assert lib.axg_append_crho_line((sw_c + ".crho").encode(), idx, *map(float, xi)) == 0
            with open(sw_p + ".crho", "a") as g:
                g.write(out.crho_line(idx, *map(float, xi)) + "\n")
            c1, c2 = np.abs(_values(rng, 2)), np.abs(_values(rng, 2))
            assert lib.axg_append_eps_line((sw_c + ".eps").encode(), idx, idx + 1, 1.0 + idx, 2.0 + idx, 0.3, 0.01,
                                           _dp(c1)[1], _dp(c2)[1]) == 0
            with open(sw_p + ".eps", "a") as g:
                g.write(out.eps_line(idx, idx + 1, 1.0 + idx, 2.0 + idx, 0.3, 0.01, c1, c2) + "\n")
    for suffix in ("", ".crho", ".eps"):
        assert open(sw_c + suffix).read() == open(sw_p + suffix).read()


def test_c_writers_report_errors(tmp_path, built):
    lib = ag.load_library()
    x, p = _dp(np.ones(2))
    AXG_ERR_ARG, AXG_ERR_IO = -1, -5  # include/axgpu.h
    assert lib.axg_write_spectrum(str(tmp_path / "no" / "such" / "dir").encode(), 1, p, p, p, p, 2) == AXG_ERR_IO
    assert lib.axg_write_covariance(None, 1, p, 2) == AXG_ERR_ARG
