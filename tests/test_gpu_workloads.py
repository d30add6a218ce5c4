"""The plain-method workload run end to end through the C-ABI against the
oracle: a 128^3 FP64 lattice of phi and six u_ij from a seeded Gaussian-flat
field, lambda = v = m_r = 1, dx = 1 / m_r, dt = 0.2 dx, a ~ tau, evolved in
intervals of 20 leapfrog steps (each interval drift-kick-drift, as
symplectic_integration between output times, evolve.f90:98-152, 238-257) to
tau ~ L / 2, with the string plaquette-winding count after every interval
and the field spectrum (spectrum.f90:242-342, masked by the classification)
and the 64-log-bin GW spectrum at the end."""
import numpy as np
import pytest

import axion_grav_gb300 as ag
from oracle import axo

pytestmark = pytest.mark.gpu


def plain_workload(n, precision):
    # V = lambda / 4 (|phi|^2 - v^2)^2 with lambda = v = 1, dx = 1 = 1 / m_r,
    # m_r = sqrt(lambda) v.  sigma_cr = 0.005 keeps dt = 0.2 dx inside the
    # leapfrog's stability limit up to tau ~ 500 (the comoving mass grows as tau sigma_cr).
    return ag.default_params(ngrid=n, precision=precision, gw_mode=ag.GW_UIJ, potential=ag.POT_QUARTIC, dspa=1.0,
                             sigma_cr=0.005, vev=1.0, n_dw=1, ma2_0=0.0, seed=1, num_bin=50, gw_log_bins=64,
                             flags=7, **{"lambda": 1.0})


@pytest.mark.parametrize("precision", [ag.PREC_FP64_PLAIN, ag.PREC_FP64_FUSED])
def test_plain_method_workload_128(precision):
    n, dt, interval, nint, t0 = 128, 0.2, 20, 16, 1.0  # 320 steps: tau 1 -> 65 = L / 2 + 1
    p = plain_workload(n, precision)
    p64 = plain_workload(n, ag.PREC_FP64_PLAIN)
    phi, phid = axo.ic_gaussian_flat(p64, kcut=1.0)
    u, ud = np.zeros((6, n, n, n)), np.zeros((6, n, n, n))
    got_wind, want_wind = [], []
    with ag.Lattice(p) as lat:
        lat.upload(phi, phid)
        lat.upload_uij(u, ud)
        t = t0
        for k in range(nint):
            lat.leapfrog(t, dt, interval, True, True)
            axo.leapfrog(p64, phi, phid, u, ud, None, t, dt, interval, True, True)
            t += dt * interval
            got_wind.append(lat.string_winding())
            want_wind.append(axo.string_winding(p64, phi))
        g_phi, g_phid = lat.download()
        counts = lat.classify_cells(7)
        fw, fpw, fcv, fct = lat.spectrum_estimation(t)
        ge, gpw, gnu, gde = lat.grav_spec_log(t)
    # the evolution is bit-exact, so every winding count is
    assert np.array_equal(g_phi, phi) and np.array_equal(g_phid, phid)
    assert np.array_equal(np.array(got_wind), np.array(want_wind))
    assert np.array(want_wind)[0].sum() > 0
    flags, wcounts = axo.classify_cells(p64, phi, 7, 0)
    assert np.array_equal(counts, wcounts)
    w, pw, cv, ct, _ = axo.spectrum_estimation(p64, phid, flags, t)
    np.testing.assert_array_equal(fct, ct)
    np.testing.assert_allclose(fcv, cv, rtol=1e-10)
    np.testing.assert_allclose(fpw, pw, rtol=1e-8, atol=1e-10 * np.max(np.abs(pw)))
    e, lpw, lnu, lde = axo.uij_grav_spec_log(p64, u, ud, t)
    np.testing.assert_allclose(ge, e, rtol=1e-14)
    np.testing.assert_array_equal(gde, lde)
    np.testing.assert_allclose(gnu, lnu, rtol=1e-9, atol=1e-12 * np.max(lnu))
    assert np.max(lnu) > 0
