"""The CUDA paths against the committed golden fixtures (tests/golden/,
oracle outputs on seeded inputs): FP64 evolution and defect fits bit for
bit, transforms and reductions within their stated tolerances."""
import os

import numpy as np
import pytest

import axion_grav_gb300 as ag

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
LEAPFROG = dict(t1=1.5, dt=0.02, nsteps=6)
GREEN = dict(t1=2.0, t2=2.4, eps=0.4)


def load(name):
    return dict(np.load(os.path.join(HERE, name + ".npz")))


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("case", ["leapfrog_uij_ref_6", "leapfrog_uij_quartic_6"])
@pytest.mark.parametrize("precision", [ag.PREC_FP64_PLAIN, ag.PREC_FP64_FUSED, ag.PREC_FP32_MIXED])
def test_leapfrog_against_golden(case, precision):
    d = load(case)
    n = d["phi0"].shape[0]
    p = ag.default_params(ngrid=n, precision=precision, gw_mode=ag.GW_UIJ, potential=int(d["potential"]),
                          dspa=0.5, sigma_cr=1.0, kappa=0.1, seed=11)
    with ag.Lattice(p) as lat:
        lat.upload(d["phi0"], d["phid0"])
        lat.upload_uij(d["u0"], d["ud0"])
        lat.leapfrog(LEAPFROG["t1"], LEAPFROG["dt"], LEAPFROG["nsteps"], True, True)
        phi, phid = lat.download()
        u, ud = lat.download_uij()
    if precision == ag.PREC_FP32_MIXED:
        assert rel(phi, d["phi"]) < 2e-5 and rel(phid, d["phid"]) < 2e-4
        assert rel(u, d["u"]) < 2e-3 and rel(ud, d["ud"]) < 2e-3
    else:
        for a, k in ((phi, "phi"), (phid, "phid"), (u, "u"), (ud, "ud")):
            assert np.array_equal(a, d[k]), k


def test_defects_against_golden():
    d = load("defects_8")
    n = d["phi"].shape[0]
    p = ag.default_params(ngrid=n, precision=ag.PREC_FP64_PLAIN, flags=7, dspa=1.0, sigma_cr=1.0, kappa=0.1, seed=5)
    with ag.Lattice(p) as lat:
        lat.upload(d["phi"], d["phid"])
        sl, wa, sv, cnt = lat.id_defects(1, 4.0)
        S, W = lat.defect_lists(int(cnt[0]), int(cnt[1]))
        flags = lat.defect_flags()
    assert np.array_equal(cnt, d["counts"])
    assert np.array_equal(flags, d["flags"])
    cols = [c for c in range(13) if c != 9]
    assert np.array_equal(S[:, cols], d["strings"][:, cols])
    np.testing.assert_allclose(S[:, 9], d["strings"][:, 9], rtol=1e-14)
    wcols = [0, 1, 2, 3, 4, 5, 7, 8]
    assert np.array_equal(W[:, wcols], d["walls"][:, wcols])
    for a, k in ((sl, "sl"), (wa, "wa"), (sv, "sv")):
        np.testing.assert_allclose(a, d[k], rtol=1e-12)


@pytest.mark.parametrize("case", ["green_ref_8", "green_intended_8", "green_degrade1_ref_16"])
def test_green_against_golden(case):
    d = load(case)
    n = d["phi0"].shape[0]
    p = ag.default_params(ngrid=n, precision=ag.PREC_FP64_PLAIN, gw_mode=ag.GW_GREEN, dspa=0.75, sigma_cr=1.0,
                          kappa=0.1, tau_cr=1.0, a_now=1.0, num_bin_grav=25, gw_log_bins=12, seed=3,
                          potential=ag.POT_QUARTIC, compat=int(d["compat"]), degrade_spec=int(d["degrade_spec"]))
    with ag.Lattice(p) as lat:
        lat.upload(d["phi0"], d["phid0"])
        assert lat.symplectic_integration(GREEN["t1"], GREEN["t2"], GREEN["eps"]) == int(d["nt"])
        phi, _ = lat.download()
        acc = lat.download_gw_green()
        w, pw, nu, de = lat.grav_spec_estimation(GREEN["t2"])
    assert np.array_equal(phi, d["phi"])
    assert rel(acc, d["acc"]) < 1e-10
    np.testing.assert_array_equal(de, d["denom"])
    np.testing.assert_allclose(w, d["wave"], rtol=1e-15)
    np.testing.assert_allclose(nu, d["numer"], rtol=1e-9)
    np.testing.assert_allclose(pw, d["power"], rtol=1e-9)


def test_spectrum_against_golden():
    d = load("spectrum_16")
    n = d["phid"].shape[0]
    p = ag.default_params(ngrid=n, precision=ag.PREC_FP64_PLAIN, flags=0, dspa=1.0, sigma_cr=1.0, kappa=0.1,
                          seed=7, num_bin=8)
    with ag.Lattice(p) as lat:
        lat.upload(np.ones((n, n, n), np.complex128), d["phid"])
        w, pw, cv, ct = lat.spectrum_estimation(3.0)
    np.testing.assert_array_equal(ct, d["count"])
    np.testing.assert_allclose(w, d["wave"], rtol=1e-15)
    np.testing.assert_allclose(cv, d["conv"], rtol=1e-10)
    np.testing.assert_allclose(pw, d["power"], rtol=1e-8, atol=1e-10 * np.max(np.abs(d["power"])))
