"""GPU field spectrum (spectrum.f90) against the oracle."""
import numpy as np
import pytest

import axion_grav_gb300 as ag
from oracle import axo

pytestmark = pytest.mark.gpu


def params(n, precision=ag.PREC_FP64_PLAIN, **kw):
    base = dict(ngrid=n, precision=precision, dspa=0.5, num_bin=8, degrade_spec=0, flags=7, seed=2)
    base.update(kw)
    return ag.default_params(**base)


def state(n, seed=0):
    p = params(n, potential=ag.POT_QUARTIC)
    phi, _ = axo.ic_gaussian_flat(p, kcut=2.0, realisation=seed)
    rng = np.random.default_rng(seed)
    phid = (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))).astype(np.complex128)
    return phi, phid


@pytest.mark.parametrize("n,deg", [(16, 0), (32, 0), (32, 1)])
@pytest.mark.parametrize("precision", [ag.PREC_FP64_PLAIN, ag.PREC_FP32_MIXED])
def test_spectrum_estimation_matches_oracle(n, deg, precision):
    phi, phid = state(n, n + deg)
    if precision == ag.PREC_FP32_MIXED:
        phi = phi.astype(np.complex64).astype(np.complex128)
        phid = phid.astype(np.complex64).astype(np.complex128)
    p = params(n, precision, degrade_spec=deg)
    flags, cnt = axo.classify_cells(params(n), phi, 7, 0)
    w, pw, cv, ct, md = axo.spectrum_estimation(params(n, degrade_spec=deg), phid, flags, 3.0)
    with ag.Lattice(p) as lat:
        lat.upload(phi, phid)
        assert np.array_equal(lat.classify_cells(7), cnt)
        gw, gpw, gcv, gct = lat.spectrum_estimation(3.0)
        rho = lat.compute_crho()
    np.testing.assert_array_equal(gct, ct)
    np.testing.assert_allclose(gw, w, rtol=1e-15)
    np.testing.assert_allclose(gcv, cv, rtol=1e-10)
    np.testing.assert_allclose(gpw, pw, rtol=1e-8, atol=1e-10 * np.max(np.abs(pw)))
    wav = np.concatenate([[0.0], np.cumsum(np.full(len(w), w[0] * 2))])
    assert rho == pytest.approx(axo.compute_crho(params(n, degrade_spec=deg), wav, pw), rel=1e-6)


def test_spectrum_classifies_when_needed():
    n = 16
    phi, phid = state(n, 5)
    with ag.Lattice(params(n)) as lat:
        lat.upload(phi, phid)
        w, pw, cv, ct = lat.spectrum_estimation(2.0)
    assert np.all(np.isfinite(pw)) and ct.sum() > 0


@pytest.mark.parametrize("n,deg", [(32, 0), (32, 1)])
def test_spectrum_covariance_matches_oracle(n, deg):
    """estimate_covmat (spectrum.f90:569-734) with a fixed number of MC
    realisations; the same Philox draws on both sides."""
    phi, phid = state(n, 40 + deg)
    p = params(n, degrade_spec=deg)
    flags, cnt = axo.classify_cells(params(n), phi, 7, 0)
    w, pw, cv, ct, md = axo.spectrum_estimation(p, phid, flags, 3.0)
    cov, it = axo.estimate_covmat(p, flags, pw, axo.mat_divided(md, ct), 6, 6, 0.05)
    wav = np.concatenate([[0.0], np.cumsum(np.full(len(w), w[0] * 2))])
    rho, drho = axo.compute_crho_cov(p, wav, pw, cov)
    with ag.Lattice(p) as lat:
        lat.upload(phi, phid)
        lat.classify_cells(7)
        lat.spectrum_estimation(3.0)
        gcov, git = lat.spectrum_covariance(6, 6, 0.05)
        grho, gdrho = lat.compute_crho_cov()
    assert git == it
    scale = np.max(np.abs(cov))
    np.testing.assert_allclose(gcov, cov, rtol=1e-7, atol=1e-9 * scale)
    assert grho == pytest.approx(rho, rel=1e-6)
    assert gdrho == pytest.approx(drho, rel=1e-6)


@pytest.mark.parametrize("n,deg", [(64, 0), (64, 1)])
def test_float_float_transforms_match_cufft(monkeypatch, n, deg):
    """Window D2Z, field Z2Z and the covariance's forward / inverse Z2Z run
    in float-float for power-of-two sizes: spectrum and covariance agree with
    the cuFFT FP64 transforms to ~1e-12."""
    phi, phid = state(n, 7 + deg)
    p = params(n, degrade_spec=deg)
    out = {}
    for ff in ("1", "0"):
        monkeypatch.setenv("AXG_FFT_FF", ff)
        with ag.Lattice(p) as lat:
            lat.upload(phi, phid)
            lat.classify_cells(7)
            w, pw, cv, ct = lat.spectrum_estimation(3.0)
            cov, it = lat.spectrum_covariance(4, 4, 0.05)
            out[ff] = (pw, cv, ct, cov, it)
    monkeypatch.delenv("AXG_FFT_FF")
    a, b = out["1"], out["0"]
    np.testing.assert_array_equal(a[2], b[2])
    np.testing.assert_allclose(a[1], b[1], rtol=1e-12)
    np.testing.assert_allclose(a[0], b[0], rtol=1e-10, atol=1e-12 * np.max(np.abs(b[0])))
    assert a[4] == b[4]
    np.testing.assert_allclose(a[3], b[3], rtol=1e-8, atol=1e-10 * np.max(np.abs(b[3])))
