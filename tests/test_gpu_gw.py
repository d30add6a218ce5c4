"""GPU gravitational-wave paths against the oracle (grav_waves.f90)."""
import numpy as np
import pytest

import axion_grav_gb300 as ag
from oracle import axo

pytestmark = pytest.mark.gpu


def params(n, precision, gw, **kw):
    base = dict(ngrid=n, precision=precision, gw_mode=gw, dspa=0.75, sigma_cr=1.0, kappa=0.1,
                tau_cr=1.0, a_now=1.0, num_bin_grav=25, gw_log_bins=12, seed=3)
    base.update(kw)
    return ag.default_params(**base)


def init_state(n, seed=1):
    p = params(n, ag.PREC_FP64_PLAIN, ag.GW_NONE, potential=ag.POT_QUARTIC)
    phi, _ = axo.ic_gaussian_flat(p, kcut=1.5, realisation=seed)
    rng = np.random.default_rng(seed)
    phid = (0.2 * (rng.standard_normal(phi.shape) + 1j * rng.standard_normal(phi.shape))).astype(np.complex128)
    return phi, phid


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("compat", [ag.COMPAT_REF, ag.COMPAT_INTENDED])
@pytest.mark.parametrize("precision", [ag.PREC_FP64_PLAIN, ag.PREC_FP64_FUSED])
def test_green_accumulators_and_spectrum(compat, precision):
    n = 32 if precision == ag.PREC_FP64_FUSED else 16
    phi, phid = init_state(n)
    p = params(n, precision, ag.GW_GREEN, compat=compat)
    acc = np.zeros((4, n, n, n), np.complex128)
    a_phi, a_phid = phi.copy(), phid.copy()
    nt = axo.symplectic_integration(p, a_phi, a_phid, None, None, acc, 2.0, 2.4, 0.4)
    w, pw, nu, de = axo.grav_spec_estimation(p, acc)
    with ag.Lattice(p) as lat:
        lat.upload(phi, phid)
        assert lat.symplectic_integration(2.0, 2.4, 0.4) == nt
        g_phi, _ = lat.download()
        g_acc = lat.download_gw_green()
        gw_, gpw, gnu, gde = lat.grav_spec_estimation(2.4)
    assert np.array_equal(g_phi, a_phi)  # the field evolution is unchanged by the GW integration
    assert rel(g_acc, acc) < 1e-10
    np.testing.assert_array_equal(gde, de)
    np.testing.assert_allclose(gw_, w, rtol=1e-15)
    np.testing.assert_allclose(gnu, nu, rtol=1e-9)
    np.testing.assert_allclose(gpw, pw, rtol=1e-9)


@pytest.mark.parametrize("compat", [ag.COMPAT_REF, ag.COMPAT_INTENDED])
@pytest.mark.parametrize("n", [16, 18])
def test_green_polarisation_table_matches_per_step_form(monkeypatch, compat, n):
    """FP64 Green accumulation with the precomputed polarisation table
    (conjugated for the k outside the stored half spectrum) and the
    float-float contraction agrees with the per-step FP64 form to ~1e-13."""
    phi, phid = init_state(n)
    p = params(n, ag.PREC_FP64_PLAIN, ag.GW_GREEN, compat=compat)
    out = {}
    for table in ("1", "0"):
        monkeypatch.setenv("AXG_GW_POL_TABLE", table)
        with ag.Lattice(p) as lat:
            lat.upload(phi, phid)
            lat.symplectic_integration(2.0, 2.4, 0.4)
            out[table] = lat.download_gw_green()
    monkeypatch.delenv("AXG_GW_POL_TABLE")
    assert np.any(out["1"] != 0)
    assert rel(out["1"], out["0"]) < 1e-12


@pytest.mark.parametrize("n", [16, 32, 64, 128])
def test_green_float_float_fft_matches_cufft(monkeypatch, n):
    """The FP64 Green path transforms its sources with the float-float D2Z
    for power-of-two N: its accumulators agree with the cuFFT FP64 path to
    about 1e-13 of their largest value."""
    phi, phid = init_state(n)
    p = params(n, ag.PREC_FP64_PLAIN, ag.GW_GREEN, compat=ag.COMPAT_INTENDED)
    out = {}
    for ff in ("1", "0"):
        monkeypatch.setenv("AXG_FFT_FF", ff)
        with ag.Lattice(p) as lat:
            lat.upload(phi, phid)
            lat.symplectic_integration(2.0, 2.4, 0.4)
            out[ff] = lat.download_gw_green()
    monkeypatch.delenv("AXG_FFT_FF")
    assert rel(out["1"], out["0"]) < 1e-12


@pytest.mark.parametrize("n", [16, 32, 64, 128, 256])
def test_green_fp32_fused_source_transform_matches_cufft(monkeypatch, n):
    """FP32-mixed Green mode forms the six sources inside its own row
    transform and runs the y and z passes in complex float for power-of-two
    N; its accumulators agree with the cuFFT R2C path to FP32 rounding."""
    phi, phid = init_state(n, 2)
    p = params(n, ag.PREC_FP32_MIXED, ag.GW_GREEN, compat=ag.COMPAT_REF)
    out = {}
    for ff in ("1", "0"):
        monkeypatch.setenv("AXG_FFT_FF", ff)
        with ag.Lattice(p) as lat:
            lat.upload(phi, phid)
            lat.set_kernel_timing(True)
            lat.symplectic_integration(2.0, 2.4, 0.4)
            lat.synchronize()
            names = set(k for k, _, _ in lat.kernel_timings())
            out[ff] = lat.download_gw_green()
        assert ("gw_source_rows_fp32" in names) == (ff == "1")
    monkeypatch.delenv("AXG_FFT_FF")
    assert np.any(out["1"] != 0)
    assert rel(out["1"], out["0"]) < 2e-5


@pytest.mark.parametrize("compat", [ag.COMPAT_REF, ag.COMPAT_INTENDED])
@pytest.mark.parametrize("n", [18, 32])
def test_green_fp32_mixed_against_fp64_oracle(compat, n):
    """FP32 sources, transforms (own passes at N = 32, cuFFT R2C at N = 18)
    and contractions with float-float accumulators: accumulators and the
    per-bin GW numerator against the FP64 oracle."""
    phi, phid = init_state(n, 4)
    p64 = params(n, ag.PREC_FP64_PLAIN, ag.GW_GREEN, compat=compat)
    acc = np.zeros((4, n, n, n), np.complex128)
    nt = axo.symplectic_integration(p64, phi.copy(), phid.copy(), None, None, acc, 2.0, 2.8, 0.4)
    w, pw, nu, de = axo.grav_spec_estimation(p64, acc)
    with ag.Lattice(params(n, ag.PREC_FP32_MIXED, ag.GW_GREEN, compat=compat)) as lat:
        lat.upload(phi, phid)
        assert lat.symplectic_integration(2.0, 2.8, 0.4) == nt
        g_acc = lat.download_gw_green()
        gw_, gpw, gnu, gde = lat.grav_spec_estimation(2.8)
    assert rel(g_acc, acc) < 1e-4
    np.testing.assert_array_equal(gde, de)
    np.testing.assert_allclose(gnu, nu, rtol=1e-3)
    np.testing.assert_allclose(gpw, pw, rtol=1e-3)


@pytest.mark.parametrize("compat", [ag.COMPAT_REF, ag.COMPAT_INTENDED])
@pytest.mark.parametrize("precision,n,deg", [
    (ag.PREC_FP64_PLAIN, 32, 1),   # GW grid 16^3: float-float D2Z of the stored sources
    (ag.PREC_FP64_PLAIN, 32, 2),   # 8^3: cuFFT D2Z
    (ag.PREC_FP64_FUSED, 64, 1),   # 32^3
    (ag.PREC_FP64_PLAIN, 24, 1),   # 12^3: cuFFT, N not a power of two
    (ag.PREC_FP32_MIXED, 32, 1),
    (ag.PREC_FP32_MIXED, 64, 2),
])
def test_green_degraded_against_oracle(compat, precision, n, deg):
    """degrade_spec > 0: the sources are the deg^3-box-summed central
    differences of data1_to_arr_dphi_degrade (grav_waves.f90:358-415) and
    the accumulation, polarisation, bins and normalisation run on the GW
    grid ngrid / deg of spacing dx deg (grav_waves.f90:37-45, 62-71).
    FP64 paths: accumulators within 1e-10 of the oracle, counts exact;
    FP32-mixed: accumulators within 1e-4, numerator and power 1e-3 per bin."""
    phi, phid = init_state(n, 5)
    p64 = params(n, ag.PREC_FP64_PLAIN, ag.GW_GREEN, compat=compat, degrade_spec=deg)
    acc = axo.green_acc_zeros(p64)
    assert acc.shape == (4, n >> deg, n >> deg, n >> deg)
    a_phi = phi.copy()
    nt = axo.symplectic_integration(p64, a_phi, phid.copy(), None, None, acc, 2.0, 2.8, 0.4)
    w, pw, nu, de = axo.grav_spec_estimation(p64, acc)
    e, lpw, lnu, lde = axo.grav_spec_log_green(p64, acc)
    with ag.Lattice(params(n, precision, ag.GW_GREEN, compat=compat, degrade_spec=deg)) as lat:
        lat.upload(phi, phid)
        assert lat.symplectic_integration(2.0, 2.8, 0.4) == nt
        g_phi, _ = lat.download()
        g_acc = lat.download_gw_green()
        gw_, gpw, gnu, gde = lat.grav_spec_estimation(2.8)
        ge, glpw, glnu, glde = lat.grav_spec_log(2.8)
    assert np.any(acc != 0)
    fp64 = precision != ag.PREC_FP32_MIXED
    if fp64:
        assert np.array_equal(g_phi, a_phi)
    assert rel(g_acc, acc) < (1e-10 if fp64 else 1e-4)
    np.testing.assert_array_equal(gde, de)
    np.testing.assert_array_equal(glde, lde)
    np.testing.assert_allclose(gw_, w, rtol=1e-15)
    np.testing.assert_allclose(ge, e, rtol=1e-14)
    tol = 1e-9 if fp64 else 1e-3
    np.testing.assert_allclose(gnu, nu, rtol=tol)
    np.testing.assert_allclose(gpw, pw, rtol=tol)
    np.testing.assert_allclose(glnu, lnu, rtol=tol)


@pytest.mark.parametrize("precision,n", [(ag.PREC_FP64_PLAIN, 16), (ag.PREC_FP64_PLAIN, 18),
                                         (ag.PREC_FP32_MIXED, 16)])
def test_green_accumulator_upload_download(precision, n):
    """The device keeps the stored half spectrum and the Nyquist-row mirrors;
    a conjugate-symmetric host array (the form the accumulation produces)
    goes up and comes back unchanged, to the float-float precision."""
    rng = np.random.default_rng(9)
    acc = rng.standard_normal((4, n, n, n)) + 1j * rng.standard_normal((4, n, n, n))
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    other = (x > n // 2) & (y != n // 2) & (z != n // 2)  # sites whose entry is a conjugate
    acc[:, other] = np.conj(acc[:, (n - z[other]) % n, (n - y[other]) % n, (n - x[other]) % n])
    with ag.Lattice(params(n, precision, ag.GW_GREEN)) as lat:
        lat.upload_gw_green(acc)
        back = lat.download_gw_green()
    assert rel(back, acc) < 1e-14


def test_green_log_bins():
    n = 16
    phi, phid = init_state(n, 2)
    p = params(n, ag.PREC_FP64_PLAIN, ag.GW_GREEN)
    acc = np.zeros((4, n, n, n), np.complex128)
    axo.symplectic_integration(p, phi.copy(), phid.copy(), None, None, acc, 2.0, 2.2, 0.4)
    e, pw, nu, de = axo.grav_spec_log_green(p, acc)
    with ag.Lattice(p) as lat:
        lat.upload(phi, phid)
        lat.symplectic_integration(2.0, 2.2, 0.4)
        ge, gpw, gnu, gde = lat.grav_spec_log(2.2)
    np.testing.assert_allclose(ge, e, rtol=1e-14)
    np.testing.assert_array_equal(gde, de)
    np.testing.assert_allclose(gnu, nu, rtol=1e-9)
    assert de.sum() == n ** 3 - 1 - np.sum(de == 0) * 0 or de.sum() > 0


@pytest.mark.parametrize("precision,tol", [(ag.PREC_FP64_PLAIN, 1e-9), (ag.PREC_FP32_MIXED, 2e-3)])
def test_uij_tt_spectrum(precision, tol):
    n = 32
    phi, phid = init_state(n, 4)
    p64 = params(n, ag.PREC_FP64_PLAIN, ag.GW_UIJ)
    u = np.zeros((6, n, n, n))
    ud = np.zeros((6, n, n, n))
    a = [phi.copy(), phid.copy(), u.copy(), ud.copy()]
    axo.symplectic_integration(p64, a[0], a[1], a[2], a[3], None, 2.0, 2.6, 0.4)
    w, pw, nu, de = axo.uij_grav_spec(p64, a[2], a[3], 2.6)
    e, lpw, lnu, lde = axo.uij_grav_spec_log(p64, a[2], a[3], 2.6)
    with ag.Lattice(params(n, precision, ag.GW_UIJ)) as lat:
        lat.upload(phi, phid)
        lat.upload_uij(u, ud)
        lat.symplectic_integration(2.0, 2.6, 0.4)
        gw_, gpw, gnu, gde = lat.grav_spec_estimation(2.6)
        ge, glpw, glnu, glde = lat.grav_spec_log(2.6)
    np.testing.assert_array_equal(gde, de)
    np.testing.assert_array_equal(glde, lde)
    np.testing.assert_allclose(gnu, nu, rtol=tol)
    np.testing.assert_allclose(glnu, lnu, rtol=tol)
    np.testing.assert_allclose(gpw, pw, rtol=tol)


@pytest.mark.parametrize("precision,tol", [(ag.PREC_FP64_PLAIN, 1e-12), (ag.PREC_FP32_MIXED, 2e-5)])
@pytest.mark.parametrize("n", [16, 64, 256])
def test_uij_spectrum_own_transforms_match_cufft(monkeypatch, precision, tol, n):
    """For power-of-two N the u_ij spectrum forms its twelve fields inside its
    own row transforms (complex float, or float-float for FP64); against the
    prepare pass + cuFFT path (AXG_FFT_FF=0) the binned numerator agrees to
    the transform precision."""
    phi, phid = init_state(n, 5)
    rng = np.random.default_rng(n)
    u, ud = 0.1 * rng.standard_normal((6, n, n, n)), 0.1 * rng.standard_normal((6, n, n, n))
    out = {}
    for ff in ("1", "0"):
        monkeypatch.setenv("AXG_FFT_FF", ff)
        with ag.Lattice(params(n, precision, ag.GW_UIJ)) as lat:
            lat.upload(phi, phid)
            lat.upload_uij(u, ud)
            lat.set_kernel_timing(True)
            out[ff] = lat.grav_spec_estimation(2.6)
            lat.synchronize()
            names = set(k for k, _, _ in lat.kernel_timings())
        own = any(k.startswith("uij_rows") for k in names)
        assert own == (ff == "1")
    monkeypatch.delenv("AXG_FFT_FF")
    np.testing.assert_array_equal(out["1"][3], out["0"][3])
    np.testing.assert_allclose(out["1"][2], out["0"][2], rtol=tol)


@pytest.mark.parametrize("precision,rs", [(ag.PREC_FP64_PLAIN, 8), (ag.PREC_FP32_MIXED, 4)])
def test_own_transforms_store_no_real_fields(monkeypatch, precision, rs):
    """With the library's own transforms the Green sources and the u_ij
    spectrum's twelve fields are formed inside the row passes: against the
    cuFFT path the context holds their real buffers less (6 fields of N^3
    reals for the Green sources; one field for the u_ij spectrum, whose
    cuFFT path transforms the twelve through one real buffer), and only a
    twiddle table more.  The complex-float half spectra of the own
    transforms have kx rows padded to a multiple of 4 entries."""
    n = 64
    mem = {}
    for ff in ("1", "0"):
        monkeypatch.setenv("AXG_FFT_FF", ff)
        with ag.Lattice(params(n, precision, ag.GW_GREEN)) as lat:
            mem[("green", ff)] = lat.memory_bytes()
        with ag.Lattice(params(n, precision, ag.GW_UIJ)) as lat:
            lat.ic_gaussian_flat(1.0)
            lat.grav_spec_estimation(2.0)
            mem[("uij", ff)] = lat.memory_bytes()
    monkeypatch.delenv("AXG_FFT_FF")
    tw = n // 2 * 16  # the own transforms' float-float twiddle table
    nh = n // 2 + 1
    pad = 0 if rs == 8 else n * n * (((nh + 3) & ~3) - nh) * 2 * rs  # per field
    assert mem[("green", "0")] - mem[("green", "1")] >= 6 * n ** 3 * rs - tw - 6 * pad
    assert mem[("uij", "0")] - mem[("uij", "1")] >= n ** 3 * rs - tw - 12 * pad


def test_green_requires_mode():
    with ag.Lattice(params(16, ag.PREC_FP64_PLAIN, ag.GW_NONE)) as lat:
        with pytest.raises(ag.AxgError):
            lat.grav_spec_estimation(1.0)


def _modes_on_gpu(n, precision, phi0, L=32.0):
    dt, steps = 0.1 * 32 / n, 100 * n // 32  # dt in proportion to dx
    kw = dict(ngrid=n, precision=precision, potential=ag.POT_QUARTIC, dspa=L / n, sigma_cr=0.05, kappa=0.1,
              compat=ag.COMPAT_INTENDED, num_bin_grav=25 * n // 32, **{"lambda": 1.0})
    out = []
    for gw in (ag.GW_GREEN, ag.GW_UIJ):
        with ag.Lattice(ag.default_params(gw_mode=gw, **kw)) as lat:
            lat.upload(phi0, np.zeros_like(phi0))
            if gw == ag.GW_UIJ:
                z = np.zeros((6, n, n, n))
                lat.upload_uij(z, z)
            lat.leapfrog(1.0, dt, steps, True, True)
            out.append(lat.grav_spec_estimation(1.0 + steps * dt)[2])
    return tuple(out)


def test_mode_u_converges_to_mode_g_on_the_gpu():
    """Mode U (u_ij leapfrog + TT spectrum) against Mode G (the reference's
    Green's-function method, grav_waves.f90:193-321) through the C-ABI, the
    same band-limited field in one box at dx = 1, 1/2, 1/4 (dt = dx / 10):
    the band-integrated difference of their numerators falls at second order
    (a factor 4 expected per halving) and is below 3 % at dx = 1.  The
    FP32-mixed paths show the same difference at dx = 1/2 to 2e-3."""
    import gw_crosscheck
    ns = (32, 64, 128)
    fields = gw_crosscheck.band_limited_fields(list(ns))
    spectra = [_modes_on_gpu(n, ag.PREC_FP64_PLAIN, f) for n, f in zip(ns, fields)]
    e = gw_crosscheck.mode_u_vs_g(spectra)
    assert e[0] < 0.03
    assert e[1] < e[0] / 3 and e[2] < e[1] / 3, e
    e32 = gw_crosscheck.mode_u_vs_g([_modes_on_gpu(64, ag.PREC_FP32_MIXED, fields[1])])[0]
    assert abs(e32 - e[1]) < 2e-3, (e32, e[1])
