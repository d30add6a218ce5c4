"""The workloads at their full sizes: 512^3 (FP64-plain and FP32-mixed),
1024^3 FP32-mixed with the axion term switched on mid-run, the 96-member
ensemble of 64^3..192^3 lattices, and the 256^3 adjoint.  Where the oracle
finishes in seconds (OpenMP) the GPU is compared with it directly, bit for
bit; otherwise through size-independent properties: time-reversibility of
the damped leapfrog, bit-identity between GPU paths, finite differences."""
import os

import numpy as np
import pytest

import axion_grav_gb300 as ag
from oracle import axo

pytestmark = pytest.mark.gpu


def _host_gib():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) / 2 ** 20
    except OSError:
        pass
    return 0.0


def _device_gib():
    import torch

    free, _ = torch.cuda.mem_get_info()
    return free / 2 ** 30


def workload(n, precision, gw):
    # the 512^3 benchmark lattice: reference potential, dx = 32 / N, kappa 0.1
    return ag.default_params(ngrid=n, precision=precision, gw_mode=gw, potential=ag.POT_REFERENCE, dspa=32.0 / n,
                             sigma_cr=1.0, kappa=0.1, seed=1)


def quartic(n, precision, gw, n_dw=2, tau_on=11.0):
    # lambda = v = m_r = 1, dx = 1 / m_r; m_a^2 = 1e-3 (tau / tau_on)^2 from tau_on on.
    # sigma_cr = 0.005 keeps dt = 0.2 inside the leapfrog's stability limit
    # (dt^2 (12/dx^2 + 6 tau^2 sigma_cr^2) < 4) up to tau ~ 500.
    return ag.default_params(ngrid=n, precision=precision, gw_mode=gw, potential=ag.POT_QUARTIC, dspa=1.0,
                             sigma_cr=0.005, vev=1.0, n_dw=n_dw, ma2_0=1e-3, tau_axion_on=tau_on, ma2_power=2.0,
                             seed=1, **{"lambda": 1.0})


def _gpu_run(p, phi, phid, u, ud, t1, dt, nsteps):
    with ag.Lattice(p) as lat:
        lat.upload(phi, phid)
        if u is not None:
            lat.upload_uij(u, ud)
        lat.leapfrog(t1, dt, nsteps, True, True)
        out = lat.download()
        ou = lat.download_uij() if u is not None else (None, None)
    return out[0], out[1], ou[0], ou[1]


@pytest.mark.parametrize("n,gw", [(512, ag.GW_NONE), (256, ag.GW_UIJ)])
def test_fp64_paths_match_oracle_at_full_size(n, gw):
    """FP64-plain (separate kick and drift) and FP64-fused (TMA kernel) equal
    the oracle bit for bit on the benchmark lattice."""
    if _host_gib() < 24:
        pytest.skip("needs ~24 GiB of host memory")
    p = workload(n, ag.PREC_FP64_PLAIN, gw)
    with ag.Lattice(p) as lat:
        lat.ic_gaussian_flat(kcut=2.0 * np.pi / (8 * p.dspa))
        phi0, phid0 = lat.download()
    rng = np.random.default_rng(11)
    phid0 = phid0 + 0.05 * (rng.standard_normal(phi0.shape) + 1j * rng.standard_normal(phi0.shape))
    u0 = 0.01 * rng.standard_normal((6, n, n, n)) if gw else None
    ud0 = 0.01 * rng.standard_normal((6, n, n, n)) if gw else None
    t1, dt, nsteps = 2.0, 0.25 * p.dspa, 3
    ref = [phi0.copy(), phid0.copy(), None if u0 is None else u0.copy(), None if ud0 is None else ud0.copy()]
    axo.leapfrog(p, ref[0], ref[1], ref[2], ref[3], None, t1, dt, nsteps, True, True)
    for prec in (ag.PREC_FP64_PLAIN, ag.PREC_FP64_FUSED):
        got = _gpu_run(workload(n, prec, gw), phi0, phid0, u0, ud0, t1, dt, nsteps)
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1]), prec
        if gw:
            assert np.array_equal(got[2], ref[2]) and np.array_equal(got[3], ref[3]), prec
        del got


def _max_abs_diff(a, b, chunk=1 << 26):
    fa, fb = a.reshape(-1), b.reshape(-1)
    m = 0.0
    for s in range(0, fa.size, chunk):
        m = max(m, float(np.max(np.abs(fa[s:s + chunk] - fb[s:s + chunk]))))
    return m


def _max_abs(a, chunk=1 << 26):
    fa = a.reshape(-1)
    return max(float(np.max(np.abs(fa[s:s + chunk]))) for s in range(0, fa.size, chunk))


def _reversibility(n, precision, nsteps, t1=10.0, dt=0.2):
    p = quartic(n, precision, ag.GW_UIJ)
    with ag.Lattice(p) as lat:
        lat.ic_gaussian_flat(kcut=1.0)
        phi0, _ = lat.download(phidot=False)
        lat.leapfrog(t1, dt, nsteps, True, True)
        t2 = t1 + nsteps * dt
        _, phid_mid = lat.download(phi=False)
        pd_scale = _max_abs(phid_mid)
        del phid_mid
        lat.leapfrog(t2, -dt, nsteps, True, True)
        phi1, _ = lat.download(phidot=False)
        err_phi = _max_abs_diff(phi1, phi0) / _max_abs(phi0)
        del phi1
        _, phid1 = lat.download(phi=False)
        err_pd = _max_abs(phid1) / pd_scale
    return err_phi, err_pd


@pytest.mark.parametrize("precision,tol", [(ag.PREC_FP64_PLAIN, 1e-12), (ag.PREC_FP32_MIXED, 2e-5)])
def test_leapfrog_time_reversible_small(precision, tol):
    """Forward nsteps then backward nsteps from t2 with -dt returns to the
    initial state (the axion term switches on between t1 and t2)."""
    err_phi, err_pd = _reversibility(64, precision, 10)
    assert err_phi < tol and err_pd < 10 * tol


def test_fp32_1024_time_reversible_with_axion_term():
    """1024^3 FP32-mixed, phi and six u_ij, N_DW = 2 axion term switched on
    mid-run: the full-size lattice returns to its initial state."""
    if _host_gib() < 48 or _device_gib() < 160:
        pytest.skip("needs ~160 GiB of device and ~48 GiB of host memory")
    err_phi, err_pd = _reversibility(1024, ag.PREC_FP32_MIXED, 10)
    assert err_phi < 2e-5 and err_pd < 2e-4


def test_full_ensemble_members_match_single_runs():
    """The 96-member ensemble (32 x 64^3, 32 x 128^3, 24 x 160^3, 8 x 192^3)
    in one persistent launch per step: the last member of each size equals
    its own single-lattice run bit for bit."""
    sizes = [(64, 32), (128, 32), (160, 24), (192, 8)]
    ps = []
    for n, cnt in sizes:
        for _ in range(cnt):
            ps.append(ag.default_params(ngrid=n, precision=ag.PREC_FP32_MIXED, gw_mode=ag.GW_UIJ,
                                        potential=ag.POT_REFERENCE, dspa=0.5, sigma_cr=1.0, kappa=0.1,
                                        seed=1 + len(ps)))
    dt, t0, nsteps = 0.05, 2.0, 6
    check = np.cumsum([c for _, c in sizes]) - 1
    with ag.Ensemble(ps) as ens:
        for i, m in enumerate(ens.members):
            m.ic_gaussian_flat(2.0 * np.pi / (8 * 0.5), i)
        ens.leapfrog(t0, dt, nsteps, True, True, use_graph=True)
        ens.leapfrog(t0 + dt * nsteps, dt, nsteps, True, True, use_graph=True)
        got = {int(i): (ens.members[i].download(), ens.members[i].download_uij()) for i in check}
    for i in check:
        with ag.Lattice(ps[i]) as lat:
            lat.ic_gaussian_flat(2.0 * np.pi / (8 * 0.5), int(i))
            lat.leapfrog(t0, dt, nsteps, True, True)
            lat.leapfrog(t0 + dt * nsteps, dt, nsteps, True, True)
            (phi, phid), (u, ud) = lat.download(), lat.download_uij()
        (gphi, gphid), (gu, gud) = got[int(i)]
        assert np.array_equal(gphi, phi) and np.array_equal(gphid, phid), i
        assert np.array_equal(gu, u) and np.array_equal(gud, ud), i


def _adjoint_256(lam, steps, stride, state=None):
    n = 256
    p = quartic(n, ag.PREC_FP64_PLAIN, ag.GW_UIJ, tau_on=1e9)
    p.update(**{"lambda": lam})
    with ag.Lattice(p) as lat:
        if state is None:
            lat.ic_gaussian_flat(kcut=1.0)
        else:
            lat.upload(state[0], state[1])
        return lat.adjoint_gw_band(1.0, 0.2, steps, stride, 0.125, 0.5, want_grads=state is not None)


def test_adjoint_256_lambda_against_finite_differences():
    """The 256^3 gradient case (J over k in [m_r/8, m_r/2], checkpoint stride
    64): dJ/dlambda against central differences."""
    eps = 1e-4
    J, dl, *_ = _adjoint_256(1.0, 128, 64)
    Jp = _adjoint_256(1.0 + eps, 128, 64)[0]
    Jm = _adjoint_256(1.0 - eps, 128, 64)[0]
    assert J > 0
    assert dl == pytest.approx((Jp - Jm) / (2 * eps), rel=1e-5)


def test_adjoint_256_dot_product_against_tangent_linear():
    """<dJ/dphi0, dphi> + <dJ/dphi'0, dphi'> + dJ/dlambda dlambda equals the
    FP64 tangent-linear oracle's directional derivative at 256^3."""
    if _host_gib() < 16:
        pytest.skip("needs ~16 GiB of host memory")
    n, steps = 256, 32
    p = quartic(n, ag.PREC_FP64_PLAIN, ag.GW_UIJ, tau_on=1e9)
    with ag.Lattice(p) as lat:
        lat.ic_gaussian_flat(kcut=1.0)
        phi0, phid0 = lat.download()
    J, dl, gphi, gpid, _, _ = _adjoint_256(1.0, steps, 8, (phi0, phid0))
    rng = np.random.default_rng(2)
    dphi = (rng.standard_normal(phi0.shape) + 1j * rng.standard_normal(phi0.shape)).astype(np.complex128)
    dpid = (rng.standard_normal(phi0.shape) + 1j * rng.standard_normal(phi0.shape)).astype(np.complex128)
    z6 = np.zeros((6, n, n, n))
    Jt, dJ = axo.tl_run(p, (phi0, phid0, z6, z6), (dphi, dpid, z6, z6), 0.5, 1.0, 0.2, steps, 0.125, 0.5)
    assert J == pytest.approx(Jt, rel=1e-9)
    adj = (float(np.sum(gphi.real * dphi.real + gphi.imag * dphi.imag)) +
           float(np.sum(gpid.real * dpid.real + gpid.imag * dpid.imag)) + 0.5 * dl)
    assert adj == pytest.approx(dJ, rel=1e-8)


def test_green_fp64_512_float_float_transforms_match_cufft(monkeypatch):
    """512^3 FP64-plain Green step: the float-float source transforms and
    contraction against cuFFT's FP64 transforms (accumulators ~1e-12 of
    their largest value)."""
    if _host_gib() < 24 or _device_gib() < 48:
        pytest.skip("needs ~48 GiB of device and ~24 GiB of host memory")
    n = 512
    p = ag.default_params(ngrid=n, precision=ag.PREC_FP64_PLAIN, gw_mode=ag.GW_GREEN, potential=ag.POT_REFERENCE,
                          dspa=32.0 / n, sigma_cr=1.0, kappa=0.1, seed=1)
    with ag.Lattice(p) as lat:
        lat.ic_gaussian_flat(kcut=2.0 * np.pi / (8 * p.dspa))
        phi0, phid0 = lat.download()
    out = {}
    for ff in ("1", "0"):
        monkeypatch.setenv("AXG_FFT_FF", ff)
        with ag.Lattice(p) as lat:
            lat.upload(phi0, phid0)
            lat.leapfrog(2.0, 0.25 * p.dspa, 2, True, True)
            out[ff] = lat.download_gw_green()
    monkeypatch.delenv("AXG_FFT_FF")
    a, b = out["1"], out["0"]
    scale = _max_abs(b)
    assert scale > 0 and _max_abs_diff(a, b) / scale < 1e-12
