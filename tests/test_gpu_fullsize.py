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


def test_adjoint_256_lambda_fd_over_the_full_2000_steps():
    """The gradient workload at its full length: 256^3, 2000 leapfrog steps
    (tau 1 -> 401), checkpoints every 64 steps, dJ/dlambda against the
    central difference (eps = 1e-4) of J from three FP64 runs."""
    eps = 1e-4
    J, dl, *_ = _adjoint_256(1.0, 2000, 64)
    Jp = _adjoint_256(1.0 + eps, 2000, 64)[0]
    Jm = _adjoint_256(1.0 - eps, 2000, 64)[0]
    assert J > 0
    assert dl == pytest.approx((Jp - Jm) / (2 * eps), rel=1e-4)


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


@pytest.mark.parametrize("precision,tol", [(ag.PREC_FP64_PLAIN, 1e-12), (ag.PREC_FP32_MIXED, 2e-5)])
def test_green_512_own_transforms_match_cufft(monkeypatch, precision, tol):
    """512^3 Green step: the own source transforms and contraction against
    cuFFT's (FP64-plain: float-float transforms against FP64 cuFFT,
    accumulators ~1e-12 of their largest value; FP32-mixed: complex-float
    transforms against FP32 cuFFT R2C, FP32 rounding)."""
    if _host_gib() < 24 or _device_gib() < 48:
        pytest.skip("needs ~48 GiB of device and ~24 GiB of host memory")
    n = 512
    p = ag.default_params(ngrid=n, precision=precision, gw_mode=ag.GW_GREEN, potential=ag.POT_REFERENCE,
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
    assert scale > 0 and _max_abs_diff(a, b) / scale < tol


REF_PI = 3.14159265359  # potential.f90:8, the classification thresholds


def _near_margin_cells(phi_slab, margin=2e-5):
    """Cells of a z-slab (all but its last plane) whose classification
    decisions (largest gap against the wrap gap, and against pi and 7 pi / 4,
    defects_3d.f90:309-349) lie within `margin` rad of a threshold: the cells
    the FP32 filter hands to the FP64 recomputation."""
    ph = np.angle(phi_slab)
    nz = ph.shape[0] - 1
    corners = []
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                corners.append(np.roll(np.roll(ph[dz:dz + nz], -dy, 1), -dx, 2))
    srt = np.sort(np.stack(corners), axis=0)
    wrap = srt[0] - srt[-1] + 2 * np.pi
    gmax = np.max(np.diff(srt, axis=0), axis=0)
    big = np.maximum(wrap, gmax)
    near = ((np.abs(gmax - wrap) < margin) | (np.abs(big - REF_PI) < margin) |
            (np.abs(big - 7 * REF_PI / 4) < margin))
    return int(np.count_nonzero(near))


def _defect_parity(p_gpu, p64, evolve):
    """Classification flags and counts and the plaquette windings of the
    GPU's own evolved state against the oracle on the same snapshot."""
    with ag.Lattice(p_gpu) as lat:
        evolve(lat)
        counts = lat.classify_cells(7)
        flags = lat.defect_flags()
        wind = lat.string_winding()
        phi, _ = lat.download(phidot=False)
    rf, rc = axo.classify_cells(p64, phi, 7, 0)
    assert np.array_equal(counts, rc), (counts, rc)
    assert np.array_equal(flags, rf)
    assert np.array_equal(wind, axo.string_winding(p64, phi))
    return counts, phi


@pytest.mark.parametrize("precision", [ag.PREC_FP64_PLAIN, ag.PREC_FP32_MIXED])
def test_defect_counts_bit_exact_on_the_512_snapshot(precision):
    """The benchmark lattice (512^3, reference potential, Gaussian-flat IC)
    after 40 steps: flags, string / wall / mask counts and windings of the
    GPU classification (FP32 filter with FP64 recomputation inside the
    margin) equal the oracle's FP64 classification of the same snapshot
    (defects_3d.f90:31-103, 309-349), for the FP64 and the FP32-mixed state."""
    if _host_gib() < 16:
        pytest.skip("needs ~16 GiB of host memory")
    n = 512
    p = workload(n, precision, ag.GW_NONE)

    def evolve(lat):
        lat.ic_gaussian_flat(kcut=2.0 * np.pi / (8 * p.dspa))
        lat.leapfrog(2.0, 0.25 * p.dspa, 40, True, True)

    counts, phi = _defect_parity(p, workload(n, ag.PREC_FP64_PLAIN, ag.GW_NONE), evolve)
    assert counts[0] > 10 ** 6 and counts[1] > 10 ** 6
    # the FP64 recomputation was exercised: a 16-plane slab alone holds near-margin cells
    assert _near_margin_cells(phi[:17]) > 0


@pytest.mark.parametrize("precision", [ag.PREC_FP64_FUSED, ag.PREC_FP32_MIXED])
def test_defect_counts_bit_exact_256_quartic_ndw2(precision):
    """256^3 quartic model with the N_DW = 2 axion term switched on mid-run
    (tau_on = 11, run from 10 to 18): counts, flags and windings bit-exact
    against the oracle on the same snapshot."""
    if _host_gib() < 8:
        pytest.skip("needs ~8 GiB of host memory")
    n = 256
    p = quartic(n, precision, ag.GW_NONE)

    def evolve(lat):
        lat.ic_gaussian_flat(kcut=1.0)
        lat.leapfrog(10.0, 0.2, 40, True, True)

    counts, _ = _defect_parity(p, quartic(n, ag.PREC_FP64_PLAIN, ag.GW_NONE), evolve)
    assert counts[0] > 0 and counts[1] > 0


def test_id_defects_fits_bit_exact_on_a_128_sample():
    """128^3 benchmark physics evolved to tau ~ 2.6 (about 10^5 string and
    3 10^5 wall cells): a random sample of 256 string and 256 wall cells of
    the GPU's id_defects lists, refitted by the oracle from the same
    snapshot, agrees bit for bit (gof, an exp, to 1e-14); the global sums
    are checked against the oracle's full call at smaller sizes."""
    n = 128
    p = workload(n, ag.PREC_FP64_PLAIN, ag.GW_NONE)
    with ag.Lattice(p) as lat:
        lat.ic_gaussian_flat(kcut=2.0 * np.pi / (8 * p.dspa))
        lat.leapfrog(2.0, 0.25 * p.dspa, 10, True, True)
        tau = 2.0 + 10 * 0.25 * p.dspa
        sl, wa, sv, cnt = lat.id_defects(1, tau)
        S, W = lat.defect_lists(int(cnt[0]), int(cnt[1]))
        phi, phid = lat.download()
    assert cnt[0] > 10 ** 4 and cnt[1] > 10 ** 4
    rng = np.random.default_rng(5)
    si = np.sort(rng.choice(int(cnt[0]), 256, replace=False))
    wi = np.sort(rng.choice(int(cnt[1]), 256, replace=False))
    fs, fw = axo.fit_cells(p, phi, phid, S[si, 11].astype(np.int64), W[wi, 8].astype(np.int64))
    cols = [0, 1, 2, 3, 4, 5, 6, 7, 8, 10, 11]
    assert np.array_equal(S[si][:, cols], fs[:, cols])
    np.testing.assert_allclose(S[si, 9], fs[:, 9], rtol=1e-14)
    wcols = [0, 1, 2, 3, 4, 5, 7, 8]
    assert np.array_equal(W[wi][:, wcols], fw[:, wcols])


@pytest.mark.parametrize("precision", [ag.PREC_FP64_PLAIN, ag.PREC_FP32_MIXED])
def test_wall_fits_bit_exact_on_every_128_cell(precision):
    """Every wall cell of the evolved 128^3 benchmark lattice (about 3 10^5),
    refitted by the oracle from the same snapshot, agrees bit for bit: the
    GPU screens the 400 wall directions in FP32 and evaluates only those
    near the minimum in FP64, which must select the reference's direction."""
    n = 128
    p = workload(n, precision, ag.GW_NONE)
    with ag.Lattice(p) as lat:
        lat.ic_gaussian_flat(kcut=2.0 * np.pi / (8 * p.dspa))
        lat.leapfrog(2.0, 0.25 * p.dspa, 10, True, True)
        tau = 2.0 + 10 * 0.25 * p.dspa
        sl, wa, sv, cnt = lat.id_defects(1, tau)
        S, W = lat.defect_lists(int(cnt[0]), int(cnt[1]))
        phi, phid = lat.download()
    assert cnt[1] > 10 ** 5
    _, fw = axo.fit_cells(p, phi, phid, np.zeros(0, np.int64), W[:, 8].astype(np.int64))
    wcols = [0, 1, 2, 3, 4, 5, 7, 8]
    assert np.array_equal(W[:, wcols], fw[:, wcols])
    np.testing.assert_allclose(W[:, 6], fw[:, 6], rtol=1e-14)

