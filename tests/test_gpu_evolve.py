"""GPU parity of the leapfrog (evolve.f90:238-339) against the CPU oracle."""
import numpy as np
import pytest

import axion_grav_gb300 as ag
from oracle import axo

pytestmark = pytest.mark.gpu


def make_params(n, precision, gw_mode=ag.GW_NONE, potential=ag.POT_REFERENCE, **kw):
    base = dict(ngrid=n, precision=precision, gw_mode=gw_mode, potential=potential, dspa=0.5,
                sigma_cr=1.0, kappa=0.1, seed=11)
    base.update(kw)
    return ag.default_params(**base)


def random_state(n, seed=0, amp_u=0.0):
    rng = np.random.default_rng(seed)
    phi = (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))).astype(np.complex128)
    phid = (0.3 * (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n)))).astype(np.complex128)
    u = amp_u * rng.standard_normal((6, n, n, n))
    ud = amp_u * rng.standard_normal((6, n, n, n))
    return phi, phid, u, ud


def run_gpu(p, state, fn):
    phi, phid, u, ud = state
    with ag.Lattice(p) as lat:
        lat.upload(phi, phid)
        if p.gw_mode == ag.GW_UIJ:
            lat.upload_uij(u, ud)
        out = fn(lat)
        g = lat.download()
        gu = lat.download_uij() if p.gw_mode == ag.GW_UIJ else (None, None)
        launches = lat.launch_count()
    return g[0], g[1], gu[0], gu[1], out, launches


@pytest.mark.parametrize("n", [6, 10, 12, 16, 32])
@pytest.mark.parametrize("gw", [ag.GW_NONE, ag.GW_UIJ])
def test_fp64_plain_drift_kick_bit_exact(n, gw):
    p = make_params(n, ag.PREC_FP64_PLAIN, gw)
    st = random_state(n, 1, 0.1)
    phi, phid, u, ud = (a.copy() for a in st)
    t = 1.7
    axo.evolve_phidot(p, phi, phid, u if gw else None, ud, t, 0.01)
    axo.evolve_phi(p, phi, phid, u if gw else None, ud, 0.005)

    def fn(lat):
        lat.evolve_phidot(t, 0.01)
        return lat.evolve_phi(t, 0.005)

    g_phi, g_phid, g_u, g_ud, tt, _ = run_gpu(p, st, fn)
    assert tt == t + 0.005
    assert np.array_equal(g_phi, phi) and np.array_equal(g_phid, phid)
    if gw:
        assert np.array_equal(g_u, u) and np.array_equal(g_ud, ud)


@pytest.mark.parametrize("dspa", [0.0625, 0.3125, 4.0])
def test_fp64_plain_spacings_bit_exact(dspa):
    """d = 2 dx a power of two (1/8, 8: exact exponent shifts on the integer
    pipe) or not (0.625: FP64 division) -- every case bit-identical to the
    oracle's IEEE operations."""
    n = 16
    p = make_params(n, ag.PREC_FP64_PLAIN, ag.GW_UIJ, dspa=dspa)
    st = random_state(n, 4, 0.1)
    phi, phid, u, ud = (a.copy() for a in st)
    axo.leapfrog(p, phi, phid, u, ud, None, 1.3, 0.01 * dspa, 5, True, True)
    g_phi, g_phid, g_u, g_ud, _, _ = run_gpu(p, st, lambda lat: lat.leapfrog(1.3, 0.01 * dspa, 5, True, True))
    assert np.array_equal(g_phi, phi) and np.array_equal(g_phid, phid)
    assert np.array_equal(g_u, u) and np.array_equal(g_ud, ud)


@pytest.mark.parametrize("potential", [ag.POT_REFERENCE, ag.POT_QUARTIC])
@pytest.mark.parametrize("gw", [ag.GW_NONE, ag.GW_UIJ])
def test_fp64_plain_symplectic_bit_exact(potential, gw):
    n = 32
    p = make_params(n, ag.PREC_FP64_PLAIN, gw, potential, ma2_0=0.3, tau_axion_on=1.6, n_dw=2)
    st = random_state(n, 2, 0.05)
    phi, phid, u, ud = (a.copy() for a in st)
    nt = axo.symplectic_integration(p, phi, phid, u if gw else None, ud, None, 1.5, 1.9, 0.4)
    g_phi, g_phid, g_u, g_ud, nt_g, _ = run_gpu(p, st, lambda lat: lat.symplectic_integration(1.5, 1.9, 0.4))
    assert nt_g == nt and nt > 5
    assert np.array_equal(g_phi, phi) and np.array_equal(g_phid, phid)
    if gw:
        assert np.array_equal(g_u, u) and np.array_equal(g_ud, ud)


@pytest.mark.parametrize("n", [32, 64])
@pytest.mark.parametrize("gw", [ag.GW_NONE, ag.GW_UIJ])
def test_fp64_fused_bit_exact_all_tiles(n, gw):
    """The TMA-staged fused kernel does the plain path's operations in the same
    order, so every tile shape reproduces the oracle bit for bit."""
    p = make_params(n, ag.PREC_FP64_FUSED, gw)
    st = random_state(n, 3, 0.05)
    phi, phid, u, ud = (a.copy() for a in st)
    axo.leapfrog(p, phi, phid, u if gw else None, ud, None, 1.5, 0.02, 7, True, True)
    lib = ag.load_library()
    ntile = lib.axg_tile_count()
    tested = 0
    for cfg in range(ntile):
        def fn(lat, cfg=cfg):
            try:
                lat.set_tile(cfg)
            except ag.AxgError:
                return False
            lat.leapfrog(1.5, 0.02, 7, True, True)
            return True
        g_phi, g_phid, g_u, g_ud, ok, _ = run_gpu(p, st, fn)
        if not ok:
            continue
        tested += 1
        assert np.array_equal(g_phi, phi) and np.array_equal(g_phid, phid), cfg
        if gw:
            assert np.array_equal(g_u, u) and np.array_equal(g_ud, ud), cfg
    assert tested >= 3


@pytest.mark.parametrize("gw", [ag.GW_NONE, ag.GW_UIJ])
def test_fp32_mixed_identical_on_all_tiles(gw):
    """Each site's FP32 arithmetic does not depend on the tile shape or on
    whether the pointwise fields arrive through registers or the TMA ring."""
    n = 64
    p = make_params(n, ag.PREC_FP32_MIXED, gw)
    st = random_state(n, 4, 0.05)
    lib = ag.load_library()
    ref, tested, pw = None, 0, 0
    for cfg in range(lib.axg_tile_count()):
        def fn(lat, cfg=cfg):
            try:
                lat.set_tile(cfg)
            except ag.AxgError:
                return False
            lat.leapfrog(1.5, 0.02, 9, True, True)
            return True
        out = run_gpu(p, st, fn)
        if not out[4]:
            continue
        tested += 1
        pw += ag.tile_table()[cfg][3]
        if ref is None:
            ref = out
            continue
        for a, b in zip(out[:4], ref[:4]):
            if a is not None:
                assert np.array_equal(a, b), cfg
    assert tested >= 4 and pw >= 2


@pytest.mark.parametrize("n", [24, 48])
@pytest.mark.parametrize("gw", [ag.GW_NONE, ag.GW_UIJ])
def test_fp64_fused_plain_kernel_bit_exact(n, gw):
    """N not a multiple of 32 has no TMA tile: the plain stencil kernel runs
    the fused step with the same operations, bit for bit."""
    p = make_params(n, ag.PREC_FP64_FUSED, gw)
    st = random_state(n, 5, 0.05)
    phi, phid, u, ud = (a.copy() for a in st)
    axo.leapfrog(p, phi, phid, u if gw else None, ud, None, 1.5, 0.02, 5, True, True)

    def fn(lat):
        lat.set_kernel_timing(True)
        lat.leapfrog(1.5, 0.02, 5, True, True)
        lat.synchronize()
        return dict((k, l) for k, l, _ in lat.kernel_timings())
    g_phi, g_phid, g_u, g_ud, kt, _ = run_gpu(p, st, fn)
    assert kt.get("fused_kd_fp64_%s_plain" % ("uij" if gw else "phi"), 0) == 5
    assert np.array_equal(g_phi, phi) and np.array_equal(g_phid, phid)
    if gw:
        assert np.array_equal(g_u, u) and np.array_equal(g_ud, ud)


@pytest.mark.parametrize("prec", [ag.PREC_FP32_MIXED, ag.PREC_FP64_FUSED])
@pytest.mark.parametrize("gw", [ag.GW_NONE, ag.GW_UIJ])
def test_plain_kernel_identical_to_tma_tiles(prec, gw, monkeypatch):
    """AXG_FUSED_PLAIN=1 forces the plain stencil kernel at N = 64; its
    per-site arithmetic is the tiled kernels' own, so the bits agree."""
    n = 64
    p = make_params(n, prec, gw)
    st = random_state(n, 6, 0.05)
    run = lambda lat: lat.leapfrog(1.5, 0.02, 6, True, True)
    ref = run_gpu(p, st, run)
    monkeypatch.setenv("AXG_FUSED_PLAIN", "1")

    def fn(lat):
        lat.set_kernel_timing(True)
        run(lat)
        lat.synchronize()
        return dict((k, l) for k, l, _ in lat.kernel_timings())
    out = run_gpu(p, st, fn)
    name = "fused_kd_%s_%s_plain" % ("fp32" if prec == ag.PREC_FP32_MIXED else "fp64", "uij" if gw else "phi")
    assert out[4].get(name, 0) == 6
    for a, b in zip(out[:4], ref[:4]):
        if a is not None:
            assert np.array_equal(a, b)


@pytest.mark.parametrize("n", [32, 48, 64])
def test_fp32_mixed_matches_fp64_oracle(n):
    """FP32 fields and stencil with Kahan drift: tolerance against FP64."""
    p64 = make_params(n, ag.PREC_FP64_PLAIN, ag.GW_UIJ)
    p32 = make_params(n, ag.PREC_FP32_MIXED, ag.GW_UIJ)
    phi0, _ = axo.ic_gaussian_flat(p64, kcut=1.5)
    phid0 = np.zeros_like(phi0)
    u0 = np.zeros((6, n, n, n))
    st = (phi0, phid0, u0, u0.copy())
    phi, phid, u, ud = (a.copy() for a in st)
    nt = axo.symplectic_integration(p64, phi, phid, u, ud, None, 1.2, 2.0, 0.3)
    g_phi, g_phid, g_u, g_ud, nt_g, _ = run_gpu(p32, st, lambda lat: lat.symplectic_integration(1.2, 2.0, 0.3))
    assert nt_g == nt
    rel = lambda a, b: np.max(np.abs(a - b)) / np.max(np.abs(b))
    assert rel(g_phi, phi) < 2e-5
    assert rel(g_phid, phid) < 2e-4
    assert rel(g_ud, ud) < 2e-3
    assert rel(g_u, u) < 2e-3


def test_fp32_kahan_drift_beats_naive_rounding():
    """Drift-only: many tiny increments; the Kahan-compensated FP32 sum stays
    at FP64 accuracy where plain FP32 accumulation would drift."""
    n = 32
    p32 = make_params(n, ag.PREC_FP32_MIXED, ag.GW_UIJ)
    rng = np.random.default_rng(5)
    phi = (1.0 + 0.1 * rng.standard_normal((n, n, n)) + 0j).astype(np.complex128)
    phid = (1e-3 * (1 + rng.random((n, n, n))) + 1j * 1e-3).astype(np.complex128)
    u = np.ones((6, n, n, n))
    ud = 1e-3 * np.ones((6, n, n, n))
    h, steps = 1e-3, 2000
    with ag.Lattice(p32) as lat:
        lat.upload(phi, phid)
        lat.upload_uij(u, ud)
        t = 1.0
        for _ in range(steps):
            t = lat.evolve_phi(t, h)
        g_phi, _ = lat.download()
        g_u, _ = lat.download_uij()
    exact = phi + steps * h * phid
    assert np.max(np.abs(g_phi - exact)) < 1e-9
    assert np.max(np.abs(g_u - (u + steps * h * ud))) < 1e-9


def test_upload_download_reference_halo_layout():
    """data1(N, N, local_0+2) with one halo plane on each side."""
    n = 16
    p = make_params(n, ag.PREC_FP64_PLAIN)
    rng = np.random.default_rng(9)
    host = (rng.standard_normal((n + 2, n, n)) + 1j * rng.standard_normal((n + 2, n, n))).astype(np.complex128)
    with ag.Lattice(p) as lat:
        f = ag.load_library().axg_upload
        import ctypes
        dp = lambda a: a.view(np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        assert f(lat.handle, dp(host), None, n * n, 1) == 0
        back = np.zeros_like(host)
        assert ag.load_library().axg_download(lat.handle, dp(back), None, n * n, 1) == 0
    assert np.array_equal(back[1:-1], host[1:-1])
    assert not np.any(back[0]) and not np.any(back[-1])


def test_ic_gaussian_flat_matches_oracle():
    n = 32
    for prec in (ag.PREC_FP64_PLAIN, ag.PREC_FP32_MIXED):
        p = make_params(n, prec, potential=ag.POT_QUARTIC)
        ref, _ = axo.ic_gaussian_flat(p, kcut=1.2, realisation=3)
        with ag.Lattice(p) as lat:
            lat.ic_gaussian_flat(1.2, 3)
            g, gd = lat.download()
        tol = 1e-12 if prec == ag.PREC_FP64_PLAIN else 1e-7
        assert np.max(np.abs(g - ref)) < tol * np.max(np.abs(ref))
        assert not np.any(gd)


def test_ic_thermal_matches_oracle():
    n = 16
    p = make_params(n, ag.PREC_FP64_PLAIN, sigma_cr=0.5, dspa=1.0)
    ref_phi, ref_phid = axo.ic_thermal(p, 0.6, 1)
    with ag.Lattice(p) as lat:
        lat.ic_thermal(0.6, 1)
        g, gd = lat.download()
    assert np.max(np.abs(g - ref_phi)) < 1e-11 * np.max(np.abs(ref_phi))
    assert np.max(np.abs(gd - ref_phid)) < 1e-11 * np.max(np.abs(ref_phid))


def test_field_moments_fp64_sums():
    n = 32
    for prec in (ag.PREC_FP64_PLAIN, ag.PREC_FP32_MIXED):
        p = make_params(n, prec)
        st = random_state(n, 4)
        ref = axo.field_moments(p, st[0], st[1], 1.3)
        with ag.Lattice(p) as lat:
            lat.upload(st[0], st[1])
            got = lat.field_moments(1.3)
        tol = 1e-12 if prec == ag.PREC_FP64_PLAIN else 1e-6
        np.testing.assert_allclose(got, ref, rtol=tol)


def test_checkpoint_roundtrip_and_crc(tmp_path):
    n = 16
    p = make_params(n, ag.PREC_FP64_PLAIN, ag.GW_UIJ)
    st = random_state(n, 6, 0.2)
    path = str(tmp_path / "run_phi_3.chk")
    with ag.Lattice(p) as lat:
        lat.upload(st[0], st[1])
        lat.upload_uij(st[2], st[3])
        lat.write_chk(path)
    raw = np.fromfile(path, dtype=np.complex128, count=2 * n ** 3)
    # io_chk layout: phi block then phidot block, x fastest (evolve.f90:498-503)
    assert np.array_equal(raw[: n ** 3].reshape(n, n, n), st[0])
    assert np.array_equal(raw[n ** 3:].reshape(n, n, n), st[1])
    with ag.Lattice(p) as lat:
        lat.read_chk(path)
        g = lat.download()
        gu = lat.download_uij()
    assert np.array_equal(g[0], st[0]) and np.array_equal(gu[1], st[3])
    data = bytearray(open(path, "rb").read())
    data[100] ^= 0x40
    open(path, "wb").write(bytes(data))
    with ag.Lattice(p) as lat:
        with pytest.raises(ag.AxgError, match="CRC"):
            lat.read_chk(path)


def test_fp32_checkpoint_resume_is_bit_exact(tmp_path):
    """FP32-mixed Mode U: stop, write_chk, read_chk into a fresh context and
    continue; the result equals the uninterrupted run bit for bit (the .fp32
    sidecar restores the Kahan compensations), and a damaged sidecar is
    rejected."""
    n = 32
    p = make_params(n, ag.PREC_FP32_MIXED, ag.GW_UIJ)
    st = random_state(n, 9, 0.2)
    path = str(tmp_path / "run_fp32.chk")
    with ag.Lattice(p) as lat:
        lat.upload(st[0], st[1])
        lat.upload_uij(st[2], st[3])
        lat.leapfrog(1.5, 0.02, 7, True, False)
        lat.write_chk(path)
        lat.leapfrog(1.64, 0.02, 6, False, True)
        want = lat.download(), lat.download_uij()
    with ag.Lattice(p) as lat:
        lat.read_chk(path)
        lat.leapfrog(1.64, 0.02, 6, False, True)
        got = lat.download(), lat.download_uij()
    for a, b in zip(got[0] + got[1], want[0] + want[1]):
        assert np.array_equal(a, b)
    data = bytearray(open(path + ".fp32", "rb").read())
    data[64] ^= 0x01
    open(path + ".fp32", "wb").write(bytes(data))
    with ag.Lattice(p) as lat:
        with pytest.raises(ag.AxgError, match="CRC"):
            lat.read_chk(path)


def test_fp32_sidecar_of_an_older_checkpoint_is_not_used(tmp_path):
    """The .fp32 sidecar records the CRC of the checkpoint it was written
    with.  An FP64 context that rewrites the checkpoint removes the old
    sidecar, and a sidecar put back beside a different checkpoint is
    ignored: the FP32 resume then takes the complex128 checkpoint's state."""
    import shutil
    n = 32
    st_a, st_b = random_state(n, 21, 0.2), random_state(n, 22, 0.2)
    path = str(tmp_path / "run.chk")
    p32 = make_params(n, ag.PREC_FP32_MIXED, ag.GW_UIJ)
    p64 = make_params(n, ag.PREC_FP64_PLAIN, ag.GW_UIJ)
    with ag.Lattice(p32) as lat:
        lat.upload(st_a[0], st_a[1])
        lat.upload_uij(st_a[2], st_a[3])
        lat.leapfrog(1.5, 0.02, 3, True, False)
        lat.write_chk(path)
    shutil.copy(path + ".fp32", str(tmp_path / "old.fp32"))
    with ag.Lattice(p64) as lat:
        lat.upload(st_b[0], st_b[1])
        lat.upload_uij(st_b[2], st_b[3])
        lat.write_chk(path)
    import os
    assert not os.path.exists(path + ".fp32")
    shutil.copy(str(tmp_path / "old.fp32"), path + ".fp32")
    with ag.Lattice(p32) as lat:
        lat.read_chk(path)
        g = lat.download()
    # state B as FP32 storage, not the state the old sidecar holds
    assert np.max(np.abs(g[0] - st_b[0])) < 1e-6 and np.max(np.abs(g[1] - st_b[1])) < 1e-6


def test_wait_timeout_status_and_recovery():
    """The give-up path of the bounded TMA stage wait: a barrier that nothing
    arrives on (no copy issued) runs out after a short limit, the call
    returns ERR_TIMEOUT with the stage-wait message, and the context keeps
    working: a fused FP64 step afterwards is bit-exact against the oracle."""
    n = 32
    p = make_params(n, ag.PREC_FP64_FUSED, ag.GW_UIJ)
    st = random_state(n, 31, 0.1)
    with ag.Lattice(p) as lat:
        lat.upload(st[0], st[1])
        lat.upload_uij(st[2], st[3])
        for _ in range(2):
            with pytest.raises(ag.AxgError, match="ERR_TIMEOUT.*timed out"):
                lat.selftest_wait_timeout(2_000_000)
        lat.leapfrog(1.5, 0.02, 4, True, True)
        g = lat.download()
        gu = lat.download_uij()
        with pytest.raises(ag.AxgError, match="ERR_ARG"):
            lat.selftest_wait_timeout(10)
    phi, phid, u, ud = (a.copy() for a in st)
    axo.leapfrog(p, phi, phid, u, ud, None, 1.5, 0.02, 4, True, True)
    assert np.array_equal(g[0], phi) and np.array_equal(g[1], phid)
    assert np.array_equal(gu[0], u) and np.array_equal(gu[1], ud)


def test_kernel_timing_and_launch_count():
    n = 64
    p = make_params(n, ag.PREC_FP32_MIXED, ag.GW_UIJ)
    with ag.Lattice(p) as lat:
        lat.ic_gaussian_flat(1.0)
        lat.set_kernel_timing(True)
        before = lat.launch_count()
        lat.leapfrog(2.0, 0.01, 10, False, False)
        lat.synchronize()
        after = lat.launch_count()
        kt = dict((k, (l, ms)) for k, l, ms in lat.kernel_timings())
    assert after - before == 10
    assert kt["fused_kd_fp32_uij"][0] == 10 and kt["fused_kd_fp32_uij"][1] > 0


def test_autotune_restores_state():
    n = 64
    p = make_params(n, ag.PREC_FP32_MIXED, ag.GW_UIJ)
    st = random_state(n, 8, 0.1)
    with ag.Lattice(p) as lat:
        lat.upload(st[0], st[1])
        lat.upload_uij(st[2], st[3])
        best, ms = lat.autotune(2)
        g = lat.download()
        gu = lat.download_uij()
    assert best >= 0 and ms > 0
    assert np.max(np.abs(g[0] - st[0])) < 1e-6 and np.max(np.abs(gu[1] - st[3])) < 1e-6


def test_bad_params_raise():
    with pytest.raises(ag.AxgError):
        ag.Lattice(make_params(15, ag.PREC_FP64_PLAIN))
    p = make_params(48, ag.PREC_FP32_MIXED)  # not a multiple of 32: no TMA tile to select
    with ag.Lattice(p) as lat:
        with pytest.raises(ag.AxgError, match="UNSUPPORTED"):
            lat.set_tile(0)
        with pytest.raises(ag.AxgError, match="UNSUPPORTED"):
            lat.autotune(1)
