"""Hand-written adjoint of the leapfrog (phi + six u_ij) against the FP64
tangent-linear reference and central finite differences."""
import numpy as np
import pytest

import axion_grav_gb300 as ag
from oracle import axo

pytestmark = pytest.mark.gpu

ARGS = dict(t1=1.5, dt=0.05, nsteps=12, stride=4, kmin=0.5, kmax=3.0)


def params(n, lam=1.0):
    return ag.default_params(ngrid=n, precision=ag.PREC_FP64_PLAIN, gw_mode=ag.GW_UIJ, potential=ag.POT_QUARTIC,
                             dspa=0.7, sigma_cr=1.0, vev=1.0, seed=4, **{"lambda": lam})


def state(n, seed=0):
    rng = np.random.default_rng(seed)
    phi = (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))).astype(np.complex128)
    phid = (0.2 * (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n)))).astype(np.complex128)
    u = 0.01 * rng.standard_normal((6, n, n, n))
    ud = 0.01 * rng.standard_normal((6, n, n, n))
    return phi, phid, u, ud


def gpu_adjoint(p, st, **kw):
    a = dict(ARGS)
    a.update(kw)
    with ag.Lattice(p) as lat:
        lat.upload(st[0], st[1])
        lat.upload_uij(st[2], st[3])
        out = lat.adjoint_gw_band(a["t1"], a["dt"], a["nsteps"], a["stride"], a["kmin"], a["kmax"])
        final = lat.download(), lat.download_uij()
    return out, final


def rdot(g, d):
    return float(np.sum(g.real * d.real + g.imag * d.imag))


@pytest.mark.parametrize("stride", [4, 5, 12, 1])
def test_adjoint_dot_product_against_tangent_linear(stride):
    n = 16
    p = params(n)
    st = state(n, 1)
    (J, dl, gphi, gpid, _, _), _ = gpu_adjoint(p, st, stride=stride)
    rng = np.random.default_rng(2)
    dphi = (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))).astype(np.complex128)
    dpid = (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))).astype(np.complex128)
    z6 = np.zeros((6, n, n, n))
    Jt, dJ = axo.tl_run(p, st, (dphi, dpid, z6, z6), 0.7, ARGS["t1"], ARGS["dt"], ARGS["nsteps"], ARGS["kmin"],
                        ARGS["kmax"])
    assert J == pytest.approx(Jt, rel=1e-9)
    adj = rdot(gphi, dphi) + rdot(gpid, dpid) + 0.7 * dl
    assert adj == pytest.approx(dJ, rel=1e-8)


def test_adjoint_lambda_against_finite_differences():
    n, eps = 16, 1e-4
    st = state(n, 3)
    (J, dl, *_), _ = gpu_adjoint(params(n), st)
    (Jp, *_), _ = gpu_adjoint(params(n, 1.0 + eps), st)
    (Jm, *_), _ = gpu_adjoint(params(n, 1.0 - eps), st)
    assert dl == pytest.approx((Jp - Jm) / (2 * eps), rel=1e-6)


def test_adjoint_mode_amplitudes_against_finite_differences():
    """32 random Fourier modes below k_cut (selection seed 7): the gradient
    with respect to each mode's amplitude is <dJ/dphi0, e^{ikx}>."""
    n, eps, kcut = 16, 1e-4, 1.5
    p = params(n)
    st = state(n, 5)
    (J, dl, gphi, gpid, _, _), _ = gpu_adjoint(p, st)
    dwav = 2 * 3.14159265359 / 0.7 / n
    q = np.fft.fftfreq(n) * n
    kz, ky, kx = np.meshgrid(q, q, q, indexing="ij")
    kmag = np.sqrt(kx ** 2 + ky ** 2 + kz ** 2) * dwav
    cand = np.argwhere((kmag <= kcut) & (kmag > 0))
    sel = cand[np.random.default_rng(7).choice(len(cand), 32, replace=False)]
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    G = np.fft.fftn(gphi)  # sum_x gphi e^{-ikx}
    for (iz, iy, ix) in sel:
        mode = np.exp(2j * np.pi * (q[ix] * x + q[iy] * y + q[iz] * z) / n)
        grad = rdot(gphi, mode)
        assert grad == pytest.approx(float(np.real(np.conj(G[iz, iy, ix]))), rel=1e-9, abs=1e-9 * abs(grad) + 1e-12)
        (Jp, *_), _ = gpu_adjoint(p, (st[0] + eps * mode, st[1], st[2], st[3]))
        (Jm, *_), _ = gpu_adjoint(p, (st[0] - eps * mode, st[1], st[2], st[3]))
        fd = (Jp - Jm) / (2 * eps)
        assert grad == pytest.approx(fd, rel=2e-5, abs=1e-7 * abs(J))


def test_adjoint_leaves_final_state_of_forward_run():
    n = 16
    p = params(n)
    st = state(n, 6)
    _, ((phi, phid), (u, ud)) = gpu_adjoint(p, st, stride=5)
    a = [x.copy() for x in st]
    axo.leapfrog(p, a[0], a[1], a[2], a[3], None, ARGS["t1"], ARGS["dt"], ARGS["nsteps"], True, True)
    assert np.array_equal(phi, a[0]) and np.array_equal(phid, a[1])
    assert np.array_equal(u, a[2]) and np.array_equal(ud, a[3])


def test_adjoint_rejects_unsupported_paths():
    p = params(16)
    p.gw_mode = ag.GW_NONE
    with ag.Lattice(p) as lat:
        with pytest.raises(ag.AxgError, match="UNSUPPORTED"):
            lat.adjoint_gw_band(1.5, 0.05, 4, 2, 0.5, 3.0)


def _with_precision(p, prec):
    q = type(p).from_buffer_copy(bytes(p))
    q.precision = prec
    return q


def test_fp64_fused_adjoint_equals_plain():
    """The fused FP64 forward is bit-identical to the plain one, so the
    adjoint built on it gives the same J and gradients."""
    n = 32
    st = state(n, 7)
    a = gpu_adjoint(params(n), st)[0]
    b = gpu_adjoint(_with_precision(params(n), ag.PREC_FP64_FUSED), st)[0]
    assert b[0] == pytest.approx(a[0], rel=1e-14)  # J is reduced with atomics: last-bit order effects
    assert b[1] == pytest.approx(a[1], rel=1e-12)
    for g, h in ((b[2], a[2]), (b[3], a[3])):
        assert np.max(np.abs(g - h)) <= 1e-12 * np.max(np.abs(h))


def test_fp32_adjoint_against_fp64_adjoint():
    """FP32-mixed forward and FP32 adjoint arithmetic (dJ/dlambda summed in
    FP64) against the FP64 adjoint of the same initial state."""
    n = 32
    st = state(n, 8)
    a = gpu_adjoint(params(n), st)[0]
    b = gpu_adjoint(_with_precision(params(n), ag.PREC_FP32_MIXED), st)[0]
    assert b[0] == pytest.approx(a[0], rel=1e-4)
    assert b[1] == pytest.approx(a[1], rel=1e-3)
    for g, h in ((b[2], a[2]), (b[3], a[3])):
        assert np.linalg.norm(g - h) <= 1e-3 * np.linalg.norm(h)


def test_fp32_adjoint_lambda_against_finite_differences():
    n, eps = 32, 1e-3
    st = state(n, 9)
    p32 = lambda lam: _with_precision(params(n, lam), ag.PREC_FP32_MIXED)
    (J, dl, *_), _ = gpu_adjoint(p32(1.0), st)
    (Jp, *_), _ = gpu_adjoint(p32(1.0 + eps), st)
    (Jm, *_), _ = gpu_adjoint(p32(1.0 - eps), st)
    assert dl == pytest.approx((Jp - Jm) / (2 * eps), rel=1e-2)


@pytest.mark.parametrize("precision", [ag.PREC_FP32_MIXED, ag.PREC_FP64_PLAIN])
@pytest.mark.parametrize("n", [32, 64])
def test_adjoint_step_kernels_agree(monkeypatch, precision, n):
    """The plain global stencil, the 3-plane shared-memory ring and the
    register-rolling z-march (which also fuses the backward re-step of phi)
    give bit-identical gradients.  dJ/dlambda is summed per site in FP64 by
    the plain kernel, per warp in the arithmetic type by the tiled ones, and
    J and dJ/dlambda go through FP64 atomics."""
    st = state(n, 10)
    p = _with_precision(params(n), precision)
    out, fin = {}, {}
    for kind in ("plain", "ring", "roll"):
        monkeypatch.setenv("AXG_ADJOINT_STEP_KERNEL", kind)
        out[kind], fin[kind] = gpu_adjoint(p, st, nsteps=9, stride=4)
    monkeypatch.delenv("AXG_ADJOINT_STEP_KERNEL")
    # the roll path ping-pongs phi through spare buffers: the context is left
    # at the end of the forward run all the same
    for kind in ("ring", "roll"):
        for a, b in zip(fin[kind][0] + fin[kind][1], fin["plain"][0] + fin["plain"][1]):
            assert np.array_equal(a, b), kind
    ref = out["plain"]
    assert np.isfinite(ref[0]) and np.all(np.isfinite(ref[2]))
    for kind in ("ring", "roll"):
        got = out[kind]
        assert got[0] == pytest.approx(ref[0], rel=1e-13), kind  # J: atomics, last-bit order effects
        assert got[1] == pytest.approx(ref[1], rel=1e-5 if precision == ag.PREC_FP32_MIXED else 1e-12), kind
        assert np.array_equal(got[2], ref[2]) and np.array_equal(got[3], ref[3]), kind
    # ring and roll sum the same per-warp values; only the FP64 atomics' order differs
    assert out["roll"][1] == pytest.approx(out["ring"][1], rel=1e-13)
