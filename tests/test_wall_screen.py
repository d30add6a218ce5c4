"""The FP32 screen of the wall-direction search (position_wall in
axion_grav_gb300/csrc/axg_defects.cu; defects_3d.f90:1135-1160).

The GPU evaluates chi2 = S - max(W, 0)^2 / m of all 400 directions in FP32
and re-evaluates in FP64, in the reference's order, only those within twice
kWallScreenErr (1e-3) of the smallest FP32 value.  That selects the
reference's direction only if the FP32 value never differs from the FP64 one
by more than kWallScreenErr; the kernel's comment derives a bound of 1.3e-4.
This test restates both evaluations in numpy (float32 rounds every operation,
as the kernel compiled with -fmad=false) and checks the bound on random and
adversarial crossing points."""
import numpy as np

K_WALL_SCREEN_ERR = 1e-3
DERIVED_BOUND = 1.3e-4


def _grid():
    # the 20 x 20 directions of the reference (mu, phi) -> d0
    imu, iphi = np.meshgrid(np.arange(1, 21), np.arange(1, 21), indexing="ij")
    mu = ((-20.0 + 2 * imu) - 1.0) / 20
    phi = 3.14159265359 * ((2 * iphi - 1.0) - 20) / 20
    sq = np.sqrt(1 - mu * mu)
    return np.stack([sq * np.cos(phi), sq * np.sin(phi), mu], axis=-1).reshape(400, 3)


def _fp64(pp, m, d0):
    # reference order: d = pp0 d0 + pp1 d1; d = d + pp2 d2; w += d; chi2 += d d
    w = np.zeros(d0.shape[0])
    c = np.zeros(d0.shape[0])
    for i in range(m):
        d = pp[i, 0] * d0[:, 0] + pp[i, 1] * d0[:, 1]
        d = d + pp[i, 2] * d0[:, 2]
        w = w + d
        c = c + d * d
    w = np.where(w < 0.0, 0.0, w / m)
    return c - m * w * w


def _fp32(pp, m, d0):
    f32 = np.float32
    g = d0.astype(f32)
    p = pp.astype(f32)
    W = np.zeros(d0.shape[0], f32)
    S = np.zeros(d0.shape[0], f32)
    for i in range(m):
        d = (p[i, 0] * g[:, 0] + p[i, 1] * g[:, 1]) + p[i, 2] * g[:, 2]
        W = W + d
        S = S + d * d
    wp = np.maximum(W, f32(0))
    return S - wp * wp / f32(m)


def test_fp32_screen_within_its_bound():
    rng = np.random.default_rng(31)
    d0 = _grid()
    worst = 0.0
    for trial in range(3000):
        m = int(rng.integers(3, 13))
        pp = rng.uniform(-0.5, 0.5, (m, 3))
        if trial % 3 == 1:  # points near a plane through the cell: W near 0 for some directions
            n = rng.normal(size=3)
            n /= np.linalg.norm(n)
            pp -= np.outer(pp @ n, n) * rng.uniform(0.98, 1.0)
            pp = np.clip(pp, -0.4999999, 0.4999999)
        if trial % 3 == 2:  # the largest magnitudes: every point near a cube corner
            pp = np.sign(rng.normal(size=(m, 3))) * rng.uniform(0.49, 0.4999999, (m, 3))
        err = np.max(np.abs(_fp32(pp, m, d0).astype(np.float64) - _fp64(pp, m, d0)))
        worst = max(worst, err)
    assert worst < DERIVED_BOUND < K_WALL_SCREEN_ERR, worst
