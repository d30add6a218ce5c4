"""GPU defect identification against the oracle: flags, counts, windings and
every per-cell fit bit-exact; global sums within 1e-12."""
import numpy as np
import pytest

import axion_grav_gb300 as ag
from oracle import axo

pytestmark = pytest.mark.gpu


def params(n, precision=ag.PREC_FP64_PLAIN, flags=7, **kw):
    base = dict(ngrid=n, precision=precision, flags=flags, dspa=1.0, sigma_cr=1.0, kappa=0.1, seed=5)
    base.update(kw)
    return ag.default_params(**base)


def fields(kind, n, seed=0):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    if kind == "random":
        return (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))).astype(np.complex128)
    if kind == "strings":
        return (np.sin(2 * np.pi * (x + 0.3) / n) + 1j * np.sin(2 * np.pi * (y + 0.45) / n)).astype(np.complex128)
    if kind == "smooth":
        p = params(n, potential=ag.POT_QUARTIC)
        phi, _ = axo.ic_gaussian_flat(p, kcut=0.9, realisation=seed)
        return phi
    if kind in ("quarter", "half"):
        # phases on multiples of pi/4 (pi/2): exact gap ties and gaps of exactly
        # pi, a hair below the reference's truncated pi -- every such cell is
        # decided by the FP64 fallback of the filtered classification
        k = rng.integers(0, 8 if kind == "quarter" else 4, (n, n, n))
        step = np.pi / 4 if kind == "quarter" else np.pi / 2
        return ((0.5 + rng.random((n, n, n))) * np.exp(1j * step * k)).astype(np.complex128)
    if kind in ("tiny", "huge"):
        # components outside the FP32 range: FP32 phases are unknown (NaN)
        scale = 1e-40 if kind == "tiny" else 1e39
        return scale * (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n)))
    raise KeyError(kind)


@pytest.mark.parametrize("kind", ["random", "strings", "smooth", "quarter", "half", "tiny", "huge"])
@pytest.mark.parametrize("n", [16, 32])
@pytest.mark.parametrize("which", [7, 1, 5, 3])
def test_classification_bit_exact(kind, n, which):
    phi = fields(kind, n, n)
    p = params(n)
    ref_flags, ref_c = axo.classify_cells(p, phi, which, 0)
    with ag.Lattice(p) as lat:
        lat.upload(phi, np.zeros_like(phi))
        c = lat.classify_cells(which)
        f = lat.defect_flags()
    assert np.array_equal(c, ref_c)
    assert np.array_equal(f, ref_flags)


@pytest.mark.parametrize("kind", ["smooth", "quarter", "random"])
def test_classification_fp32_state(kind):
    """FP32-mixed: the flags are those of the FP64 classification of the
    upcast FP32 snapshot."""
    n = 32
    phi = fields(kind, n, 2).astype(np.complex64).astype(np.complex128)
    ref_flags, ref_c = axo.classify_cells(params(n), phi, 7, 0)
    with ag.Lattice(params(n, ag.PREC_FP32_MIXED)) as lat:
        lat.upload(phi, np.zeros_like(phi))
        assert np.array_equal(lat.classify_cells(7), ref_c)
        assert np.array_equal(lat.defect_flags(), ref_flags)
        assert np.array_equal(lat.string_winding(), axo.string_winding(params(n), phi))


@pytest.mark.parametrize("kind", ["random", "strings", "smooth", "quarter", "half", "tiny"])
def test_winding_bit_exact(kind):
    n = 32
    phi = fields(kind, n, 7)
    ref = axo.string_winding(params(n), phi)
    with ag.Lattice(params(n)) as lat:
        lat.upload(phi, np.zeros_like(phi))
        got = lat.string_winding()
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("kind", ["strings", "smooth", "random"])
def test_id_defects_fits_bit_exact(kind):
    n = 16
    phi = fields(kind, n, 3)
    rng = np.random.default_rng(4)
    phid = (0.1 * (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n)))).astype(np.complex128)
    p = params(n)
    sl, wa, sv, cnt, S, W, _ = axo.id_defects(p, phi, phid, 4.0)
    with ag.Lattice(p) as lat:
        lat.upload(phi, phid)
        gsl, gwa, gsv, gcnt = lat.id_defects(1, 4.0)
        gS, gW = lat.defect_lists(int(gcnt[0]), int(gcnt[1]))
    assert np.array_equal(gcnt, cnt)
    # every per-cell result except gof (exp) is bit-identical
    cols = [0, 1, 2, 3, 4, 5, 6, 7, 8, 10, 11]
    assert np.array_equal(gS[:, cols], S[:, cols])
    np.testing.assert_allclose(gS[:, 9], S[:, 9], rtol=1e-14)
    wcols = [0, 1, 2, 3, 4, 5, 7, 8]
    assert np.array_equal(gW[:, wcols], W[:, wcols])
    np.testing.assert_allclose(gsl, sl, rtol=1e-12)
    np.testing.assert_allclose(gwa, wa, rtol=1e-12)
    np.testing.assert_allclose(gsv, sv, rtol=1e-12)


def test_id_defects_empty_lattice():
    n = 16
    phi = np.ones((n, n, n), np.complex128)
    with ag.Lattice(params(n)) as lat:
        lat.upload(phi, np.zeros_like(phi))
        sl, wa, sv, cnt = lat.id_defects(0, 2.0)
    assert np.array_equal(cnt, [0, 0, 0]) and not np.any(sl) and not np.any(wa) and not np.any(sv)


def test_flags_require_fresh_classification():
    n = 16
    with ag.Lattice(params(n)) as lat:
        lat.upload(fields("random", n), np.zeros((n, n, n), np.complex128))
        with pytest.raises(ag.AxgError, match="STATE"):
            lat.defect_flags()


@pytest.mark.parametrize("kind,n", [("random", 16), ("smooth", 32), ("strings", 32)])
def test_grouping_matches_oracle(kind, n):
    flags = 7 | ag.F_GROUP_STRINGS | ag.F_GROUP_WALLS
    phi = fields(kind, n, 9)
    p = params(n, flags=flags, width_cr=1.2, thickness_cr=2.0)
    sl, wa, sv, cnt, S, W, _ = axo.id_defects(p, phi, np.zeros_like(phi), 3.0)
    with ag.Lattice(p) as lat:
        lat.upload(phi, np.zeros_like(phi))
        gsl, gwa, gsv, gcnt = lat.id_defects(1, 3.0)
        gS, gW = lat.defect_lists(int(gcnt[0]), int(gcnt[1]))
    assert np.array_equal(gcnt, cnt)
    assert np.array_equal(gS[:, 12], S[:, 12]) and np.array_equal(gW[:, 9], W[:, 9])
    np.testing.assert_allclose(gsl, sl, rtol=1e-12)
    np.testing.assert_allclose(gwa, wa, rtol=1e-12)
