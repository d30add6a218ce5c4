"""Known answers of the defect restatement (defects_3d.f90) on CPU."""
import numpy as np
import pytest

from oracle import axo
import axion_grav_gb300 as ag


def params(n, **kw):
    base = dict(ngrid=n, precision=0, gw_mode=0, num_bin=10, degrade_spec=0, flags=7, compat=1,
                potential=0, n_dw=1, num_bin_grav=25, gw_log_bins=16, dspa=1.0, sigma_cr=1.0, kappa=1.0,
                tau_cr=1.0, a_now=1.0, width_cr=0.7, thickness_cr=1.0, vev=1.0, ma2_power=2.0, seed=1)
    base.update(kw)
    return ag.Params().update(**base)


def grid(n):
    return np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")


def four_strings(n, a=0.3, b=0.45):
    z, y, x = grid(n)
    return (np.sin(2 * np.pi * (x + a) / n) + 1j * np.sin(2 * np.pi * (y + b) / n)).astype(np.complex128)


@pytest.mark.parametrize("n", [8, 16, 24])
def test_straight_strings_counts_and_length(n):
    """Four straight strings along z: 4 string cells and 4 pierced xy-plaquettes
    per z-plane; fitted length ~ 1 lattice unit per cell (defects_3d.f90:1027)."""
    p = params(n)
    phi = four_strings(n)
    flags, c = axo.classify_cells(p, phi, ag.F_ID_STRINGS, 0)
    assert c[0] == 4 * n
    assert np.array_equal(axo.string_winding(p, phi), [0, 0, 4 * n])
    sl, wa, sv, cnt, S, W, _ = axo.id_defects(p, phi, np.zeros_like(phi), 5.0)
    assert cnt[0] == 4 * n
    assert sl[0] / (4 * n) == pytest.approx(1.0, abs=0.05)
    # fitted directions are along +-z
    assert np.all(np.abs(S[:, 5]) > 0.85) and np.median(np.abs(S[:, 5])) > 0.95
    # phidot = 0 -> zero velocity, <gamma> = 1
    assert np.allclose(sv, [0, 0, 1])


def test_plane_wall_area():
    """A phase winding once along x has one wall sheet (phase crossing +-pi)
    through N^2 cells, each of area ~1 (defects_3d.f90:1058-1233)."""
    n = 16
    z, y, x = grid(n)
    phi = np.exp(2j * np.pi * (x + 0.37) / n).astype(np.complex128)
    p = params(n)
    flags, c = axo.classify_cells(p, phi, 7, 0)
    assert c[1] == n * n and c[0] == 0
    sl, wa, sv, cnt, S, W, _ = axo.id_defects(p, phi, np.zeros_like(phi), 5.0)
    assert wa[0] / (n * n) == pytest.approx(1.0, abs=0.03)
    assert np.all(np.abs(W[:, 3]) > 0.95)  # normal along x


def test_moving_string_velocity():
    """phi(x - v t): phidot = -v d_x phi gives the string velocity +v x."""
    n, v = 16, 0.3
    z, y, x = grid(n)
    kx = 2 * np.pi / n
    phi = four_strings(n)
    phid = (-v * kx * np.cos(2 * np.pi * (x + 0.3) / n)).astype(np.complex128)
    p = params(n)
    sl, wa, sv, cnt, S, W, _ = axo.id_defects(p, phi, phid, 5.0)
    assert np.median(np.abs(S[:, 6])) == pytest.approx(v, rel=0.1)
    assert np.max(np.abs(S[:, 7])) < 0.05
    assert sv[0] == pytest.approx(v, rel=0.1)


def test_libm_and_project_atan2_agree_on_counts():
    """The literal reference uses libm atan2; the project's deterministic atan2
    differs by <= 1 ulp, which flips no flag on these fields."""
    rng = np.random.default_rng(0)
    for n in (8, 16):
        p = params(n)
        for seed in range(3):
            phi = (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))).astype(np.complex128)
            f0, c0 = axo.classify_cells(p, phi, 7, 0)
            f1, c1 = axo.classify_cells(p, phi, 7, 1)
            assert np.array_equal(f0, f1) and np.array_equal(c0, c1)


def test_id_with_phase_cases():
    """Single cells: phases spread over the circle -> string; clustered -> none;
    a wall when the largest gap is interior (does not straddle +-pi)."""
    n = 4
    p = params(n)
    phi = np.ones((n, n, n), np.complex128)
    flags, c = axo.classify_cells(p, phi, 7, 0)
    assert np.array_equal(c, [0, 0, 0])


def test_pp_inverse_matches_numpy():
    rng = np.random.default_rng(3)
    for n in (1, 4, 7, 12):
        a = rng.standard_normal((n, n))
        m = a @ a.T + n * np.eye(n)
        ap = np.concatenate([m[: j + 1, j] for j in range(n)])  # upper packed, column major
        inv, info = axo.pp_inverse(ap, n)
        assert info == 0
        ref = np.linalg.inv(m)
        got = np.zeros((n, n))
        k = 0
        for j in range(n):
            for i in range(j + 1):
                got[i, j] = got[j, i] = inv[k]
                k += 1
        np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-12)


def test_string_length_geometry():
    # a string along z through the cell centre crosses the z faces: length 1
    assert axo.string_length([0, 0, 0], [0, 0, 1]) == pytest.approx(1.0)
    # along the body diagonal: sqrt(3) > 2*0.866 is rejected by the atmax0 cut
    d = np.array([1, 1, 1]) / np.sqrt(3)
    assert axo.string_length([0, 0, 0], d) == pytest.approx(2 * 0.5 * np.sqrt(3), rel=1e-12) or \
        axo.string_length([0, 0, 0], d) == 0.0


def _components(pos, n, th):
    from scipy.sparse import csr_matrix
    from scipy.sparse.csgraph import connected_components
    d = np.abs(pos[:, None, :] - pos[None, :, :])
    d = np.minimum(d, n - d)
    adj = np.sqrt((d ** 2).sum(-1)) <= th
    ncomp, lab = connected_components(csr_matrix(adj), directed=False)
    return ncomp, lab


def test_grouping_matches_connected_components():
    """group_strings / group_walls: single-linkage groups under the periodic
    threshold max(2, (w^2 hor)^(1/3)) (defects_3d.f90:1235-1652, 1735-2143)."""
    n = 16
    rng = np.random.default_rng(11)
    phi = (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))).astype(np.complex128)
    tau = 3.0
    p = params(n, flags=ag.F_ID_STRINGS | ag.F_ID_WALLS | ag.F_SPEC_EST | ag.F_GROUP_STRINGS | ag.F_GROUP_WALLS,
               width_cr=1.2, thickness_cr=2.0)
    sl, wa, sv, cnt, S, W, _ = axo.id_defects(p, phi, np.zeros_like(phi), tau)
    hor = tau / p.dspa
    for rows, gcol, vcol, wid, t2, t3, out in (
            (S, 12, 10, p.width_cr / p.dspa / tau, 2 * hor, 2 * 3.14159265359 * hor, sl),
            (W, 9, 7, p.thickness_cr / p.dspa / tau, 3.14159265359 * hor ** 2, 4 * 3.14159265359 * hor ** 2, wa)):
        th = max(2.0, (wid * wid * hor) ** (1 / 3))
        ncomp, lab = _components(rows[:, :3], n, th)
        groups = rows[:, gcol].astype(int)
        # same partition, labelled by the smallest member index
        for c in range(ncomp):
            members = np.where(lab == c)[0]
            assert np.all(groups[members] == members.min())
        tot = np.array([rows[lab == c, vcol].sum() for c in range(ncomp)])
        assert out[0] == pytest.approx(tot.sum(), rel=1e-12)
        assert out[1] == pytest.approx(tot[tot > t2].sum(), rel=1e-12, abs=1e-12)
        assert out[2] == pytest.approx(tot[tot > t3].sum(), rel=1e-12, abs=1e-12)


def test_grouping_four_straight_strings():
    n = 16
    p = params(n, flags=ag.F_ID_STRINGS | ag.F_GROUP_STRINGS, width_cr=0.5)
    sl, wa, sv, cnt, S, W, _ = axo.id_defects(p, four_strings(n), np.zeros((n, n, n), np.complex128), 2.0)
    assert len(set(S[:, 12].astype(int))) == 4
    # each string is one group of length ~N; 2*hor = 4 < N so all count as long strings
    assert sl[1] == pytest.approx(sl[0]) and sl[0] / (4 * n) == pytest.approx(1.0, abs=0.05)


def test_fit_cells_reproduces_id_defects_rows():
    # the per-cell fits for a chosen subset equal the rows of the full call
    n = 12
    rng = np.random.default_rng(17)
    phi = (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))).astype(np.complex128)
    phid = (0.1 * (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n)))).astype(np.complex128)
    p = params(n)
    sl, wa, sv, cnt, S, W, _ = axo.id_defects(p, phi, phid, 3.0)
    assert cnt[0] > 10 and cnt[1] > 10
    si = rng.choice(int(cnt[0]), 7, replace=False)
    wi = rng.choice(int(cnt[1]), 5, replace=False)
    fs, fw = axo.fit_cells(p, phi, phid, S[si, 11].astype(np.int64), W[wi, 8].astype(np.int64))
    assert np.array_equal(fs, S[si]) and np.array_equal(fw, W[wi])


def test_float_float_chi2_matches_fp64():
    """The string-fit chi2 runs in float-float arithmetic (about 48 bits) on
    the FP32 pipes; over the fit's parameter box and random corner phases
    it agrees with the FP64 evaluation of defects_3d.f90:385-433 to 1e-13
    of its scale."""
    rng = np.random.default_rng(11)
    lo = np.array([-1.0, -np.pi, 0.0, -np.pi])
    hi = np.array([1.0, np.pi, np.sqrt(3.0) / 2, np.pi])
    worst = 0.0
    for _ in range(4000):
        ph = np.ascontiguousarray(rng.uniform(-np.pi, np.pi, 8))
        pr = np.ascontiguousarray(lo + (hi - lo) * rng.random(4))
        a = axo.lib().axo_chi2_string_ff(axo.dptr(ph), axo.dptr(pr))
        b = axo.lib().axo_chi2_string_fp64(axo.dptr(ph), axo.dptr(pr))
        worst = max(worst, abs(a - b) / max(abs(b), 1.0))
    assert worst < 1e-13, worst


def _chi2_string_numpy(ph, pr):
    """defects_3d.f90:385-433 restated in numpy FP64 with the platform's
    libm sin, cos and atan2: shares no code with the oracle or the kernels.
    ph: (S, 8) corner phases, pr: (S, 4) = (mu, phi, r, theta)."""
    ref_pi = 3.14159265359  # potential.f90:8
    mu, phi, r, th = pr[:, 0], pr[:, 1], pr[:, 2], pr[:, 3]
    u0, v0 = r * np.cos(th), r * np.sin(th)
    sm, sp, cp = np.sqrt(1.0 - mu * mu), np.sin(phi), np.cos(phi)
    a = np.zeros(len(pr))
    b = np.zeros(len(pr))
    near = np.zeros(len(pr), bool)
    for iz in range(2):
        for iy in range(2):
            for ix in range(2):
                x, y, z = ix - 0.5, iy - 0.5, iz - 0.5
                du = -u0 + mu * (x * cp + y * sp) - z * sm
                dv = -v0 - x * sp + y * cp
                d = ph[:, (iz * 2 + iy) * 2 + ix] - np.arctan2(dv, du)
                near |= np.abs(np.abs(d) - ref_pi) < 1e-9
                d = np.where(d >= ref_pi, d - 2 * ref_pi, np.where(d < -ref_pi, d + 2 * ref_pi, d))
                a += d * d
                b += d
    a, b = a / 8, b / 8
    return a - b * b, near


def test_float_float_chi2_matches_independent_libm_restatement():
    """The chi2 the oracle and the kernels share (float-float, project atan2
    and sin/cos) against an independent numpy restatement on libm: equal to
    1e-12 of max(chi2, 1) over the fit's parameter box, corner phases drawn
    uniformly and from near-string configurations (small chi2)."""
    rng = np.random.default_rng(12)
    lo = np.array([-1.0, -np.pi, 0.0, -np.pi])
    hi = np.array([1.0, np.pi, np.sqrt(3.0) / 2, np.pi])
    S = 3000
    pr = lo + (hi - lo) * rng.random((S, 4))
    ph = rng.uniform(-np.pi, np.pi, (S, 8))
    # half the cells: phases of the model at a nearby parameter point plus noise
    pr2 = np.clip(pr + 0.05 * rng.standard_normal((S, 4)), lo, hi)
    mu, phi, r, th = pr2[:, 0], pr2[:, 1], pr2[:, 2], pr2[:, 3]
    u0, v0 = r * np.cos(th), r * np.sin(th)
    sm, sp, cp = np.sqrt(1.0 - mu * mu), np.sin(phi), np.cos(phi)
    for i, (ix, iy, iz) in enumerate((ix, iy, iz) for iz in range(2) for iy in range(2) for ix in range(2)):
        x, y, z = ix - 0.5, iy - 0.5, iz - 0.5
        du = -u0 + mu * (x * cp + y * sp) - z * sm
        dv = -v0 - x * sp + y * cp
        ph[S // 2:, i] = (np.arctan2(dv, du) + 0.01 * rng.standard_normal(S))[S // 2:]
    ph = np.mod(ph + np.pi, 2 * np.pi) - np.pi
    ref, near = _chi2_string_numpy(ph, pr)
    worst = 0.0
    for s in np.flatnonzero(~near):
        a = axo.lib().axo_chi2_string_ff(axo.dptr(np.ascontiguousarray(ph[s])), axo.dptr(np.ascontiguousarray(pr[s])))
        worst = max(worst, abs(a - ref[s]) / max(abs(ref[s]), 1.0))
    assert (~near).sum() > 0.99 * S
    assert worst < 1e-12, worst
