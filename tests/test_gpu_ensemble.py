"""Batched ensembles of uneven lattices (one launch per step, graph-captured
intervals) reproduce single-lattice runs bit for bit."""
import numpy as np
import pytest

import axion_grav_gb300 as ag
from oracle import axo

pytestmark = pytest.mark.gpu


def member_params(n, seed, precision=ag.PREC_FP32_MIXED, gw=ag.GW_UIJ):
    return ag.default_params(ngrid=n, precision=precision, gw_mode=gw, potential=ag.POT_REFERENCE, dspa=0.5,
                             sigma_cr=1.0, kappa=0.1, seed=seed)


SIZES = [32, 64, 32, 96, 64]


def run_single(p, nint, nsteps, dt, t0):
    with ag.Lattice(p) as lat:
        lat.ic_gaussian_flat(1.5, int(p.seed))
        t = t0
        for k in range(nint):
            lat.leapfrog(t, dt, nsteps, True, True)
            t += dt * nsteps
        return lat.download(), lat.download_uij()


@pytest.mark.parametrize("use_graph", [False, True])
def test_ensemble_matches_single_runs(use_graph):
    ps = [member_params(n, 100 + i) for i, n in enumerate(SIZES)]
    dt, t0, nsteps, nint = 0.02, 1.6, 5, 3
    with ag.Ensemble(ps) as ens:
        for i, m in enumerate(ens.members):
            m.ic_gaussian_flat(1.5, 100 + i)
        l0 = ens.launch_count()
        t = t0
        for k in range(nint):
            ens.leapfrog(t, dt, nsteps, True, True, use_graph=use_graph)
            t += dt * nsteps
        launches = ens.launch_count() - l0
        got = [(m.download(), m.download_uij()) for m in ens.members]
    # one batched launch per step plus one half-drift per member per interval
    assert launches == nint * (nsteps + len(SIZES))
    for i, p in enumerate(ps):
        (phi, phid), (u, ud) = run_single(p, nint, nsteps, dt, t0)
        (gphi, gphid), (gu, gud) = got[i]
        assert np.array_equal(gphi, phi) and np.array_equal(gphid, phid), i
        assert np.array_equal(gu, u) and np.array_equal(gud, ud), i


@pytest.mark.parametrize("persistent", [False, True])
def test_ensemble_every_tile_matches_single_runs(persistent):
    """The batched kernel on every tile shape that fits all members, with the
    pointwise fields in registers or in the TMA ring, launched with one CTA
    per work item or as resident CTAs walking the items."""
    sizes = [32, 64, 96]
    ps = [member_params(n, 200 + i) for i, n in enumerate(sizes)]
    dt, t0, nsteps = 0.02, 1.6, 6
    singles = [run_single(p, 1, nsteps, dt, t0) for p in ps]
    lib = ag.load_library()
    tested = 0
    for cfg in range(lib.axg_tile_count()):
        with ag.Ensemble(ps) as ens:
            try:
                ens.set_tile(cfg)
            except ag.AxgError:
                continue
            ens.set_launch_mode(persistent)
            assert ens.launch_mode() == persistent
            for i, m in enumerate(ens.members):
                m.ic_gaussian_flat(1.5, 200 + i)
            ens.leapfrog(t0, dt, nsteps, True, True, use_graph=True)
            got = [(m.download(), m.download_uij()) for m in ens.members]
        tested += 1
        for ((phi, phid), (u, ud)), ((gphi, gphid), (gu, gud)) in zip(singles, got):
            assert np.array_equal(gphi, phi) and np.array_equal(gphid, phid), cfg
            assert np.array_equal(gu, u) and np.array_equal(gud, ud), cfg
    assert tested >= 4


def test_fp64_fused_ensemble_matches_oracle():
    sizes = [32, 64]
    ps = [member_params(n, 7 + i, ag.PREC_FP64_FUSED) for i, n in enumerate(sizes)]
    rng = np.random.default_rng(3)
    states = []
    for n in sizes:
        phi = (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))).astype(np.complex128)
        phid = (0.1 * rng.standard_normal((n, n, n)) + 0j).astype(np.complex128)
        u = 0.01 * rng.standard_normal((6, n, n, n))
        ud = 0.01 * rng.standard_normal((6, n, n, n))
        states.append((phi, phid, u, ud))
    with ag.Ensemble(ps) as ens:
        for m, (phi, phid, u, ud) in zip(ens.members, states):
            m.upload(phi, phid)
            m.upload_uij(u, ud)
        ens.leapfrog(1.5, 0.02, 6, True, True, use_graph=True)
        ens.leapfrog(1.62, 0.02, 6, True, True, use_graph=True)
        got = [(m.download(), m.download_uij()) for m in ens.members]
    for p, (phi, phid, u, ud), ((gphi, gphid), (gu, gud)) in zip(ps, states, got):
        a = [phi.copy(), phid.copy(), u.copy(), ud.copy()]
        axo.leapfrog(p, a[0], a[1], a[2], a[3], None, 1.5, 0.02, 6, True, True)
        axo.leapfrog(p, a[0], a[1], a[2], a[3], None, 1.62, 0.02, 6, True, True)
        assert np.array_equal(gphi, a[0]) and np.array_equal(gphid, a[1])
        assert np.array_equal(gu, a[2]) and np.array_equal(gud, a[3])


def test_ensemble_autotune_restores_state_and_spectra_per_member():
    ps = [member_params(n, 30 + i) for i, n in enumerate([32, 64, 96])]
    with ag.Ensemble(ps) as ens:
        for i, m in enumerate(ens.members):
            m.ic_gaussian_flat(1.5, i)
        before = [m.download()[0] for m in ens.members]
        best, ms = ens.autotune(2)
        after = [m.download()[0] for m in ens.members]
        ens.leapfrog(1.6, 0.02, 4, True, True)
        spec = [m.grav_spec_estimation(1.68) for m in ens.members]
        xi = [m.id_defects(1, 1.68)[0][0] for m in ens.members]
    assert best >= 0 and ms > 0
    for b, a in zip(before, after):
        assert np.array_equal(a, b)
    assert all(np.all(np.isfinite(s[1])) for s in spec) and all(np.isfinite(x) for x in xi)


def test_ensemble_rejects_mixed_physics():
    with pytest.raises(ag.AxgError):
        ag.Ensemble([member_params(32, 1), member_params(32, 2).update(dspa=0.25)])


def test_ensemble_means_equal_the_mean_of_single_runs():
    """The ensemble outputs of the batched workload (config of 96
    realisations, here 5 uneven members): the mean GW spectrum and the mean
    string and wall parameters equal the mean over each realisation's own
    single-lattice results (the members are bit-identical to single runs),
    with the standard error of that mean."""
    ps = [member_params(n, 300 + i) for i, n in enumerate(SIZES)]
    dt, t0, nsteps = 0.02, 1.6, 10
    tau = t0 + dt * nsteps
    with ag.Ensemble(ps) as ens:
        for i, m in enumerate(ens.members):
            m.ic_gaussian_flat(1.5, 300 + i)
        ens.leapfrog(t0, dt, nsteps, True, True, use_graph=True)
        w, pm, ps_, de = ens.grav_spec_mean(tau)
        xm, xs, am, as_ = ens.defect_mean(1, tau)
    singles = []
    for i, p in enumerate(ps):
        with ag.Lattice(p) as lat:
            lat.ic_gaussian_flat(1.5, 300 + i)
            lat.leapfrog(t0, dt, nsteps, True, True)
            sw, spw, snu, sde = lat.grav_spec_estimation(tau)
            sl, wa, sv, cnt = lat.id_defects(1, tau)
        h = tau / p.dspa
        singles.append((sw, spw, sde, h * h * sl / p.ngrid ** 3 / 4, h * wa / p.ngrid ** 3 / 2))
    np.testing.assert_array_equal(w, singles[0][0])
    np.testing.assert_array_equal(de, np.sum([s[2] for s in singles], axis=0))
    for k in range(len(w)):
        vals = [s[1][k] for s in singles if s[2][k] > 0]
        want = np.mean(vals) if vals else 0.0
        assert pm[k] == pytest.approx(want, rel=1e-13, abs=0.0)
        if len(vals) > 1:
            assert ps_[k] == pytest.approx(np.std(vals, ddof=1) / np.sqrt(len(vals)), rel=1e-9)
    xi = np.array([s[3] for s in singles])
    ar = np.array([s[4] for s in singles])
    np.testing.assert_allclose(xm, xi.mean(axis=0), rtol=1e-13)
    np.testing.assert_allclose(xs, xi.std(axis=0, ddof=1) / np.sqrt(len(ps)), rtol=1e-9)
    np.testing.assert_allclose(am, ar.mean(axis=0), rtol=1e-13)
    assert xm[0] > 0 and np.all(pm[1:] >= 0) and pm.max() > 0
