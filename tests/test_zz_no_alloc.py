"""axg_field_moments_noalloc: the volume moments for callers that cannot
allocate device memory (their device memory belongs to their own allocator or
pool).  Its scratch is a fixed array inside the library, so it must agree with
the context entry point axg_field_moments (which reduces through memory the
context allocated) on consecutive calls that reuse that array.  This file is
collected last so a failure here never hides the other tests."""
import numpy as np
import pytest

import axion_grav_gb300 as ag

pytestmark = pytest.mark.gpu


def state(n, seed):
    rng = np.random.default_rng(seed)
    phi = (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))).astype(np.complex128)
    phid = (0.5 * (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n)))).astype(np.complex128)
    return phi, phid


def test_noalloc_moments_match_context_entry_point():
    torch = pytest.importorskip("torch")
    n = 32
    p = ag.default_params(ngrid=n, precision=ag.PREC_FP64_PLAIN, dspa=0.5, sigma_cr=1.0, kappa=0.1)
    for call, (seed, tau) in enumerate([(1, 1.3), (2, 2.7)]):
        phi, phid = state(n, seed)
        with ag.Lattice(p) as lat:
            lat.upload(phi, phid)
            ref = lat.field_moments(tau)
        d_phi = torch.from_numpy(phi.view(np.float64).copy()).cuda()
        d_phid = torch.from_numpy(phid.view(np.float64).copy()).cuda()
        torch.cuda.synchronize()
        got = ag.field_moments_noalloc(p, d_phi.data_ptr(), d_phid.data_ptr(), tau)
        np.testing.assert_allclose(got, ref, rtol=1e-12, err_msg=f"call {call}")
        # the same inputs again: the shared scratch from the previous call is overwritten
        again = ag.field_moments_noalloc(p, d_phi.data_ptr(), d_phid.data_ptr(), tau)
        np.testing.assert_array_equal(again, got)


@pytest.mark.parametrize("n", [32, 24])
def test_noalloc_moments_match_oracle(n):
    """Directly against the FP64 oracle (axo.field_moments), also for a
    lattice side that is not a power of two, on two calls in a row."""
    torch = pytest.importorskip("torch")
    from oracle import axo
    p = ag.default_params(ngrid=n, precision=ag.PREC_FP64_PLAIN, dspa=0.5, sigma_cr=1.0, kappa=0.1)
    for seed, tau in ((3, 1.1), (4, 2.3)):
        phi, phid = state(n, seed)
        want = axo.field_moments(p, phi, phid, tau)
        d_phi = torch.from_numpy(phi.view(np.float64).copy()).cuda()
        d_phid = torch.from_numpy(phid.view(np.float64).copy()).cuda()
        torch.cuda.synchronize()
        got = ag.field_moments_noalloc(p, d_phi.data_ptr(), d_phid.data_ptr(), tau)
        np.testing.assert_allclose(got, want, rtol=1e-12)


def test_noalloc_rejects_lattices_beyond_its_scratch():
    p = ag.default_params(ngrid=2050)
    with pytest.raises(ag.AxgError, match="scratch limit"):
        ag.field_moments_noalloc(p, 1, 1, 1.0)
