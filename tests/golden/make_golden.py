"""Regenerate the golden fixtures in this folder from the CPU oracle.

The reference (Fortran + MPI + FFTW + MKL) cannot be built here, so these
are not reference outputs: they pin the oracle's results on small seeded
inputs, which are stored beside them, so that a change in the oracle shows
up as a failed regression test on the CPU, and the GPU tests compare
against committed numbers.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import axion_grav_gb300 as ag  # noqa: E402  (constants only; maps no GPU library)
from oracle import axo  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def cplx(rng, shape, scale=1.0):
    return (scale * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))).astype(np.complex128)


# evolve.f90:238-339 leapfrog of phi and six u_ij, 6^3, both potentials
LEAPFROG = dict(n=6, t1=1.5, dt=0.02, nsteps=6)


def leapfrog_case(potential):
    n = LEAPFROG["n"]
    rng = np.random.default_rng(101 + potential)
    p = axo.default_params(ngrid=n, precision=ag.PREC_FP64_PLAIN, gw_mode=ag.GW_UIJ, potential=potential,
                          dspa=0.5, sigma_cr=1.0, kappa=0.1, seed=11)
    phi0, phid0 = cplx(rng, (n, n, n)), cplx(rng, (n, n, n), 0.3)
    u0, ud0 = 0.05 * rng.standard_normal((6, n, n, n)), 0.05 * rng.standard_normal((6, n, n, n))
    phi, phid, u, ud = phi0.copy(), phid0.copy(), u0.copy(), ud0.copy()
    axo.leapfrog(p, phi, phid, u, ud, None, LEAPFROG["t1"], LEAPFROG["dt"], LEAPFROG["nsteps"], True, True)
    return dict(phi0=phi0, phid0=phid0, u0=u0, ud0=ud0, phi=phi, phid=phid, u=u, ud=ud,
                potential=np.int64(potential))


# defects_3d.f90:31-603 id_defects with the fits, 8^3 random field
DEFECTS = dict(n=8, tau=4.0)


def defects_case():
    n = DEFECTS["n"]
    rng = np.random.default_rng(202)
    p = axo.default_params(ngrid=n, precision=ag.PREC_FP64_PLAIN, flags=7, dspa=1.0, sigma_cr=1.0, kappa=0.1, seed=5)
    phi, phid = cplx(rng, (n, n, n)), cplx(rng, (n, n, n), 0.1)
    sl, wa, sv, cnt, S, W, flags = axo.id_defects(p, phi, phid, DEFECTS["tau"])
    return dict(phi=phi, phid=phid, sl=sl, wa=wa, sv=sv, counts=cnt, strings=S, walls=W, flags=flags)


# grav_waves.f90:193-321 Green's-function accumulation and spectrum, 8^3
GREEN = dict(n=8, t1=2.0, t2=2.4, eps=0.4)


def green_case(compat, n=GREEN["n"], degrade_spec=0):
    rng = np.random.default_rng(303 + compat + 10 * degrade_spec)
    p = axo.default_params(ngrid=n, precision=ag.PREC_FP64_PLAIN, gw_mode=ag.GW_GREEN, dspa=0.75, sigma_cr=1.0,
                           kappa=0.1, tau_cr=1.0, a_now=1.0, num_bin_grav=25, gw_log_bins=12, seed=3,
                           potential=ag.POT_QUARTIC, compat=compat, degrade_spec=degrade_spec)
    phi0, phid0 = cplx(rng, (n, n, n)), cplx(rng, (n, n, n), 0.2)
    phi, phid = phi0.copy(), phid0.copy()
    acc = axo.green_acc_zeros(p)
    nt = axo.symplectic_integration(p, phi, phid, None, None, acc, GREEN["t1"], GREEN["t2"], GREEN["eps"])
    w, pw, nu, de = axo.grav_spec_estimation(p, acc)
    return dict(phi0=phi0, phid0=phid0, phi=phi, acc=acc, nt=np.int64(nt), wave=w, power=pw, numer=nu, denom=de,
                compat=np.int64(compat), degrade_spec=np.int64(degrade_spec))


# spectrum.f90:242-567 field spectrum (no mask), 16^3
SPECTRUM = dict(n=16, tau=3.0)


def spectrum_case():
    n = SPECTRUM["n"]
    rng = np.random.default_rng(404)
    p = axo.default_params(ngrid=n, precision=ag.PREC_FP64_PLAIN, flags=0, dspa=1.0, sigma_cr=1.0, kappa=0.1,
                          seed=7, num_bin=8)
    phid = cplx(rng, (n, n, n))
    w, pw, cv, ct, md = axo.spectrum_estimation(p, phid, None, SPECTRUM["tau"])
    return dict(phid=phid, wave=w, power=pw, conv=cv, count=ct, mat_div=md)


def cases():
    return {
        "leapfrog_uij_ref_6": lambda: leapfrog_case(ag.POT_REFERENCE),
        "leapfrog_uij_quartic_6": lambda: leapfrog_case(ag.POT_QUARTIC),
        "defects_8": defects_case,
        "green_ref_8": lambda: green_case(ag.COMPAT_REF),
        "green_intended_8": lambda: green_case(ag.COMPAT_INTENDED),
        # grav_waves.f90:358-415 degraded sources on the 8^3 GW grid of a 16^3 lattice
        "green_degrade1_ref_16": lambda: green_case(ag.COMPAT_REF, 16, 1),
        "spectrum_16": spectrum_case,
    }


def main():
    for name, fn in cases().items():
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **fn())
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
