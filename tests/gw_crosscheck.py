"""Helpers of the Mode U / Mode G cross-check (tests only).

Mode G is the reference's Green's-function GW method (grav_waves.f90:193-321);
Mode U evolves six u_ij on the lattice and TT-projects them at output.  Both
are driven by the same phi and the same sources; they differ only in how the
waves propagate, so their spectra agree up to O((k dx)^2).  The check runs
one band-limited field on lattices of one box at two or more spacings."""
import numpy as np


def band_limited_fields(n_list, kcut_int=4, seed=7):
    """One band-limited complex field (Fourier modes |k| <= kcut_int of the
    coarsest lattice, complex normal) sampled on lattices of the same box
    with n_list[i] sites a side: the same continuum field at each spacing."""
    nc = n_list[0]
    rng = np.random.default_rng(seed)
    k1 = np.fft.fftfreq(nc, 1.0 / nc).astype(int)
    kz, ky, kx = np.meshgrid(k1, k1, k1, indexing="ij")
    sel = kx ** 2 + ky ** 2 + kz ** 2 <= kcut_int ** 2
    modes = rng.standard_normal(np.count_nonzero(sel)) + 1j * rng.standard_normal(np.count_nonzero(sel))
    out = []
    for n in n_list:
        F = np.zeros((n, n, n), complex)
        F[kz[sel] % n, ky[sel] % n, kx[sel] % n] = modes
        out.append(np.fft.ifftn(F) * n ** 3)
    s = np.sqrt(np.mean(np.abs(out[0]) ** 2))
    return [np.ascontiguousarray(o / s) for o in out]


def mode_u_vs_g(spectra):
    """Band-integrated relative difference sum |U - G| / sum G of the u_ij
    spectrum numerator (Mode U) and the Green's-function numerator (Mode G)
    over the bins with k <= pi / (2 dx) of the coarsest lattice."""
    out = []
    for nug, nuu in spectra:
        band = slice(1, 12)
        out.append(float(np.sum(np.abs(nuu[band] - nug[band])) / np.sum(nug[band])))
    return out

