"""Shared builders for the tests: small seeded cases and closed-form expectations."""
import json

import numpy as np

from nemaktis_gb300 import workloads


def rand_director(dims, seed=0, smooth=False):
    Nx, Ny, Nz = dims
    rng = np.random.default_rng(seed)
    n = rng.normal(size=(Nz, Ny, Nx, 3))
    if smooth:
        from scipy.ndimage import gaussian_filter
        for c in range(3):
            n[..., c] = gaussian_filter(n[..., c], 1.5, mode="wrap")
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    return n


def rand_qtensor(dims, seed=0):
    n = rand_director(dims, seed)
    S = 0.6
    Q = np.empty(n.shape[:-1] + (6,))
    idx = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    for k, (a, b) in enumerate(idx):
        Q[..., k] = S * (1.5 * n[..., a] * n[..., b] - 0.5 * (a == b))
    return Q


def case(dims, wavelengths=(0.6,), q=((0.0, 0.0),), seed=0, **kw):
    lc = kw.pop("lc", None)
    if lc is None:
        lc = rand_director(dims, seed, smooth=kw.pop("smooth", False))
    js = workloads.settings_json(dims, kw.pop("spacings", (0.25, 0.25, 0.25)), list(wavelengths),
                                 np.asarray(q, float), **kw)
    shape = (len(wavelengths), len(q), 4, dims[1], dims[0])
    return js, lc, shape


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def sqrt_eps_tr(n, no, ne):
    """Approximate sqrt of the transverse permittivity for a uniform director
    (PermittivityTensorField.cpp:70-99)."""
    ep, ea = no ** 2, ne ** 2 - no ** 2
    e = ep * np.eye(3) + ea * np.outer(n, n)
    xx = e[0, 0] - e[0, 2] ** 2 / e[2, 2]
    yy = e[1, 1] - e[1, 2] ** 2 / e[2, 2]
    xy = e[0, 1] - e[0, 2] * e[1, 2] / e[2, 2]
    det, tr = xx * yy - xy * xy, 0.5 * (xx + yy)
    neff = np.sqrt(tr) if tr * tr - det < 1e-8 else 0.5 * (np.sqrt(tr + np.sqrt(tr * tr - det)) + np.sqrt(tr - np.sqrt(tr * tr - det)))
    return np.array([[neff + (xx - yy) / (4 * neff), xy / (2 * neff)], [xy / (2 * neff), neff + (yy - xx) / (4 * neff)]])


def uniform_jones(n, no, ne, nin, nout, wavelength, dz, Nz):
    """Closed-form output for a uniform director at normal incidence with a uniform beam: the
    diffraction operator vanishes on a uniform field, so the result is
    Fout * exp(i k0 dz (S - no))^(Nz-1) * Fin applied to the x / y input polarisations."""
    S = sqrt_eps_tr(np.asarray(n, float), no, ne)
    k0 = 2 * np.pi / wavelength
    w, V = np.linalg.eigh(S - no * np.eye(2))
    P = V @ np.diag(np.exp(1j * k0 * dz * w * (Nz - 1))) @ V.T
    nxx, nyy, nxy = S[0, 0], S[1, 1], S[0, 1]
    d = (nin + nxx) * (nin + nyy) - nxy ** 2
    Fin = np.array([[2 * nin * (nin + nyy) / d, -2 * nin * nxy / d], [-2 * nin * nxy / d, 2 * nin * (nin + nxx) / d]])
    d = (nout + nxx) * (nout + nyy) - nxy ** 2
    Fout = 2 * np.array([[1 - nout * (nout + nyy) / d, nout * nxy / d], [nout * nxy / d, 1 - nout * (nout + nxx) / d]])
    return Fout @ P @ Fin  # columns: input pol x, pol y
