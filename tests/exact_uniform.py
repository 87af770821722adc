"""Exact forward propagation through a uniform birefringent slab, the known answer of the
reference's BPM accuracy benchmark (HighLevelPythonInterface/examples/benchmarks/3D/
propagate_fields.py:13-126, error measure 01_run_bpm_benchmarks.py:137-196), restated in numpy.

In Fourier space (transverse wave vector p = k_perp/k0) the wave equation for E_perp in a
homogeneous medium is E'' + i R E' + Q E = 0 (derivatives in k0 z). As a first-order system in
(E, E'/nref) it has four eigenmodes per p; the two forward ones (largest Re + Im of the
eigenvalue p_z) carry the field: E(z + dz) = T diag(exp(i p_z k0 dz)) T^-1 E(z), T = the E-part
of the forward eigenvectors."""
import numpy as np


def _p_grids(Nx, Ny, dx, dy, k0):
    px = 2 * np.pi * np.fft.fftfreq(Nx, k0 * dx)[None, :] * np.ones((Ny, 1))
    py = 2 * np.pi * np.fft.fftfreq(Ny, k0 * dy)[:, None] * np.ones((1, Nx))
    return px, py


def evolution_operator(eps, Nx, Ny, dx, dy, dz, wavelength):
    """(Ny, Nx, 2, 2) operator advancing the Fourier components of (Ex, Ey) by dz."""
    k0 = 2 * np.pi / wavelength
    px, py = _p_grids(Nx, Ny, dx, dy, k0)
    p2 = px ** 2 + py ** 2
    e = np.asarray(eps, float)
    den = e[2, 2] - p2
    # transverse permittivity seen by a plane wave of transverse index p
    t00 = e[0, 0] - e[0, 2] ** 2 / den
    t01 = e[0, 1] - e[0, 2] * e[1, 2] / den
    t11 = e[1, 1] - e[1, 2] ** 2 / den
    Q = np.empty((Ny, Nx, 2, 2))
    Q[..., 0, 0] = t00 - px * (px * t00 + py * t01) / e[2, 2] - py ** 2
    Q[..., 0, 1] = t01 - px * (px * t01 + py * t11) / e[2, 2] + px * py
    Q[..., 1, 0] = t01 - py * (px * t00 + py * t01) / e[2, 2] + px * py
    Q[..., 1, 1] = t11 - py * (px * t01 + py * t11) / e[2, 2] - px ** 2
    corr = (e[0, 2] * py ** 2 - e[1, 2] * px * py) / (e[2, 2] * den)
    corr2 = (e[1, 2] * px ** 2 - e[0, 2] * px * py) / (e[2, 2] * den)
    R = np.empty((Ny, Nx, 2, 2))
    R[..., 0, 0] = 2 * px * e[0, 2] / e[2, 2] + px * corr
    R[..., 0, 1] = (px * e[1, 2] + py * e[0, 2]) / e[2, 2] + py * corr
    R[..., 1, 0] = (px * e[1, 2] + py * e[0, 2]) / e[2, 2] + px * corr2
    R[..., 1, 1] = 2 * py * e[1, 2] / e[2, 2] + py * corr2
    nref = np.sqrt(np.mean(np.linalg.eigvals(e)))
    A = np.zeros((Ny, Nx, 4, 4), complex)
    A[..., 0:2, 2:4] = nref * np.eye(2)
    A[..., 2:4, 0:2] = Q / nref
    A[..., 2:4, 2:4] = -R
    w, V = np.linalg.eig(A)
    fwd = np.argsort(np.real(w) + np.imag(w), axis=-1)[..., [-1, -2]]
    pz = np.take_along_axis(w, fwd, axis=-1)
    if np.any(np.imag(pz) < -1e-8):
        raise ValueError("forward-mode selection failed (negative imaginary p_z)")
    T = np.take_along_axis(V[..., 0:2, :], fwd[..., None, :], axis=-1)
    ph = np.exp(1j * pz * k0 * dz)
    return T @ (ph[..., :, None] * np.linalg.inv(T))


def propagate(E0, eps, Nz, dx, dy, dz, wavelength):
    """Planes (Nz, Ny, Nx, 2) from the entrance plane E0 (Ny, Nx, 2)."""
    Ny, Nx = E0.shape[:2]
    U = evolution_operator(eps, Nx, Ny, dx, dy, dz, wavelength)
    F = np.fft.fft2(E0, axes=(0, 1))
    out = np.empty((Nz, Ny, Nx, 2), complex)
    out[0] = E0
    for iz in range(1, Nz):
        F = np.squeeze(U @ F[..., None], -1)
        out[iz] = np.fft.ifft2(F, axes=(0, 1))
    return out


def fourier_error(exact, bpm, dx, wavelength, n, NA=0.4):
    """Mean over the planes and the Fourier components with q^2 < NA^2 (1 - (q/n)^2) of
    |FFT(exact - bpm)| / (2 |FFT exact|) (both (Nz, Ny, Nx, 2), square mesh spacing dx)."""
    k0 = 2 * np.pi / wavelength
    Nz, Ny, Nx, _ = exact.shape
    fe = np.fft.fft2(exact, axes=(1, 2))
    fd = np.fft.fft2(exact - bpm, axes=(1, 2))
    amp = np.sqrt(np.sum(np.abs(fe) ** 2, axis=-1))
    err = np.sqrt(np.sum(np.abs(fd) ** 2, axis=-1)) / (1e-8 + 2 * amp)
    qx = 2 * np.pi * np.fft.fftfreq(Nx, dx)[None, :] / k0
    qy = 2 * np.pi * np.fft.fftfreq(Ny, dx)[:, None] / k0
    q2 = qx ** 2 + qy ** 2
    mask = np.broadcast_to(q2 < NA ** 2 * (1 - q2 / n ** 2), err.shape)
    return float(np.mean(err[mask]))
