"""Seeded synthetic inputs for the benchmark configurations.

The reference publishes no datasets for this path; every input here is synthetic, built from
a seed, with the shapes and value distributions of the five benchmark configurations:

1. twisted nematic 64x64x40 (d = 0.25 um), phi = pi/2*z/L plus smoothed tilt noise
2. cholesteric droplet 512x512x128 (d = 0.2 um), radius 40 um, pitch 5 um, masked
3. eight +-1/2 defects 256x256x64 (d = 0.25 um), 16 wavelengths x 13 wave vectors
4. four random smooth samples 1024^2x200, 768^2x160, 512^2x96, 256^2x48 (d = 0.2 um)
5. a serving mix of the above generators

``settings_json`` emits the JSON tree the nemaktis front end builds
(HighLevelPythonInterface/nemaktis/light_propagator.py:152-186).
"""
import json
import math

import numpy as np

try:
    from scipy.ndimage import gaussian_filter
except Exception:  # pragma: no cover
    gaussian_filter = None


def settings_json(dims, spacings, wavelengths, wavevectors=(0.0, 0.0), no="1.5", ne="1.7", nhost="1.5",
                  nin="1", nout="1", ne_imag="0", n_woodbury=2, NA=1.0, beam="UniformBeam",
                  lc_type="Director", iso_thick=(), iso_index=(), z_shift=0.0, bulk_name=None,
                  results_folder=""):
    """JSON settings string in the layout of light_propagator.py:152-186."""
    wv = [float(v) for v in np.asarray(wavevectors, float).ravel()]
    return json.dumps({
        "Algorithm settings": {
            "General": {"LC field type": lc_type, "Results folder name": results_folder},
            "Beam propagation": {"N Woodbury steps": int(n_woodbury), "Number of substeps per slab": 1}},
        "Physics settings": {
            "Initial conditions": {
                "Beam profile": beam, "LC field file": "",
                "Mesh dimensions": [int(d) for d in dims], "Mesh spacings": [float(s) for s in spacings],
                "Basis convention": "XYZ"},
            "Coefficients": {
                "no": str(no), "ne": str(ne), "ne_imag": str(ne_imag), "nhost": str(nhost),
                "nin": str(nin), "nout": str(nout),
                "Wavelengths": [float(w) for w in wavelengths], "Wavevectors": wv}},
        "Postprocessor settings": {
            "Bulk output": {"Activate": bulk_name is not None, "Base name": bulk_name or ""},
            "Screen output": {
                "Activate": True, "Base name": "",
                "Isotropic layer thicknesses": [float(t) for t in iso_thick],
                "Isotropic layer refractive indices": [float(n) for n in iso_index],
                "Focalisation z-shift": float(z_shift), "Numerical aperture": float(NA)}}})


def hex_wavevectors(Nr, NA):
    """Koehler q-grid of LightPropagator (light_propagator.py:95-103): 1 + 3*Nr*(Nr-1) points."""
    q = [(0.0, 0.0)]
    for ir in range(1, Nr):
        beta = ir * NA / (Nr - 1)
        for iphi in range(6 * ir):
            phi = iphi * np.pi / (3 * ir)
            q.append((beta * np.cos(phi), beta * np.sin(phi)))
    return np.array(q)


def hex_lattice_13(spacing=0.1):
    """13 points of a hexagonal lattice of the given spacing with |q| < 2*spacing."""
    q = [(0.0, 0.0)]
    for k in range(6):
        a = k * np.pi / 3
        q.append((spacing * np.cos(a), spacing * np.sin(a)))
    for k in range(6):
        a = np.pi / 6 + k * np.pi / 3
        q.append((spacing * np.sqrt(3) * np.cos(a), spacing * np.sqrt(3) * np.sin(a)))
    return np.array(q)


def _smooth(a, sigma_vox, axes):
    if gaussian_filter is None:
        raise RuntimeError("scipy is required for the smoothed synthetic fields")
    sig = [0.0] * a.ndim
    for ax in axes:
        sig[ax] = sigma_vox
    return gaussian_filter(a, sigma=sig, mode="wrap")


def twisted_nematic(dims=(64, 64, 40), d=0.25, tilt_sigma=0.05, corr_len=1.0, seed=0):
    """Twisted-nematic director: n = (cos phi cos t, sin phi cos t, sin t), phi = pi/2*z/L, t smoothed noise."""
    Nx, Ny, Nz = dims
    rng = np.random.default_rng(seed)
    L = d * (Nz - 1) if Nz > 1 else 1.0
    z = np.arange(Nz) * d
    phi = (np.pi / 2 * z / L)[:, None, None] * np.ones((1, Ny, Nx))
    t = rng.normal(0.0, 1.0, size=(Nz, Ny, Nx))
    t = _smooth(t, corr_len / d, (0, 1, 2))
    t *= tilt_sigma / max(t.std(), 1e-300)
    n = np.stack([np.cos(phi) * np.cos(t), np.sin(phi) * np.cos(t), np.sin(t)], axis=-1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    return np.ascontiguousarray(n)


def cholesteric_droplet(dims=(512, 512, 128), d=0.2, radius=40.0, pitch=5.0):
    """Cholesteric-droplet director + mask: radial r^ rotated by 2*pi*|r|/p about the azimuthal axis z x r^."""
    Nx, Ny, Nz = dims
    x = (np.arange(Nx) - 0.5 * (Nx - 1)) * d
    y = (np.arange(Ny) - 0.5 * (Ny - 1)) * d
    z = (np.arange(Nz) - 0.5 * (Nz - 1)) * d
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    rs = np.maximum(r, 1e-12)
    rh = np.stack([X / rs, Y / rs, Z / rs], axis=-1)
    ax = np.stack([-Y, X, np.zeros_like(X)], axis=-1)  # z x r
    an = np.linalg.norm(ax, axis=-1, keepdims=True)
    ax = np.where(an > 1e-12, ax / np.maximum(an, 1e-300), np.array([1.0, 0.0, 0.0]))
    psi = (2 * np.pi * r / pitch)[..., None]
    n = np.cos(psi) * rh + np.sin(psi) * np.cross(ax, rh)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    mask = radius ** 2 - X ** 2 - Y ** 2 - Z ** 2
    n = np.where((mask >= 0)[..., None], n, np.array([0.0, 0.0, 1.0]))
    formula = "%g-x^2-y^2-z^2" % (radius ** 2)
    return np.ascontiguousarray(n), np.ascontiguousarray(mask), formula


def point_defects(dims=(256, 256, 64), d=0.25, n_defects=8, smooth_len=1.0, seed=0):
    """Point-defect director: in-plane angle sum_k s_k atan2(y-y_k, x-x_k), s_k = +-1/2."""
    Nx, Ny, Nz = dims
    rng = np.random.default_rng(seed)
    x = (np.arange(Nx) - 0.5 * (Nx - 1)) * d
    y = (np.arange(Ny) - 0.5 * (Ny - 1)) * d
    Y, X = np.meshgrid(y, x, indexing="ij")
    Lx, Ly = d * (Nx - 1), d * (Ny - 1)
    xs = rng.uniform(-0.4 * Lx, 0.4 * Lx, n_defects)
    ys = rng.uniform(-0.4 * Ly, 0.4 * Ly, n_defects)
    s = np.where(np.arange(n_defects) % 2 == 0, 0.5, -0.5)
    phi = np.zeros_like(X)
    for k in range(n_defects):
        phi += s[k] * np.arctan2(Y - ys[k], X - xs[k])
    c2, s2 = _smooth(np.cos(2 * phi), smooth_len / d, (0, 1)), _smooth(np.sin(2 * phi), smooth_len / d, (0, 1))
    ph = 0.5 * np.arctan2(s2, c2)
    n2 = np.stack([np.cos(ph), np.sin(ph), np.zeros_like(ph)], axis=-1)
    n = np.broadcast_to(n2[None], (Nz, Ny, Nx, 3))
    return np.ascontiguousarray(n)


def random_smooth(dims, d=0.2, corr_len=2.0, seed=0, dtype=np.float64):
    """Random smooth director: seeded random unit vectors, Gaussian-filtered, normalised."""
    Nx, Ny, Nz = dims
    rng = np.random.default_rng(seed)
    n = rng.normal(size=(Nz, Ny, Nx, 3)).astype(np.float32)
    for c in range(3):
        n[..., c] = _smooth(n[..., c], corr_len / d, (0, 1, 2))
    n = n.astype(dtype)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    return np.ascontiguousarray(n)


KOEHLER_WAVELENGTHS = list(np.linspace(0.40, 0.80, 16))
UNEVEN_WAVELENGTHS = [0.45, 0.55, 0.65, 0.75]
UNEVEN_MESHES = [(1024, 1024, 200), (768, 768, 160), (512, 512, 96), (256, 256, 48)]


def twisted_nematic_cell(seed=0, dims=(64, 64, 40)):
    lc = twisted_nematic(dims=dims, seed=seed)
    js = settings_json(dims, (0.25, 0.25, 0.25), [0.6], (0.0, 0.0), no="1.5", ne="1.7", nhost="1.5", NA=1.0)
    return {"json": js, "lc": lc, "shape": (1, 1, 4, dims[1], dims[0])}


def droplet_cell(dims=(512, 512, 128)):
    lc, mask, formula = cholesteric_droplet(dims=dims)
    js = settings_json(dims, (0.2, 0.2, 0.2), [0.55], (0.0, 0.0), no="1.5", ne="1.7", nhost="1.55", NA=1.0)
    return {"json": js, "lc": lc, "mask": mask, "formula": formula, "shape": (1, 1, 4, dims[1], dims[0])}


def koehler_micrograph(seed=0, dims=(256, 256, 64), n_wavelengths=16):
    lc = point_defects(dims=dims, seed=seed)
    wl = list(np.linspace(0.40, 0.80, n_wavelengths))
    q = hex_lattice_13(0.1)
    js = settings_json(dims, (0.25, 0.25, 0.25), wl, q, no="1.52+0.008/lambda^2", ne="1.74+0.008/lambda^2",
                       nhost="1.52", NA=0.4)
    return {"json": js, "lc": lc, "shape": (len(wl), len(q), 4, dims[1], dims[0])}


def uneven_sample(i, seed=0):
    dims = UNEVEN_MESHES[i]
    lc = random_smooth(dims, d=0.2, corr_len=2.0, seed=seed + i)
    q = hex_wavevectors(2, 0.15)
    js = settings_json(dims, (0.2, 0.2, 0.2), UNEVEN_WAVELENGTHS, q, no="1.5", ne="1.75", nhost="1.5", NA=0.4)
    return {"json": js, "lc": lc, "shape": (4, len(q), 4, dims[1], dims[0])}


SERVE_MESHES = [(64, 64, 32), (128, 128, 48), (256, 256, 64), (512, 512, 128)]
SERVE_MESH_P = [0.4, 0.3, 0.2, 0.1]


def serving_trace(n_requests, rate=50.0, seed=0, d=0.25, director_pool=0):
    """Serving mix: Poisson arrivals at `rate` per second; mesh drawn from 64^2x32, 128^2x48,
    256^2x64, 512^2x128 with p = .4/.3/.2/.1; director from {twisted nematic, cholesteric
    droplet (masked), random smooth}, seeded per request; N_lambda ~ U{1..32} on [0.40, 0.80];
    N_q ~ U{1..19}: the first N_q points of the 3-ring hexagonal Koehler grid at NA 0.25.
    director_pool > 0 draws each request's director seed from that many seeds per (generator,
    mesh) and shares the arrays between requests with the same seed (bounded generation time and
    host memory for long traces; the run time does not depend on the director's values)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    pool = {}
    q19 = hex_wavevectors(3, 0.25)
    for i in range(n_requests):
        t += rng.exponential(1.0 / rate)
        dims = SERVE_MESHES[rng.choice(4, p=SERVE_MESH_P)]
        kind = ["tn", "droplet", "smooth"][rng.integers(3)]
        nl = int(rng.integers(1, 33))
        nq = int(rng.integers(1, 20))
        wl = list(np.linspace(0.40, 0.80, nl)) if nl > 1 else [0.6]
        q = q19[:nq]
        req = {"arrival": t, "kind": kind, "dims": dims, "n_wavelengths": nl, "n_q": nq}
        Nx, Ny, Nz = dims
        dseed = seed * 1000 + (i if director_pool <= 0 else int(rng.integers(director_pool)))
        pkey = (kind, dims, dseed if kind != "droplet" else 0)
        if pkey in pool:
            lc, mask, formula = pool[pkey]
        else:
            if kind == "tn":
                lc = twisted_nematic(dims=dims, d=d, seed=dseed)
                mask = formula = None
            elif kind == "droplet":
                lc, mask, formula = cholesteric_droplet(dims=dims, d=d, radius=0.4 * d * (Nx - 1), pitch=5.0)
            else:
                lc = random_smooth(dims, d=d, corr_len=2.0, seed=dseed)
                mask = formula = None
            if director_pool > 0:
                pool[pkey] = (lc, mask, formula)
        req.update({"json": settings_json(dims, (d, d, d), wl, q, no="1.5", ne="1.7", nhost="1.55", NA=0.4),
                    "lc": lc, "mask": mask, "formula": formula, "shape": (len(wl), nq, 4, Ny, Nx),
                    "voxel_steps": Nx * Ny * (Nz - 1) * len(wl) * nq * 2})
        out.append(req)
    return out


def voxel_steps(shape, Nz):
    Nl, Nq, _, Ny, Nx = shape
    return Nx * Ny * (Nz - 1) * Nl * Nq * 2


def new_fields(shape):
    return np.zeros(shape, dtype=np.complex128)
