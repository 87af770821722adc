"""CPU tests of the oracle: its FFT, expression evaluator, settings restatement and
closed-form checks of the propagation."""
import json

import numpy as np
import pytest

import oracle
from oracle import expr, settings
from tests.helpers import case, rand_director, rel_l2, uniform_jones
from nemaktis_gb300 import workloads


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 7, 8, 12, 16, 30, 64, 97, 128, 210, 768])
def test_fft_matches_numpy(n):
    rng = np.random.default_rng(n)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    assert np.allclose(oracle.fft1d(x, -1), np.fft.fft(x), rtol=0, atol=1e-12 * max(1, n))
    assert np.allclose(oracle.fft1d(x, +1), np.fft.ifft(x) * n, rtol=0, atol=1e-12 * max(1, n))


@pytest.mark.parametrize("e,lam,val", [
    ("1.5", 0.6, 1.5),
    ("1.52+0.008/lambda^2", 0.5, 1.52 + 0.008 / 0.25),
    ("-2^2", 0, -4.0),
    ("2^-1", 0, 0.5),
    ("2^3^2", 0, 512.0),
    ("sqrt(2)*_pi", 0, np.sqrt(2) * np.pi),
    ("lambda>0.5 ? 1.7 : 1.6", 0.6, 1.7),
    ("max(1,2,3)+min(4,5)", 0, 7.0),
    ("1e-3*lambda", 2.0, 2e-3),
])
def test_expr(e, lam, val):
    assert expr.evaluate(e, **{"lambda": lam}) == pytest.approx(val, rel=1e-15)


def test_settings_defaults_and_lists():
    js = workloads.settings_json((8, 8, 4), (0.2, 0.2, 0.2), [0.5, 0.6], [(0.0, 0.0), (0.1, 0.0)], nhost="1.55")
    s = settings.parse(js)
    assert s["wavelengths"] == [0.5, 0.6]
    assert s["q"] == [(0.0, 0.0), (0.1, 0.0)]
    assert s["nhost_vals"] == [1.55, 1.55]
    j = json.loads(js)
    co = j["Physics settings"]["Coefficients"]
    del co["Wavelengths"], co["Wavevectors"], co["nout"]
    co.update({"Mean wavelength": 0.6, "Spectral FWHM": 0.2, "N wavelengths": 3,
               "Condenser numerical aperture": 0.2, "N radial illumination directions": 2})
    s = settings.parse(json.dumps(j))
    assert np.allclose(s["wavelengths"], [0.5, 0.6, 0.7])
    assert len(s["q"]) == 7 and np.allclose(s["q"][2], (0.1, 0.2 * np.sin(np.pi / 3)))
    assert s["nout_vals"] == [1.0] * 3


def test_uniform_director_closed_form():
    """Uniform tilted director, q = 0: the whole chain reduces to Fresnel and phase matrices."""
    dims = (8, 6, 7)
    n = np.array([np.sin(0.7) * np.cos(0.3), np.sin(0.7) * np.sin(0.3), np.cos(0.7)])
    lc = np.broadcast_to(n, (dims[2], dims[1], dims[0], 3)).copy()
    js, _, shape = case(dims, lc=lc, no="1.5", ne="1.7", nin="1.2", nout="1.1", NA=0.5)
    E = np.zeros(shape, np.complex128)
    oracle.run_backend_without_mask(js, lc, E)
    J = uniform_jones(n, 1.5, 1.7, 1.2, 1.1, 0.6, 0.25, dims[2])
    for pol in range(2):
        for comp in range(2):
            assert np.allclose(E[0, 0, 2 * pol + comp], J[comp, pol], rtol=0, atol=1e-12)


def test_x_invariant_reduces_to_narrow_mesh():
    """An x-invariant structure gives the same fields on Nx = 3 (x-derivatives dropped) as on Nx = 8."""
    Ny, Nz = 12, 6
    rng = np.random.default_rng(3)
    col = rng.normal(size=(Nz, Ny, 1, 3))
    col /= np.linalg.norm(col, axis=-1, keepdims=True)
    outs = []
    for Nx in (3, 8):
        lc = np.broadcast_to(col, (Nz, Ny, Nx, 3)).copy()
        js, _, shape = case((Nx, Ny, Nz), lc=lc, NA=10.0)
        E = np.zeros(shape, np.complex128)
        oracle.run_backend_without_mask(js, lc, E, stages=1)
        outs.append(E[..., 0])
    assert rel_l2(outs[1], outs[0]) < 1e-12


def test_energy_without_absorption():
    """With nin = nout = no and no absorption the screen energy stays close to the input
    energy for a weakly anisotropic smooth sample (sanity bound)."""
    dims = (16, 16, 8)
    js, lc, shape = case(dims, no="1.5", ne="1.55", nin="1.5", nout="1.5", nhost="1.5", NA=10, smooth=True)
    E = np.zeros(shape, np.complex128)
    oracle.run_backend_without_mask(js, lc, E, stages=1)
    e = np.mean(np.abs(E[0, 0, 0]) ** 2 + np.abs(E[0, 0, 1]) ** 2)
    assert 0.95 < e < 1.05


def test_qtensor_of_a_director_gives_the_director_fields():
    """The Q-tensor permittivity eps = (eps_perp + eps_a/3) I + (2 eps_a / 3) Q
    (PermittivityTensorField.cpp:3-99) with Q = 3/2 (n n - I/3) is the director's
    eps_perp I + eps_a n n: both inputs give the same fields."""
    from tests.helpers import case, rand_director
    dims = (10, 9, 6)
    n = rand_director(dims, 4)
    Q = np.empty(n.shape[:-1] + (6,))
    for k, (a, b) in enumerate([(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]):
        Q[..., k] = 1.5 * n[..., a] * n[..., b] - 0.5 * (a == b)
    q = ((0.0, 0.0), (0.08, -0.05))
    js_n, _, shape = case(dims, lc=n, q=q)
    js_q, _, _ = case(dims, lc=Q, lc_type="Q-tensor", q=q)
    En = np.zeros(shape, np.complex128)
    Eq = np.zeros(shape, np.complex128)
    oracle.run_backend_without_mask(js_n, n, En)
    oracle.run_backend_without_mask(js_q, Q, Eq)
    assert np.linalg.norm(Eq - En) / np.linalg.norm(En) < 1e-12


def test_isotropic_uniform_medium_leaves_the_beam_unchanged():
    """ne = no (to 1e-10) = nhost = nin = nout: the Fresnel operators, the phase operator and the
    diffraction step are the identity on a uniform beam, so the screen field equals the input
    polarisation at every point. With ne exactly equal to no the absorption factor
    ne_imag / (ne - no) is 0/0 and the fields are NaN, as in the reference
    (PhaseEvolutionOperator.cpp:12)."""
    from tests.helpers import case, rand_director
    dims = (12, 10, 7)
    n = rand_director(dims, 6)
    js, _, shape = case(dims, lc=n, no="1.5", ne="1.5000000001", nhost="1.5", nin="1.5", nout="1.5")
    E = np.zeros(shape, np.complex128)
    oracle.run_backend_without_mask(js, n, E)
    np.testing.assert_allclose(E[0, 0, 0], 1.0, atol=1e-8)   # x input, Ex
    np.testing.assert_allclose(E[0, 0, 1], 0.0, atol=1e-8)   # x input, Ey
    np.testing.assert_allclose(E[0, 0, 2], 0.0, atol=1e-8)   # y input, Ex (cos(pi/2))
    np.testing.assert_allclose(E[0, 0, 3], 1.0, atol=1e-8)   # y input, Ey
    js, _, shape = case(dims, lc=n, no="1.5", ne="1.5", nhost="1.5", nin="1.5", nout="1.5")
    E = np.zeros(shape, np.complex128)
    oracle.run_backend_without_mask(js, n, E)
    assert np.isnan(E).all()
