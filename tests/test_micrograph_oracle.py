"""The micrograph oracle (objective focalisation, incoherent spectra) against golden vectors
written by the reference's own OpticalFields/FieldViewer code (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from oracle import micrograph as om

GOLD = os.path.join(os.path.dirname(__file__), "golden", "micrograph_golden.npz")
SETTINGS = [
    dict(pol=True, pol_angle=0.0, ana=True, ana_angle=90.0),
    dict(pol=True, pol_angle=30.0, ana=True, ana_angle=100.0, lower="Quarter-wave", lower_angle=15.0,
         upper="Tint-sensitive", upper_angle=40.0),
    dict(),
    dict(pol=True, pol_angle=-20.0, lower="Half-wave", lower_angle=70.0),
]
NA_COND = [0.0, 0.1, 0.25]
K1_NA_COND = [0.0, 0.07, 0.15, 0.2]


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def test_wavevectors(g):
    q = om.wavevectors(0.3, 3)
    np.testing.assert_array_equal(q, g["wavevectors"])
    q1 = om.wavevectors(0.2, 3, koehler_1D=True, dims=(14, 1))
    np.testing.assert_array_equal(q1, g["k1_wavevectors"])


@pytest.mark.parametrize("k", [0, 1, 2])
def test_focus_fields(g, k):
    Nx, Ny = int(g["Nx"]), int(g["Ny"])
    f = om.focus_fields(g["vals"], g["wavelengths"], g["n_out"], g["wavevectors"], Nx, Ny, float(g["dx"]),
                        float(g["dy"]), float(g["na_objective_%d" % k]), float(g["zfoc_NA_corr"]),
                        float(g["z_focus"][k]))
    assert rel(f, g["focused_%d" % k]) < 1e-13


def test_focus_fields_koehler_1d(g):
    for z, key in ((0.8, "k1_focused"), (0.0, "k1_viewer_focused")):
        f = om.focus_fields(g["k1_vals"], g["wavelengths"], 1.0, g["k1_wavevectors"], 14, 1, 0.2, 0.5, 0.4, 0.0, z)
        assert rel(f, g[key]) < 1e-13



@pytest.mark.parametrize("i", range(len(SETTINGS)))
def test_spectrum(g, i):
    pre, post = om.optics_matrices(g["wavelengths"], **SETTINGS[i])
    for j, na in enumerate(NA_COND):
        qs, w = om.koehler_weights(na, 0.3, 3)
        s = om.spectrum(g["focused_0"], pre, post, qs, w)
        assert rel(s, g["spectrum_%d_%d" % (i, j)]) < 1e-13, (i, j)


@pytest.mark.parametrize("i", range(len(SETTINGS)))
def test_spectrum_koehler_1d(g, i):
    pre, post = om.optics_matrices(g["wavelengths"], **SETTINGS[i])
    for j, na in enumerate(K1_NA_COND):
        qs, w = om.koehler_weights(na, 0.2, 3, koehler_1D=True)
        s = om.spectrum(g["k1_viewer_focused"], pre, post, qs, w)
        assert rel(s, g["k1_spectrum_%d_%d" % (i, j)]) < 1e-13, (i, j)


def test_koehler_weights_integrate_g():
    # The ring weights integrate g(q) = q/(1-q^2) over the disc exactly for constant spectra:
    # sum(w) * NA^2/2 = int_0^NA q/(1-q^2) dq = -log(1-NA^2)/2 (2-D rule).
    for na in (0.05, 0.1, 0.17, 0.3):
        _, w = om.koehler_weights(na, 0.3, 4)
        assert abs(w.sum() * na ** 2 / 2 + np.log(1 - na * na) / 2) < 1e-12
