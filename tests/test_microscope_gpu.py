"""GPU objective focalisation and spectra (nbpm_microscope_*) against the golden vectors of
the reference's own OpticalFields/FieldViewer code and against the micrograph oracle."""
import os

import numpy as np
import pytest

from nemaktis_gb300 import _lib
from oracle import micrograph as om

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "micrograph_golden.npz")
SETTINGS = [
    dict(polariser=True, polariser_angle=0.0, analyser=True, analyser_angle=90.0),
    dict(polariser=True, polariser_angle=30.0, analyser=True, analyser_angle=100.0, lower_waveplate="Quarter-wave",
         lower_waveplate_angle=15.0, upper_waveplate="Tint-sensitive", upper_waveplate_angle=40.0),
    dict(polariser=False, analyser=False),
    dict(polariser=True, polariser_angle=-20.0, analyser=False, lower_waveplate="Half-wave",
         lower_waveplate_angle=70.0),
]
TOL = 1e-12  # FP64 relative L2


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def oracle_settings(st):
    return dict(pol=st.get("polariser", False), pol_angle=st.get("polariser_angle", 0.0),
                ana=st.get("analyser", False), ana_angle=st.get("analyser_angle", 0.0),
                lower=st.get("lower_waveplate", "No"), lower_angle=st.get("lower_waveplate_angle", 0.0),
                upper=st.get("upper_waveplate", "No"), upper_angle=st.get("upper_waveplate_angle", 0.0))


def viewer(of, st, na):
    from nemaktis_gb300.microscope import FieldViewer
    fv = FieldViewer.__new__(FieldViewer)
    fv._optical_fields = of
    fv._q_averaged_specter = np.zeros((of._Ny, of._Nx, len(of.get_wavelengths())))
    fv.polariser = fv.analyser = False
    for k, v in st.items():
        setattr(fv, k, v)
    fv.NA_condenser = na
    return fv


@pytest.fixture(scope="module")
def g(gpu):
    return dict(np.load(GOLD))


def golden_fields(g):
    from nemaktis_gb300.microscope import OpticalFields
    Nx, Ny = int(g["Nx"]), int(g["Ny"])
    of = OpticalFields(wavelengths=g["wavelengths"], max_NA_objective=float(g["max_NA_objective"]),
                       max_NA_condenser=float(g["max_NA_condenser"]), N_radial_wavevectors=int(g["N_radial"]),
                       mesh_lengths=(float(g["dx"]) * (Nx - 1), float(g["dy"]) * (Ny - 1)), mesh_dimensions=(Nx, Ny),
                       n_out=g["n_out"], zfoc_NA_corr=float(g["zfoc_NA_corr"]))
    of.vals = g["vals"]
    return of


def test_wavevector_grid(g):
    of = golden_fields(g)
    np.testing.assert_array_equal(of.get_wavevectors(), g["wavevectors"])


@pytest.mark.parametrize("k", [0, 1, 2])
def test_focus_vs_golden(g, k):
    of = golden_fields(g)
    of.update_NA_objective(float(g["na_objective_%d" % k]))
    of.focus_fields(float(g["z_focus"][k]))
    assert rel(of.focused_vals, g["focused_%d" % k]) < TOL


def test_spectra_vs_golden(g):
    from nemaktis_gb300.microscope import FieldViewer
    of = golden_fields(g)
    FieldViewer(of)  # refocuses at z = 0 like the reference's constructor
    for i, st in enumerate(SETTINGS):
        for j, na in enumerate([0.0, 0.1, 0.25]):
            fv = viewer(of, st, na)
            fv.update_image()
            assert rel(fv._q_averaged_specter, g["spectrum_%d_%d" % (i, j)]) < TOL, (i, j)


def test_koehler_1d_vs_golden(g):
    from nemaktis_gb300.microscope import OpticalFields
    of = OpticalFields(wavelengths=g["wavelengths"], max_NA_objective=0.4, max_NA_condenser=0.2,
                       N_radial_wavevectors=3, koehler_1D=True, mesh_lengths=(0.2 * 13, 0.5), mesh_dimensions=(14, 1),
                       n_out=1.0, zfoc_NA_corr=0.0)
    np.testing.assert_array_equal(of.get_wavevectors(), g["k1_wavevectors"])
    of.vals = g["k1_vals"]
    of.focus_fields(0.8)
    assert rel(of.focused_vals, g["k1_focused"]) < TOL
    of.focus_fields(0.0)
    assert rel(of.focused_vals, g["k1_viewer_focused"]) < TOL
    for i, st in enumerate(SETTINGS):
        for j, na in enumerate([0.0, 0.07, 0.15, 0.2]):
            fv = viewer(of, st, na)
            fv.update_image()
            assert rel(fv._q_averaged_specter, g["k1_spectrum_%d_%d" % (i, j)]) < TOL, (i, j)


@pytest.mark.parametrize("Nx,Ny", [(63, 50), (1, 24), (128, 96)])
def test_focus_and_spectrum_vs_oracle(gpu, Nx, Ny):
    """Odd, prime-factor and 1-D meshes, explicit wavevectors, several wavelengths."""
    from nemaktis_gb300.microscope import OpticalFields, FieldViewer
    rng = np.random.default_rng(Nx * 1000 + Ny)
    wl = np.array([0.45, 0.55, 0.7])
    nout = np.array([1.0, 1.33, 1.5])
    q = om.wavevectors(0.2, 3)
    Lx, Ly = 0.2 * max(Nx - 1, 1), 0.25 * max(Ny - 1, 1)
    of = OpticalFields(wavelengths=wl, max_NA_objective=0.6, max_NA_condenser=0.2, N_radial_wavevectors=3,
                       mesh_lengths=(Lx, Ly), mesh_dimensions=(Nx, Ny), n_out=nout, zfoc_NA_corr=0.7, wavevectors=q)
    vals = rng.normal(size=of._vals.shape) + 1j * rng.normal(size=of._vals.shape)
    of.vals = vals
    dx, dy = om.spacing(Lx, Nx), om.spacing(Ly, Ny)
    for z, na in ((0.0, 0.6), (-2.37, 0.45), (5.5, 0.3)):
        of.update_NA_objective(na)
        of.focus_fields(z)
        ref = om.focus_fields(vals, wl, nout, q, Nx, Ny, dx, dy, na, 0.7, z)
        assert rel(of.focused_vals, ref) < TOL, (z, na)
    fv = FieldViewer.__new__(FieldViewer)
    for st in SETTINGS:
        for na_c in (0.0, 0.13, 0.2):
            fv = viewer(of, st, na_c)
            fv.update_image()
            pre, post = om.optics_matrices(wl, **oracle_settings(st))
            qs, w = om.koehler_weights(na_c, 0.2, 3)
            ref = om.spectrum(of.focused_vals, pre, post, qs, w)
            assert rel(fv._q_averaged_specter, ref) < TOL, (st, na_c)


def test_spectrum_needs_enough_wavevectors(gpu):
    from nemaktis_gb300.microscope import OpticalFields
    of = OpticalFields(wavelengths=[0.5], max_NA_objective=0.4, max_NA_condenser=0.3, N_radial_wavevectors=3,
                       mesh_lengths=(3.0, 3.0), mesh_dimensions=(16, 16), wavevectors=[[0, 0], [0.1, 0]])
    of.focus_fields(0)
    fv = viewer(of, {}, 0.25)
    with pytest.raises(_lib.NbpmError) as e:
        fv.update_image()
    assert e.value.code == 2
    fv.NA_condenser = 0.0
    fv.update_image()


def test_wrong_field_shape(gpu):
    from nemaktis_gb300.microscope import OpticalFields
    of = OpticalFields(wavelengths=[0.5, 0.6], max_NA_objective=0.4, mesh_lengths=(3.0, 3.0), mesh_dimensions=(8, 8))
    with pytest.raises(Exception, match="Wrong shape"):
        of.vals = np.zeros((2, 1, 4, 8, 9), complex)


def test_fields_from_plan(gpu):
    """Plan output handed over on the device equals the host route (FP64 and FP32 plans)."""
    from nemaktis_gb300 import api, workloads
    from nemaktis_gb300.microscope import OpticalFields, FieldViewer
    Nx, Ny, Nz = 24, 20, 6
    js = workloads.settings_json((Nx, Ny, Nz), (0.25, 0.25, 0.25), [0.5, 0.6], [[0, 0], [0.05, 0]], no="1.5", ne="1.7")
    lc = workloads.random_smooth((Nx, Ny, Nz), seed=3)
    for prec in ("fp64", "fp32"):
        E = np.zeros((2, 2, 4, Ny, Nx), np.complex128)
        with api.Plan([{"json": js, "lc": lc, "E": E}], precision=prec) as p:
            p.upload()
            p.execute()
            p.download()
            a = OpticalFields(wavelengths=[0.5, 0.6], max_NA_objective=0.4, mesh_lengths=(0.25 * (Nx - 1), 0.25 * (Ny - 1)),
                              mesh_dimensions=(Nx, Ny), wavevectors=[[0, 0], [0.05, 0]])
            a.set_vals_from_plan(p, 0)
            a.focus_fields(1.5)
            b = OpticalFields(wavelengths=[0.5, 0.6], max_NA_objective=0.4, mesh_lengths=(0.25 * (Nx - 1), 0.25 * (Ny - 1)),
                              mesh_dimensions=(Nx, Ny), wavevectors=[[0, 0], [0.05, 0]])
            b.vals = E
            b.focus_fields(1.5)
            np.testing.assert_array_equal(a.focused_vals, b.focused_vals)
            sa, sb = FieldViewer(a), FieldViewer(b)
            sa.update_image()
            sb.update_image()
            np.testing.assert_array_equal(sa.get_spectrum(), sb.get_spectrum())
