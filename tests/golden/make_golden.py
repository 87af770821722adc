"""Golden vectors for objective focalisation and incoherent spectra, produced by the
reference's own Python code.

Imports HighLevelPythonInterface/nemaktis/light_propagator.py (OpticalFields: objective filter
:618-646, focus_fields :708-719) and field_viewer.py (FieldViewer._update_specter :348-388,
_update_averaged_specter :391-455) from a reference checkout whose root is the required first
argument (``python make_golden.py <nemaktis checkout>``). Their GUI, VTK, dtmm and bpm_backend imports
are replaced by empty stand-ins that the exercised code never calls, and pyfftw by numpy.fft
with pyfftw's documented FFTW.__call__ semantics (forward unnormalised, backward normalised by
the transform size). Writes micrograph_golden.npz next to this script. Not run by the tests;
the fixture it wrote is committed.
"""
import os
import sys
import types

import numpy as np

REF = None  # root of the reference checkout, set from the command line
HERE = os.path.dirname(os.path.abspath(__file__))


def _stub(name, **attrs):
    m = types.ModuleType(name)
    m.__dict__.update(attrs)
    sys.modules[name] = m
    return m


class _FFTW:
    def __init__(self, a, b, axes=(-2, -1), threads=1, direction="FFTW_FORWARD"):
        self.a, self.b, self.axes, self.fwd = a, b, tuple(axes), direction == "FFTW_FORWARD"

    def __call__(self):
        if self.fwd:
            self.b[...] = np.fft.fftn(self.a, axes=self.axes)
        else:
            self.b[...] = np.fft.ifftn(self.a, axes=self.axes)


def load_reference():
    _stub("pyfftw", empty_aligned=lambda shape, dtype: np.empty(shape, dtype=dtype), FFTW=_FFTW,
          config=types.SimpleNamespace(NUM_THREADS=1))
    _stub("bpm_backend")
    dt = _stub("dtmm", conf=types.SimpleNamespace(set_verbose=lambda v: None))
    dt.color = _stub("dtmm.color")
    vtk = _stub("vtk", vtkImageData=object, vtkXMLImageDataReader=object, vtkXMLImageDataWriter=object)
    vtk.util = _stub("vtk.util")
    vtk.util.numpy_support = _stub("vtk.util.numpy_support")
    mpl = _stub("matplotlib", use=lambda *a, **k: None, rcParams={})
    mpl.pyplot = _stub("matplotlib.pyplot")
    mpl.figure = _stub("matplotlib.figure", Figure=object)
    pkg = types.ModuleType("nemaktis")
    pkg.__path__ = [os.path.join(REF, "HighLevelPythonInterface", "nemaktis")]
    sys.modules["nemaktis"] = pkg
    _stub("nemaktis.field_viewer_ui")
    from nemaktis.light_propagator import OpticalFields
    from nemaktis.field_viewer import FieldViewer
    return OpticalFields, FieldViewer


SETTINGS = [
    # (polariser, polariser_angle, analyser, analyser_angle, lower, lower_angle, upper, upper_angle)
    (True, 0.0, True, 90.0, "No", 0.0, "No", 0.0),
    (True, 30.0, True, 100.0, "Quarter-wave", 15.0, "Tint-sensitive", 40.0),
    (False, 0.0, False, 0.0, "No", 0.0, "No", 0.0),
    (True, -20.0, False, 0.0, "Half-wave", 70.0, "No", 0.0),
]
NA_CONDENSER = [0.0, 0.1, 0.25]
Z_FOCUS = [0.0, 1.3, -0.7]


def spectra(of, FieldViewer, out, prefix, na_list):
    # FieldViewer refocuses at z = 0 on construction (field_viewer.py:85); the spectra below are
    # computed from those fields (for the 2-D case they equal focused_0, which is not stored twice).
    fv = FieldViewer(of, cmf=np.zeros((len(of.get_wavelengths()), 3)))
    if prefix:
        out[prefix + "viewer_focused"] = of.focused_vals.copy()
    else:
        assert np.array_equal(of.focused_vals, out["focused_0"])
    for i, st in enumerate(SETTINGS):
        (fv.polariser, fv.polariser_angle, fv.analyser, fv.analyser_angle, fv.lower_waveplate,
         fv.lower_waveplate_angle, fv.upper_waveplate, fv.upper_waveplate_angle) = st
        for j, na in enumerate(na_list):
            fv.NA_condenser = na
            fv._update_specter()
            fv._update_averaged_specter()
            out["%sspectrum_%d_%d" % (prefix, i, j)] = np.array(fv._q_averaged_specter, dtype=np.float64).copy()


def main():
    OpticalFields, FieldViewer = load_reference()
    rng = np.random.default_rng(7)
    Nx, Ny, dx, dy = 10, 9, 0.25, 0.3
    wl = np.array([0.5, 0.62])
    nout = np.array([1.0, 1.05])
    of = OpticalFields(wavelengths=wl, max_NA_objective=0.45, max_NA_condenser=0.3, N_radial_wavevectors=3,
                       mesh_lengths=(dx * (Nx - 1), dy * (Ny - 1)), mesh_dimensions=(Nx, Ny), n_out=nout,
                       zfoc_NA_corr=0.3)
    shape = of.vals.shape
    vals = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    of.vals = vals
    out = {"vals": vals, "wavelengths": wl, "n_out": nout, "wavevectors": of.get_wavevectors(),
           "Nx": Nx, "Ny": Ny, "dx": dx, "dy": dy, "max_NA_objective": 0.45, "max_NA_condenser": 0.3,
           "N_radial": 3, "zfoc_NA_corr": 0.3, "z_focus": np.array(Z_FOCUS)}
    for k, z in enumerate(Z_FOCUS):
        of.update_NA_objective(0.45 if k != 1 else 0.35)
        of.focus_fields(z)
        out["focused_%d" % k] = of.focused_vals.copy()
        out["na_objective_%d" % k] = of._NA
    of.update_NA_objective(0.45)
    spectra(of, FieldViewer, out, "", NA_CONDENSER)

    # Koehler 1-D illumination of a 1-D mesh (Ny = 1): 2*Nr-1 wavevectors along x.
    k1 = OpticalFields(wavelengths=wl, max_NA_objective=0.4, max_NA_condenser=0.2, N_radial_wavevectors=3,
                       koehler_1D=True, mesh_lengths=(0.2 * 13, 0.5), mesh_dimensions=(14, 1), n_out=1.0,
                       zfoc_NA_corr=0.0)
    kv = rng.normal(size=k1.vals.shape) + 1j * rng.normal(size=k1.vals.shape)
    k1.vals = kv
    out.update({"k1_vals": kv, "k1_wavevectors": k1.get_wavevectors()})
    k1.focus_fields(0.8)
    out["k1_focused"] = k1.focused_vals.copy()
    spectra(k1, FieldViewer, out, "k1_", [0.0, 0.07, 0.15, 0.2])
    np.savez_compressed(os.path.join(HERE, "micrograph_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "micrograph_golden.npz"))


if __name__ == "__main__":
    if len(sys.argv) != 2 or not os.path.isdir(os.path.join(sys.argv[1], "HighLevelPythonInterface")):
        raise SystemExit("usage: python make_golden.py <root of a Nemaktis checkout>")
    REF = os.path.abspath(sys.argv[1])
    main()
