"""Objective focalisation and micrograph spectra on the GPU (FP64), mirroring the reference's
OpticalFields / FieldViewer post-processing.

    OpticalFields   HighLevelPythonInterface/nemaktis/light_propagator.py:420-845
                    (constructor :448-646, update_NA_objective :702-705, focus_fields :708-719)
    FieldViewer     nemaktis/field_viewer.py (update_image :341-345 without the colour step,
                    _update_specter :348-388, _update_averaged_specter :391-455,
                    get_spectrum :335-338)

Both run through libnbpm's nbpm_microscope_* entry points; nothing here computes on the CPU.
The spectrum -> RGB conversion of _update_POM_image needs dtmm's colour tables and is not
provided: FieldViewer.update_image stops at the q-averaged spectrum.
"""
import ctypes

import numpy as np

from . import _lib


class OpticalFields:
    """Field container with the reference's constructor keywords (mesh_dimensions,
    mesh_lengths, wavelengths, max_NA_objective, max_NA_condenser=0, N_radial_wavevectors=1,
    koehler_1D=False, n_out=1, zfoc_NA_corr=0) plus wavevectors= (explicit (Nq, 2) list,
    e.g. the one given to the backend) and device=. The vti_file constructor is not provided."""

    def __init__(self, **kw):
        if "vti_file" in kw:
            raise NotImplementedError("OpticalFields(vti_file=...) is not provided; set vals instead")
        dims = np.array(kw["mesh_dimensions"])
        lengths = np.array(kw["mesh_lengths"], dtype=np.float64)
        if len(dims) != 2:
            raise Exception("mesh_dimensions should be an array-like object of size 2")
        if len(lengths) != 2:
            raise Exception("mesh_lengths should be an array-like object of size 2")
        self._wavelengths = np.atleast_1d(np.array(kw["wavelengths"], dtype=np.float64))
        Nl = len(self._wavelengths)
        self._n_out_arg = kw.get("n_out", 1)
        self._n_out = np.ascontiguousarray(np.broadcast_to(np.asarray(self._n_out_arg, np.float64), (Nl,)))
        self._zfoc_NA_corr = float(kw.get("zfoc_NA_corr", 0))
        self._max_NA_objective = float(kw["max_NA_objective"])
        self._max_NA_condenser = float(kw.get("max_NA_condenser", 0))
        self._N_radial_wavevectors = int(kw.get("N_radial_wavevectors", 1))
        self._koehler_1D = bool(kw.get("koehler_1D", False))
        self._NA = self._max_NA_objective
        self._z = 0
        (self._Nx, self._Ny) = (int(dims[0]), int(dims[1]))
        (self._Lx, self._Ly) = (float(lengths[0]), float(lengths[1]))
        (self._dx, self._dy) = tuple(lengths / np.maximum(np.ones(2), dims - 1))
        q = kw.get("wavevectors")
        qarr = None if q is None else np.ascontiguousarray(np.asarray(q, np.float64).reshape(-1, 2))
        self._device = int(kw.get("device", 0))
        self._wl_c = np.ascontiguousarray(self._wavelengths)
        p = _lib.MicroscopeParams()
        p.Nx, p.Ny, p.Lx, p.Ly = self._Nx, self._Ny, self._Lx, self._Ly
        p.n_wavelengths = Nl
        p.wavelengths = self._wl_c.ctypes.data
        p.n_out = self._n_out.ctypes.data
        p.max_NA_objective, p.max_NA_condenser = self._max_NA_objective, self._max_NA_condenser
        p.N_radial_wavevectors, p.koehler_1D = self._N_radial_wavevectors, int(self._koehler_1D)
        p.zfoc_NA_corr = self._zfoc_NA_corr
        p.n_wavevectors = 0 if qarr is None else len(qarr)
        p.wavevectors = None if qarr is None else qarr.ctypes.data
        p.device = self._device
        lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(lib.nbpm_microscope_create(ctypes.byref(p), ctypes.byref(h)))
        self._h = h
        nl, nq, ny, nx = (ctypes.c_int() for _ in range(4))
        _lib.check(lib.nbpm_microscope_shape(h, ctypes.byref(nl), ctypes.byref(nq), ctypes.byref(ny), ctypes.byref(nx)))
        self._wavevectors = np.zeros((nq.value, 2))
        _lib.check(lib.nbpm_microscope_wavevectors(h, self._wavevectors.ctypes.data, nq.value))
        if self._N_radial_wavevectors > 1 and self._max_NA_condenser > 0:
            self._delta_qr = self._max_NA_condenser / (self._N_radial_wavevectors - 1)
        else:
            self._delta_qr = 1
        shape = (Nl, nq.value, 4, self._Ny, self._Nx)
        self._vals = np.zeros(shape, np.complex128)
        self._focused = np.zeros(shape, np.complex128)
        self._vals_dirty = False      # host vals newer than the device copy
        self._focused_stale = False   # device focused newer than the host copy

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.load().nbpm_microscope_destroy(h)
            self._h = None

    def copy(self):
        new = OpticalFields(wavelengths=self._wavelengths, max_NA_objective=self._max_NA_objective,
                            max_NA_condenser=self._max_NA_condenser, N_radial_wavevectors=self._N_radial_wavevectors,
                            koehler_1D=self._koehler_1D, zfoc_NA_corr=self._zfoc_NA_corr, n_out=self._n_out_arg,
                            mesh_dimensions=(self._Nx, self._Ny), mesh_lengths=(self._Lx, self._Ly),
                            wavevectors=self._wavevectors, device=self._device)
        new.vals = self.vals
        return new

    # --- fields -------------------------------------------------------------------------
    @property
    def vals(self):
        """(N_wavelengths, N_wavevectors, 4, Ny, Nx) complex128 fields. The array may be
        modified in place (e.g. by the backend call); the next focus_fields uploads it."""
        self._vals_dirty = True
        return self._vals

    @vals.setter
    def vals(self, fields_ndarray):
        if self._vals.shape == np.shape(fields_ndarray):
            self._vals[:] = fields_ndarray
            self._vals_dirty = True
        else:
            raise Exception("Wrong shape for the optical field ndarray")

    def set_vals_from_plan(self, plan, sample=0):
        """Take the fields of an executed nemaktis_gb300.api.Plan directly from device memory."""
        _lib.check(_lib.load().nbpm_microscope_set_fields_from_plan(self._h, plan._h, int(sample)))
        self._vals_dirty = False

    @property
    def focused_vals(self):
        if self._focused_stale:
            _lib.check(_lib.load().nbpm_microscope_get_focused(self._h, self._focused.ctypes.data, self._focused.size))
            self._focused_stale = False
        return self._focused

    @property
    def z_focus(self):
        return self._z

    def update_NA_objective(self, new_NA):
        self._NA = max(0, min(self._max_NA_objective, new_NA))

    def focus_fields(self, z_focus=None):
        if z_focus is not None:
            self._z = z_focus
        lib = _lib.load()
        if self._vals_dirty:
            _lib.check(lib.nbpm_microscope_set_fields(self._h, self._vals.ctypes.data, self._vals.size))
            self._vals_dirty = False
        _lib.check(lib.nbpm_microscope_focus(self._h, float(self._z), float(self._NA)))
        self._focused_stale = True

    def timing(self):
        """(focus ms, spectrum ms, device bytes) of the last calls."""
        f, s, b = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        _lib.check(_lib.load().nbpm_microscope_timing(self._h, ctypes.byref(f), ctypes.byref(s), ctypes.byref(b)))
        return f.value, s.value, b.value

    # --- accessors of the reference --------------------------------------------------------
    def get_pos(self, ix, iy):
        return np.array([ix * self._dx - self._Lx / 2, iy * self._dy - self._Ly / 2])

    def get_wavelengths(self):
        return self._wavelengths

    def get_wavevectors(self):
        return self._wavevectors

    def get_mesh_dimensions(self):
        return (self._Nx, self._Ny)

    def get_mesh_lengths(self):
        return (self._Lx, self._Ly)

    def get_mesh_spacings(self):
        return (self._dx, self._dy)

    def get_qr_index(self, NA_condenser):
        return int(np.ceil(NA_condenser / self._delta_qr))

    def get_delta_qr(self):
        return self._delta_qr


class FieldViewer:
    """Spectrum part of the reference's FieldViewer: optical elements as attributes
    (polariser, analyser: bool; *_angle in degrees; upper/lower_waveplate in "No",
    "Quarter-wave", "Half-wave", "Tint-sensitive"; NA_condenser), update_image() computes the
    q-averaged spectrum on the GPU, get_spectrum() returns it tiled and flipped as the
    reference does. No GUI and no colour conversion."""

    polariser = True
    analyser = True
    upper_waveplate = "No"
    lower_waveplate = "No"
    polariser_angle = 0
    analyser_angle = 90
    upper_waveplate_angle = 0
    lower_waveplate_angle = 0
    NA_condenser = 0
    n_tiles_x = 1
    n_tiles_y = 1

    def __init__(self, optical_fields):
        if not isinstance(optical_fields, OpticalFields):
            raise TypeError("optical_fields should be an OpticalFields object")
        self._optical_fields = optical_fields
        optical_fields.focus_fields(0)
        shape = optical_fields._vals.shape
        self._q_averaged_specter = np.zeros((shape[3], shape[4], shape[0]))

    @property
    def z_focus(self):
        return self._optical_fields.z_focus

    @z_focus.setter
    def z_focus(self, new_z):
        self._optical_fields.focus_fields(new_z)

    @property
    def NA_objective(self):
        return self._optical_fields._NA

    @NA_objective.setter
    def NA_objective(self, new_NA):
        self._optical_fields.update_NA_objective(new_NA)
        self._optical_fields.focus_fields()

    def settings(self):
        s = _lib.ViewerSettings()
        _lib.load().nbpm_default_viewer_settings(ctypes.byref(s))
        s.polariser, s.polariser_angle = int(bool(self.polariser)), float(self.polariser_angle)
        s.analyser, s.analyser_angle = int(bool(self.analyser)), float(self.analyser_angle)
        s.lower_waveplate = _lib.WAVEPLATES[self.lower_waveplate]
        s.lower_waveplate_angle = float(self.lower_waveplate_angle)
        s.upper_waveplate = _lib.WAVEPLATES[self.upper_waveplate]
        s.upper_waveplate_angle = float(self.upper_waveplate_angle)
        s.NA_condenser = float(self.NA_condenser)
        return s

    def update_image(self):
        """_update_specter + _update_averaged_specter on the GPU (colour step not provided)."""
        out = self._q_averaged_specter
        s = self.settings()
        _lib.check(_lib.load().nbpm_microscope_spectrum(self._optical_fields._h, ctypes.byref(s), out.ctypes.data,
                                                        out.size))

    def get_spectrum(self):
        return np.flip(np.tile(self._q_averaged_specter, (self.n_tiles_y, self.n_tiles_x, 1)), axis=0)
