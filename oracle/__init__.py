"""CPU oracle for the Nemaktis bpm-solver backend path.

TEST INFRASTRUCTURE ONLY. Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU
baseline leg import this package; the nemaktis_gb300 product never does.

Parity status: UNPINNED against the reference binary (the reference cannot be compiled
here: Eigen, FFTW, muParser, Boost and VTK are absent, and it ships no golden vectors for
this path). The restatement is checked by physical invariants, by the analytic
uniform-crystal propagator of the reference's benchmark scripts, and its FFT against
numpy.fft. The Python tail (objective focalisation, incoherent spectra) is pinned against
the reference's own Python code by the fixtures in tests/golden/.

``run_backend_without_mask`` / ``run_backend_with_mask`` mirror the reference entry points
(BeamPropagationSolver/src/PythonBackend/bpm_backend.cpp:7-83, 85-164): JSON settings and
float64 director/mask arrays in, complex128 fields of shape (Nl, Nq, 4, Ny, Nx) written in
place.
"""
import ctypes
import os
import subprocess

import numpy as np

from . import settings as _settings
from .expr import evaluate

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


def build(force=False):
    """Compile oracle/_build/liboracle.so with the committed Makefile."""
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "nbpm_oracle.cpp")):
        subprocess.run(["make", "-s", "-C", _HERE, "_build/liboracle.so"], check=True)
    return _LIB_PATH


class _Params(ctypes.Structure):
    _fields_ = [
        ("Nx", ctypes.c_int), ("Ny", ctypes.c_int), ("Nz", ctypes.c_int),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
        ("field_dim", ctypes.c_int), ("n_woodbury", ctypes.c_int), ("beam_type", ctypes.c_int),
        ("waist", ctypes.c_double),
        ("n_wavelengths", ctypes.c_int), ("wavelengths", ctypes.POINTER(ctypes.c_double)),
        ("no", ctypes.POINTER(ctypes.c_double)), ("ne", ctypes.POINTER(ctypes.c_double)),
        ("ne_imag", ctypes.POINTER(ctypes.c_double)), ("nhost", ctypes.POINTER(ctypes.c_double)),
        ("nin", ctypes.POINTER(ctypes.c_double)), ("nout", ctypes.POINTER(ctypes.c_double)),
        ("n_q", ctypes.c_int), ("q", ctypes.POINTER(ctypes.c_double)),
        ("n_iso", ctypes.c_int), ("iso_thick", ctypes.POINTER(ctypes.c_double)),
        ("iso_index", ctypes.POINTER(ctypes.c_double)),
        ("z_foc", ctypes.c_double), ("numerical_aperture", ctypes.c_double),
        ("nout_06", ctypes.c_double),
    ]


def _load():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB_PATH)
        _lib.oracle_run.restype = ctypes.c_int
        _lib.oracle_run.argtypes = [ctypes.POINTER(_Params), ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        _lib.oracle_run_bulk.restype = ctypes.c_int
        _lib.oracle_run_bulk.argtypes = [ctypes.POINTER(_Params), ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        _lib.oracle_fft1d.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        _lib.oracle_num_threads.restype = ctypes.c_int
    return _lib


def num_threads():
    return _load().oracle_num_threads()


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def mask_interp_weights(mask_vals, formula, dims, spacings):
    """Boolean mask and per-cell z interpolation weights.

    Restates VectorField.cpp:43-114: mask = (mask_val >= 0); where the formula changes sign
    inside a z-cell, bisection to 1e-3*dz gives w0 = (z* - z_i)/dz, w1 = 1 - w0; otherwise
    0.5/0.5. If a sign change contradicts the mask values the reference falls back to the
    defaults (its resize at :111 is ill-formed, see the quirk list; the intended all-0.5
    weights are used here). Returns (mask uint8 (Nz,Ny,Nx), weights float64 (Nz-1,Ny,Nx,2)).
    """
    Nx, Ny, Nz = dims
    dx, dy, dz = spacings
    m = (np.asarray(mask_vals, float).reshape(Nz, Ny, Nx) >= 0)
    w = np.full((max(Nz - 1, 0), Ny, Nx, 2), 0.5)
    if not formula or Nz < 2:
        return m.astype(np.uint8), w
    x = ((np.arange(Nx) - 0.5 * (Nx - 1)) * dx)[None, :]
    y = ((np.arange(Ny) - 0.5 * (Ny - 1)) * dy)[:, None]
    X = np.broadcast_to(x, (Ny, Nx))
    Y = np.broadcast_to(y, (Ny, Nx))

    def f(zarr):
        return np.broadcast_to(np.asarray(evaluate(formula, x=X, y=Y, z=zarr), float), (Ny, Nx)).copy()

    failed = False
    for iz in range(Nz - 1):
        zi = (iz - 0.5 * (Nz - 1)) * dz
        zm = np.full((Ny, Nx), zi)
        zp = np.full((Ny, Nx), (iz + 1 - 0.5 * (Nz - 1)) * dz)
        fm = f(zm)
        fp = f(zp)
        cross = fm * fp <= 0
        if not cross.any():
            continue
        if np.any(cross & (m[iz] == m[iz + 1])):
            failed = True
        z = zm.copy()
        active = cross.copy()
        while active.any():
            active &= np.abs(zp - zm) >= 1e-3 * dz
            if not active.any():
                break
            fm_ = f(zm)
            zmid = 0.5 * (zp + zm)
            fmid = f(zmid)
            z = np.where(active, zmid, z)
            hit = active & (fmid == 0)
            lo = active & ~hit & (fmid * fm_ < 0)
            hi = active & ~hit & ~(fmid * fm_ < 0)
            zp = np.where(lo, zmid, zp)
            zm = np.where(hi, zmid, zm)
            active &= ~hit
        w0 = (z - zi) / dz
        w[iz, :, :, 0] = np.where(cross, w0, 0.5)
        w[iz, :, :, 1] = np.where(cross, 1 - w0, 0.5)
    if failed:
        w[:] = 0.5
    return m.astype(np.uint8), w


def _run(json_str, lc_vals, E, mask_vals=None, mask_formula="", stages=3, bulk=None):
    s = _settings.parse(json_str)
    Nx, Ny, Nz = s["dims"]
    nv = Nx * Ny * Nz
    lc = np.ascontiguousarray(np.asarray(lc_vals, dtype=np.float64).ravel())
    if lc.size != nv * (lc.size // nv):
        raise ValueError("Wrong dimension for the user pointer array (VectorField)")
    fd = lc.size // nv
    if fd not in (3, 6):
        raise ValueError("Unexpected dimension for the LC orientational field, should be 3 or 6.")
    Nl, Nq = len(s["wavelengths"]), len(s["q"])
    if not (isinstance(E, np.ndarray) and E.dtype == np.complex128 and E.flags.c_contiguous):
        raise TypeError("E must be a C-contiguous complex128 array")
    if E.size != Nl * Nq * 4 * Nx * Ny:
        raise ValueError("Wrong dimension for the user pointer array (OpticalFieldCollection)")
    if mask_vals is not None:
        mask, w = mask_interp_weights(mask_vals, mask_formula, s["dims"], s["spacings"])
        mask = np.ascontiguousarray(mask)
    else:
        mask = None
        w = np.full((max(Nz - 1, 0), Ny, Nx, 2), 0.5)
    w = np.ascontiguousarray(w)
    arrs = {k: np.ascontiguousarray(np.asarray(s[k + "_vals"], float)) for k in
            ("no", "ne", "ne_imag", "nhost", "nin", "nout")}
    lam = np.ascontiguousarray(np.asarray(s["wavelengths"], float))
    q = np.ascontiguousarray(np.asarray(s["q"], float).ravel())
    it = np.ascontiguousarray(np.asarray(s["iso_thick"] or [0.0], float))
    ii = np.ascontiguousarray(np.asarray(s["iso_index"] or [1.0], float))
    p = _Params(Nx, Ny, Nz, *s["spacings"], fd, s["n_woodbury"], s["beam_type"], s["waist"],
                Nl, _dptr(lam), _dptr(arrs["no"]), _dptr(arrs["ne"]), _dptr(arrs["ne_imag"]),
                _dptr(arrs["nhost"]), _dptr(arrs["nin"]), _dptr(arrs["nout"]),
                Nq, _dptr(q), len(s["iso_thick"]), _dptr(it), _dptr(ii),
                s["z_foc"], s["NA"], s["nout_06"])
    lib = _load()
    if bulk is not None:
        if not (bulk.dtype == np.complex128 and bulk.flags.c_contiguous and bulk.size == Nl * Nq * 2 * Nz * 2 * Nx * Ny):
            raise ValueError("bulk must be a C-contiguous complex128 (Nl, Nq, 2, Nz, 2, Ny, Nx) array")
    rc = lib.oracle_run_bulk(ctypes.byref(p), lc.ctypes.data,
                             None if mask is None else mask.ctypes.data, w.ctypes.data,
                             E.ctypes.data, stages, None if bulk is None else bulk.ctypes.data)
    if rc != 0:
        raise RuntimeError("oracle failed")
    return s


def run_backend_without_mask(json_str, lc_vals, E, stages=3, bulk=None):
    """In-place on E (complex128, (Nl,Nq,4,Ny,Nx)); stages bit0 = z-loop, bit1 = screen filter.
    bulk: optional (Nl, Nq, 2, Nz, 2, Ny, Nx) complex128 array receiving every plane's fields
    (the bulk output of BPMIteration.cpp:111-121, 153-168)."""
    return _run(json_str, lc_vals, E, stages=stages, bulk=bulk)


def run_backend_with_mask(json_str, mask_formula, lc_vals, mask_vals, E, stages=3):
    return _run(json_str, lc_vals, E, mask_vals=mask_vals, mask_formula=mask_formula, stages=stages)


def fft1d(x, sign=-1):
    """Unnormalised DFT of a complex line with the oracle's own mixed-radix transform."""
    a = np.ascontiguousarray(np.asarray(x, np.complex128)).copy()
    _load().oracle_fft1d(a.ctypes.data, a.size, sign)
    return a
