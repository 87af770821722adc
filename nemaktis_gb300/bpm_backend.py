"""Drop-in replacement for the reference's ``bpm_backend`` extension module.

The reference exposes two functions through SWIG (BeamPropagationSolver/src/PythonBackend/
bpm_backend.i:1-20, bpm_backend.h:4-13) and nemaktis calls them as
``bpm.run_backend_without_mask(json_str, lc_vals, output_fields.vals)`` and
``bpm.run_backend_with_mask(json_str, mask_formula, lc_vals, mask_vals, output_fields.vals)``
(HighLevelPythonInterface/nemaktis/light_propagator.py:226-228). Same names, argument
meaning and error behaviour here:

* ``lc_field_vals`` / ``mask_vals``: any array-like convertible to a 1-D float64 array
  (numpy.i IN_ARRAY1); a contiguous copy is made when needed.
* ``E_field_vals``: a C-contiguous complex128 ndarray of any shape (numpy.i
  INPLACE_ARRAY_FLAT), read (Beam profile "None") and overwritten in place with the screen
  fields, shape (Nl, Nq, 4, Ny, Nx).
* Errors inside the backend are printed to stderr in the reference's format and the call
  returns None, leaving the caller to continue (bpm_backend.cpp:48-82). Call
  ``set_strict(True)`` (or set NBPM_STRICT=1) to raise ``NbpmError`` instead.

The computation runs on the GPU through libnbpm.so; there is no CPU fallback.
``set_precision("fp32")`` switches to the batched FP32 mode (default "fp64").
``install()`` registers this module as ``bpm_backend`` so that ``import bpm_backend`` in
nemaktis resolves to it.
"""
import ctypes
import os
import sys

import numpy as np

from ._lib import FP32, FP64, NbpmError, Timing, check, load, options

_state = {"precision": FP64, "strict": os.environ.get("NBPM_STRICT", "0") == "1",
          "groups_per_pass": 0, "timing": None}


def set_precision(p):
    """"fp64" (reference parity, default) or "fp32" (mixed-precision batched mode)."""
    p = str(p).lower()
    if p not in ("fp64", "fp32"):
        raise ValueError("precision must be 'fp64' or 'fp32'")
    _state["precision"] = FP64 if p == "fp64" else FP32


def set_strict(flag=True):
    _state["strict"] = bool(flag)


def set_groups_per_pass(n):
    """Wavelengths propagated together per launch (0 = all, 1 = one at a time)."""
    _state["groups_per_pass"] = int(n)


def last_timing():
    """nbpm_timing of the last successful call, as a dict."""
    t = _state["timing"]
    if t is None:
        return None
    return {k: getattr(t, k) for k, _ in Timing._fields_}


def _in_array1(a, name):
    arr = np.asarray(a, dtype=np.float64)
    if arr.ndim != 1:
        raise TypeError("Array must have 1 dimensions.  Given array has %d dimensions" % arr.ndim)
    return np.ascontiguousarray(arr)


def _inplace_flat(a):
    if not isinstance(a, np.ndarray):
        raise TypeError("Array of type 'complex double' required.  A '%s' was given" % type(a).__name__)
    if a.dtype != np.complex128:
        raise TypeError("Array of type 'complex double' required.  Array of type '%s' given" % a.dtype)
    if not (a.flags.c_contiguous or a.flags.f_contiguous):
        raise TypeError("Array must be contiguous.  A non-contiguous array was given")
    if not a.flags.writeable:
        raise TypeError("Array must be writeable")
    return a


def _report(exc):
    msg = exc.msg if isinstance(exc, NbpmError) else str(exc)
    sys.stderr.write("\n\n-------------------------------------------------\n"
                     "Exception on processing: \n" + msg + "\nAborting!\n"
                     "-------------------------------------------------\n")
    sys.stderr.flush()


def _call(json_str, mask_formula, lc_field_vals, mask_vals, E_field_vals):
    lc = _in_array1(lc_field_vals, "lc_field_vals")
    mask = None if mask_vals is None else _in_array1(mask_vals, "mask_vals")
    E = _inplace_flat(E_field_vals)
    lib = load()
    opts = options(precision=_state["precision"], groups_per_pass=_state["groups_per_pass"])
    tm = Timing()
    try:
        rc = lib.nbpm_run_backend_ex(
            json_str.encode() if isinstance(json_str, str) else json_str,
            None if mask_formula is None else mask_formula.encode(),
            lc.ctypes.data, int(lc.size),
            None if mask is None else mask.ctypes.data, 0 if mask is None else int(mask.size),
            E.ctypes.data, int(E.size), ctypes.byref(opts), ctypes.byref(tm))
        check(rc)
        _state["timing"] = tm
    except NbpmError as e:
        if _state["strict"]:
            raise
        _report(e)
    return None


def run_backend_without_mask(json_str, lc_field_vals, E_field_vals):
    """bpm_backend.cpp:7-83."""
    return _call(json_str, None, lc_field_vals, None, E_field_vals)


def run_backend_with_mask(json_str, mask_formula, lc_field_vals, mask_vals, E_field_vals):
    """bpm_backend.cpp:85-164."""
    return _call(json_str, mask_formula if mask_formula is not None else "", lc_field_vals, mask_vals,
                 E_field_vals)


def install():
    """Make ``import bpm_backend`` return this module."""
    sys.modules["bpm_backend"] = sys.modules[__name__]
    return sys.modules[__name__]
