"""ctypes binding of libnbpm.so (declarations mirror include/nbpm.h).

The product path has no fallback: if the library cannot be loaded, or no CUDA device is
usable, calls fail with NbpmError instead of computing anything on the CPU.
"""
import ctypes
import os

from . import build as _build

c_int, c_double, c_char_p, c_void_p, c_ll = ctypes.c_int, ctypes.c_double, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_longlong

ERRORS = {0: "NBPM_OK", 1: "NBPM_ERR_SETTINGS", 2: "NBPM_ERR_SIZE", 3: "NBPM_ERR_EXPR", 4: "NBPM_ERR_CUDA",
          5: "NBPM_ERR_MEMORY", 6: "NBPM_ERR_ARG", 7: "NBPM_ERR_INTERNAL", 8: "NBPM_ERR_TIMEOUT"}
FP64, FP32 = 0, 1


class NbpmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (ERRORS.get(code, code), msg))
        self.code = code
        self.msg = msg


class Options(ctypes.Structure):
    _fields_ = [("precision", c_int), ("groups_per_pass", c_int), ("use_graph", c_int),
                ("device", c_int), ("verbose", c_int), ("tune", c_int), ("solve_config", c_char_p)]


class Timing(ctypes.Structure):
    _fields_ = [("upload_ms", c_double), ("compute_ms", c_double), ("download_ms", c_double),
                ("total_ms", c_double), ("voxel_steps", c_ll), ("kernel_launches", c_int)]


class Sample(ctypes.Structure):
    _fields_ = [("json_str", c_char_p), ("mask_formula", c_char_p), ("lc_field_vals", c_void_p),
                ("n_lc_vals", c_int), ("mask_vals", c_void_p), ("n_mask_vals", c_int),
                ("E_field_vals", c_void_p), ("n_E_vals", c_int)]


class MicroscopeParams(ctypes.Structure):
    _fields_ = [("Nx", c_int), ("Ny", c_int), ("Lx", c_double), ("Ly", c_double), ("n_wavelengths", c_int),
                ("wavelengths", c_void_p), ("n_out", c_void_p), ("max_NA_objective", c_double),
                ("max_NA_condenser", c_double), ("N_radial_wavevectors", c_int), ("koehler_1D", c_int),
                ("zfoc_NA_corr", c_double), ("n_wavevectors", c_int), ("wavevectors", c_void_p), ("device", c_int)]


class ViewerSettings(ctypes.Structure):
    _fields_ = [("polariser", c_int), ("polariser_angle", c_double), ("analyser", c_int),
                ("analyser_angle", c_double), ("lower_waveplate", c_int), ("lower_waveplate_angle", c_double),
                ("upper_waveplate", c_int), ("upper_waveplate_angle", c_double), ("NA_condenser", c_double)]


class ServerOptions(ctypes.Structure):
    _fields_ = [("precision", c_int), ("device", c_int), ("hbm_budget_gb", c_double), ("slabs_per_round", c_int),
                ("max_active", c_int), ("round_voxel_steps", c_double)]


class RequestInfo(ctypes.Structure):
    _fields_ = [("state", c_int), ("error_code", c_int), ("error", ctypes.c_char * 256), ("voxel_steps", c_ll),
                ("device_bytes", c_ll), ("queue_ms", c_double), ("latency_ms", c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("queued", c_int), ("running", c_int), ("done", c_ll), ("failed", c_ll), ("cancelled", c_ll),
                ("bytes_in_use", c_ll), ("peak_bytes", c_ll), ("budget_bytes", c_ll), ("voxel_steps_done", c_ll),
                ("rounds", c_int)]


REQ_STATES = {0: "queued", 1: "running", 2: "done", 3: "failed", 4: "cancelled"}

WAVEPLATES = {"No": 0, "Quarter-wave": 1, "Half-wave": 2, "Tint-sensitive": 3}

EXPORTS = {
    "nbpm_default_options": (None, [ctypes.POINTER(Options)]),
    "nbpm_release_plan_cache": (c_int, []),
    "nbpm_run_backend_without_mask": (c_int, [c_char_p, c_void_p, c_int, c_void_p, c_int]),
    "nbpm_run_backend_with_mask": (c_int, [c_char_p, c_char_p, c_void_p, c_int, c_void_p, c_int, c_void_p, c_int]),
    "nbpm_run_backend_ex": (c_int, [c_char_p, c_char_p, c_void_p, c_int, c_void_p, c_int, c_void_p, c_int,
                                    ctypes.POINTER(Options), ctypes.POINTER(Timing)]),
    "nbpm_run_batch": (c_int, [c_int, ctypes.POINTER(Sample), ctypes.POINTER(Options), ctypes.POINTER(Timing)]),
    "nbpm_plan_create": (c_int, [c_int, ctypes.POINTER(Sample), ctypes.POINTER(Options), ctypes.POINTER(c_void_p)]),
    "nbpm_plan_upload": (c_int, [c_void_p]),
    "nbpm_plan_execute": (c_int, [c_void_p, ctypes.POINTER(Timing)]),
    "nbpm_plan_download": (c_int, [c_void_p]),
    "nbpm_plan_slab_ms": (c_int, [c_void_p, ctypes.POINTER(c_double)]),
    "nbpm_plan_destroy": (c_int, [c_void_p]),
    "nbpm_plan_device_bytes": (c_ll, [c_void_p]),
    "nbpm_plan_profile": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, ctypes.POINTER(c_int)]),
    "nbpm_plan_solve_config": (c_int, [c_void_p, c_int, c_void_p, c_int, c_void_p, c_int]),
    "nbpm_solve_candidates": (c_int, [c_char_p, c_int, c_int, c_void_p, c_int]),
    "nbpm_tune_cache_clear": (c_int, []),
    "nbpm_eval_index": (c_int, [c_char_p, c_double, ctypes.POINTER(c_double)]),
    "nbpm_mask_weights": (c_int, [c_char_p, c_char_p, c_void_p, c_int, c_void_p, c_void_p]),
    "nbpm_periodic_tridiag_solve": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "nbpm_periodic_tridiag_solve_noalloc": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                                    c_void_p]),
    "nbpm_default_server_options": (None, [ctypes.POINTER(ServerOptions)]),
    "nbpm_server_create": (c_int, [ctypes.POINTER(ServerOptions), ctypes.POINTER(c_void_p)]),
    "nbpm_server_destroy": (c_int, [c_void_p]),
    "nbpm_server_submit": (c_int, [c_void_p, ctypes.POINTER(Sample), ctypes.POINTER(c_ll)]),
    "nbpm_server_poll": (c_int, [c_void_p, c_ll, ctypes.POINTER(RequestInfo)]),
    "nbpm_server_wait": (c_int, [c_void_p, c_ll, c_double, ctypes.POINTER(RequestInfo)]),
    "nbpm_server_cancel": (c_int, [c_void_p, c_ll]),
    "nbpm_server_release": (c_int, [c_void_p, c_ll]),
    "nbpm_server_get_stats": (c_int, [c_void_p, ctypes.POINTER(ServerStats)]),
    "nbpm_default_viewer_settings": (None, [ctypes.POINTER(ViewerSettings)]),
    "nbpm_microscope_create": (c_int, [ctypes.POINTER(MicroscopeParams), ctypes.POINTER(c_void_p)]),
    "nbpm_microscope_destroy": (c_int, [c_void_p]),
    "nbpm_microscope_shape": (c_int, [c_void_p, ctypes.POINTER(c_int), ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                                      ctypes.POINTER(c_int)]),
    "nbpm_microscope_wavevectors": (c_int, [c_void_p, c_void_p, c_int]),
    "nbpm_microscope_set_fields": (c_int, [c_void_p, c_void_p, c_ll]),
    "nbpm_microscope_set_fields_from_plan": (c_int, [c_void_p, c_void_p, c_int]),
    "nbpm_microscope_focus": (c_int, [c_void_p, c_double, c_double]),
    "nbpm_microscope_get_focused": (c_int, [c_void_p, c_void_p, c_ll]),
    "nbpm_microscope_spectrum": (c_int, [c_void_p, ctypes.POINTER(ViewerSettings), c_void_p, c_ll]),
    "nbpm_microscope_timing": (c_int, [c_void_p, ctypes.POINTER(c_double), ctypes.POINTER(c_double),
                                       ctypes.POINTER(c_ll)]),
    "nbpm_last_error": (c_char_p, []),
    "nbpm_version": (c_char_p, []),
}

_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libnbpm.so (building it first if needed); raise if it cannot be loaded."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing and _build._stale():
        _build.build()
    if not os.path.exists(path):
        raise NbpmError(4, "libnbpm.so is not built (%s)" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in EXPORTS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(rc):
    if rc != 0:
        msg = load().nbpm_last_error().decode("utf-8", "replace")
        raise NbpmError(rc, msg)
    return rc


def options(precision=FP64, groups_per_pass=0, use_graph=1, device=0, verbose=0, tune=1, solve_config=None):
    """nbpm_options; solve_config ("<x>;<y>", see solve_candidates) must stay referenced by the
    caller while the options are in use (ctypes keeps the bytes object alive on the struct)."""
    o = Options()
    load().nbpm_default_options(ctypes.byref(o))
    o.precision, o.groups_per_pass, o.use_graph, o.device, o.verbose = precision, groups_per_pass, use_graph, device, verbose
    o.tune = int(tune)
    o.solve_config = None if solve_config is None else solve_config.encode()
    return o


def solve_candidates(json_str, precision=FP64, groups_per_pass=0):
    """Candidate line-solve configurations for the settings' mesh and slots:
    {"x": [...], "y": [...], "default": "<x>;<y>"}."""
    buf = ctypes.create_string_buffer(8192)
    js = json_str.encode() if isinstance(json_str, str) else json_str
    check(load().nbpm_solve_candidates(js, precision, groups_per_pass, buf, len(buf)))
    out = {}
    for line in buf.value.decode().splitlines():
        k, v = line.split("=", 1)
        out[k] = v.split("|") if k in ("x", "y") else v
    return out
