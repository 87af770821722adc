"""Python front end of libnbpm beyond the reference's two entry points.

* ``run(json_str, lc, E, ...)``: one sample with explicit options, returns the timing dict.
* ``run_batch(samples, ...)``: several samples of uneven mesh size in one run.
* ``Plan``: validate and upload once, then execute on the device repeatedly (benchmarks).
Samples are dicts with keys ``json`` (str), ``lc`` (float64 array, (Nz,Ny,Nx,3|6)),
``E`` (C-contiguous complex128 array, (Nl,Nq,4,Ny,Nx)) and optionally ``mask`` (float64
(Nz,Ny,Nx)) and ``formula`` (mask formula string).
"""
import ctypes

import numpy as np

from ._lib import FP32, FP64, NbpmError, Sample, Timing, check, load, options


def _precision(p):
    if p in (FP64, FP32):
        return p
    return {"fp64": FP64, "fp32": FP32}[str(p).lower()]


def _timing_dict(t):
    return {k: getattr(t, k) for k, _ in Timing._fields_}


class _Samples:
    """Keeps the numpy buffers alive while C holds raw pointers to them."""

    def __init__(self, samples):
        self.keep = []
        self.arr = (Sample * len(samples))()
        for i, s in enumerate(samples):
            lc = np.ascontiguousarray(np.asarray(s["lc"], dtype=np.float64)).ravel()
            E = s["E"]
            if not (isinstance(E, np.ndarray) and E.dtype == np.complex128 and E.flags.c_contiguous):
                raise TypeError("E must be a C-contiguous complex128 ndarray")
            mask = s.get("mask")
            if mask is not None:
                mask = np.ascontiguousarray(np.asarray(mask, dtype=np.float64)).ravel()
            js = s["json"].encode() if isinstance(s["json"], str) else s["json"]
            fm = s.get("formula")
            fm = None if fm is None else fm.encode()
            self.keep += [lc, E, mask, js, fm]
            self.arr[i] = Sample(js, fm, lc.ctypes.data, lc.size,
                                 None if mask is None else mask.ctypes.data, 0 if mask is None else mask.size,
                                 E.ctypes.data, E.size)


def run(json_str, lc, E, mask=None, formula=None, precision="fp64", groups_per_pass=0, use_graph=True, tune=True,
        solve_config=None):
    return run_batch([{"json": json_str, "lc": lc, "E": E, "mask": mask, "formula": formula}],
                     precision, groups_per_pass, use_graph, tune, solve_config)


def run_batch(samples, precision="fp64", groups_per_pass=0, use_graph=True, tune=True, solve_config=None):
    """solve_config: None (tuned or rule-based line solves, see tune) or "<x>;<y>" forcing one of
    the candidates listed by _lib.solve_candidates for every sample."""
    S = _Samples(samples)
    o = options(precision=_precision(precision), groups_per_pass=groups_per_pass, use_graph=int(use_graph),
                tune=int(tune), solve_config=solve_config)
    t = Timing()
    check(load().nbpm_run_batch(len(samples), S.arr, ctypes.byref(o), ctypes.byref(t)))
    return _timing_dict(t)


class Plan:
    """Device-resident plan (nbpm_plan_*)."""

    def __init__(self, samples, precision="fp64", groups_per_pass=0, use_graph=True, tune=True, solve_config=None):
        self._S = _Samples(samples)
        self._lib = load()
        o = options(precision=_precision(precision), groups_per_pass=groups_per_pass, use_graph=int(use_graph),
                    tune=int(tune), solve_config=solve_config)
        h = ctypes.c_void_p()
        check(self._lib.nbpm_plan_create(len(samples), self._S.arr, ctypes.byref(o), ctypes.byref(h)))
        self._h = h

    def upload(self):
        check(self._lib.nbpm_plan_upload(self._h))

    def execute(self):
        t = Timing()
        check(self._lib.nbpm_plan_execute(self._h, ctypes.byref(t)))
        return _timing_dict(t)

    def download(self):
        check(self._lib.nbpm_plan_download(self._h))

    def solve_config(self, sample=0):
        """(configuration "<x>;<y>", how it was chosen) of one sample's line solves."""
        cfg = ctypes.create_string_buffer(256)
        rep = ctypes.create_string_buffer(4096)
        check(self._lib.nbpm_plan_solve_config(self._h, sample, cfg, len(cfg), rep, len(rep)))
        return cfg.value.decode(), rep.value.decode()

    def device_bytes(self):
        return int(self._lib.nbpm_plan_device_bytes(self._h))

    def close(self):
        if self._h:
            self._lib.nbpm_plan_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
