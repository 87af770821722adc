"""Continuous-batching request server (nbpm_server_*): several samples in flight on one GPU,
admitted under a device-memory budget and advanced slab by slab side by side.

    srv = Server(precision="fp32", hbm_budget_gb=150)
    req = srv.submit(json_str, director, E)        # E: (Nl, Nq, 4, Ny, Nx) complex128, written on completion
    info = req.wait()                              # {"state": "done", "latency_ms": ..., ...}

Requests use the backend's JSON settings and arrays (the arguments of
bpm_backend.run_backend_without_mask / _with_mask). A request's result equals a standalone
run of the same precision bit for bit.
"""
import ctypes

import numpy as np

from . import _lib


def _info_dict(i):
    return {"state": _lib.REQ_STATES.get(i.state, i.state), "error_code": i.error_code,
            "error": i.error.decode("utf-8", "replace"), "voxel_steps": i.voxel_steps,
            "device_bytes": i.device_bytes, "queue_ms": i.queue_ms, "latency_ms": i.latency_ms}


class Request:
    def __init__(self, server, rid, keep):
        self._server = server
        self.id = rid
        self._keep = keep  # host buffers borrowed by the library until the request finishes

    def poll(self):
        i = _lib.RequestInfo()
        _lib.check(_lib.load().nbpm_server_poll(self._server._h, self.id, ctypes.byref(i)))
        return _info_dict(i)

    def wait(self, timeout=None):
        i = _lib.RequestInfo()
        _lib.check(_lib.load().nbpm_server_wait(self._server._h, self.id, -1.0 if timeout is None else float(timeout),
                                                ctypes.byref(i)))
        d = _info_dict(i)
        if d["state"] in ("done", "failed", "cancelled"):
            self._keep = None
        if d["state"] == "failed":
            raise _lib.NbpmError(d["error_code"], d["error"])
        return d

    def cancel(self):
        _lib.check(_lib.load().nbpm_server_cancel(self._server._h, self.id))


class Server:
    def __init__(self, precision="fp32", hbm_budget_gb=150.0, slabs_per_round=8, max_active=0, device=0,
                 round_voxel_steps=4e8):
        lib = _lib.load()
        o = _lib.ServerOptions()
        lib.nbpm_default_server_options(ctypes.byref(o))
        o.precision = {"fp64": _lib.FP64, "fp32": _lib.FP32}[precision]
        o.hbm_budget_gb = float(hbm_budget_gb)
        o.slabs_per_round = int(slabs_per_round)
        o.max_active = int(max_active)
        o.round_voxel_steps = float(round_voxel_steps)
        o.device = int(device)
        h = ctypes.c_void_p()
        _lib.check(lib.nbpm_server_create(ctypes.byref(o), ctypes.byref(h)))
        self._h = h

    def submit(self, json_str, lc, E, mask=None, formula=None):
        if not (isinstance(E, np.ndarray) and E.dtype == np.complex128 and E.flags.c_contiguous):
            raise TypeError("E must be a C-contiguous complex128 ndarray")
        lc = np.ascontiguousarray(np.asarray(lc, dtype=np.float64)).ravel()
        m = None if mask is None else np.ascontiguousarray(np.asarray(mask, dtype=np.float64)).ravel()
        js = json_str.encode() if isinstance(json_str, str) else json_str
        fm = None if formula is None else formula.encode()
        s = _lib.Sample(js, fm, lc.ctypes.data, lc.size, None if m is None else m.ctypes.data,
                        0 if m is None else m.size, E.ctypes.data, E.size)
        rid = ctypes.c_longlong()
        _lib.check(_lib.load().nbpm_server_submit(self._h, ctypes.byref(s), ctypes.byref(rid)))
        return Request(self, rid.value, (lc, m, E, js, fm))

    def stats(self):
        st = _lib.ServerStats()
        _lib.check(_lib.load().nbpm_server_get_stats(self._h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in _lib.ServerStats._fields_}

    def close(self):
        if self._h:
            _lib.load().nbpm_server_destroy(self._h)
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
