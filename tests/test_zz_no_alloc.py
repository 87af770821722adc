"""GPU test of the allocation-free periodic line solve (nbpm_periodic_tridiag_solve_noalloc).

Callers that run real-time loops that must not go through the device allocator, or that hand
the whole device memory to their own pool, cannot let the library call cudaMalloc. For them
the library offers a variant of the periodic line solve whose scratch is a fixed device array
reserved when the library loads. This test calls it through the C ABI twice in a row, with
different systems, and checks each result against the allocating entry point on the same
inputs; it also checks that sizes above the fixed scratch are refused with a clear error. It
lives in a file of its own that pytest collects last."""
import ctypes

import numpy as np
import pytest

from nemaktis_gb300 import _lib

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative L2, the tolerance of the periodic line-solve tests


def systems(L, nlines, seed):
    rng = np.random.default_rng(seed)
    shape = (nlines, L)
    inf = 0.15 * (rng.normal(size=shape) + 1j * rng.normal(size=shape))
    sup = 0.15 * (rng.normal(size=shape) + 1j * rng.normal(size=shape))
    mid = 1 + 0.3j * rng.normal(size=shape) + 0.05 * rng.normal(size=shape)
    rhs = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    return inf, mid, sup, rhs


def solve(fn, arrays):
    torch = pytest.importorskip("torch")
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrays]
    x = torch.zeros_like(dev[3])
    L, n = arrays[3].shape[1], arrays[3].shape[0]
    _lib.check(fn(L, n, *[ctypes.c_void_p(t.data_ptr()) for t in dev], ctypes.c_void_p(x.data_ptr()), None))
    torch.cuda.synchronize()
    return x.cpu().numpy()


def test_noalloc_matches_allocating_solve_twice(gpu):
    for call, (L, nlines) in enumerate([(257, 96), (65, 300)]):
        arrays = systems(L, nlines, seed=100 + call)
        ref = solve(gpu.nbpm_periodic_tridiag_solve, arrays)
        out = solve(gpu.nbpm_periodic_tridiag_solve_noalloc, arrays)
        assert np.isfinite(out).all()
        assert np.linalg.norm(out - ref) / np.linalg.norm(ref) <= TOL


def test_noalloc_rejects_sizes_above_its_scratch(gpu):
    L, nlines = 1025, 600  # 5*600*1024 + 1200 > 2*1024*1024
    rc = gpu.nbpm_periodic_tridiag_solve_noalloc(L, nlines, *([ctypes.c_void_p(1)] * 5), None)
    assert rc == 2
    assert b"fixed" in gpu.nbpm_last_error() and b"maximum" in gpu.nbpm_last_error()
