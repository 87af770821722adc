"""GPU test of the periodic tridiagonal line-solve primitive (nbpm_periodic_tridiag_solve)
against a dense solve of the same periodic systems."""
import ctypes

import numpy as np
import pytest

from nemaktis_gb300 import _lib

pytestmark = pytest.mark.gpu


def periodic_systems(L, nlines, seed=0):
    """Diagonally dominant complex periodic systems like those of the ADI half-steps."""
    rng = np.random.default_rng(seed)
    shape = (nlines, L)
    inf = 0.15 * (rng.normal(size=shape) + 1j * rng.normal(size=shape))
    sup = 0.15 * (rng.normal(size=shape) + 1j * rng.normal(size=shape))
    mid = 1 + 0.3j * rng.normal(size=shape) + 0.05 * rng.normal(size=shape)
    rhs = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    return inf, mid, sup, rhs


def dense_reference(inf, mid, sup, rhs):
    nlines, L = rhs.shape
    n = L - 1
    out = np.empty_like(rhs)
    for l in range(nlines):
        A = np.zeros((n, n), complex)
        for i in range(n):
            A[i, (i - 1) % n] += inf[l, i]
            A[i, i] += mid[l, i]
            A[i, (i + 1) % n] += sup[l, i]
        x = np.linalg.solve(A, rhs[l, :n])
        out[l, :n] = x
        out[l, n] = x[0]
    return out


def gpu_solve(fn, inf, mid, sup, rhs):
    torch = pytest.importorskip("torch")
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (inf, mid, sup, rhs)]
    x = torch.zeros_like(dev[3])
    L, n = rhs.shape[1], rhs.shape[0]
    rc = fn(L, n, *[ctypes.c_void_p(t.data_ptr()) for t in dev], ctypes.c_void_p(x.data_ptr()), None)
    _lib.check(rc)
    torch.cuda.synchronize()
    return x.cpu().numpy()


@pytest.mark.parametrize("L,nlines", [(4, 3), (17, 40), (257, 64)])
def test_periodic_tridiag_solve_matches_dense(gpu, L, nlines):
    inf, mid, sup, rhs = periodic_systems(L, nlines, seed=L)
    x = gpu_solve(gpu.nbpm_periodic_tridiag_solve, inf, mid, sup, rhs)
    ref = dense_reference(inf, mid, sup, rhs)
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-12


def test_periodic_tridiag_rejects_bad_sizes(lib):
    assert lib.nbpm_periodic_tridiag_solve(3, 1, None, None, None, None, None, None) == 6
