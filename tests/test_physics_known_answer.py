"""Known answer of the reference's BPM accuracy benchmark: a uniform crystal with its optic
axis at 45 degrees in the xz plane (ne 1.75, no 1.5), a Gaussian input beam of waist 0.5 um at
0.6 um, a 10 um cube, four Woodbury steps (HighLevelPythonInterface/examples/benchmarks/3D/
01_run_bpm_benchmarks.py:14-70). Every plane of the backend's bulk output is compared with the
exact forward propagation of its entrance plane (tests/exact_uniform.py) through the
benchmark's Fourier error measure. The reference documents about 1 % on fine meshes
(doc/source/intro/benchmarks.rst:149-154); the bounds below are those of the oracle on the
same meshes (N = 31: 8.7 %, 61: 3.0 %, 101: 1.64 %) with a small margin."""
import json
import os

import numpy as np
import pytest

import oracle
from exact_uniform import fourier_error, propagate
from nemaktis_gb300 import workloads

L, WL, NE, NO = 10.0, 0.6, 1.75, 1.5
THETA = np.pi / 4


def _case(N, **kw):
    d = L / (N - 1)
    js = workloads.settings_json((N, N, N), (d, d, d), [WL], [(0.0, 0.0)], no=str(NO), ne=str(NE), nhost=str(NO),
                                 nin=str(NO), n_woodbury=4, beam="GaussianBeam(0.5)", **kw)
    lc = np.zeros((N, N, N, 3))
    lc[..., 0] = np.sin(THETA)
    lc[..., 2] = np.cos(THETA)
    return js, lc, d


def _error(bpm, N, d):
    """bpm: (Nz, Ny, Nx, 2) planes for the x-polarised input."""
    a = np.array([np.sin(THETA), 0.0, np.cos(THETA)])
    eps = NO ** 2 * np.eye(3) + (NE ** 2 - NO ** 2) * np.outer(a, a)
    exact = propagate(bpm[0], eps, N, d, d, d, WL)
    # the backend's fields carry no k0*no*z phase
    exact = exact * np.exp(-2j * np.pi / WL * NO * np.arange(N) * d)[:, None, None, None]
    return fourier_error(exact, bpm, d, WL, NO)


def _oracle_error(N):
    js, lc, d = _case(N)
    E = np.zeros((1, 1, 4, N, N), complex)
    bulk = np.zeros((1, 1, 2, N, 2, N, N), complex)
    oracle.run_backend_without_mask(js, lc, E, stages=3, bulk=bulk)
    return _error(bulk[0, 0, 0].transpose(0, 2, 3, 1), N, d)


def test_oracle_against_exact_solution():
    e31, e61 = _oracle_error(31), _oracle_error(61)
    assert e61 < 0.033
    assert e31 < 0.095
    assert e61 < 0.5 * e31  # converges with the mesh


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gpu_against_exact_solution(gpu, tmp_path, precision):
    from nemaktis_gb300 import api, vti_io
    N = 101
    folder = str(tmp_path / "res")
    js, lc, d = _case(N, bulk_name="bulk", results_folder=folder)
    E = np.zeros((1, 1, 4, N, N), complex)
    api.run(js, lc, E, precision=precision)
    v = vti_io.read_vti(os.path.join(folder, "bulk.vti"))["point"]
    re_, im_ = v["E_real_inputX_0_0"], v["E_imag_inputX_0_0"]
    bpm = (re_[:, :2] + 1j * im_[:, :2]).reshape(N, N, N, 2)
    assert _error(bpm, N, d) < 0.018
