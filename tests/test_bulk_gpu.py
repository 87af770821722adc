"""Bulk output (fields of every transverse plane, BPMIteration.cpp:111-121, 153-168) written as
a .vti file by the GPU backend, against the oracle's record of the same planes."""
import os

import numpy as np
import pytest

import oracle
from nemaktis_gb300 import api, workloads
from vti import read_vti

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def bulk_from_vti(d, Nl, Nq, Nx, Ny, Nz):
    out = np.zeros((Nl, Nq, 2, Nz, 2, Ny, Nx), np.complex128)
    for w in range(Nl):
        for q in range(Nq):
            for pol, tag in enumerate(("inputX_", "inputY_")):
                re_ = d["arrays"]["E_real_%s%d_%d" % (tag, q, w)]
                im_ = d["arrays"]["E_imag_%s%d_%d" % (tag, q, w)]
                assert re_.shape == (Nx * Ny * Nz, 3) and not re_[:, 2].any() and not im_[:, 2].any()
                v = (re_[:, :2] + 1j * im_[:, :2]).reshape(Nz, Ny, Nx, 2)
                out[w, q, pol] = v.transpose(0, 3, 1, 2)
    return out


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-4)])
@pytest.mark.parametrize("gpp", [0, 1])
def test_bulk_output_vs_oracle(gpu, tmp_path, precision, tol, gpp):
    Nx, Ny, Nz = 24, 20, 7
    q = [(0.0, 0.0), (0.06, -0.04)]
    wl = [0.5, 0.62]
    folder = str(tmp_path / "res")
    js = workloads.settings_json((Nx, Ny, Nz), (0.25, 0.3, 0.25), wl, q, no="1.5", ne="1.7",
                                 bulk_name="bulk_test", results_folder=folder)
    lc = workloads.random_smooth((Nx, Ny, Nz), seed=11)
    E = np.zeros((2, 2, 4, Ny, Nx), np.complex128)
    api.run(js, lc, E, precision=precision, groups_per_pass=gpp)
    path = os.path.join(folder, "bulk_test.vti")
    assert os.path.exists(path)
    d = read_vti(path)
    assert d["dims"] == (Nx, Ny, Nz)
    np.testing.assert_allclose(d["spacing"], [0.25, 0.3, 0.25])
    np.testing.assert_allclose(d["origin"], [-0.25 * (Nx - 1) / 2, -0.3 * (Ny - 1) / 2, -0.25 * (Nz - 1) / 2])
    np.testing.assert_allclose(d["arrays"]["lambda"], wl)
    np.testing.assert_allclose(d["arrays"]["qx"], [v[0] for v in q])
    got = bulk_from_vti(d, 2, 2, Nx, Ny, Nz)
    ref_bulk = np.zeros_like(got)
    E_ref = np.zeros_like(E)
    oracle.run_backend_without_mask(js, lc, E_ref, stages=3, bulk=ref_bulk)
    assert rel(got, ref_bulk) < tol
    assert rel(E, E_ref) < tol
