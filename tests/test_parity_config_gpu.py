"""GPU parity at the benchmark configurations' scale.

FP64 GPU vs the CPU oracle (<= 1e-10 relative L2 over the whole (Nl,Nq,4,Ny,Nx) result) on
downsized configurations that keep the production meshes' line lengths and slot counts, and
the FP32 batched mode against the FP64 mode (<= 1e-4 relative L2) on the full configurations:
the 512x512x128 cholesteric droplet with its mask formula, the 256x256x64 16-wavelength x
13-q Koehler workload and the 512x512x96 sample of the four-sample uneven workload."""
import numpy as np
import pytest

import oracle
from nemaktis_gb300 import api, workloads
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
FP32_TOL = 1e-4


def _oracle(js, lc, shape, mask=None, formula=None):
    ref = np.zeros(shape, np.complex128)
    if mask is None:
        oracle.run_backend_without_mask(js, lc, ref)
    else:
        oracle.run_backend_with_mask(js, formula or "", lc, mask, ref)
    return ref


def droplet_case(dims=(128, 128, 32), d=0.2, radius=10.0, q=((0.0, 0.0), (0.08, -0.05))):
    """The 512x512x128 droplet workload scaled down: cholesteric droplet (pitch 5 um) of radius 10 um in a 25.6 um box,
    nhost 1.55, mask formula r^2 - x^2 - y^2 - z^2, one normal and one tilted wave vector."""
    lc, mask, formula = workloads.cholesteric_droplet(dims=dims, d=d, radius=radius)
    js = workloads.settings_json(dims, (d, d, d), [0.55], np.asarray(q, float), no="1.5", ne="1.7",
                                 nhost="1.55", NA=1.0)
    return js, lc, mask, formula, (1, len(q), 4, dims[1], dims[0])


def test_droplet_128_mask_formula_fp64(gpu):
    js, lc, mask, formula, shape = droplet_case()
    ref = _oracle(js, lc, shape, mask, formula)
    out = np.zeros(shape, np.complex128)
    api.run(js, lc, out, mask=mask, formula=formula, precision="fp64")
    assert rel_l2(out, ref) <= FP64_TOL


def koehler_case(Nz=8, n_wavelengths=2):
    """The Koehler micrograph workload with its 256x256 planes, its 13-point hexagonal q grid and 2 polarisations
    (26 slots per wavelength, as in production), fewer wavelengths and planes."""
    c = workloads.koehler_micrograph(dims=(256, 256, Nz), n_wavelengths=n_wavelengths)
    return c["json"], c["lc"], c["shape"]


def test_koehler_256_fp64(gpu):
    js, lc, shape = koehler_case()
    ref = _oracle(js, lc, shape)
    out = np.zeros(shape, np.complex128)
    api.run(js, lc, out, precision="fp64")
    assert rel_l2(out, ref) <= FP64_TOL


def _fp32_vs_fp64(samples, k=0):
    e64 = np.zeros(samples[k]["shape"], np.complex128)
    s = samples[k]
    api.run(s["json"], s["lc"], e64, mask=s.get("mask"), formula=s.get("formula"), precision="fp64",
            groups_per_pass=1)
    bufs = [{"json": c["json"], "lc": c["lc"], "E": np.zeros(c["shape"], np.complex128), "mask": c.get("mask"),
             "formula": c.get("formula")} for c in samples]
    api.run_batch(bufs, precision="fp32")
    return rel_l2(bufs[k]["E"], e64)


def test_droplet_fp32_error_budget(gpu):
    assert _fp32_vs_fp64([workloads.droplet_cell()]) <= FP32_TOL


def test_koehler_fp32_error_budget(gpu):
    assert _fp32_vs_fp64([workloads.koehler_micrograph()]) <= FP32_TOL


def test_uneven_sample_fp32_error_budget(gpu):
    """The 512x512x96 sample of the uneven workload, run in FP32 in one batch with the 256x256x48
    sample (uneven sizes in one plan), against its FP64 plain run."""
    samples = [workloads.uneven_sample(2), workloads.uneven_sample(3)]
    assert _fp32_vs_fp64(samples, 0) <= FP32_TOL
