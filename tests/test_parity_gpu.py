"""GPU parity: the sm_103a kernels through the C ABI against the CPU oracle.

Tolerances: FP64 mode <= 1e-10 relative L2 over the whole (Nl,Nq,4,Ny,Nx) result; FP32 mode
<= 1e-4 relative L2 against the FP64 result."""
import numpy as np
import pytest

import oracle
from nemaktis_gb300 import _lib, api, bpm_backend, workloads
from tests.helpers import case, rand_director, rand_qtensor, rel_l2, uniform_jones

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
FP32_TOL = 1e-4


def _both(js, lc, shape, mask=None, formula=None, precision="fp64", stages=3, E0=None):
    ref = np.zeros(shape, np.complex128) if E0 is None else E0.copy()
    if mask is None:
        oracle.run_backend_without_mask(js, lc, ref, stages=stages)
    else:
        oracle.run_backend_with_mask(js, formula or "", lc, mask, ref, stages=stages)
    out = np.zeros(shape, np.complex128) if E0 is None else E0.copy()
    api.run(js, lc, out, mask=mask, formula=formula, precision=precision)
    return out, ref


CASES = {
    "random_q0": dict(dims=(16, 12, 8)),
    "random_tilted_q": dict(dims=(16, 14, 9), q=((0.0, 0.0), (0.12, -0.07), (-0.3, 0.25))),
    "two_wavelengths_dispersion": dict(dims=(12, 12, 6), wavelengths=(0.45, 0.7),
                                       no="1.52+0.008/lambda^2", ne="1.74+0.008/lambda^2"),
    "gaussian_beam": dict(dims=(20, 16, 7), beam="GaussianBeam(1.2)", q=((0.05, 0.05),)),
    "absorption": dict(dims=(12, 10, 6), ne_imag="0.02"),
    "woodbury4": dict(dims=(14, 14, 6), n_woodbury=4),
    "woodbury0": dict(dims=(14, 10, 5), n_woodbury=0),
    "iso_layers_focus": dict(dims=(16, 16, 6), iso_thick=(1.0, 2.0), iso_index=(1.4, 1.6), z_shift=0.7,
                             q=((0.0, 0.0), (0.1, 0.0)), NA=0.6),
    "nx3_invariant": dict(dims=(3, 16, 6)),
    "ny2_invariant": dict(dims=(16, 2, 6)),
    "odd_sizes": dict(dims=(15, 11, 5), q=((0.07, 0.02),)),
    "nz1": dict(dims=(8, 8, 1)),
    "nin_nout": dict(dims=(12, 12, 6), nin="1.3", nout="1.2"),
    # several warps per x-line (Nx - 1 > 256) and the long-y-line solve (Ny - 1 > 512)
    "long_x_lines": dict(dims=(300, 10, 4), q=((0.0, 0.0), (0.1, -0.05))),
    "long_x_lines_1030": dict(dims=(1030, 6, 3), q=((0.04, 0.02),)),
    "long_y_lines": dict(dims=(10, 530, 4), q=((0.0, 0.0), (-0.06, 0.09))),
    "sequential_x_lines": dict(dims=(2100, 5, 3), q=((0.03, 0.0),)),
    "tall_mesh": dict(dims=(12, 200, 5), q=((0.0, 0.0), (0.05, 0.08))),
    # many slots per wavelength (>= 4 chunks of two slots), Ny <= 3 with them
    "many_slots": dict(dims=(40, 24, 6), q=((0.0, 0.0), (0.1, 0.0), (0.0, 0.1), (-0.07, 0.05), (0.05, -0.12))),
    "many_slots_256": dict(dims=(256, 6, 4), q=((0.0, 0.0), (0.08, 0.0), (0.0, -0.08), (0.06, 0.06))),
    "many_slots_ny3": dict(dims=(40, 3, 4), q=((0.0, 0.0), (0.1, 0.0), (0.0, 0.1), (-0.07, 0.05))),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_parity(gpu, name):
    kw = dict(CASES[name])
    dims = kw.pop("dims")
    js, lc, shape = case(dims, seed=hash(name) % 1000, **kw)
    out, ref = _both(js, lc, shape)
    assert np.isfinite(out).all()
    assert rel_l2(out, ref) <= FP64_TOL


def test_fp64_parity_qtensor(gpu):
    dims = (14, 12, 7)
    lc = rand_qtensor(dims, 5)
    js, _, shape = case(dims, lc=lc, lc_type="Q-tensor", q=((0.0, 0.0), (0.1, 0.1)))
    out, ref = _both(js, lc, shape)
    assert rel_l2(out, ref) <= FP64_TOL


def test_fp64_parity_mask_formula(gpu):
    dims, d = (20, 18, 10), 0.3
    Nx, Ny, Nz = dims
    x = (np.arange(Nx) - 0.5 * (Nx - 1)) * d
    y = (np.arange(Ny) - 0.5 * (Ny - 1)) * d
    z = (np.arange(Nz) - 0.5 * (Nz - 1)) * d
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    formula = "2.4^2-x^2-y^2-z^2"
    mask = 2.4 ** 2 - X ** 2 - Y ** 2 - Z ** 2
    js, lc, shape = case(dims, spacings=(d, d, d), nhost="1.55", q=((0.0, 0.0), (0.1, 0.05)))
    out, ref = _both(js, lc, shape, mask=mask, formula=formula)
    assert rel_l2(out, ref) <= FP64_TOL
    out2, ref2 = _both(js, lc, shape, mask=mask, formula="")
    assert rel_l2(out2, ref2) <= FP64_TOL


def test_fp64_parity_beam_none(gpu):
    dims = (12, 10, 6)
    js, lc, shape = case(dims, beam="None", q=((0.0, 0.0), (0.1, 0.0)))
    rng = np.random.default_rng(2)
    E0 = (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(np.complex128)
    out, ref = _both(js, lc, shape, E0=E0)
    assert rel_l2(out, ref) <= FP64_TOL


def test_twisted_nematic_fp64_parity(gpu):
    c = workloads.twisted_nematic_cell()
    out, ref = _both(c["json"], c["lc"], c["shape"])
    assert rel_l2(out, ref) <= FP64_TOL


def test_uniform_director_closed_form_gpu(gpu):
    dims = (8, 6, 7)
    n = np.array([np.sin(0.7) * np.cos(0.3), np.sin(0.7) * np.sin(0.3), np.cos(0.7)])
    lc = np.broadcast_to(n, (dims[2], dims[1], dims[0], 3)).copy()
    js, _, shape = case(dims, lc=lc, no="1.5", ne="1.7", nin="1.2", nout="1.1", NA=0.5)
    E = np.zeros(shape, np.complex128)
    api.run(js, lc, E)
    J = uniform_jones(n, 1.5, 1.7, 1.2, 1.1, 0.6, 0.25, dims[2])
    for pol in range(2):
        for comp in range(2):
            assert np.allclose(E[0, 0, 2 * pol + comp], J[comp, pol], rtol=0, atol=1e-12)


@pytest.mark.parametrize("name", ["random_tilted_q", "two_wavelengths_dispersion", "iso_layers_focus", "long_x_lines",
                                  "tall_mesh", "many_slots", "many_slots_256", "many_slots_ny3"])
def test_fp32_error_budget(gpu, name):
    kw = dict(CASES[name])
    dims = kw.pop("dims")
    js, lc, shape = case(dims, seed=7, smooth=True, **kw)
    e64 = np.zeros(shape, np.complex128)
    e32 = np.zeros(shape, np.complex128)
    api.run(js, lc, e64, precision="fp64")
    api.run(js, lc, e32, precision="fp32")
    assert rel_l2(e32, e64) <= FP32_TOL


def test_twisted_nematic_fp32_error_budget(gpu):
    c = workloads.twisted_nematic_cell()
    e64 = np.zeros(c["shape"], np.complex128)
    e32 = np.zeros(c["shape"], np.complex128)
    api.run(c["json"], c["lc"], e64, precision="fp64")
    api.run(c["json"], c["lc"], e32, precision="fp32")
    assert rel_l2(e32, e64) <= FP32_TOL


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_plain_equals_batched(gpu, precision):
    """One wavelength per pass (plain) and all wavelengths per launch give identical bits."""
    js, lc, shape = case((12, 10, 6), wavelengths=(0.45, 0.55, 0.7), q=((0.0, 0.0), (0.1, -0.05)))
    a = np.zeros(shape, np.complex128)
    b = np.zeros(shape, np.complex128)
    # the same line-solve configuration in both (the tuner may pick per pass width)
    cfg = _lib.solve_candidates(js, _lib.FP32 if precision == "fp32" else _lib.FP64)["default"]
    api.run(js, lc, a, precision=precision, groups_per_pass=0, solve_config=cfg)
    api.run(js, lc, b, precision=precision, groups_per_pass=1, solve_config=cfg)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_of_uneven_samples_equals_alone(gpu, precision):
    s1 = case((16, 12, 8), q=((0.0, 0.0), (0.1, 0.0)), seed=1)
    s2 = case((10, 14, 5), wavelengths=(0.5, 0.7), seed=2)
    alone = []
    for js, lc, shape in (s1, s2):
        E = np.zeros(shape, np.complex128)
        api.run(js, lc, E, precision=precision)
        alone.append(E)
    batch = [np.zeros(s[2], np.complex128) for s in (s1, s2)]
    api.run_batch([{"json": s[0], "lc": s[1], "E": E} for s, E in zip((s1, s2), batch)], precision=precision)
    for a, b in zip(alone, batch):
        assert np.array_equal(a, b)


def test_graph_and_eager_identical(gpu):
    js, lc, shape = case((12, 12, 6), q=((0.05, 0.0),))
    a = np.zeros(shape, np.complex128)
    b = np.zeros(shape, np.complex128)
    api.run(js, lc, a, use_graph=True)
    api.run(js, lc, b, use_graph=False)
    assert np.array_equal(a, b)


def test_drop_in_module(gpu):
    js, lc, shape = case((12, 10, 5), q=((0.0, 0.0), (0.1, 0.0)))
    E = np.zeros(shape, np.complex128)
    assert bpm_backend.run_backend_without_mask(js, lc.ravel(), E) is None
    ref = np.zeros(shape, np.complex128)
    oracle.run_backend_without_mask(js, lc, ref)
    assert rel_l2(E, ref) <= FP64_TOL
