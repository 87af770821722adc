"""The plan kept between blocking calls (nbpm_run_batch and the reference-shaped entries): a
call that reuses it gives the bits of a call that builds its plan afresh."""
import numpy as np
import pytest

from nemaktis_gb300 import _lib, api, workloads

pytestmark = pytest.mark.gpu


def _case(seed, wl=(0.5, 0.6)):
    dims = (24, 20, 7)
    js = workloads.settings_json(dims, (0.25, 0.25, 0.25), list(wl), [(0.0, 0.0), (0.06, -0.03)], no="1.5", ne="1.7")
    lc = workloads.random_smooth(dims, seed=seed)
    return js, lc, (len(wl), 2, 4, dims[1], dims[0])


def _fresh(js, lc, shape, precision, monkeypatch, mask=None):
    monkeypatch.setenv("NBPM_PLAN_CACHE", "0")
    E = np.zeros(shape, np.complex128)
    api.run(js, lc, E, mask=mask, precision=precision)
    monkeypatch.delenv("NBPM_PLAN_CACHE")
    return E


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_reused_plan_gives_fresh_results(gpu, monkeypatch, precision):
    lib = _lib.load()
    monkeypatch.delenv("NBPM_PLAN_CACHE", raising=False)
    assert lib.nbpm_release_plan_cache() == 0
    runs = [_case(1), _case(2), _case(2, wl=(0.55, 0.6)), _case(3)]
    for js, lc, shape in runs:  # second call reuses the first's plan; the third has other settings
        E = np.zeros(shape, np.complex128)
        api.run(js, lc, E, precision=precision)
        np.testing.assert_array_equal(E, _fresh(js, lc, shape, precision, monkeypatch))
    # masked calls: the same formula-free mask twice with other values, then a mask formula
    js, lc, shape = runs[-1]
    for cut in (5, 9):
        mask = np.ones(lc.shape[:3])
        mask[:, :cut, :] = -1.0
        E = np.zeros(shape, np.complex128)
        api.run(js, lc, E, mask=mask, precision=precision)
        np.testing.assert_array_equal(E, _fresh(js, lc, shape, precision, monkeypatch, mask=mask))
    Nz, Ny, Nx = lc.shape[:3]
    z, y, x = np.meshgrid((np.arange(Nz) - (Nz - 1) / 2) * 0.25, (np.arange(Ny) - (Ny - 1) / 2) * 0.25,
                          (np.arange(Nx) - (Nx - 1) / 2) * 0.25, indexing="ij")
    formula = "4-x^2-y^2-z^2"
    for r2 in (4.0, 3.0):  # the second mask disagrees with the formula: uniform weights
        mask = r2 - x ** 2 - y ** 2 - z ** 2
        E = np.zeros(shape, np.complex128)
        api.run(js, lc, E, mask=mask, formula=formula, precision=precision)
        monkeypatch.setenv("NBPM_PLAN_CACHE", "0")
        ref = np.zeros(shape, np.complex128)
        api.run(js, lc, ref, mask=mask, formula=formula, precision=precision)
        monkeypatch.delenv("NBPM_PLAN_CACHE")
        np.testing.assert_array_equal(E, ref)
    E = np.zeros(shape, np.complex128)
    api.run(js, lc[::-1].copy(), E, precision=precision)
    np.testing.assert_array_equal(E, _fresh(js, lc[::-1].copy(), shape, precision, monkeypatch))
    assert lib.nbpm_release_plan_cache() == 0


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_page_locked_result_array(gpu, precision):
    """A page-locked result array (written by the widening kernel directly in FP32 mode) holds
    the same bits as an ordinary one."""
    torch = pytest.importorskip("torch")
    js, lc, shape = _case(5)
    n = int(np.prod(shape)) * 16
    t = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    E_pinned = t.numpy().view(np.complex128).reshape(shape)
    E_pinned[...] = 0
    E = np.zeros(shape, np.complex128)
    api.run(js, lc, E_pinned, precision=precision)
    api.run(js, lc, E, precision=precision)
    np.testing.assert_array_equal(E_pinned, E)
