"""CPU tests of libnbpm's host side: exports, settings validation with the reference's
messages, expression and mask-weight evaluation against the oracle, and the bpm_backend
drop-in's argument handling. No kernel runs here."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

import oracle
from oracle import expr as oexpr
from nemaktis_gb300 import _lib, api, bpm_backend, workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "nbpm.h")).read()
    return sorted(set(re.findall(r"\b(nbpm_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(lib):
    syms = header_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(_lib.EXPORTS)


def _run(js, lc, E, mask=None, formula=None):
    with pytest.raises(_lib.NbpmError) as ei:
        api.run(js, lc, E, mask=mask, formula=formula)
    return ei.value


def _base():
    return workloads.settings_json((8, 6, 4), (0.25, 0.25, 0.25), [0.6], [0.0, 0.0])


@pytest.mark.parametrize("mut,code,msg", [
    (lambda j: j.pop("Physics settings"), 1, 'The section "Physics settings" is missing from the setting file'),
    (lambda j: j["Algorithm settings"]["General"].update({"LC field type": "Foo"}), 1,
     'Parsing error: "LC field type" must be "Director" or "Q-tensor"'),
    (lambda j: j["Physics settings"]["Initial conditions"].update({"Beam profile": "Gauss(1)"}), 1,
     "Unrecognised beam profile"),
    (lambda j: j["Physics settings"]["Coefficients"].update({"ne": "1.7+"}), 3, "Wrong expression for ne"),
    (lambda j: j["Physics settings"]["Coefficients"].update({"nout": "lamda"}), 3, "Wrong expression for nin"),
    (lambda j: j["Physics settings"]["Coefficients"].update({"Wavevectors": [0.1]}), 1,
     'Wrong number of values for the "Wavevectors" entry,\nshould be a multiple of 2'),
    (lambda j: j["Postprocessor settings"]["Screen output"].update({"Isotropic layer thicknesses": [1.0]}), 1,
     "Inconsistent number of isotropic layers"),
    (lambda j: j["Algorithm settings"]["Beam propagation"].pop("N Woodbury steps"), 1,
     'Error when parsing variable "N Woodbury steps" in section "Beam propagation"'),
])
def test_settings_errors(lib, mut, code, msg):
    j = json.loads(_base())
    mut(j)
    lc = np.zeros((4, 6, 8, 3))
    E = np.zeros((1, 1, 4, 6, 8), np.complex128)
    err = _run(json.dumps(j), lc, E)
    assert err.code == code
    assert err.msg.startswith(msg)


def test_size_errors(lib):
    js = _base()
    E = np.zeros((1, 1, 4, 6, 8), np.complex128)
    assert _run(js, np.zeros(8 * 6 * 4 * 3 + 1), E).msg == "Wrong dimension for the user pointer array (VectorField)"
    assert _run(js, np.zeros(8 * 6 * 4 * 4), E).msg == \
        "Unexpected dimension for the LC orientational field, should be 3 or 6."
    assert _run(js, np.zeros((4, 6, 8, 3)), np.zeros((1, 1, 4, 6, 7), np.complex128)).msg == \
        "Wrong dimension for the user pointer array (OpticalFieldCollection)"
    assert _run(js, np.zeros((4, 6, 8, 3)), E, mask=np.zeros(5)).msg == "Wrong dimension for the mask pointer array"
    err = _run("{not json", np.zeros((4, 6, 8, 3)), E)
    assert err.code == 1 and "parse_error" in err.msg


@pytest.mark.parametrize("e", ["1.5", "1.52+0.008/lambda^2", "-lambda^2+3", "sqrt(lambda)*2^-1",
                               "lambda>=0.6 ? 1.7 : 1.5*exp(-lambda)", "avg(1,lambda,3)", "ln(lambda)+log10(100)"])
def test_expression_evaluator_matches_oracle(lib, e):
    for lam in (0.4, 0.6, 0.8):
        out = ctypes.c_double()
        assert lib.nbpm_eval_index(e.encode(), lam, ctypes.byref(out)) == 0
        assert out.value == pytest.approx(oexpr.evaluate(e, **{"lambda": lam}), rel=1e-14, abs=1e-15)


def test_mask_weights_match_oracle(lib):
    dims = (10, 9, 12)
    d = 0.3
    js = workloads.settings_json(dims, (d, d, d), [0.6], [0.0, 0.0])
    Nx, Ny, Nz = dims
    x = (np.arange(Nx) - 0.5 * (Nx - 1)) * d
    y = (np.arange(Ny) - 0.5 * (Ny - 1)) * d
    z = (np.arange(Nz) - 0.5 * (Nz - 1)) * d
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    formula = "2.2^2-x^2-y^2-(z-0.1)^2"
    mask_vals = 2.2 ** 2 - X ** 2 - Y ** 2 - (Z - 0.1) ** 2
    m = np.zeros(Nx * Ny * Nz, np.uint8)
    w = np.zeros(2 * Nx * Ny * (Nz - 1))
    mv = np.ascontiguousarray(mask_vals.ravel())
    assert lib.nbpm_mask_weights(js.encode(), formula.encode(), mv.ctypes.data, mv.size, m.ctypes.data,
                                 w.ctypes.data) == 0
    m_ref, w_ref = oracle.mask_interp_weights(mask_vals, formula, dims, (d, d, d))
    assert np.array_equal(m, m_ref.ravel())
    assert np.allclose(w, w_ref.ravel(), rtol=0, atol=1e-12)
    assert (w != 0.5).sum() > 20  # the sphere crosses cells


def test_bpm_backend_argument_checks(lib):
    js = _base()
    lc = np.zeros((4, 6, 8, 3))
    with pytest.raises(TypeError):
        bpm_backend.run_backend_without_mask(js, lc, np.zeros((1, 1, 4, 6, 8), np.complex64))
    with pytest.raises(TypeError):
        bpm_backend.run_backend_without_mask(js, lc.reshape(4, 6, 8, 3), np.zeros((1, 1, 4, 6, 8), np.complex128))
    with pytest.raises(TypeError):
        bpm_backend.run_backend_without_mask(js, lc.ravel(), np.zeros((1, 1, 4, 6, 16), np.complex128)[..., ::2])


def test_bpm_backend_reports_like_reference(lib, capsys):
    """Errors are printed in the reference's format and the call returns None
    (bpm_backend.cpp:48-82); strict mode raises instead."""
    js = _base()
    E = np.zeros((1, 1, 4, 6, 8), np.complex128)
    r = bpm_backend.run_backend_without_mask(js, np.zeros(10), E)
    assert r is None
    err = capsys.readouterr().err
    assert "Exception on processing: \nWrong dimension for the user pointer array (VectorField)\nAborting!" in err
    bpm_backend.set_strict(True)
    try:
        with pytest.raises(_lib.NbpmError):
            bpm_backend.run_backend_without_mask(js, np.zeros(10), E)
    finally:
        bpm_backend.set_strict(False)


def test_install_as_module():
    import sys
    m = bpm_backend.install()
    import bpm_backend as bb
    assert bb is m and hasattr(bb, "run_backend_with_mask")
    del sys.modules["bpm_backend"]


def test_solve_candidates_cover_the_kernel_families(lib):
    """Host-side candidate lists (no device needed): the rule-based default is a candidate, and
    each mesh offers the kernel families its line lengths allow."""
    from nemaktis_gb300 import _lib, workloads

    def cands(dims, q=((0.0, 0.0),), prec=_lib.FP64):
        js = workloads.settings_json(dims, (0.25, 0.25, 0.25), [0.6], np.asarray(q, float))
        return _lib.solve_candidates(js, prec)

    for dims in [(40, 24, 4), (300, 12, 4), (600, 6, 3), (2100, 5, 3), (12, 200, 5), (10, 530, 4), (3, 16, 4), (16, 2, 4)]:
        c = cands(dims)
        dx, dy = c["default"].split(";")
        assert dx in c["x"] and dy in c["y"], (dims, c)
    assert cands((3, 16, 4))["x"] == ["xseq"]
    assert cands((16, 2, 4))["y"] == ["yseq"]
    assert any(x.startswith("xw:") for x in cands((300, 12, 4))["x"])
    assert any(x.startswith("xs:") for x in cands((600, 6, 3))["x"])
    assert cands((2100, 5, 3))["x"] == ["xseq"]
    y200 = cands((12, 200, 5), q=((0.0, 0.0), (0.1, 0.0)), prec=_lib.FP32)["y"]
    assert any(y.endswith(":W1024") for y in y200) and any(y.startswith("yq:") for y in y200)
    y530 = cands((10, 530, 4))["y"]
    assert "yseq" in y530 and not any(y.startswith("yc:") for y in y530)
    with pytest.raises(_lib.NbpmError):
        _lib.solve_candidates("{}", _lib.FP64)
