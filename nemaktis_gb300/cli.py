"""File-based run of the GPU backend, the counterpart of the reference's `bpm-solver -x
settings.json` (BeamPropagationSolver/src/main.cpp:169-257, RootSettings.cpp:14-58):

    python -m nemaktis_gb300.cli -x settings.json [--precision fp64|fp32]

* the settings file may hold comment lines (starting with '#') and empty lines, which are
  dropped before parsing (main.cpp:149-166);
* the LC field comes from the .vti file named by "LC field file", read with the basis
  convention of the settings (vti_io.lc_field_from_vti); voxels whose field is zero
  (norm <= 1e-8) are outside the LC domain (VectorField::set_mask_from_nonzeros,
  VectorField.cpp:183-195);
* the results folder is created; bulk output, when activated, is written by the backend;
  the screen fields, when "Screen output" is activated, go to <folder>/<base name>.vti with
  the arrays of ScreenOutput::apply (ScreenOutput.cpp:90-181): E_real/E_imag_inputX|Y_<wave>_<q>,
  three components (Ex, Ey, 0), field data lambda/qx/qy, spacing (dx, dy, 0).

On failure the reference's framed message goes to stderr and the exit status is 1.
"""
import argparse
import json
import os
import re
import sys

import numpy as np

from . import api, vti_io
from ._lib import NbpmError


def minify_json(path):
    """Settings text without empty and comment lines (main.cpp:149-166)."""
    if not os.path.exists(path):
        raise NbpmError(1, "Could not open the specified setting file")
    keep = []
    with open(path) as f:
        for line in f:
            s = line.rstrip("\n")
            if re.fullmatch(r"\s*", s) or re.fullmatch(r"\s*#.*", s):
                continue
            keep.append(s)
    return "\n".join(keep) + "\n"


def run_from_settings(settings_text, precision="fp64"):
    """Runs one settings file's worth of propagation; returns the screen fields
    (Nl, Nq, 4, Ny, Nx) and the parsed settings."""
    st = json.loads(settings_text)
    gen = st["Algorithm settings"]["General"]
    ic = st["Physics settings"]["Initial conditions"]
    lc_type = gen["LC field type"]
    path = ic["LC field file"]
    if not path.endswith(".vti"):
        raise NbpmError(1, "Unrecognised initial solution filetype: must be a path to a vti file.")
    basis = ic.get("Basis convention", "XYZ")
    if basis not in ("XYZ", "YZX", "ZXY"):
        raise NbpmError(1, 'Parsing error: "Basis convention" must be "XYZ", "YZX" or "ZXY"')
    lc_dim = 3 if lc_type == "Director" else 6
    try:
        vals, dims, spac = vti_io.lc_field_from_vti(path, lc_dim, basis)
    except vti_io.VtiError as e:
        raise NbpmError(1, str(e))
    folder = gen.get("Results folder name", "")
    if folder:
        os.makedirs(folder, exist_ok=True)
    # the mesh is the file's; the settings' mesh keys are replaced by it
    ic["Mesh dimensions"] = [int(v) for v in dims]
    ic["Mesh spacings"] = [float(v) for v in spac]
    js = json.dumps(st)
    norm = np.sqrt((vals ** 2).sum(axis=-1))
    mask = np.where(norm > 1e-8, 1.0, -1.0)
    wl = _wavelengths(st)
    q = _wavevectors(st)
    E = np.zeros((len(wl), len(q), 4, dims[1], dims[0]), np.complex128)
    api.run(js, vals, E, mask=mask, formula=None, precision=precision)
    scr = st["Postprocessor settings"]["Screen output"]
    if scr.get("Activate", False):
        base = scr.get("Base name", "")
        out = os.path.join(folder, base + ".vti") if folder and folder != "." else base + ".vti"
        _write_screen(out, E, wl, q, dims, spac)
    return E, st


def _wavelengths(st):
    c = st["Physics settings"]["Coefficients"]
    if "Wavelengths" in c:
        return [float(v) for v in c["Wavelengths"]]
    m, w, n = float(c["Mean wavelength"]), float(c["Spectral FWHM"]), int(c["N wavelengths"])
    if n == 1:
        return [m]
    return [m + w * (float(i) / (n - 1.0) - 0.5) for i in range(n)]  # PhysicsSettings.cpp:46-57


def _wavevectors(st):
    c = st["Physics settings"]["Coefficients"]
    if "Wavevectors" in c:
        v = [float(x) for x in c["Wavevectors"]]
        if len(v) % 2 != 0:
            raise NbpmError(1, 'Wrong number of values for the "Wavevectors" entry,\nshould be a multiple of 2')
        return [(v[2 * i], v[2 * i + 1]) for i in range(len(v) // 2)]
    na, nr = float(c["Condenser numerical aperture"]), int(c["N radial illumination directions"])
    q = [(0.0, 0.0)]
    for ir in range(1, nr):
        for k in range(6 * ir):
            phi = k * 3.1415926535897932 / 3  # the backend's ring angle (PhysicsSettings.cpp:70-80)
            q.append((ir * na / (nr - 1) * np.cos(phi), ir * na / (nr - 1) * np.sin(phi)))
    return q


def _write_screen(path, E, wl, q, dims, spac):
    Nx, Ny = dims[0], dims[1]
    pts = []
    pols = ("inputX_", "inputY_")
    for w in range(len(wl)):
        for iq in range(len(q)):
            for pol in range(2):
                f = E[w, iq, 2 * pol: 2 * pol + 2].reshape(2, Nx * Ny)
                re_ = np.zeros((Nx * Ny, 3))
                im_ = np.zeros((Nx * Ny, 3))
                re_[:, :2] = f.real.T
                im_[:, :2] = f.imag.T
                tag = "%s%d_%d" % (pols[pol], w, iq)
                pts.append(("E_real_" + tag, re_))
                pts.append(("E_imag_" + tag, im_))
    fld = [("lambda", np.asarray(wl, float)), ("qx", np.asarray([v[0] for v in q], float)),
           ("qy", np.asarray([v[1] for v in q], float))]
    vti_io.write_vti(path, (Nx, Ny, 1), (spac[0], spac[1], 0.0),
                     (-spac[0] * (Nx - 1) / 2.0, -spac[1] * (Ny - 1) / 2.0, 0.0), pts, fld)


def _fail(msg):
    sys.stderr.write("\n\n-------------------------------------------------\nException on processing: \n"
                     "%s\nAborting!\n-------------------------------------------------\n" % msg)
    return 1


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m nemaktis_gb300.cli",
                                 description="Beam propagation of an LC field file on the GPU (bpm-solver -x).")
    ap.add_argument("-x", dest="settings", required=True, help="JSON settings file")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    a = ap.parse_args(argv)
    try:
        run_from_settings(minify_json(a.settings), a.precision)
    except NbpmError as e:
        return _fail(e.msg)
    except (ValueError, KeyError) as e:
        return _fail(str(e))
    return 0


if __name__ == "__main__":
    sys.exit(main())
