"""JSON settings of the bpm backend, restated for the oracle.

TEST INFRASTRUCTURE ONLY: part of the CPU oracle, never imported by the product.

Restates the keys the reference backend reads (BeamPropagationSolver/src/SettingsLib/
PhysicsSettings.cpp:26-83, AlgorithmSettings.cpp:13-16, PostprocessorSettings.cpp:9-14,
BaseSettings.cpp:8-22), the wavelength list (PhysicsSettings.cpp:43-58), the q-list
including the C++ default hexagonal ring ``iphi*pi/3`` (PhysicsSettings.cpp:60-82) and
the beam-profile regex (BeamPropagationLib/BPMIteration.cpp:21-50).
"""
import json
import math
import re

from .expr import evaluate

PI_REF = 3.1415926535897932


class SettingsError(ValueError):
    pass


def _sec(node, name):
    if name not in node:
        raise SettingsError('The section "%s" is missing from the setting file' % name)
    return node[name]


def parse(json_str):
    j = json.loads(json_str)
    alg = _sec(j, "Algorithm settings")
    gen = _sec(alg, "General")
    bpm = _sec(alg, "Beam propagation")
    phys = _sec(j, "Physics settings")
    ic = _sec(phys, "Initial conditions")
    co = _sec(phys, "Coefficients")
    post = _sec(j, "Postprocessor settings")
    bulk = _sec(post, "Bulk output")
    scr = _sec(post, "Screen output")

    s = {}
    s["lc_field_type"] = gen["LC field type"]
    s["n_woodbury"] = int(bpm["N Woodbury steps"])
    s["beam_profile"] = ic["Beam profile"]
    s["dims"] = [int(v) for v in ic["Mesh dimensions"]]
    s["spacings"] = [float(v) for v in ic["Mesh spacings"]]
    s["no"] = co["no"]
    s["ne"] = co["ne"]
    s["ne_imag"] = co.get("ne_imag", "0")
    s["nhost"] = co.get("nhost", "1")
    s["nin"] = co.get("nin", "1")
    s["nout"] = co.get("nout", "1")
    if "Wavelengths" in co:
        s["wavelengths"] = [float(v) for v in co["Wavelengths"]]
    else:
        mean, fwhm, n = float(co["Mean wavelength"]), float(co["Spectral FWHM"]), int(co["N wavelengths"])
        if n == 1:
            s["wavelengths"] = [mean]
        else:
            s["wavelengths"] = [mean + fwhm * (i / (n - 1.) - 0.5) for i in range(n)]
    if "Wavevectors" in co:
        raw = [float(v) for v in co["Wavevectors"]]
        if len(raw) % 2:
            raise SettingsError('Wrong number of values for the "Wavevectors" entry,\nshould be a multiple of 2')
        s["q"] = [(raw[2 * i], raw[2 * i + 1]) for i in range(len(raw) // 2)]
    else:
        NA = float(co["Condenser numerical aperture"])
        Nc = int(co["N radial illumination directions"])
        q = [(0.0, 0.0)]
        for ir in range(1, Nc):
            for iphi in range(6 * ir):
                phi = iphi * PI_REF / 3
                q.append((ir * NA / (Nc - 1) * math.cos(phi), ir * NA / (Nc - 1) * math.sin(phi)))
        s["q"] = q
    s["bulk_activate"] = bool(bulk["Activate"])
    s["iso_thick"] = [float(v) for v in scr["Isotropic layer thicknesses"]]
    s["iso_index"] = [float(v) for v in scr["Isotropic layer refractive indices"]]
    s["z_foc"] = float(scr["Focalisation z-shift"])
    s["NA"] = float(scr["Numerical aperture"])
    if len(s["iso_thick"]) != len(s["iso_index"]):
        raise SettingsError("Inconsistent number of isotropic layers")

    bp = s["beam_profile"]
    if bp == "UniformBeam":
        s["beam_type"], s["waist"] = 0, 0.0
    elif bp == "None":
        s["beam_type"], s["waist"] = 2, 0.0
    else:
        m = re.fullmatch(r"GaussianBeam\(([0-9]+\.?[0-9]*)\)", bp)
        if not m:
            raise SettingsError("Unrecognised beam profile")
        s["beam_type"], s["waist"] = 1, float(m.group(1))

    lam = s["wavelengths"]
    for key in ("no", "ne", "ne_imag", "nhost", "nin", "nout"):
        s[key + "_vals"] = [float(evaluate(s[key], **{"lambda": l})) for l in lam]
    s["nout_06"] = float(evaluate(s["nout"], **{"lambda": 0.6}))
    return s
