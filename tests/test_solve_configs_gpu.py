"""Every line-solve configuration the tuner can pick, forced one at a time, against the oracle.

The plan times the candidate configurations of a mesh (nbpm_solve_candidates) once per shape
and keeps the fastest, so each candidate is a product path: FP64 with each forced candidate must
match the CPU oracle to 1e-10 relative L2, and FP32 with each forced candidate must stay within
1e-4 of the FP64 result. The meshes cover every kernel family: warp-per-line x solves (chunk
lengths 2-32, 1-4 slots per thread), x chunks in shared memory, several warps per x-line,
sequential x-lines, chunked y solves (16- and 32-warp Woodbury blocks), sequential-per-column y
solves, y chunks in a scratch field and sequential y-lines."""
import numpy as np
import pytest

import oracle
from nemaktis_gb300 import _lib, api
from tests.helpers import case, rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
FP32_TOL = 1e-4

Q4 = ((0.0, 0.0), (0.1, -0.05))
Q5 = ((0.0, 0.0), (0.1, 0.0), (0.0, 0.1), (-0.07, 0.05), (0.05, -0.12))
MESHES = {
    "slots10": dict(dims=(40, 24, 5), q=Q5),
    "x300": dict(dims=(300, 12, 4), q=Q4),
    "x600": dict(dims=(600, 6, 3), q=((0.03, 0.01),)),
    "x2100": dict(dims=(2100, 5, 3), q=((0.03, 0.0),)),
    "y200": dict(dims=(12, 200, 5), q=Q4),
    "y530": dict(dims=(10, 530, 4), q=Q4),
}


def configs(js, precision):
    c = _lib.solve_candidates(js, precision)
    # every x candidate with the default y, every y candidate with the default x (the transposed-
    # frame y solves "yx" need an x solve that hands the fields over, "xc" or "xw")
    dx, dy = c["default"].split(";")
    hand = [x for x in c["x"] if x.startswith(("xc:", "xw:"))]
    out = {x + ";" + dy for x in c["x"]}
    for y in c["y"]:
        if not y.startswith("yx:"):
            out.add(dx + ";" + y)
        elif hand:
            out.add((dx if dx.startswith(("xc:", "xw:")) else hand[0]) + ";" + y)
    return sorted(out)


@pytest.mark.parametrize("name", sorted(MESHES))
def test_every_candidate_fp64_matches_oracle(gpu, name):
    kw = dict(MESHES[name])
    dims = kw.pop("dims")
    js, lc, shape = case(dims, seed=11, **kw)
    ref = np.zeros(shape, np.complex128)
    oracle.run_backend_without_mask(js, lc, ref)
    for cfg in configs(js, _lib.FP64):
        out = np.zeros(shape, np.complex128)
        api.run(js, lc, out, precision="fp64", solve_config=cfg)
        assert rel_l2(out, ref) <= FP64_TOL, cfg


@pytest.mark.parametrize("name", ["slots10", "x600", "y200", "y530"])
def test_every_candidate_fp32_within_budget(gpu, name):
    kw = dict(MESHES[name])
    dims = kw.pop("dims")
    js, lc, shape = case(dims, seed=12, smooth=True, **kw)
    e64 = np.zeros(shape, np.complex128)
    api.run(js, lc, e64, precision="fp64")
    for cfg in configs(js, _lib.FP32):
        e32 = np.zeros(shape, np.complex128)
        api.run(js, lc, e32, precision="fp32", solve_config=cfg)
        assert rel_l2(e32, e64) <= FP32_TOL, cfg


def test_koehler_shape_fp32_candidates(gpu):
    """The 256x256, 13-q, 2-pol production shape (two wavelengths, four planes): each FP32
    candidate within 1e-4 of FP64, and the FP64 run of the configuration FP32 production uses
    matches the oracle."""
    from nemaktis_gb300 import workloads
    c = workloads.koehler_micrograph(dims=(256, 256, 4), n_wavelengths=2)
    js, lc, shape = c["json"], c["lc"], c["shape"]
    e64 = np.zeros(shape, np.complex128)
    api.run(js, lc, e64, precision="fp64")
    for cfg in configs(js, _lib.FP32):
        e32 = np.zeros(shape, np.complex128)
        api.run(js, lc, e32, precision="fp32", solve_config=cfg)
        assert rel_l2(e32, e64) <= FP32_TOL, cfg
    bufs = [{"json": js, "lc": lc, "E": np.zeros(shape, np.complex128)}]
    with api.Plan(bufs, precision="fp32") as p:
        prod, _ = p.solve_config(0)
    ref = np.zeros(shape, np.complex128)
    oracle.run_backend_without_mask(js, lc, ref)
    out = np.zeros(shape, np.complex128)
    api.run(js, lc, out, precision="fp64", solve_config=prod)
    assert rel_l2(out, ref) <= FP64_TOL


def test_tuner_picks_a_candidate_and_is_reproducible(gpu):
    """A tuned plan reports its timings, picks one of the candidates, and a run forced to the
    picked configuration gives the same bits."""
    js, lc, shape = case((40, 24, 5), q=Q5, seed=3)
    _lib.load().nbpm_tune_cache_clear()
    bufs = [{"json": js, "lc": lc, "E": np.zeros(shape, np.complex128)}]
    with api.Plan(bufs, precision="fp32", tune=True) as p:
        cfg, report = p.solve_config(0)
        p.upload()
        p.execute()
        p.download()
    cands = _lib.solve_candidates(js, _lib.FP32)
    x, y = cfg.split(";")
    assert x in cands["x"] and y in cands["y"]
    assert "tuned" in report and "ms" in report
    forced = np.zeros(shape, np.complex128)
    api.run(js, lc, forced, precision="fp32", solve_config=cfg)
    assert np.array_equal(forced, bufs[0]["E"])
    with api.Plan([{"json": js, "lc": lc, "E": np.zeros(shape, np.complex128)}], precision="fp32", tune=True) as p2:
        cfg2, report2 = p2.solve_config(0)
    assert cfg2 == cfg and "cached" in report2


def test_tune_cache_file_is_reused_by_a_new_process(gpu, tmp_path):
    """With NBPM_TUNE_CACHE set, the tuned configuration of a shape is written to the file, and a
    later process reads it from there instead of timing the candidates again."""
    import json
    import os
    import subprocess
    import sys
    cache = tmp_path / "tune.tsv"
    script = (
        "import json, numpy as np\n"
        "from tests.helpers import case\n"
        "from nemaktis_gb300 import api\n"
        "js, lc, shape = case((40, 24, 5), q=((0.0, 0.0), (0.1, 0.0), (0.0, 0.1)), seed=4)\n"
        "with api.Plan([{'json': js, 'lc': lc, 'E': np.zeros(shape, np.complex128)}], precision='fp32') as p:\n"
        "    print(json.dumps(p.solve_config(0)))\n")
    env = dict(os.environ, NBPM_TUNE_CACHE=str(cache))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    runs = []
    for _ in range(2):
        out = subprocess.run([sys.executable, "-c", script], env=env, cwd=root, capture_output=True, text=True,
                             timeout=600)
        assert out.returncode == 0, out.stderr
        runs.append(json.loads(out.stdout.strip().splitlines()[-1]))
    assert cache.exists() and cache.read_text().count("\t") >= 2
    (cfg1, rep1), (cfg2, rep2) = runs
    assert "tuned" in rep1 and cfg1 == cfg2
    assert "cached" in rep2 and "tuned" not in rep2
