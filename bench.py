"""Benchmark of the GB300 bpm backend (one JSON line on stdout).

Metric: voxel-steps/s (one transverse point advanced one z-slab for one (wavelength,
wave vector, polarisation) propagation). A "step" is one full run of the workload: every
slab of every propagation plus the screen filter, with inputs resident in HBM (``value``).
``e2e`` is the same metric through the reference-facing C ABI call (nbpm_run_batch, the
entry behind nbpm_run_backend_ex) with pinned host buffers: director upload, the run and the
complex128 field download inside the timed region of every step; the device plan of the
untimed first call is kept and reused by the timed calls, as for any repeated call with the
same settings.

Default workload: batched Koehler micrograph, 256x256x64 mesh, 16 wavelengths x 13 wave
vectors x 2 polarisations = 416 propagations, FP32 batched mode. The FP64 plain mode (one
wavelength per launch) is measured on the same workload beside it, and the FP32 result's
relative L2 error against the FP64 result is reported.

--impl reference times the CPU oracle (FP64 C++/OpenMP restatement of the reference; the
reference itself cannot be built here) on a bounded sample of the same workload.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

MEASURED = os.path.join(HERE, "MEASURED_PEAKS.json")
L2_BYTES = 126e6
NO_FLUSH_BYTES = 4 * L2_BYTES  # working sets at least this large are not flushed between steps


def peaks():
    try:
        with open(MEASURED) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_aggregate(vs, steps, dev_ms, world, device):
    """Replicas (one process per GPU, the same workload on each): the step time is the slowest
    rank's (max over ranks), and the value is the voxel-steps of all ranks over that time.
    Returns (max ms, voxel-steps/s). With world == 1 no collective is made."""
    if world > 1:
        import torch
        import torch.distributed as dist
        tt = torch.tensor([dev_ms], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        dev_ms = float(tt.item())
    return dev_ms, vs * steps * world / (dev_ms / 1e3)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) >= 9:
                for k, n in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def workload(name):
    from nemaktis_gb300 import workloads as W
    if name == "koehler":
        c = W.koehler_micrograph()
        c["desc"] = "batched Koehler micrograph 256x256x64 d=0.25um, 16 wavelengths x 13 q x 2 pol (416 propagations)"
        c["Nz"] = 64
        return [c]
    if name == "koehler_small":
        c = W.koehler_micrograph(dims=(256, 256, 8), n_wavelengths=8)
        c["desc"] = "reduced batched Koehler case for profiling: 256x256x8, 8 wavelengths x 13 q x 2 pol"
        c["Nz"] = 8
        return [c]
    if name == "tn":
        c = W.twisted_nematic_cell()
        c["desc"] = "twisted nematic 64x64x40 d=0.25um, 1 wavelength x 1 q x 2 pol"
        c["Nz"] = 40
        return [c]
    if name == "droplet":
        c = W.droplet_cell()
        c["desc"] = "cholesteric droplet 512x512x128 d=0.2um (mask + formula), 1 wavelength x 1 q x 2 pol"
        c["Nz"] = 128
        return [c]
    if name == "uneven":
        out = []
        for i in range(4):
            c = W.uneven_sample(i)
            c["Nz"] = W.UNEVEN_MESHES[i][2]
            out.append(c)
        out[0]["desc"] = "4 uneven samples 1024^2x200, 768^2x160, 512^2x96, 256^2x48 d=0.2um, 4 wl x 7 q x 2 pol"
        return out
    raise SystemExit("unknown workload " + name)


def voxel_steps(samples):
    from nemaktis_gb300 import workloads as W
    return sum(W.voxel_steps(c["shape"], c["Nz"]) for c in samples)


def pinned(shape, dtype):
    import torch
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    t = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    a = t.numpy().view(dtype).reshape(shape)
    return a, t


def run_ours(args):
    import torch
    from nemaktis_gb300 import _lib, api

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    lib = _lib.load()
    samples = workload(args.workload)
    vs = voxel_steps(samples)
    prec = "fp32" if args.precision == "fp32" else "fp64"

    # Device-resident plan for the timed value.
    bufs = []
    for c in samples:
        E = np.zeros(c["shape"], np.complex128)
        bufs.append({"json": c["json"], "lc": c["lc"], "E": E, "mask": c.get("mask"), "formula": c.get("formula")})
    plan = api.Plan(bufs, precision=prec, groups_per_pass=0, tune=not args.no_tune, solve_config=args.solve_config)
    solve_cfg = [plan.solve_config(i) for i in range(len(samples))]
    plan.upload()
    for _ in range(args.warmup):
        plan.execute()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clk = Clocks(local)
    # A step's working set (fields and director) of at least NO_FLUSH_BYTES (four times the 126 MB
    # L2) cannot be served from it; a smaller one is flushed by a 512 MB write before each timed
    # step (outside the step's CUDA-event window).
    ws = sum(np.prod(c["shape"]) * (8 if prec == "fp32" else 16) + c["lc"].size * 8 for c in samples)
    flush = None
    if ws < NO_FLUSH_BYTES:
        try:
            flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device="cuda")
        except Exception:
            flush = None
    l2_note = ("inputs larger than L2 (fields and director %.0f MB per step, >= 4x L2: not flushed)" % (ws / 1e6)
               if ws >= NO_FLUSH_BYTES
               else "L2 flushed before every timed step (512 MB write; working set %.0f MB < 4x L2)" % (ws / 1e6)
               if flush is not None else "working set %.0f MB < 4x L2, flush buffer unavailable" % (ws / 1e6))
    clk.start()
    t0 = time.perf_counter()
    ms = []
    launches = 0
    for _ in range(args.steps):
        if flush is not None:
            flush.fill_(1.0)
            torch.cuda.synchronize()
        t = plan.execute()
        ms.append(t["compute_ms"])
        launches += t["kernel_launches"]
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    dev_ms, value = replica_aggregate(vs, args.steps, float(np.sum(ms)), world, "cuda")
    plan.download()
    out32 = [b["E"].copy() for b in bufs]
    if args.only_value:
        plan.close()
        if rank == 0:
            print(json.dumps({"metric": "voxel-steps/s", "value": value, "unit": "voxel-steps/s", "steps": args.steps,
                              "warmup": args.warmup, "ms_per_step": dev_ms / args.steps,
                              "config": {"workload": samples[0]["desc"], "precision": prec,
                                         "line_solves": [c for c, _ in solve_cfg],
                                         "tuning": [r for _, r in solve_cfg]},
                              "gpu_launches": launches, "clocks": clocks}))
        return
    prof = profile_kernels(plan, lib)
    plan.close()

    # The rule-based line-solve configuration on the same workload, for the tuner's gain.
    tuning = {"configs": [c for c, _ in solve_cfg], "how": [r for _, r in solve_cfg]}
    if not args.no_tune and args.solve_config is None:
        hb = [{"json": c["json"], "lc": c["lc"], "E": np.zeros(c["shape"], np.complex128), "mask": c.get("mask"),
               "formula": c.get("formula")} for c in samples]
        with api.Plan(hb, precision=prec, groups_per_pass=0, tune=False) as hp:
            hp.upload()
            hp.execute()
            hms = [hp.execute()["compute_ms"] for _ in range(2)]
            tuning["rule_based_configs"] = [hp.solve_config(i)[0] for i in range(len(samples))]
        tuning["rule_based_ms_per_step"] = float(np.mean(hms))
        tuning["tuned_ms_per_step"] = dev_ms / args.steps

    # FP64 plain path on the same workload (one wavelength per launch), one step.
    fp64 = None
    if not args.skip_fp64:
        b64 = []
        for c in samples:
            b64.append({"json": c["json"], "lc": c["lc"], "E": np.zeros(c["shape"], np.complex128),
                        "mask": c.get("mask"), "formula": c.get("formula")})
        p64 = api.Plan(b64, precision="fp64", groups_per_pass=1)
        p64.upload()
        p64.execute()
        t64 = p64.execute()
        p64.download()
        p64.close()
        err = float(np.sqrt(sum(np.linalg.norm(a - b["E"]) ** 2 for a, b in zip(out32, b64)) /
                            sum(np.linalg.norm(b["E"]) ** 2 for b in b64)))
        fp64 = {"value": vs / (t64["compute_ms"] / 1e3), "unit": "voxel-steps/s", "ms_per_step": t64["compute_ms"],
                "mode": "FP64, one wavelength per launch", "fp32_rel_l2_vs_fp64": err,
                "speedup_fp32_batched": value / world / (vs / (t64["compute_ms"] / 1e3))}

    # End-to-end through the C ABI with pinned host buffers.
    e2e = e2e_measure(samples, prec, args.e2e_steps)

    hbm, src = peaks()
    # DRAM bytes per launch of the dominant kernel from one ncu capture (dram__bytes_read.sum +
    # dram__bytes_write.sum), scaled to this workload's launch by the slots it processes; the
    # capture and its command are summarised under profiles/.
    PROF = "profiles/solve_xc_koehler_256x256x8_fp32.md"
    PSF = "profiles/shift_fused_koehler_256x256x8_fp32.md"
    W = 2 * (319.7e6 + 190.0e6 + 560.9e6 + 196.6e6) / 2  # mean of the two Woodbury launches, x2 slots
    TRAFFIC = {("koehler", "fp32", "wood_solve_x"): (W, PROF),
               ("koehler", "fp32", "wood_solve_y"): (W, PROF + " (the same kernel in the transposed frame)"),
               ("koehler", "fp32", "expl_solve_x"): (2 * (345.0e6 + 188.0e6), PROF),
               ("koehler", "fp32", "expl_solve_y"): (2 * (345.0e6 + 188.0e6), PROF + " (the same kernel in the transposed frame)"),
               ("koehler", "fp32", "shift_fused"): (2 * (242.6e6 + 181.1e6), PSF)}
    roof = None
    if prof:
        top = max(prof, key=lambda k: prof[k]["ms"])
        r = prof[top]
        ach = r["bytes"] / (r["ms"] / r["launches"] / 1e3) / 1e9 / r["launches"] if r["launches"] else 0
        tr = TRAFFIC.get((args.workload, args.precision, top))
        roof = {"bound": "hbm", "kernel": top, "achieved": ach, "peak": hbm, "unit": "GB/s",
                "frac": ach / hbm, "peak_source": src, "traffic": tr[0] if tr else None,
                "traffic_source": tr[1] if tr else None,
                "share_of_step": r["ms"] / sum(v["ms"] for v in prof.values()),
                "algorithmic_bytes_per_launch": r["bytes"] / max(1, r["launches"])}
    peaks_meas = None
    if not args.only_value:
        peaks_meas = fma_peaks()
    unev = None
    if rank == 0 and args.workload == "koehler" and not args.skip_uneven:
        unev = uneven_batch_record()
    cpu = None
    if rank == 0 and not args.skip_cpu:
        cpu = cpu_baseline(samples, args.cpu_seconds)
    line = {
        "metric": "voxel-steps/s FP32-batched vs FP64 plain, 1 GB300, <=1e-4 rel err; p50/p99 latency",
        "value": value, "unit": "voxel-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak" if world > 1 else "weak",
        "vs_baseline": None, "dtype": "complex-f32 (f64 phase argument and Sherman-Morrison scalars)"
        if prec == "fp32" else "complex-f64",
        "data": "synthetic (seeded director fields, no dataset)",
        "config": {"workload": samples[0]["desc"], "precision": prec, "voxel_steps_per_step": vs,
                   "l2": l2_note,
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "clocks": clocks, "gpu_launches": launches, "wall_s": wall,
        "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "fp64_plain": fp64, "fma_peaks_measured": peaks_meas,
        "uneven": unev, "line_solves": tuning,
        "kernel_profile": {k: {"ms_per_step": v["ms"], "launches_per_step": v["launches"]} for k, v in (prof or {}).items()},
    }
    if rank == 0:
        print(json.dumps(line))


def uneven_batch_record(steps=2):
    """Sub-record for the largest single-GPU configuration (four uneven samples 1024^2x200,
    768^2x160, 512^2x96, 256^2x48, FP32 batched, one plan): device-resident value over `steps`
    timed executions after one warm-up, e2e through nbpm_run_batch with pinned host buffers (one
    warm-up call, one timed call), and the FP32 relative L2 error of the 512^2x96 sample against
    an FP64 plain run of that sample alone."""
    import torch
    from nemaktis_gb300 import api
    samples = workload("uneven")
    vs = voxel_steps(samples)
    bufs = [{"json": c["json"], "lc": c["lc"], "E": np.zeros(c["shape"], np.complex128)} for c in samples]
    plan = api.Plan(bufs, precision="fp32", groups_per_pass=0)
    tuned_cfg = [plan.solve_config(i)[0] for i in range(len(samples))]
    plan.upload()
    plan.execute()
    torch.cuda.synchronize()
    ms = [plan.execute()["compute_ms"] for _ in range(steps)]
    launches = plan.execute()["kernel_launches"]
    plan.download()
    plan.close()
    # the rule-based line-solve configuration on the same batch, for the tuner's gain
    rb = [{"json": c["json"], "lc": c["lc"], "E": np.zeros(c["shape"], np.complex128)} for c in samples]
    with api.Plan(rb, precision="fp32", groups_per_pass=0, tune=False) as pr:
        pr.upload()
        pr.execute()
        rule_ms = float(pr.execute()["compute_ms"])
        rule_cfg = [pr.solve_config(i)[0] for i in range(len(samples))]
    # each sample alone (its own plan), for the gain of running the samples side by side
    alone_ms = []
    for c in samples:
        b1 = [{"json": c["json"], "lc": c["lc"], "E": np.zeros(c["shape"], np.complex128)}]
        with api.Plan(b1, precision="fp32", groups_per_pass=0) as p1:
            p1.upload()
            p1.execute()
            alone_ms.append(float(np.mean([p1.execute()["compute_ms"] for _ in range(steps)])))
    k = 2  # the 512^2x96 sample
    E64 = np.zeros(samples[k]["shape"], np.complex128)
    api.run(samples[k]["json"], samples[k]["lc"], E64, precision="fp64", groups_per_pass=1)
    err = float(np.linalg.norm(bufs[k]["E"] - E64) / np.linalg.norm(E64))
    e2e = e2e_measure(samples, "fp32", 1)
    return {"workload": samples[0]["desc"], "voxel_steps_per_step": vs, "precision": "fp32",
            "value": vs * steps / (float(np.sum(ms)) / 1e3), "unit": "voxel-steps/s",
            "ms_per_step": float(np.mean(ms)), "steps": steps, "warmup": 1, "gpu_launches_per_step": launches,
            "samples_alone_ms": alone_ms, "samples_alone_sum_ms": float(np.sum(alone_ms)),
            "line_solves": {"configs": tuned_cfg, "rule_based_configs": rule_cfg, "rule_based_ms_per_step": rule_ms},
            "e2e": e2e, "fp32_rel_l2_vs_fp64": {"sample": "512x512x96", "value": err}}


def fma_peaks():
    """FP32/FP64 FMA throughput of the device, from the bench-only probe library."""
    try:
        from nemaktis_gb300 import build as nb
        lib = ctypes.CDLL(nb.build_bench())
    except Exception as e:  # the probe is a reported extra, never a reason to fail the bench
        return {"unavailable": str(e)[:200]}
    f = lib.nbpm_bench_fma_peak
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    out = {}
    for name, prec in (("fp32_tflops", 1), ("fp64_tflops", 0)):
        t = ctypes.c_double()
        if f(prec, ctypes.byref(t)) == 0:
            out[name] = t.value
    return out


def profile_kernels(plan, lib):
    """Per-kernel event timing of one eager execution (nbpm_plan_profile), if available."""
    try:
        f = lib.nbpm_plan_profile
    except AttributeError:
        return None
    n = 32
    names = (ctypes.c_char * 48 * n)()
    ms = (ctypes.c_double * n)()
    cnt = (ctypes.c_int * n)()
    by = (ctypes.c_double * n)()
    k = ctypes.c_int(n)
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.POINTER(ctypes.c_int)]
    rc = f(plan._h, names, ms, cnt, by, ctypes.byref(k))
    if rc != 0:
        return None
    out = {}
    for i in range(k.value):
        nm = bytes(names[i]).split(b"\0")[0].decode()
        out[nm] = {"ms": ms[i], "launches": cnt[i], "bytes": by[i]}
    return out


def e2e_measure(samples, prec, steps):
    from nemaktis_gb300 import _lib
    lib = _lib.load()
    keep = []
    arr = (_lib.Sample * len(samples))()
    h2d = d2h = 0
    for i, c in enumerate(samples):
        lc, t1 = pinned(c["lc"].shape, np.float64)
        lc[...] = c["lc"]
        E, t2 = pinned(c["shape"], np.complex128)
        E[...] = 0
        mask = None
        if c.get("mask") is not None:
            mask, t3 = pinned(c["mask"].shape, np.float64)
            mask[...] = c["mask"]
            keep.append(t3)
            h2d += mask.nbytes
        js = c["json"].encode()
        fm = c.get("formula")
        fm = None if fm is None else fm.encode()
        keep += [lc, E, mask, t1, t2, js, fm]
        arr[i] = _lib.Sample(js, fm, lc.ctypes.data, lc.size, None if mask is None else mask.ctypes.data,
                             0 if mask is None else mask.size, E.ctypes.data, E.size)
        h2d += lc.nbytes
        d2h += E.nbytes
    o = _lib.options(precision=_lib.FP32 if prec == "fp32" else _lib.FP64)
    t = _lib.Timing()
    _lib.check(lib.nbpm_run_batch(len(samples), arr, ctypes.byref(o), ctypes.byref(t)))  # warm-up
    walls = []
    for _ in range(steps):
        t0 = time.perf_counter()
        _lib.check(lib.nbpm_run_batch(len(samples), arr, ctypes.byref(o), ctypes.byref(t)))
        walls.append(time.perf_counter() - t0)
    vs = voxel_steps(samples)
    w = float(np.median(walls))
    return {"value": vs / w, "unit": "voxel-steps/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": w * 1e3, "api": "nbpm_run_batch (C ABI, pinned host buffers; the device plan is kept between calls with the same settings)",
            "breakdown_ms": {"upload": t.upload_ms, "compute": t.compute_ms, "download": t.download_ms,
                             "total": t.total_ms}}


def cpu_sample(samples):
    """The CPU baseline's bounded sample of a workload: the first wavelength with every wave vector
    and both polarisations (2*Nq propagations sharing that wavelength's permittivity, operators and
    factorisations, as in BPMIteration.cpp:127-146), every slab, plus the screen filter, of the
    workload's smallest sample. Returns (json, sample dict, shape, voxel-steps of one run)."""
    import json as _json
    c = min(samples, key=lambda c: int(np.prod(c["shape"][-2:])) * c["Nz"])
    j = _json.loads(c["json"])
    co = j["Physics settings"]["Coefficients"]
    co["Wavelengths"] = co["Wavelengths"][:1]
    Nl, Nq, _, Ny, Nx = c["shape"]
    shape = (1, Nq, 4, Ny, Nx)
    vs = Nx * Ny * (c["Nz"] - 1) * 2 * Nq
    return _json.dumps(j), c, shape, vs


def cpu_baseline(samples, seconds, max_runs=50):
    """Oracle (FP64 C++/OpenMP, all host threads) on the bounded sample of cpu_sample(), repeated
    until `seconds` have elapsed (at least one run)."""
    import oracle
    js, c, shape, vs = cpu_sample(samples)
    runs, t0 = 0, time.perf_counter()
    while True:
        E = np.zeros(shape, np.complex128)
        if c.get("mask") is not None:
            oracle.run_backend_with_mask(js, c.get("formula") or "", c["lc"], c["mask"], E)
        else:
            oracle.run_backend_without_mask(js, c["lc"], E)
        runs += 1
        el = time.perf_counter() - t0
        if el > seconds or runs >= max_runs:
            break
    Ny, Nx = shape[-2:]
    return {"value": vs * runs / el, "unit": "voxel-steps/s", "cores": oracle.num_threads(), "kind": "port",
            "seconds": el, "runs": runs, "voxel_steps_per_run": vs,
            "sample": "1 wavelength x %d q x 2 pol (%d propagations sharing the wavelength's operators) of the "
                      "%dx%dx%d sample, all %d slabs + screen filter, %d run(s) in %.1f s"
                      % (shape[1], 2 * shape[1], Nx, Ny, c["Nz"], c["Nz"] - 1, runs, el)}


def run_reference(args):
    """The reference arm: the CPU oracle (the reference's algorithm restated in FP64 C++/OpenMP;
    the reference itself cannot be built here) on all host threads. Each step is one timed run
    of the bounded sample of cpu_sample(); value = its voxel-steps / its time."""
    world, rank, local = dist_env()
    if rank != 0:
        return
    samples = workload(args.workload)
    recs = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(samples, 0.0, max_runs=1)
        if i >= args.warmup:
            recs.append(r)
    secs = [r["seconds"] for r in recs]
    vs_run = recs[0]["voxel_steps_per_run"]
    v = vs_run * len(recs) / float(np.sum(secs))
    cpu = recs[-1]
    line = {"impl": "reference", "metric": "voxel-steps/s FP32-batched vs FP64 plain, 1 GB300, <=1e-4 rel err; p50/p99 latency",
            "value": v, "unit": "voxel-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * float(np.mean(secs)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "complex-f64",
            "data": "synthetic (seeded director fields, no dataset)",
            "config": {"workload": samples[0]["desc"], "precision": "fp64 CPU oracle (reference not buildable here)",
                       "step": "one run of the bounded sample: " + cpu["sample"].split(", %d run" % cpu["runs"])[0],
                       "voxel_steps_per_step": vs_run},
            "cpu_baseline": {"value": v, "unit": "voxel-steps/s", "cores": cpu["cores"], "kind": "port",
                             "sample": cpu["sample"]},
            "e2e": {"value": v, "unit": "voxel-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def _replay(srv, trace, keep_outputs, sample_every=0.25):
    """Submits each request of the trace at its arrival time (real time) and waits for all.
    Returns (infos, wall seconds, outputs of the requests in keep_outputs, queue samples)."""
    from nemaktis_gb300 import workloads
    samples = []
    stop = threading.Event()
    t0 = time.perf_counter()

    def sampler():
        while not stop.is_set():
            st = srv.stats()
            samples.append((time.perf_counter() - t0, st["queued"], st["running"], st["done"]))
            stop.wait(sample_every)

    th = threading.Thread(target=sampler, daemon=True)
    th.start()
    hs, outs = [], {}
    for k, t in enumerate(trace):
        dt = t0 + t["arrival"] - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        E = workloads.new_fields(t["shape"])
        if k in keep_outputs:
            outs[k] = E
        hs.append(srv.submit(t["json"], t["lc"], E, t["mask"], t["formula"]))
        del E
    infos = []
    for h in hs:
        infos.append(h.wait())  # a finished request drops its buffers
    wall = time.perf_counter() - t0
    stop.set()
    th.join(timeout=2)
    return infos, wall, outs, samples


def _fifo(trace, service_s):
    """Latencies (ms) of a one-at-a-time FIFO server with the given service times."""
    clock, lat = 0.0, []
    for t, svc in zip(trace, service_s):
        clock = max(clock, t["arrival"]) + svc
        lat.append(1e3 * (clock - t["arrival"]))
    return np.array(lat), clock


def run_serve(args):
    """Serving (the Poisson request-stream configuration: 50 req/s, meshes 64^2x32 .. 512^2x128,
    1-32 wavelengths, 1-19 wave vectors, 2 polarisations, FP32, 150 GB device budget).

    1. Offered load: a window of `--serve-requests` arrivals of the seeded 50 req/s trace,
       replayed in real time against the FP32 server. The mix needs far more device time than 50
       req/s leaves, so the queue grows: reported are the completion rate while the server is
       backlogged (its saturation throughput on this mix), the ratio of offered to served rate,
       the queue length over time and p50/p99 latency of the window.
    2. Below saturation: `--serve-below` requests of the same mix arriving at half the measured
       saturation rate; p50/p99 latency of a stable queue.
    3. FP64 one request at a time: the plain FP64 path's service time measured on a sample of the
       requests (one per mesh size where present), modelled per voxel-step for the others, and a
       FIFO queue simulated on both traces; the FP32 results of the sampled requests are compared
       with the FP64 ones (relative L2).
    Directors are drawn from a pool of seeds per generator and mesh (run time does not depend on
    their values)."""
    from nemaktis_gb300 import api, workloads
    from nemaktis_gb300.serving import Server
    n_over = args.serve_requests
    trace = workloads.serving_trace(n_over, rate=50.0, seed=0, director_pool=3)
    # FP64 sample: the first request of each mesh size
    sample_idx, seen = [], set()
    for k, t in enumerate(trace):
        if t["dims"] not in seen:
            seen.add(t["dims"])
            sample_idx.append(k)
    wu = workloads.serving_trace(1, seed=99)[0]
    clk = Clocks()
    with Server(precision="fp32") as srv:
        E = workloads.new_fields(wu["shape"])
        srv.submit(wu["json"], wu["lc"], E, wu["mask"], wu["formula"]).wait()
        del E
        clk.start()
        infos, wall, outs32, qs = _replay(srv, trace, set(sample_idx))
        st = srv.stats()
    lat = np.array([i["latency_ms"] for i in infos])
    vs = np.array([t["voxel_steps"] for t in trace], float)
    # saturation: completions while the queue was non-empty after the last arrival
    t_last = trace[-1]["arrival"]
    busy = [q for q in qs if q[0] >= t_last and q[1] + q[2] > 0]
    if len(busy) >= 2:
        sat_rps = (busy[-1][3] - busy[0][3]) / max(1e-9, busy[-1][0] - busy[0][0])
    else:
        sat_rps = len(trace) / wall
    sat_vs = float(vs.sum() / wall)
    # below saturation
    rate_below = max(0.05, 0.5 * sat_rps)
    trace_b = workloads.serving_trace(args.serve_below, rate=rate_below, seed=1, director_pool=3)
    with Server(precision="fp32") as srv:
        infos_b, wall_b, _, qs_b = _replay(srv, trace_b, set())
    clocks = clk.stop()
    lat_b = np.array([i["latency_ms"] for i in infos_b])
    # FP64 one at a time: measured on the sample, per voxel-step for the rest
    svc64, errs = {}, []
    for k in sample_idx:
        t = trace[k]
        E = workloads.new_fields(t["shape"])
        # the first call of a shape also tunes its line solves and builds its graph: time the second
        api.run(t["json"], t["lc"], E, mask=t["mask"], formula=t["formula"], precision="fp64", groups_per_pass=1)
        s0 = time.perf_counter()
        api.run(t["json"], t["lc"], E, mask=t["mask"], formula=t["formula"], precision="fp64", groups_per_pass=1)
        svc64[k] = time.perf_counter() - s0
        errs.append(float(np.linalg.norm(outs32[k] - E) / np.linalg.norm(E)))
    by_dims = {trace[k]["dims"]: svc64[k] / trace[k]["voxel_steps"] for k in sample_idx}

    def model(tr):
        return [svc64.get(k, by_dims.get(t["dims"], np.mean(list(by_dims.values()))) * t["voxel_steps"])
                if tr is trace else by_dims.get(t["dims"], np.mean(list(by_dims.values()))) * t["voxel_steps"]
                for k, t in enumerate(tr)]

    lat64, mk64 = _fifo(trace, model(trace))
    lat64_b, mk64_b = _fifo(trace_b, model(trace_b))
    qgrowth = [{"t_s": round(q[0], 2), "queued": q[1], "running": q[2], "done": q[3]} for q in qs[::max(1, len(qs) // 40)]]
    line = {
        "metric": "serving: voxel-steps/s and p50/p99 end-to-end latency, FP32 continuous batching vs FP64 one at a time",
        "value": sat_vs, "unit": "voxel-steps/s", "n_gpus": 1, "steps": 1, "warmup": 1,
        "higher_is_better": True, "dtype": "complex-f32", "data": "synthetic (seeded trace, director pool of 3 seeds per generator and mesh)",
        "config": {"workload": "serving mix: Poisson 50 req/s, meshes 64^2x32..512^2x128 (p .4/.3/.2/.1), 1-32 "
                               "wavelengths, 1-19 q, 2 pol, d=0.25um, device budget 150 GB",
                   "window_requests": len(trace), "window_arrival_s": t_last,
                   "mean_request_voxel_steps": float(vs.mean())},
        "offered_load": {"rate_rps": 50.0, "served_rps_saturated": sat_rps, "overload_factor": 50.0 / max(1e-9, sat_rps),
                         "wall_s": wall, "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                         "mean_queue_ms": float(np.mean([i["queue_ms"] for i in infos])),
                         "peak_device_gb": st["peak_bytes"] / 1e9, "queue_over_time": qgrowth,
                         "done": st["done"], "failed": st["failed"]},
        "below_saturation": {"rate_rps": rate_below, "requests": len(trace_b), "wall_s": wall_b,
                             "p50_ms": float(np.percentile(lat_b, 50)), "p99_ms": float(np.percentile(lat_b, 99))},
        "fp64_one_at_a_time": {"measured_requests": len(sample_idx), "service_s_per_voxel_step": {"x".join(map(str, d)): v for d, v in by_dims.items()},
                               "offered_load": {"value": float(vs.sum() / mk64), "makespan_s": mk64,
                                                "p50_ms": float(np.percentile(lat64, 50)), "p99_ms": float(np.percentile(lat64, 99))},
                               "below_saturation": {"p50_ms": float(np.percentile(lat64_b, 50)),
                                                    "p99_ms": float(np.percentile(lat64_b, 99))}},
        "max_rel_l2_fp32_vs_fp64": max(errs) if errs else None,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="koehler", choices=["tn", "droplet", "koehler", "koehler_small", "uneven", "serve"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-uneven", action="store_true", help="no four-sample (uneven batch) sub-record in the default line")
    ap.add_argument("--no-tune", action="store_true", help="rule-based line-solve configuration (no timing runs)")
    ap.add_argument("--solve-config", default=None, help='force a line-solve configuration "<x>;<y>"')
    ap.add_argument("--only-value", action="store_true", help="time the device-resident run only")
    ap.add_argument("--serve-requests", type=int, default=100, help="arrivals of the 50 req/s window")
    ap.add_argument("--serve-below", type=int, default=30, help="requests of the below-saturation trace")
    args = ap.parse_args()
    world, rank, local = dist_env()
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "serve":
        run_serve(args)
    else:
        run_ours(args)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
