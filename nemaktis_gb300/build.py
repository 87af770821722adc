"""Compile libnbpm.so (the sm_103a CUDA backend) in-tree with nvcc.

Output: nemaktis_gb300/_build/libnbpm.so (git-ignored), compiled from a few translation units
in parallel with one -gencode (compute_103a / sm_103a), so a rebuild on a fresh machine takes
well under a minute. build_bench() compiles the benchmark's FMA probe (bench_peaks.cu beside
bench.py) into its own library, libnbpm_bench.so, which the product library does not contain.
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libnbpm.so")
SOURCES = ["nbpm.cu", "solve_x_f32.cu", "solve_x_f64.cu", "solve_y_f32.cu", "solve_y_f64.cu", "linesolve.cu",
           "linesolve_noalloc.cu", "micrograph.cu", "serve.cu"]
HEADERS = ["bpm_kernels.cuh", "fft_kernels.cuh", "cplx.cuh", "host_settings.h", "host_expr.h", "host_json.h",
           "solve_dispatch.cuh", "solve_config.h", "plan_iface.h", "vti_writer.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
BENCH_SRC = os.path.join(HERE, "..", "bench_peaks.cu")
BENCH_LIB = os.path.join(BUILD, "libnbpm_bench.so")


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnbpm.so")
    return exe


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(HERE, "..", "include", "nbpm.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False, extra=()):
    """Build libnbpm.so if it is missing or older than its sources; returns its path.

    The translation units compile in parallel (one nvcc process each), then link."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    flags = ["-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp", *extra]
    procs, objs = [], []
    for f in SOURCES:
        obj = os.path.join(BUILD, f.replace(".cu", ".o"))
        cmd = [nvcc(), *flags, "-c", "-o", obj, os.path.join(CSRC, f)]
        if verbose:
            print(" ".join(cmd))
        procs.append((f, subprocess.Popen(cmd)))
        objs.append(obj)
    bad = [f for f, p in procs if p.wait() != 0]
    if bad:
        raise RuntimeError("nvcc failed for " + ", ".join(bad))
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lgomp"], check=True)
    os.replace(tmp, LIB)
    return LIB


def build_bench(force=False):
    """Build libnbpm_bench.so (the benchmark's FMA throughput probe) if missing or stale."""
    if not force and os.path.exists(BENCH_LIB) and os.path.getmtime(BENCH_LIB) >= os.path.getmtime(BENCH_SRC):
        return BENCH_LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = BENCH_LIB + ".tmp%d" % os.getpid()
    subprocess.run([nvcc(), "-O3", "-std=c++17", *ARCH, "-Xcompiler", "-fPIC", "-shared", "-o", tmp, BENCH_SRC],
                   check=True)
    os.replace(tmp, BENCH_LIB)
    return BENCH_LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
