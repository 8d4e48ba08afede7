"""Build recipe of libnomad_gpu.so and the nomad_gpu command-line driver.

CUDA sources are compiled by nvcc for sm_103a only; host sources by g++.  Objects are
rebuilt when a source or header is newer than the object, and translation units
compile in parallel, so a rebuild after a small change takes seconds.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libnomad_gpu.so")
CLI = os.path.join(BUILD, "nomad_gpu")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["kernels_async.cu", "kernels_sgd.cu", "kernels_eval.cu", "csc_device.cu", "layout_device.cu"]
CPP_SOURCES = ["ctx.cpp", "batch.cpp", "host_layout.cpp", "host_io.cpp", "host_synth.cpp", "host_stage.cpp"]
CLI_SOURCES = ["nomad_main.cpp"]

NVCC_FLAGS = [GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-pthread", "-Wall", "-Wextra",
             "-Wno-unused-parameter", "-I" + INCLUDE, "-I" + CSRC,
             "-I" + os.path.join(CUDA_HOME, "include")]


def _headers():
    hs = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh", ".hpp")):
                hs.append(os.path.join(d, f))
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _compile(src, ptxas_verbose=False):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if not _stale(obj, [path] + _headers()):
        return obj, ""
    if src.endswith(".cu"):
        cmd = [NVCC] + NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_verbose else []) + \
              ["-c", path, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-c", path, "-o", obj]
    return obj, _run(cmd)


def build(verbose=False, ptxas_verbose=False, jobs=None):
    """Compile everything; return the path of libnomad_gpu.so."""
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(BUILD, exist_ok=True)
    srcs = CU_SOURCES + CPP_SOURCES + CLI_SOURCES
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 1)) as ex:
        results = list(ex.map(lambda s: _compile(s, ptxas_verbose), srcs))
    objs = {s: o for s, (o, _) in zip(srcs, results)}
    if verbose:
        for s, (_, out) in zip(srcs, results):
            if out.strip():
                print(f"== {s}\n{out}")
    lib_objs = [objs[s] for s in CU_SOURCES + CPP_SOURCES]
    if _stale(LIB, lib_objs):
        _run([NVCC, GENCODE, "-shared", "-o", LIB] + lib_objs + ["-lpthread", "-ldl", "-lrt"])
    cli_objs = [objs[s] for s in CLI_SOURCES]
    if _stale(CLI, cli_objs + [LIB]):
        _run([NVCC, GENCODE, "-o", CLI] + cli_objs + lib_objs + ["-lpthread", "-ldl", "-lrt"])
    return LIB


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)


if __name__ == "__main__":
    build(verbose=True, ptxas_verbose="-v" in sys.argv)
    print(LIB)
