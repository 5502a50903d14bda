"""Build the native library libfwant_gb300.so in-tree (fwant_gb300/lib/).

CUDA sources are compiled for sm_103a only; host sources go through nvcc as well so
that the CUDA include and library paths come from the toolkit.  Objects are rebuilt
only when a source or header is newer.  Usage: ``python -m fwant_gb300.build``.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libfwant_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
            "-Xptxas", "-O3"]
# the reference-order units: every product and sum rounds separately, as in the
# reference's FP32 source expressions
EXACT_FLAGS = ["-fmad=false"]
# -ffp-contract=off: host set-up arithmetic (PML profiles, source weights) must not
# contract into FMAs on aarch64, where GCC would otherwise do so by default.
CPP_FLAGS = ["-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]

SOURCES = ["stage_fast_rk0.cu", "stage_fast_rk1.cu", "stage_fast_rk2.cu", "stage_exact_rk0.cu",
           "stage_exact_rk1.cu", "stage_exact_rk2.cu", "stage_fast16_rk0.cu", "stage_fast16_rk1.cu",
           "stage_fast16_rk2.cu", "stage_exact16_rk0.cu", "stage_exact16_rk1.cu", "stage_exact16_rk2.cu", "stage_bf16_rk0.cu", "stage_bf16_rk1.cu",
           "stage_bf16_rk2.cu", "stage_fp16_rk0.cu", "stage_fp16_rk1.cu", "stage_fp16_rk2.cu",
           "stage_topo_rk0.cu", "stage_topo_rk1.cu", "stage_topo_rk2.cu", "stage_topo_exact_rk0.cu",
           "stage_topo_exact_rk1.cu", "stage_topo_exact_rk2.cu", "stage_fast_rk3.cu", "stage_fast_rk4.cu",
           "stage_fast_rk5.cu", "stage_fast16_rk3.cu", "stage_fast16_rk4.cu", "stage_fast16_rk5.cu", "stage_topo_rk3.cu",
           "stage_topo_rk4.cu", "stage_topo_rk5.cu", "stage_bf16_rk3.cu", "stage_bf16_rk4.cu", "stage_bf16_rk5.cu",
           "stage_fp16_rk3.cu", "stage_fp16_rk4.cu", "stage_fp16_rk5.cu", "topo.cu",
           "stage_dispatch.cu", "waits.cu", "aux.cu", "snapshot.cu", "sgtker.cu", "surrogate.cu", "lsqr.cu", "media.cu", "assm.cu", "kerinfo.cu", "solver.cpp", "sgtker_api.cpp"]
# units whose FP32 expressions must round like the reference's source (no contraction)
EXACT_SOURCES = {"media.cu"}


EXE = os.path.join(HERE, "bin", "fwant_wave")
EXE_SOURCES = ["fwant_wave.cpp", "netcdf3.cpp", "conf.cpp"]
KER_EXE = os.path.join(HERE, "bin", "fwant_ker")
KER_SOURCES = ["fwant_ker.cpp", "netcdf3.cpp", "conf.cpp"]
LSQR_EXE = os.path.join(HERE, "bin", "fwant_lsqr")
LSQR_SOURCES = ["fwant_lsqr.cpp"]
MEDIA_EXE = os.path.join(HERE, "bin", "fwant_media")
MEDIA_SOURCES = ["fwant_media.cpp", "netcdf3.cpp", "conf.cpp"]
PREP_EXE = os.path.join(HERE, "bin", "fwant_prep")
PREP_SOURCES = ["fwant_prep.cpp", "netcdf3.cpp", "conf.cpp"]
ASSM_EXE = os.path.join(HERE, "bin", "fwant_assm")
ASSM_SOURCES = ["fwant_assm.cpp", "netcdf3.cpp", "conf.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)
    return r


def build(verbose: bool = False, force: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    jobs_todo = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OBJ, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + hdrs):
            flags = CU_FLAGS + ARCH if src.endswith(".cu") else CPP_FLAGS
            if "exact" in src or src in EXACT_SOURCES:
                flags = flags + EXACT_FLAGS
            jobs_todo.append([nvcc, *flags, "-I", CSRC, "-I", INCLUDE, "-c", path, "-o", obj])
    if jobs_todo:
        # one nvcc per core, up to 24 (each stage unit takes ~15 s and a few hundred MB)
        with ThreadPoolExecutor(max_workers=jobs or max(1, min(24, os.cpu_count() or 8, len(jobs_todo)))) as ex:
            list(ex.map(lambda c: _run(c, verbose), jobs_todo))
    if force or jobs_todo or _stale(LIB, objs):
        _run([nvcc, "-shared", *ARCH, "-o", LIB, *objs, "-lcudart"], verbose)
    # the programs over the C ABI: the solver stage (SeisFD3D.conf + NetCDF files in and
    # out), the sensitivity-kernel stage (TomoKernel.conf, sgt_ files in, kernel files out)
    # the inversion (data list, kernel rows, smoothing operator in; model files out), the
    # medium preprocessor (media configuration and model files in; media file out) and the
    # grid, metric, source and station preprocessors (configuration in; coord_, metric_,
    # source_ and station_ files out) and the kernel assembly (kernel files and inversion
    # blocks in; compact kernel rows out)
    for exe, srcs in ((EXE, EXE_SOURCES), (KER_EXE, KER_SOURCES), (LSQR_EXE, LSQR_SOURCES),
                      (MEDIA_EXE, MEDIA_SOURCES), (PREP_EXE, PREP_SOURCES), (ASSM_EXE, ASSM_SOURCES)):
        exe_src = [os.path.join(CSRC, f) for f in srcs]
        if force or _stale(exe, exe_src + hdrs + [LIB]):
            os.makedirs(os.path.dirname(exe), exist_ok=True)
            _run(["g++", "-O2", "-std=c++17", "-Wall", "-ffp-contract=off", "-I", CSRC, "-I", INCLUDE, *exe_src,
                  "-o", exe, "-L", LIB_DIR, "-lfwant_gb300", "-Wl,-rpath,$ORIGIN/../lib"], verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
