"""Build libinca_gpu.so (sm_103a) and the inca_gpu driver in-tree.

    python -m inca_parallel_gb300.build            # or build() from Python

nvcc compiles each translation unit in parallel for sm_103a only; objects go to
inca_parallel_gb300/_build/, the library and driver next to this file. The screening
translation unit is compiled with -fmad=false (bit-identical screening values).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libinca_gpu.so")
DRIVER = os.path.join(HERE, "inca_gpu")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-I", INCLUDE, "-I", CSRC,
          "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr"]
UNITS = {
    "api.cu": [],
    "quartet_prep.cu": ["-fmad=false"],
    "intracule_eval.cu": [],
    "mixed_eval.cu": [],
    "cube_eval.cu": [],
    "grid_build.cu": ["-fmad=false"],
    "noalloc_eval.cu": [],
    "peak_probe.cu": [],
    "batch.cu": [],
    "mlp.cu": [],
    "host_tables.cpp": [],
}
DRIVER_SRC = os.path.join(CSRC, "driver", "inca_main.cpp")


def nvcc():
    for cand in [shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]:
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))] + \
           [os.path.join(INCLUDE, "inca_gpu.h")]


def _compile(unit, extra, verbose=False):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OBJ, unit + ".o")
    if not _newer(obj, [src] + _headers()):
        return obj
    lang = ["-x", "cu"] if unit.endswith(".cu") else ["-x", "c++"]
    cmd = [nvcc()] + ARCH + COMMON + extra + lang + ["-c", src, "-o", obj + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose=False, ptxas_info=False):
    os.makedirs(OBJ, exist_ok=True)
    extra_info = ["-Xptxas", "-v"] if ptxas_info else []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_compile, u, e + extra_info, verbose) for u, e in UNITS.items()]
        objs = [f.result() for f in futs]
    if _newer(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart_static"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    if os.path.exists(DRIVER_SRC) and _newer(DRIVER, [DRIVER_SRC, LIB] + _headers()):
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", INCLUDE, DRIVER_SRC, "-o", DRIVER + ".tmp",
               "-L", HERE, "-linca_gpu", "-Wl,-rpath,$ORIGIN"]
        subprocess.run(cmd, check=True)
        os.replace(DRIVER + ".tmp", DRIVER)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
