"""Build recipe of libb2d.so, the CUDA library behind include/b2d.h.

Each translation unit is compiled for sm_103a only, in parallel, then linked
into app-binary2d_gb300/_build/libb2d.so.  Flags per unit:

  kernels_f64.cu   --fmad=false   FP64 parity kernels: every operation rounds as written
  api.cu           --fmad=false   Kepler solve and time bookkeeping in exact FP64
  kernels_f32.cu   fast FP32      -ftz, approximate division and square root
  kernels_f32e.cu  fast FP32      the paired Euler kernel, same flags
  host_ic.cpp      g++ -ffp-contract=off   geometry and initial states
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libb2d.so")
# The read-set check build (B2D_POISON, see csrc/tma.cuh): the same library
# with never-written shared-memory slots and unused guard values set to NaN.
# Tests load it to show that the states do not change; it is built on demand.
POISON_BUILD = os.path.join(HERE, "_build_poison")
POISON_LIB = os.path.join(POISON_BUILD, "libb2d.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE]

UNITS = {
    "kernels_f64.cu": ["--fmad=false"],
    "api.cu": ["--fmad=false"],
    "kernels_f32.cu": ["-ftz=true", "-prec-div=false", "-prec-sqrt=false", "--fmad=true"],
    "kernels_f32e.cu": ["-ftz=true", "-prec-div=false", "-prec-sqrt=false", "--fmad=true"],
}
HOST_UNITS = {"host_ic.cpp": ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread"]}


def _nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return path


def _sources():
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(INCLUDE, "b2d.h"))
    return deps


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(force: bool = False, verbose: bool = False, poison: bool = False) -> str:
    """Compile libb2d.so (poison=True: the read-set check variant in
    _build_poison/) if a source is newer than it; returns its path."""
    build_dir, lib = (POISON_BUILD, POISON_LIB) if poison else (BUILD, LIB)
    extra = ["-DB2D_POISON"] if poison else []
    deps = _sources() + [os.path.abspath(__file__)]
    if not force and not _stale(lib, deps):
        return lib
    os.makedirs(build_dir, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src, flags in UNITS.items():
        obj = os.path.join(build_dir, src + ".o")
        objs.append(obj)
        cmd = [nvcc] + ARCH + NVCC_COMMON + flags + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        jobs.append(cmd)
    for src, flags in HOST_UNITS.items():
        obj = os.path.join(build_dir, src + ".o")
        objs.append(obj)
        jobs.append(["g++"] + flags + ["-I", INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_compile, jobs))
    if verbose:
        for o in outs:
            print(o)
    tmp = lib + ".tmp%d" % os.getpid()
    _compile([nvcc] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs + ["-lpthread"])
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv))
