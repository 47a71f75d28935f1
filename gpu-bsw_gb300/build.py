"""Builds the package's native libraries in-tree (no cmake, no setup.py).

* ``_lib/libgbsw.so``       -- the product: CUDA kernels (sm_103a only) + C ABI +
                               the C++ drop-in of gpu_bsw_driver, by nvcc.
* ``_lib/libgbsw_synth.so`` -- host-only synthetic workload generator, by g++.
* ``_lib/program_gpu``      -- the command-line front end with the reference
                               program's I/O conventions, by g++ over libgbsw.so.

Translation units compile in parallel; a library is rebuilt only when one of
its sources or headers is newer than it.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

from ._paths import CSRC, INCLUDE, LIBDIR, GBSW_LIB

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                     "-I" + INCLUDE, "-I" + CSRC] + os.environ.get("GBSW_NVCC_FLAGS", "").split()
GBSW_SOURCES = ["sw_kernels.cu", "sw_wide.cu", "sw_dual.cu", "traceback.cu", "schedule.cu", "capi.cu", "calib.cu",
                "noalloc.cu", "unpack.cu", "pack.cpp", "driver.cpp",
                "pinned_pool.cpp",
                "server.cpp"]
SYNTH_LIB = os.path.join(LIBDIR, "libgbsw_synth.so")
PROGRAM = os.path.join(LIBDIR, "program_gpu")


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
            + glob.glob(os.path.join(CSRC, "*.inc"))
            + glob.glob(os.path.join(INCLUDE, "*.h")) + glob.glob(os.path.join(INCLUDE, "*", "*.hpp")))


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build_gbsw(force=False, verbose=False):
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in GBSW_SOURCES]
    if not force and not _stale(GBSW_LIB, srcs + _headers()):
        return GBSW_LIB
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    jobs = []
    for s in srcs:
        obj = os.path.join(objdir, os.path.basename(s) + ".o")
        extra = ["-x", "cu"] if s.endswith(".cu") else []
        jobs.append(([NVCC] + NVCC_FLAGS + extra + ["-c", s, "-o", obj], obj))
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(lambda j: _run(j[0]), jobs))
    if verbose:
        for o in outs:
            print(o, end="")
    tmp = GBSW_LIB + ".tmp"
    _run([NVCC] + ARCH + ["-shared", "-o", tmp] + [o for _, o in jobs] + ["-lpthread"])
    os.replace(tmp, GBSW_LIB)
    return GBSW_LIB


def build_synth(force=False):
    os.makedirs(LIBDIR, exist_ok=True)
    src = os.path.join(CSRC, "synth.cpp")
    if not force and not _stale(SYNTH_LIB, [src, os.path.join(INCLUDE, "gbsw_synth.h")]):
        return SYNTH_LIB
    tmp = SYNTH_LIB + ".tmp"
    _run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", tmp, src])
    os.replace(tmp, SYNTH_LIB)
    return SYNTH_LIB


def build_program(force=False):
    """program_gpu, linked against libgbsw.so in the same folder (found through $ORIGIN)."""
    src = os.path.join(CSRC, "program.cpp")
    deps = [src, GBSW_LIB] + glob.glob(os.path.join(INCLUDE, "gpu_bsw", "*.hpp"))
    if not force and not _stale(PROGRAM, deps):
        return PROGRAM
    tmp = PROGRAM + ".tmp"
    _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, "-o", tmp, src, "-L" + LIBDIR, "-lgbsw",
          "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, PROGRAM)
    return PROGRAM


def build_all(force=False, verbose=False):
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_gbsw, force, verbose)
        b = ex.submit(build_synth, force)
        lib, synth = a.result(), b.result()
    build_program(force)
    return lib, synth


if __name__ == "__main__":
    print(build_all(force=True, verbose=True))
