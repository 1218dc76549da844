"""Build recipe for libgg_gridder.so (the C-ABI library) with nvcc, in tree.

Every translation unit is compiled for sm_103a only, in parallel, and linked
against cuFFT.  Objects go to multigpugridder_gb300/_build/, the library to
multigpugridder_gb300/libgg_gridder.so (both git-ignored).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgg_gridder.so")
INCLUDE = os.path.join(ROOT, "include")
SOURCES = ["gg_project.cu", "gg_cas.cu", "gg_api.cu", "gg_noalloc.cu", "gg_serve.cu", "gg_compat.cu", "gg_fft2.cu",
           "gg_measure.cu", "gg_kb.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home():
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hdrs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hdrs + [__file__]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = os.path.join(cuda_home(), "bin", "nvcc")
    if not os.path.exists(nvcc):
        nvcc = "nvcc"
    common = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE] + ARCH
    deps = _deps()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or _stale(o, deps + [s]):
            jobs.append([nvcc] + common + ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        libdir = os.path.join(cuda_home(), "lib64")
        if not os.path.isdir(libdir):
            libdir = os.path.join(cuda_home(), "lib")
        tmp = LIB + ".tmp%d" % os.getpid()
        run([nvcc, "-shared"] + ARCH + ["-o", tmp] + objs +
            ["-L" + libdir, "-lcufft", "-Xlinker", "-rpath=" + libdir])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
