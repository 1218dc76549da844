"""Build recipe for the oracle (test infrastructure only).

* ``build_oracle()`` compiles ``gg_oracle.c`` (the CPU restatement of the
  reference projection kernels) into ``oracle/_build/libgg_oracle.so`` with
  gcc.  ``-ffp-contract=off`` keeps x86-64 and aarch64 results bit-identical.
* ``build_ref()`` compiles the reference's own projection kernels
  (``src/Projection/gpuForwardProject.cu`` and ``gpuBackProject.cu`` of
  tagarelab/MultiGPUGridder) and its twelve filters (``src/Filters/*Filter.cu``),
  read in place from the reference checkout, into cubins under
  ``oracle/_ref/``.  Nothing from the reference is copied: nvcc reads the
  sources where they lie and writes only the compiled device code.  The
  filters include ``nvToolsExt.h`` by its pre-CUDA-12 path; a one-line header
  written under ``oracle/_build/shim/`` forwards it to the toolkit's
  ``nvtx3/nvToolsExt.h``.
  The cubins hold GPU code only, so they run on any host architecture; the
  runner in ``oracle/ref_kernels.py`` loads them through the CUDA driver API.
  It is skipped when the reference checkout is absent; a machine without the
  checkout uses cubins built where it was present.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "libgg_oracle.so")
# The reference checkout this recipe reads (GG_REFERENCE_ROOT overrides it).
REFERENCE_ROOT = os.environ.get("GG_REFERENCE_ROOT", "/root/reference")
REF_CUBINS = {
    "fp": ("src/Projection/gpuForwardProject.cu", os.path.join(REF_DIR, "ref_fp.cubin")),
    "bp": ("src/Projection/gpuBackProject.cu", os.path.join(REF_DIR, "ref_bp.cubin")),
}
REF_FILTERS = ("ComplexToCAS", "CASToComplex", "FFTShift2D", "FFTShift3D", "PadVolume", "CropVolume",
               "DivideVolume", "MultiplyVolume", "AddVolume", "DivideScalar", "RealToComplex", "ComplexToReal")
for _f in REF_FILTERS:
    REF_CUBINS["filter_" + _f] = ("src/Filters/%sFilter.cu" % _f, os.path.join(REF_DIR, "ref_%s.cubin" % _f))
SHIM_DIR = os.path.join(BUILD_DIR, "shim")


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    src = os.path.join(HERE, "gg_oracle.c")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and not _stale(ORACLE_SO, [src, __file__]):
        return ORACLE_SO
    cc = shutil.which("gcc") or "cc"
    tmp = ORACLE_SO + ".tmp%d" % os.getpid()
    cmd = [cc, "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-std=c11", src, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_available():
    return os.path.isdir(os.path.join(REFERENCE_ROOT, "src", "Projection"))


def build_ref(force=False):
    """Compile the reference kernels to sm_103a cubins; returns the paths or None."""
    if not reference_available():
        return None
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    os.makedirs(REF_DIR, exist_ok=True)
    os.makedirs(SHIM_DIR, exist_ok=True)
    shim = os.path.join(SHIM_DIR, "nvToolsExt.h")
    if not os.path.exists(shim):
        with open(shim, "w") as f:
            f.write("#include <nvtx3/nvToolsExt.h>\n")
    jobs, out = [], {}
    for key, (rel, dst) in REF_CUBINS.items():
        src = os.path.join(REFERENCE_ROOT, rel)
        if force or _stale(dst, [src]):
            jobs.append([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                         "-I" + os.path.join(REFERENCE_ROOT, "src", "Structs"),
                         "-I" + os.path.join(REFERENCE_ROOT, "src", "Filters"), "-I" + SHIM_DIR, src,
                         "-o", dst + ".tmp%d" % os.getpid()])
        out[key] = dst

    def run(cmd):
        subprocess.run(cmd, check=True, capture_output=True)
        os.replace(cmd[-1], cmd[-1].rsplit(".tmp", 1)[0])

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
