"""Build recipe for the reference-kernel harness (test infrastructure).

- oracle/_ref/cuda_gvdb_module.ptx: the reference's own kernel module, compiled
  from its source file source/gvdb_library/kernels/cuda_gvdb_module.cu of the
  reference checkout ($GVDB_REFERENCE, or the first argument) with the flags of
  its CMake project (PTX, --use_fast_math).  Built only where the reference sources are
  present; the PTX is text, so it also runs on a GPU machine without those
  sources, where the CUDA driver JIT-compiles it.  It is loaded and launched, never
  read.
- oracle/_ref/libref_harness.so: oracle/ref_harness.cu (our restatement of the
  reference's host orchestration) built with nvcc; built on demand.
Outputs go to oracle/_ref/ only (git-ignored).
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# the reference checkout: $GVDB_REFERENCE, else the directory this recipe was set up with
REF_ROOT = os.environ.get("GVDB_REFERENCE", "/root/reference")
REF_KERNELS = os.path.join(REF_ROOT, "source", "gvdb_library", "kernels")
PTX = os.path.join(OUT, "cuda_gvdb_module.ptx")
HARNESS_SRC = os.path.join(HERE, "ref_harness.cu")
HARNESS = os.path.join(OUT, "libref_harness.so")


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def build_ptx():
    src = os.path.join(REF_KERNELS, "cuda_gvdb_module.cu")
    if not os.path.exists(src):
        return PTX if os.path.exists(PTX) else None
    if os.path.exists(PTX) and os.path.getmtime(PTX) >= os.path.getmtime(src):
        return PTX
    os.makedirs(OUT, exist_ok=True)
    cmd = [_nvcc(), "-ptx", "-arch=compute_100", "--use_fast_math", "-std=c++14", "-w", src, "-o", PTX + ".tmp"]
    subprocess.check_call(cmd, cwd=REF_KERNELS)
    os.replace(PTX + ".tmp", PTX)
    return PTX


def build_harness():
    if os.path.exists(HARNESS) and os.path.getmtime(HARNESS) >= os.path.getmtime(HARNESS_SRC):
        return HARNESS
    os.makedirs(OUT, exist_ok=True)
    cmd = [_nvcc(), "-shared", "-Xcompiler", "-fPIC", "-O2", "-std=c++17", "-gencode",
           "arch=compute_103a,code=sm_103a", HARNESS_SRC, "-o", HARNESS + ".tmp", "-lcuda"]
    subprocess.check_call(cmd)
    os.replace(HARNESS + ".tmp", HARNESS)
    return HARNESS


def build():
    """PTX only (quick); the harness library is built by its users."""
    return build_ptx()


if __name__ == "__main__":
    import sys

    if len(sys.argv) > 1:  # python oracle/ref_build.py <reference checkout>
        REF_KERNELS = os.path.join(sys.argv[1], "source", "gvdb_library", "kernels")
    print(build_ptx())
    print(build_harness())
