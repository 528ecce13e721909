"""Build recipe for the reference's own GPU bar (test infrastructure only).

Compiles the reference's CUDA program cuda/schwarzschild_render.cu, from its
source where it lies in the reference checkout, to a device-only cubin for the
GB300 in oracle/_ref/. Only its `trace_kernel` is used: bench.py's render
workload loads the cubin through the CUDA driver API and times the kernel at
the program's own launch shape (16x16 blocks, one pixel per thread) and its
parameters, as the FP64 GPU bar the new FP64 kernel is compared with. Nothing
here is copied into this repository; the cubin is a build output (git-ignored)
made only where the reference checkout exists, and travels as a prebuilt file.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
CUBIN = os.path.join(OUT, "schwarzschild_render.cubin")
# the reference checkout: GEON_REFERENCE_DIR, else a checkout named "reference"
# beside this repository
REFERENCE = os.environ.get("GEON_REFERENCE_DIR") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
SRC = os.path.join(REFERENCE, "cuda", "schwarzschild_render.cu")
# the kernel's mangled name: trace_kernel(int, int, double, double, double,
# double, int, double, double, int*, double*)
KERNEL = "_Z12trace_kerneliiddddiddPiPd"


def build(force=False):
    """Compile the cubin when the reference checkout is present; returns its
    path, or None when neither the source nor a prebuilt cubin exists."""
    if not os.path.exists(SRC):
        return CUBIN if os.path.exists(CUBIN) else None
    if not force and os.path.exists(CUBIN) and os.path.getmtime(CUBIN) >= os.path.getmtime(SRC):
        return CUBIN
    os.makedirs(OUT, exist_ok=True)
    nvcc = "nvcc"
    for cand in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(cand):
            nvcc = cand
    tmp = CUBIN + ".tmp%d" % os.getpid()
    # the reference builds with nvcc defaults (-arch=sm_100, fused multiply-add on)
    subprocess.run([nvcc, "-cubin", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", SRC, "-o", tmp],
                   check=True)
    os.replace(tmp, CUBIN)
    return CUBIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
