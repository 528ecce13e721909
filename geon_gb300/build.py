"""Build the CUDA library in-tree: geon_gb300/_lib/libgeon_gpu.so (sm_103a),
and the C++ ports of the reference's executables over include/geon.hpp
(geon_gb300/_lib/bin/: validate_shadow, energy_conditions, render).

Every translation unit is compiled by nvcc in parallel, then linked into one
shared library that exports the C ABI of include/geon_gpu.h. The FP64 parity
units are compiled with --fmad=false: the reference never fuses a*b+c, and the
GPU results must match it bit for bit. Host code is compiled with
-ffp-contract=off for the same reason (aarch64 gcc would fuse by default).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libgeon_gpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
          "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", f"-I{INCLUDE}"]
# (source, extra flags)
UNITS = [
    ("trace_fp64.cu", ["--fmad=false"]),
    ("trace_mixed.cu", ["--fmad=false"]),
    ("trace_adaptive.cu", ["--fmad=false"]),
    ("trace_fp64fast.cu", ["--fmad=false"]),
    ("curvature_fp64.cu", ["--fmad=false"]),
    ("capi.cu", ["--fmad=false"]),
    ("noalloc.cu", ["--fmad=false"]),
    ("serve.cu", ["--fmad=false"]),
    ("energy.cu", ["--fmad=false"]),
]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build geon_gb300")
    return cand


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))]
    files.append(os.path.join(INCLUDE, "geon_gpu.h"))
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


CPP = os.path.join(HERE, "cpp")
BIN = os.path.join(OUT, "bin")
# C++ ports of the reference's executables (bin/validate_shadow.rs,
# bin/energy_conditions.rs, bin/render.rs) over include/geon.hpp
PROGRAMS = ("validate_shadow", "energy_conditions", "render")


def build_programs(force=False):
    """Compile the C++ executables against the library (g++, C++17)."""
    os.makedirs(BIN, exist_ok=True)
    deps = [LIB, os.path.join(INCLUDE, "geon.hpp"), os.path.join(CPP, "rust_fmt.hpp"), os.path.abspath(__file__)]
    newest = max(os.path.getmtime(f) for f in deps)
    out = []
    for name in PROGRAMS:
        exe = os.path.join(BIN, name)
        src = os.path.join(CPP, name + ".cpp")
        out.append(exe)
        if not force and os.path.exists(exe) and os.path.getmtime(exe) >= max(newest, os.path.getmtime(src)):
            continue
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{INCLUDE}", f"-I{CPP}", src, "-o", exe + ".tmp",
               f"-L{OUT}", "-lgeon_gpu", "-Wl,-rpath,$ORIGIN/.."]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed on {name}.cpp:\n{r.stdout}\n{r.stderr}")
        os.replace(exe + ".tmp", exe)
    return out


def build(force=False, verbose=False):
    lib = build_library(force, verbose)
    build_programs(force)
    return lib


def build_library(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    nv = nvcc()

    def compile_unit(unit):
        src, extra = unit
        obj = os.path.join(OUT, src.rsplit(".", 1)[0] + ".o")
        cmd = [nv, *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(16, len(UNITS), os.cpu_count() or 8)) as ex:
        results = list(ex.map(compile_unit, UNITS))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp%d" % os.getpid()
    r = subprocess.run([nv, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
