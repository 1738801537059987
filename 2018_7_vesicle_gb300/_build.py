"""Build recipe of the CUDA library: every ``csrc/*.cu`` compiled for sm_103a in parallel
and linked into ``lib/libvsl_gb300.so`` (in-tree, git-ignored).

    __graft_entry__.build()  (or the package's build())

``python 2018_7_vesicle_gb300/_build.py --nvtx`` rebuilds every object with NVTX ranges around
the C-ABI operations (-DVSL_NVTX, for timeline profilers); run it without ``--nvtx`` (it
rebuilds every object too) to return to the default library.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(OUT_DIR, "libvsl_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE]
# The plain FP64 form rounds every product and sum separately, as the reference's kernels
# (and the host oracle) do, so it can match them to the last bit: no mul+add contraction.
FILE_FLAGS = {
    "vsl_plain.cu": ["-fmad=false"],
    "vsl_fused_f64.cu": ["-fmad=false"],
    "vsl_toolbox.cu": ["-fmad=false"],
    # The mixed form's FP32 stencils use the hardware-approximate quotient and square root
    # (FP64 code in the same file keeps IEEE division and square root).
    "vsl_fused_f32.cu": ["-prec-div=false", "-prec-sqrt=false"],
    "vsl_toolbox_f32.cu": ["-prec-div=false", "-prec-sqrt=false"],
    "vsl_relax_f64.cu": ["-fmad=false"],
    "vsl_relax_f32.cu": ["-prec-div=false", "-prec-sqrt=false"],
    "vsl_spectral.cu": ["-fmad=false"],
    "vsl_auxi_f64.cu": ["-fmad=false"],
    "vsl_auxi_f32.cu": ["-prec-div=false", "-prec-sqrt=false"],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, extra) -> str:
    obj = os.path.join(OUT_DIR, "obj", os.path.basename(src)[:-3] + ".o")
    if _stale(obj, [src, *headers()]):
        per_file = FILE_FLAGS.get(os.path.basename(src), [])
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *per_file, *extra, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj


def build(force: bool = False, extra_flags=()) -> str:
    os.makedirs(os.path.join(OUT_DIR, "obj"), exist_ok=True)
    if force and os.path.exists(LIB):
        os.remove(LIB)
    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra_flags)), srcs))
    if _stale(LIB, objs):
        tmp = LIB + ".tmp"
        cuda_lib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "lib64")
        # the NVTX ranges' loader of a profiler's injection library needs dlopen
        libdl = ["-ldl"] if "-DVSL_NVTX" in extra_flags else []
        r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcufft", *libdl, "-Xlinker",
                            "-rpath," + cuda_lib], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys

    if len(sys.argv) > 1:
        # an explicit variant: rebuild every object with its flags
        shutil.rmtree(os.path.join(OUT_DIR, "obj"), ignore_errors=True)
        print(build(force=True, extra_flags=["-DVSL_NVTX"] if "--nvtx" in sys.argv[1:] else []))
    else:
        print(build())
