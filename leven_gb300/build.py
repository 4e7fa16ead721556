"""Builds liblvn.so in-tree for sm_103a with nvcc (no torch extension
machinery): each .cu translation unit is compiled in parallel, then linked
into leven_gb300/liblvn.so."""
import concurrent.futures
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "liblvn.so"
SOURCES = ["lvn_kernels.cu", "lvn_api.cu", "lvn_noalloc.cu", "lvn_surrogate.cu", "lvn_clipmap.cu",
           "lvn_seam.cu", "lvn_collapse.cu", "lvn_render.cu"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
# -fmad=false: no implicit multiply-add contraction, so that density signs are
# the exact IEEE sequence the kernels spell out (explicit fmaf where fused).
NVCC_FLAGS = ["-O3", "-std=c++17", ARCH, "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; liblvn needs the CUDA 13 toolkit")
    return cand


def _compile(src: str) -> pathlib.Path:
    obj = BUILD / (pathlib.Path(src).stem + ".o")
    cmd = [nvcc(), *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)]
    subprocess.run(cmd, check=True)
    return obj


def build(force: bool = False) -> pathlib.Path:
    BUILD.mkdir(exist_ok=True)
    deps = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + \
        [PKG.parent / "include" / "lvn.h"]
    if LIB.exists() and not force:
        newest = max(p.stat().st_mtime for p in deps)
        if LIB.stat().st_mtime >= newest:
            return LIB
    with concurrent.futures.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run([nvcc(), ARCH, "-shared", "-cudart=static", "-o", str(tmp), *map(str, objs)], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
