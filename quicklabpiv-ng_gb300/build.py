"""Builds libqlpiv_gpu.so in-tree (quicklabpiv-ng_gb300/_build/) with nvcc for sm_103a.

Each translation unit under csrc/ is compiled in parallel, then linked into one shared
library whose exported symbols are the C ABI of include/qlpiv.h.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libqlpiv_gpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without FMA contraction (-ffp-contract=off) so float/double host
# expressions round the same way on x86_64 and aarch64.
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3,-ffp-contract=off",
                     "-I", str(ROOT / "include"), "-I", str(CSRC)]
# Per-file device flags: the adaptive stages are bit-identical to the CPU oracle only
# without FMA contraction.
FILE_FLAGS = {"qlpiv_adaptive.cu": ["--fmad=false"], "qlpiv_validate.cu": ["--fmad=false"],
              "qlpiv_dense.cu": ["--fmad=false"]}


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (cand == "nvcc" or Path(cand).exists()):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _deps():
    return list(CSRC.glob("*")) + [ROOT / "include" / "qlpiv.h"]


def up_to_date():
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def build(force=False, verbose=False, ptxas_info=False):
    """Compile and link; returns the library path.  Raises CalledProcessError on failure."""
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_one(src):
        obj = BUILD / (src.stem + ".o")
        cmd = [nvcc, *NVCC_FLAGS, *FILE_FLAGS.get(src.name, []), *extra, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise subprocess.CalledProcessError(r.returncode, cmd, r.stdout, r.stderr)
        if verbose or ptxas_info:
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    srcs = _sources()
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = BUILD / (LIB.name + ".tmp")
    subprocess.run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
