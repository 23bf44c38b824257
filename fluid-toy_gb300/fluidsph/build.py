"""Build recipe for libfluidsph.so (the sm_103a SPH step library).

Every translation unit under ``fluid-toy_gb300/csrc`` is compiled in parallel
with nvcc for ``sm_103a`` only and linked in-tree into
``fluid-toy_gb300/fluidsph/libfluidsph.so``. Numerics flags:
``-fmad=false`` keeps every float expression in the shaders' evaluation order
(no fused multiply-add), IEEE division and square root are nvcc's defaults,
and host code is built with ``-ffp-contract=off`` for the same reason.
The reverse-pass kernels (``adj_kernels.cu``) reproduce no reference bits:
they are built with fused multiply-add and the approximate division and
square root (``FILE_FLAGS``).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
ROOT = PKG_DIR.parent
CSRC = ROOT / "csrc"
INCLUDE = ROOT.parent / "include"
BUILD_DIR = ROOT / "_build"
LIB_PATH = PKG_DIR / "libfluidsph.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-std=c++17",
    "-O3",
    "-lineinfo",
    "-fmad=false",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC,-ffp-contract=off,-O2",
    "-I",
    str(INCLUDE),
]


# per-file replacements of NVCC_FLAGS entries
FILE_FLAGS = {
    "adj_kernels.cu": {"-fmad=false": ["-fmad=true", "-prec-div=false", "-prec-sqrt=false"]},
}


def _flags_for(src: Path) -> list[str]:
    sub = FILE_FLAGS.get(src.name, {})
    out: list[str] = []
    for f in NVCC_FLAGS:
        out.extend(sub.get(f, [f]))
    return out


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build libfluidsph.so")
    return cand


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _stale(lib: Path, srcs: list[Path]) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = srcs + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    deps.append(Path(__file__))
    return any(p.stat().st_mtime > t for p in deps)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link libfluidsph.so if any source is newer than it."""
    srcs = sources()
    if not force and not _stale(LIB_PATH, srcs):
        return LIB_PATH
    nvcc = _nvcc()
    BUILD_DIR.mkdir(parents=True, exist_ok=True)

    def compile_one(src: Path) -> Path:
        obj = BUILD_DIR / (src.name + ".o")
        cmd = [nvcc, *ARCH, *_flags_for(src), "-c", str(src), "-o", str(obj)]
        if src.suffix == ".cpp":
            cmd = [nvcc, *NVCC_FLAGS, "-x", "c++", "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
        return obj

    workers = min(len(srcs), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of libfluidsph.so failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True))
