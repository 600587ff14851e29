"""Build recipe for libsmg_gpu.so (sm_103a) — the CUDA kernels and the C ABI.

Every translation unit under csrc/ is compiled in parallel with nvcc for
sm_103a only and linked in-tree into schwinger_mg_gb300/libsmg_gpu.so.
Nothing is installed into site-packages.  Re-running is incremental: an
object is rebuilt when its source or any csrc/ header is newer.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libsmg_gpu.so"
KTRACE_SRC = PKG / "profiling" / "kernel_trace.cpp"
KTRACE_LIB = PKG / "libsmg_ktrace.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-Xptxas", "-O3"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsmg_gpu.so")
    return cand


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _compile(src: Path, hdr_mtime: float, verbose: bool, extra: list[str]) -> Path:
    obj = BUILD / (src.name + ".o")
    if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, hdr_mtime):
        return obj
    if src.suffix == ".cu":
        cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", *CXX_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {src.name} failed:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, file=sys.stderr)
    return obj


def build_library(verbose: bool = False, ptxas_verbose: bool = False) -> Path:
    """Compiles csrc/*.cu and csrc/*.cpp and links libsmg_gpu.so in-tree."""
    BUILD.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    hdr = _headers_mtime()
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []
    jobs = max(1, min(len(srcs), os.cpu_count() or 4))
    with ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, hdr, verbose, extra), srcs))
    newest = max(o.stat().st_mtime for o in objs)
    if LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-lrt", "-lpthread",
           "-ldl"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"linking libsmg_gpu.so failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def _cuda_root() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def build_kernel_trace(verbose: bool = False) -> Path | None:
    """The optional CUPTI kernel tracer (libsmg_ktrace.so) used by the benchmark's
    --kernel-trace; returns None when CUPTI is not available."""
    if KTRACE_LIB.exists() and KTRACE_LIB.stat().st_mtime >= KTRACE_SRC.stat().st_mtime:
        return KTRACE_LIB
    root = _cuda_root()
    incs = [root / "include", *root.glob("targets/*/include"), root / "extras" / "CUPTI" / "include"]
    libs = [root / "lib64", *root.glob("targets/*/lib"), root / "extras" / "CUPTI" / "lib64"]
    if not any((i / "cupti.h").exists() for i in incs):
        return None
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", *[f"-I{i}" for i in incs if i.exists()], str(KTRACE_SRC),
           *[f"-L{d}" for d in libs if d.exists()], "-lcupti", "-o", str(KTRACE_LIB)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        print(f"kernel tracer not built (CUPTI): {r.stderr.strip()[:200]}", file=sys.stderr)
        return None
    return KTRACE_LIB


if __name__ == "__main__":
    p = build_library(verbose=True, ptxas_verbose="-v" in sys.argv)
    print(p)
    print(build_kernel_trace(verbose=True))
