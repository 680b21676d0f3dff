"""Build libtw_gb300.so (the CUDA kernels + C-ABI) in-tree for sm_103a.

Each .cu file is compiled to an object in parallel, then nvcc links the
shared library next to this file.  All units use -fmad=false: the FP64
arithmetic must round exactly as written so that decisions are bit-identical
to the CPU oracle (explicit fma() calls are still emitted as FMA).
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
ROOT = PKG.parent
BUILD = PKG / "_build"
LIB = PKG / "libtw_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
    "-Xcompiler", "-fvisibility=hidden", f"-I{ROOT / 'include'}", f"-I{CSRC}",
    "--expt-relaxed-constexpr",
]
SOURCES = ["tw_amips.cu", "tw_lbvh.cu", "tw_envelope.cu", "tw_newton.cu", "tw_capi.cu",
           "tw_noalloc.cu", "tw_server.cu", "tw_swap.cu",
           "tw_schedule.cu"]


def nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = Path(cuda) / "bin" / "nvcc"
    return str(cand) if cand.exists() else (shutil.which("nvcc") or "nvcc")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, extra: list[str] | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [ROOT / "include" / "tw_gb300.h"]
    flags = NVCC_FLAGS + (extra or [])

    def compile_one(src: str) -> Path:
        s = CSRC / src
        o = BUILD / (src + ".o")
        if force or _stale(o, [s, *headers, Path(__file__)]):
            cmd = [nvcc(), *ARCH, *flags, "-c", str(s), "-o", str(o)]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
            if verbose and r.stderr:
                print(r.stderr, flush=True)
        return o

    with ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    extra = [a for a in sys.argv[1:] if a.startswith("-X") or a.startswith("--")]
    print(build(verbose=v, force="-f" in sys.argv, extra=extra))
