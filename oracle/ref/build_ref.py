"""Recipe: compile the reference's own hot-path sources into oracle/_ref/.

TEST INFRASTRUCTURE ONLY.  Two stages:

1. ``slice`` (needs the reference checkout, named by the environment
   variable TW_REFERENCE_ROOT; nothing is sliced when it is unset): copies
   the exact line ranges listed in SLICES, and the whole files listed in
   COPIES, into oracle/_ref/src/.  Each slice is checked against the first
   line it must start with, so a moved line range fails loudly instead of
   compiling the wrong code.  oracle/_ref/ is git-ignored:
   nothing from the reference is committed.
2. ``compile`` (needs only oracle/_ref/src): builds oracle/_ref/libtwref.so
   from those files, the geogram shim (oracle/ref/shim) and the oracle C code,
   with FP contraction off (the reference's default x86-64 scalar build has
   no fused multiply-add).

Usage: python oracle/ref/build_ref.py [slice|compile|all]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref"
SRC = OUT / "src"

# (reference file, first line, last line, output name, expected start of first line)
SLICES = [
    ("src/tetwild/LocalOperations.cpp", 28, 291, "amips_slice.inc",
     "double LocalOperations::comformalAMIPSEnergy_new"),
    ("src/tetwild/LocalOperations.cpp", 1034, 1109, "envelope_slice.inc",
     "bool LocalOperations::isPointOutEnvelop"),
    ("src/tetwild/Common.cpp", 143, 255, "sample_slice.inc",
     "void sampleTriangle("),
    ("src/tetwild/LocalOperations.cpp", 605, 693, "sweeps_slice.inc",
     "void LocalOperations::getAvgMaxEnergy"),
]
COPIES = [
    ("src/tetwild/geogram/mesh_AABB.cpp", "mesh_AABB.cpp"),
    ("src/tetwild/geogram/mesh_AABB.h", "tetwild/geogram/mesh_AABB.h"),
    ("src/tetwild/DistanceQuery.h", "tetwild/DistanceQuery.h"),
]


def reference_root() -> Path | None:
    root = os.environ.get("TW_REFERENCE_ROOT")
    return Path(root) if root else None


def do_slice() -> bool:
    root = reference_root()
    if root is None or not (root / "src/tetwild/LocalOperations.cpp").is_file():
        return False
    SRC.mkdir(parents=True, exist_ok=True)
    for rel, lo, hi, name, head in SLICES:
        lines = (root / rel).read_text().splitlines(keepends=True)
        chunk = lines[lo - 1:hi]
        if not chunk or not chunk[0].startswith(head):
            raise RuntimeError(f"{rel}:{lo} does not start with {head!r}")
        if chunk[-1].strip() != "}":
            raise RuntimeError(f"{rel}:{hi} is not the closing brace of the slice")
        (SRC / name).write_text(f"// sliced from {rel}:{lo}-{hi}\n" + "".join(chunk))
    for rel, name in COPIES:
        dst = SRC / name
        dst.parent.mkdir(parents=True, exist_ok=True)
        shutil.copyfile(root / rel, dst)
    return True


def do_compile() -> Path | None:
    if not all((SRC / name).is_file() for _, _, _, name, _ in SLICES):
        return None
    OUT.mkdir(parents=True, exist_ok=True)
    obj = OUT / "tw_oracle_ref.o"
    so = OUT / "libtwref.so"
    cflags = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]
    subprocess.run(["gcc", "-std=c99", *cflags, "-c", str(ORACLE / "tw_oracle.c"), "-o", str(obj)],
                   check=True)
    subprocess.run(
        ["g++", "-std=c++17", *cflags, "-w", "-shared", "-o", str(so),
         f"-I{HERE / 'shim'}", f"-I{SRC}", f"-I{ORACLE}",
         str(HERE / "ref_api.cpp"), str(SRC / "mesh_AABB.cpp"), str(obj), "-lpthread", "-lm"],
        check=True)
    return so


def main(argv: list[str]) -> int:
    what = argv[1] if len(argv) > 1 else "all"
    if what in ("slice", "all"):
        if not do_slice() and what == "slice":
            print("reference checkout not found (TW_REFERENCE_ROOT); nothing sliced", file=sys.stderr)
            return 1
    if what in ("compile", "all"):
        so = do_compile()
        if so is None:
            print("oracle/_ref/src missing; nothing compiled", file=sys.stderr)
            return 1
        print(so)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
