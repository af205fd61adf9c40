"""Build librett.so in-tree with nvcc for sm_103a.

Translation units compile in parallel into librett_gb300/_build/ and link
into librett_gb300/librett.so (static CUDA runtime).  A unit is rebuilt
only when it or any header under csrc/ or include/ is newer than its object.

Usage: python -m librett_gb300.build [--force] [--verbose]
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "librett.so"

SOURCES = ["api.cpp", "plan.cpp", "select.cpp", "k_misc.cu", "k_tile4.cu", "k_tile8.cu",
           "k_tile16.cu", "k_group4.cu", "k_group4h.cu", "k_group8.cu", "k_group16.cu",
           "noalloc.cu", "mlp.cu", "group.cu", "verify.cu"]
# flat and bulk-copy tile kernels: three units per element size, by tile rank count
SOURCES += [f"k_flat{es}_{g}.cu" for es in (4, 8, 16) for g in "abc"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          f"-I{INCLUDE}", f"-I{CSRC}"]
# Host inference of the plan selector: let the compiler fuse its vector
# multiply-adds (ISO C++ mode turns contraction off; on Arm hosts this halves
# the instructions of the network's dense layers).
FILE_FLAGS = {"select.cpp": ["-Xcompiler", "-ffp-contract=fast"]}


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librett.so")
    return exe


def _headers_mtime() -> float:
    files = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.inc"))
    files += list(INCLUDE.glob("*.h"))
    return max((f.stat().st_mtime for f in files), default=0.0)


def _compile(src: str, force: bool, verbose: bool, extra: list[str]) -> Path:
    srcp = CSRC / src
    obj = BUILD / (src + ".o")
    if (not force and obj.exists()
            and obj.stat().st_mtime >= max(srcp.stat().st_mtime, _headers_mtime())):
        return obj
    cmd = [nvcc(), *ARCH, *COMMON, *FILE_FLAGS.get(src, []), *extra, "-c", str(srcp), "-o",
           str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{res.stdout}\n{res.stderr}")
    if verbose and (res.stdout or res.stderr):
        print(res.stdout, res.stderr, flush=True)
    return obj


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> Path:
    """Compile every translation unit for sm_103a and link librett.so.

    LIBRETT_NVCC_FLAGS (environment) appends flags to every compile, e.g.
    -DLT_FLAT_ASYNC_MIN_NL=32 to keep every flat tile kernel on register
    loads; use --force after changing it."""
    BUILD.mkdir(parents=True, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []
    extra += os.environ.get("LIBRETT_NVCC_FLAGS", "").split()
    workers = min(len(SOURCES), max(1, os.cpu_count() or 1))
    with ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, verbose, extra), SOURCES))
    newest = max(o.stat().st_mtime for o in objs)
    if force or not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    return LIB


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas-verbose", action="store_true",
                    help="print per-kernel registers / spills / smem")
    args = ap.parse_args(argv)
    lib = build(force=args.force, verbose=args.verbose or args.ptxas_verbose,
                ptxas_verbose=args.ptxas_verbose)
    print(lib)
    return 0


if __name__ == "__main__":
    sys.exit(main())
