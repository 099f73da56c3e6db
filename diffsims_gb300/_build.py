"""Build libdiffsims_gb300.so (sm_103a) in-tree with nvcc.

Each translation unit under ``csrc/`` compiles to an object in parallel, then
one link step writes ``diffsims_gb300/libdiffsims_gb300.so``.  No cmake, no
torch extension machinery: the library is a plain C-ABI shared object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

PKG = pathlib.Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = PKG / "libdiffsims_gb300.so"
LIB_DEBUG = PKG / "libdiffsims_gb300_debug.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build diffsims_gb300")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                   "-I", str(INCLUDE), "--expt-relaxed-constexpr", *extra]


def build(verbose: bool = False, ptxas_verbose: bool = False, force: bool = False,
          debug: bool = False) -> pathlib.Path:
    """Compile csrc/*.cu and link the library; ``debug`` builds the
    bounds-checked variant (-DDS_DEBUG_BOUNDS) as libdiffsims_gb300_debug.so."""
    lib = LIB_DEBUG if debug else LIB
    objdir = BUILD / "debug" if debug else BUILD
    sources = sorted(CSRC.glob("*.cu"))
    deps = sources + sorted(CSRC.glob("*.cuh")) + [INCLUDE / "diffsims_gb300.h", pathlib.Path(__file__)]
    if not force and lib.exists() and lib.stat().st_mtime > max(p.stat().st_mtime for p in deps):
        return lib
    objdir.mkdir(parents=True, exist_ok=True)
    nvcc = nvcc_path()
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []
    if debug:
        extra.append("-DDS_DEBUG_BOUNDS")

    def compile_one(src: pathlib.Path):
        obj = objdir / (src.stem + ".o")
        cmd = [nvcc, *_flags(extra), "-c", str(src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stderr}")
        return obj, res.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, len(sources))) as ex:
        results = list(ex.map(compile_one, sources))
    if verbose or ptxas_verbose:
        for obj, log in results:
            if log.strip():
                print(f"--- {obj.name}\n{log}", file=sys.stderr)
    tmp = lib.with_suffix(".so.tmp")
    # the CUDA runtime is linked statically (nvcc's default): no libcudart.so
    # lookup at load time, on either machine
    cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *[str(o) for o, _ in results]]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose=True, ptxas_verbose="-v" in sys.argv, force="-f" in sys.argv, debug="--debug" in sys.argv))
