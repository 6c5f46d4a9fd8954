"""Builds the in-tree CUDA library ``_build/libccs_gpu.so`` for sm_103a.

Every translation unit is compiled in parallel with nvcc and linked into one
shared library with the CUDA runtime linked statically.  Host code is compiled
with ``-ffp-contract=off``: the FP64 set-up arithmetic (metric products, halo
transforms) must not be fused on aarch64 hosts, where gcc contracts by default.
The FP64 parity kernels are compiled with ``-fmad=false`` for the same reason, and
so is the mixed lane, whose FMAs are all written out: the tile-shape variants of its
stage kernel then round identically.
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
LIB = BUILD / "libccs_gpu.so"
DRIVER = BUILD / "ccsm_gpu"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

# (source, extra flags)
UNITS = [
    ("ccs_fp64.cu", ["-fmad=false"]),
    ("ccs_mixed.cu", ["-fmad=false"]),  # FMAs explicit: every tile variant rounds alike
    ("ccs_api.cu", []),
    ("ccs_host.cpp", []),
    ("ccs_noalloc.cu", []),
]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA library cannot be built")
    return cand


def _common(nvcc: str) -> list[str]:
    # CCS_BUILD_FLAGS: extra nvcc flags (tuning macros such as -DCCS_MIXED_MIN_CTAS=3)
    extra = os.environ.get("CCS_BUILD_FLAGS", "").split()
    return [nvcc] + extra + [
        ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", f"-I{CSRC}", f"-I{PKG.parent / 'include'}",
    ]


def _deps() -> list[Path]:
    return ([CSRC / s for s, _ in UNITS] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) +
            [CSRC / "ccsm_gpu.cpp", PKG.parent / "include" / "ccs_gpu.h", Path(__file__)])


def _fresh(lib: Path) -> bool:
    if not lib.exists():
        return False
    t = lib.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in _deps())


def _build_lib(out_dir: Path, defines: list[str], verbose: bool) -> Path:
    """Compiles every translation unit in parallel with `defines` and links
    out_dir/libccs_gpu.so (CUDA runtime linked statically)."""
    out_dir.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    common = _common(nvcc) + defines

    def compile_one(unit):
        src, extra = unit
        obj = out_dir / (Path(src).stem + ".o")
        cmd = common + extra + ["-c", str(CSRC / src), "-o", str(obj)]
        if src.endswith(".cpp"):
            cmd = common + extra + ["-x", "c++", "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, UNITS))
    lib = out_dir / "libccs_gpu.so"
    tmp = out_dir / "libccs_gpu.so.tmp"
    cmd = [nvcc, ARCH, "-shared", "-cudart", "static", "-o", str(tmp)] + [str(o) for o in objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile and link; returns the library path.  Skips work when up to date."""
    if not force and _fresh(LIB):
        return LIB
    _build_lib(BUILD, [], verbose)
    # the model program over the C ABI (a C++ host driver linked against the library)
    nvcc = _nvcc()
    cmd = [nvcc, "-O2", "-std=c++17", "-x", "c++", "-Xcompiler", "-ffp-contract=off", f"-I{PKG.parent / 'include'}",
           str(CSRC / "ccsm_gpu.cpp"), f"-L{BUILD}", "-lccs_gpu", "-Xlinker", "-rpath,$ORIGIN", "-o", str(DRIVER)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


BOUNDS_LIB = BUILD / "bounds" / "libccs_gpu.so"


def build_bounds(verbose: bool = False, force: bool = False) -> Path:
    """The bounds-checked library (-DCCS_BOUNDS): every kernel checks the indices of
    its array accesses and skips an out-of-range one, recording it for
    ccs_debug_bounds.  Same ABI, slower; not part of build().  Select it for a
    process with CCS_GPU_LIB=<returned path>."""
    if not force and _fresh(BOUNDS_LIB):
        return BOUNDS_LIB
    return _build_lib(BOUNDS_LIB.parent, ["-DCCS_BOUNDS"], verbose)


if __name__ == "__main__":
    if "--bounds" in sys.argv:
        print(build_bounds(verbose=True, force="--force" in sys.argv))
    else:
        print(build(verbose=True, force="--force" in sys.argv))
