"""Build recipe for the CUDA library (sm_103a) and its in-tree output.

Compiles every translation unit of ``csrc/`` with nvcc in parallel and links
``lib/libethersph_gpu.so``.  Per-unit flags:
  sph_fp64.cu  -fmad=false            (plain FP64 path: no a*b+c contraction)
  sph_probe.cu -fmad=false            (FP64 interpolation, same rounding as the oracle)
  sph_buffer.cu -fmad=false           (inlet/outlet moves and transfer decisions, as the oracle)
  sph_api.cu   -ffp-contract=off      (host constants round like the device code)
"""
from __future__ import annotations

import os
import sys

# Run as a script, this file's directory would come first on sys.path, and the package's
# types.py (the mirror of the reference's type tree) would shadow the standard library's
# `types` module for every import below: drop it.
if sys.path and os.path.abspath(sys.path[0] or ".") == os.path.dirname(os.path.abspath(__file__)):
    sys.path.pop(0)

import concurrent.futures as cf  # noqa: E402
import shutil  # noqa: E402
import subprocess  # noqa: E402
from pathlib import Path  # noqa: E402

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIB_DIR = PKG / "lib"
LIB = LIB_DIR / "libethersph_gpu.so"
BUILD = PKG / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-Xcompiler", "-Wall", "-I", str(PKG.parent / "include")]
UNIT_FLAGS = {
    "sph_fp64.cu": ["-fmad=false"],
    "sph_probe.cu": ["-fmad=false"],
    "sph_buffer.cu": ["-fmad=false"],
    "sph_api.cu": ["-Xcompiler", "-ffp-contract=off"],
}


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA library cannot be built")
    return exe


def _compile(src: Path, verbose: bool) -> Path:
    obj = BUILD / (src.stem + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *UNIT_FLAGS.get(src.name, []), "-c", str(src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False) -> Path:
    """Compile and link the library; returns the path of the shared object."""
    BUILD.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), sources))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
