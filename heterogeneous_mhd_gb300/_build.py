"""Build of libmhd_gb300.so (the C ABI + sm_103a kernels), in tree.

nvcc compiles the kernel sets for sm_103a only:
  * kernels_fast.cu  - FP32 with FMA contraction (production path);
  * kernels_exact.cu - FP32/FP64 with --fmad=false, bit-identical to the
    reference's C arithmetic;
  * mhd_abi.cu       - host code of the C ABI (single box);
  * mhd_batch.cu     - host code of the batched-box API;
  * mhd_noalloc.cu   - the allocation-free calcfl;
  * closure.cu       - the learned closure (BF16 tensor-core convolutions,
    loss, optimiser, filter and correction kernels);
and gcc compiles the seeded initial conditions (mhd_init.c) with
-ffp-contract=off so they are identical on x86-64 and aarch64, and the
file formats (mhd_io.c).  The
translation units build in parallel; the result is
heterogeneous_mhd_gb300/lib/libmhd_gb300.so.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
OBJDIR = PKG / "lib" / "_obj"
LIBNAME = "libmhd_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                      "-Xcompiler", "-fvisibility=hidden", "-I", str(ROOT / "include")]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmhd_gb300")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        sys.stderr.write(res.stdout + res.stderr)
        raise RuntimeError(f"build step failed: {' '.join(cmd[:3])} ... {cmd[-1]}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def lib_path() -> Path:
    return LIBDIR / LIBNAME


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every translation unit that changed and link the library."""
    nvcc = _nvcc()
    OBJDIR.mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted((ROOT / "include").glob("*.h"))
    units = [
        ("kernels_fast.cu", [nvcc, *NVCC_COMMON, "-Xptxas", "-v"] if verbose else [nvcc, *NVCC_COMMON]),
        ("kernels_exact.cu", [nvcc, *NVCC_COMMON, "--fmad=false", "-prec-div=true", "-prec-sqrt=true"]),
        ("mhd_abi.cu", [nvcc, *NVCC_COMMON]),
        ("mhd_noalloc.cu", [nvcc, *NVCC_COMMON]),
        ("mhd_batch.cu", [nvcc, *NVCC_COMMON]),
        ("closure.cu", [nvcc, *NVCC_COMMON]),
    ]
    jobs = []
    for src, base in units:
        obj = OBJDIR / (src + ".o")
        if force or _stale(obj, [CSRC / src, *headers]):
            jobs.append(base + ["-c", str(CSRC / src), "-o", str(obj)])
    c_objs = []
    for csrc in ("mhd_init.c", "mhd_io.c"):  # host C: initial conditions, file formats
        obj = OBJDIR / (csrc + ".o")
        c_objs.append(obj)
        if force or _stale(obj, [CSRC / csrc, *sorted((ROOT / "include").glob("*.h"))]):
            jobs.append(["gcc", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
                         "-fvisibility=hidden", "-I", str(ROOT / "include"), "-c", str(CSRC / csrc),
                         "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(4, min(8, os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    objs = [OBJDIR / (u[0] + ".o") for u in units] + c_objs
    lib = lib_path()
    if force or jobs or _stale(lib, objs):
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-Xcompiler", "-fopenmp",
              *[str(o) for o in objs], "-o", str(lib), "-lgomp"])
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
