"""Build libnpbmz_gpu.so (sm_103a) in-tree with nvcc.

The translation units compile in parallel:
  common_kernels.cu  -fmad=false  set-up, exch_qbc, norms, layout conversion
  step_exact.cu      -fmad=false  FP64 step kernels in the reference's order
  step_fast.cu       -fmad=true   FP64 (FMA) and FP32 line-solve kernels
  npbmz_api.cu                    the C ABI (include/npbmz.h)
  noalloc.cu         -fmad=true   the x sweep over a file-scope device array
  adjoint.cu         -fmad=true   the discrete adjoint of the BT and SP steps
  lu.cu                           the C ABI of LU-MZ's SSOR iteration (include/npbmz_lu.h)
  lu_exact.cu        -fmad=false  its kernels (lu_kernels.cuh) with the reference's rounding
  lu_fast.cu         -fmad=true   the same kernels with FMA contraction (NPBMZ_LU_FMA)
and are linked into npbapps.jl_gb300/npbmz/_build/libnpbmz_gpu.so.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG.parent / "csrc"
INCLUDE = PKG.parent.parent / "include"
OUT = PKG / "_build"
LIB = OUT / "libnpbmz_gpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(CSRC), "-I", str(INCLUDE)]
UNITS = {
    "common_kernels.cu": ["-fmad=false"],
    "step_exact.cu": ["-fmad=false"],
    "step_fast.cu": ["-fmad=true"],
    "npbmz_api.cu": [],
    "noalloc.cu": ["-fmad=true"],
    "adjoint.cu": ["-fmad=true"],
    "lu.cu": [],
    "lu_exact.cu": ["-fmad=false"],
    "lu_fast.cu": ["-fmad=true"],
}


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found")
    return exe


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def up_to_date():
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _sources())


def build(force=False, verbose=False, ptxas_info=False):
    """Compile and link; returns the path of the shared library."""
    if not force and up_to_date():
        return LIB
    OUT.mkdir(parents=True, exist_ok=True)
    cc = nvcc()

    def compile_unit(item):
        name, flags = item
        obj = OUT / (Path(name).stem + ".o")
        cmd = [cc, *ARCH, *COMMON, *flags, "-c", str(CSRC / name), "-o", str(obj)]
        if ptxas_info:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(compile_unit, UNITS.items()))
    if verbose or ptxas_info:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    tmp = OUT / (LIB.name + ".tmp")
    cmd = [cc, *ARCH, "-shared", "-cudart", "shared", "-o", str(tmp), *[str(o) for o, _ in results]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
