"""Builds libopensps_gb300.so (the C-ABI library with its sm_103a kernels) in-tree with nvcc.

The translation units compile in parallel, one -gencode (sm_103a), then link into one shared library under
``libopensps_gb300/_lib``. No CMake and no torch extension machinery: the product is a plain C-ABI ``.so`` that C,
Fortran and ctypes callers load directly.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_lib"
LIB = OUT / "libopensps_gb300.so"
SOURCES = ["capi.cu", "context.cu", "batch.cu", "csp_contract.cu", "csp_aux.cu", "band_gemm.cu", "gemm_bf16x3.cu",
           "adjoint.cu", "noalloc.cu", "sfh.cu", "ssp_op.cu", "fp64_path.cu", "emulator.cu",
           "emulator_train.cu", "datalib.cu", "dust_curves.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_LIB = "/usr/local/cuda/lib64"   # cuBLAS (the plain FP64 path's DGEMM)


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((HERE.parent / "include").glob("*.h"))
    return any(d.stat().st_mtime > obj.stat().st_mtime for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    objdir = OUT / "obj"
    objdir.mkdir(exist_ok=True)
    cc = nvcc()
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3,-fopenmp", "--expt-relaxed-constexpr",
                    "-I", str(CSRC), "-I", str(HERE.parent / "include")]
    if verbose:
        flags += ["-Xptxas", "-v"]

    def compile_one(src: str) -> tuple[str, Path]:
        s = CSRC / src
        o = objdir / (Path(src).stem + ".o")
        if force or _stale(o, s):
            cmd = [cc, "-c", str(s), "-o", str(o)] + flags
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
            if verbose and r.stderr:
                sys.stderr.write(r.stderr)
        return src, o

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = [o for _, o in ex.map(compile_one, SOURCES)]
    if force or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [cc, "-shared", "-o", str(tmp)] + [str(o) for o in objs] + ARCH + [
            "-lcudart_static", "-lrt", "-lpthread", "-ldl", "-lcublas", "-lgomp", "-Xlinker", "-rpath=" + CUDA_LIB]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
