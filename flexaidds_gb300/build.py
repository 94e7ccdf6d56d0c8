"""Builds the CUDA backend in-tree: flexaidds_gb300/libfxe.so (sm_103a)."""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfxe.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# (source, extra flags): the pose build and the clustering RMSDs are evaluated without fused
# multiply-adds, like the reference's single-precision arithmetic
UNITS = [("fxe_build.cu", ["--fmad=false"]), ("fxe_contacts.cu", []), ("fxe_thermo.cu", []), ("fxe_ga.cu", []),
         ("fxe_cluster.cu", ["--fmad=false"]), ("fxe_ensemble.cu", []), ("fxe_prepare.cu", ["--fmad=false"]),
         ("fxe_capi.cu", []),
         # the polyhedron kernel twice: single precision, and double precision with the
         # reference's expressions and every operation rounded separately
         ("fxe_voronoi.cu", ["-DFXE_REAL=float", "-DFXE_VARIANT=f32"], "fxe_voronoi_f32.o"),
         ("fxe_voronoi.cu", ["-DFXE_REAL=double", "-DFXE_VARIANT=f64", "-DFXE_REFERENCE_FORMULAS=1",
                             "--fmad=false"], "fxe_voronoi_f64.o")]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise FileNotFoundError("nvcc not found")
    return p


def _compile(unit):
    src, extra = unit[0], unit[1]
    obj = os.path.join(BUILD, unit[2] if len(unit) > 2 else src.replace(".cu", ".o"))
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xptxas", "-v" if os.environ.get("FXE_PTXAS_VERBOSE") else "-O3", *extra,
           "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        res = list(ex.map(_compile, UNITS))
    if verbose:
        for _, log in res:
            sys.stderr.write(log)
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *[o for o, _ in res], "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
