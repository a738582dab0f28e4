"""Build the sm_103a shared library ``opencslsolver_gb300/_lib/libocsl_gb300.so``.

Plain nvcc, one -gencode, every translation unit compiled in parallel, then
linked with -shared.  Device code is compiled with --fmad=false: every fused
multiply-add in the kernels is an explicit fma(), mirroring the reference's
a*x + y expressions, so results are bit-reproducible against the CPU oracle.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libocsl_gb300.so")

SOURCES = ["kernels_krylov.cu", "kernels_ilu.cu", "kernels_box.cu", "kernels_wave.cu", "solver.cu",
           "pattern.cpp",
           "noalloc.cu", "adjoint.cu", "assembly.cu", "flow.cu", "batch.cpp", "mesh.cpp", "vtk.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _flags(src: str) -> list[str]:
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]
    # tuning overrides, e.g. OCSL_NVCC_DEFINES="-DOCSL_BOX_PF=16 -DOCSL_BOX_DF=2" (rebuild with -f)
    common += os.environ.get("OCSL_NVCC_DEFINES", "").split()
    if src.endswith(".cu"):
        return common + ARCH + ["-lineinfo", "--fmad=false", "-Xptxas", "-v"]
    return common


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "include", "ocsl.h"))
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    cc = nvcc()
    jobs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ_DIR, s + ".o")
        if force or _stale(obj, src):
            jobs.append((src, obj))

    def compile_one(job):
        src, obj = job
        cmd = [cc, *_flags(src), "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, r

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for src, r in ex.map(compile_one, jobs):
            if r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
                raise RuntimeError(f"nvcc failed on {os.path.basename(src)}")
            if verbose:
                sys.stderr.write(r.stderr)
    objs = [os.path.join(OBJ_DIR, s + ".o") for s in SOURCES]
    if jobs or not os.path.exists(LIB):
        cmd = [cc, "-shared", *ARCH, "--cudart=static", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
