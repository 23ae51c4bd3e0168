"""Builds libnclr_gpu.so (the C ABI of include/nclr_gpu.h) for sm_103a with nvcc.

Each translation unit is compiled in parallel, then linked into
nuclearmpm_gb300/_build/libnclr_gpu.so (git-ignored; rebuilt on every machine, since the
library is architecture-specific host code plus sm_103a device code); the headless solver
nuclearmpm_gb300/_build/nclr_solver is linked against it.

    python -m nuclearmpm_gb300.build [-v]
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
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libnclr_gpu.so")
SOLVER = os.path.join(OUT_DIR, "nclr_solver")  # the headless solver (cli/nclr_solver.cpp)
SOURCES = ["nclr_gpu.cu", "step2d.cu", "step3d.cu", "step3d_mat.cu", "scan.cu", "noalloc.cu",
           "adjoint.cu", "scene_build.cu", "render.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.isfile(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnclr_gpu.so")


def flags(extra: list[str] | None = None) -> list[str]:
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                   "-I", os.path.join(ROOT, "include"), "-I", CSRC] + (extra or [])


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    objs = [os.path.join(OUT_DIR, os.path.splitext(s)[0] + ".o") for s in SOURCES]

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)

    cmds = [[cc] + flags(extra) + ["-c", os.path.join(CSRC, s), "-o", o]
            for s, o in zip(SOURCES, objs)]
    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        list(ex.map(run, cmds))
    tmp = LIB + ".tmp"
    run([cc] + ARCH + ["-shared", "-o", tmp] + objs)
    os.replace(tmp, LIB)
    # the headless solver (cli/nclr_solver.cpp), linked against the library next to it
    run([cc, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
         os.path.join(HERE, "cli", "nclr_solver.cpp"), "-o", SOLVER, "-L", OUT_DIR, "-lnclr_gpu",
         "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"])
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    extra = [a for a in sys.argv[1:] if a != "-v"]
    print(build(verbose=v, extra=extra))
