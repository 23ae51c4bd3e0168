"""Build recipe for the CPU oracle (test infrastructure only).

Outputs (all git-ignored, rebuilt on each machine):
  oracle/_build/liboracle.so       the restatement, strict IEEE (-O2 -ffp-contract=off): the
                                   parity checker;
  oracle/_build/liboracle_fast.so  the same source built like the reference build
                                   (-Ofast, CMakeLists.txt:9-10): the timed CPU baseline;
  oracle/_ref/libnclr_ref.so       the reference's own src/nclr.h + src/nclr_math.h compiled
                                   in place against the Eigen-API shim in oracle/ref_shim/;
                                   only built where the reference tree exists.

The reference's src/ directory is taken from the environment variable NCLR_REFERENCE_SRC;
without it, from the read-only checkout this recipe was written against.  A missing tree
only skips the third library.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_SRC = os.environ.get("NCLR_REFERENCE_SRC") or "/root/reference/src"


def _cmds():
    cxx = os.environ.get("CXX", "g++")
    common = [cxx, "-std=c++17", "-fPIC", "-shared", "-w", "-pthread"]
    src = os.path.join(HERE, "oracle_capi.cpp")
    out = [
        (common + ["-O2", "-ffp-contract=off", src, "-o",
                   os.path.join(HERE, "_build", "liboracle.so")]),
        (common + ["-Ofast", src, "-o", os.path.join(HERE, "_build", "liboracle_fast.so")]),
    ]
    if os.path.isfile(os.path.join(REFERENCE_SRC, "nclr.h")):
        out.append(common + ["-O2", "-ffp-contract=off", "-I", os.path.join(HERE, "ref_shim"),
                             "-I", REFERENCE_SRC, os.path.join(HERE, "ref_capi.cpp"), "-o",
                             os.path.join(HERE, "_ref", "libnclr_ref.so")])
    return out


def build(verbose: bool = False) -> None:
    os.makedirs(os.path.join(HERE, "_build"), exist_ok=True)
    os.makedirs(os.path.join(HERE, "_ref"), exist_ok=True)
    cmds = _cmds()

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr}")

    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        list(ex.map(run, cmds))


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
