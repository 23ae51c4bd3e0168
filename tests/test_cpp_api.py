"""The drop-in C++ header (include/nclr.h): compiles and links against libnclr_gpu.so here;
on a GPU its example program runs the README snow scene and matches the CPU oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import field_err

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "nuclearmpm_gb300", "_build")
SRC = os.path.join(ROOT, "tests", "cpp", "nclr_api_check.cpp")


def compile_check(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "nclr_api_check")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-L", LIBDIR, "-lnclr_gpu", f"-Wl,-rpath,{LIBDIR}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_header_compiles_and_links(tmp_path):
    compile_check(tmp_path)


@pytest.mark.gpu
def test_header_example_matches_oracle(tmp_path, oracle):
    exe = compile_check(tmp_path)
    out = str(tmp_path / "state.bin")
    r = subprocess.run([exe, out, "1"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    rec = 2 + 2 + 4 + 4 + 1
    data = np.fromfile(out, dtype=np.float32).reshape(2, 5000, rec)

    def unpack(a):
        return {"x": a[:, 0:2], "v": a[:, 2:4], "F": a[:, 4:8].reshape(-1, 2, 2),
                "C": a[:, 8:12].reshape(-1, 2, 2), "Jp": a[:, 12]}

    init, final = unpack(data[0]), unpack(data[1])
    init["mass"] = np.ones(5000, np.float32)
    init["volume"] = np.ones(5000, np.float32)
    ref, _, st, _ = oracle.advance(init, dim=2, model=0, res=64, steps=1)
    assert st == 0
    for f in ("x", "v", "F", "C", "Jp"):
        assert field_err(final[f], ref[f], f) <= 1e-5, f
    # the extensions: neo-Hookean stress, one E / nu per particle
    raw = np.fromfile(out + ".ext", dtype=np.float32)
    states = raw[:2 * 5000 * rec].reshape(2, 5000, rec)
    E, nu = raw[2 * 5000 * rec:].reshape(2, 5000)
    init, final = unpack(states[0]), unpack(states[1])
    init["mass"] = np.ones(5000, np.float32)
    init["volume"] = np.ones(5000, np.float32)
    ref, _, st, _ = oracle.advance(init, dim=2, model=0, res=64, steps=1, stress=1,
                                   E_particles=E, nu_particles=nu)
    assert st == 0
    for f in ("x", "v", "F", "C", "Jp"):
        assert field_err(final[f], ref[f], f) <= 1e-5, f
