"""The binary dump reader (nuclearmpm_gb300.dumpio) on a synthetic dump written here: the
header, record layout, the per-particle timestep and lame columns of the reference's text
dump (src/solver.cpp:75-104), and the reference's stride-res grid indexing
(src/solver.cpp:117) under reference_grid_layout."""
import struct

import numpy as np
import pytest

from nuclearmpm_gb300 import dumpio


def write_dump(path, dim, res, n, steps, seed=0, truncate=0):
    rng = np.random.default_rng(seed)
    N = res + 1
    nodes = N ** dim
    recs = []
    with open(path, "wb") as f:
        f.write(struct.pack("<8s4Iq4f", b"NCLRDMP1", dim, res, 0, 0, n, 1e-4, 2.5, 3.5, 10.0))
        for s in range(steps):
            r = {"x": rng.random((n, dim)), "v": rng.random((n, dim)), "F": rng.random((n, dim, dim)),
                 "C": rng.random((n, dim, dim)), "Jp": rng.random(n), "velocity": rng.random((nodes, dim)),
                 "mass": rng.random(nodes)}
            r = {k: v.astype(np.float32) for k, v in r.items()}
            ts = np.float32(1e-4) * np.float32(s) if s > 0 else np.float32(1e-4)
            f.write(struct.pack("<qff", s, ts, 0.0))
            for k in ("x", "v", "F", "C", "Jp", "velocity", "mass"):
                f.write(r[k].tobytes())
            recs.append((ts, r))
        if truncate:
            f.write(b"\0" * truncate)  # a partial record (a dump cut short) is ignored
    return recs


@pytest.mark.parametrize("dim", [2, 3])
def test_load_returns_every_record_in_the_reference_structure(tmp_path, dim):
    p = tmp_path / "dump.nclr"
    recs = write_dump(p, dim, 6, 40, 3, truncate=100)
    h = dumpio.read_header(str(p))
    assert (h["dim"], h["res"], h["n"]) == (dim, 6, 40)
    out = dumpio.load(str(p))
    assert sorted(out) == ["0_", "1_", "2_"]
    for s, (ts, r) in enumerate(recs):
        got = out[f"{s}_"]
        for k in ("x", "v", "F", "C", "Jp"):
            assert got.__dict__[k].dtype == np.float64
            assert np.array_equal(got.__dict__[k], r[k].astype(np.float64)), k
        assert got.velocity.shape == (7,) * dim + (dim,)
        assert np.array_equal(got.velocity.reshape(-1, dim), r["velocity"])
        assert np.array_equal(got.mass.reshape(-1), r["mass"])
        assert np.array_equal(got.timestep, np.full(40, ts, np.float32))
        assert np.array_equal(got.lame, np.tile(np.float32([25.0, 35.0]), (40, 1)))


def test_reference_grid_layout_reads_stride_res(tmp_path):
    p = tmp_path / "dump.nclr"
    res = 5
    recs = write_dump(p, 2, res, 3, 1)
    got = dumpio.load(str(p), reference_grid_layout=True)["0_"]
    mass = recs[0][1]["mass"]
    for ii in range(res + 1):
        for jj in range(res + 1):
            assert got.mass[ii, jj] == mass[ii * res + jj]


def test_rejects_other_files(tmp_path):
    p = tmp_path / "x.bin"
    p.write_bytes(b"not a dump" * 10)
    with pytest.raises(ValueError):
        dumpio.load(str(p))
