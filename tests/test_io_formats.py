"""Statistics and file formats against the reference's own output
(tests/golden/io_tiny7.npz, written by src/statistics.cpp and src/io.cpp
through oracle/ref_harness.cpp): the oracle's statistics restatement and the
library's host-side writers and reader, byte for byte.  No GPU."""
import os

import numpy as np
import pytest

import les_gb300 as G

GOLD = os.path.join(os.path.dirname(__file__), "golden", "io_tiny7.npz")
KEYS = ("u", "v", "w", "p", "uu", "vv", "ww", "uv", "uw", "vw")


@pytest.fixture(scope="module")
def gd():
    return np.load(GOLD)


def _mesh(gd):
    nx, ny, nz, dx, dy, dz = gd["mesh"]
    return G.Mesh(int(nx), int(ny), int(nz), float(dx), float(dy), float(dz))


def _lib_or_skip():
    try:
        return G.load()
    except FileNotFoundError:
        pytest.skip("libles_gb300.so not built")


def test_oracle_statistics_sums_match_reference(oracle_lib, gd):
    n = gd["stats_in0_u"].size
    sums = [np.zeros(n) for _ in range(10)]
    samples = 0
    for s in range(3):
        if s <= 0:   # start_step 0: the reference skips step 0 (src/statistics.cpp:101-103)
            continue
        samples += 1
        oracle_lib.stats_update(*[gd["stats_in%d_%s" % (s, k)] for k in ("u", "v", "w", "p")], sums)
    assert samples == int(gd["stats_samples"][0])
    for q, k in enumerate(KEYS):
        assert np.array_equal(sums[q], gd["stats_sum_" + k]), k


def test_statistics_file_matches_reference(oracle_lib, gd, tmp_path):
    _lib_or_skip()
    sums = [gd["stats_sum_" + k].copy() for k in KEYS]
    out = oracle_lib.stats_finalize(int(gd["stats_samples"][0]), sums)
    path = tmp_path / "stats.vtk"
    G.format_stats_vtk(_mesh(gd), out[:4], out[4:], path)
    assert path.read_bytes() == bytes(gd["stats_vtk"])


def test_field_file_matches_reference(gd, tmp_path):
    _lib_or_skip()
    f = {k: gd["io_" + k] for k in ("u", "v", "w", "p", "nu_t")}
    path = tmp_path / "out.vtk"
    G.format_field_vtk(_mesh(gd), int(gd["io_vtk_step"][0]), f, gd["io_solid"], path)
    assert path.read_bytes() == bytes(gd["io_vtk"])


def test_checkpoint_files_match_reference(gd, tmp_path):
    _lib_or_skip()
    f = {k: gd["io_" + k] for k in ("u", "v", "w", "p", "nu_t")}
    t, dt, nxt = gd["ckpt_args"]
    G.write_checkpoint_files(_mesh(gd), f, gd["io_solid"], float(t), float(dt), int(nxt), tmp_path)
    assert (tmp_path / "checkpoint.meta").read_bytes() == bytes(gd["ckpt_meta"])
    assert (tmp_path / "checkpoint.data").read_bytes() == bytes(gd["ckpt_data"])


def test_checkpoint_reader_reads_reference_files(gd, tmp_path):
    _lib_or_skip()
    (tmp_path / "checkpoint.meta").write_bytes(bytes(gd["ckpt_meta"]))
    (tmp_path / "checkpoint.data").write_bytes(bytes(gd["ckpt_data"]))
    step, t, dt, f, solid, _ = G.read_checkpoint_files(_mesh(gd), tmp_path)
    t0, dt0, nxt = gd["ckpt_args"]
    assert step == int(nxt) and t == float(t0) and dt == float(dt0)
    for k in ("u", "v", "w", "p", "nu_t"):
        assert np.array_equal(f[k], gd["io_" + k]), k
    assert np.array_equal(solid, gd["io_solid"])
    # no metadata file: step 0, like load_state's "start from scratch"
    empty = tmp_path / "none"
    empty.mkdir()
    assert G.read_checkpoint_files(_mesh(gd), empty)[0] == 0


def test_checkpoint_side_file_round_trip(gd, tmp_path):
    _lib_or_skip()
    f = {k: gd["io_" + k] for k in ("u", "v", "w", "p", "nu_t")}
    u3 = [gd["io_u"] * 2, gd["io_v"] * 3, gd["io_w"] * 4]
    G.write_checkpoint_files(_mesh(gd), f, gd["io_solid"], 1.5, 2e-4, 9, tmp_path, unew3=u3)
    step, t, dt, g, solid, r3 = G.read_checkpoint_files(_mesh(gd), tmp_path, with_unew=True)
    assert (step, t, dt) == (9, 1.5, 2e-4)
    for a, b in zip(u3, r3):
        assert np.array_equal(a, b)
