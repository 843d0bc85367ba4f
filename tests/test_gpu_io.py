"""Device-resident statistics and files written from device fields, against
the reference's own output (tests/golden/io_tiny7.npz): sums bit-exact,
statistics file, field file and checkpoint byte-exact, checkpoint reload."""
import os

import numpy as np
import pytest

import les_gb300 as G

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "io_tiny7.npz")
KEYS = ("u", "v", "w", "p", "uu", "vv", "ww", "uv", "uw", "vw")


@pytest.fixture(scope="module")
def gd():
    return np.load(GOLD)


def _mesh(gd):
    nx, ny, nz, dx, dy, dz = gd["mesh"]
    return G.Mesh(int(nx), int(ny), int(nz), float(dx), float(dy), float(dz))


def test_device_statistics_match_reference(gd, tmp_path):
    with G.Context(_mesh(gd)) as c:
        c.stats_begin(0)
        for s in range(3):
            for k in ("u", "v", "w", "p"):
                c.upload(k, gd["stats_in%d_%s" % (s, k)])
            c.stats_update(s)
        sums, ns = c.stats_read()
        assert ns == int(gd["stats_samples"][0])
        for k in KEYS:
            assert np.array_equal(sums[k], gd["stats_sum_" + k]), k
        path = tmp_path / "stats.vtk"
        c.stats_save_vtk(path)
    assert path.read_bytes() == bytes(gd["stats_vtk"])


def _upload_io(c, gd):
    for k in ("u", "v", "w", "p", "nu_t"):
        c.upload(k, gd["io_" + k])
    c.upload_mask(gd["io_solid"])


def test_field_file_from_device_matches_reference(gd, tmp_path):
    path = tmp_path / "output_42.vtk"
    with G.Context(_mesh(gd)) as c:
        _upload_io(c, gd)
        c.write_vtk(int(gd["io_vtk_step"][0]), path)
        for k in ("u", "v", "w"):          # the caller may go on at once: the file holds the snapshot
            c.upload(k, np.zeros(c.n))
        c.io_wait()
    assert path.read_bytes() == bytes(gd["io_vtk"])


def test_checkpoint_from_device_matches_reference_and_reloads(gd, tmp_path):
    t, dt, nxt = (float(x) for x in gd["ckpt_args"])
    with G.Context(_mesh(gd)) as c:
        _upload_io(c, gd)
        c.save_state(tmp_path, t, dt, int(nxt))
        c.io_wait()
    assert (tmp_path / "checkpoint.meta").read_bytes() == bytes(gd["ckpt_meta"])
    assert (tmp_path / "checkpoint.data").read_bytes() == bytes(gd["ckpt_data"])
    with G.Context(_mesh(gd)) as c:
        step, t1, dt1 = c.load_state(tmp_path)
        assert (step, t1, dt1) == (int(nxt), t, dt)
        for k in ("u", "v", "w", "p", "nu_t"):
            assert np.array_equal(c.download(k), gd["io_" + k]), k
        assert np.array_equal(c.download_mask(), gd["io_solid"])
        # no checkpoint: step 0 and the fields untouched (load_state's fresh start)
        assert c.load_state(tmp_path / "missing")[0] == 0
        assert np.array_equal(c.download("u"), gd["io_u"])
