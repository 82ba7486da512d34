"""The minimal HDF5 codec: reads files written by the HDF5 library (the
reference's own fixtures, when its sources are present) and round-trips the
snapshot layout of include/io/hdf5_writer.hpp (t<step>/<field>, float32)."""
import os
from pathlib import Path

import numpy as np
import pytest

from tecs_gb300 import h5

REF = Path(os.environ.get("TECS_REFERENCE", "/root/reference"))
FIXTURES = [REF / "examples" / "data" / "sphere_ic.h5", REF / "examples" / "tribolium" / "initial_data" / "serosa.h5",
            REF / "examples" / "tribolium" / "initial_data" / "surface.h5"]


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: p.name)
def test_reads_library_written_fixtures(path):
    if not path.exists():
        pytest.skip("reference fixtures not present")
    f = h5.H5File(path)
    keys = f.keys()
    assert "POINTS" in keys
    pts = f.read("POINTS")
    assert pts.ndim == 2 and pts.shape[1] == 3 and pts.dtype == np.float32 and np.isfinite(pts).all()
    if "cell_type" in keys:
        ct = f.read("cell_type")
        assert ct.shape == (pts.shape[0],) and ct.dtype == np.int32


def test_snapshot_roundtrip_many_groups(tmp_path):
    rng = np.random.default_rng(1)
    w = h5.H5Writer(tmp_path / "sim.h5")
    ref = {}
    for step in range(0, 2100, 100):  # 21 groups: several symbol table nodes
        n = 50 + step
        x = rng.standard_normal((n, 3)).astype(np.float32)
        p = rng.standard_normal((n, 2)).astype(np.float32)
        w.write_group(f"t{step}", {"position": x, "polarity": p})
        ref[step] = (x, p)
    w.close()
    f = h5.H5File(tmp_path / "sim.h5")
    assert sorted(f.keys()) == sorted(f"t{s}" for s in ref)
    for s, (x, p) in ref.items():
        assert f.keys(f"t{s}") == ["polarity", "position"]
        np.testing.assert_array_equal(f.read(f"t{s}/position"), x)
        np.testing.assert_array_equal(f.read(f"t{s}/polarity"), p)


def test_readable_while_streaming(tmp_path):
    w = h5.H5Writer(tmp_path / "live.h5")
    w.write_group("t0", {"position": np.zeros((4, 3), np.float32)})
    assert h5.H5File(tmp_path / "live.h5").keys() == ["t0"]
    w.write_group("t100", {"position": np.ones((5, 3), np.float32)})
    f = h5.H5File(tmp_path / "live.h5")
    assert f.keys() == ["t0", "t100"] and f.read("t100/position").shape == (5, 3)
    w.close()


def test_empty_dataset_and_int_types(tmp_path):
    w = h5.H5Writer(tmp_path / "e.h5")
    w.write_group("static", {"cell_type": np.arange(7, dtype=np.int32), "empty": np.zeros((0, 3), np.float32)})
    w.close()
    f = h5.H5File(tmp_path / "e.h5")
    np.testing.assert_array_equal(f.read("static/cell_type"), np.arange(7))
    assert f.read("static/empty").shape == (0, 3)


def test_last_snapshot_is_the_newest_group(tmp_path):
    from tecs_gb300 import h5

    sink = h5.SnapshotSink(tmp_path)
    rng = np.random.default_rng(3)
    pos = {k: rng.standard_normal((7, 3)).astype(np.float32) for k in (50, 100, 150)}
    pol = {k: rng.standard_normal((7, 2)).astype(np.float32) for k in (50, 100, 150)}
    for k in (50, 100, 150):
        sink(4, k, pos[k], pol[k])
    sink(5, 50, pos[50], None)
    sink.close()
    step, p, q = h5.last_snapshot(tmp_path, 4)
    assert step == 150
    np.testing.assert_array_equal(p, pos[150])
    np.testing.assert_array_equal(q, pol[150])
    step, p, q = h5.last_snapshot(tmp_path, 5)
    assert step == 50 and q is None
    np.testing.assert_array_equal(p, pos[50])
    assert h5.last_snapshot(tmp_path, 6) is None  # no file
    (tmp_path / "request_00007.h5").write_bytes(b"\0" * 64)  # a file never closed: no superblock
    assert h5.last_snapshot(tmp_path, 7) is None
