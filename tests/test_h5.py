"""The minimal HDF5 codec: reads files written by the HDF5 library (the
reference's own fixtures, when its sources are present) and round-trips the
snapshot layout of include/io/hdf5_writer.hpp (t<step>/<field>, float32)."""
from pathlib import Path

import numpy as np
import pytest

from tecs_gb300 import h5

import oracle

# the reference checkout ($TECS_REFERENCE or a "reference" directory beside
# the repository); the fixtures below are skipped without it
REF = oracle.reference_root() or Path("/nonexistent")
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
    (tmp_path / "request_00007.h5").write_bytes(b"\0" * 64)  # not an HDF5 file
    assert h5.last_snapshot(tmp_path, 7) is None


def test_last_snapshot_of_a_file_whose_writer_stopped(tmp_path):
    """A server that stops mid-run leaves its files unclosed; every group written before the stop is
    complete on disk (each write rewrites and flushes the root metadata), so the newest one resumes."""
    w = h5.H5Writer(tmp_path / "request_00003.h5")
    assert h5.last_snapshot(tmp_path, 3) is None  # no group yet
    pos = {k: np.full((5, 3), k, np.float32) for k in (100, 200, 300)}
    for k in (100, 200, 300):
        w.write_group(f"t{k}", {"position": pos[k]})
        step, p, q = h5.last_snapshot(tmp_path, 3)
        assert step == k and q is None
        np.testing.assert_array_equal(p, pos[k])
    w.f.close()  # the process ends without close(): no final truncation


def _root_tree(path):
    """(the root node's level, {level: [(node, left sibling, right sibling)] left to right}, the group
    names in tree order); asserts each node's keys bound its children's names."""
    import struct

    b = Path(path).read_bytes()
    btree, heap = struct.unpack_from("<QQ", b, 56 + 24)  # the scratch pad of the superblock's root entry
    assert b[heap:heap + 4] == b"HEAP"
    size, _, data = struct.unpack_from("<QQQ", b, heap + 8)

    def name(off):
        assert off < size
        return b[data + off:b.index(b"\0", data + off)].decode()

    levels = {}

    def walk(node):
        assert b[node:node + 4] == b"TREE"
        _, level, used, left, right = struct.unpack_from("<BBHQQ", b, node + 4)
        keys = [name(struct.unpack_from("<Q", b, node + 24 + 16 * k)[0]) for k in range(used + 1)]
        kids = [struct.unpack_from("<Q", b, node + 32 + 16 * k)[0] for k in range(used)]
        levels.setdefault(level, []).append((node, left, right))
        names = []
        for k, c in enumerate(kids):
            if level:
                sub = walk(c)
            else:
                assert b[c:c + 4] == b"SNOD"
                nsym = struct.unpack_from("<H", b, c + 6)[0]
                sub = [name(struct.unpack_from("<Q", b, c + 8 + 40 * e)[0]) for e in range(nsym)]
            # the library's lookup rule: a child holds the names above its left key and up to its right key
            assert all(keys[k].encode() < s.encode() <= keys[k + 1].encode() for s in sub)
            assert sub[-1] == keys[k + 1]
            names += sub
        return names

    names = walk(btree)
    return b[btree + 5], levels, names


@pytest.mark.parametrize("count, fmt", [(300, "t{}"), (2001, "t{}"), (9000, "t{:05d}")])
def test_root_group_takes_any_number_of_groups(tmp_path, count, fmt):
    """Past 256 groups (32 symbol table nodes) the root B-tree gains a level, past 8,192 a second, and
    past 1,024 short names the name heap moves to a larger segment; every node keeps the library's key
    rule and sibling links, and every group reads back."""
    w = h5.H5Writer(tmp_path / "long.h5")
    for s in range(count):
        w.write_group(fmt.format(s), {"position": np.full((1, 3), s, np.float32)})
    w.close()
    top, levels, names = _root_tree(tmp_path / "long.h5")
    want = sorted((fmt.format(s) for s in range(count)), key=str.encode)
    assert names == want
    assert top == (0 if count <= 256 else 1 if count <= 8192 else 2)
    for level, nodes in levels.items():
        for j, (node, left, right) in enumerate(nodes):
            assert left == (nodes[j - 1][0] if j else h5.UNDEF)
            assert right == (nodes[j + 1][0] if j + 1 < len(nodes) else h5.UNDEF)
    f = h5.H5File(tmp_path / "long.h5")
    assert f.keys() == sorted(want)
    for s in (0, count // 3, count - 1):
        np.testing.assert_array_equal(f.read(fmt.format(s) + "/position"), np.full((1, 3), s, np.float32))


GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("name", ["lk_writer", "lk_writer_nolinks"])
def test_xdmf_sidecar_matches_reference(tmp_path, name):
    """XdmfSidecar gives, byte for byte, the reference writer's sidecar for its write sequence:
    write_static(cell_type), then (position, polarity, links) at t = 0, dt, 2 dt; with links each grid's
    topology is the links' polylines, without them the cells as vertices."""
    g = dict(np.load(GOLDEN / f"{name}.npz"))
    n, dt = len(g["x0"]), float(g["dt"])
    x = h5.XdmfSidecar(tmp_path / "out", threshold=1000)  # several partial writes before the end
    x.write_static([("cell_type", np.zeros(n, np.float32))])
    for k in range(int(g["steps"]) + 1):
        x.write(k * dt, f"t{k}", [("position", g["x0"]), ("polarity", g["p0"]), ("links", g["links"])],
                links=("links",))
    x.close()
    assert (tmp_path / "out.xmf").read_bytes() == (GOLDEN / f"{name}.xmf").read_bytes()


def test_snapshot_sink_sidecar_points_at_its_datasets(tmp_path):
    import xml.etree.ElementTree as ET

    sink = h5.SnapshotSink(tmp_path, dt=0.05)
    rng = np.random.default_rng(5)
    data = {}
    for req, pol in ((2, True), (7, False)):
        for step in (100, 200, 300):
            x = rng.standard_normal((11 + req, 3)).astype(np.float32)
            p = rng.standard_normal((11 + req, 2)).astype(np.float32) if pol else None
            sink(req, step, x, p)
            data[(req, step)] = (x, p)
    sink.close()
    for req in (2, 7):
        root = ET.parse(tmp_path / f"request_{req:05d}.xmf").getroot()
        grids = root.find("Domain").find("Grid").findall("Grid")
        assert [gr.get("Name") for gr in grids] == ["t100", "t200", "t300"]
        f = h5.H5File(tmp_path / f"request_{req:05d}.h5")
        for gr in grids:
            step = int(gr.get("Name")[1:])
            assert gr.find("Time").get("Value") == f"{step * 0.05:f}"
            assert gr.find("Topology").get("TopologyType") == "Polyvertex"
            items = gr.iter("DataItem")
            for item in items:
                fname, path = item.text.strip().split(":")
                assert fname == f"request_{req:05d}.h5"
                arr = f.read(path)
                assert [int(v) for v in item.get("Dimensions").split()] == list(arr.shape)
            x, p = data[(req, step)]
            np.testing.assert_array_equal(f.read(f"t{step}/position"), x)
            names = [a.get("Name") for a in gr.findall("Attribute")]
            assert names == (["polarity"] if p is not None else [])


@pytest.mark.parametrize("first, closed", [(5, True), (300, True), (300, False), (0, True)])
def test_append_continues_as_one_writer(tmp_path, first, closed):
    """A file continued with append=True -- after a clean close, or after a writer that stopped mid-run --
    ends byte for byte as one writer's file of all the groups (here past one B-tree node and the first
    name heap)."""
    total = first + 80 if first < 300 else 2100

    def group(s):
        return {"position": np.full((1 + s % 3, 3), s, np.float32)}

    one = h5.H5Writer(tmp_path / "one.h5")
    for s in range(total):
        one.write_group(f"t{s}", group(s))
    one.close()
    w = h5.H5Writer(tmp_path / "two.h5")
    for s in range(first):
        w.write_group(f"t{s}", group(s))
    if closed:
        w.close()
    else:
        w.f.close()
    w = h5.H5Writer(tmp_path / "two.h5", append=True)
    assert w.order == sorted(f"t{s}" for s in range(first))
    for s in range(first, total):
        w.write_group(f"t{s}", group(s))
    w.close()
    assert (tmp_path / "two.h5").read_bytes() == (tmp_path / "one.h5").read_bytes()


def test_append_refuses_a_foreign_file(tmp_path):
    p = tmp_path / "x.h5"
    p.write_bytes(b"not hdf5" * 20)
    with pytest.raises(ValueError, match="not written by this writer"):
        h5.H5Writer(p, append=True)


def test_sink_append_keeps_earlier_snapshots_and_sidecar(tmp_path):
    """A resumed server's sink continues each request's file; file and sidecar end as one run's."""
    pos = {k: np.full((4, 3), k, np.float32) for k in (100, 200, 300, 400)}
    pol = {k: np.full((4, 2), -k, np.float32) for k in (100, 200, 300, 400)}
    one = h5.SnapshotSink(tmp_path / "one", dt=0.05)
    for k in (100, 200, 300, 400):
        one(9, k, pos[k], pol[k])
    one.close()
    two = h5.SnapshotSink(tmp_path / "two", dt=0.05)
    for k in (100, 200):
        two(9, k, pos[k], pol[k])
    two.files[9].f.close()  # the server stops: the file is left unclosed, the sidecar unwritten
    two = h5.SnapshotSink(tmp_path / "two", dt=0.05, append=True)
    for k in (300, 400):
        two(9, k, pos[k], pol[k])
    two.close()
    for name in ("request_00009.h5", "request_00009.xmf"):
        assert (tmp_path / "two" / name).read_bytes() == (tmp_path / "one" / name).read_bytes()


def _cpp_reader(tmp_path):
    import shutil
    import subprocess

    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    import tecs_gb300 as tg

    root = Path(__file__).resolve().parents[1]
    lib = Path(tg.library_path())
    exe = tmp_path / "h5_reader"
    r = subprocess.run(["g++", "-std=c++20", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{root / 'include'}",
                        str(root / "tests" / "cpp" / "h5_reader.cpp"), f"-L{lib.parent}", "-l" + lib.stem[3:],
                        f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _cpp_read(exe, path, name, kind, tmp_path):
    import subprocess

    out = tmp_path / f"{name.replace('/', '_')}.bin"
    r = subprocess.run([str(exe), str(path), name, kind, str(out)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    dims = tuple(int(v) for v in r.stdout.split())
    dtype = np.int32 if kind == "int" else np.float32
    cols = {"vec3": 3, "polarity": 2, "float": 1, "int": 1}[kind]
    return dims, np.fromfile(out, dtype).reshape(-1, cols) if cols > 1 else np.fromfile(out, dtype)


def test_cpp_reader_reads_the_codecs_files(tmp_path):
    """io::HDF5_Reader (include/tecs/hdf5_reader.hpp) against the Python codec's files: float32 rows,
    int32 and uint32 datasets converted into float and int views, in nested groups."""
    tg = pytest.importorskip("tecs_gb300")
    del tg
    exe = _cpp_reader(tmp_path)
    rng = np.random.default_rng(7)
    x = rng.standard_normal((300, 3)).astype(np.float32)
    p = rng.standard_normal((300, 2)).astype(np.float32)
    t = rng.integers(-5, 5, 300).astype(np.int32)
    u = rng.integers(0, 1000, 300).astype(np.uint32)
    w = h5.H5Writer(tmp_path / "in.h5")
    w.write_group("t0", {"position": x, "polarity": p, "cell_type": t, "ids": u})
    w.close()
    dims, got = _cpp_read(exe, tmp_path / "in.h5", "t0/position", "vec3", tmp_path)
    assert dims == (300, 3)
    np.testing.assert_array_equal(got, x)
    np.testing.assert_array_equal(_cpp_read(exe, tmp_path / "in.h5", "t0/polarity", "polarity", tmp_path)[1], p)
    np.testing.assert_array_equal(_cpp_read(exe, tmp_path / "in.h5", "t0/cell_type", "int", tmp_path)[1], t)
    np.testing.assert_array_equal(_cpp_read(exe, tmp_path / "in.h5", "t0/cell_type", "float", tmp_path)[1],
                                  t.astype(np.float32))
    np.testing.assert_array_equal(_cpp_read(exe, tmp_path / "in.h5", "t0/ids", "int", tmp_path)[1], u.astype(np.int32))


def test_cpp_reader_reads_library_written_fixture(tmp_path):
    """The reference's library-written initial state (examples/data/sphere_ic.h5) through the C++ reader
    equals the Python reader's."""
    path = FIXTURES[0]
    if not path.exists():
        pytest.skip("reference fixtures not present")
    exe = _cpp_reader(tmp_path)
    f = h5.H5File(path)
    for name, kind in (("POINTS", "vec3"), ("polarity", "polarity"), ("cell_type", "int")):
        dims, got = _cpp_read(exe, path, name, kind, tmp_path)
        ref = f.read(name)
        assert dims == ref.shape
        np.testing.assert_array_equal(got, ref)
