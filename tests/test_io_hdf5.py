"""Snapshot files (tupan_gb300.io, tupan/io/hdf5io.py:23-146) on the CPU.

* The reader against an HDF5 file written by the HDF5 library itself (the
  MATLAB 7.3 file scipy ships as test data): superblock 0 behind a 512-byte
  user block, a symbol-table root group, a contiguous float64 dataset and a
  fixed-length string attribute.
* The writer: round trips through the reader, appends across sessions
  (merging the partial last chunk), groups and datasets large enough for
  multi-level B-trees, and a structure walk that checks the rules the HDF5
  library applies when it reads a file: nodes allocated at full size and not
  overlapping, entry counts within 2K, sorted keys that bound their
  children, local heaps whose free list ends in 1, global heap collections
  of at least 4 KiB ending in a free-space object, message sizes in
  multiples of 8, and the end-of-file address.
* The IO interface with particle sets on the CPU: snapshots (plain and
  numbered), appends, worldlines, the background writer, the error paths.
* PSDF streams (tupan/io/psdfio.py): the text PyYAML writes for the
  `!Particle` mappings, block and flow sequences read back, exact round
  trips and the conversions between the two formats.
"""
import os
import struct
import warnings

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from tupan_gb300.io import BODIES_DTYPE, IO, class_of, hdf5, pickled_class  # noqa: E402
from tupan_gb300.particles import ParticleSystem  # noqa: E402

SCIPY_HDF5 = None
try:
    import scipy.io.matlab as _m
    SCIPY_HDF5 = os.path.join(os.path.dirname(_m.__file__), "tests", "data", "testhdf5_7.4_GLNX86.mat")
except ImportError:
    pass


def test_reader_on_a_library_written_file():
    if SCIPY_HDF5 is None or not os.path.exists(SCIPY_HDF5):
        pytest.skip("scipy's HDF5 test file is not installed")
    with hdf5.File(SCIPY_HDF5) as f:
        assert f.sb_at == 512 and f.keys() == ["testdouble"]
        d = f["testdouble"]
        assert d.shape == (9, 1) and d.dtype == np.float64 and d.layout[0] == "contiguous"
        assert d.attrs == {"MATLAB_class": "double"}
        # the MATLAB variable 0:pi/4:2*pi
        assert np.array_equal(d.read().ravel(), np.arange(9) * (np.pi / 4))
    _walk(SCIPY_HDF5)                           # the structure rules hold for the library's own file


def test_append_to_a_library_written_file(tmp_path):
    # new groups and a dataset added behind the library's own structures
    # (addresses relative to the 512-byte user block); the original dataset
    # and its attribute stay readable
    if SCIPY_HDF5 is None or not os.path.exists(SCIPY_HDF5):
        pytest.skip("scipy's HDF5 test file is not installed")
    p = tmp_path / "lib.hdf5"
    p.write_bytes(open(SCIPY_HDF5, "rb").read())
    with hdf5.File(str(p), "a") as f:            # opened for writing, nothing changed:
        f.keys()
    assert p.read_bytes() == open(SCIPY_HDF5, "rb").read()     # not a byte written
    rows = _rows(100, 0, np.random.default_rng(5))
    with hdf5.File(str(p), "a") as f:
        f.require_group("Worldline/particlesystem").append_rows("bodies", rows)
    with hdf5.File(str(p), "r+") as f:
        f["Worldline/particlesystem"].append_rows("bodies", rows)
    _walk(str(p))
    with hdf5.File(str(p)) as f:
        assert f.keys() == ["Worldline", "testdouble"]
        assert np.array_equal(f["testdouble"].read().ravel(), np.arange(9) * (np.pi / 4))
        assert f["testdouble"].attrs == {"MATLAB_class": "double"}
        assert np.array_equal(f["Worldline/particlesystem/bodies"].read(), np.concatenate([rows, rows]))


# ---- structure walk ----------------------------------------------------------------------

def _walk(path):
    """Every structure reachable from the superblock, checked; returns the
    extents [(start, end, what)]."""
    f = hdf5.File(path)
    ext = [(f.sb_at - f.base, f.sb_at - f.base + 96, "superblock")]     # addresses relative to the base
    size = os.path.getsize(path)
    sb = f._read(-f.base + f.sb_at, 96)
    eof = struct.unpack_from("<Q", sb, 40)[0]
    assert eof <= size                          # stored as an absolute address; an aborted write may trail it
    ik, lk, ck = f.internal_k, f.leaf_k, f.chunk_k

    def header(addr):
        pre = f._read(addr, 16)
        assert pre[0] == 1
        nmsg, _r, hsize = struct.unpack_from("<HII", pre, 2)
        ext.append((addr, addr + 16 + hsize, "header"))
        buf = f._read(addr + 16, hsize)
        p = count = 0
        while p < hsize:
            mtype, msize = struct.unpack_from("<HH", buf, p)
            assert msize % 8 == 0
            p += 8 + msize
            count += 1
        assert p == hsize and count == nmsg

    def gcol(addr):
        hdr = f._read(addr, 16)
        assert hdr[:4] == b"GCOL"
        n = struct.unpack_from("<Q", hdr, 8)[0]
        assert n >= 4096
        buf = f._read(addr, n)
        p = 16
        while True:
            idx = struct.unpack_from("<H", buf, p)[0]
            osz = struct.unpack_from("<Q", buf, p + 8)[0]
            if idx == 0:
                assert p + osz == n            # the free-space object's size includes its header
                break
            p += 16 + ((osz + 7) & ~7)
        ext.append((addr, addr + n, "gcol"))

    def tree(addr, ntype, ksz, node_size, cap, leaf):
        hdr = f._read(addr, 24)
        assert hdr[:4] == b"TREE" and hdr[4] == ntype
        level, n = hdr[5], struct.unpack_from("<H", hdr, 6)[0]
        assert n <= cap
        ext.append((addr, addr + node_size, "tree%d" % ntype))
        body = f._read(addr + 24, n * (ksz + 8) + ksz)
        keys = [body[i * (ksz + 8):i * (ksz + 8) + ksz] for i in range(n + 1)]
        kids = [struct.unpack_from("<Q", body, i * (ksz + 8) + ksz)[0] for i in range(n)]
        out = []
        for i, c in enumerate(kids):
            if level:
                out += tree(c, ntype, ksz, node_size, cap, leaf)
            else:
                out.append((keys[i], keys[i + 1], c))
                leaf(keys[i], keys[i + 1], c)
        return out

    objs_seen = set()

    def group(addr):
        msgs = f._messages(addr)
        header(addr)
        st = [m for m in msgs if m[0] == hdf5.MSG_SYMTAB][0][3]
        btree, heap = struct.unpack_from("<QQ", st, 0)
        h = f._read(heap, 32)
        assert h[:4] == b"HEAP"
        hsize, free, daddr = struct.unpack_from("<QQQ", h, 8)
        ext.append((heap, heap + 32, "heap"))
        ext.append((daddr, daddr + hsize, "heapdata"))
        data = f._read(daddr, hsize)
        assert free == 1 or free + 16 <= hsize
        while free != 1:                        # the free list ends in 1
            nxt, fsz = struct.unpack_from("<QQ", data, free)
            assert fsz >= 16 and free + fsz <= hsize
            free = nxt
        name_at = lambda k: hdf5._cstr(data, struct.unpack_from("<Q", k)[0]).encode()
        children = []

        def snod(lkey, rkey, c):
            hd = f._read(c, 8)
            assert hd[:4] == b"SNOD"
            ns = struct.unpack_from("<H", hd, 6)[0]
            assert 0 < ns <= 2 * lk
            ext.append((c, c + 8 + 2 * lk * 40, "snod"))
            ents = f._read(c + 8, 40 * ns)
            names = []
            for i in range(ns):
                noff, oaddr, ctype = struct.unpack_from("<QQI", ents, 40 * i)
                nm = hdf5._cstr(data, noff).encode()
                assert noff % 8 == 0
                names.append(nm)
                children.append((oaddr, ctype, ents[40 * i + 24:40 * i + 40]))
            assert names == sorted(names) and len(set(names)) == ns
            assert names[0] > name_at(lkey) and names[-1] == name_at(rkey)

        tree(btree, 0, 8, 24 + 2 * ik * 8 + (2 * ik + 1) * 8, 2 * ik, snod)
        for oaddr, ctype, cache in children:
            if oaddr in objs_seen:
                continue
            objs_seen.add(oaddr)
            kinds = {m[0] for m in f._messages(oaddr)}
            if hdf5.MSG_SYMTAB in kinds:
                if ctype == 1:                  # a cached symbol table matches the message
                    st2 = [m for m in f._messages(oaddr) if m[0] == hdf5.MSG_SYMTAB][0][3]
                    assert cache == st2
                group(oaddr)
            else:
                dataset(oaddr)
        for m in msgs:
            if m[0] == hdf5.MSG_ATTRIBUTE:
                attr(m[3])

    def attr(data):
        if data[0] != 1:                        # what this walk follows: v1 heap references
            return
        nn, nt, ns = struct.unpack_from("<HHH", data, 2)
        p = 8 + hdf5._pad8(nn)
        if data[p] & 0x0F == 9:                 # variable-length string: heap reference
            q = p + hdf5._pad8(nt) + hdf5._pad8(ns)
            _len, coll, _idx = struct.unpack_from("<IQI", data, q)
            if coll not in [e[0] for e in ext if e[2] == "gcol"]:
                gcol(coll)

    def dataset(addr):
        header(addr)
        ds = f._load_node("?", addr)
        for m in f._messages(addr):
            if m[0] == hdf5.MSG_ATTRIBUTE:
                attr(m[3])
        if ds.layout[0] != "chunked" or ds.layout[2] == hdf5.UNDEF:
            return
        rank = len(ds.layout[1])
        ksz = 8 + 8 * (rank + 1)
        c = ds.layout[1][0]

        def chunk(lkey, rkey, caddr):
            nb, _mask, off = struct.unpack_from("<IIQ", lkey)
            roff = struct.unpack_from("<Q", rkey, 8)[0]
            assert off % c == 0 and roff >= off + c and off < ds.shape[0]
            ext.append((caddr, caddr + nb, "chunk"))

        leaves = tree(ds.layout[2], 1, ksz, 24 + 2 * ck * 8 + (2 * ck + 1) * ksz, 2 * ck, chunk)
        offs = [struct.unpack_from("<Q", lk_, 8)[0] for lk_, _r, _c in leaves]
        assert offs == sorted(offs) and offs == list(range(0, ds.shape[0], c))

    root = f.addr
    objs_seen.add(root)
    group(root)
    ctype, _r, bt, hp = struct.unpack_from("<IIQQ", sb, 72)
    st = [m for m in f._messages(root) if m[0] == hdf5.MSG_SYMTAB][0][3]
    assert ctype == 1 and struct.pack("<QQ", bt, hp) == st
    ext.sort()
    for (a0, a1, w0), (b0, b1, w1) in zip(ext, ext[1:]):
        assert a1 <= b0, "%s [%d,%d) overlaps %s [%d,%d)" % (w0, a0, a1, w1, b0, b1)
    assert ext[-1][1] <= eof - f.base
    f.close()
    return ext


def _rows(n, start, rng):
    a = np.zeros(n, BODIES_DTYPE)
    a["id"] = np.arange(start, start + n)
    for k in ("mass", "rx", "vy", "time"):
        a[k] = rng.random(n)
    a["nstep"] = rng.integers(0, 1 << 40, n)
    return a


def test_writer_round_trip_and_appends(tmp_path):
    p = str(tmp_path / "t.hdf5")
    rng = np.random.default_rng(7)
    parts = []
    with hdf5.File(p, "w") as f:
        g = f.require_group("Snapshot/particlesystem")
        g.set_attr("Class", pickled_class("tupan.particles.allparticles", "ParticleSystem"))
        parts.append(_rows(1000, 0, rng))
        g.append_rows("bodies", parts[-1]).set_attr("Class", pickled_class("tupan.particles.body", "Bodies"))
    _walk(p)
    for k in range(4):                          # appends into the partial last chunk, new groups
        assert os.path.getsize(p) == struct.unpack_from("<Q", open(p, "rb").read(48), 40)[0]
        with hdf5.File(p, "a") as f:
            g = f.require_group("Snapshot/particlesystem")
            g.set_attr("Class", pickled_class("tupan.particles.allparticles", "ParticleSystem"))
            parts.append(_rows(1 + 2000 * k, 1000, rng))
            g.append_rows("bodies", parts[-1])
            for j in range(70):
                f.require_group("Snapshot_%06d" % (70 * k + j))
        _walk(p)
    with hdf5.File(p) as f:
        assert len(f) == 281 and f.keys()[0] == "Snapshot"
        d = f["Snapshot/particlesystem/bodies"]
        assert d.chunks == (64,) and d.maxshape == (None,)
        assert [x[0] for x in d.filters] == [hdf5.FILTER_SHUFFLE, hdf5.FILTER_DEFLATE]
        assert class_of(d.attrs["Class"]) == ("tupan.particles.body", "Bodies")
        got = d.read()
    assert got.dtype == BODIES_DTYPE and np.array_equal(got, np.concatenate(parts))
    with pytest.raises(ValueError):
        hdf5.File(p).require_group("x")          # read-only
    # rows of other fields are stored by field name, the dataset's others zero
    part = np.zeros(3, np.dtype([("rx", "<f8"), ("id", "<u8")]))
    part["rx"], part["id"] = 1.5, 9
    with hdf5.File(p, "a") as f:
        f["Snapshot/particlesystem"].append_rows("bodies", part)
        with pytest.raises(ValueError):
            f["Snapshot/particlesystem"].append_rows("bodies", np.zeros(1, [("nope", "<f8")]))
    with hdf5.File(p) as f:
        tail = f["Snapshot/particlesystem/bodies"].read()[-3:]
    assert (tail["rx"] == 1.5).all() and (tail["id"] == 9).all() and (tail["mass"] == 0).all()
    # an exception inside the block leaves the file at its previous state
    with pytest.raises(RuntimeError):
        with hdf5.File(p, "a") as f:
            f["Snapshot/particlesystem"].append_rows("bodies", _rows(500, 0, rng))
            f.require_group("never")
            raise RuntimeError("stop")
    _walk(p)
    with hdf5.File(p) as f:
        assert "never" not in f and len(f["Snapshot/particlesystem/bodies"]) == len(got) + 3


def test_three_level_chunk_tree(tmp_path):
    # 1024-row chunks of 8-byte records: 4100 chunks need a root over 65
    # internal nodes over leaves of 64
    p = str(tmp_path / "big.hdf5")
    n = 4100 * 1024 - 5
    a = np.zeros(n, np.dtype([("k", "<u8")]))
    a["k"] = np.arange(n) // 3
    with hdf5.File(p, "w") as f:
        f.append_rows("d", a, level=1)
    ext = _walk(p)
    assert sum(1 for e in ext if e[2] == "tree1") == 67 + 1
    with hdf5.File(p) as f:
        assert np.array_equal(f["d"].read(), a)


def test_empty_and_nested_groups(tmp_path):
    p = str(tmp_path / "g.hdf5")
    with hdf5.File(p, "w") as f:
        f.require_group("a/b/c")
        f.require_group("a/empty")
        f.set_attr("note", "root é")
    _walk(p)
    with hdf5.File(p, "r+") as f:
        assert f.attrs["note"] == "root é"
        assert f["a"].keys() == ["b", "empty"] and len(f["a/empty"]) == 0
        f["a/b/c"].append_rows("x", np.arange(5, dtype="<f8"))
    _walk(p)
    with hdf5.File(p) as f:
        assert np.array_equal(f["a/b/c/x"][...], np.arange(5.0))
    with pytest.raises(FileExistsError):
        hdf5.File(p, "x")


# ---- the IO interface ----------------------------------------------------------------------

def _set(n, seed):
    rng = np.random.default_rng(seed)
    ps = ParticleSystem(n, device="cpu")
    for k in ("mass", "eps2", "rx", "ry", "rz", "vx", "vy", "vz", "time", "tstep"):
        ps.set_array(k, rng.random(n))
    ps.set_array("nstep", rng.integers(0, 100, n))
    ps.set_array("id", rng.permutation(n))
    return ps


FIELDS = [k for k, _t in [("id", 0), ("mass", 0), ("eps2", 0), ("rx", 0), ("ry", 0), ("rz", 0), ("vx", 0),
                          ("vy", 0), ("vz", 0), ("time", 0), ("nstep", 0), ("tstep", 0)]]


def _same(a, b):
    return a.n == b.n and all(torch.equal(getattr(a, k).cpu(), getattr(b, k).cpu()) for k in FIELDS)


def test_snapshots_and_worldlines(tmp_path):
    p = str(tmp_path / "run.hdf5")
    ps = _set(700, 1)
    io = IO(p, "a")
    io.dump_snapshot(ps)
    io.dump_snapshot(ps[:300], 12)
    io.dump_snapshot(ps[300:], 12)               # a second dump into a snapshot appends
    io.dump_worldline(ps[:5])
    io.dump_worldline(ps[0:0])                   # an empty worldline writes the group only
    io.dump_worldline(ps[5:9])
    _walk(p)
    r = IO(p, "r")
    assert _same(r.load_snapshot(device="cpu"), ps)
    assert _same(r.load_snapshot(12, device="cpu"), ps)
    assert _same(r.load_worldline(device="cpu"), ps[:9])
    with hdf5.File(p) as f:
        assert f.keys() == ["Snapshot", "Snapshot_000012", "Worldline"]
        g = f["Snapshot_000012/particlesystem"]
        assert class_of(g.attrs["Class"]) == ("tupan.particles.allparticles", "ParticleSystem")
        assert f["Worldline/particlesystem/bodies"].dtype == BODIES_DTYPE


def test_background_writer(tmp_path):
    p = str(tmp_path / "bg.hdf5")
    ps = _set(2000, 2)
    io = IO(p, "a", background=True)
    for k in range(10):
        io.dump_worldline(ps[200 * k:200 * (k + 1)])
    assert _same(io.load_worldline(device="cpu"), ps)     # load waits for the queue
    io.close()
    q = str(tmp_path / "bg2.hdf5")
    IO(q, "a", background=True).dump_snapshot(ps)        # queued by an object never flushed
    assert _same(IO(q, "r").load_snapshot(device="cpu"), ps)
    bad = IO(str(tmp_path / "missing_dir" / "x.hdf5"), "a", background=True)
    bad.dump_worldline(ps)
    with pytest.raises(FileNotFoundError):
        bad.flush()
    bad.close()


def test_multi_kind_file_loads_as_one_set(tmp_path):
    # a reference-layout file with two particle kinds (allparticles.py:29-39)
    p = str(tmp_path / "kinds.hdf5")
    rng = np.random.default_rng(3)
    bodies = _rows(10, 0, rng)
    sdt = np.dtype(BODIES_DTYPE.descr + [("spinx", "<f8"), ("age", "<f8")])
    stars = np.zeros(4, sdt)
    stars["id"] = np.arange(10, 14)
    stars["mass"] = 2.0
    stars["age"] = 5.0
    with hdf5.File(p, "w") as f:
        g = f.require_group("Snapshot/particlesystem")
        g.append_rows("stars", stars)
        g.append_rows("bodies", bodies)
    ps = IO(p, "r").load_snapshot(device="cpu")
    assert ps.n == 14
    assert np.array_equal(ps.id.numpy(), np.arange(14))          # bodies before stars (name order)
    assert np.array_equal(ps.age.numpy(), [0.0] * 10 + [5.0] * 4)


def test_numpy_particle_sets(tmp_path):
    # what the reference's integrators hand their dumpper: a set whose
    # attributes are numpy arrays (an empty one at the start of a step)
    class NumpySet(object):
        pass
    ps = _set(50, 4)
    q = NumpySet()
    q.n = ps.n
    for k in FIELDS:
        setattr(q, k, getattr(ps, k).numpy().astype(np.uint64 if k in ("id", "nstep") else np.float64))
    empty = NumpySet()
    empty.n = 0
    p = str(tmp_path / "np.hdf5")
    io = IO(p, "a")
    io.dump_worldline(q)
    io.dump_worldline(empty)
    io.dump_snapshot(q, 0)
    assert _same(io.load_worldline(device="cpu"), ps) and _same(io.load_snapshot(0, device="cpu"), ps)
    # a queued dump holds the values of the call, not later ones
    bg = IO(str(tmp_path / "np_bg.hdf5"), "a", background=True)
    bg._submit(lambda: __import__("time").sleep(0.2))       # keep the writer busy
    bg.dump_snapshot(q)
    q.rx[...] = -1.0
    assert _same(bg.load_snapshot(device="cpu"), ps)
    bg.close()


def test_error_paths(tmp_path):
    ps = _set(3, 0)
    with pytest.raises(NotImplementedError, match="Unknown format: 'txt'"):
        IO(str(tmp_path / "x.txt"), "a").dump_worldline(ps)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        with pytest.raises(SystemExit):
            IO(str(tmp_path / "none.hdf5"), "r").load_snapshot()
    assert "No such file" in str(w[0].message)
    junk = tmp_path / "junk.hdf5"
    junk.write_bytes(b"\0" * 2048)
    with pytest.raises(ValueError, match="File not in a supported format"):
        IO(str(junk), "r").load_snapshot()
    assert class_of(pickled_class("m.n", "C")) == ("m.n", "C") and class_of("x") is None


# ---- PSDF streams ------------------------------------------------------------------------

def test_psdf_text_is_what_pyyaml_writes(tmp_path):
    # one particle, the keys of psdfio.py's Stream.to_yaml in sorted order,
    # floats as PyYAML represents them
    from tupan_gb300.io import psdf
    cols = {"id": np.array([3]), "mass": np.array([0.5]), "eps2": np.array([1e-3]),
            "rx": np.array([1.0]), "ry": np.array([-2.5]), "rz": np.array([1e-5]),
            "vx": np.array([0.0]), "vy": np.array([np.inf]), "vz": np.array([-0.0]),
            "time": np.array([0.125])}
    assert psdf.dump_text(cols) == (
        "--- !Particle\neps2: 0.001\nid: 3\nm: 0.5\nr:\n- 1.0\n- -2.5\n- 1.0e-05\n"
        "t: 0.125\ntype: body\nv:\n- 0.0\n- .inf\n- -0.0\n")
    assert [psdf.yaml_float(x) for x in (1e20, 2.5e-300, float("nan"), -np.inf)] == \
        ["1.0e+20", "2.5e-300", ".nan", "-.inf"]


def test_psdf_reads_block_and_flow_forms():
    from tupan_gb300.io import psdf
    text = ("%YAML 1.1\n# a comment line\n--- !Particle\nid: 0\nm: 1.0\nt: 0.0\nr: [1.0, 2.0, 3.0]  # flow form\n"
            "v:\n  - 0.5\n  - -0.5\n  - 0\npot: -1.25\neps2: 0.0\n---\nid: 1\nm: 2.0\nt: 0.0\n"
            "type: blackhole\nr: [0, 0, 0]\nv: [0, 0, 1.0e-3]\npot: -2.0\neps2: 0.0\n...\n")
    cols = psdf.columns_from_docs(psdf.parse_text(text))
    assert list(cols["id"]) == [0, 1] and list(cols["mass"]) == [1.0, 2.0]
    assert list(cols["rz"]) == [3.0, 0.0] and list(cols["vz"]) == [0.0, 1e-3]
    assert list(cols["phi"]) == [-1.25, -2.0] and "ax" not in cols
    with pytest.raises(ValueError):
        psdf.columns_from_docs(psdf.parse_text("---\nid: 0\nm: 1.0\n"))        # no r, v, t
    with pytest.raises(ValueError):
        psdf.columns_from_docs(psdf.parse_text("---\nid: 0\nm: 1\nt: 0\nr: [0,0,0]\nv: [0,0,0]\ntype: gas\n"))


def test_psdf_round_trip_and_conversions(tmp_path):
    ps = _set(40, 9)
    ps.register_auxiliary_attribute("phi", "real")
    ps.phi.copy_(-ps.mass * 3.0)
    for k in ("ax", "ay", "az"):
        ps.register_auxiliary_attribute(k, "real")
        getattr(ps, k).copy_(ps.rx * 0.5)
    p = str(tmp_path / "s.psdf")
    io = IO(p, "w")
    io.dump_snapshot(ps[:25])
    IO(p, "a").dump_worldline(ps[25:])              # appends to the stream
    back = IO(p, "r").load_snapshot(device="cpu")
    for k in ("id", "mass", "eps2", "rx", "ry", "rz", "vx", "vy", "vz", "time", "phi", "ax", "az"):
        assert torch.equal(getattr(back, k), getattr(ps, k)), k
    IO(p, "r").to_hdf5()                             # s.hdf5 beside it
    h = IO(str(tmp_path / "s.hdf5"), "r")
    assert torch.equal(h.load_snapshot(device="cpu").rx, ps.rx)
    os.remove(p)
    h.to_psdf()                                      # and back
    assert torch.equal(IO(p, "r").load_snapshot(device="cpu").vz, ps.vz)
    with pytest.raises(ValueError, match="already in 'psdf'"):
        IO(p, "r").to_psdf()
    with pytest.raises(ValueError, match="already in 'hdf5'"):
        h.to_hdf5()


def test_reader_paths_the_writer_does_not_make(tmp_path):
    # objects assembled here message by message, as other writers of the
    # same format version lay them out: contiguous and compact storage, a
    # big-endian float, a version-2 dataspace, a version-2 compound with an
    # array member and a fixed string, the Fletcher-32 filter through a
    # version-2 pipeline message, version-2 and -3 attributes, and an object
    # header whose attribute sits in a continuation block
    p = str(tmp_path / "hand.hdf5")

    def msg(mtype, data, flags=0):
        data = data + b"\0" * (hdf5._pad8(len(data)) - len(data))
        return struct.pack("<HHB3x", mtype, len(data), flags) + data

    def header(f, msgs):
        body = b"".join(msgs)
        return f._append(struct.pack("<BxHII4x", 1, len(msgs), 1, len(body)) + body)

    be_f4 = bytes([0x11, 0x21, 31, 0]) + struct.pack("<IHHBBBBI", 4, 0, 32, 23, 8, 0, 23, 127)
    f8 = hdf5._encode_dtype(np.dtype("<f8"))
    arr3 = bytes([0x2A, 0, 0, 0]) + struct.pack("<I", 24) + bytes([1, 0, 0, 0]) + struct.pack("<II", 3, 0) + f8
    s4 = bytes([0x13, 0, 0, 0]) + struct.pack("<I", 4)
    comp = (bytes([0x26, 2, 0, 0]) + struct.pack("<I", 28) + b"pos\0\0\0\0\0" + struct.pack("<I", 0) + arr3
            + b"tag\0\0\0\0\0" + struct.pack("<I", 24) + s4)
    cdt = np.dtype({"names": ["pos", "tag"], "formats": [("<f8", (3,)), "S4"], "offsets": [0, 24],
                    "itemsize": 28})
    recs = np.zeros(5, cdt)
    recs["pos"] = np.arange(15.0).reshape(5, 3)
    recs["tag"] = [b"ab", b"cd", b"ef", b"gh", b"ij"]
    with hdf5.File(p, "w") as f:
        # contiguous big-endian float32 (2, 3), dataspace version 2
        data = (np.arange(6).reshape(2, 3) / 4).astype(">f4")
        daddr = f._append(data.tobytes())
        attr3 = (struct.pack("<BBHHHB", 3, 0, 5, 8, 8, 0) + b"unit\0" + bytes([0x13, 0, 0, 0])
                 + struct.pack("<I", 3) + bytes([1, 0, 0, 0, 0, 0, 0, 0]) + b"kpc")
        block = msg(hdf5.MSG_ATTRIBUTE, attr3)
        cont = f._append(block)
        contig = header(f, [msg(hdf5.MSG_DATASPACE, bytes([2, 2, 0, 1]) + struct.pack("<QQ", 2, 3)),
                            msg(hdf5.MSG_DATATYPE, be_f4, 1),
                            msg(hdf5.MSG_LAYOUT, struct.pack("<BBQQ", 3, 1, daddr, data.nbytes)),
                            msg(hdf5.MSG_CONTINUATION, struct.pack("<QQ", cont, len(block)))])
        # compact int16 (4,), version-2 attribute with three int32 values
        i2 = np.array([-1, 2, -3, 4], "<i2")
        attr2 = (struct.pack("<BBHHH", 2, 0, 5, 12, 16) + b"dims\0" + hdf5._encode_dtype(np.dtype("<i4"))
                 + bytes([1, 1, 0, 0, 0, 0, 0, 0]) + struct.pack("<Q", 3) + np.array([7, 8, 9], "<i4").tobytes())
        compact = header(f, [msg(hdf5.MSG_DATASPACE, bytes([1, 1, 0, 0, 0, 0, 0, 0]) + struct.pack("<Q", 4)),
                             msg(hdf5.MSG_DATATYPE, hdf5._encode_dtype(np.dtype("<i2")), 1),
                             msg(hdf5.MSG_LAYOUT, struct.pack("<BBH", 3, 0, i2.nbytes) + i2.tobytes()),
                             msg(hdf5.MSG_ATTRIBUTE, attr2)])
        # chunked compound, 2-record chunks, Fletcher-32 (checksum appended, not checked)
        entries = []
        for k in range(3):
            chunk = np.zeros(2, cdt)
            part = recs[2 * k:2 * k + 2]
            chunk[:len(part)] = part
            raw = chunk.tobytes() + b"\x12\x34\x56\x78"
            entries.append(((2 * k,), (f._append(raw), len(raw), 0)))
        bt, _nodes = f._write_chunk_btree(entries, 2, 28)
        pipe = struct.pack("<BB", 2, 1) + struct.pack("<HHH", hdf5.FILTER_FLETCHER32, 1, 0)
        chunked = header(f, [msg(hdf5.MSG_DATASPACE, bytes([1, 1, 1, 0, 0, 0, 0, 0]) + struct.pack("<QQ", 5, hdf5.UNDEF)),
                             msg(hdf5.MSG_DATATYPE, comp, 1),
                             msg(hdf5.MSG_LAYOUT, struct.pack("<BBBQII", 3, 2, 2, bt, 2, 28)),
                             msg(hdf5.MSG_PIPELINE, pipe, 1)])
        f._entries().update({"contig": contig, "compact": compact, "chunked": chunked})
        f._mark_dirty()
    _walk(p)
    with hdf5.File(p) as f:
        c = f["contig"]
        assert c.shape == (2, 3) and c.dtype == np.dtype(">f4") and np.array_equal(c.read(), data)
        assert c.attrs == {"unit": "kpc"}
        assert np.array_equal(f["compact"].read(), i2)
        assert list(f["compact"].attrs["dims"]) == [7, 8, 9]
        got = f["chunked"].read()
        assert got.dtype == cdt and np.array_equal(got, recs)


ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "baseline", "_ref")

REF_CHILD = r"""
import sys
import numpy as np
sys.path.insert(0, %(ref)r)
sys.path.insert(1, %(root)r)
import tupan.lib
import tupan_gb300.lib.extensions as backend
tupan.lib.extensions = backend
sys.modules["tupan.lib.extensions"] = backend
from tupan.particles.allparticles import ParticleSystem
from tupan_gb300.io import IO
ps = ParticleSystem(nstars=5)
ps.rx[...] = np.arange(5.0) + 0.25
ps.mass[...] = 0.2
ps.stars.age[...] = 3.0
IO(%(path)r, "a").dump_snapshot(ps, 2)
IO(%(path)r, "a").dump_worldline(ps)
IO(%(path)r, "a").dump_worldline(type(ps)())
"""


def test_reference_particle_sets_keep_their_kinds(tmp_path):
    # the reference's own ParticleSystem handed to this IO (as its
    # integrators hand their dumpper): each kind's dataset holds that kind's
    # get_state() records under its own Class, as hdf5io.py:51-66 stores them
    import subprocess
    import sys
    if not os.path.isdir(os.path.join(REF, "tupan", "particles")):
        pytest.skip("no installed reference tree (baseline/_ref)")
    path = str(tmp_path / "ref.hdf5")
    env = dict(os.environ, HOME=str(tmp_path))
    r = subprocess.run([sys.executable, "-c", REF_CHILD % {"ref": REF, "root": ROOT, "path": path}],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    _walk(path)
    with hdf5.File(path) as f:
        g = f["Snapshot_000002/particlesystem"]
        assert g.keys() == ["stars"]
        assert class_of(g.attrs["Class"]) == ("tupan.particles.allparticles", "ParticleSystem")
        assert class_of(g["stars"].attrs["Class"]) == ("tupan.particles.star", "Stars")
        rec = g["stars"].read()
        assert rec.dtype.names[:12] == BODIES_DTYPE.names and "metallicity" in rec.dtype.names
        assert list(rec["rx"]) == [0.25, 1.25, 2.25, 3.25, 4.25] and (rec["age"] == 3.0).all()
    back = IO(path, "r").load_snapshot(2, device="cpu")
    assert back.n == 5 and torch.equal(back.age, torch.full((5,), 3.0, dtype=torch.float64))
    assert IO(path, "r").load_worldline(device="cpu").n == 5


def test_worldline_selection_matches_numpy_remainder():
    # Base.record selects with torch.fmod; the reference with numpy's %:
    # zero at exactly the same times, for either sign of the step
    from tupan_gb300.integrator import Base

    class Dumpper(object):
        def __init__(self):
            self.sets = []

        def dump_worldline(self, wl):
            self.sets.append(wl)

    rng = np.random.default_rng(11)
    tau = 2.0 ** -7
    t = np.concatenate([np.arange(64) * tau, rng.random(64), np.arange(64) * (tau / 3), [0.1, 0.3, 1e-300]])
    for sign in (1.0, -1.0):
        for freq in (1, 2, 4, 3):
            ps = ParticleSystem(len(t), device="cpu")
            ps.set_array("time", sign * t)
            b = Base(sign * tau, 0.0, ps, dumpper=Dumpper(), dump_freq=freq)
            b.wl = ps[0:0]
            b.record(ps, sign * tau)
            want = np.nonzero(np.remainder(sign * t, freq * sign * tau) == 0)[0]
            assert np.array_equal(b.wl.id.numpy(), want), (sign, freq)


def test_appends_rewrite_only_the_index_edge(tmp_path):
    # a worldline appended in 150 separate sessions (one per dump, as the IO
    # layer opens the file): the chunk index keeps its full nodes and
    # rewrites only its right edge, so the file stays within 30% of the same
    # rows written at once (a full index rewrite per append made it 2.2
    # times that size here)
    p, q = str(tmp_path / "many.hdf5"), str(tmp_path / "once.hdf5")
    rng = np.random.default_rng(1)
    parts = [_rows(700, 700 * k, rng) for k in range(150)]
    for r in parts:
        with hdf5.File(p, "a") as f:
            f.require_group("Worldline/particlesystem").append_rows("bodies", r)
    with hdf5.File(q, "w") as f:
        f.require_group("Worldline/particlesystem").append_rows("bodies", np.concatenate(parts))
    assert os.path.getsize(p) < 1.3 * os.path.getsize(q)
    _walk(p)
    with hdf5.File(p) as f:
        assert np.array_equal(f["Worldline/particlesystem/bodies"].read(), np.concatenate(parts))
