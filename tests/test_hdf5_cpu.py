"""The HDF5 writer (ptarmigan_gb300/hdf5.py) against its reader: every
datatype the final-state output uses, nested groups, aliases (hard links),
groups spread over several symbol-table nodes, empty and scalar datasets,
and the structural invariants of the format."""
import struct

import numpy as np
import pytest

from ptarmigan_gb300 import hdf5


def _tree(tmp_path):
    root = hdf5.Group()
    b = root.group("build")
    b.dataset("version", "1.5.0")
    b.dataset("features", "")
    cfg = root.group("config")
    cfg.dataset("mpi-tasks", 1)
    ctl = cfg.group("control")
    ctl.dataset("dt_multiplier", 0.5)
    ctl.dataset("radiation_reaction", True)
    ctl.dataset("classical", False)
    ctl.dataset("rng_seed", 12345678901234)
    ctl.dataset("offset", -3)
    fs = root.group("final-state").group("photon")
    rng = np.random.default_rng(1)
    w = rng.random(37)
    x = rng.normal(size=(37, 4))
    pol = rng.normal(size=(37, 4))
    ids = np.arange(37, dtype=np.uint64) * 3
    fs.dataset("weight", w, unit="1", desc="number of real photons each macrophoton represents")
    fs.dataset("position", x, unit="m", desc="four-position of the photon")
    fs.dataset("polarization", pol, unit="1", desc="Stokes parameters of the photon: I, Q, U, V",
               alias="polarisation")
    fs.dataset("id", ids, desc="unique ID of the photon")
    fs.dataset("empty", np.zeros(0))
    fs.dataset("flags", np.array([True, False, True]))
    fs.dataset("n32", np.arange(5, dtype=np.int32) - 2)
    fs.dataset("f32", np.linspace(0, 1, 6, dtype=np.float32))
    many = root.group("many")
    for k in range(40):
        many.dataset("m%02d" % (39 - k), float(k))
    path = tmp_path / "t.h5"
    hdf5.write(str(path), root)
    return path, w, x, pol, ids


def test_round_trip(tmp_path):
    path, w, x, pol, ids = _tree(tmp_path)
    r = hdf5.read(str(path))
    m = r["members"]
    assert m["build"]["members"]["version"]["value"] == "1.5.0"
    assert m["build"]["members"]["features"]["value"] == ""
    c = m["config"]["members"]
    assert c["mpi-tasks"]["value"] == 1 and c["mpi-tasks"]["shape"] == ()
    ctl = c["control"]["members"]
    assert ctl["dt_multiplier"]["value"] == 0.5
    assert ctl["radiation_reaction"]["value"] is True and ctl["radiation_reaction"]["type"] == "bool"
    assert ctl["classical"]["value"] is False
    assert ctl["rng_seed"]["value"] == 12345678901234
    assert ctl["offset"]["value"] == -3
    ph = m["final-state"]["members"]["photon"]["members"]
    assert np.array_equal(ph["weight"]["value"], w)
    assert ph["weight"]["attrs"] == {"desc": "number of real photons each macrophoton represents", "unit": "1"}
    assert ph["position"]["type"] == "array" and ph["position"]["shape"] == (37,)
    assert np.array_equal(ph["position"]["value"], x)
    assert np.array_equal(ph["polarization"]["value"], pol)
    # the alias is a second hard link to the same object header
    assert ph["polarisation"]["addr"] == ph["polarization"]["addr"]
    assert ph["polarization"]["refs"] == 2
    assert ph["id"]["value"].dtype == np.uint64 and np.array_equal(ph["id"]["value"], ids)
    assert ph["empty"]["shape"] == (0,) and ph["empty"]["value"].size == 0
    assert ph["flags"]["value"].tolist() == [True, False, True]
    assert ph["n32"]["value"].dtype == np.int32 and ph["n32"]["value"].tolist() == [-2, -1, 0, 1, 2]
    assert ph["f32"]["value"].dtype == np.float32
    many = m["many"]["members"]
    assert list(many) == sorted(many) and len(many) == 40
    assert all(many["m%02d" % (39 - k)]["value"] == float(k) for k in range(40))


def test_structure(tmp_path):
    path, *_ = _tree(tmp_path)
    data = path.read_bytes()
    assert data[:8] == b"\x89HDF\r\n\x1a\n"
    # superblock v0, 8-byte offsets and lengths, K = 4 / 16
    assert data[8:16] == bytes([0, 0, 0, 0, 0, 8, 8, 0])
    assert struct.unpack_from("<HH", data, 16) == (4, 16)
    base, free, eof, drv = struct.unpack_from("<QQQQ", data, 24)
    assert base == 0 and free == hdf5.UNDEF and drv == hdf5.UNDEF and eof == len(data)
    # every object header: version 1, messages 8-aligned and filling the size
    r = hdf5._Reader(data)
    seen = []

    def walk(addr):
        ver, _, nmsg, refs, size = struct.unpack_from("<BBHII", data, addr)
        assert ver == 1 and refs >= 1 and size % 8 == 0
        p = addr + 16
        for _ in range(nmsg):
            _, msize, _ = struct.unpack_from("<HHB", data, p)
            assert msize % 8 == 0
            p += 8 + msize
        assert p == addr + 16 + size
        seen.append(addr)
        o = r.obj(addr)
        if o["kind"] == "group":
            for v in o["members"].values():
                walk(v["addr"])

    walk(r.root)
    assert len(seen) > 60
    # the "many" group needed 5 symbol-table nodes of at most 8 entries
    many = r.obj(r.root)["members"]["many"]
    msgs, _ = r.header(many["addr"])
    tree, heap = struct.unpack_from("<QQ", dict(msgs)[hdf5.MSG_STAB], 0)
    assert data[tree:tree + 4] == b"TREE" and struct.unpack_from("<H", data, tree + 6)[0] == 5


def test_rejects_unsupported(tmp_path):
    root = hdf5.Group()
    with pytest.raises(TypeError):
        root.dataset("c", np.array([1 + 2j]))
    root.dataset("x", 1.0)
    with pytest.raises(ValueError):
        root.dataset("x", 2.0)
    with pytest.raises(ValueError):
        root.group("x")


def test_names_and_text(tmp_path):
    """Link names are checked; UTF-8 text and names that sort by byte
    (upper case before lower) round-trip; an empty group is readable."""
    root = hdf5.Group()
    for bad in ("", "a/b", ".", ".."):
        with pytest.raises(ValueError):
            root.dataset(bad, 1.0)
    root.dataset("x", 1.0)
    with pytest.raises(ValueError):
        root.dataset("y", 2.0, alias="x")
    g = root.group("names")
    for name in ("b", "B", "a", "A", "_", "Z9", "z"):
        g.dataset(name, name)
    root.group("empty")
    root.dataset("text", "µm, γ and χ")
    path = tmp_path / "n.h5"
    hdf5.write(str(path), root)
    r = hdf5.read(str(path))["members"]
    assert list(r["names"]["members"]) == sorted(["b", "B", "a", "A", "_", "Z9", "z"], key=lambda s: s.encode())
    assert all(v["value"] == k for k, v in r["names"]["members"].items())
    assert r["empty"]["kind"] == "group" and r["empty"]["members"] == {}
    assert r["text"]["value"] == "µm, γ and χ"


def test_files_open_in_h5py(tmp_path):
    """Where h5py (libhdf5) is installed, the files this module writes open
    in it with the same structure, values and attributes."""
    h5py = pytest.importorskip("h5py")
    from ptarmigan_gb300 import hdf5
    root = hdf5.Group()
    g = root.group("final-state").group("photon")
    x = np.arange(12, dtype=np.float64).reshape(3, 4)
    g.dataset("position", x, unit="m", desc="four-position of the photon")
    g.dataset("id", np.arange(3, dtype=np.uint64), desc="unique ID of the photon")
    root.group("config").dataset("input-file", "laser:\n  a0: 1.0\n")
    fn = str(tmp_path / "f.h5")
    hdf5.write(fn, root)
    with h5py.File(fn, "r") as f:
        np.testing.assert_array_equal(f["final-state/photon/position"][...], x)
        assert f["final-state/photon/position"].attrs["unit"] in (b"m", "m")
        np.testing.assert_array_equal(f["final-state/photon/id"][...], np.arange(3))
