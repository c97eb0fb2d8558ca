"""The HDF5 subset of ``cardiax_gb300.h5`` and the data-set functions of ``cardiax_gb300.io``
(cardiax/io.py:13-115), on the CPU.

No HDF5 library exists where these tests run, so the files are checked two ways: read back
through the package's reader, and walked structure by structure against the byte layout of the
HDF5 File Format Specification (superblock version 0, version-1 object headers, group B-trees,
symbol-table nodes, local heaps, dataspace/datatype/fill-value/layout messages).
"""
import struct

import numpy as np
import pytest
import torch

from cardiax_gb300 import h5, io
from cardiax_gb300.params import PARAMSET_3, Params
from cardiax_gb300.stimulus import Protocol, Stimulus

UNDEF = 0xFFFFFFFFFFFFFFFF


def _raw(path):
    with open(path, "rb") as fh:
        return fh.read()


def test_round_trip_types_shapes_and_groups(tmp_path):
    p = tmp_path / "a.h5"
    rng = np.random.default_rng(0)
    data = {
        "f32": rng.standard_normal((4, 3, 7, 9)).astype(np.float32),
        "f64": rng.standard_normal((5,)),
        "i64": np.arange(-3, 9, dtype=np.int64).reshape(3, 4),
        "i32": np.array([1, -2, 3], dtype=np.int32),
        "u8": np.arange(200, 216, dtype=np.uint8),
        "empty": np.zeros((0, 7, 9), np.float32),
        "g/deep/x": np.float32(2.5),
        "g/y": np.array(7),
    }
    with h5.File(p, "w") as f:
        for k, v in data.items():
            f.create_dataset(k, data=v)
        f.create_dataset("scalar", data=0.01)
        f.create_dataset("zeros", shape=(3, 5), dtype="float32")
        f.create_group("empty_group")
    with h5.File(p) as f:
        assert list(f) == sorted(list(f), key=str.encode)
        assert set(f) == {"f32", "f64", "i64", "i32", "u8", "empty", "g", "scalar", "zeros",
                          "empty_group"}
        for k, v in data.items():
            got = f[k][()]
            assert np.asarray(got).dtype == np.asarray(v).dtype, k
            np.testing.assert_array_equal(got, v)
        s = f["scalar"][...]
        assert s.shape == () and s.dtype == np.float64 and s == 0.01
        np.testing.assert_array_equal(f["zeros"][:], np.zeros((3, 5), np.float32))
        assert len(f["empty_group"]) == 0
        assert isinstance(f["g"], h5.Group) and list(f["g"]) == ["deep", "y"]
        np.testing.assert_array_equal(f["f32"][1:4:2, 2], data["f32"][1:4:2, 2])


def test_row_writes_go_straight_to_the_file(tmp_path):
    p = tmp_path / "rows.h5"
    f = h5.File(p, "w")
    d = f.create_dataset("states", shape=(6, 3, 33, 40), dtype="float32")
    rows = np.random.default_rng(1).random((6, 3, 33, 40), dtype=np.float32)
    for t in (4, 0, 2):
        d[t] = rows[t]
    d[5, 1] = rows[5, 1]
    f.close()
    with h5.File(p) as f:
        got = f["states"][:]
    want = np.zeros_like(rows)
    want[[0, 2, 4]] = rows[[0, 2, 4]]
    want[5, 1] = rows[5, 1]
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("n", [0, 1, 8, 9, 17, 64, 256])
def test_many_members_span_symbol_table_nodes(tmp_path, n):
    p = tmp_path / f"m{n}.h5"
    names = [f"v{i:03d}_{'x' * (i % 13)}" for i in range(n)]
    with h5.File(p, "w") as f:
        for i, name in enumerate(names):
            f.create_dataset("grp/" + name, data=np.float64(i))
        if n == 0:
            f.create_group("grp")
    with h5.File(p) as f:
        assert list(f["grp"]) == sorted(names, key=str.encode)
        for i, name in enumerate(names):
            assert f["grp"][name][()] == i


def test_more_members_than_one_btree_node_is_refused(tmp_path):
    f = h5.File(tmp_path / "big.h5", "w")
    for i in range(257):
        f.create_dataset(f"d{i}", data=np.int64(i))
    with pytest.raises(ValueError):
        f.close()


def test_errors(tmp_path):
    p = tmp_path / "e.h5"
    with h5.File(p, "w") as f:
        f.create_dataset("a", data=np.zeros(3))
        with pytest.raises(ValueError):
            f.create_dataset("a", data=np.zeros(3))
        with pytest.raises(TypeError):
            f.create_dataset("s", data=np.array(["x"]))
        with pytest.raises(TypeError):
            f.create_dataset("c", data=np.zeros(2, np.complex64))
        with pytest.raises(KeyError):
            f.create_dataset("a/b", data=np.zeros(1))
    with h5.File(p) as f:
        with pytest.raises(KeyError):
            f["missing"]
        with pytest.raises(OSError):
            f["a"][0] = 1.0
        with pytest.raises(OSError):
            f.create_dataset("b", data=np.zeros(1))
    bad = tmp_path / "not.h5"
    bad.write_bytes(b"\0" * 200)
    with pytest.raises(OSError):
        h5.File(bad)
    raw = _raw(p)
    short = tmp_path / "short.h5"
    short.write_bytes(raw[:-8])
    with pytest.raises(OSError):
        h5.File(short)


# ---------------------------------------------------------------------------------------------
# structure walk against the specification's byte layouts

def _header(raw, addr):
    version, _, nmsg, refcount, size = struct.unpack_from("<BBHII", raw, addr)
    assert version == 1 and refcount == 1
    assert raw[addr + 12:addr + 16] == b"\0" * 4
    msgs, p = [], addr + 16
    while p < addr + 16 + size:
        mtype, msize, flags = struct.unpack_from("<HHB", raw, p)
        assert msize % 8 == 0 and raw[p + 5:p + 8] == b"\0\0\0"
        msgs.append((mtype, flags, raw[p + 8:p + 8 + msize]))
        p += 8 + msize
    assert p == addr + 16 + size and len(msgs) == nmsg
    return msgs


def _walk_group(raw, header, cached=None):
    msgs = _header(raw, header)
    assert [m[0] for m in msgs] == [0x11]
    btree, heap = struct.unpack_from("<QQ", msgs[0][2], 0)
    if cached is not None:
        assert cached == (btree, heap)
    assert raw[heap:heap + 8] == b"HEAP\0\0\0\0"
    hsize, free, hdata = struct.unpack_from("<QQQ", raw, heap + 8)
    assert free == 1 and hsize % 8 == 0 and raw[hdata] == 0
    names = raw[hdata:hdata + hsize]
    assert raw[btree:btree + 6] == b"TREE\0\0"
    used, left, right = struct.unpack_from("<HQQ", raw, btree + 6)
    assert left == UNDEF and right == UNDEF and used <= 32
    keys = [struct.unpack_from("<Q", raw, btree + 24 + 16 * i)[0] for i in range(used + 1)]
    kids = [struct.unpack_from("<Q", raw, btree + 32 + 16 * i)[0] for i in range(used)]
    assert keys[0] == 0
    members = {}
    for i, c in enumerate(kids):
        assert raw[c:c + 6] == b"SNOD\x01\0"
        nsym = struct.unpack_from("<H", raw, c + 6)[0]
        assert 1 <= nsym <= 8
        got = []
        for j in range(nsym):
            off, hdr, cache, res = struct.unpack_from("<QQII", raw, c + 8 + 40 * j)
            assert res == 0
            name = names[off:names.index(b"\0", off)]
            got.append(name)
            scratch = struct.unpack_from("<QQ", raw, c + 32 + 40 * j)
            members[name.decode()] = (hdr, cache, scratch)
        assert got == sorted(got)
        assert names[keys[i + 1]:names.index(b"\0", keys[i + 1])] == got[-1]
        if i:
            prev = names[keys[i]:names.index(b"\0", keys[i])]
            assert prev < got[0]
    return members


F32_TYPE = bytes.fromhex("11201f00040000000000200017080017" "7f000000")
F64_TYPE = bytes.fromhex("11203f00080000000000400034" "0b0034" "ff030000")
I64_TYPE = bytes.fromhex("1008000008000000" "00004000")


def test_bytes_follow_the_format_specification(tmp_path):
    p = tmp_path / "s.h5"
    with h5.File(p, "w") as f:
        f.create_dataset("states", shape=(2, 3, 5, 6), dtype="float32")
        f.create_dataset("params/dt", data=0.02)
        f.create_dataset("start", data=[0, 10])
        f.create_dataset("field", data=np.zeros((0,), np.float64))
    raw = _raw(p)
    # superblock version 0
    assert raw[:8] == b"\x89HDF\r\n\x1a\n"
    assert raw[8:16] == bytes([0, 0, 0, 0, 0, 8, 8, 0])
    assert struct.unpack_from("<HHI", raw, 16) == (4, 16, 0)
    base, freespace, eof, driver = struct.unpack_from("<QQQQ", raw, 24)
    assert (base, freespace, driver) == (0, UNDEF, UNDEF) and eof == len(raw)
    name_off, root, cache, res, bt, hp = struct.unpack_from("<QQIIQQ", raw, 56)
    assert (name_off, cache, res) == (0, 1, 0)
    members = _walk_group(raw, root, cached=(bt, hp))
    assert sorted(members) == ["field", "params", "start", "states"]
    # a group member caches its B-tree and heap, a dataset member caches nothing
    hdr, cache, scratch = members["params"]
    assert cache == 1
    assert list(_walk_group(raw, hdr, cached=scratch)) == ["dt"]
    dt_hdr = _walk_group(raw, hdr)["dt"][0]

    def dataset(hdr):
        msgs = {m[0]: m for m in _header(raw, hdr)}
        assert sorted(msgs) == [0x1, 0x3, 0x5, 0x8]
        assert msgs[0x3][1] == 1 and msgs[0x5][1] == 1
        assert msgs[0x5][2][:8] == bytes([2, 2, 2, 1, 0, 0, 0, 0])
        return msgs

    st_hdr, cache, _ = members["states"]
    assert cache == 0
    m = dataset(st_hdr)
    assert m[0x1][2] == struct.pack("<BBBB4x4Q4Q", 1, 4, 1, 0, 2, 3, 5, 6, 2, 3, 5, 6)
    assert m[0x3][2][:20] == F32_TYPE
    layout = m[0x8][2]
    assert layout[:2] == bytes([3, 1])
    addr, size = struct.unpack_from("<QQ", layout, 2)
    assert size == 2 * 3 * 5 * 6 * 4 and addr + size <= len(raw)
    assert raw[addr:addr + size] == b"\0" * size
    m = dataset(dt_hdr)
    assert m[0x1][2] == bytes([1, 0, 0, 0, 0, 0, 0, 0])
    assert m[0x3][2][:20] == F64_TYPE
    addr, size = struct.unpack_from("<QQ", m[0x8][2], 2)
    assert size == 8 and struct.unpack_from("<d", raw, addr)[0] == 0.02
    m = dataset(members["start"][0])
    assert m[0x3][2][:12] == I64_TYPE
    m = dataset(members["field"][0])
    addr, size = struct.unpack_from("<QQ", m[0x8][2], 2)
    assert (addr, size) == (UNDEF, 0)


# ---------------------------------------------------------------------------------------------
# cardiax/io.py functions (no resizing: that needs the GPU)

def test_io_data_set_like_the_reference_writes_it(tmp_path):
    shape = (12, 16)
    path = str(tmp_path / "sub" / "run.hdf5")
    params = PARAMSET_3
    D = np.full(shape, 0.001, np.float32)
    fields = [torch.zeros(shape), torch.ones(shape)]
    stimuli = [Stimulus(Protocol(0, 2, 1e9), fields[0]), Stimulus(Protocol(400, 2, 0), fields[1])]
    hdf5 = io.init(path, shape, n_iter=5, n_stimuli=len(stimuli))
    assert io.add_params(hdf5, params, D, 0.02, 0.015)
    assert io.add_stimuli(hdf5, stimuli)
    assert io.add_diffusivity(hdf5, D)
    states = np.random.default_rng(3).random((4, 3) + shape, dtype=np.float32)
    dset = hdf5["states"]
    for i in range(3):
        assert io.add_state(dset, tuple(torch.from_numpy(states[i])), i)
    assert io.add_states(dset, states[3:4], 3, 4)
    hdf5.close()

    with h5.File(path) as f:
        assert f["states"].shape == (5, 3) + shape and f["states"].dtype == np.float32
        assert f["stimuli"].shape == (2,) + shape
        np.testing.assert_array_equal(f["states"][:4], states)
        np.testing.assert_array_equal(f["states"][4], 0)
        assert f["params/dt"][...] == 0.02 and f["params/dt"].dtype == np.float64
        assert set(f["params"]) == set(Params._fields) | {"D", "dt", "dx"}
        np.testing.assert_array_equal(f["field"][1], np.ones(shape, np.float32))
        assert f["period"].dtype == np.float64 and list(f["start"][:]) == [0, 400]
        assert io.load_state(f["states"], 0, 4, 2).shape == (2, 3) + shape
        back = io.load_stimuli(f)
        assert [tuple(s.protocol) for s in back] == [(0, 2, 1e9), (400, 2, 0)]
        np.testing.assert_array_equal(back[1].field, fields[1].numpy())
    p2, D2 = io.load_params(path)
    assert p2 == Params(*(float(np.float64(x)) for x in params))
    np.testing.assert_array_equal(D2, D)
    np.testing.assert_array_equal(io.load_diffusivity(path), D)
    # the root holds the params group, which h5py refuses to slice as well
    with pytest.raises(TypeError):
        io.load(path)


def test_io_load_slices_every_root_dataset(tmp_path):
    path = str(tmp_path / "plain.hdf5")
    hdf5 = io.init(path, (4, 5), n_iter=6, n_stimuli=1)
    x = np.arange(6 * 3 * 20, dtype=np.float32).reshape(6, 3, 4, 5)
    io.add_states(hdf5["states"], x, 0, 6)
    hdf5.close()
    got = io.load(path, 1, 6, 2)
    assert len(got) == 2  # states, stimuli (name order)
    np.testing.assert_array_equal(got[0], x[1:6:2])
    assert got[1].shape == (0, 4, 5)


def test_random_trees_round_trip(tmp_path):
    """Seeded random trees of groups and datasets (names, dtypes, shapes, nesting) read back
    exactly, and every file passes the structure walk."""
    rng = np.random.default_rng(2024)
    dtypes = [np.float32, np.float64, np.int64, np.int32, np.int16, np.uint8, np.uint32]
    for case in range(12):
        p = tmp_path / f"r{case}.h5"
        want = {}
        with h5.File(p, "w") as f:
            for k in range(int(rng.integers(1, 40))):
                depth = int(rng.integers(0, 3))
                parts = [f"g{int(rng.integers(0, 4))}" for _ in range(depth)]
                name = "/".join(parts + [f"d{k}_{'z' * int(rng.integers(0, 9))}"])
                if any(name.startswith(w + "/") or w.startswith(name + "/") for w in want):
                    continue
                dt = dtypes[int(rng.integers(0, len(dtypes)))]
                shape = tuple(int(x) for x in rng.integers(0, 6, size=int(rng.integers(0, 4))))
                v = (rng.standard_normal(shape) * 100).astype(dt)
                f.create_dataset(name, data=v)
                want[name] = v
        raw = _raw(p)
        _, root, _, _, bt, hp = struct.unpack_from("<QQIIQQ", raw, 56)
        todo = [(root, (bt, hp))]
        while todo:  # every group of the tree, its cached B-tree and heap checked
            hdr, cached = todo.pop()
            for _, (child, cache, scratch) in _walk_group(raw, hdr, cached=cached).items():
                if cache == 1:
                    todo.append((child, scratch))
        with h5.File(p) as f:
            for name, v in want.items():
                got = f[name][()]
                assert np.asarray(got).dtype == v.dtype and np.array_equal(got, v), name
