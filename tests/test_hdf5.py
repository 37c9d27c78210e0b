"""The HDF5 checkpoint writer (mhdflows.jl_gb300/hdf5.py) on the CPU.

1. Round trip: datasets written by ``hdf5.write`` come back bit for bit through ``hdf5.read``.
2. Structure: an independent walk of the written bytes, following the HDF5 file format
   specification field by field (superblock version 0, the root group's version-1 object header
   and symbol table message, its local heap, the group B-tree node and symbol table node, each
   dataset's dataspace / datatype / fill value / layout messages and raw data), written here
   without the module's reader.
"""
import struct
from importlib import import_module

import numpy as np
import pytest

UNDEF = 0xFFFFFFFFFFFFFFFF


@pytest.fixture(scope="module")
def hdf5(pkg):
    return import_module(pkg.__name__ + ".hdf5")


def _sample():
    rng = np.random.default_rng(7)
    return {
        "i_velocity": rng.standard_normal((6, 5, 4)).astype(np.float32),
        "j_velocity": rng.standard_normal((6, 5, 4)).astype(np.float32),
        "k_velocity": rng.standard_normal((6, 5, 4)).astype(np.float32),
        "i_mag_field": rng.standard_normal((6, 5, 4)).astype(np.float32),
        "j_mag_field": rng.standard_normal((6, 5, 4)).astype(np.float32),
        "k_mag_field": rng.standard_normal((6, 5, 4)).astype(np.float32),
        "time": np.float64(1.25),
    }


def test_round_trip(hdf5, tmp_path):
    data = _sample()
    p = str(tmp_path / "run_t_0001.h5")
    hdf5.write(p, data)
    back = hdf5.read(p)
    assert set(back) == set(data)
    for k, v in data.items():
        got = back[k]
        assert np.asarray(got).dtype == np.asarray(v).dtype
        assert np.array_equal(np.asarray(got), np.asarray(v)), k
    part = hdf5.read(p, ["time", "k_velocity"])
    assert set(part) == {"time", "k_velocity"}


def test_rejects_other_formats(hdf5, tmp_path):
    p = tmp_path / "x.h5"
    p.write_bytes(b"not hdf5" * 20)
    with pytest.raises(ValueError):
        hdf5.read(str(p))
    with pytest.raises(TypeError):
        hdf5.write(str(tmp_path / "y.h5"), {"a": np.zeros(3, np.int32)})


def _messages(buf, addr):
    """Messages of a version-1 object header, parsed from the specification's layout."""
    version, reserved, nmsg, refcount, size = struct.unpack_from("<BBHII", buf, addr)
    assert (version, reserved, refcount) == (1, 0, 1)
    assert size % 8 == 0
    out, p = [], addr + 16  # the 12-byte prefix is padded to 16
    for _ in range(nmsg):
        mtype, msize, flags = struct.unpack_from("<HHB", buf, p)
        assert msize % 8 == 0 and buf[p + 5:p + 8] == b"\0\0\0"
        out.append((mtype, flags, buf[p + 8:p + 8 + msize]))
        p += 8 + msize
    assert p == addr + 16 + size
    return out


def test_structure_follows_the_specification(hdf5, tmp_path):
    data = _sample()
    p = tmp_path / "run_t_0002.h5"
    hdf5.write(str(p), data)
    buf = p.read_bytes()
    # superblock version 0
    assert buf[:8] == b"\x89HDF\r\n\x1a\n"
    assert tuple(buf[8:16]) == (0, 0, 0, 0, 0, 8, 8, 0)
    leaf_k, internal_k, flags = struct.unpack_from("<HHI", buf, 16)
    assert (leaf_k, internal_k, flags) == (4, 16, 0)
    base, freespace, eof, driver = struct.unpack_from("<QQQQ", buf, 24)
    assert base == 0 and freespace == UNDEF and driver == UNDEF and eof == len(buf)
    name0, root, cache, _res, bt_addr, heap_addr = struct.unpack_from("<QQII QQ".replace(" ", ""), buf, 56)
    assert name0 == 0 and cache == 1
    # root group: one symbol table message pointing at the same B-tree and heap
    msgs = _messages(buf, root)
    assert [m[0] for m in msgs] == [0x11]
    assert struct.unpack_from("<QQ", msgs[0][2], 0) == (bt_addr, heap_addr)
    # local heap
    assert buf[heap_addr:heap_addr + 4] == b"HEAP" and buf[heap_addr + 4] == 0
    dsize, free_head, daddr = struct.unpack_from("<QQQ", buf, heap_addr + 8)
    assert free_head == 1 or free_head < dsize  # no free block, or a block inside the segment
    heap = buf[daddr:daddr + dsize]
    assert heap[0] == 0  # offset 0 is the empty name

    def name_at(off):
        return heap[off:heap.index(b"\0", off)].decode()

    # group B-tree: a level-0 node of type 0 with one child, full size for K = 16
    assert buf[bt_addr:bt_addr + 4] == b"TREE"
    ntype, level, used, left, right = struct.unpack_from("<BBHQQ", buf, bt_addr + 4)
    assert (ntype, level, used, left, right) == (0, 0, 1, UNDEF, UNDEF)
    key0, child, key1 = struct.unpack_from("<QQQ", buf, bt_addr + 24)
    assert name_at(key0) == ""
    assert bt_addr + 24 + 2 * 16 * 8 + 33 * 8 <= len(buf)
    # symbol table node: entries in name order, the B-tree's right key is the last name
    assert buf[child:child + 4] == b"SNOD" and buf[child + 4] == 1
    nsym = struct.unpack_from("<H", buf, child + 6)[0]
    assert nsym == len(data) and child + 8 + 8 * 40 <= len(buf)
    entries = []
    for i in range(nsym):
        off, oh, ctype, _r = struct.unpack_from("<QQII", buf, child + 8 + 40 * i)
        assert ctype == 0 and buf[child + 8 + 40 * i + 24:child + 8 + 40 * i + 40] == b"\0" * 16
        entries.append((name_at(off), oh))
    names = [e[0] for e in entries]
    assert names == sorted(data) and name_at(key1) == names[-1]
    for nm, oh in entries:
        want = np.asarray(data[nm])
        types = {}
        for mtype, mflags, body in _messages(buf, oh):
            types[mtype] = (mflags, body)
        assert set(types) == {0x1, 0x3, 0x5, 0x8}
        # dataspace version 1: rank, no maximum dimensions, dims in C order
        sp = types[0x1][1]
        assert sp[0] == 1 and sp[1] == want.ndim and sp[2] == 0
        assert struct.unpack_from("<%dQ" % want.ndim, sp, 8) == want.shape
        # datatype: floating point class 1, version 1, little endian, IEEE field layout
        dt = types[0x3][1]
        assert dt[0] == 0x11 and dt[1] & 1 == 0 and (dt[1] >> 4) & 3 == 2
        size = struct.unpack_from("<I", dt, 4)[0]
        off, prec, eloc, esize, mloc, msize, bias = struct.unpack_from("<HHBBBBI", dt, 8)
        ieee = {4: (0, 32, 23, 8, 0, 23, 127), 8: (0, 64, 52, 11, 0, 52, 1023)}[size]
        assert (off, prec, eloc, esize, mloc, msize, bias) == ieee and dt[2] == prec - 1
        assert size == want.dtype.itemsize
        # fill value version 2, nothing defined
        assert types[0x5][1][0] == 2 and types[0x5][1][3] == 0
        # layout version 3, contiguous, the raw bytes
        lay = types[0x8][1]
        assert lay[0] == 3 and lay[1] == 1
        addr, nbytes = struct.unpack_from("<QQ", lay, 2)
        assert nbytes == want.nbytes and addr + nbytes <= len(buf)
        raw = np.frombuffer(buf[addr:addr + nbytes], dtype=want.dtype).reshape(want.shape)
        assert np.array_equal(raw, want), nm
