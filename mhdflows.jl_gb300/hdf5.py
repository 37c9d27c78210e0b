"""A small HDF5 writer and reader for the checkpoint files of savefile / Restart / readMHDFlows.

The reference writes its checkpoints with HDF5.jl (src/integrator.jl:259-288) and reads them
back in Restart! (src/integrator.jl:208-258) and readMHDFlows (src/utils/IC.jl:245-257): one file
per snapshot holding the datasets i_velocity, j_velocity, k_velocity, i_mag_field, j_mag_field,
k_mag_field (Float32, Julia (nx, ny, nz)) and the scalar time.  No HDF5 library exists on this
system, so this module writes and reads those files directly from the published HDF5 file format
specification, using its oldest object formats, which every HDF5 library reads and which
libhdf5 itself writes by default:

* superblock version 0 (8-byte offsets and lengths, group K values 4 / 16);
* the root group as an "old-style" group: a version-1 object header with a symbol table
  message, a version-1 B-tree of group nodes, one symbol table node, and a local heap of names;
* each dataset as a version-1 object header with a dataspace (version 1; rank 0 for the scalar
  time), a little-endian IEEE float datatype, a fill value message (version 2, undefined) and a
  contiguous data layout message (version 3), followed by its raw data.

A Julia (nx, ny, nz) column-major array is stored with HDF5 dimensions (nz, ny, nx) and the same
bytes, which is what HDF5.jl writes, so ``read(f, "i_velocity")`` returns (nx, ny, nz) there.

The reader follows the same structures and also accepts what libhdf5 adds to such files with
default settings (object header continuation messages, modification times and other messages it
skips, B-trees of more than one level, several symbol table nodes).  Files written with the
newer object formats (superblock 2 / 3, version-2 object headers, link messages) are not read.
"""
from __future__ import annotations

import struct

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
LEAF_K = 4        # symbol table node capacity is 2 * LEAF_K entries
INTERNAL_K = 16   # group B-tree nodes hold up to 2 * INTERNAL_K children
FREE_NULL = 1     # "no free block" in a local heap's free-list head (what libhdf5 writes)

MSG_NIL, MSG_DATASPACE, MSG_DATATYPE, MSG_FILL_NEW, MSG_LAYOUT = 0x0000, 0x0001, 0x0003, 0x0005, 0x0008
MSG_CONTINUATION, MSG_SYMBOL_TABLE = 0x0010, 0x0011


def _pad8(n: int) -> int:
    return (n + 7) // 8 * 8


def _message(mtype: int, body: bytes, flags: int = 0) -> bytes:
    body = body + b"\0" * (_pad8(len(body)) - len(body))
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _object_header(messages) -> bytes:
    data = b"".join(messages)
    return struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(data)) + data


def _dataspace(shape) -> bytes:
    return struct.pack("<BBBB4x", 1, len(shape), 0, 0) + b"".join(struct.pack("<Q", d) for d in shape)


def _float_type(dtype) -> bytes:
    dt = np.dtype(dtype)
    if dt == np.float32:
        size, prec, eloc, esize, msize, bias = 4, 32, 23, 8, 23, 127
    elif dt == np.float64:
        size, prec, eloc, esize, msize, bias = 8, 64, 52, 11, 52, 1023
    else:
        raise TypeError(f"only float32 / float64 datasets are written, not {dt}")
    # class 1 (floating point), version 1; little endian, implied-msb mantissa normalisation,
    # sign bit at the top
    bits = bytes([0x20, prec - 1, 0])
    return bytes([0x11]) + bits + struct.pack("<I", size) + struct.pack("<HHBBBBI", 0, prec, eloc, esize, 0, msize, bias)


def _fill_value() -> bytes:
    # version 2: allocation time early, fill time "if set", no fill value defined
    return struct.pack("<BBBB", 2, 1, 2, 0)


def _layout(addr: int, size: int) -> bytes:
    return struct.pack("<BBQQ", 3, 1, addr, size)


def _dataset_header(shape, dtype, addr, size) -> bytes:
    return _object_header([
        _message(MSG_DATASPACE, _dataspace(shape)),
        _message(MSG_DATATYPE, _float_type(dtype), flags=1),
        _message(MSG_FILL_NEW, _fill_value()),
        _message(MSG_LAYOUT, _layout(addr, size)),
    ])


def write(path: str, datasets: dict) -> None:
    """Write ``datasets`` ({name: numpy array or scalar}) into a new HDF5 file at ``path``.

    Arrays are written with HDF5 dimensions equal to their numpy shape in C order; pass
    ``np.asarray(julia_like).T`` to store a Fortran-ordered (nx, ny, nz) array the way HDF5.jl
    does.  Scalars become rank-0 datasets.  At most 2 * LEAF_K = 8 datasets (one symbol table node).
    """
    names = sorted(datasets)  # symbol table nodes hold their entries in name order
    if not 0 < len(names) <= 2 * LEAF_K:
        raise ValueError(f"between 1 and {2 * LEAF_K} datasets per file")
    arrays = {}
    for nm in names:
        v = datasets[nm]
        a = np.asarray(v, dtype=np.float64) if isinstance(v, float) else np.asarray(v)
        if a.dtype not in (np.float32, np.float64):
            raise TypeError(f"dataset {nm!r}: only float32 / float64 data is written, not {a.dtype}")
        arrays[nm] = a.copy(order="C")  # keeps rank 0 for scalars

    # local heap: "" at offset 0, then the names, each NUL-terminated and padded to 8 bytes
    heap_data = bytearray(b"\0" * 8)
    name_off = {}
    for nm in names:
        name_off[nm] = len(heap_data)
        raw = nm.encode("ascii") + b"\0"
        heap_data += raw + b"\0" * (_pad8(len(raw)) - len(raw))

    sb_size = 96
    root_oh = _object_header([_message(MSG_SYMBOL_TABLE, b"\0" * 16)])  # addresses patched below
    root_addr = sb_size
    heap_addr = root_addr + len(root_oh)
    heap_data_addr = heap_addr + 32
    btree_addr = heap_data_addr + len(heap_data)
    btree_size = 24 + 2 * INTERNAL_K * 8 + (2 * INTERNAL_K + 1) * 8
    snod_addr = btree_addr + btree_size
    snod_size = 8 + 2 * LEAF_K * 40
    pos = snod_addr + snod_size
    oh_addr, oh_size = {}, {}
    for nm in names:
        a = arrays[nm]
        oh_addr[nm] = pos
        oh_size[nm] = len(_dataset_header(a.shape, a.dtype, 0, 0))
        pos += oh_size[nm]
    data_addr = {}
    for nm in names:
        pos = _pad8(pos)
        data_addr[nm] = pos
        pos += arrays[nm].nbytes
    eof = pos

    out = bytearray(eof)
    # superblock version 0 with the root group's symbol table entry (cache type 1: the scratch pad
    # holds the B-tree and heap addresses)
    sb = SIGNATURE + struct.pack("<BBBBBBBB", 0, 0, 0, 0, 0, 8, 8, 0) + struct.pack("<HHI", LEAF_K, INTERNAL_K, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
    sb += struct.pack("<QQII", 0, root_addr, 1, 0) + struct.pack("<QQ", btree_addr, heap_addr)
    assert len(sb) == sb_size
    out[0:sb_size] = sb
    root_oh = _object_header([_message(MSG_SYMBOL_TABLE, struct.pack("<QQ", btree_addr, heap_addr))])
    out[root_addr:root_addr + len(root_oh)] = root_oh
    out[heap_addr:heap_addr + 32] = b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap_data), FREE_NULL, heap_data_addr)
    out[heap_data_addr:heap_data_addr + len(heap_data)] = heap_data
    # one leaf B-tree node with one child: keys are heap offsets of names; key 0 is the empty
    # string and key 1 the last (largest) name of the child
    bt = b"TREE" + struct.pack("<BBHQQ", 0, 0, 1, UNDEF, UNDEF)
    bt += struct.pack("<QQQ", 0, snod_addr, name_off[names[-1]])
    out[btree_addr:btree_addr + len(bt)] = bt
    sn = b"SNOD" + struct.pack("<BBH", 1, 0, len(names))
    for nm in names:
        sn += struct.pack("<QQII16x", name_off[nm], oh_addr[nm], 0, 0)
    out[snod_addr:snod_addr + len(sn)] = sn
    for nm in names:
        a = arrays[nm]
        oh = _dataset_header(a.shape, a.dtype, data_addr[nm], a.nbytes)
        assert len(oh) == oh_size[nm]
        out[oh_addr[nm]:oh_addr[nm] + len(oh)] = oh
        out[data_addr[nm]:data_addr[nm] + a.nbytes] = a.tobytes()
    with open(path, "wb") as f:
        f.write(out)


class _Reader:
    def __init__(self, buf: bytes):
        self.b = buf
        if buf[:8] != SIGNATURE:
            raise ValueError("not an HDF5 file (signature)")
        ver = buf[8]
        if ver not in (0, 1):
            raise ValueError(f"HDF5 superblock version {ver} is not supported (only 0 and 1)")
        so, sl = buf[13], buf[14]
        if so != 8 or sl != 8:
            raise ValueError("only 8-byte offsets and lengths are supported")
        p = 24 + (4 if ver == 1 else 0)
        self.base = struct.unpack_from("<Q", buf, p)[0]
        p += 32  # base, free space, end of file, driver block
        # root symbol table entry: link name offset, object header address, cache, reserved, scratch
        self.root = struct.unpack_from("<Q", buf, p + 8)[0]

    def addr(self, a: int) -> int:
        return self.base + a

    def messages(self, oh: int):
        """(type, body) of every message of a version-1 object header, continuations included."""
        b = self.b
        p = self.addr(oh)
        if b[p] != 1:
            raise ValueError(f"object header version {b[p]} is not supported (only 1)")
        nmsg, _, size = struct.unpack_from("<HII", b, p + 2)
        chunks = [(p + 16, size)]
        out = []
        while chunks and len(out) < nmsg:
            start, size = chunks.pop(0)
            q = start
            while q + 8 <= start + size and len(out) < nmsg:
                mtype, msize, _flags = struct.unpack_from("<HHB", b, q)
                body = b[q + 8:q + 8 + msize]
                out.append((mtype, body))
                if mtype == MSG_CONTINUATION:
                    caddr, clen = struct.unpack_from("<QQ", body, 0)
                    chunks.append((self.addr(caddr), clen))
                q += 8 + msize
        return out

    def group_entries(self, oh: int):
        """{name: object header address} of an old-style group."""
        stab = [body for t, body in self.messages(oh) if t == MSG_SYMBOL_TABLE]
        if not stab:
            raise ValueError("group without a symbol table message (new-style groups are not supported)")
        btree, heap = struct.unpack_from("<QQ", stab[0], 0)
        hp = self.addr(heap)
        if self.b[hp:hp + 4] != b"HEAP":
            raise ValueError("bad local heap signature")
        dsize, _free, daddr = struct.unpack_from("<QQQ", self.b, hp + 8)
        heap_data = self.b[self.addr(daddr):self.addr(daddr) + dsize]
        out = {}
        self._walk(btree, heap_data, out)
        return out

    def _walk(self, node: int, heap_data: bytes, out: dict):
        b = self.b
        p = self.addr(node)
        if b[p:p + 4] == b"SNOD":
            nsym = struct.unpack_from("<H", b, p + 6)[0]
            for i in range(nsym):
                off, oh = struct.unpack_from("<QQ", b, p + 8 + 40 * i)
                name = heap_data[off:heap_data.index(b"\0", off)].decode("ascii")
                out[name] = oh
            return
        if b[p:p + 4] != b"TREE":
            raise ValueError("bad B-tree node signature")
        ntype, _level, used = struct.unpack_from("<BBH", b, p + 4)
        if ntype != 0:
            raise ValueError("not a group B-tree")
        q = p + 24
        for i in range(used):
            child = struct.unpack_from("<Q", b, q + 8 + 16 * i)[0]
            self._walk(child, heap_data, out)

    def dataset(self, oh: int):
        shape, dtype, layout = None, None, None
        for t, body in self.messages(oh):
            if t == MSG_DATASPACE:
                ver, rank, flags = body[0], body[1], body[2]
                off = 8 if ver == 1 else 4
                shape = tuple(struct.unpack_from("<%dQ" % rank, body, off)) if rank else ()
            elif t == MSG_DATATYPE:
                cls, ver = body[0] & 0x0F, body[0] >> 4
                size = struct.unpack_from("<I", body, 4)[0]
                if cls != 1 or (body[1] & 1):
                    raise ValueError("only little-endian floating-point datasets are supported")
                dtype = {4: np.float32, 8: np.float64}[size]
            elif t == MSG_LAYOUT:
                if body[0] != 3:
                    raise ValueError(f"data layout message version {body[0]} is not supported (only 3)")
                cls = body[1]
                if cls == 1:
                    layout = ("contiguous",) + struct.unpack_from("<QQ", body, 2)
                elif cls == 0:
                    n = struct.unpack_from("<H", body, 2)[0]
                    layout = ("compact", bytes(body[4:4 + n]))
                else:
                    raise ValueError("chunked datasets are not supported")
        if shape is None or dtype is None or layout is None:
            raise ValueError("dataset without dataspace, datatype or layout")
        count = int(np.prod(shape)) if shape else 1
        if layout[0] == "contiguous":
            a = self.addr(layout[1])
            raw = self.b[a:a + count * np.dtype(dtype).itemsize]
        else:
            raw = layout[1]
        arr = np.frombuffer(raw, dtype=dtype, count=count).reshape(shape)
        return arr.copy()


def read(path: str, names=None) -> dict:
    """{name: array} of the root group's datasets (all of them, or ``names``); HDF5 dimension
    order (C order), rank-0 datasets as numpy scalars."""
    with open(path, "rb") as f:
        buf = f.read()
    r = _Reader(buf)
    entries = r.group_entries(r.root)
    want = entries if names is None else {n: entries[n] for n in names}
    out = {}
    for nm, oh in want.items():
        a = r.dataset(oh)
        out[nm] = a[()] if a.ndim == 0 else a
    return out
