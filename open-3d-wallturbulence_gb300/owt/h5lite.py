"""A small HDF5 writer and reader for the snapshot files, from the published
HDF5 file format specification (no HDF5 library is installed with this
package).

The reference writes each snapshot ``DATA/F-%08d.H5`` through the HDF5
library: one file, datasets in the root group, each a float64 array of shape
[NZ][NXH][NY] (src/IO.cpp:102-156, 198-235).  ``write`` produces the same
kind of file in the format the library uses for default file creation
properties:

* superblock version 0 (8-byte offsets and lengths, group leaf K 4,
  group internal K 16), the root group's symbol-table entry caching its
  B-tree and local-heap addresses;
* the root group as a version-1 object header with a symbol-table message,
  a local heap of the link names and a version-1 group B-tree with one leaf
  pointing to one symbol-table node (up to 2 x 4 links, names sorted);
* each dataset as a version-1 object header with dataspace (version 1),
  datatype (IEEE 754 binary64, little endian), fill value (version 2, none
  defined) and layout (version 3, contiguous) messages, its data stored
  contiguously after the metadata.

``read`` parses files of exactly this shape (it is the inverse used by the
tests and by ``load_instant_field``, not a general HDF5 reader).
"""
import struct

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
LEAF_K = 4       # group leaf node K: a symbol-table node holds 2K links
INTERNAL_K = 16  # group internal node K: a B-tree node holds 2K children

# header message types
MSG_DATASPACE, MSG_DATATYPE, MSG_FILL, MSG_LAYOUT, MSG_SYMBOL_TABLE = 0x0001, 0x0003, 0x0005, 0x0008, 0x0011


def _pad8(b):
    return b + b"\0" * (-len(b) % 8)


def _message(mtype, data):
    data = _pad8(data)
    return struct.pack("<HHB3x", mtype, len(data), 0) + data


def _object_header(messages):
    body = b"".join(messages)
    # version 1, reserved, message count, reference count 1, header size,
    # then 4 bytes that align the first message on 8 bytes
    return struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(body)) + body


def _f64_datatype():
    # class 1 (floating point), version 1; bit field: little endian, mantissa
    # normalisation 2 (implied leading one), sign bit 63; size 8; bit offset
    # 0, precision 64, exponent at bit 52 with 11 bits, mantissa at 0 with 52
    # bits, exponent bias 1023
    return struct.pack("<B3BI", 0x11, 0x20, 63, 0, 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)


def _dataset_header(shape, data_addr, nbytes):
    dims = struct.pack("<BBB5x", 1, len(shape), 0) + b"".join(struct.pack("<Q", d) for d in shape)
    fill = struct.pack("<BBBB", 2, 2, 2, 0)  # version 2; allocation late; write if set; no fill value
    layout = struct.pack("<BBQQ", 3, 1, data_addr, nbytes)
    return _object_header([_message(MSG_DATASPACE, dims), _message(MSG_DATATYPE, _f64_datatype()),
                           _message(MSG_FILL, fill), _message(MSG_LAYOUT, layout)])


def write(path, datasets):
    """Write {name: float64 array} as datasets of the root group of a new
    HDF5 file at ``path`` (at most 8 datasets, names of ASCII characters)."""
    names = sorted(datasets)
    if not 1 <= len(names) <= 2 * LEAF_K:
        raise ValueError("between 1 and %d datasets" % (2 * LEAF_K))
    arrays = {}
    for n in names:
        if not n or not n.isascii() or "\0" in n or "/" in n:
            raise ValueError("bad dataset name %r" % n)
        a = np.ascontiguousarray(datasets[n], dtype="<f8")
        if a.ndim == 0:
            raise ValueError("dataset %r: scalars are not supported" % n)
        arrays[n] = a

    # local heap data: "" at offset 0, then the names, each 8-byte aligned
    heap = bytearray(b"\0" * 8)
    name_off = {}
    for n in names:
        name_off[n] = len(heap)
        heap += _pad8(n.encode() + b"\0")

    SUPER = 96
    root_len = len(_object_header([_message(MSG_SYMBOL_TABLE, b"\0" * 16)]))
    root_at = SUPER
    heap_at = root_at + root_len
    heap_data_at = heap_at + 32
    btree_at = heap_data_at + len(heap)
    btree_size = 24 + (2 * INTERNAL_K + 1) * 8 + 2 * INTERNAL_K * 8
    snod_at = btree_at + btree_size
    snod_size = 8 + 2 * LEAF_K * 40
    at = snod_at + snod_size
    hdr_at = {}
    for n in names:
        hdr_at[n] = at
        at += len(_dataset_header(arrays[n].shape, 0, 0))
    data_at = {}
    for n in names:
        at += -at % 8
        data_at[n] = at
        at += arrays[n].nbytes
    eof = at

    out = bytearray(eof)
    # superblock
    sb = SIGNATURE + struct.pack("<8BHHI", 0, 0, 0, 0, 0, 8, 8, 0, LEAF_K, INTERNAL_K, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
    sb += struct.pack("<QQII", 0, root_at, 1, 0) + struct.pack("<QQ", btree_at, heap_at)
    assert len(sb) == SUPER
    out[0:SUPER] = sb
    # root group object header (symbol table message: B-tree, heap)
    root_hdr = _object_header([_message(MSG_SYMBOL_TABLE, struct.pack("<QQ", btree_at, heap_at))])
    out[root_at:root_at + len(root_hdr)] = root_hdr
    # local heap: data size, no free block, data address
    out[heap_at:heap_at + 32] = b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap), UNDEF, heap_data_at)
    out[heap_data_at:heap_data_at + len(heap)] = heap
    # group B-tree: one leaf; keys are heap offsets (0, then the last name)
    bt = b"TREE" + struct.pack("<BBHQQ", 0, 0, 1, UNDEF, UNDEF)
    bt += struct.pack("<QQQ", 0, snod_at, name_off[names[-1]])
    out[btree_at:btree_at + len(bt)] = bt
    # symbol-table node: the links in name order
    sn = b"SNOD" + struct.pack("<BBH", 1, 0, len(names))
    for n in names:
        sn += struct.pack("<QQII", name_off[n], hdr_at[n], 0, 0) + b"\0" * 16
    out[snod_at:snod_at + len(sn)] = sn
    # dataset headers and data
    for n in names:
        a = arrays[n]
        h = _dataset_header(a.shape, data_at[n], a.nbytes)
        out[hdr_at[n]:hdr_at[n] + len(h)] = h
        out[data_at[n]:data_at[n] + a.nbytes] = a.tobytes()
    with open(path, "wb") as f:
        f.write(out)
    return path


def read(path):
    """The root group's float64 datasets of a file of the shape ``write``
    produces, as {name: array}."""
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:8] != SIGNATURE:
        raise ValueError("not an HDF5 file")
    if buf[8] != 0 or buf[13] != 8 or buf[14] != 8:
        raise ValueError("superblock version 0 with 8-byte offsets and lengths expected")
    eof = struct.unpack_from("<Q", buf, 40)[0]
    if eof > len(buf):
        raise ValueError("truncated file")
    _, root_at, cache, _, btree_at, heap_at = struct.unpack_from("<QQIIQQ", buf, 56)
    if buf[heap_at:heap_at + 4] != b"HEAP":
        raise ValueError("local heap expected")
    heap_size, _, heap_data_at = struct.unpack_from("<QQQ", buf, heap_at + 8)
    heap = buf[heap_data_at:heap_data_at + heap_size]
    if buf[btree_at:btree_at + 4] != b"TREE":
        raise ValueError("group B-tree expected")
    ntype, level, used = struct.unpack_from("<BBH", buf, btree_at + 4)
    if ntype != 0 or level != 0:
        raise ValueError("one-level group B-tree expected")
    out = {}
    for c in range(used):
        snod_at = struct.unpack_from("<Q", buf, btree_at + 24 + 8 + 16 * c)[0]
        if buf[snod_at:snod_at + 4] != b"SNOD":
            raise ValueError("symbol-table node expected")
        nsym = struct.unpack_from("<H", buf, snod_at + 6)[0]
        for e in range(nsym):
            noff, hdr = struct.unpack_from("<QQ", buf, snod_at + 8 + 40 * e)
            name = heap[noff:heap.index(b"\0", noff)].decode()
            out[name] = _read_dataset(buf, hdr)
    return out


def _read_dataset(buf, at):
    version, _, nmsg, _, size = struct.unpack_from("<BBHII", buf, at)
    if version != 1:
        raise ValueError("version-1 object header expected")
    p, end = at + 16, at + 16 + size
    shape = addr = nbytes = None
    for _ in range(nmsg):
        mtype, msize = struct.unpack_from("<HH", buf, p)
        d = p + 8
        if mtype == MSG_DATASPACE:
            rank = buf[d + 1]
            shape = struct.unpack_from("<%dQ" % rank, buf, d + 8)
        elif mtype == MSG_DATATYPE:
            cls, size_t = buf[d] & 0x0F, struct.unpack_from("<I", buf, d + 4)[0]
            if cls != 1 or size_t != 8 or (buf[d + 1] & 1):
                raise ValueError("little-endian float64 expected")
        elif mtype == MSG_LAYOUT:
            if buf[d] != 3 or buf[d + 1] != 1:
                raise ValueError("contiguous layout (version 3) expected")
            addr, nbytes = struct.unpack_from("<QQ", buf, d + 2)
        p = d + msize
        if p > end:
            raise ValueError("object header overrun")
    if shape is None or addr is None:
        raise ValueError("dataspace and layout messages expected")
    return np.frombuffer(buf, dtype="<f8", count=nbytes // 8, offset=addr).reshape(shape).copy()
