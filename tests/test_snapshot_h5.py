"""The snapshot files' HDF5 encoding (owt/h5lite.py) on the CPU: the
structures the HDF5 file format specification defines for a version-0
superblock, a symbol-table root group and contiguous float64 datasets, at
the byte offsets the writer places them, and the round trip through the
reader.  The reference's snapshot is six [NZ][NXH][NY] float64 datasets in
the root group (src/IO.cpp:198-235)."""
import struct

import numpy as np
import pytest

from owt import h5lite
from owt.snapshot import load_instant_field, save_instant_field

NAMES = ["velx_real", "velx_imag", "vely_real", "vely_imag", "velz_real", "velz_imag"]


def test_round_trip_and_layout(tmp_path):
    rng = np.random.default_rng(0)
    d = {n: rng.standard_normal((12, 7, 17)) for n in NAMES}
    path = str(tmp_path / "F-00000003.H5")
    h5lite.write(path, d)
    got = h5lite.read(path)
    assert sorted(got) == sorted(NAMES)
    for n in NAMES:
        np.testing.assert_array_equal(got[n], d[n])
        assert got[n].dtype == np.float64 and got[n].shape == (12, 7, 17)
    buf = open(path, "rb").read()
    # superblock version 0: signature, versions, 8-byte offsets/lengths,
    # K values, end-of-file address equal to the size, root entry cached
    assert buf[:8] == b"\x89HDF\r\n\x1a\n"
    assert buf[8:16] == bytes([0, 0, 0, 0, 0, 8, 8, 0])
    assert struct.unpack_from("<HH", buf, 16) == (4, 16)
    base, free, eof, drv = struct.unpack_from("<QQQQ", buf, 24)
    assert (base, free, eof, drv) == (0, h5lite.UNDEF, len(buf), h5lite.UNDEF)
    _, root, cache, _, btree, heap = struct.unpack_from("<QQIIQQ", buf, 56)
    assert cache == 1 and root == 96
    assert buf[btree:btree + 4] == b"TREE" and buf[heap:heap + 4] == b"HEAP"
    # the root group's object header holds one symbol-table message with the
    # same B-tree and heap
    ver, _, nmsg, refc, size = struct.unpack_from("<BBHII", buf, root)
    assert (ver, nmsg, refc) == (1, 1, 1)
    mtype, msize = struct.unpack_from("<HH", buf, root + 16)
    assert mtype == 0x11 and struct.unpack_from("<QQ", buf, root + 24) == (btree, heap)
    # the IEEE binary64 little-endian datatype message
    assert h5lite._f64_datatype().hex() == "1120" + "3f00" + "08000000" + "0000" + "4000" + "340b" + "0034" + "ff030000"


def test_rejects_what_it_cannot_write(tmp_path):
    with pytest.raises(ValueError):
        h5lite.write(str(tmp_path / "a.H5"), {})
    with pytest.raises(ValueError):
        h5lite.write(str(tmp_path / "b.H5"), {"a/b": np.zeros(3)})
    with pytest.raises(ValueError):
        h5lite.write(str(tmp_path / "c.H5"), {str(i): np.zeros(2) for i in range(9)})
    (tmp_path / "d.H5").write_bytes(b"not hdf5")
    with pytest.raises(ValueError):
        h5lite.read(str(tmp_path / "d.H5"))


class _Fields:
    """A stand-in for GpuSolver.get on the host."""

    def __init__(self, shape, seed):
        rng = np.random.default_rng(seed)
        self.f = {n: rng.standard_normal(shape) + 1j * rng.standard_normal(shape) for n in ("velx", "vely", "velz")}

    def get(self, name):
        return self.f[name]


def test_snapshot_file_name_and_datasets(tmp_path):
    s = _Fields((8, 5, 9), 1)
    path = save_instant_field(s, 40, directory=str(tmp_path / "DATA"))
    assert path.endswith("DATA/F-00000040.H5")
    got = load_instant_field(path)
    for n in ("velx", "vely", "velz"):
        np.testing.assert_array_equal(got[n], s.get(n))
    assert sorted(h5lite.read(path)) == sorted(NAMES)
