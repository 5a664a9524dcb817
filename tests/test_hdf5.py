"""OPS-layout HDF5 files (opensbli_gb300.hdf5): encoding against the file format specification's
fixed structures, round trips, and the OPS block/dat attributes of
utilities/helperfunctions.py:80-127 (set_hdf5_metadata, output_hdf5)."""
import struct

import numpy as np
import pytest

from opensbli_gb300 import hdf5 as H

NAMES3 = ["rho_B0", "rhou0_B0", "rhou1_B0", "rhou2_B0", "rhoE_B0"]


def _state(npts, halo, seed=0, nv=5):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal(tuple(n + 2 * halo for n in reversed(npts))) for _ in range(nv)]


def test_round_trip_ops_state(tmp_path):
    p = tmp_path / "opensbli_output.h5"
    arrs = _state((12, 10, 8), 5)
    H.write_ops_state(str(p), NAMES3, arrs, (12, 10, 8), 5)
    out, halo, npts = H.read_ops_state(str(p), NAMES3)
    assert halo == 5 and npts == (12, 10, 8)
    for a, b in zip(arrs, out):
        assert a.shape == (18, 20, 22) and np.array_equal(a, b)


def test_ops_attributes_are_those_of_set_hdf5_metadata(tmp_path):
    p = tmp_path / "data.h5"
    arrs = _state((9, 7), 5, nv=4)
    H.write_ops_state(str(p), ["rho_B0", "rhou0_B0", "rhou1_B0", "rhoE_B0"], arrs, (9, 7), 5)
    g = H.read_file(str(p))["children"]["opensbliblock00"]
    assert g["attrs"]["ops_type"] == b"ops_block"
    assert list(g["attrs"]["dims"]) == [2] and list(g["attrs"]["index"]) == [0]
    a = g["children"]["rhoE_B0"]["attrs"]
    assert list(a["d_p"]) == [5, 5] and list(a["d_m"]) == [-5, -5] and list(a["dim"]) == [1]
    assert a["ops_type"] == b"ops_dat" and a["type"] == b"double" and a["block"] == b"opensbliblock00"
    assert list(a["block_index"]) == [0] and list(a["base"]) == [0, 0] and list(a["size"]) == [9, 7]
    assert a["d_p"].dtype == np.int32 and a["size"].dtype == np.int32


def test_datatype_encodings_match_the_standard_types():
    # H5T_IEEE_F64LE and H5T_STD_I32LE as the specification lays them out (class/version, bit
    # field, size, properties)
    assert H._dtype_message(np.float64).hex() == "11203f0008000000000040003" "40b0034ff030000"
    assert H._dtype_message(np.int32).hex() == "100800000400000000002000"
    assert H._dtype_message(np.dtype("S10")).hex() == "130100000a000000"


def test_file_structure(tmp_path):
    p = tmp_path / "s.h5"
    H.write_ops_state(str(p), NAMES3, _state((8, 8, 8), 2), (8, 8, 8), 2)
    b = p.read_bytes()
    assert b[:8] == b"\x89HDF\r\n\x1a\n"
    # superblock v0: versions 0, 8-byte offsets and lengths, K = 4 / 16, base 0, EOF = file size
    assert b[8:16] == bytes([0, 0, 0, 0, 0, 8, 8, 0])
    leaf_k, internal_k, flags = struct.unpack_from("<HHI", b, 16)
    assert (leaf_k, internal_k, flags) == (4, 16, 0)
    base, free, eof, drv = struct.unpack_from("<QQQQ", b, 24)
    assert base == 0 and free == H.UNDEF and drv == H.UNDEF and eof == len(b)
    # the root entry caches its B-tree and heap; they must be the root object's symbol table
    name_off, root, cache = struct.unpack_from("<QQI", b, 56)
    btree, heap = struct.unpack_from("<QQ", b, 80)
    assert name_off == 0 and cache == 1 and root % 8 == 0
    stab = [m for t, m in H._Reader(b).messages(root) if t == H.MSG_STAB][0]
    assert struct.unpack_from("<QQ", stab, 0) == (btree, heap)
    # local heap: version 0, free list terminated the way libhdf5 encodes it, "" at offset 0
    assert b[heap:heap + 5] == b"HEAP\0"
    size, free_head, data = struct.unpack_from("<QQQ", b, heap + 8)
    assert free_head == H.HEAP_FREE_NULL and b[data] == 0 and size % 8 == 0
    # B-tree leaf: keys bracket the child's names
    assert b[btree:btree + 4] == b"TREE"
    ntype, level, used = struct.unpack_from("<BBH", b, btree + 4)
    k0, child, k1 = struct.unpack_from("<QQQ", b, btree + 24)
    assert (ntype, level, used, k0) == (0, 0, 1, 0)
    names = b[data:data + size]
    assert names[k1:names.index(b"\0", k1)] == b"opensbliblock00"
    assert b[child:child + 5] == b"SNOD\x01"


def test_many_objects_span_several_symbol_table_nodes(tmp_path):
    rng = np.random.default_rng(3)
    dsets = {"d%03d" % i: (rng.standard_normal((3, 5)), {"i": np.array([i], np.int32)}) for i in range(41)}
    p = tmp_path / "m.h5"
    H.write_file(str(p), {"blk": (H.ops_block_attrs(2), dsets)})
    kids = H.read_file(str(p))["children"]["blk"]["children"]
    assert sorted(kids) == sorted(dsets)
    for k, (a, attrs) in dsets.items():
        assert np.array_equal(kids[k]["data"], a) and int(kids[k]["attrs"]["i"][0]) == int(attrs["i"][0])


def test_reader_rejects_other_files(tmp_path):
    p = tmp_path / "x.h5"
    p.write_bytes(b"not an hdf5 file" * 8)
    with pytest.raises(ValueError):
        H.read_file(str(p))


def test_shape_checked(tmp_path):
    with pytest.raises(ValueError):
        H.write_ops_state(str(tmp_path / "y.h5"), ["rho_B0"], [np.zeros((4, 4, 4))], (4, 4, 4), 5)
