"""BlockSparse storage in HDF5 files (NDTensors/ext/NDTensorsHDF5Ext/blocksparse.jl:5-72).

- The reader is pinned to an HDF5 file written by the reference through libhdf5:
  test/base/utils/testfilev0.1.41.h5 (copied to tests/golden/itensor_v0.1.41_dense.h5),
  an ITensor with indices of dimensions 2, 3, 4 and Dense{Float64} storage; the
  reference's own test asks that its ITensor group hold a `store` key
  (test/base/test_readwrite.jl:182-190).
- The writer's attribute, link, group-info, datatype and dataspace messages are byte-equal
  to the ones libhdf5 wrote in that file for the same content.
- BlockSparse write -> read is bit-exact, with the reference's layout: group attributes
  type = "BlockSparse{Float64}", version = 1; datasets ndims, data, offsets (block numbers
  then offset per block, blocksparse.jl:5-33).
- Groups held in a symbol table (B-tree, symbol-table node, local heap) are read too.
- A GPU test writes a device tensor and loads it back onto the device.
No libhdf5 exists in this image or on the GPU machine, so files written here are read by
this reader only.
"""
import struct
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).parent / "golden" / "itensor_v0.1.41_dense.h5"


def _h5():
    from ndtensors_gb300 import hdf5io
    return hdf5io


def test_reads_reference_file():
    h = _h5()
    f = h.H5Reader(GOLDEN)
    assert f.keys("/") == ["ITensorv0.1.41"]
    top = "ITensorv0.1.41"
    assert "store" in f.keys(top)                               # test_readwrite.jl:188
    assert f.attributes(top) == {"type": "ITensor", "version": 1}
    assert f.attributes(f"{top}/store") == {"type": "Dense{Float64}", "version": 1}
    assert f.attributes(f"{top}/inds") == {"type": "IndexSet", "version": 1}
    assert f.read(f"{top}/inds/length") == 3
    dims, tags = [], []
    for k in range(1, 4):
        ix = f"{top}/inds/index_{k}"
        assert f.attributes(ix)["type"] == "Index"
        dims.append(f.read(f"{ix}/dim"))
        tags.append(f.read(f"{ix}/tags/tags"))
        assert f.read(f"{ix}/plev") == 0
    assert dims == [2, 3, 4] and tags == ["i", "j", "k"]
    data = f.read(f"{top}/store/data")
    assert data.dtype == np.float64 and data.shape == (24,) and np.all(np.isfinite(data))


def _fixture_messages(path):
    h = _h5()
    r = h._Reader(GOLDEN)
    return r.messages(r.lookup(path))


def test_writer_messages_match_libhdf5():
    h = _h5()
    top = _fixture_messages("ITensorv0.1.41")
    attrs = [d for t, d in top if t == h.MSG_ATTR]
    mine = [h._attr_msg("type", "ITensor")[8:], h._attr_msg("version", np.int64(1))[8:]]
    assert sorted(attrs) == sorted(mine)
    # link info and group info of a compact group, and a link message
    linfo = [d for t, d in top if t == h.MSG_LINKINFO][0]
    ginfo = [d for t, d in top if t == h.MSG_GROUPINFO][0]
    w = h._Writer()
    g = w.group({"inds": 0x1234})
    mg = h._Reader.__new__(h._Reader)
    mg.b = bytes(w.buf)
    msgs = mg.messages(g)
    assert [d for t, d in msgs if t == h.MSG_LINKINFO][0] == linfo
    assert [d for t, d in msgs if t == h.MSG_GROUPINFO][0] == ginfo
    root = _fixture_messages("/")
    link = [d for t, d in root if t == h.MSG_LINK][0]
    r = h._Reader(GOLDEN)
    target = r.lookup("ITensorv0.1.41")
    assert link.rstrip(b"\0") == h._msg(h.MSG_LINK, bytes([1, 0x10, 1, 14]) + b"ITensorv0.1.41" +
                                        struct.pack("<Q", target))[8:].rstrip(b"\0")
    # dataset messages: dataspace, datatype, fill value and layout encodings
    ds = dict((t, d) for t, d in _fixture_messages("ITensorv0.1.41/store/data"))
    assert ds[h.MSG_DATASPACE] == h._dataspace_bytes((24,))
    assert ds[h.MSG_DATATYPE][:20] == h._dt_bytes(np.zeros(24))[0]
    assert ds[h.MSG_FILL] == bytes([2, 2, 2, 1]) + struct.pack("<I", 0)
    assert ds[h.MSG_LAYOUT][:2] == bytes([3, 1])
    sc = dict((t, d) for t, d in _fixture_messages("ITensorv0.1.41/inds/length"))
    assert sc[h.MSG_DATASPACE] == h._dataspace_bytes(())
    assert sc[h.MSG_DATATYPE][:12] == h._dt_bytes(np.int64(3))[0]


def test_blocksparse_round_trip(tmp_path):
    h = _h5()
    rng = np.random.default_rng(7)
    inds = [(3, 4, 2), (5, 1), (2, 6, 3)]
    blocks = [(1, 1, 2), (2, 2, 1), (3, 1, 3), (1, 2, 1)]
    offs, n = [], 0
    for b in blocks:
        offs.append(n)
        n += inds[0][b[0] - 1] * inds[1][b[1] - 1] * inds[2][b[2] - 1]
    data = rng.standard_normal(n)
    data[3] = -0.0
    data[5] = 2.0 ** -1070                                      # subnormal
    p = tmp_path / "bs.h5"
    h.write_blocksparse(p, "T", blocks, offs, data)
    b2, o2, d2 = h.read_blocksparse(p, "T")
    assert b2 == blocks and o2 == offs
    assert d2.tobytes() == data.tobytes()                         # bit-exact, signs of zero kept
    f = h.H5Reader(p)
    assert f.keys("/") == ["T"] and f.keys("T") == ["data", "ndims", "offsets"]
    assert f.attributes("T") == {"type": "BlockSparse{Float64}", "version": 1}
    assert f.read("T/ndims") == 3
    np.testing.assert_array_equal(f.read("T/offsets"), h.offsets_to_array(blocks, offs))
    # the offsets layout of blocksparse.jl:5-19: N block numbers then the offset, per block
    assert list(f.read("T/offsets")[:4]) == [1, 1, 2, 0]
    # empty storage
    h.write_blocksparse(tmp_path / "e.h5", "E", [], [], np.zeros(0), ndims=2)
    assert h.read_blocksparse(tmp_path / "e.h5", "E")[0] == []


def test_multidimensional_dataset(tmp_path):
    """Row-major data with the file's dims (a column-major writer lists them reversed)."""
    h = _h5()
    a = np.arange(24, dtype=np.float64).reshape(2, 3, 4) * 0.5
    w = h._Writer()
    root = w.group({"a": w.dataset(a), "s": w.dataset("text"), "i": w.dataset(np.int64(-7))})
    p = tmp_path / "nd.h5"
    p.write_bytes(w.finish(root))
    f = h.H5Reader(p)
    np.testing.assert_array_equal(f.read("a"), a)
    assert f.read("s") == "text" and f.read("i") == -7


def test_read_rejects_other_storage(tmp_path):
    h = _h5()
    with pytest.raises(h.HDF5FormatError):
        h.read_blocksparse(GOLDEN, "ITensorv0.1.41/store")         # Dense{Float64}, not BlockSparse
    p = tmp_path / "junk.h5"
    p.write_bytes(b"not an hdf5 file at all" * 8)
    with pytest.raises(h.HDF5FormatError):
        h.H5Reader(p)


def test_reads_symbol_table_groups(tmp_path):
    """A root group held in a symbol table: v1 B-tree (one leaf), symbol-table node and
    local heap, the structure of libhdf5's original group format."""
    h = _h5()
    w = h._Writer()
    dset = w.dataset(np.arange(5, dtype=np.float64))
    names = b"\0" * 8 + b"vec\0".ljust(8, b"\0")                 # "" at 0, "vec" at 8
    heap_data = w._alloc(names + b"\0" * 16)
    heap = w._alloc(b"HEAP" + bytes(4) + struct.pack("<QQQ", len(names) + 16, 1, heap_data))
    snod = w._alloc(b"SNOD" + bytes([1, 0]) + struct.pack("<H", 1) +
                    struct.pack("<QQII", 8, dset, 0, 0) + bytes(16) + bytes(40 * 7))
    btree = w._alloc(b"TREE" + bytes([0, 0]) + struct.pack("<H", 1) + struct.pack("<QQ", h.UNDEF, h.UNDEF) +
                     struct.pack("<QQQ", 0, snod, 8) + bytes(544 - 48))
    root = w._object_header([h._msg(h.MSG_STAB, struct.pack("<QQ", btree, heap))])
    p = tmp_path / "stab.h5"
    p.write_bytes(w.finish(root))
    f = h.H5Reader(p)
    assert f.keys("/") == ["vec"]
    np.testing.assert_array_equal(f.read("vec"), np.arange(5, dtype=np.float64))


@pytest.mark.gpu
def test_save_load_device_tensor(nd, tmp_path):
    from oracle import blocksparse as obs
    from oracle import dense as odense
    from oracle import networks
    A, B, _ = networks.qn_pair(256, seed=31)
    T = nd.BlockSparseTensor.from_oracle(A)
    p = tmp_path / "qn.h5"
    nd.save_blocksparse(p, "A", T)
    R = nd.load_blocksparse(p, "A", T.inds)
    assert R.blocks == T.blocks and R.offsets == T.offsets
    assert R.data.device.type == "cuda"
    assert R.data_numpy().tobytes() == T.data_numpy().tobytes()
    # the loaded tensor contracts like the original
    la, lb, lr = (1, 2, -1), (-1, 3, 4), (1, 2, 3, 4)
    ref, _ = obs.contract(A, la, B, lb, lr)
    out = nd.contract(R, la, nd.BlockSparseTensor.from_oracle(B), lb, lr)
    assert out.blocks == [tuple(b) for b in ref.blocks] and out.offsets == list(ref.offsets)
    assert odense.rel_frobenius_error(out.data_numpy(), ref.data) <= 1e-13
