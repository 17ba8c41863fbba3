"""BlockSparse storage in HDF5 files, without an HDF5 library.

Replaces NDTensors' HDF5 extension for BlockSparse storage
(NDTensors/ext/NDTensorsHDF5Ext/blocksparse.jl:5-72): a group with attributes
``type = "BlockSparse{Float64}"`` and ``version = 1`` and three datasets, ``ndims``
(Int64 scalar), ``offsets`` (Int64, per block its N block numbers then its element
offset, blocksparse.jl:5-19) and ``data`` (Float64, the flat storage).

No HDF5 library is available here, so this module reads and writes the subset of the
published HDF5 file format (File Format Specification, version 0 superblock) that
the reference's writer produces through libhdf5 with its default settings:

* superblock version 0 (offsets and lengths of 8 bytes);
* version 1 object headers, with continuation blocks;
* groups whose members are compact link messages (link info + group info + link
  messages in the group's object header), as in the reference's own test file
  ``test/base/utils/testfilev0.1.41.h5``; groups held in a symbol table (v1 B-tree,
  symbol-table nodes, local heap) are read as well;
* datasets with contiguous or compact layout (no filters), of fixed-size little-endian
  integers, IEEE floats or fixed-length strings, and attributes (message versions
  1-3) of those types.

Files written here use exactly those structures: a version 0 superblock, version 1
object headers, compact-link groups and contiguous datasets.  The reader is checked
against the reference's test file; files written here are read back by the same
reader (no libhdf5 in this image or on the GPU machine to read them independently).
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b"\x89HDF\r\n\x1a\n"

# object header message types
MSG_NIL, MSG_DATASPACE, MSG_LINKINFO, MSG_DATATYPE, MSG_FILL_OLD, MSG_FILL = 0x0, 0x1, 0x2, 0x3, 0x4, 0x5
MSG_LINK, MSG_LAYOUT, MSG_GROUPINFO, MSG_FILTERS, MSG_ATTR = 0x6, 0x8, 0xA, 0xB, 0xC
MSG_CONT, MSG_STAB, MSG_MTIME = 0x10, 0x11, 0x12


class HDF5FormatError(ValueError):
    pass


def _pad8(n: int) -> int:
    return (n + 7) & ~7


# ---------------------------------------------------------------------------
# reading
# ---------------------------------------------------------------------------

class _Reader:
    def __init__(self, path):
        self.b = Path(path).read_bytes()
        b = self.b
        if b[:8] != SIGNATURE:
            raise HDF5FormatError("not an HDF5 file (signature)")
        ver = b[8]
        if ver in (0, 1):
            self.so, self.sl = b[13], b[14]
            p = 24 + (4 if ver == 1 else 0)
            p += 4 * self.so                            # base, free space, end of file, driver info
            self.root = self._off(p + self.so)          # root symbol table entry: name offset, header address
        elif ver in (2, 3):
            self.so, self.sl = b[9], b[10]
            self.root = self._off(12 + 3 * self.so)
        else:
            raise HDF5FormatError(f"superblock version {ver} not supported")
        if self.so != 8 or self.sl != 8:
            raise HDF5FormatError("only 8-byte offsets and lengths are supported")

    def _off(self, p):
        return struct.unpack_from("<Q", self.b, p)[0]

    def messages(self, addr):
        """(type, payload bytes) of every message of the object header at addr."""
        b = self.b
        if b[addr:addr + 4] == b"OHDR":
            raise HDF5FormatError("version 2 object headers are not supported")
        if b[addr] != 1:
            raise HDF5FormatError(f"object header version {b[addr]} at {addr}")
        size = struct.unpack_from("<I", b, addr + 8)[0]
        blocks, out = [(addr + 16, size)], []
        while blocks:
            p, n = blocks.pop(0)
            end = p + n
            while p + 8 <= end:
                t, s = struct.unpack_from("<HH", b, p)
                data = b[p + 8:p + 8 + s]
                if t == MSG_CONT:
                    blocks.append((struct.unpack_from("<Q", data, 0)[0], struct.unpack_from("<Q", data, 8)[0]))
                elif t != MSG_NIL:
                    out.append((t, data))
                p += 8 + s
        return out

    # -- groups ------------------------------------------------------------
    def members(self, addr):
        """{name: object header address} of the group at addr."""
        out = {}
        for t, d in self.messages(addr):
            if t == MSG_LINK:
                name, target = self._link(d)
                if target is not None:
                    out[name] = target
            elif t == MSG_STAB:
                btree, heap = struct.unpack_from("<QQ", d, 0)
                out.update(self._symbol_table(btree, heap))
            elif t == MSG_LINKINFO:
                fheap = struct.unpack_from("<Q", d, 2 + (8 if d[1] & 1 else 0))[0]
                if fheap != UNDEF:
                    raise HDF5FormatError("groups with dense link storage are not supported")
        return out

    def _link(self, d):
        if d[0] != 1:
            raise HDF5FormatError(f"link message version {d[0]}")
        flags, p = d[1], 2
        ltype = 0
        if flags & 0x8:
            ltype = d[p]; p += 1
        if flags & 0x4:
            p += 8                                      # creation order
        if flags & 0x10:
            p += 1                                      # name character set
        nlen_size = 1 << (flags & 3)
        nlen = int.from_bytes(d[p:p + nlen_size], "little"); p += nlen_size
        name = d[p:p + nlen].decode("utf-8"); p += nlen
        if ltype != 0:
            return name, None                           # soft / external links are not followed
        return name, struct.unpack_from("<Q", d, p)[0]

    def _heap_string(self, heap, off):
        b = self.b
        if b[heap:heap + 4] != b"HEAP":
            raise HDF5FormatError("local heap signature")
        data = struct.unpack_from("<Q", b, heap + 24)[0]
        end = b.index(b"\0", data + off)
        return b[data + off:end].decode("utf-8")

    def _symbol_table(self, btree, heap):
        b, out = self.b, {}
        if b[btree:btree + 4] != b"TREE" or b[btree + 4] != 0:
            raise HDF5FormatError("group B-tree node")
        level, used = b[btree + 5], struct.unpack_from("<H", b, btree + 6)[0]
        p = btree + 24
        for i in range(used):
            child = struct.unpack_from("<Q", b, p + 8 + 16 * i)[0]
            if level > 0:
                out.update(self._symbol_table(child, heap))
                continue
            if b[child:child + 4] != b"SNOD":
                raise HDF5FormatError("symbol table node")
            n = struct.unpack_from("<H", b, child + 6)[0]
            for e in range(n):
                q = child + 8 + 40 * e
                name_off, hdr = struct.unpack_from("<QQ", b, q)
                out[self._heap_string(heap, name_off)] = hdr
        return out

    def lookup(self, path):
        addr = self.root
        for part in [p for p in path.split("/") if p]:
            m = self.members(addr)
            if part not in m:
                raise KeyError(path)
            addr = m[part]
        return addr

    # -- datasets and attributes ----------------------------------------------
    @staticmethod
    def _dataspace(d):
        ver, rank, flags = d[0], d[1], d[2]
        if ver == 1:
            p = 8
        elif ver == 2:
            p = 4
            if d[3] == 2:
                return None                             # null dataspace
        else:
            raise HDF5FormatError(f"dataspace version {ver}")
        dims = tuple(struct.unpack_from("<Q", d, p + 8 * k)[0] for k in range(rank))
        return dims

    @staticmethod
    def _dataspace_size(d):
        ver, rank, flags = d[0], d[1], d[2]
        head = 8 if ver == 1 else 4
        return head + 8 * rank * (2 if flags & 1 else 1)

    @staticmethod
    def _datatype(d):
        """(numpy dtype or ('str', size), encoded size)."""
        cls, bits0, size = d[0] & 0x0F, d[1], struct.unpack_from("<I", d, 4)[0]
        if cls == 0:                                     # fixed point
            if bits0 & 1:
                raise HDF5FormatError("big-endian integers are not supported")
            return np.dtype(("<i" if bits0 & 8 else "<u") + str(size)), 12
        if cls == 1:                                     # floating point
            if bits0 & 1 or size not in (4, 8):
                raise HDF5FormatError("only little-endian IEEE floats are supported")
            return np.dtype("<f" + str(size)), 20
        if cls == 3:                                     # fixed-length string
            return ("str", size), 8
        raise HDF5FormatError(f"datatype class {cls} not supported")

    @staticmethod
    def _value(dt, dims, raw):
        if isinstance(dt, tuple):
            n = int(np.prod(dims)) if dims else 1
            s = [raw[i * dt[1]:(i + 1) * dt[1]].split(b"\0", 1)[0].rstrip(b" ").decode("utf-8") for i in range(n)]
            return s[0] if not dims else s
        n = int(np.prod(dims)) if dims else 1
        a = np.frombuffer(raw, dtype=dt, count=n).copy()
        if not dims:
            return a[0].item()
        # HDF5 stores row-major with the file's dims (a column-major writer such as Julia
        # lists its dims reversed); returned in the file's order, as h5py does
        return a.reshape(tuple(int(d) for d in dims))

    def attributes(self, addr):
        out = {}
        for t, d in self.messages(addr):
            if t != MSG_ATTR:
                continue
            ver = d[0]
            nsz, tsz, ssz = struct.unpack_from("<HHH", d, 2)
            p = 8 + (1 if ver == 3 else 0)
            pad = _pad8 if ver == 1 else (lambda n: n)
            name = d[p:p + nsz].split(b"\0", 1)[0].decode("utf-8"); p += pad(nsz)
            dt, _ = self._datatype(d[p:p + tsz]); p += pad(tsz)
            dims = self._dataspace(d[p:p + ssz]); p += pad(ssz)
            out[name] = self._value(dt, dims, d[p:])
        return out

    def dataset(self, addr):
        dims = dt = layout = None
        for t, d in self.messages(addr):
            if t == MSG_DATASPACE:
                dims = self._dataspace(d)
            elif t == MSG_DATATYPE:
                dt, _ = self._datatype(d)
            elif t == MSG_LAYOUT:
                layout = d
            elif t == MSG_FILTERS:
                raise HDF5FormatError("filtered (compressed) datasets are not supported")
        if layout is None or dt is None:
            raise HDF5FormatError("not a dataset")
        n = int(np.prod(dims)) if dims else 1
        esize = dt[1] if isinstance(dt, tuple) else dt.itemsize
        ver = layout[0]
        if ver == 3:
            cls = layout[1]
            if cls == 0:
                sz = struct.unpack_from("<H", layout, 2)[0]
                raw = layout[4:4 + sz]
            elif cls == 1:
                a, sz = struct.unpack_from("<QQ", layout, 2)
                raw = self.b[a:a + sz] if a != UNDEF else bytes(n * esize)
            else:
                raise HDF5FormatError("chunked datasets are not supported")
        elif ver in (1, 2):
            rank, cls = layout[1], layout[2]
            if cls == 1:
                a = struct.unpack_from("<Q", layout, 8)[0]
                raw = self.b[a:a + n * esize] if a != UNDEF else bytes(n * esize)
            elif cls == 0:
                p = 8 + 4 * rank
                sz = struct.unpack_from("<I", layout, p)[0]
                raw = layout[p + 4:p + 4 + sz]
            else:
                raise HDF5FormatError("chunked datasets are not supported")
        else:
            raise HDF5FormatError(f"layout version {ver}")
        return self._value(dt, dims, raw[:n * esize])

    def is_group(self, addr):
        return any(t in (MSG_LINKINFO, MSG_STAB, MSG_GROUPINFO) for t, _ in self.messages(addr))


class H5Reader:
    """Read-only access to groups, datasets and attributes of an HDF5 file."""

    def __init__(self, path):
        self._r = _Reader(path)

    def keys(self, group="/"):
        return sorted(self._r.members(self._r.lookup(group)))

    def is_group(self, path):
        return self._r.is_group(self._r.lookup(path))

    def attributes(self, path):
        return self._r.attributes(self._r.lookup(path))

    def read(self, path):
        return self._r.dataset(self._r.lookup(path))


# ---------------------------------------------------------------------------
# writing
# ---------------------------------------------------------------------------

def _dt_bytes(value):
    """(datatype message bytes, raw little-endian data, dims) of a value."""
    if isinstance(value, str):
        raw = value.encode("utf-8")
        size = max(len(raw), 1)
        dt = bytes([0x13, 0x10, 0, 0]) + struct.pack("<I", size)           # string, null-terminated pad, UTF-8
        return dt, raw.ljust(size, b"\0"), ()
    a = np.asarray(value)
    if a.dtype.kind in "iu":
        a = a.astype("<i8")
        dt = bytes([0x10, 0x08, 0, 0]) + struct.pack("<I", 8) + struct.pack("<HH", 0, 64)
    elif a.dtype.kind == "f":
        a = a.astype("<f8")
        dt = (bytes([0x11, 0x20, 63, 0]) + struct.pack("<I", 8) +
              struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023))
    else:
        raise TypeError(f"cannot write {a.dtype} to HDF5")
    return dt, np.ascontiguousarray(a.reshape(-1)).tobytes(), tuple(a.shape)


def _dataspace_bytes(dims):
    """Dataspace message, version 1 (rank 0 is a scalar); a simple dataspace carries its
    maximum dims (equal to the dims), as libhdf5 writes it."""
    if not dims:
        return bytes([1, 0, 0, 0, 0, 0, 0, 0])
    d = b"".join(struct.pack("<Q", int(x)) for x in dims)
    return bytes([1, len(dims), 1, 0, 0, 0, 0, 0]) + d + d


def _msg(t, payload, flags=0):
    payload = payload.ljust(_pad8(len(payload)), b"\0")
    return struct.pack("<HHB3x", t, len(payload), flags) + payload


def _attr_msg(name, value):
    dt, raw, dims = _dt_bytes(value)
    ds = _dataspace_bytes(dims)
    nm = name.encode("utf-8") + b"\0"
    head = struct.pack("<BBHHHB", 3, 0, len(nm), len(dt), len(ds), 1)   # version 3, UTF-8 name
    return _msg(MSG_ATTR, head + nm + dt + ds + raw)


class _Writer:
    def __init__(self):
        self.buf = bytearray(96)                        # superblock, written last

    def _alloc(self, data: bytes) -> int:
        a = len(self.buf)
        self.buf += data
        self.buf += b"\0" * (_pad8(len(self.buf)) - len(self.buf))
        return a

    def _object_header(self, msgs) -> int:
        body = b"".join(msgs)
        head = struct.pack("<BBHII", 1, 0, len(msgs), 1, len(body)) + b"\0" * 4
        return self._alloc(head + body)

    def dataset(self, value, attrs=None) -> int:
        dt, raw, dims = _dt_bytes(value)
        addr = self._alloc(raw) if raw else UNDEF
        msgs = [_msg(MSG_DATASPACE, _dataspace_bytes(dims)),
                _msg(MSG_DATATYPE, dt, flags=1),
                _msg(MSG_FILL, bytes([2, 2, 2, 1]) + struct.pack("<I", 0), flags=1),   # v2: late alloc, library default
                _msg(MSG_LAYOUT, bytes([3, 1]) + struct.pack("<QQ", addr, len(raw)))]
        msgs += [_attr_msg(k, v) for k, v in (attrs or {}).items()]
        return self._object_header(msgs)

    def group(self, members: dict, attrs=None) -> int:
        msgs = [_msg(MSG_LINKINFO, bytes([0, 0]) + struct.pack("<QQ", UNDEF, UNDEF)),
                _msg(MSG_GROUPINFO, bytes([0, 0]), flags=1)]
        for name, addr in members.items():
            nm = name.encode("utf-8")
            if len(nm) > 255:
                raise ValueError("link names longer than 255 bytes are not supported")
            msgs.append(_msg(MSG_LINK, bytes([1, 0x10, 1, len(nm)]) + nm + struct.pack("<Q", addr)))
        msgs += [_attr_msg(k, v) for k, v in (attrs or {}).items()]
        return self._object_header(msgs)

    def finish(self, root: int) -> bytes:
        eof = len(self.buf)
        sb = (SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0) +
              struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF) +
              struct.pack("<QQII", 0, root, 0, 0) + b"\0" * 16)      # root entry: no cached symbol table
        assert len(sb) == 96
        self.buf[:96] = sb
        return bytes(self.buf)


# ---------------------------------------------------------------------------
# BlockSparse storage (NDTensors/ext/NDTensorsHDF5Ext/blocksparse.jl)
# ---------------------------------------------------------------------------

def offsets_to_array(blocks, offsets):
    """Per block its block numbers (1-based) then its element offset
    (blocksparse.jl:5-19)."""
    out = []
    for b, o in zip(blocks, offsets):
        out.extend(int(x) for x in b)
        out.append(int(o))
    return np.asarray(out, dtype=np.int64)


def array_to_offsets(a, n):
    """Inverse of offsets_to_array (blocksparse.jl:21-33)."""
    a = np.asarray(a, dtype=np.int64).reshape(-1, n + 1)
    return [tuple(int(x) for x in r[:n]) for r in a], [int(r[n]) for r in a]


def write_blocksparse(path, name, blocks, offsets, data, ndims=None):
    """Write BlockSparse storage as group `name` of a new file at `path`
    (HDF5.write(parent, name, ::BlockSparse), blocksparse.jl:35-50): attributes
    type = "BlockSparse{Float64}" and version = 1, datasets ndims, data, offsets.
    `data` is a host array or a torch tensor (copied to the host)."""
    if hasattr(data, "detach"):
        data = data.detach().cpu().numpy()
    data = np.ascontiguousarray(np.asarray(data, dtype=np.float64).reshape(-1))
    n = int(ndims if ndims is not None else (len(blocks[0]) if blocks else 0))
    w = _Writer()
    g = w.group({"ndims": w.dataset(np.int64(n)),
                 "data": w.dataset(data),
                 "offsets": w.dataset(offsets_to_array(blocks, offsets))},
                attrs={"type": "BlockSparse{Float64}", "version": np.int64(1)})
    root = w.group({name: g})
    Path(path).write_bytes(w.finish(root))


def read_blocksparse(path, name):
    """(blocks, offsets, data) of the BlockSparse storage in group `name`
    (HDF5.read(parent, name, ::Type{<:BlockSparse}), blocksparse.jl:52-72); raises if
    the group's type attribute is not BlockSparse{Float64}."""
    f = H5Reader(path)
    typ = f.attributes(name).get("type")
    if typ != "BlockSparse{Float64}":
        raise HDF5FormatError(f"HDF5 group or file does not contain BlockSparse{{Float64}} data (type {typ!r})")
    n = int(f.read(f"{name}/ndims"))
    blocks, offsets = array_to_offsets(f.read(f"{name}/offsets"), n)
    return blocks, offsets, np.asarray(f.read(f"{name}/data"), dtype=np.float64)


def save_blocksparse(path, name, T):
    """Write a BlockSparseTensor's storage (device data copied to the host) as group
    `name` of a new HDF5 file."""
    write_blocksparse(path, name, list(T.blocks), list(T.offsets), T.data, ndims=T.rank)


def load_blocksparse(path, name, inds, device=0):
    """BlockSparseTensor on `device` from the BlockSparse storage in group `name`, with
    the index block dimensions `inds` (the storage does not hold them: the reference
    rebuilds the tensor from the stored offsets and its IndexSet)."""
    import torch
    from .tensors import BlockSparseTensor, blockoffsets
    blocks, offsets, data = read_blocksparse(path, name)
    inds = [tuple(int(x) for x in i) for i in inds]
    if len(inds) != (len(blocks[0]) if blocks else len(inds)):
        raise HDF5FormatError("index count does not match the stored block rank")
    # every stored block must fit its offsets: offsets of a block list are unique
    sizes = {tuple(b): int(np.prod([inds[k][b[k] - 1] for k in range(len(b))])) for b in blocks}
    for b, o in zip(blocks, offsets):
        if o < 0 or o + sizes[tuple(b)] > data.size:
            raise HDF5FormatError(f"block {b} at offset {o} runs past the stored data")
    return BlockSparseTensor(inds, [tuple(b) for b in blocks], list(offsets),
                             torch.from_numpy(data).to(f"cuda:{device}"))
