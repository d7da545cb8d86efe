"""The reference's HDF5 field output (src/hdf5_io.F90:1-549,
src/WriteOutput_corner1.F90:21-78), written without the HDF5 library.

Neither machine this package runs on carries libhdf5 or h5py, so this module
writes and reads the part of the HDF5 file format the reference's files use.
It follows the HDF Group's published HDF5 File Format Specification, using
the structures libhdf5 writes under its default ("earliest") format bounds:

- superblock version 0: 8-byte offsets and lengths, group leaf K 4, group
  internal K 16, base address 0;
- groups indexed by a symbol table: one version-1 B-tree node (type 0) over
  symbol-table nodes ("SNOD", 2 x leaf K entries each), with the link names
  in the group's local heap ("HEAP"); offset 0 of the heap is the empty name
  that is the B-tree's first key, and each later key is the last name of the
  child to its left;
- datasets in version-1 object headers with a dataspace (version 1), a
  datatype (IEEE little-endian FP64 or little-endian 64-bit two's-complement
  integer, the reference's H5T_NATIVE_DOUBLE and H5T_STD_I64LE), a fill-value
  message and a contiguous layout (version 3); the raw data is the Fortran
  array in memory order, so the file's dims are the array's reversed -- what
  the HDF5 Fortran API writes;
- scalars as attributes (version-1 attribute messages) of the group, as
  hdf5_write_real/int store them (src/hdf5_io.F90:341-367).

The reader covers what the writer emits and what libhdf5 writes for simple
files: a user block before the superblock, superblock versions 0 and 1,
continuation messages, layout versions 1-3 and fixed-length string
attributes.  It checks the invariants libhdf5 checks when it opens such a
file (message counts and sizes, heap and B-tree signatures, sorted names
within the B-tree's key ranges) and raises ``H5FormatError`` otherwise.
"""
from __future__ import annotations

import os
import struct
from dataclasses import dataclass, field
from pathlib import Path
from typing import Dict, Optional, Union

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF      # the undefined address
LEAF_K = 4                      # symbol-table node capacity is 2 * LEAF_K
INTERNAL_K = 16                 # B-tree node capacity is 2 * INTERNAL_K children
HEAP_FREE_NULL = 1              # end of a local heap's free list on disk

MSG_NIL, MSG_SPACE, MSG_TYPE, MSG_FILL = 0x0000, 0x0001, 0x0003, 0x0005
MSG_LAYOUT, MSG_ATTR, MSG_CONT, MSG_STAB = 0x0008, 0x000C, 0x0010, 0x0011

SNOD_BYTES = 8 + 2 * LEAF_K * 40
BTREE_BYTES = 24 + (2 * INTERNAL_K + 1) * 8 + 2 * INTERNAL_K * 8

F8 = np.dtype("<f8")
I8 = np.dtype("<i8")


class H5FormatError(ValueError):
    """A file that is not HDF5, or uses a structure this module does not read."""


def _pad8(n: int) -> int:
    return (n + 7) & ~7


# ---------------------------------------------------------------------------
# in-memory tree
# ---------------------------------------------------------------------------

@dataclass
class Dataset:
    """A dataset: file dims (C order) and element type.  ``data`` is an array
    of shape ``dims`` in C order, or None while the bytes stay in a file
    (``src``, ``addr``)."""
    dims: tuple
    dtype: np.dtype
    data: Optional[np.ndarray] = None
    src: Optional[str] = None
    addr: int = UNDEF
    attrs: Dict[str, object] = field(default_factory=dict)

    @property
    def nbytes(self) -> int:
        return int(np.prod(self.dims, dtype=np.int64)) * self.dtype.itemsize

    def read(self) -> np.ndarray:
        """The dataset as a C-ordered array of shape ``dims``."""
        if self.data is not None:
            return self.data
        n = int(np.prod(self.dims, dtype=np.int64))
        if n == 0 or self.addr == UNDEF:
            return np.zeros(self.dims, dtype=self.dtype)
        return np.fromfile(self.src, dtype=self.dtype, count=n, offset=self.addr).reshape(self.dims)


@dataclass
class Group:
    children: Dict[str, Union["Group", Dataset]] = field(default_factory=dict)
    attrs: Dict[str, object] = field(default_factory=dict)

    def find(self, path: str, create: bool = False) -> "Group":
        """The group at ``path`` ("/", "/a", "a/b"), created when asked."""
        g = self
        for part in (p for p in path.split("/") if p):
            nxt = g.children.get(part)
            if nxt is None:
                if not create:
                    raise KeyError(f"no group {path!r}")
                nxt = g.children[part] = Group()
            if not isinstance(nxt, Group):
                raise KeyError(f"{path!r}: {part!r} is a dataset")
            g = nxt
        return g


# ---------------------------------------------------------------------------
# message encoders
# ---------------------------------------------------------------------------

def _type_msg(dt: np.dtype) -> bytes:
    """Datatype message (version 1) of a little-endian number type."""
    dt = np.dtype(dt)
    if dt.kind == "f" and dt.itemsize in (4, 8):
        # class 1; bit fields: byte order LE, mantissa normalised with an
        # implied leading bit (bits 4-5 = 2), sign bit position
        w = dt.itemsize * 8
        man, exp, bias = (52, 11, 1023) if w == 64 else (23, 8, 127)
        return (struct.pack("<BBBBI", 0x11, 0x20, w - 1, 0, dt.itemsize)
                + struct.pack("<HHBBBBI", 0, w, man, exp, 0, man, bias))
    if dt.kind in "iu" and dt.itemsize in (1, 2, 4, 8):
        # class 0; bit 3 of the bit fields = two's-complement signed
        return (struct.pack("<BBBBI", 0x10, 0x08 if dt.kind == "i" else 0, 0, 0, dt.itemsize)
                + struct.pack("<HH", 0, 8 * dt.itemsize))
    raise TypeError(f"no HDF5 encoding for {dt}")


def _space_msg(dims) -> bytes:
    """Dataspace message (version 1); rank 0 is a scalar."""
    return struct.pack("<BBBBI", 1, len(dims), 0, 0, 0) + b"".join(struct.pack("<Q", int(d)) for d in dims)


# fill value message, version 1: allocation time late, fill written if set
# by the user, fill value defined with size 0 (the type's default, zero)
_FILL_MSG = bytes([1, 2, 2, 1]) + struct.pack("<I", 0)


def _layout_msg(addr: int, size: int) -> bytes:
    """Data layout message, version 3, contiguous class: address and size."""
    return struct.pack("<BBQQ", 3, 1, addr, size)


def _attr_value(value) -> np.ndarray:
    if isinstance(value, (bool, np.bool_)):
        raise TypeError("boolean attributes are not written")
    a = np.asarray(value)
    if a.ndim != 0:
        raise TypeError("only scalar attributes are written")
    if a.dtype.kind == "f":
        return a.astype(F8)
    if a.dtype.kind in "iu":
        return a.astype(I8)
    raise TypeError(f"no HDF5 encoding for attribute of type {a.dtype}")


def _attr_msg(name: str, value) -> bytes:
    """Attribute message, version 1: name, datatype and dataspace each padded
    to 8 bytes, then the value."""
    a = _attr_value(value)
    nm = name.encode() + b"\0"
    dt, sp = _type_msg(a.dtype), _space_msg(())
    return (struct.pack("<BBHHH", 1, 0, len(nm), len(dt), len(sp))
            + nm.ljust(_pad8(len(nm)), b"\0") + dt.ljust(_pad8(len(dt)), b"\0")
            + sp.ljust(_pad8(len(sp)), b"\0") + a.tobytes())


def _object_header(msgs) -> bytes:
    """Version-1 object header: 16-byte prefix (version, message count,
    reference count 1, size of the message data), then each message as type,
    size, flags and its data padded to 8 bytes."""
    body = bytearray()
    for mtype, flags, data in msgs:
        data = bytes(data).ljust(_pad8(len(data)), b"\0")
        if len(data) > 0xFFFF:
            raise ValueError("object header message too large")
        body += struct.pack("<HHB3x", mtype, len(data), flags) + data
    return struct.pack("<BBHII4x", 1, 0, len(msgs), 1, len(body)) + bytes(body)


def _entry(name_off: int, oh: int, cache: int = 0, scratch: bytes = bytes(16)) -> bytes:
    """Symbol-table entry: link name offset, object header address, cache
    type (1: the group's B-tree and heap addresses in the scratch pad)."""
    return struct.pack("<QQII", name_off, oh, cache, 0) + scratch


# ---------------------------------------------------------------------------
# writer
# ---------------------------------------------------------------------------

class _Out:
    def __init__(self, f):
        self.f = f
        self.pos = 0

    def put(self, b) -> int:
        """Append at the next 8-byte boundary; returns the address."""
        pad = _pad8(self.pos) - self.pos
        if pad:
            self.f.write(bytes(pad))
            self.pos += pad
        addr = self.pos
        mv = memoryview(b).cast("B")
        self.f.write(mv)
        self.pos += mv.nbytes
        return addr

    def here(self) -> int:
        return _pad8(self.pos)


def _emit_dataset(out: _Out, d: Dataset) -> int:
    """Raw data (little-endian, C order of the file dims), then the object header."""
    le = d.dtype.newbyteorder("<")
    n = d.nbytes
    addr = UNDEF
    if n:
        a = np.ascontiguousarray(d.read(), dtype=le)
        addr = out.put(a.reshape(-1).view(np.uint8))
    msgs = [(MSG_SPACE, 0, _space_msg(d.dims)), (MSG_TYPE, 1, _type_msg(le)),
            (MSG_FILL, 1, _FILL_MSG), (MSG_LAYOUT, 0, _layout_msg(addr, n))]
    msgs += [(MSG_ATTR, 0, _attr_msg(k, v)) for k, v in d.attrs.items()]
    return out.put(_object_header(msgs))


def _emit_group(out: _Out, g: Group):
    """Writes the children, then the group's heap, symbol-table nodes, B-tree
    node and object header; returns (object header, B-tree, heap) addresses."""
    names = sorted(g.children, key=lambda s: s.encode())
    if len(names) > 2 * LEAF_K * 2 * INTERNAL_K:
        raise ValueError(f"a group holds at most {4 * LEAF_K * INTERNAL_K} names here")
    ents = []
    for name in names:
        c = g.children[name]
        if "/" in name or not name:
            raise ValueError(f"bad link name {name!r}")
        if isinstance(c, Group):
            oh, bt, hp = _emit_group(out, c)
            ents.append((name, oh, 1, struct.pack("<QQ", bt, hp)))
        else:
            ents.append((name, _emit_dataset(out, c), 0, bytes(16)))
    # local heap: the empty name at offset 0, then each name NUL-terminated
    # and padded to 8 bytes; no free block
    seg = bytearray(8)
    off = {}
    for name in names:
        off[name] = len(seg)
        b = name.encode() + b"\0"
        seg += b.ljust(_pad8(len(b)), b"\0")
    heap_at = out.here()
    heap = b"HEAP" + bytes(4) + struct.pack("<QQQ", len(seg), HEAP_FREE_NULL, heap_at + 32) + bytes(seg)
    assert out.put(heap) == heap_at
    chunks = [ents[i:i + 2 * LEAF_K] for i in range(0, len(ents), 2 * LEAF_K)]
    snods = []
    for ch in chunks:
        b = b"SNOD" + struct.pack("<BBH", 1, 0, len(ch)) + b"".join(
            _entry(off[n], oh, cache, scr) for n, oh, cache, scr in ch)
        snods.append(out.put(b.ljust(SNOD_BYTES, b"\0")))
    keys = [0] + [off[ch[-1][0]] for ch in chunks]
    tree = b"TREE" + struct.pack("<BBH", 0, 0, len(snods)) + struct.pack("<QQ", UNDEF, UNDEF)
    for i, a in enumerate(snods):
        tree += struct.pack("<QQ", keys[i], a)
    tree += struct.pack("<Q", keys[len(snods)])
    bt = out.put(tree.ljust(BTREE_BYTES, b"\0"))
    msgs = [(MSG_STAB, 1, struct.pack("<QQ", bt, heap_at))]
    msgs += [(MSG_ATTR, 0, _attr_msg(k, v)) for k, v in g.attrs.items()]
    return out.put(_object_header(msgs)), bt, heap_at


def write_file(path, root: Group) -> None:
    """Writes the tree as a new file (through a temporary file in the same
    directory, renamed over ``path`` when complete, so datasets still held
    in the old file can be copied from it)."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    tmp = path.with_name(path.name + f".tmp{os.getpid()}")
    try:
        with open(tmp, "wb") as f:
            out = _Out(f)
            out.put(bytes(96))
            oh, bt, hp = _emit_group(out, root)
            eof = out.pos
            sb = (SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", LEAF_K, INTERNAL_K, 0)
                  + struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF) + _entry(0, oh, 1, struct.pack("<QQ", bt, hp)))
            assert len(sb) == 96
            f.seek(0)
            f.write(sb)
        os.replace(tmp, path)
    finally:
        if tmp.exists():
            tmp.unlink()


# ---------------------------------------------------------------------------
# reader
# ---------------------------------------------------------------------------

class _In:
    def __init__(self, path):
        self.path = str(path)
        self.f = open(path, "rb")
        self.size = os.fstat(self.f.fileno()).st_size
        self.base = self._superblock()

    def close(self):
        self.f.close()

    def at(self, addr: int, n: int) -> bytes:
        a = self.base + addr
        if addr == UNDEF or a + n > self.size:
            raise H5FormatError(f"read of {n} bytes at {addr:#x} past the end of the file")
        self.f.seek(a)
        return self.f.read(n)

    def _superblock(self) -> int:
        off = 0
        while off + 8 <= self.size:
            self.f.seek(off)
            if self.f.read(8) == SIGNATURE:
                break
            off = 512 if off == 0 else 2 * off
        else:
            raise H5FormatError("no HDF5 signature")
        self.f.seek(off)
        b = self.f.read(100)
        ver = b[8]
        if ver not in (0, 1):
            raise H5FormatError(f"superblock version {ver} not read here")
        if b[13] != 8 or b[14] != 8:
            raise H5FormatError("only 8-byte offsets and lengths are read here")
        self.leaf_k, self.internal_k = struct.unpack_from("<HH", b, 16)
        p = 24 + (4 if ver == 1 else 0)
        base, _free, eof, _drv = struct.unpack_from("<QQQQ", b, p)
        self.eof = eof
        p += 32
        _name, oh, cache, _r = struct.unpack_from("<QQII", b, p)
        if self.leaf_k == 0 or self.internal_k == 0:
            raise H5FormatError("zero B-tree K")
        self.root_oh = oh
        return base

    def messages(self, addr: int):
        """The messages of a version-1 object header, continuation chunks
        followed; checks the message count and that the messages fill each
        chunk exactly."""
        pre = self.at(addr, 16)
        if pre[:4] == b"OHDR":
            raise H5FormatError("version-2 object headers are not read here")
        ver, _r, nmsg, _refc, size = struct.unpack_from("<BBHII", pre)
        if ver != 1:
            raise H5FormatError(f"object header version {ver}")
        chunks = [(addr + 16, size)]
        out = []
        while chunks:
            ca, cs = chunks.pop(0)
            data = self.at(ca, cs)
            p = 0
            while p < cs:
                if p + 8 > cs:
                    raise H5FormatError("truncated message header")
                mtype, msize, flags = struct.unpack_from("<HHB", data, p)
                p += 8
                if msize % 8 or p + msize > cs:
                    raise H5FormatError("object header message misaligned or past its chunk")
                body = data[p:p + msize]
                p += msize
                if mtype == MSG_CONT:
                    chunks.append(struct.unpack_from("<QQ", body))
                out.append((mtype, flags, body))
        if len(out) != nmsg:
            raise H5FormatError(f"object header at {addr:#x}: {len(out)} messages, prefix says {nmsg}")
        return out

    def heap(self, addr: int) -> bytes:
        b = self.at(addr, 32)
        if b[:4] != b"HEAP" or b[4] != 0:
            raise H5FormatError(f"no local heap at {addr:#x}")
        dsize, free, daddr = struct.unpack_from("<QQQ", b, 8)
        if free != HEAP_FREE_NULL and free >= dsize:
            raise H5FormatError("bad heap free list")
        return self.at(daddr, dsize)

    def symbols(self, btree: int, heap: bytes):
        """(name, entry) pairs of a group's symbol table, in B-tree order."""
        def name(o):
            if o >= len(heap):
                raise H5FormatError("name offset past the heap")
            return heap[o:heap.index(b"\0", o)].decode()

        res = []

        def walk(addr, lo, hi):
            b = self.at(addr, 24)
            if b[:4] != b"TREE" or b[4] != 0:
                raise H5FormatError(f"no group B-tree node at {addr:#x}")
            level, n = b[5], struct.unpack_from("<H", b, 6)[0]
            if n > 2 * self.internal_k:
                raise H5FormatError("B-tree node over capacity")
            kc = self.at(addr + 24, (2 * n + 1) * 8)
            vals = struct.unpack(f"<{2 * n + 1}Q", kc)
            keys, kids = vals[0::2], vals[1::2]
            for i, kid in enumerate(kids):
                klo, khi = name(keys[i]), name(keys[i + 1])
                if level:
                    walk(kid, klo, khi)
                    continue
                s = self.at(kid, 8)
                if s[:4] != b"SNOD" or s[4] != 1:
                    raise H5FormatError(f"no symbol-table node at {kid:#x}")
                m = struct.unpack_from("<H", s, 6)[0]
                if m > 2 * self.leaf_k:
                    raise H5FormatError("symbol-table node over capacity")
                eb = self.at(kid + 8, 40 * m)
                for j in range(m):
                    no, oh, cache, _r = struct.unpack_from("<QQII", eb, 40 * j)
                    nm = name(no)
                    if not (klo.encode() < nm.encode() <= khi.encode()):
                        raise H5FormatError(f"name {nm!r} outside its B-tree key range")
                    if res and res[-1][0].encode() >= nm.encode():
                        raise H5FormatError("symbol-table names out of order")
                    res.append((nm, oh))

        walk(btree, "", None)
        return res


def _parse_type(b: bytes) -> np.dtype:
    cls, ver = b[0] & 0x0F, b[0] >> 4
    bits = b[1] | (b[2] << 8) | (b[3] << 16)
    size = struct.unpack_from("<I", b, 4)[0]
    order = ">" if bits & 1 else "<"
    if cls == 0:
        return np.dtype(f"{order}{'i' if bits & 8 else 'u'}{size}")
    if cls == 1 and size in (4, 8):
        return np.dtype(f"{order}f{size}")
    if cls == 3:
        return np.dtype(f"S{size}")
    raise H5FormatError(f"datatype class {cls} (version {ver}) not read here")


def _parse_space(b: bytes):
    ver, rank, flags = b[0], b[1], b[2]
    if ver == 1:
        p = 8
    elif ver == 2:
        p = 4
        if b[3] == 2:
            return None  # null dataspace
    else:
        raise H5FormatError(f"dataspace version {ver}")
    return tuple(struct.unpack_from(f"<{rank}Q", b, p)) if rank else ()


def _parse_layout(b: bytes):
    """(address, size) of a contiguous (or compact: (None, data)) layout."""
    ver = b[0]
    if ver in (1, 2):
        ndims, cls = b[1], b[2]
        p = 8
        if cls == 0:
            dims = struct.unpack_from(f"<{ndims}I", b, p)
            p += 4 * ndims
            n = struct.unpack_from("<I", b, p)[0]
            return None, b[p + 4:p + 4 + n]
        if cls != 1:
            raise H5FormatError("chunked layout not read here")
        addr = struct.unpack_from("<Q", b, p)[0]
        dims = struct.unpack_from(f"<{ndims}I", b, p + 8)
        return addr, int(np.prod(dims, dtype=np.int64))
    if ver == 3:
        cls = b[1]
        if cls == 0:
            n = struct.unpack_from("<H", b, 2)[0]
            return None, b[4:4 + n]
        if cls == 1:
            return struct.unpack_from("<QQ", b, 2)
        raise H5FormatError("chunked layout not read here")
    raise H5FormatError(f"layout version {ver} not read here")


def _parse_attr(b: bytes):
    ver = b[0]
    if ver == 1:
        nsz, tsz, ssz = struct.unpack_from("<HHH", b, 2)
        p = 8
        name = b[p:p + nsz].split(b"\0")[0].decode()
        p += _pad8(nsz)
        dt = _parse_type(b[p:p + tsz])
        p += _pad8(tsz)
        dims = _parse_space(b[p:p + ssz])
        p += _pad8(ssz)
    elif ver in (2, 3):
        nsz, tsz, ssz = struct.unpack_from("<HHH", b, 2)
        p = 8 + (1 if ver == 3 else 0)
        name = b[p:p + nsz].split(b"\0")[0].decode()
        p += nsz
        dt = _parse_type(b[p:p + tsz])
        p += tsz
        dims = _parse_space(b[p:p + ssz])
        p += ssz
    else:
        raise H5FormatError(f"attribute version {ver}")
    n = int(np.prod(dims, dtype=np.int64)) if dims else 1
    a = np.frombuffer(b, dtype=dt, count=n, offset=p)
    v = a.reshape(dims) if dims else a[0]
    if dt.kind == "S":
        return name, bytes(v).split(b"\0")[0]
    return name, (v.astype(dt.newbyteorder("=")) if dims else v.item())


def _load(r: _In, oh: int, path=()):
    if oh in path:
        raise H5FormatError(f"group at {oh:#x} links to itself")
    msgs = r.messages(oh)
    attrs = dict(_parse_attr(m[2]) for m in msgs if m[0] == MSG_ATTR)
    stab = [m for m in msgs if m[0] == MSG_STAB]
    if stab:
        bt, hp = struct.unpack_from("<QQ", stab[0][2])
        heap = r.heap(hp)
        g = Group(attrs=attrs)
        for name, child in r.symbols(bt, heap):
            g.children[name] = _load(r, child, path + (oh,))
        return g
    kinds = {m[0]: m[2] for m in msgs}
    if MSG_LAYOUT not in kinds or MSG_TYPE not in kinds or MSG_SPACE not in kinds:
        raise H5FormatError(f"object at {oh:#x} is neither a group nor a dataset")
    dt = _parse_type(kinds[MSG_TYPE])
    dims = _parse_space(kinds[MSG_SPACE]) or ()
    addr, size = _parse_layout(kinds[MSG_LAYOUT])
    d = Dataset(dims=dims, dtype=dt, attrs=attrs, src=r.path)
    nbytes = int(np.prod(dims, dtype=np.int64)) * dt.itemsize
    if addr is None:
        d.data = np.frombuffer(size, dtype=dt, count=nbytes // dt.itemsize).reshape(dims).copy()
    else:
        if addr != UNDEF and size != nbytes:
            raise H5FormatError(f"layout size {size} != {nbytes} bytes of the dataspace")
        if addr != UNDEF and r.base + addr + nbytes > r.size:
            raise H5FormatError("dataset data past the end of the file")
        d.addr = UNDEF if addr == UNDEF else r.base + addr
    return d


def read_file(path) -> Group:
    """The file's group tree; dataset bytes are read on ``Dataset.read()``."""
    r = _In(path)
    try:
        return _load(r, r.root_oh)
    except (struct.error, IndexError, UnicodeDecodeError) as e:
        raise H5FormatError(f"{path}: malformed HDF5 structure ({e})") from e
    finally:
        r.close()


# ---------------------------------------------------------------------------
# the reference's interface (src/hdf5_io.F90)
# ---------------------------------------------------------------------------

def _one_input(scalar_input, arrays):
    given = [a for a in (scalar_input, *arrays) if a is not None]
    if len(given) != 1:
        raise ValueError("More than one argument present hdf5_write" if given else "no input given to hdf5_write")


def _write(filename, dtype, scalar_input, arrays, key, group):
    _one_input(scalar_input, arrays)
    root = read_file(filename) if os.path.exists(filename) else Group()
    g = root.find(group, create=True)
    if scalar_input is not None:
        g.attrs[key] = dtype.type(scalar_input)
    else:
        rank, a = next((r, a) for r, a in enumerate(arrays, 1) if a is not None)
        a = np.asarray(a)
        if a.ndim != rank:
            raise ValueError(f"array_input_{rank}d has rank {a.ndim}")
        if dtype.kind == "i" and a.dtype.kind not in "iub":
            raise TypeError("hdf5_write_int takes integer arrays")
        # the Fortran array in memory order: the file's dims are reversed
        g.children[key] = Dataset(dims=a.shape[::-1], dtype=dtype, data=np.ascontiguousarray(a.T, dtype=dtype))
    write_file(filename, root)


def hdf5_write_real(filename, scalar_input=None, array_input_1d=None, array_input_2d=None,
                    array_input_3d=None, *, key: str, group: str) -> None:
    """hdf5_write_real (src/hdf5_io.F90:263-404): adds a FP64 scalar (as an
    attribute of ``group``) or a 1-3 dimensional Fortran-indexed array (as
    dataset ``group/key``) to ``filename``, creating the file and the group
    when absent.  Exactly one input must be given; an existing key is
    replaced."""
    _write(filename, F8, scalar_input, (array_input_1d, array_input_2d, array_input_3d), key, group)


def hdf5_write_int(filename, scalar_input=None, array_input_1d=None, array_input_2d=None,
                   array_input_3d=None, *, key: str, group: str) -> None:
    """hdf5_write_int (src/hdf5_io.F90:406-547): as hdf5_write_real with
    64-bit little-endian integers (H5T_STD_I64LE)."""
    _write(filename, I8, scalar_input, (array_input_1d, array_input_2d, array_input_3d), key, group)


def _read_array(filename, group, key, rank, dtype):
    d = read_file(filename).find(group).children.get(key)
    if not isinstance(d, Dataset):
        raise KeyError(f"no dataset {group}/{key} in {filename}")
    if len(d.dims) != rank:
        raise ValueError(f"{group}/{key} has rank {len(d.dims)}, not {rank}")
    # the Fortran view of the file's C-ordered dims
    return np.asfortranarray(d.read().astype(dtype).T)


def _read_scalar(filename, group, key):
    g = read_file(filename).find(group)
    if key not in g.attrs:
        raise KeyError(f"no attribute {key} on {group} in {filename}")
    return g.attrs[key]


def hdf5_read_real_3d(filename, group, key):
    """hdf5_read_real_3d (src/hdf5_io.F90:23-52): dataset as a FP64 Fortran array."""
    return _read_array(filename, group, key, 3, F8)


def hdf5_read_real_2d(filename, group, key):
    """hdf5_read_real_2d (src/hdf5_io.F90:85-114)."""
    return _read_array(filename, group, key, 2, F8)


def hdf5_read_real_1d(filename, group, key):
    """hdf5_read_real_1d (src/hdf5_io.F90:147-176)."""
    return _read_array(filename, group, key, 1, F8)


def hdf5_read_int_3d(filename, group, key):
    """hdf5_read_int_3d (src/hdf5_io.F90:54-83): dataset as an int64 Fortran array."""
    return _read_array(filename, group, key, 3, I8)


def hdf5_read_int_2d(filename, group, key):
    """hdf5_read_int_2d (src/hdf5_io.F90:116-145)."""
    return _read_array(filename, group, key, 2, I8)


def hdf5_read_int_1d(filename, group, key):
    """hdf5_read_int_1d (src/hdf5_io.F90:178-207)."""
    return _read_array(filename, group, key, 1, I8)


def hdf5_read_real_scalar(filename, group, key) -> float:
    """hdf5_read_real_scalar (src/hdf5_io.F90:209-234): the group's attribute as FP64."""
    return float(_read_scalar(filename, group, key))


def hdf5_read_int_scalar(filename, group, key) -> int:
    """hdf5_read_int_scalar (src/hdf5_io.F90:236-261): the group's attribute as an integer."""
    return int(_read_scalar(filename, group, key))


# ---------------------------------------------------------------------------
# write_output_hdf5 (src/WriteOutput_corner1.F90:21-78)
# ---------------------------------------------------------------------------

def field_name_hdf5(ita: int, block_id: int) -> str:
    """The file write_output_hdf5 writes (src/WriteOutput_corner1.F90:42)."""
    return f"out/timestep_{ita:05d}_block_{block_id:05d}.h5"


def write_fields_hdf5(path, x1, y1, z1, fields: dict, tags: dict, totime: float) -> None:
    """One block's field file: datasets u1, v1, w1 (cell-centred velocities
    (u(i)+u(i-1))/2 etc.), p, xp, yp, zp (cell centres) over the interior
    cells, the int64 tags cell, cell_n and cell_pr, and the attributes zonei,
    zonej, zonek and totime on the root group.  zonej holds nx, as the
    reference writes it (src/WriteOutput_corner1.F90:58-59).  The file is
    written whole in one pass (the reference adds the items one call at a
    time to the same layout)."""
    u, v, w, p = (np.asarray(fields[k], dtype=np.float64) for k in ("u", "v", "w", "p"))
    nx, ny, nz = u.shape[0] - 2, u.shape[1] - 2, u.shape[2] - 2
    c = lambda a: 0.5 * (a[1:] + a[:-1])
    xp = c(np.asarray(x1, dtype=np.float64))[1:nx + 1]
    yp = c(np.asarray(y1, dtype=np.float64))[1:ny + 1]
    zp = c(np.asarray(z1, dtype=np.float64))[1:nz + 1]
    arr = {
        "u1": 0.5 * (u[1:-1, 1:-1, 1:-1] + u[:-2, 1:-1, 1:-1]),
        "v1": 0.5 * (v[1:-1, 1:-1, 1:-1] + v[1:-1, :-2, 1:-1]),
        "w1": 0.5 * (w[1:-1, 1:-1, 1:-1] + w[1:-1, 1:-1, :-2]),
        "xp": xp, "yp": yp, "zp": zp,
        "p": p[1:-1, 1:-1, 1:-1],
    }
    root = Group()
    for k, a in arr.items():
        root.children[k] = Dataset(dims=a.shape[::-1], dtype=F8, data=np.ascontiguousarray(a.T))
    for k in ("cell", "cell_n", "cell_pr"):
        a = np.asarray(tags[k])[1:nx + 1, 1:ny + 1, 1:nz + 1].astype(I8)
        root.children[k] = Dataset(dims=a.shape[::-1], dtype=I8, data=np.ascontiguousarray(a.T))
    root.attrs.update(zonei=np.int64(nx), zonej=np.int64(nx), zonek=np.int64(nz), totime=np.float64(totime))
    write_file(path, root)
