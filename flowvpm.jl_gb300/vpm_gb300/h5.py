"""A minimal HDF5 file writer and reader for particle-field files, with no HDF5 library.

The reference's `save` writes its datasets through HDF5.jl (src/FLOWVPM_utils.jl:175-221):
scalar int64 datasets np and nt, a scalar float64 t, and float64 arrays stored contiguously.
Under its default (earliest) format bounds libhdf5 writes such a file in the original formats:
a version-0 superblock, version-1 object headers and groups held as a symbol table (a version-1
B-tree of symbol-table nodes, with the names in a local heap). This module writes exactly that
subset, in the layouts libhdf5 itself writes for it:

* superblock version 0, 8-byte offsets and lengths, group leaf K 4 and internal K 16;
* the root group: an object header holding a symbol-table message (plus a NIL message, as
  libhdf5 pads it to 32 bytes), a local heap of the names, one leaf B-tree node (allocated at its
  full 2K-child size) and symbol-table nodes of at most 2 x 4 entries (allocated at full size);
* one object header per dataset with a fill-value (version 1), datatype (version 1),
  dataspace (version 1) and data-layout (version 3, contiguous) message;
* little-endian IEEE float64 and signed int64 data, C order (the first dimension slowest).

The reader follows the same formats and a little more: superblock version 0 or 1 with a user
block before it, 4- or 8-byte offsets, object-header continuation messages, B-trees of any
depth, data-layout versions 1 to 4 with contiguous or compact storage, and fixed-point or
floating-point types of either byte order. Chunked or filtered datasets, and the newer file
formats (superblock 2 and 3, version-2 object headers, link messages), raise NotImplementedError.
"""
from __future__ import annotations

import struct

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
LEAF_K = 4            # symbol-table node: at most 2 x LEAF_K entries
INTERNAL_K = 16       # group B-tree node: at most 2 x INTERNAL_K children
HEAP_FREE_NULL = 1    # "no free block" in a local heap's free-list head

MSG_NIL, MSG_DATASPACE, MSG_DATATYPE, MSG_FILL_OLD, MSG_FILL = 0x0, 0x1, 0x3, 0x4, 0x5
MSG_LAYOUT, MSG_CONTINUATION, MSG_SYMTAB = 0x8, 0x10, 0x11
FLAG_CONSTANT = 1

_SNOD_BYTES = 8 + 2 * LEAF_K * 40
_TREE_BYTES = 24 + 2 * INTERNAL_K * 8 + (2 * INTERNAL_K + 1) * 8


def _pad8(n: int) -> int:
    return (n + 7) & ~7


# ----------------------------------------------------------------------------------------------
# writer
# ----------------------------------------------------------------------------------------------

def _datatype_msg(dtype: np.dtype) -> bytes:
    """Datatype message, version 1: float64 (IEEE, little-endian) or signed int64."""
    if dtype == np.float64:
        # class 1; bit field: mantissa normalisation 2 (implied leading 1), sign at bit 63
        return struct.pack("<B3BI HHBBBBI", 0x11, 0x20, 63, 0, 8, 0, 64, 52, 11, 0, 52, 1023)
    if dtype == np.int64:
        # class 0; bit field: signed, little-endian
        return struct.pack("<B3BI HH", 0x10, 0x08, 0, 0, 8, 0, 64)
    raise TypeError(f"unsupported dataset type {dtype}")


def _dataspace_msg(shape) -> bytes:
    """Dataspace message, version 1 (rank 0 is a scalar), no maximum dimensions."""
    return struct.pack("<BBBBI", 1, len(shape), 0, 0, 0) + b"".join(struct.pack("<Q", d) for d in shape)


def _object_header(msgs) -> bytes:
    """Version-1 object header: the 16-byte prefix, then (type, flags, data) messages, each
    padded to 8 bytes; the stored message size counts the padding."""
    body = b""
    for typ, flags, data in msgs:
        size = _pad8(len(data))
        body += struct.pack("<HHB3x", typ, size, flags) + data + b"\0" * (size - len(data))
    return struct.pack("<BBHII4x", 1, 0, len(msgs), 1, len(body)) + body


def write(path: str, datasets: dict) -> None:
    """Write `datasets` ({name: int, float or numpy array}) as datasets of the root group of a
    new HDF5 file at `path` (truncating it). Python ints and int64 arrays are stored as signed
    int64, everything else as float64; arrays keep their shape, 0-d values are scalars."""
    items = []
    for name, value in datasets.items():
        b = name.encode()
        if not b or b"/" in b or b"\0" in b or b == b".":
            raise ValueError(f"bad dataset name {name!r}")
        a = np.asarray(value)
        items.append((b, np.array(a, dtype="<i8" if a.dtype.kind in "iub" else "<f8", order="C")))
    items.sort(key=lambda it: it[0])          # symbol-table nodes hold the names in byte order
    if len(items) > 2 * LEAF_K * 2 * INTERNAL_K:
        raise ValueError("too many datasets for one B-tree node")

    # local heap of the names: "" first (the B-tree's leftmost key), each name padded to 8 bytes
    heap_data, name_off = b"\0" * 8, []
    for b, _ in items:
        name_off.append(len(heap_data))
        heap_data += b + b"\0" * (_pad8(len(b) + 1) - len(b))

    # consecutive runs of at most 2 x LEAF_K names, one symbol-table node each
    snods = [list(range(i, min(i + 2 * LEAF_K, len(items)))) for i in range(0, len(items), 2 * LEAF_K)]

    # addresses: superblock, root object header, heap header + data, B-tree, SNODs, dataset
    # object headers, then the raw data
    off = 96
    root_ohdr = off
    root_ohdr_bytes = _object_header([(MSG_SYMTAB, FLAG_CONSTANT, b"\0" * 16), (MSG_NIL, 0, b"")])
    off += len(root_ohdr_bytes)
    heap = off
    off += 32 + len(heap_data)
    tree = off
    off += _TREE_BYTES
    snod_addr = []
    for _ in snods:
        snod_addr.append(off)
        off += _SNOD_BYTES
    # fill value (version 1: allocation late, fill if set, no value), datatype, dataspace, and
    # the contiguous layout (version 3), whose address is filled in below
    ohdrs, ohdr_addr = [], []
    for b, a in items:
        msgs = [(MSG_FILL, FLAG_CONSTANT, struct.pack("<BBBBI", 1, 2, 2, 1, 0)),
                (MSG_DATATYPE, FLAG_CONSTANT, _datatype_msg(a.dtype)),
                (MSG_DATASPACE, 0, _dataspace_msg(a.shape)),
                (MSG_LAYOUT, FLAG_CONSTANT, b"\0" * 18)]
        ohdrs.append(msgs)
        ohdr_addr.append(off)
        off += len(_object_header(msgs))
    data_addr = []
    off = _pad8(off)
    for _, a in items:
        data_addr.append(off)
        off = _pad8(off + a.nbytes)
    eof = off

    out = bytearray(eof)
    # superblock version 0
    out[0:96] = (SIGNATURE + struct.pack("<8BHHI", 0, 0, 0, 0, 0, 8, 8, 0, LEAF_K, INTERNAL_K, 0)
                 + struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
                 + struct.pack("<QQII", 0, root_ohdr, 1, 0) + struct.pack("<QQ", tree, heap))
    symtab = struct.pack("<QQ", tree, heap)
    root_ohdr_bytes = _object_header([(MSG_SYMTAB, FLAG_CONSTANT, symtab), (MSG_NIL, 0, b"")])
    out[root_ohdr:root_ohdr + len(root_ohdr_bytes)] = root_ohdr_bytes
    # local heap, its data segment right after the header, no free block
    out[heap:heap + 32] = b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap_data), HEAP_FREE_NULL, heap + 32)
    out[heap + 32:heap + 32 + len(heap_data)] = heap_data
    # leaf B-tree node: key i is the heap offset of the last name in child i-1 ("" for key 0)
    node = b"TREE" + struct.pack("<BBHQQ", 0, 0, len(snods), UNDEF, UNDEF)
    node += struct.pack("<Q", 0)
    for k, idx in enumerate(snods):
        node += struct.pack("<QQ", snod_addr[k], name_off[idx[-1]])
    out[tree:tree + len(node)] = node
    # symbol-table nodes
    for k, idx in enumerate(snods):
        s = b"SNOD" + struct.pack("<BBH", 1, 0, len(idx))
        for i in idx:
            s += struct.pack("<QQII16x", name_off[i], ohdr_addr[i], 0, 0)
        out[snod_addr[k]:snod_addr[k] + len(s)] = s
    # dataset object headers (now with the data addresses) and the data
    for i, ((_, a), msgs) in enumerate(zip(items, ohdrs)):
        msgs[3] = (MSG_LAYOUT, FLAG_CONSTANT, struct.pack("<BBQQ", 3, 1, data_addr[i], a.nbytes))
        h = _object_header(msgs)
        out[ohdr_addr[i]:ohdr_addr[i] + len(h)] = h
        out[data_addr[i]:data_addr[i] + a.nbytes] = a.tobytes()
    with open(path, "wb") as f:
        f.write(out)


# ----------------------------------------------------------------------------------------------
# reader
# ----------------------------------------------------------------------------------------------

class _File:
    def __init__(self, data: bytes):
        self.d = data
        for base in [0] + [512 << k for k in range(20)]:
            if base + 8 > len(data):
                raise ValueError("not an HDF5 file (no signature)")
            if data[base:base + 8] == SIGNATURE:
                break
        sb = base
        ver = data[sb + 8]
        if ver not in (0, 1):
            raise NotImplementedError(f"HDF5 superblock version {ver} (only 0 and 1 are read)")
        self.so, self.sl = data[sb + 13], data[sb + 14]
        if self.so not in (4, 8) or self.sl not in (4, 8):
            raise NotImplementedError("offset or length size other than 4 or 8")
        p = sb + 24 + (4 if ver == 1 else 0)
        base_addr = self.addr(p)
        # addresses are relative to the base address (the superblock's own position when the
        # file has a user block)
        self.base = base_addr if base_addr != self.undef else sb
        p += 4 * self.so
        self.root_ohdr = self.addr(p + self.so)
        cache = struct.unpack_from("<I", data, p + 2 * self.so)[0]
        self.root_cache = (self.addr(p + 2 * self.so + 8), self.addr(p + 3 * self.so + 8)) if cache == 1 else None

    @property
    def undef(self):
        return (1 << (8 * self.so)) - 1

    def addr(self, p):
        return int.from_bytes(self.d[p:p + self.so], "little")

    def length(self, p):
        return int.from_bytes(self.d[p:p + self.sl], "little")

    def at(self, a):
        return self.base + a

    def messages(self, ohdr):
        """[(type, data bytes)] of a version-1 object header, continuation chunks included."""
        p = self.at(ohdr)
        if self.d[p] != 1:
            raise NotImplementedError(f"object header version {self.d[p]} (only 1 is read)")
        nmsg, _, size = struct.unpack_from("<HII", self.d, p + 2)
        chunks, out = [(p + 16, size)], []
        while chunks:
            q, size = chunks.pop(0)
            end = q + size
            while q + 8 <= end and len(out) < nmsg:
                typ, msize = struct.unpack_from("<HH", self.d, q)
                body = self.d[q + 8:q + 8 + msize]
                if typ == MSG_CONTINUATION:
                    chunks.append((self.at(self.addr(q + 8)), self.length(q + 8 + self.so)))
                out.append((typ, body))
                q += 8 + msize
        return out

    def group(self, ohdr, cache=None):
        """{name: object header address} of a symbol-table group."""
        if cache is None:
            st = [b for t, b in self.messages(ohdr) if t == MSG_SYMTAB]
            if not st:
                raise NotImplementedError("group without a symbol-table message (newer format)")
            cache = (int.from_bytes(st[0][:self.so], "little"), int.from_bytes(st[0][self.so:2 * self.so], "little"))
        tree, heap = cache
        h = self.at(heap)
        if self.d[h:h + 4] != b"HEAP":
            raise ValueError("bad local heap")
        hdata = self.at(self.addr(h + 8 + 2 * self.sl))

        def name(off):
            s = hdata + off
            return self.d[s:self.d.index(b"\0", s)].decode()
        out = {}

        def walk(node):
            n = self.at(node)
            if self.d[n:n + 4] != b"TREE" or self.d[n + 4] != 0:
                raise ValueError("bad group B-tree node")
            level, used = self.d[n + 5], struct.unpack_from("<H", self.d, n + 6)[0]
            q = n + 8 + 2 * self.so + self.sl        # past the header and key 0
            for _ in range(used):
                child = self.addr(q)
                q += self.so + self.sl
                if level > 0:
                    walk(child)
                    continue
                s = self.at(child)
                if self.d[s:s + 4] != b"SNOD":
                    raise ValueError("bad symbol-table node")
                for e in range(struct.unpack_from("<H", self.d, s + 6)[0]):
                    ent = s + 8 + e * (self.sl + self.so + 24)
                    out[name(self.length(ent))] = self.addr(ent + self.sl)
        walk(tree)
        return out

    def dataset(self, ohdr) -> np.ndarray:
        msgs = dict()
        for t, b in self.messages(ohdr):
            msgs.setdefault(t, b)
        if MSG_SYMTAB in msgs:
            raise ValueError("object is a group, not a dataset")
        ds, dt, lay = msgs[MSG_DATASPACE], msgs[MSG_DATATYPE], msgs[MSG_LAYOUT]
        # dataspace (versions 1 and 2)
        rank = ds[1]
        p = 8 if ds[0] == 1 else 4
        shape = tuple(int.from_bytes(ds[p + i * self.sl:p + (i + 1) * self.sl], "little") for i in range(rank))
        if ds[0] == 2 and ds[3] == 2:
            shape = (0,)                                   # null dataspace
        # datatype: fixed-point (class 0) or floating-point (class 1)
        cls, size = dt[0] & 0x0F, struct.unpack_from("<I", dt, 4)[0]
        order = ">" if dt[1] & 1 else "<"
        if cls == 0:
            dtype = np.dtype(f"{order}{'i' if dt[1] & 0x08 else 'u'}{size}")
        elif cls == 1 and size in (2, 4, 8):
            dtype = np.dtype(f"{order}f{size}")
        else:
            raise NotImplementedError(f"datatype class {cls} of size {size}")
        n = int(np.prod(shape, dtype=np.int64)) if shape else 1
        # data layout
        ver = lay[0]
        if ver in (1, 2):
            ndims, cls = lay[1], lay[2]
            q = 8
            if cls == 1:
                addr = int.from_bytes(lay[q:q + self.so], "little")
                q += self.so
            q += 4 * ndims
            if cls == 0:
                csize = struct.unpack_from("<I", lay, q)[0]
                raw = lay[q + 4:q + 4 + csize]
        elif ver in (3, 4):
            cls = lay[1]
            if cls == 0:
                csize = struct.unpack_from("<H", lay, 2)[0]
                raw = lay[4:4 + csize]
            elif cls == 1:
                addr = int.from_bytes(lay[2:2 + self.so], "little")
        else:
            raise NotImplementedError(f"data-layout message version {ver}")
        if cls == 1:
            if addr == self.undef:
                return np.zeros(shape, dtype=dtype.newbyteorder("="))       # never written: fill
            a = self.at(addr)
            raw = self.d[a:a + n * dtype.itemsize]
        elif cls != 0:
            raise NotImplementedError("chunked or virtual dataset storage")
        return np.frombuffer(raw, dtype=dtype, count=n).reshape(shape).astype(dtype.newbyteorder("="))


def read(path: str, names=None) -> dict:
    """{name: numpy array} of the datasets in the root group of the HDF5 file at `path`
    (only `names`, if given; a name missing from the file raises KeyError). Scalars come
    back as 0-d arrays."""
    with open(path, "rb") as f:
        hf = _File(f.read())
    entries = hf.group(hf.root_ohdr, hf.root_cache)
    out = {}
    for name in (entries if names is None else names):
        out[name] = hf.dataset(entries[name])
    return out


def keys(path: str) -> list:
    """Names in the root group of the HDF5 file at `path`."""
    with open(path, "rb") as f:
        hf = _File(f.read())
    return sorted(hf.group(hf.root_ohdr, hf.root_cache))
