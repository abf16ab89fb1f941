"""A small HDF5 reader and writer for the files of the k-Wave C++ binary.

The C++ code of k-Wave takes its input from an HDF5 file and writes its
results to another (kwave/solvers/cpp_simulation.py:139-312 writes and reads
them through h5py; kwave/utils/io.py:52-188 writes one matrix).  Neither h5py
nor the HDF5 library is a dependency of this package, so this module writes
and reads the subset of the HDF5 format those files use, from the published
HDF5 file format specification:

* superblock version 0 (version 1 read as well), 8-byte offsets and lengths;
* one root group held as a symbol table: version-1 B-tree of group nodes,
  symbol table nodes, local heap of names;
* datasets with version-1 object headers (continuation blocks followed when
  reading): simple dataspaces, IEEE little-endian float32/float64 and
  little-endian integers, contiguous or chunked storage (a single leaf
  B-tree node of chunks when writing, any depth when reading) and compact
  storage (read);
* the filters h5py applies to chunks (``compression=level``, ``shuffle``,
  ``fletcher32``): deflate (zlib) and shuffle written and read, the Fletcher
  checksum read (stripped, not verified); filter pipeline messages of
  version 1 (written) and 1 or 2 (read), per-chunk filter masks honoured;
* attributes of fixed-length ASCII strings (``<S{n}``, null-padded, scalar),
  on datasets and on the root group.

Data are written and read as stored: the dimensions in the file are the
array's shape (C order).  Other filters (szip, n-bit, scale-offset),
variable-length types, version-2 object headers and newer superblocks are
refused with NotImplementedError.  The format subset is checked by round trips and by
structural tests; no HDF5 library is available to cross-check against.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b"\x89HDF\r\n\x1a\n"
LEAF_K = 4        # group leaf node K: a symbol table node holds 2 K entries
INTERNAL_K = 16   # group internal node K: a B-tree node holds 2 K children

# object header message types
MSG_NIL, MSG_DATASPACE, MSG_DATATYPE, MSG_FILL, MSG_LAYOUT = 0x0, 0x1, 0x3, 0x5, 0x8
MSG_FILTERS, MSG_ATTRIBUTE, MSG_CONTINUATION, MSG_SYMBOL_TABLE = 0xB, 0xC, 0x10, 0x11


def _pad8(n):
    return (n + 7) & ~7


def _padb(b):
    return b + b"\0" * (_pad8(len(b)) - len(b))


# ---------------------------------------------------------------------------
# datatypes
# ---------------------------------------------------------------------------

def _datatype_message(dt):
    """Datatype message bytes for a numpy dtype (version 1)."""
    dt = np.dtype(dt)
    if dt.kind == "f":
        if dt.itemsize == 4:
            sign, eloc, esize, msize, bias = 31, 23, 8, 23, 127
        elif dt.itemsize == 8:
            sign, eloc, esize, msize, bias = 63, 52, 11, 52, 1023
        else:
            raise NotImplementedError(f"float of {dt.itemsize} bytes")
        head = struct.pack("<BBBBI", (1 << 4) | 1, 0x20, sign, 0, dt.itemsize)
        return head + struct.pack("<HHBBBBI", 0, 8 * dt.itemsize, eloc, esize, 0, msize, bias)
    if dt.kind in "iu":
        flags = 0x08 if dt.kind == "i" else 0x00
        head = struct.pack("<BBBBI", (1 << 4) | 0, flags, 0, 0, dt.itemsize)
        return head + struct.pack("<HH", 0, 8 * dt.itemsize)
    if dt.kind == "S":
        # null-padded ASCII (padding type 1, character set 0)
        return struct.pack("<BBBBI", (1 << 4) | 3, 0x01, 0, 0, dt.itemsize)
    raise NotImplementedError(f"dtype {dt}")


def _parse_datatype(b, off):
    """numpy dtype of the datatype message at b[off:]."""
    cv, f0, f1, f2, size = struct.unpack_from("<BBBBI", b, off)
    cls = cv & 0x0F
    if cls == 0:
        if f0 & 0x01:
            raise NotImplementedError("big-endian integers")
        return np.dtype(("<i" if f0 & 0x08 else "<u") + str(size))
    if cls == 1:
        if f0 & 0x01 or f0 & 0x40:
            raise NotImplementedError("non-little-endian floating point")
        if size not in (4, 8):
            raise NotImplementedError(f"float of {size} bytes")
        return np.dtype("<f" + str(size))
    if cls == 3:
        return np.dtype("S" + str(size))
    raise NotImplementedError(f"HDF5 datatype class {cls}")


def _dataspace_message(shape):
    return struct.pack("<BBBBI", 1, len(shape), 0, 0, 0) + b"".join(struct.pack("<Q", int(d)) for d in shape)


def _parse_dataspace(b, off):
    version, rank, flags = b[off], b[off + 1], b[off + 2]
    if version == 1:
        p = off + 8
    elif version == 2:
        if b[off + 3] == 2:  # null dataspace
            return None
        p = off + 4
    else:
        raise NotImplementedError(f"dataspace version {version}")
    return tuple(struct.unpack_from("<Q", b, p + 8 * i)[0] for i in range(rank))


# ---------------------------------------------------------------------------
# writer
# ---------------------------------------------------------------------------

def _object_header(messages):
    """Version-1 object header: [(type, payload bytes)] -> bytes."""
    body = b"".join(struct.pack("<HHB3x", t, _pad8(len(p)), 0) + _padb(p) for t, p in messages)
    return struct.pack("<BBHII", 1, 0, len(messages), 1, len(body)) + b"\0" * 4 + body


def _attribute_message(name, value):
    """Version-1 attribute message: scalar fixed-length string `value`."""
    nm = name.encode("ascii") + b"\0"
    data = value.encode("ascii") if isinstance(value, str) else bytes(value)
    dt = _datatype_message(np.dtype("S" + str(max(1, len(data)))))
    ds = _dataspace_message(())
    data = data if data else b"\0"
    return (struct.pack("<BBHHH", 1, 0, len(nm), len(dt), len(ds)) + _padb(nm) + _padb(dt) + _padb(ds) + data)


def _attr_messages(attrs):
    return [(MSG_ATTRIBUTE, _attribute_message(k, v)) for k, v in (attrs or {}).items()]


ISTORE_K = 32  # indexed storage internal node K of a version-0 superblock

FILTER_DEFLATE, FILTER_SHUFFLE, FILTER_FLETCHER32 = 1, 2, 3


def _filter_message(filters):
    """Filter pipeline message, version 1: [(filter id, [client data])] for
    the predefined filters (no names), each optional (flags 0)."""
    body = struct.pack("<BB6x", 1, len(filters))
    for fid, cd in filters:
        body += struct.pack("<HHHH", fid, 0, 0, len(cd)) + b"".join(struct.pack("<I", v) for v in cd)
        if len(cd) % 2:
            body += b"\0" * 4
    return body


def _parse_filters(b, off):
    """[(filter id, [client data])] of a filter pipeline message (versions 1
    and 2 of the format specification)."""
    version, n = b[off], b[off + 1]
    p = off + (8 if version == 1 else 2)
    if version not in (1, 2):
        raise NotImplementedError(f"filter pipeline message version {version}")
    out = []
    for _ in range(n):
        fid = struct.unpack_from("<H", b, p)[0]
        p += 2
        name_len = 0
        if version == 1 or fid >= 256:
            name_len = struct.unpack_from("<H", b, p)[0]
            p += 2
        _flags, ncd = struct.unpack_from("<HH", b, p)
        p += 4
        p += _pad8(name_len) if version == 1 else name_len
        cd = list(struct.unpack_from("<" + "I" * ncd, b, p))
        p += 4 * ncd
        if version == 1 and ncd % 2:
            p += 4
        out.append((fid, cd))
    return out


def _shuffle(raw, size):
    n = len(raw) // size
    head = np.frombuffer(raw, dtype=np.uint8, count=n * size).reshape(n, size).T.tobytes()
    return head + raw[n * size:]


def _unshuffle(raw, size):
    n = len(raw) // size
    head = np.frombuffer(raw, dtype=np.uint8, count=n * size).reshape(size, n).T.tobytes()
    return head + raw[n * size:]


def _decode_chunk(raw, filters, mask, itemsize):
    """Undo the pipeline on one chunk's stored bytes, last filter first;
    bit i of ``mask`` set means filter i was skipped for this chunk."""
    data = bytes(raw)
    for i in range(len(filters) - 1, -1, -1):
        if (mask >> i) & 1:
            continue
        fid, cd = filters[i]
        if fid == FILTER_DEFLATE:
            data = zlib.decompress(data)
        elif fid == FILTER_SHUFFLE:
            data = _unshuffle(data, int(cd[0]) if cd else itemsize)
        elif fid == FILTER_FLETCHER32:
            # the checksum the filter appended (4 bytes): stripped, not verified
            data = data[:-4]
        else:
            raise NotImplementedError(f"HDF5 filter {fid}")
    return data


def _chunk_grid(shape, chunk):
    """Offsets (in elements) of the chunks covering `shape`, in C order."""
    counts = [-(-int(d) // int(c)) for d, c in zip(shape, chunk)]
    return [tuple(int(i) * int(c) for i, c in zip(idx, chunk)) for idx in np.ndindex(*counts)]


def write_file(path, datasets, attrs=None, root_attrs=None, chunks=None, compression=None, shuffle=None):
    """Write an HDF5 file with datasets in its root group.

    datasets: {name: ndarray} (stored as given: shape and C-order data);
    attrs: {name: {attr: str}}; root_attrs: {attr: str}; chunks: {name:
    chunk shape} for datasets stored in chunks (at most 2 * 32 chunks each,
    one B-tree node), the others contiguous; compression: {name: deflate
    level 1-9} and shuffle: {name, ...} filter chunked datasets as h5py's
    ``compression=level`` and ``shuffle=True`` do (shuffle first).  Names are
    sorted in the group, as the format requires."""
    attrs = attrs or {}
    chunks = {k: tuple(int(c) for c in v) for k, v in (chunks or {}).items()}
    compression = {k: int(v) for k, v in (compression or {}).items() if v}
    shuffle = set(shuffle or ())
    for n in set(compression) | shuffle:
        if n not in chunks:
            raise ValueError(f"{n}: filters need chunked storage")
        if n in compression and not 1 <= compression[n] <= 9:
            raise ValueError(f"{n}: deflate level {compression[n]}")
    names = sorted(datasets)
    for n in names:
        if "/" in n or not n:
            raise ValueError(f"dataset name {n!r}")
    arrays = {n: np.array(datasets[n], order="C", copy=True) for n in names}
    for n, a in arrays.items():
        if a.dtype.byteorder == ">":
            arrays[n] = a.astype(a.dtype.newbyteorder("<"))

    # local heap of link names: offset 0 is the empty name; a 16-byte free
    # block closes the data segment (next-free offset 1 ends the list, the
    # HDF5 library's convention)
    heap = bytearray(b"\0" * 8)
    name_off = {}
    for n in names:
        name_off[n] = len(heap)
        heap += _padb(n.encode("ascii") + b"\0")
    free_off = len(heap)
    heap += struct.pack("<QQ", 1, 16)
    # symbol table nodes of 2 LEAF_K entries, one B-tree node over them
    groups = [names[i:i + 2 * LEAF_K] for i in range(0, len(names), 2 * LEAF_K)] or [[]]
    if len(groups) > 2 * INTERNAL_K:
        raise NotImplementedError(f"{len(names)} datasets in one group (at most {4 * LEAF_K * INTERNAL_K})")

    sb_size = 96
    snod_size = 8 + 2 * LEAF_K * 40
    btree_size = 24 + 2 * INTERNAL_K * 8 + (2 * INTERNAL_K + 1) * 8
    heap_hdr = 32
    root_msgs = [(MSG_SYMBOL_TABLE, b"\0" * 16)] + _attr_messages(root_attrs)
    root_size = len(_object_header(root_msgs))

    # addresses
    a_root = sb_size
    a_heap = a_root + root_size
    a_heap_data = a_heap + heap_hdr
    a_btree = a_heap_data + len(heap)
    a_snods = [a_btree + btree_size + i * snod_size for i in range(len(groups))]
    p = a_btree + btree_size + len(groups) * snod_size

    def pipeline(n):
        f = []
        if n in shuffle:
            f.append((FILTER_SHUFFLE, [arrays[n].itemsize]))
        if n in compression:
            f.append((FILTER_DEFLATE, [compression[n]]))
        return f

    def dset_msgs(n, data_addr):
        a = arrays[n]
        filt = []
        if n in chunks:
            ch = chunks[n]
            layout = (struct.pack("<BBBQ", 3, 2, a.ndim + 1, data_addr) +
                      b"".join(struct.pack("<I", c) for c in ch) + struct.pack("<I", a.itemsize))
            if pipeline(n):
                filt = [(MSG_FILTERS, _filter_message(pipeline(n)))]
        else:
            layout = struct.pack("<BBQQ", 3, 1, data_addr if a.nbytes else UNDEF, a.nbytes)
        return ([(MSG_DATASPACE, _dataspace_message(a.shape)), (MSG_DATATYPE, _datatype_message(a.dtype)),
                 (MSG_FILL, struct.pack("<BBBB", 2, 2, 2, 0))] + filt + [(MSG_LAYOUT, layout)] +
                _attr_messages(attrs.get(n)))

    def chunk_blocks(n):
        """(offsets, stored bytes) of each chunk of a chunked dataset (edge
        chunks zero-filled to the full chunk shape, then filtered)."""
        a, ch = arrays[n], chunks[n]
        out = []
        for o in _chunk_grid(a.shape, ch):
            blk = np.zeros(ch, dtype=a.dtype)
            sl = tuple(slice(x, min(x + c, d)) for x, c, d in zip(o, ch, a.shape))
            blk[tuple(slice(0, t.stop - t.start) for t in sl)] = a[sl]
            raw = blk.tobytes()
            for fid, cd in pipeline(n):
                raw = _shuffle(raw, cd[0]) if fid == FILTER_SHUFFLE else zlib.compress(raw, cd[0])
            out.append((o, raw))
        return out

    for n, ch in chunks.items():
        a = arrays[n]
        if len(ch) != a.ndim or a.ndim == 0 or min(ch) < 1:
            raise ValueError(f"chunk shape {ch} for {n} of shape {a.shape}")
        if len(_chunk_grid(a.shape, ch)) > 2 * ISTORE_K:
            raise NotImplementedError(f"{n}: more than {2 * ISTORE_K} chunks")

    a_obj = {}
    for n in names:
        a_obj[n] = p
        p += len(_object_header(dset_msgs(n, 0)))
    a_data, a_chunks, blocks = {}, {}, {}
    for n in names:
        p = _pad8(p)
        a_data[n] = p
        if n in chunks:
            a = arrays[n]
            ksize = 8 + 8 * (a.ndim + 1)
            p += 24 + 2 * ISTORE_K * 8 + (2 * ISTORE_K + 1) * ksize
            blocks[n] = chunk_blocks(n)
            a_chunks[n] = []
            for _, raw in blocks[n]:
                p = _pad8(p)
                a_chunks[n].append(p)
                p += len(raw)
        else:
            p += arrays[n].nbytes
    eof = _pad8(p)

    out = bytearray(eof)
    root_entry = struct.pack("<QQI4xQQ", 0, a_root, 1, a_btree, a_heap)
    out[0:sb_size] = (SIGNATURE + struct.pack("<BBBBBBBB", 0, 0, 0, 0, 0, 8, 8, 0) +
                      struct.pack("<HHI", LEAF_K, INTERNAL_K, 0) + struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF) +
                      root_entry)
    root_msgs[0] = (MSG_SYMBOL_TABLE, struct.pack("<QQ", a_btree, a_heap))
    out[a_root:a_root + root_size] = _object_header(root_msgs)
    out[a_heap:a_heap + heap_hdr] = b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap), free_off, a_heap_data)
    out[a_heap_data:a_heap_data + len(heap)] = heap
    # B-tree: key i+1 = last name of child i, key 0 = the empty name
    bt = bytearray(b"TREE" + struct.pack("<BBHQQ", 0, 0, len(groups), UNDEF, UNDEF))
    bt += struct.pack("<Q", 0)
    for g, a in zip(groups, a_snods):
        bt += struct.pack("<QQ", a, name_off[g[-1]] if g else 0)
    out[a_btree:a_btree + len(bt)] = bt
    for g, a in zip(groups, a_snods):
        sn = bytearray(b"SNOD" + struct.pack("<BBH", 1, 0, len(g)))
        for n in g:
            sn += struct.pack("<QQI4x16x", name_off[n], a_obj[n], 0)
        out[a:a + len(sn)] = sn
    for n in names:
        oh = _object_header(dset_msgs(n, a_data[n]))
        out[a_obj[n]:a_obj[n] + len(oh)] = oh
        a = arrays[n]
        if n not in chunks:
            b = a.tobytes()
            out[a_data[n]:a_data[n] + len(b)] = b
            continue
        # one leaf B-tree node (type 1): key i = (chunk bytes, filter mask 0,
        # chunk offsets, 0), child i = chunk address; the last key bounds the
        # dataset
        ch = chunks[n]
        bt = bytearray(b"TREE" + struct.pack("<BBHQQ", 1, 0, len(blocks[n]), UNDEF, UNDEF))
        for (o, raw), ca in zip(blocks[n], a_chunks[n]):
            bt += struct.pack("<II", len(raw), 0) + b"".join(struct.pack("<Q", x) for x in o) + struct.pack("<Q", 0)
            bt += struct.pack("<Q", ca)
            out[ca:ca + len(raw)] = raw
        end = tuple(-(-d // c) * c for d, c in zip(a.shape, ch))
        bt += struct.pack("<II", 0, 0) + b"".join(struct.pack("<Q", x) for x in end) + struct.pack("<Q", 0)
        out[a_data[n]:a_data[n] + len(bt)] = bt
    with open(path, "wb") as f:
        f.write(out)


# ---------------------------------------------------------------------------
# reader
# ---------------------------------------------------------------------------

class _Reader:
    def __init__(self, b):
        self.b = b
        if b[:8] != SIGNATURE:
            raise ValueError("not an HDF5 file (signature)")
        version = b[8]
        if version not in (0, 1):
            raise NotImplementedError(f"HDF5 superblock version {version}")
        if b[13] != 8 or b[14] != 8:
            raise NotImplementedError("offsets or lengths other than 8 bytes")
        p = 16
        self.leaf_k, self.internal_k = struct.unpack_from("<HH", b, p)
        p += 8
        if version == 1:
            p += 4
        self.base = struct.unpack_from("<Q", b, p)[0]
        p += 32
        _, self.root_addr = struct.unpack_from("<QQ", b, p)

    def addr(self, a):
        return self.base + a

    def messages(self, addr):
        """Messages of the object header at addr: [(type, offset of payload, size)]."""
        b = self.b
        a = self.addr(addr)
        version = b[a]
        if version != 1:
            if b[a:a + 4] == b"OHDR":
                raise NotImplementedError("version-2 object headers")
            raise ValueError(f"object header version {version}")
        nmsg, _, size = struct.unpack_from("<HII", b, a + 2)
        blocks = [(a + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            start, size = blocks.pop(0)
            p, end = start, start + size
            while p + 8 <= end and len(out) < nmsg:
                t, sz, _flags = struct.unpack_from("<HHB", b, p)
                if t == MSG_CONTINUATION:
                    off, ln = struct.unpack_from("<QQ", b, p + 8)
                    blocks.append((self.addr(off), ln))
                out.append((t, p + 8, sz))
                p += 8 + sz
        return out

    def heap_name(self, heap_data, off):
        b = self.b
        e = b.index(b"\0", heap_data + off)
        return b[heap_data + off:e].decode("ascii")

    def group_entries(self, btree, heap):
        b = self.b
        h = self.addr(heap)
        if b[h:h + 4] != b"HEAP":
            raise ValueError("local heap signature")
        heap_data = self.addr(struct.unpack_from("<Q", b, h + 24)[0])
        entries = []

        def walk(node):
            n = self.addr(node)
            if b[n:n + 4] != b"TREE":
                raise ValueError("B-tree signature")
            ntype, level, used = struct.unpack_from("<BBH", b, n + 4)
            if ntype != 0:
                raise ValueError("group B-tree node type")
            p = n + 24 + 8  # key 0
            for _ in range(used):
                child = struct.unpack_from("<Q", b, p)[0]
                p += 16
                if level > 0:
                    walk(child)
                else:
                    s = self.addr(child)
                    if b[s:s + 4] != b"SNOD":
                        raise ValueError("symbol table node signature")
                    count = struct.unpack_from("<H", b, s + 6)[0]
                    for i in range(count):
                        e = s + 8 + 40 * i
                        name_off, obj = struct.unpack_from("<QQ", b, e)
                        entries.append((self.heap_name(heap_data, name_off), obj))

        walk(btree)
        return entries

    def attribute(self, off):
        b = self.b
        version = b[off]
        if version == 1:
            nsz, tsz, ssz = struct.unpack_from("<HHH", b, off + 2)
            p = off + 8
            name = b[p:p + nsz - 1].decode("ascii")
            p += _pad8(nsz)
            dt = _parse_datatype(b, p)
            p += _pad8(tsz)
            shape = _parse_dataspace(b, p)
            p += _pad8(ssz)
        elif version == 3:
            nsz, tsz, ssz = struct.unpack_from("<HHH", b, off + 2)
            p = off + 9
            name = b[p:p + nsz - 1].decode("utf-8")
            p += nsz
            dt = _parse_datatype(b, p)
            p += tsz
            shape = _parse_dataspace(b, p)
            p += ssz
        else:
            raise NotImplementedError(f"attribute message version {version}")
        count = int(np.prod(shape)) if shape else 1
        val = np.frombuffer(b, dtype=dt, count=count, offset=p)
        if dt.kind == "S":
            val = val[0].rstrip(b"\0").decode("ascii") if count == 1 else val.copy()
        else:
            val = val.reshape(shape).copy() if shape else val[0]
        return name, val

    def chunks(self, btree, rank, dt, shape, chunk, filters=()):
        """Assemble a chunked dataset from its version-1 B-tree, undoing the
        filter pipeline on each chunk."""
        b = self.b
        out = np.zeros(shape, dtype=dt)
        ksize = 8 + 8 * (rank + 1)

        def walk(node):
            n = self.addr(node)
            if b[n:n + 4] != b"TREE":
                raise ValueError("chunk B-tree signature")
            ntype, level, used = struct.unpack_from("<BBH", b, n + 4)
            if ntype != 1:
                raise ValueError("chunk B-tree node type")
            p = n + 24
            for _ in range(used):
                csize, fmask = struct.unpack_from("<II", b, p)
                offs = struct.unpack_from("<" + "Q" * rank, b, p + 8)
                child = struct.unpack_from("<Q", b, p + ksize)[0]
                p += ksize + 8
                if level > 0:
                    walk(child)
                    continue
                count = int(np.prod(chunk))
                if filters:
                    start = self.addr(child)
                    raw = _decode_chunk(b[start:start + csize], filters, fmask, dt.itemsize)
                    blk = np.frombuffer(raw, dtype=dt, count=count).reshape(chunk)
                else:
                    blk = np.frombuffer(b, dtype=dt, count=count, offset=self.addr(child)).reshape(chunk)
                sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, chunk, shape))
                out[sl] = blk[tuple(slice(0, s.stop - s.start) for s in sl)]

        if btree != UNDEF:
            walk(btree)
        return out

    def dataset(self, addr):
        b = self.b
        dt = shape = None
        layout = None
        filters = []
        attrs = {}
        for t, off, sz in self.messages(addr):
            if t == MSG_DATASPACE:
                shape = _parse_dataspace(b, off)
            elif t == MSG_DATATYPE:
                dt = _parse_datatype(b, off)
            elif t == MSG_LAYOUT:
                layout = off
            elif t == MSG_FILTERS:
                filters = _parse_filters(b, off)
            elif t == MSG_ATTRIBUTE:
                k, v = self.attribute(off)
                attrs[k] = v
        if dt is None or layout is None:
            return None, attrs
        shape = shape or ()
        version, cls = b[layout], b[layout + 1]
        if version != 3:
            raise NotImplementedError(f"layout message version {version}")
        count = int(np.prod(shape)) if shape else 1
        if filters and cls != 2:
            raise ValueError("a filter pipeline on a dataset that is not chunked")
        if cls == 1:
            data_addr, size = struct.unpack_from("<QQ", b, layout + 2)
            if data_addr == UNDEF:
                arr = np.zeros(shape, dtype=dt)
            else:
                arr = np.frombuffer(b, dtype=dt, count=count, offset=self.addr(data_addr)).reshape(shape).copy()
        elif cls == 0:
            size = struct.unpack_from("<H", b, layout + 2)[0]
            arr = np.frombuffer(b, dtype=dt, count=count, offset=layout + 4).reshape(shape).copy()
        elif cls == 2:
            nd = b[layout + 2]
            bt = struct.unpack_from("<Q", b, layout + 3)[0]
            dims = struct.unpack_from("<" + "I" * nd, b, layout + 11)
            arr = self.chunks(bt, nd - 1, dt, shape, dims[:-1], filters)
        else:
            raise NotImplementedError(f"layout class {cls}")
        return arr, attrs


def read_file(path):
    """Read the root group of an HDF5 file: (datasets, attrs, root_attrs)
    with datasets {name: ndarray}, attrs {name: {attr: value}} and the root
    group's attributes."""
    with open(path, "rb") as f:
        b = f.read()
    r = _Reader(b)
    btree = heap = None
    root_attrs = {}
    for t, off, sz in r.messages(r.root_addr):
        if t == MSG_SYMBOL_TABLE:
            btree, heap = struct.unpack_from("<QQ", b, off)
        elif t == MSG_ATTRIBUTE:
            k, v = r.attribute(off)
            root_attrs[k] = v
    if btree is None:
        raise NotImplementedError("root group without a symbol table (newer group format)")
    datasets, attrs = {}, {}
    for name, obj in r.group_entries(btree, heap):
        arr, at = r.dataset(obj)
        if arr is not None:
            datasets[name] = arr
            attrs[name] = at
    return datasets, attrs, root_attrs
