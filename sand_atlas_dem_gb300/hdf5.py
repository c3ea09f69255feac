"""A small HDF5 reader and writer for the reference's file formats, with no h5py.

The reference keeps checkpoints (``sand-dem-checkpoint/3|4|5``,
``src/sand_atlas_dem/simulation.py:87-136``) and shape libraries
(``sand-dem-shapes/1``, ``src/sand_atlas_dem/geometry.py:114-163``) in HDF5
files written by h5py with its default (earliest) format: a version-0
superblock, version-1 object headers, groups as symbol tables (a version-1
B-tree of symbol nodes over a local heap), attributes with variable-length
UTF-8 strings in a global heap, and gzip-compressed chunked datasets.

:func:`read` parses that subset (plus contiguous and compact layouts,
shuffle and Fletcher-32 filters) into nested :class:`Group` objects.
:func:`write` produces the same structures (contiguous datasets, optionally
gzip-chunked) that the reader, and HDF5 itself, read back: a tree of
:class:`Group` with numpy arrays for datasets and str, int, float, bool or
numpy values for attributes.

The structures follow the published HDF5 File Format Specification
(version 2.0 of the document; superblock v0, object header v1, data layout
message v3, B-tree v1, local and global heaps).
"""

import struct
import zlib

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEFINED = 0xFFFFFFFFFFFFFFFF


class Group:
    """One HDF5 group: ``attrs`` (name -> value) and ``members`` (name ->
    Group or numpy array), in name order as HDF5 stores them."""

    def __init__(self, attrs=None, members=None):
        self.attrs = dict(attrs or {})
        self.members = dict(members or {})

    def __getitem__(self, name):
        node = self
        for part in name.strip("/").split("/"):
            node = node.members[part]
        return node

    def __contains__(self, name):
        return name in self.members

    def __iter__(self):
        return iter(self.members)


# ------------------------------------------------------------------- reading
class _Reader:
    def __init__(self, data):
        self.d = data
        if data[:8] != SIGNATURE:
            raise ValueError("Not an HDF5 file")
        version = data[8]
        if version not in (0, 1):
            raise ValueError(f"Unsupported HDF5 superblock version {version}")
        self.so, self.sl = data[13], data[14]
        if (self.so, self.sl) != (8, 8):
            raise ValueError("Only 8-byte offsets and lengths are supported")
        at = 24 + (4 if version == 1 else 0)
        self.base = self.u(at, 8)
        root_entry = at + 32
        self.root = self.u(root_entry + 8, 8)

    def u(self, at, n):
        return int.from_bytes(self.d[at:at + n], "little")

    # -- object headers
    def messages(self, address):
        d = self.d
        if d[address] != 1:
            raise ValueError(f"Unsupported object header version {d[address]} at {address}")
        count = self.u(address + 2, 2)
        size = self.u(address + 8, 4)
        blocks = [(address + 16, size)]
        out = []
        while blocks and len(out) < count:
            start, length = blocks.pop(0)
            at, end = start, start + length
            while at + 8 <= end and len(out) < count:
                kind, msize, flags = self.u(at, 2), self.u(at + 2, 2), d[at + 4]
                body = at + 8
                if kind == 0x10:  # continuation
                    blocks.append((self.u(body, 8), self.u(body + 8, 8)))
                out.append((kind, body, msize, flags))
                at = body + msize
        return out

    def object(self, address):
        msgs = self.messages(address)
        kinds = {k for k, _, _, _ in msgs}
        attrs = {}
        for kind, body, size, flags in msgs:
            if kind == 0x0C:
                name, value = self.attribute(body)
                attrs[name] = value
        if 0x11 in kinds:
            body = next(b for k, b, _, _ in msgs if k == 0x11)
            members = {}
            for name, child in self.group_entries(self.u(body, 8), self.u(body + 8, 8)):
                members[name] = self.object(child)
            return Group(attrs, dict(sorted(members.items())))
        if 0x08 in kinds:
            return self.dataset(msgs)
        return Group(attrs)

    # -- groups (symbol tables)
    def heap_data(self, heap):
        if self.d[heap:heap + 4] != b"HEAP":
            raise ValueError("Bad local heap")
        return self.u(heap + 24, 8)

    def cstring(self, at):
        end = self.d.index(b"\x00", at)
        return self.d[at:end].decode("utf-8")

    def group_entries(self, btree, heap):
        data = self.heap_data(heap)
        out = []
        for child in self.btree_children(btree, 0):
            if self.d[child:child + 4] != b"SNOD":
                raise ValueError("Bad symbol table node")
            n = self.u(child + 6, 2)
            for k in range(n):
                entry = child + 8 + 40 * k
                out.append((self.cstring(data + self.u(entry, 8)), self.u(entry + 8, 8)))
        return out

    def btree_children(self, node, kind, rank=0):
        """Leaf children of a version-1 B-tree (kind 0: symbol nodes; kind 1:
        (chunk address, chunk size, filter mask, offsets))."""
        d = self.d
        if d[node:node + 4] != b"TREE" or d[node + 4] != kind:
            raise ValueError("Bad B-tree node")
        level, used = d[node + 5], self.u(node + 6, 2)
        key = 8 if kind == 0 else 8 + 8 * (rank + 1)
        at = node + 24
        out = []
        for i in range(used):
            k, child = at, at + key
            at = child + 8
            address = self.u(child, 8)
            if level > 0:
                out.extend(self.btree_children(address, kind, rank))
            elif kind == 0:
                out.append(address)
            else:
                offsets = [self.u(k + 8 + 8 * j, 8) for j in range(rank)]
                out.append((address, self.u(k, 4), self.u(k + 4, 4), offsets))
        return out

    # -- datatypes and dataspaces
    def datatype(self, at):
        """(numpy dtype or a tag, size, bytes used) of the datatype message at `at`."""
        d = self.d
        cls, version = d[at] & 0x0F, d[at] >> 4
        bits = d[at + 1] | (d[at + 2] << 8) | (d[at + 3] << 16)
        size = self.u(at + 4, 4)
        props = at + 8
        if cls == 0:  # fixed point
            order = ">" if bits & 1 else "<"
            return np.dtype(f"{order}{'i' if bits & 8 else 'u'}{size}"), size, 12
        if cls == 1:  # floating point
            order = ">" if bits & 1 else "<"
            return np.dtype(f"{order}f{size}"), size, 20
        if cls == 3:  # fixed-length string
            return ("fixed-string", size), size, 8
        if cls == 8:  # enumeration (h5py booleans): the base type's values
            base, _, used = self.datatype(props)
            return base, size, 8 + used  # member names and values are not needed
        if cls == 9:  # variable length
            kind = bits & 0x0F
            base, _, used = self.datatype(props)
            return (("vlen-string",) if kind == 1 else ("vlen", base)), size, 8 + used
        raise ValueError(f"Unsupported HDF5 datatype class {cls} (version {version})")

    def dataspace(self, at):
        d = self.d
        version, rank, flags = d[at], d[at + 1], d[at + 2]
        if version == 1:
            dims_at = at + 8
        elif version == 2:
            dims_at = at + 4
            if d[at + 3] == 2:  # null dataspace
                return None
        else:
            raise ValueError(f"Unsupported dataspace version {version}")
        return tuple(self.u(dims_at + 8 * k, 8) for k in range(rank))

    def vlen_strings(self, at, count):
        out = []
        for k in range(count):
            e = at + 16 * k
            length, collection, index = self.u(e, 4), self.u(e + 4, 8), self.u(e + 12, 4)
            out.append(self.global_object(collection, index)[:length].decode("utf-8"))
        return out

    def global_object(self, collection, index):
        d = self.d
        if d[collection:collection + 4] != b"GCOL":
            raise ValueError("Bad global heap collection")
        size = self.u(collection + 8, 8)
        at, end = collection + 16, collection + size
        while at + 16 <= end:
            obj, length = self.u(at, 2), self.u(at + 8, 8)
            if obj == index:
                return d[at + 16:at + 16 + length]
            if obj == 0:
                break
            at += 16 + (length + 7) // 8 * 8
        raise ValueError("Global heap object not found")

    def decode(self, dtype, shape, at, nbytes=None):
        count = int(np.prod(shape)) if shape else 1
        if isinstance(dtype, tuple) and dtype[0] == "vlen-string":
            values = self.vlen_strings(at, count)
            return values[0] if not shape else np.array(values, dtype=object).reshape(shape)
        if isinstance(dtype, tuple) and dtype[0] == "fixed-string":
            raw = [self.d[at + k * dtype[1]:at + (k + 1) * dtype[1]].split(b"\x00")[0] for k in range(count)]
            return raw[0] if not shape else np.array(raw).reshape(shape)
        array = np.frombuffer(self.d, dtype=dtype, count=count, offset=at).copy()
        return array.reshape(shape) if shape else array[0]

    def attribute(self, at):
        d = self.d
        version = d[at]
        name_size, type_size, space_size = self.u(at + 2, 2), self.u(at + 4, 2), self.u(at + 6, 2)
        if version == 1:
            pad = lambda n: (n + 7) // 8 * 8  # noqa: E731
            p = at + 8
        elif version in (2, 3):
            pad = lambda n: n  # noqa: E731
            p = at + 8 + (1 if version == 3 else 0)
        else:
            raise ValueError(f"Unsupported attribute message version {version}")
        name = self.d[p:p + name_size].split(b"\x00")[0].decode("utf-8")
        p += pad(name_size)
        dtype, _, _ = self.datatype(p)
        p += pad(type_size)
        shape = self.dataspace(p)
        p += pad(space_size)
        return name, self.decode(dtype, shape, p)

    # -- datasets
    def dataset(self, msgs):
        dtype = shape = layout = None
        filters = []
        attrs = {}
        for kind, body, size, flags in msgs:
            if kind == 0x01:
                shape = self.dataspace(body)
            elif kind == 0x03:
                dtype, element, _ = self.datatype(body)
            elif kind == 0x08:
                layout = body
            elif kind == 0x0B:
                filters = self.filter_pipeline(body)
            elif kind == 0x0C:
                name, value = self.attribute(body)
                attrs[name] = value
        if isinstance(dtype, tuple):
            raise ValueError("String datasets are not supported")
        d = self.d
        if d[layout] != 3:
            raise ValueError(f"Unsupported data layout version {d[layout]}")
        cls = d[layout + 1]
        shape = shape or ()
        count = int(np.prod(shape)) if shape else 1
        if cls == 0:  # compact
            size = self.u(layout + 2, 2)
            raw = d[layout + 4:layout + 4 + size]
            return np.frombuffer(raw, dtype=dtype, count=count).reshape(shape).copy()
        if cls == 1:  # contiguous
            address = self.u(layout + 2, 8)
            if address == UNDEFINED:
                return np.zeros(shape, dtype)
            return np.frombuffer(d, dtype=dtype, count=count, offset=address).reshape(shape).copy()
        if cls != 2:
            raise ValueError(f"Unsupported data layout class {cls}")
        rank = d[layout + 2] - 1
        btree = self.u(layout + 3, 8)
        chunk = tuple(self.u(layout + 11 + 4 * k, 4) for k in range(rank))
        out = np.zeros(shape, dtype)
        if btree == UNDEFINED:
            return out
        itemsize = np.dtype(dtype).itemsize
        for address, size, mask, offsets in self.btree_children(btree, 1, rank):
            raw = d[address:address + size]
            for index, (fid, client) in reversed(list(enumerate(filters))):
                if mask & (1 << index):
                    continue
                raw = _unfilter(fid, client, raw, itemsize)
            block = np.frombuffer(raw, dtype=dtype, count=int(np.prod(chunk))).reshape(chunk)
            target = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offsets, chunk, shape))
            out[target] = block[tuple(slice(0, t.stop - t.start) for t in target)]
        return out

    def filter_pipeline(self, at):
        d = self.d
        version, count = d[at], d[at + 1]
        p = at + (8 if version == 1 else 2)
        out = []
        for _ in range(count):
            fid, name_len = self.u(p, 2), 0
            if version == 1 or fid >= 256:
                name_len = self.u(p + 2, 2)
                flags, nvalues = self.u(p + 4, 2), self.u(p + 6, 2)
                p += 8
            else:
                flags, nvalues = self.u(p + 2, 2), self.u(p + 4, 2)
                p += 6
            p += (name_len + 7) // 8 * 8 if version == 1 else name_len
            client = [self.u(p + 4 * k, 4) for k in range(nvalues)]
            p += 4 * nvalues + (4 if version == 1 and nvalues % 2 else 0)
            out.append((fid, client))
        return out


def _unfilter(fid, client, raw, itemsize):
    if fid == 1:  # deflate
        return zlib.decompress(raw)
    if fid == 2:  # shuffle
        n = len(raw) // itemsize
        return np.frombuffer(raw[:n * itemsize], np.uint8).reshape(itemsize, n).T.tobytes() + raw[n * itemsize:]
    if fid == 3:  # Fletcher-32: the checksum is the last four bytes
        return raw[:-4]
    raise ValueError(f"Unsupported HDF5 filter {fid}")


def read(path):
    """The file's root group, every dataset read into memory."""
    with open(path, "rb") as f:
        data = f.read()
    r = _Reader(data)
    return r.object(r.root)


# ------------------------------------------------------------------- writing
GROUP_LEAF_K = 4       # symbol-table node capacity 2K = 8 entries
GROUP_INTERNAL_K = 16  # group B-tree node capacity 2K = 32 children
SNOD_SIZE = 8 + 2 * GROUP_LEAF_K * 40
GROUP_TREE_SIZE = 24 + (2 * GROUP_INTERNAL_K + 1) * 8 + 2 * GROUP_INTERNAL_K * 8
HEAP_FREE_NULL = 1     # the on-disk end of a local heap's free list


def _pad8(b):
    return b + b"\x00" * (-len(b) % 8)


def _datatype(dtype):
    """Datatype message of a numeric numpy dtype (version 1, little endian)."""
    dtype = np.dtype(dtype)
    size = dtype.itemsize
    if dtype.kind == "f":
        exponent, mantissa, bias = {4: (8, 23, 127), 8: (11, 52, 1023)}[size]
        sign = 8 * size - 1
        return (bytes([0x11, 0x20, sign, 0]) + struct.pack("<I", size)
                + struct.pack("<HHBBBBI", 0, 8 * size, mantissa, exponent, 0, mantissa, bias))
    if dtype.kind in "iub":
        signed = 0x08 if dtype.kind == "i" else 0
        return bytes([0x10, signed, 0, 0]) + struct.pack("<I", size) + struct.pack("<HH", 0, 8 * size)
    raise ValueError(f"Unsupported dataset dtype {dtype}")


VLEN_STRING = bytes([0x19, 0x01, 0x01, 0]) + struct.pack("<I", 16) + _datatype(np.uint8)


def _dataspace(shape):
    return bytes([1, len(shape), 0, 0, 0, 0, 0, 0]) + b"".join(struct.pack("<Q", int(n)) for n in shape)


def _message(kind, body):
    body = _pad8(body)
    return struct.pack("<HHB3x", kind, len(body), 0) + body


class _Writer:
    def __init__(self):
        self.buf = bytearray(b"\x00" * 96)  # superblock, filled last
        self.strings = {}                   # str -> global heap object index
        self.gcol = None

    def alloc(self, data):
        address = len(self.buf)
        self.buf += _pad8(bytes(data))
        return address

    def collect_strings(self, group):
        for value in group.attrs.values():
            if isinstance(value, str):
                self.strings.setdefault(value, len(self.strings) + 1)
        for member in group.members.values():
            if isinstance(member, Group):
                self.collect_strings(member)

    def global_heap(self):
        objects = b""
        for text, index in self.strings.items():
            data = text.encode("utf-8")
            objects += struct.pack("<HH4xQ", index, 0, len(data)) + _pad8(data)
        size = max(4096, 16 + len(objects) + 16)
        free = size - 16 - len(objects)
        body = b"GCOL" + bytes([1, 0, 0, 0]) + struct.pack("<Q", size) + objects
        body += struct.pack("<HH4xQ", 0, 0, free) + b"\x00" * (free - 16)
        self.gcol = self.alloc(body)

    def attribute(self, name, value):
        if isinstance(value, str):
            data = value.encode("utf-8")
            dtype, space = VLEN_STRING, _dataspace(())
            raw = struct.pack("<IQI", len(data), self.gcol, self.strings[value])
        else:
            array = np.asarray(value)
            if array.dtype == bool:
                array = array.astype(np.int8)
            elif array.dtype.kind == "i":
                array = array.astype(np.int64)
            elif array.dtype.kind == "u":
                array = array.astype(np.uint64)
            elif array.dtype.kind == "f":
                array = array.astype(np.float64)
            dtype, space, raw = _datatype(array.dtype), _dataspace(array.shape), array.astype(array.dtype.newbyteorder("<")).tobytes()
        encoded = name.encode("utf-8") + b"\x00"
        head = struct.pack("<BxHHH", 1, len(encoded), len(dtype), len(space))
        return _message(0x0C, head + _pad8(encoded) + _pad8(dtype) + _pad8(space) + raw)

    def header(self, messages):
        body = b"".join(messages)
        if len(body) < 24:  # leave room as libhdf5's own headers do
            body += _message(0x0000, b"\x00" * (16 - 8))
        count = len(messages) + (1 if len(b"".join(messages)) < 24 else 0)
        return self.alloc(struct.pack("<BxHII4x", 1, count, 1, len(body)) + body)

    def dataset(self, array, compress):
        array = np.ascontiguousarray(array)
        if array.dtype.byteorder == ">":
            array = array.astype(array.dtype.newbyteorder("<"))
        messages = [_message(0x01, _dataspace(array.shape)), _message(0x03, _datatype(array.dtype)),
                    _message(0x05, bytes([2, 1, 2, 0]))]
        if compress and array.size:
            rows = max(1, min(array.shape[0], (1 << 20) // max(1, array[0:1].nbytes)))
            chunk = (rows, *array.shape[1:])
            messages.append(_message(0x0B, bytes([1, 1, 0, 0, 0, 0, 0, 0])
                                     + struct.pack("<HHHH", 1, 8, 1, 1) + _pad8(b"deflate\x00")
                                     + struct.pack("<I4x", 6)))
            tree = self.chunk_tree(array, chunk)
            dims = b"".join(struct.pack("<I", c) for c in (*chunk, array.itemsize))
            layout = bytes([3, 2, array.ndim + 1]) + struct.pack("<Q", tree) + dims
        else:
            address = self.alloc(array.tobytes()) if array.size else UNDEFINED
            layout = bytes([3, 1]) + struct.pack("<QQ", address, array.nbytes)
        messages.append(_message(0x08, layout))
        return self.header(messages)

    def chunk_tree(self, array, chunk):
        """Chunks along the first axis, each deflated, under one B-tree node
        (or a two-level tree when there are more than 64 chunks)."""
        entries = []
        for start in range(0, array.shape[0], chunk[0]):
            block = np.zeros(chunk, array.dtype)
            part = array[start:start + chunk[0]]
            block[:len(part)] = part
            data = zlib.compress(block.tobytes(), 6)
            offsets = (start, *([0] * (array.ndim - 1)), 0)
            entries.append((self.alloc(data), len(data), offsets))
        return self.chunk_node(entries, array.ndim + 1, array.shape)

    def chunk_node(self, entries, rank, shape, level=0, fanout=64):
        if len(entries) > fanout:
            children = [entries[i:i + fanout] for i in range(0, len(entries), fanout)]
            nodes = [(self.chunk_node(c, rank, shape, level, fanout), 0, c[0][2]) for c in children]
            return self.chunk_node(nodes, rank, shape, level + 1, fanout)
        key = lambda size, offsets: struct.pack("<II", size, 0) + b"".join(  # noqa: E731
            struct.pack("<Q", o) for o in offsets)
        body = b"TREE" + bytes([1, level]) + struct.pack("<HQQ", len(entries), UNDEFINED, UNDEFINED)
        for address, size, offsets in entries:
            body += key(size, offsets) + struct.pack("<Q", address)
        end = (shape[0], *([0] * (rank - 1)))
        body += key(0, end)
        full = 24 + (2 * fanout + 1) * (8 + 8 * rank) + 2 * fanout * 8
        return self.alloc(body + b"\x00" * (full - len(body)))

    def group(self, group, compress):
        names = sorted(group.members)
        addresses = {}
        for name in names:
            member = group.members[name]
            if isinstance(member, Group):
                addresses[name] = self.group(member, compress)
            else:
                addresses[name] = (self.dataset(member, compress), None)
        # Local heap: the empty string at offset 0, then every name.
        heap_data, offsets = b"\x00" * 8, {}
        for name in names:
            offsets[name] = len(heap_data)
            heap_data += _pad8(name.encode("utf-8") + b"\x00")
        heap_data += b"\x00" * 8
        data_address = self.alloc(heap_data)
        heap = self.alloc(b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(heap_data), HEAP_FREE_NULL,
                                                                     data_address))
        # Symbol nodes of at most 2K entries each, names in order.
        per = 2 * GROUP_LEAF_K
        snods = []
        for i in range(0, max(len(names), 1), per):
            chunk = names[i:i + per]
            body = b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(chunk))
            for name in chunk:
                header, cache = addresses[name]
                body += self.entry(offsets[name], header, cache)
            snods.append((self.alloc(body + b"\x00" * (SNOD_SIZE - len(body))), offsets[chunk[-1]] if chunk else 0))
            if not chunk:
                break
        if len(snods) > 2 * GROUP_INTERNAL_K:
            raise ValueError("Groups of more than 256 members are not supported")
        body = b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", len(snods) if names else 0, UNDEFINED, UNDEFINED)
        body += struct.pack("<Q", 0)
        for address, last in (snods if names else []):
            body += struct.pack("<QQ", address, last)
        tree = self.alloc(body + b"\x00" * (GROUP_TREE_SIZE - len(body)))
        messages = [_message(0x11, struct.pack("<QQ", tree, heap))]
        messages += [self.attribute(k, v) for k, v in group.attrs.items()]
        return self.header(messages), (tree, heap)

    @staticmethod
    def entry(name_offset, header, cache):
        if cache is None:
            return struct.pack("<QQII16x", name_offset, header, 0, 0)
        return struct.pack("<QQIIQQ", name_offset, header, 1, 0, *cache)

    def finish(self, root):
        header, cache = root
        sb = SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", GROUP_LEAF_K, GROUP_INTERNAL_K, 0)
        sb += struct.pack("<QQQQ", 0, UNDEFINED, len(self.buf), UNDEFINED)
        sb += self.entry(0, header, cache)
        self.buf[:96] = sb
        return bytes(self.buf)


def write(path, root, *, compress=False):
    """Write a :class:`Group` tree (datasets as numpy arrays; attributes as
    str, int, float, bool or numpy values); ``compress`` stores datasets as
    deflated chunks, as h5py's ``compression="gzip"`` does."""
    w = _Writer()
    w.collect_strings(root)
    if w.strings:
        w.global_heap()
    data = w.finish(w.group(root, compress))
    with open(path, "wb") as f:
        f.write(data)
