"""HDF5 files without h5py: a writer and a reader for the subset of the
format that the measurement products need.

The reference writes its products with h5py (``write_data.py:1-56``), whose
default ('earliest') file layout is what this module produces: superblock
version 0 (offsets and lengths of 8 bytes, group leaf node K = 4, group
internal node K = 16), version-1 object headers, groups as symbol tables (a
version-1 B-tree of symbol-table nodes, names in a local heap; group entries
cache the B-tree and heap addresses), and datasets with a version-1
dataspace (current = maximum dimensions), an IEEE float or two's-complement
integer datatype, a version-2 fill-value message and contiguous storage
(layout message version 3).  Every structure follows the public HDF5 file
format specification; the conventions h5py leaves in such files (the local
heap's trailing free block, B-tree nodes allocated for 2K children, the
datatype and fill messages marked constant) are kept so that the files look
like h5py's.

The reader covers the same layout plus what h5py and the HDF5 library write
into it: continuation messages, B-trees of several levels, compact storage,
version-2 dataspaces, and chunked storage (version-1 chunk B-tree) with the
deflate, shuffle and fletcher32 filters.  Anything else raises
``NotImplementedError``.  The writer can store a dataset chunked and
deflate-compressed (``chunks=``); no HDF5 library exists on the hosts this was
built on, so chunked files have only been read back by this module.
"""

from __future__ import annotations

import functools
import mmap
import os
import struct
import threading
import zlib

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b"\x89HDF\r\n\x1a\n"
LEAF_K = 4                       # symbols per symbol-table node: 2 * LEAF_K
NODE_K = 16                      # children per group B-tree node: 2 * NODE_K
SNOD_BYTES = 8 + 2 * LEAF_K * 40
BTREE_BYTES = 24 + (2 * NODE_K + 1) * 8 + 2 * NODE_K * 8
FREE_NULL = 1                    # end of a local heap's free list
SUPERBLOCK_BYTES = 96

_MSG_DATASPACE, _MSG_DATATYPE, _MSG_FILL, _MSG_LAYOUT = 0x0001, 0x0003, 0x0005, 0x0008
_MSG_FILTERS, _MSG_CONTINUATION, _MSG_SYMBOL_TABLE = 0x000B, 0x0010, 0x0011
CHUNK_K = 32                     # indexed-storage K of superblock version 0: 2K chunks per B-tree node
FILTER_DEFLATE, FILTER_SHUFFLE, FILTER_FLETCHER32 = 1, 2, 3


def _pad8(n):
    return (n + 7) & ~7


# ----------------------------------------------------------------------------
# writer
# ----------------------------------------------------------------------------

def _datatype(dt: np.dtype) -> bytes:
    if dt.kind == "f" and dt.itemsize in (4, 8):
        if dt.itemsize == 8:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
            sign = 63
        else:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
            sign = 31
        # class 1 (floating point), version 1; little endian, mantissa msb implied
        return bytes([0x11, 0x20, sign, 0x00]) + struct.pack("<I", dt.itemsize) + props
    if dt.kind in "iu" and dt.itemsize in (1, 2, 4, 8):
        bits = 0x08 if dt.kind == "i" else 0x00
        return bytes([0x10, bits, 0x00, 0x00]) + struct.pack("<IHH", dt.itemsize, 0, 8 * dt.itemsize)
    raise TypeError(f"dtype {dt} is not supported by the HDF5 writer")


def _dataspace(shape) -> bytes:
    rank = len(shape)
    head = struct.pack("<BBBBI", 1, rank, 1 if rank else 0, 0, 0)
    dims = b"".join(struct.pack("<Q", int(d)) for d in shape)
    return head + dims + dims


def _message(mtype, data, flags=0) -> bytes:
    body = data + b"\0" * (_pad8(len(data)) - len(data))
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _object_header(messages) -> bytes:
    body = b"".join(messages)
    return struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(body)) + body


class _Image:
    """The file as a growing byte array; every allocation is 8-byte aligned."""

    def __init__(self):
        self.b = bytearray(SUPERBLOCK_BYTES)

    def alloc(self, n):
        a = len(self.b)
        self.b += b"\0" * _pad8(n)
        return a

    def put(self, addr, data):
        self.b[addr:addr + len(data)] = data


def _entry(name_off, header, scratch=None) -> bytes:
    if scratch is None:
        return struct.pack("<QQII16x", name_off, header, 0, 0)
    return struct.pack("<QQIIQQ", name_off, header, 1, 0, *scratch)


def _write_chunked(img: _Image, v: np.ndarray, dt: np.dtype, chunk_rows: int, level: int) -> int:
    """A dataset split into chunks of ``chunk_rows`` rows, each shuffled and
    deflated, indexed by a version-1 chunk B-tree (leaves of up to 2K chunks)."""
    if v.ndim == 0:
        raise ValueError("a scalar cannot be chunked")
    a = np.ascontiguousarray(v, dtype=dt)
    rows = max(1, int(chunk_rows))
    cdims = [rows] + list(a.shape[1:])
    esize = dt.itemsize
    rank = a.ndim
    chunks = []
    for r0 in range(0, max(a.shape[0], 1), rows):
        block = np.zeros(cdims, dtype=dt)
        part = a[r0:r0 + rows]
        block[:len(part)] = part
        raw = block.tobytes()
        shuffled = np.frombuffer(raw, np.uint8).reshape(-1, esize).T.tobytes()
        data = zlib.compress(shuffled, level)
        at = img.alloc(len(data))
        img.put(at, data)
        chunks.append((r0, at, len(data)))
    nodes = []
    per = 2 * CHUNK_K
    key_bytes = 8 + 8 * (rank + 1)

    def key(size, r0):
        return struct.pack("<II", size, 0) + struct.pack("<Q", r0) + b"\0" * (8 * rank)

    groups = [chunks[i:i + per] for i in range(0, len(chunks), per)] or [[]]
    node_bytes = 24 + (2 * per + 1) * key_bytes
    addrs = [img.alloc(node_bytes) for _ in groups]
    for j, g in enumerate(groups):
        left = addrs[j - 1] if j > 0 else UNDEF
        right = addrs[j + 1] if j + 1 < len(groups) else UNDEF
        body = b""
        for r0, at, size in g:
            body += key(size, r0) + struct.pack("<Q", at)
        end = (g[-1][0] + rows) if g else 0
        body += key(0, end)
        img.put(addrs[j], b"TREE" + struct.pack("<BBHQQ", 1, 0, len(g), left, right) + body)
        nodes.append((addrs[j], g[0][0] if g else 0))
    if len(nodes) > 1:
        top = img.alloc(node_bytes)
        body = b""
        for at, r0 in nodes:
            body += key(0, r0) + struct.pack("<Q", at)
        body += key(0, (chunks[-1][0] + rows))
        img.put(top, b"TREE" + struct.pack("<BBHQQ", 1, 1, len(nodes), UNDEF, UNDEF) + body)
        root = top
    else:
        root = nodes[0][0]
    filt = struct.pack("<BB6x", 1, 2)
    filt += struct.pack("<HHHH", FILTER_SHUFFLE, 0, 1, 1) + struct.pack("<I", esize) + b"\0" * 4
    filt += struct.pack("<HHHH", FILTER_DEFLATE, 0, 1, 1) + struct.pack("<I", level) + b"\0" * 4
    layout = struct.pack("<BBBQ", 3, 2, rank + 1, root) + b"".join(struct.pack("<I", d) for d in cdims + [esize])
    hdr = _object_header([
        _message(_MSG_DATASPACE, _dataspace(v.shape)),
        _message(_MSG_DATATYPE, _datatype(np.dtype(dt)), flags=1),
        _message(_MSG_FILL, bytes([2, 2, 2, 1]) + struct.pack("<I", 0), flags=1),
        _message(_MSG_FILTERS, filt),
        _message(_MSG_LAYOUT, layout)])
    addr = img.alloc(len(hdr))
    img.put(addr, hdr)
    return addr


@functools.lru_cache(maxsize=256)
def _contiguous_header(shape, dtype_str):
    """Object header of a contiguous dataset of this shape and type, with the
    layout message's address and size left to fill in: (bytes, offset of the
    address field).  Datasets of one shape and type share everything else."""
    dt = np.dtype(dtype_str)
    hdr = _object_header([
        _message(_MSG_DATASPACE, _dataspace(shape)),
        _message(_MSG_DATATYPE, _datatype(dt), flags=1),
        _message(_MSG_FILL, bytes([2, 2, 2, 1]) + struct.pack("<I", 0), flags=1),
        _message(_MSG_LAYOUT, struct.pack("<BBQQ", 3, 1, UNDEF, 0))])
    # the layout message is last: its data (version, class, address, size) ends
    # the header after 6 bytes of padding to 8
    return hdr, len(hdr) - 6 - 16


def _le(dtype):
    """The little-endian form of a dataset's type (the file's byte order)."""
    return dtype.newbyteorder("<") if dtype.byteorder != "|" else dtype


def _write_dataset(img: _Image, value: np.ndarray, chunks=None, slots=None, path=None) -> int:
    v = np.asarray(value)
    if v.dtype.kind == "b":
        raise TypeError("boolean datasets are not supported by the HDF5 writer")
    dt = _le(v.dtype)
    hdr, at = _contiguous_header(tuple(int(d) for d in v.shape), np.dtype(dt).str)
    if chunks:
        return _write_chunked(img, v, np.dtype(dt), chunks, 4)
    raw = np.ascontiguousarray(v, dtype=dt).tobytes()
    addr = img.alloc(len(hdr))
    data_at = img.alloc(len(raw)) if raw else UNDEF   # an empty dataset has no storage
    img.put(addr, hdr)
    struct.pack_into("<QQ", img.b, addr + at, data_at, len(raw))
    if raw:
        img.put(data_at, raw)
        if slots is not None:
            slots.append((path, data_at, len(raw)))
    return addr


def _write_group(img: _Image, children: dict, chunks=None, slots=None, prefix=()) -> tuple[int, int, int]:
    """Writes a group and (recursively) its members; returns the addresses
    of its object header, B-tree root and local heap.  ``slots`` collects
    (member path, data address, bytes) of every contiguous dataset."""
    names = sorted(children, key=lambda s: s.encode())
    # member objects first, so that their entries can be filled in
    entries = {}
    for n in names:
        c = children[n]
        if isinstance(c, dict):
            h, bt, hp = _write_group(img, c, chunks, slots, prefix + (n,))
            entries[n] = (h, (bt, hp))
        else:
            entries[n] = (_write_dataset(img, c, chunks, slots, prefix + (n,)), None)
    # local heap: "" at offset 0, the names, then one free block
    heap_data = bytearray(b"\0" * 8)
    offs = {}
    for n in names:
        offs[n] = len(heap_data)
        enc = n.encode() + b"\0"
        heap_data += enc + b"\0" * (_pad8(len(enc)) - len(enc))
    free_at = len(heap_data)
    heap_data += struct.pack("<QQ", FREE_NULL, 16)
    heap = img.alloc(32)
    heap_seg = img.alloc(len(heap_data))
    img.put(heap, b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(heap_data), free_at, heap_seg))
    img.put(heap_seg, bytes(heap_data))
    # symbol-table nodes of up to 2 * LEAF_K entries each, in name order
    per = 2 * LEAF_K
    leaves = []
    for i in range(0, len(names), per):
        chunk = names[i:i + per]
        at = img.alloc(SNOD_BYTES)
        body = b"".join(_entry(offs[n], entries[n][0], entries[n][1]) for n in chunk)
        img.put(at, b"SNOD" + struct.pack("<BBH", 1, 0, len(chunk)) + body)
        leaves.append((at, offs[chunk[-1]]))          # (address, heap offset of its largest name)
    # B-tree levels of up to 2 * NODE_K children until one root remains
    level = 0
    nodes = leaves
    while True:
        groups = [nodes[i:i + 2 * NODE_K] for i in range(0, len(nodes), 2 * NODE_K)] or [[]]
        addrs = [img.alloc(BTREE_BYTES) for _ in groups]
        parents = []
        left_key = 0
        for j, g in enumerate(groups):
            left = addrs[j - 1] if j > 0 else UNDEF
            right = addrs[j + 1] if j + 1 < len(groups) else UNDEF
            body = struct.pack("<Q", left_key)
            for child, key in g:
                body += struct.pack("<QQ", child, key)
            img.put(addrs[j], b"TREE" + struct.pack("<BBHQQ", 0, level, len(g), left, right) + body)
            top_key = g[-1][1] if g else 0
            parents.append((addrs[j], top_key))
            left_key = top_key
        if len(parents) == 1:
            btree = parents[0][0]
            break
        nodes = parents
        level += 1
    hdr = _object_header([_message(_MSG_SYMBOL_TABLE, struct.pack("<QQ", btree, heap))])
    h = img.alloc(len(hdr))
    img.put(h, hdr)
    return h, btree, heap


def _tree(datasets: dict) -> dict:
    root: dict = {}
    for path, value in datasets.items():
        parts = [p for p in path.split("/") if p]
        if not parts:
            raise ValueError("empty dataset path")
        node = root
        for p in parts[:-1]:
            nxt = node.setdefault(p, {})
            if not isinstance(nxt, dict):
                raise ValueError(f"'{p}' in '{path}' is a dataset, not a group")
            node = nxt
        if isinstance(node.get(parts[-1]), dict):
            raise ValueError(f"'{path}' is a group")
        node[parts[-1]] = np.asarray(value)
    return root


# file images of recent contiguous writes, by their layout key: every byte of
# the file but the datasets' data depends only on the member paths, shapes and
# types, so a write of the same products again (a measurement repeated into
# one file) copies the image and places the new data at the recorded addresses
_IMAGES: dict = {}
_IMAGES_MAX = 8
_IMAGES_LOCK = threading.Lock()


def _image(datasets: dict, chunks):
    if chunks:
        img = _Image()
        h, bt, hp = _write_group(img, _tree(datasets), chunks)
        return _finish(img, h, bt, hp)
    vals = {p: np.asarray(v) for p, v in datasets.items()}
    key = tuple(sorted((p, v.shape, _le(v.dtype).str) for p, v in vals.items()))
    with _IMAGES_LOCK:
        hit = _IMAGES.get(key)
    if hit is not None:
        template, slots = hit
        b = bytearray(template)
        for p, at, n in slots:
            v = vals[p]
            b[at:at + n] = np.ascontiguousarray(v, dtype=_le(v.dtype)).tobytes()
        return b
    img = _Image()
    slots = []
    h, bt, hp = _write_group(img, _tree(vals), None, slots)
    b = _finish(img, h, bt, hp)
    flat = {tuple(q for q in p.split("/") if q): p for p in vals}
    entry = (bytes(b), [(flat[path], at, n) for path, at, n in slots])
    with _IMAGES_LOCK:
        while len(_IMAGES) >= _IMAGES_MAX:
            _IMAGES.pop(next(iter(_IMAGES)))
        _IMAGES[key] = entry
    return b


def _finish(img: _Image, h, bt, hp) -> bytearray:
    sb = SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", LEAF_K, NODE_K, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, len(img.b), UNDEF) + _entry(0, h, (bt, hp))
    img.put(0, sb)
    return img.b


def write_file(path, datasets: dict, chunks=None) -> None:
    """Writes ``{'group/sub/name': array}`` as a new HDF5 file at ``path``
    (replacing it atomically: the file appears complete or not at all).
    ``chunks=n`` stores every non-scalar dataset in chunks of n rows,
    shuffled and deflate-compressed."""
    b = _image(datasets, chunks)
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "wb") as f:
        f.write(b)
    os.replace(tmp, path)


# ----------------------------------------------------------------------------
# reader
# ----------------------------------------------------------------------------

class _Reader:
    def __init__(self, data: bytes):
        self.b = data
        if data[:8] != SIGNATURE:
            raise ValueError("not an HDF5 file")
        ver = data[8]
        if ver not in (0, 1):
            raise NotImplementedError(f"superblock version {ver}")
        if data[13] != 8 or data[14] != 8:
            raise NotImplementedError("offsets or lengths other than 8 bytes")
        root = 24 + (4 if ver == 1 else 0) + 32
        self.root = self.u("Q", root + 8)[0]

    def u(self, fmt, off):
        return struct.unpack_from("<" + fmt, self.b, off)

    def messages(self, addr):
        if self.b[addr] != 1:
            raise NotImplementedError(f"object header version {self.b[addr]}")
        nmsg, = self.u("H", addr + 2)
        size, = self.u("I", addr + 8)
        blocks, out = [(addr + 16, size)], []
        while blocks and len(out) < nmsg:
            start, length = blocks.pop(0)
            p = start
            while p + 8 <= start + length and len(out) < nmsg:
                mtype, msize = self.u("HH", p)
                if mtype == _MSG_CONTINUATION:
                    blocks.append(self.u("QQ", p + 8))
                out.append((mtype, p + 8, msize))
                p += 8 + msize
        return out

    def name(self, heap, off):
        if self.b[heap:heap + 4] != b"HEAP":
            raise ValueError("bad local heap")
        seg, = self.u("Q", heap + 24)
        s = seg + off
        return bytes(self.b[s:self.b.find(b"\0", s)]).decode()

    def members(self, btree, heap):
        out, stack = {}, [btree]
        while stack:
            node = stack.pop()
            if self.b[node:node + 4] != b"TREE" or self.b[node + 4] != 0:
                raise ValueError("bad group B-tree node")
            level, used = self.b[node + 5], self.u("H", node + 6)[0]
            for k in range(used):
                child, = self.u("Q", node + 32 + 16 * k)
                if level > 0:
                    stack.append(child)
                    continue
                if self.b[child:child + 4] != b"SNOD":
                    raise ValueError("bad symbol-table node")
                for s in range(self.u("H", child + 6)[0]):
                    e = child + 8 + 40 * s
                    name_off, hdr = self.u("QQ", e)
                    out[self.name(heap, name_off)] = hdr
        return out

    def dataset(self, msgs):
        t = {m[0]: m for m in msgs}
        _, d, _ = t[_MSG_DATASPACE]
        ver, rank = self.b[d], self.b[d + 1]
        if ver == 2 and self.b[d + 3] == 2:
            return np.zeros(0)                      # null dataspace
        dims_at = d + (8 if ver == 1 else 4)
        shape = tuple(self.u("Q", dims_at + 8 * i)[0] for i in range(rank))
        _, a, _ = t[_MSG_DATATYPE]
        cls, bits, size = self.b[a] & 0x0F, self.b[a + 1], self.u("I", a + 4)[0]
        order = ">" if bits & 1 else "<"
        if cls == 1:
            dt = np.dtype(f"{order}f{size}")
        elif cls == 0:
            dt = np.dtype(f"{order}{'i' if bits & 0x08 else 'u'}{size}")
        else:
            raise NotImplementedError(f"datatype class {cls}")
        _, lay, _ = t[_MSG_LAYOUT]
        if self.b[lay] != 3:
            raise NotImplementedError(f"layout message version {self.b[lay]}")
        n = int(np.prod(shape)) if rank else 1
        if self.b[lay + 1] == 2:
            return self._chunked(t, lay, shape, dt)
        if self.b[lay + 1] == 1:
            addr, _ = self.u("QQ", lay + 2)
            raw = b"" if addr == UNDEF else self.b[addr:addr + n * size]
            if addr == UNDEF:
                return np.zeros(shape, dt.newbyteorder("="))
        elif self.b[lay + 1] == 0:
            nbytes, = self.u("H", lay + 2)
            raw = self.b[lay + 4:lay + 4 + nbytes]
        else:
            raise NotImplementedError(f"layout class {self.b[lay + 1]}")
        return np.frombuffer(raw, dtype=dt, count=n).reshape(shape).astype(dt.newbyteorder("="))

    def _filters(self, t):
        """[(filter id, client data)] of the filter pipeline message, in order."""
        if _MSG_FILTERS not in t:
            return []
        _, p, _ = t[_MSG_FILTERS]
        ver, nf = self.b[p], self.b[p + 1]
        q = p + (8 if ver == 1 else 2)
        out = []
        for _ in range(nf):
            fid, = self.u("H", q)
            q += 2
            nlen = 0
            if ver == 1 or fid >= 256:
                nlen, = self.u("H", q)
                q += 2
            _flags, ncd = self.u("HH", q)
            q += 4
            if ver == 1:
                q += (nlen + 7) & ~7
            else:
                q += nlen
            cd = list(self.u(f"{ncd}I", q)) if ncd else []
            q += 4 * ncd
            if ver == 1 and ncd % 2:
                q += 4
            out.append((fid, cd))
        return out

    def _chunked(self, t, lay, shape, dt):
        dims = self.b[lay + 2]
        btree, = self.u("Q", lay + 3)
        cd = [self.u("I", lay + 11 + 4 * i)[0] for i in range(dims)]
        cdims, esize = cd[:-1], cd[-1]
        rank = len(shape)
        filters = self._filters(t)
        out = np.zeros(shape, dtype=dt.newbyteorder("="))
        if btree == UNDEF:
            return out
        key_bytes = 8 + 8 * dims
        stack = [btree]
        while stack:
            node = stack.pop()
            if self.b[node:node + 4] != b"TREE" or self.b[node + 4] != 1:
                raise ValueError("bad chunk B-tree node")
            level, used = self.b[node + 5], self.u("H", node + 6)[0]
            p = node + 24
            for _ in range(used):
                size, mask = self.u("II", p)
                offs = self.u(f"{rank}Q", p + 8)
                child, = self.u("Q", p + key_bytes)
                p += key_bytes + 8
                if level > 0:
                    stack.append(child)
                    continue
                raw = self.b[child:child + size]
                for k in range(len(filters) - 1, -1, -1):
                    fid, cdv = filters[k]
                    if mask & (1 << k):
                        continue
                    if fid == FILTER_DEFLATE:
                        raw = zlib.decompress(raw)
                    elif fid == FILTER_SHUFFLE:
                        es = cdv[0] if cdv else esize
                        a = np.frombuffer(raw, np.uint8)
                        m = len(a) // es
                        raw = a[:m * es].reshape(es, m).T.tobytes() + a[m * es:].tobytes()
                    elif fid == FILTER_FLETCHER32:
                        raw = raw[:-4]
                    else:
                        raise NotImplementedError(f"HDF5 filter {fid}")
                block = np.frombuffer(raw, dtype=dt, count=int(np.prod(cdims))).reshape(cdims)
                sl_out = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cdims, shape))
                sl_in = tuple(slice(0, x.stop - x.start) for x in sl_out)
                out[sl_out] = block[sl_in]
        return out


class File:
    """Read access to one HDF5 file by dataset path, the file memory-mapped
    (a dataset's bytes are read when it is asked for)."""

    def __init__(self, path):
        self._f = open(path, "rb")
        try:
            self._m = mmap.mmap(self._f.fileno(), 0, access=mmap.ACCESS_READ)
            self.r = _Reader(self._m)
        except Exception:
            self.close()
            raise

    def close(self):
        for x in ("_m", "_f"):
            obj = getattr(self, x, None)
            if obj is not None:
                obj.close()
                setattr(self, x, None)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _find(self, path):
        addr = self.r.root
        for part in [p for p in str(path).split("/") if p]:
            msgs = self.r.messages(addr)
            st = [m for m in msgs if m[0] == _MSG_SYMBOL_TABLE]
            if not st:
                raise KeyError(f"'{path}': '{part}' is inside a dataset")
            members = self.r.members(*self.r.u("QQ", st[0][1]))
            if part not in members:
                raise KeyError(f"Unable to open object '{part}' (no such member in '{path}')")
            addr = members[part]
        return addr

    def keys(self, group=""):
        msgs = self.r.messages(self._find(group))
        st = [m for m in msgs if m[0] == _MSG_SYMBOL_TABLE]
        if not st:
            raise KeyError(f"'{group}' is not a group")
        return sorted(self.r.members(*self.r.u("QQ", st[0][1])))

    def __contains__(self, path):
        try:
            self._find(path)
            return True
        except KeyError:
            return False

    def read(self, path):
        msgs = self.r.messages(self._find(path))
        if not any(m[0] == _MSG_LAYOUT for m in msgs):
            raise KeyError(f"'{path}' is not a dataset")
        return self.r.dataset(msgs)

    def contiguous_extent(self, path):
        """(file offset, bytes, dtype, shape) of a contiguous dataset, else None."""
        msgs = self.r.messages(self._find(path))
        t = {m[0]: m for m in msgs}
        if _MSG_LAYOUT not in t or _MSG_FILTERS in t:
            return None
        _, lay, _ = t[_MSG_LAYOUT]
        if self.r.b[lay] != 3 or self.r.b[lay + 1] != 1:
            return None
        addr, nbytes = self.r.u("QQ", lay + 2)
        if addr == UNDEF:
            return None
        _, d, _ = t[_MSG_DATASPACE]
        ver, rank = self.r.b[d], self.r.b[d + 1]
        dims_at = d + (8 if ver == 1 else 4)
        shape = tuple(self.r.u("Q", dims_at + 8 * i)[0] for i in range(rank))
        _, a, _ = t[_MSG_DATATYPE]
        cls, bits, size = self.r.b[a] & 0x0F, self.r.b[a + 1], self.r.u("I", a + 4)[0]
        order = ">" if bits & 1 else "<"
        if cls == 1:
            dt = np.dtype(f"{order}f{size}")
        elif cls == 0:
            dt = np.dtype(f"{order}{'i' if bits & 0x08 else 'u'}{size}")
        else:
            return None
        return addr, nbytes, dt, shape


def read_file(path) -> dict:
    """``{'group/sub/name': array}`` for every dataset in an HDF5 file."""
    with open(path, "rb") as f:
        r = _Reader(f.read())
    out, stack, seen = {}, [("", r.root)], set()
    while stack:
        prefix, addr = stack.pop()
        if addr in seen:
            continue
        seen.add(addr)
        msgs = r.messages(addr)
        st = [m for m in msgs if m[0] == _MSG_SYMBOL_TABLE]
        if st:
            btree, heap = r.u("QQ", st[0][1])
            for n, hdr in r.members(btree, heap).items():
                stack.append((f"{prefix}/{n}" if prefix else n, hdr))
        elif any(m[0] == _MSG_LAYOUT for m in msgs):
            out[prefix] = r.dataset(msgs)
    return out
