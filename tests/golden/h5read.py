"""Minimal read-only HDF5 parser for the reference's golden output files.

Covers what h5py's default ('earliest') file layout uses for those files:
superblock version 0/1, version-1 object headers with continuation blocks,
old-style groups (symbol-table message, v1 B-tree of SNOD nodes, local
heap), dataspace messages v1/v2, fixed-point and IEEE floating-point
datatypes, and data-layout message v3 with contiguous or compact storage.
Anything else raises ``NotImplementedError``.  Used only to turn the
reference's golden files into npz fixtures (``make_golden.py``).
"""

from __future__ import annotations

import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


class _H5:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.b = f.read()
        if self.b[:8] != b"\x89HDF\r\n\x1a\n":
            raise ValueError("not an HDF5 file")
        sb_ver = self.b[8]
        if sb_ver not in (0, 1):
            raise NotImplementedError(f"superblock version {sb_ver}")
        self.so = self.b[13]
        self.sl = self.b[14]
        if self.so != 8 or self.sl != 8:
            raise NotImplementedError("offset/length sizes other than 8")
        pos = 24 + (4 if sb_ver == 1 else 0)
        pos += 8 * 4  # base, free-space, end-of-file, driver info
        self.root_entry = self._entry(pos)

    def u(self, fmt, off):
        return struct.unpack_from("<" + fmt, self.b, off)

    def _entry(self, off):
        name_off, hdr, cache = self.u("QQI", off)
        scratch = self.b[off + 24: off + 40]
        return dict(name_off=name_off, hdr=hdr, cache=cache, scratch=scratch)

    def messages(self, addr):
        ver = self.b[addr]
        if ver != 1:
            raise NotImplementedError(f"object header version {ver}")
        nmsg, = self.u("H", addr + 2)
        size, = self.u("I", addr + 8)
        blocks = [(addr + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            start, length = blocks.pop(0)
            p = start
            while p + 8 <= start + length and len(out) < nmsg:
                mtype, msize, flags = self.u("HHB", p)
                data = p + 8
                if mtype == 0x10:
                    caddr, clen = self.u("QQ", data)
                    blocks.append((caddr, clen))
                out.append((mtype, data, msize))
                p = data + msize
        return out

    def heap_name(self, heap_addr, off):
        if self.b[heap_addr:heap_addr + 4] != b"HEAP":
            raise ValueError("bad local heap")
        data_addr, = self.u("Q", heap_addr + 24)
        s = data_addr + off
        e = self.b.index(b"\x00", s)
        return self.b[s:e].decode()

    def group_children(self, btree, heap):
        out = {}
        stack = [btree]
        while stack:
            node = stack.pop()
            if self.b[node:node + 4] != b"TREE":
                raise ValueError("bad B-tree node")
            ntype, level, nused = self.b[node + 4], self.b[node + 5], self.u("H", node + 6)[0]
            if ntype != 0:
                raise NotImplementedError("chunk B-tree")
            p = node + 8 + 16 + 8  # header, siblings, key 0
            for _ in range(nused):
                child, = self.u("Q", p)
                p += 16  # child + next key
                if level > 0:
                    stack.append(child)
                else:
                    if self.b[child:child + 4] != b"SNOD":
                        raise ValueError("bad symbol node")
                    nsym, = self.u("H", child + 6)
                    for k in range(nsym):
                        ent = self._entry(child + 8 + 40 * k)
                        out[self.heap_name(heap, ent["name_off"])] = ent
        return out

    def read_object(self, addr):
        msgs = self.messages(addr)
        types = {m[0]: m for m in msgs}
        if 0x11 in types:
            btree, heap = self.u("QQ", types[0x11][1])
            return "group", self.group_children(btree, heap)
        if 0x0008 in types:
            return "dataset", self._dataset(types)
        return "other", None

    def _dataset(self, types):
        _, d, _ = types[0x0001]
        ver = self.b[d]
        ndim = self.b[d + 1]
        flags = self.b[d + 2]
        p = d + (8 if ver == 1 else 4)
        shape = tuple(self.u("Q", p + 8 * i)[0] for i in range(ndim))
        _, t, _ = types[0x0003]
        cls = self.b[t] & 0x0F
        bits0 = self.b[t + 1]
        size, = self.u("I", t + 4)
        order = ">" if (bits0 & 1) else "<"
        if cls == 1:
            dt = np.dtype(f"{order}f{size}")
        elif cls == 0:
            dt = np.dtype(f"{order}{'i' if (bits0 & 0x08) else 'u'}{size}")
        else:
            raise NotImplementedError(f"datatype class {cls}")
        _, l, _ = types[0x0008]
        lver, lclass = self.b[l], self.b[l + 1]
        if lver != 3:
            raise NotImplementedError(f"layout version {lver}")
        n = int(np.prod(shape)) if ndim else 1
        if lclass == 1:
            addr, nbytes = self.u("QQ", l + 2)
            if addr == UNDEF:
                return np.zeros(shape, dt)
            raw = self.b[addr: addr + n * size]
        elif lclass == 0:
            nbytes, = self.u("H", l + 2)
            raw = self.b[l + 4: l + 4 + nbytes]
        else:
            raise NotImplementedError("chunked layout")
        return np.frombuffer(raw, dtype=dt, count=n).reshape(shape).astype(dt.newbyteorder("="))


def read_all(path):
    """{'group/sub/dataset': ndarray} for every dataset in the file."""
    h = _H5(path)
    out = {}
    stack = [("", h.root_entry["hdr"])]
    seen = set()
    while stack:
        prefix, addr = stack.pop()
        if addr in seen:
            continue
        seen.add(addr)
        kind, val = h.read_object(addr)
        if kind == "group":
            for name, ent in val.items():
                stack.append((f"{prefix}/{name}" if prefix else name, ent["hdr"]))
        elif kind == "dataset":
            out[prefix] = val
    return out
