"""A strict reader of the classic HDF5 file layout, for the tests of the
library's HDF5 writer (no HDF5 library or h5py is installed here).

It follows the published HDF5 file-format specification for the structures
that layout uses: a version-0 or -1 superblock (at byte 0, 512, 1024, ...),
groups indexed by version-1 B-trees of node type 0 over symbol-table nodes
and a local heap of names, version-1 object headers (with continuation
blocks), dataspace messages version 1 and 2, datatype classes 0 (integer),
1 (floating point) and 3 (string), data-layout messages versions 1-3
(compact and contiguous), fill-value messages and attribute messages
version 1. Besides reading, it checks what a conforming writer must get
right: signatures and versions, 8-byte-aligned message sizes, the message
count of every header, sorted symbol-table entries bracketed by their
B-tree keys, a well-formed local-heap free list, the end-of-file address and
that every structure lies inside the file. Its correctness is pinned on a
file written by the HDF5 library (tests/test_h5_writer.py).
"""
from __future__ import annotations

import struct

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class FormatError(ValueError):
    pass


def _need(cond, msg):
    if not cond:
        raise FormatError(msg)


class Dataset:
    def __init__(self, name, shape, dtype, raw, attrs, messages):
        self.name, self.shape, self.dtype, self.attrs, self.messages = name, shape, dtype, attrs, messages
        self._raw = raw

    def __getitem__(self, key):
        return self.read()[key]

    def read(self):
        return np.frombuffer(self._raw, dtype=self.dtype).reshape(self.shape).copy()


class File:
    """Root group of an HDF5 file: ``f[name]`` gives a Dataset (or a File
    for a subgroup), ``f.attrs`` the root attributes, ``f.keys()`` the names
    in the order of the symbol table."""

    def __init__(self, path_or_bytes, _sub=None):
        if _sub is not None:
            parent, header = _sub
            for k in ("_b", "base", "oa", "la", "eof", "leaf_k", "internal_k"):
                setattr(self, k, getattr(parent, k))
            self._load_group(header)
            return
        b = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
        self._b = bytes(b)
        base = 0
        while base < len(self._b) and self._b[base:base + 8] != SIGNATURE:
            base = 512 if base == 0 else 2 * base
        _need(base < len(self._b), "no HDF5 signature")
        self.base = base
        sb = self._b[base:]
        ver = sb[8]
        _need(ver in (0, 1), f"superblock version {ver} not supported")
        _need(sb[9] == 0 and sb[10] == 0 and sb[12] == 0, "free-space / root entry / shared header versions must be 0")
        self.oa, self.la = sb[13], sb[14]
        _need(self.oa == 8 and self.la == 8, "only 8-byte offsets and lengths are read")
        self.leaf_k, self.internal_k = struct.unpack_from("<HH", sb, 16)
        _need(self.leaf_k > 0 and self.internal_k > 0, "group K values must be positive")
        p = 24 if ver == 0 else 28
        base_addr, fs_addr, eof, drv = struct.unpack_from("<4Q", sb, p)
        _need(base_addr == base, "base address must be the superblock's position")
        self.eof = eof
        _need(eof == len(self._b), f"end-of-file address {eof} != file size {len(self._b)}")
        entry = self._entry(base + p + 32)
        _need(entry["cache"] in (0, 1), "root entry cache type")
        self.superblock = dict(version=ver, leaf_k=self.leaf_k, internal_k=self.internal_k,
                               free_space=fs_addr, driver=drv, root=entry)
        self._load_group(entry["header"], entry)

    # ------------------------------------------------------------ helpers
    def _at(self, addr, n):
        _need(addr != UNDEF, "undefined address dereferenced")
        a = self.base + addr
        _need(0 <= addr and a + n <= len(self._b), f"structure at {addr} (+{n}) lies outside the file")
        return self._b[a:a + n]

    def _entry(self, absolute):
        name_off, header, cache = struct.unpack_from("<QQI", self._b, absolute)
        scratch = struct.unpack_from("<QQ", self._b, absolute + 24)
        return dict(name=name_off, header=header, cache=cache, scratch=scratch)

    def _heap(self, addr):
        h = self._at(addr, 32)
        _need(h[:4] == b"HEAP" and h[4] == 0, "local heap signature / version")
        size, free, data = struct.unpack_from("<3Q", h, 8)
        _need(size > 0 and size % 8 == 0, "heap data segment size")
        seg = self._at(data, size)
        _need(seg[0] == 0, "offset 0 of a group heap must hold the empty name")
        seen = set()
        while free != 1:                 # 1 ends the free list
            _need(free < size and free % 8 == 0 and free not in seen, f"bad heap free list entry {free}")
            seen.add(free)
            nxt, blk = struct.unpack_from("<QQ", seg, free)
            _need(blk >= 16 and free + blk <= size, "bad heap free block")
            free = nxt
        return seg

    def _name(self, heap, off):
        _need(off < len(heap), "name offset outside the heap")
        end = heap.index(b"\0", off)
        return heap[off:end].decode()

    def _messages(self, addr):
        h = self._at(addr, 16)
        _need(h[0] == 1, f"object header version {h[0]} not supported")
        nmsg = struct.unpack_from("<H", h, 2)[0]
        refs, size = struct.unpack_from("<II", h, 4)
        _need(refs >= 1, "object reference count")
        blocks, msgs = [(addr + 16, size)], []
        while blocks:
            start, length = blocks.pop(0)
            blk = self._at(start, length)
            p = 0
            while p + 8 <= length:
                mtype, msize, flags = struct.unpack_from("<HHB", blk, p)
                _need(msize % 8 == 0, f"message of type {mtype:#x} not 8-byte aligned ({msize})")
                _need(p + 8 + msize <= length, "message runs past its header block")
                body = blk[p + 8:p + 8 + msize]
                msgs.append((mtype, flags, body))
                if mtype == 0x10:
                    off, ln = struct.unpack_from("<QQ", body, 0)
                    blocks.append((off, ln))
                p += 8 + msize
            _need(p == length, "header block not filled by its messages")
        _need(len(msgs) == nmsg, f"header says {nmsg} messages, found {len(msgs)}")
        return msgs

    def _btree_children(self, addr, heap, lo=None, hi=None):
        """Symbol-table node addresses under a type-0 B-tree node, checking
        that each child's names lie in (key_i, key_i+1]."""
        k2 = 2 * self.internal_k
        n = 24 + k2 * 8 + (k2 + 1) * 8
        node = self._at(addr, n)
        _need(node[:4] == b"TREE" and node[4] == 0, "B-tree signature / node type")
        level, used = node[5], struct.unpack_from("<H", node, 6)[0]
        _need(used <= k2, "B-tree node overfull")
        keys = [self._name(heap, struct.unpack_from("<Q", node, 24 + 16 * i)[0]) for i in range(used + 1)]
        kids = [struct.unpack_from("<Q", node, 32 + 16 * i)[0] for i in range(used)]
        _need(all(keys[i].encode() < keys[i + 1].encode() for i in range(used)), "B-tree keys out of order")
        out = []
        for i, c in enumerate(kids):
            if level > 0:
                out += self._btree_children(c, heap, keys[i], keys[i + 1])
            else:
                out.append((c, keys[i], keys[i + 1]))
        return out

    def _symbols(self, snod, heap, lo, hi):
        n = 8 + 2 * self.leaf_k * 40
        node = self._at(snod, n)
        _need(node[:4] == b"SNOD" and node[4] == 1, "symbol-table node signature / version")
        cnt = struct.unpack_from("<H", node, 6)[0]
        _need(cnt <= 2 * self.leaf_k, "symbol-table node overfull")
        ents = [self._entry(self.base + snod + 8 + 40 * i) for i in range(cnt)]
        names = [self._name(heap, e["name"]) for e in ents]
        _need(names == sorted(names, key=lambda s: s.encode()), "symbol-table entries not sorted")
        for nm in names:
            _need(lo.encode() < nm.encode() <= hi.encode(), f"name {nm!r} outside its B-tree keys")
        return list(zip(names, ents))

    # ------------------------------------------------------------ objects
    def _load_group(self, header, entry=None):
        msgs = self._messages(header)
        stab = [m for m in msgs if m[0] == 0x11]
        _need(len(stab) == 1, "a group needs one symbol-table message")
        btree, heap_addr = struct.unpack_from("<QQ", stab[0][2], 0)
        if entry is not None and entry["cache"] == 1:
            _need(entry["scratch"] == (btree, heap_addr), "root entry scratch pad differs from the symbol table")
        heap = self._heap(heap_addr)
        self.attrs = self._attributes(msgs)
        self._objects = {}
        self._order = []
        for snod, lo, hi in self._btree_children(btree, heap):
            for name, e in self._symbols(snod, heap, lo, hi):
                _need(name not in self._objects, f"duplicate name {name!r}")
                self._order.append(name)
                self._objects[name] = e["header"]
        self.messages = msgs

    def keys(self):
        return list(self._order)

    def __contains__(self, name):
        return name in self._objects

    def __getitem__(self, name):
        addr = self._objects[name]
        msgs = self._messages(addr)
        if any(m[0] == 0x11 for m in msgs):
            return File(None, _sub=(self, addr))
        return self._dataset(name, msgs)

    def _dataset(self, name, msgs):
        by = {}
        for t, fl, body in msgs:
            by.setdefault(t, []).append(body)
        for t in (0x1, 0x3, 0x8):
            _need(len(by.get(t, [])) == 1, f"dataset {name!r} needs one message of type {t:#x}")
        shape = self._dataspace(by[0x1][0])
        dtype = self._datatype(by[0x3][0])
        raw = self._layout(by[0x8][0], shape, dtype)
        return Dataset(name, shape, dtype, raw, self._attributes(msgs), msgs)

    def _dataspace(self, b):
        ver, rank, flags = b[0], b[1], b[2]
        if ver == 1:
            p = 8
        else:
            _need(ver == 2, "dataspace version")
            p = 4
            if b[3] == 0:
                return ()
        dims = struct.unpack_from(f"<{rank}Q", b, p)
        if flags & 1:
            mx = struct.unpack_from(f"<{rank}Q", b, p + 8 * rank)
            _need(all(m == UNDEF or m >= d for m, d in zip(mx, dims)), "maximum dimension below dimension")
        return tuple(dims)

    def _datatype(self, b):
        cls, ver = b[0] & 0x0F, b[0] >> 4
        _need(ver in (1, 2, 3), "datatype version")
        bits = b[1] | (b[2] << 8) | (b[3] << 16)
        size = struct.unpack_from("<I", b, 4)[0]
        order = ">" if bits & 1 else "<"
        if cls == 1:
            _need(size in (4, 8), "float size")
            off, prec, eloc, esz, mloc, msz, bias = struct.unpack_from("<HHBBBBI", b, 8)
            ieee = {4: (0, 32, 23, 8, 0, 23, 127, 31), 8: (0, 64, 52, 11, 0, 52, 1023, 63)}[size]
            _need((off, prec, eloc, esz, mloc, msz, bias, (bits >> 8) & 0xFF) == ieee, "not an IEEE float layout")
            _need((bits >> 4) & 3 == 2, "IEEE floats have an implied mantissa bit")
            return np.dtype(f"{order}f{size}")
        if cls == 0:
            signed = bool(bits & 8)
            return np.dtype(f"{order}{'i' if signed else 'u'}{size}")
        if cls == 3:
            return np.dtype(f"S{size}")
        raise FormatError(f"datatype class {cls} not supported")

    def _layout(self, b, shape, dtype):
        ver = b[0]
        n = int(np.prod(shape)) if shape else 1
        nbytes = n * dtype.itemsize
        if ver in (1, 2):
            ndim, cls = b[1], b[2]
            p = 8
            if cls == 0:   # compact
                dims = struct.unpack_from(f"<{ndim}I", b, p)
                sz = struct.unpack_from("<I", b, p + 4 * ndim)[0]
                _need(sz == nbytes, "compact size")
                return b[p + 4 * ndim + 4:p + 4 * ndim + 4 + sz]
            _need(cls == 1, "only compact and contiguous layouts are read")
            addr = struct.unpack_from("<Q", b, p)[0]
            dims = struct.unpack_from(f"<{ndim}I", b, p + 8)
            _need(ndim == len(shape) + 1 and tuple(dims[:-1]) == tuple(shape) and dims[-1] == dtype.itemsize,
                  "layout dimensions differ from the dataspace")
            return self._at(addr, nbytes)
        _need(ver == 3, "layout version")
        cls = b[1]
        if cls == 0:
            sz = struct.unpack_from("<H", b, 2)[0]
            _need(sz == nbytes, "compact size")
            return b[4:4 + sz]
        _need(cls == 1, "only compact and contiguous layouts are read")
        addr, sz = struct.unpack_from("<QQ", b, 2)
        _need(sz == nbytes, "contiguous size differs from the dataspace")
        return self._at(addr, nbytes)

    def _attributes(self, msgs):
        out = {}
        for t, fl, b in msgs:
            if t != 0x0C:
                continue
            _need(b[0] == 1, "attribute message version")
            nlen, tlen, slen = struct.unpack_from("<HHH", b, 2)
            p = 8
            name = b[p:p + nlen].split(b"\0")[0].decode()
            _need(b[p + nlen - 1] == 0, "attribute name must be NUL-terminated")
            p += (nlen + 7) // 8 * 8
            dt = self._datatype(b[p:p + tlen])
            p += (tlen + 7) // 8 * 8
            shape = self._dataspace(b[p:p + slen])
            p += (slen + 7) // 8 * 8
            n = int(np.prod(shape)) if shape else 1
            _need(p + n * dt.itemsize <= len(b), "attribute data runs past its message")
            val = np.frombuffer(b[p:p + n * dt.itemsize], dtype=dt).reshape(shape).copy()
            _need(name not in out, f"duplicate attribute {name!r}")
            out[name] = val
        return out
