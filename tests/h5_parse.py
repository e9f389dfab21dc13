"""An independent reader of the HDF5 subset the library writes (test infrastructure).

Written from the HDF5 File Format Specification in plain Python/NumPy, separately from the
library's C++ reader, so that the tests check the files against the format rather than
against the code that wrote them: superblock version 0, version 1 object headers,
symbol-table groups (local heap, version 1 B-tree, symbol table nodes), version 1 dataspaces,
float / integer / string datatypes, contiguous layout (version 3) and version 1 attributes.
"""
from __future__ import annotations

import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


def _up8(n):
    return (n + 7) // 8 * 8


class File:
    def __init__(self, path):
        self.b = open(path, "rb").read()
        assert self.b[:8] == b"\x89HDF\r\n\x1a\n", "signature"
        assert self.b[8] == 0, "superblock version 0"
        assert self.b[13] == 8 and self.b[14] == 8, "8-byte offsets and lengths"
        self.leaf_k, self.node_k = struct.unpack_from("<HH", self.b, 16)
        eof = struct.unpack_from("<Q", self.b, 40)[0]
        assert eof == len(self.b), "end-of-file address"
        name_off, self.root, cache = struct.unpack_from("<QQI", self.b, 56)
        assert cache == 1
        self.root_btree, self.root_heap = struct.unpack_from("<QQ", self.b, 80)
        self.root_obj = self.header(self.root)
        self.attrs = self.root_obj["attrs"]
        assert (self.root_obj["btree"], self.root_obj["heap"]) == (self.root_btree, self.root_heap)

    def u(self, fmt, at):
        return struct.unpack_from(fmt, self.b, at)

    def header(self, at):
        ver, _, nmsg, refc, size = self.u("<BBHII", at)
        assert ver == 1 and refc >= 1
        p, end = at + 16, at + 16 + size
        out = {"attrs": {}, "dims": None, "dtype": None, "data": None, "btree": None, "heap": None}
        for _ in range(nmsg):
            typ, msize, flags = self.u("<HHB", p)
            assert msize % 8 == 0, "message sizes are multiples of 8 in version 1 headers"
            d = p + 8
            if typ == 0x0001:
                out["dims"] = self.space(d)
            elif typ == 0x0003:
                out["dtype"] = self.dtype(d)
            elif typ == 0x0008:
                ver3, cls = self.u("<BB", d)
                assert ver3 == 3 and cls == 1
                out["data"] = self.u("<QQ", d + 2)
            elif typ == 0x0011:
                out["btree"], out["heap"] = self.u("<QQ", d)
            elif typ == 0x000C:
                name, val = self.attribute(d)
                out["attrs"][name] = val
            p = d + msize
        assert p == end, "object header size"
        return out

    def space(self, d):
        ver, rank, flags = self.u("<BBB", d)
        assert ver == 1 and flags == 0
        return list(self.u("<%dQ" % rank, d + 8)) if rank else []

    def dtype(self, d):
        cv, b1, b2, b3, size = self.u("<BBBBI", d)
        cls, ver = cv & 15, cv >> 4
        assert ver == 1
        if cls == 1:
            assert (b1 & 1) == 0 and size == 8 and b2 == 63
            off, prec, eloc, esz, mloc, msz, bias = self.u("<HHBBBBI", d + 8)
            assert (prec, eloc, esz, mloc, msz, bias) == (64, 52, 11, 0, 52, 1023)
            return ("<f8", 20)
        if cls == 0:
            assert size == 4 and (b1 & 1) == 0
            return ("<i4" if b1 & 8 else "<u4", 12)
        if cls == 3:
            return ("S%d" % size, 8)
        raise AssertionError(f"datatype class {cls}")

    def attribute(self, d):
        ver, _, nl, dl, sl = self.u("<BBHHH", d)
        assert ver == 1
        q = d + 8
        name = self.b[q:q + nl - 1].decode()
        assert self.b[q + nl - 1] == 0
        q += _up8(nl)
        dt, dsize = self.dtype(q)
        assert dsize == dl
        q += _up8(dl)
        dims = self.space(q)
        q += _up8(sl)
        n = int(np.prod(dims)) if dims else 1
        if dt.startswith("S"):
            size = int(dt[1:])
            return name, self.b[q:q + size * n].decode()
        arr = np.frombuffer(self.b, dtype=dt, count=n, offset=q)
        return name, arr.tolist()

    def heap_name(self, heap, off):
        assert self.b[heap:heap + 4] == b"HEAP" and self.b[heap + 4] == 0
        size, free, seg = self.u("<QQQ", heap + 8)
        assert off < size
        end = self.b.index(b"\0", seg + off)
        return self.b[seg + off:end].decode()

    def group_members(self, btree, heap):
        assert self.b[btree:btree + 4] == b"TREE"
        ntype, level, used = self.u("<BBH", btree + 4)
        assert ntype == 0 and level == 0
        out = {}
        prev_key = None
        for c in range(used):
            key, child = self.u("<QQ", btree + 24 + 16 * c)
            last_key = self.u("<Q", btree + 24 + 16 * c + 16)[0]
            assert self.b[child:child + 4] == b"SNOD" and self.b[child + 4] == 1
            ns = self.u("<H", child + 6)[0]
            assert ns <= 2 * self.leaf_k
            names = []
            for e in range(ns):
                noff, hdr, cache = self.u("<QQI", child + 8 + 40 * e)
                names.append(self.heap_name(heap, noff))
                out[names[-1]] = hdr
            assert names == sorted(names), "symbol table nodes are sorted"
            assert self.heap_name(heap, last_key) == names[-1], "B-tree key = last name of the child"
            if prev_key is not None:
                assert self.heap_name(heap, key) == prev_key
            prev_key = names[-1]
        return out

    def members(self, group=""):
        obj = self.root_obj if not group else self.header(self.group_members(self.root_btree, self.root_heap)[group])
        return sorted(self.group_members(obj["btree"], obj["heap"]))

    def obj(self, path):
        o = self.root_obj
        for part in path.split("/"):
            kids = self.group_members(o["btree"], o["heap"])
            o = self.header(kids[part])
        return o

    def dataset(self, path):
        o = self.obj(path)
        addr, size = o["data"]
        dt = o["dtype"][0]
        n = int(np.prod(o["dims"]))
        assert size == n * np.dtype(dt).itemsize
        return np.frombuffer(self.b, dtype=dt, count=n, offset=addr).reshape(o["dims"])
