"""A small, independent HDF5 reader used only by the tests to check signal files.

Written in Python from the HDF5 file-format specification, separately from the C++
writer, for the classic encoding: superblock 0/1, version-1 object headers, symbol-
table groups (v1 B-tree + symbol-table nodes + local heap), dataspace v1/v2, fixed-point
/ floating-point / string datatypes, contiguous and chunked (v1 B-tree) layouts. Besides
reading, it checks structural invariants a library reader relies on (signatures, end-of-
file address, sorted symbol tables, B-tree keys, heap free-list marker).
"""
import struct

import numpy as np

SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(Exception):
    pass


class File:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.b = f.read()
        if self.b[:8] != SIG:
            raise H5Error("no HDF5 signature at offset 0")
        ver = self.b[8]
        if ver not in (0, 1):
            raise H5Error("superblock version %d" % ver)
        self.so, self.sl = self.b[13], self.b[14]
        if (self.so, self.sl) != (8, 8):
            raise H5Error("sizes of offsets/lengths %d/%d" % (self.so, self.sl))
        self.leaf_k, self.internal_k = struct.unpack_from("<HH", self.b, 16)
        p = 24 + (4 if ver == 1 else 0)
        base, freespace, eof, driver = struct.unpack_from("<4Q", self.b, p)
        if base != 0:
            raise H5Error("base address %d" % base)
        if eof != len(self.b):
            raise H5Error("end-of-file address %d != file size %d" % (eof, len(self.b)))
        ent = p + 32
        self.root_addr = struct.unpack_from("<Q", self.b, ent + 8)[0]
        cache_type = struct.unpack_from("<I", self.b, ent + 16)[0]
        if cache_type == 1:
            self.root_cache = struct.unpack_from("<QQ", self.b, ent + 24)
        self.root = self.group(self.root_addr)

    # -- object headers ------------------------------------------------------------------
    def messages(self, addr):
        b = self.b
        ver, _, nmsg, refc, size = struct.unpack_from("<BBHII", b, addr)
        if ver != 1:
            raise H5Error("object header version %d at %d" % (ver, addr))
        out = []
        blocks = [(addr + 16, size)]
        while blocks:
            p, n = blocks.pop(0)
            end = p + n
            if end > len(b):
                raise H5Error("object header past end of file")
            while p + 8 <= end:
                mtype, msize, flags = struct.unpack_from("<HHB", b, p)
                if msize % 8:
                    raise H5Error("message size %d not 8-aligned" % msize)
                data = b[p + 8:p + 8 + msize]
                if mtype == 0x10:
                    blocks.append(struct.unpack_from("<QQ", data, 0))
                else:
                    out.append((mtype, flags, data))
                p += 8 + msize
        if len(out) + sum(1 for _ in ()) < 1:
            raise H5Error("empty object header")
        return out

    # -- groups --------------------------------------------------------------------------
    def group(self, addr):
        stab = [d for t, _, d in self.messages(addr) if t == 0x11]
        if not stab:
            raise H5Error("object at %d is not a symbol-table group" % addr)
        btree, heap = struct.unpack_from("<QQ", stab[0], 0)
        b = self.b
        if b[heap:heap + 4] != b"HEAP":
            raise H5Error("bad local heap signature")
        hsize, free, data = struct.unpack_from("<QQQ", b, heap + 8)
        if free != 1 and free >= hsize:
            raise H5Error("bad heap free-list offset %d" % free)
        if data + hsize > len(b):
            raise H5Error("heap data past end of file")

        def name(off):
            e = b.index(b"\0", data + off)
            return b[data + off:e].decode()

        entries = {}

        def walk(node, depth=0):
            if b[node:node + 4] != b"TREE" or b[node + 4] != 0:
                raise H5Error("bad group B-tree node")
            level, used = b[node + 5], struct.unpack_from("<H", b, node + 6)[0]
            keys = [struct.unpack_from("<Q", b, node + 24 + 16 * i)[0] for i in range(used + 1)]
            for i in range(used):
                child = struct.unpack_from("<Q", b, node + 24 + 8 + 16 * i)[0]
                if level:
                    walk(child, depth + 1)
                    continue
                if b[child:child + 4] != b"SNOD" or b[child + 4] != 1:
                    raise H5Error("bad symbol-table node")
                n = struct.unpack_from("<H", b, child + 6)[0]
                if n > 2 * self.leaf_k:
                    raise H5Error("symbol-table node over-full")
                names = []
                for e in range(n):
                    off, hdr, ctype = struct.unpack_from("<QQI", b, child + 8 + 40 * e)
                    names.append(name(off))
                    entries[names[-1]] = hdr
                if names != sorted(names):
                    raise H5Error("symbol-table entries not sorted: %s" % names)
                if name(keys[i + 1]) != names[-1] or (keys[i] and name(keys[i]) >= names[0]):
                    raise H5Error("group B-tree keys do not bound the node's names")

        walk(btree)
        return entries

    # -- datasets ------------------------------------------------------------------------
    def dataset(self, addr):
        shape = dtype = layout = None
        for t, flags, d in self.messages(addr):
            if t == 0x01:
                ver, rank, fl = d[0], d[1], d[2]
                off = 8 if ver == 1 else 4
                shape = tuple(struct.unpack_from("<%dQ" % rank, d, off)) if rank else ()
                maxdims = (tuple(struct.unpack_from("<%dQ" % rank, d, off + 8 * rank))
                           if rank and fl & 1 else shape)
            elif t == 0x03:
                cls, size = d[0] & 0x0F, struct.unpack_from("<I", d, 4)[0]
                if cls == 1 and size == 8:
                    if d[1] & 1:
                        raise H5Error("big-endian float")
                    dtype = np.dtype("<f8")
                elif cls == 0 and size == 1:
                    dtype = np.dtype("i1") if d[1] & 0x08 else np.dtype("u1")
                elif cls == 3:
                    dtype = np.dtype("S%d" % size)
                else:
                    raise H5Error("datatype class %d size %d" % (cls, size))
            elif t == 0x08:
                if d[0] != 3:
                    raise H5Error("layout version %d" % d[0])
                if d[1] == 1:
                    layout = ("contiguous",) + struct.unpack_from("<QQ", d, 2)
                elif d[1] == 2:
                    nd = d[2]
                    bt = struct.unpack_from("<Q", d, 3)[0]
                    cd = struct.unpack_from("<%dI" % nd, d, 11)
                    layout = ("chunked", bt, cd)
                else:
                    raise H5Error("layout class %d" % d[1])
            elif t == 0x0B:
                raise H5Error("filters not supported")
        if shape is None or dtype is None or layout is None:
            raise H5Error("dataset header incomplete")
        self.last_info = {"shape": shape, "maxdims": maxdims, "layout": layout[0],
                          "chunk": tuple(layout[2]) if layout[0] == "chunked" else None,
                          "btree": layout[1] if layout[0] == "chunked" else None}
        n = int(np.prod(shape)) if shape else 1
        if layout[0] == "contiguous":
            a, size = layout[1], layout[2]
            if size != n * dtype.itemsize:
                raise H5Error("contiguous size %d != %d" % (size, n * dtype.itemsize))
            raw = self.b[a:a + size]
            if len(raw) != size:
                raise H5Error("contiguous data past end of file")
            arr = np.frombuffer(raw, dtype=dtype).copy()
        else:
            arr = np.zeros(n, dtype=dtype)
            bt, cd = layout[1], layout[2][:-1]
            if layout[2][-1] != dtype.itemsize:
                raise H5Error("chunk element size %d" % layout[2][-1])
            if bt != UNDEF:
                self.tree_depth = 0
                self._chunks(bt, len(shape), cd, shape, arr, dtype)
            elif n:
                raise H5Error("chunked dataset with rows but no chunk index")
        return arr.reshape(shape) if shape else arr[0]

    def _chunks(self, node, rank, cd, shape, arr, dtype, depth=0):
        b = self.b
        if b[node:node + 4] != b"TREE" or b[node + 4] != 1:
            raise H5Error("bad chunk B-tree node")
        level, used = b[node + 5], struct.unpack_from("<H", b, node + 6)[0]
        self.tree_depth = max(self.tree_depth, depth + 1)
        if used > 64:
            raise H5Error("chunk B-tree node over-full (%d > 2K = 64)" % used)
        kb = 8 + 8 * (rank + 1)
        full = arr.reshape(shape)
        keys = [struct.unpack_from("<%dQ" % rank, b, node + 24 + i * (kb + 8) + 8)
                for i in range(used + 1)]
        if any(keys[i] >= keys[i + 1] for i in range(used)):
            raise H5Error("chunk B-tree keys not increasing")
        for i in range(used):
            k = node + 24 + i * (kb + 8)
            child = struct.unpack_from("<Q", b, k + kb)[0]
            if level:
                first = struct.unpack_from("<%dQ" % rank, b, child + 24 + 8)
                if first != keys[i]:
                    raise H5Error("internal chunk key differs from the child's first key")
                self._chunks(child, rank, cd, shape, arr, dtype, depth + 1)
                continue
            if struct.unpack_from("<I", b, k)[0] != int(np.prod(cd)) * dtype.itemsize:
                raise H5Error("chunk size field")
            offs = struct.unpack_from("<%dQ" % rank, b, k + 8)
            cnt = int(np.prod(cd))
            chunk = np.frombuffer(b[child:child + cnt * dtype.itemsize], dtype=dtype).reshape(cd)
            sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cd, shape))
            full[sl] = chunk[tuple(slice(0, s.stop - s.start) for s in sl)]

    def info(self, path):
        """Shape, maximum dimensions, layout and chunk dimensions of a dataset."""
        self.read(path)
        return self.last_info

    def read(self, path):
        parts = [p for p in path.split("/") if p]
        entries = self.root
        for p in parts[:-1]:
            entries = self.group(entries[p])
        return self.dataset(entries[parts[-1]])
