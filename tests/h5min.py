"""A small numpy reader of the HDF5 files the observers read and write
(MeshedScreen, src/mesh.cpp:31-218 and 428-736; ScreenObserver,
src/screen.cpp:298-560), written from the HDF5 file-format specification
independently of the C++ reader in include/teufel_hdf5_read.hpp, so that the
two check each other and the C++ writer.

Handles superblock version 0, a symbol-table root group, version-1 object
headers (with continuation blocks), dataspace versions 1-2, little-endian
fixed-point and IEEE float types, contiguous/compact layouts and scalar
attributes of numeric type.  Test infrastructure only.
"""
import struct

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"


class H5Min:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.b = f.read()
        b = self.b
        if b[:8] != SIGNATURE:
            raise ValueError("not an HDF5 file")
        if b[8] != 0 or b[13] != 8 or b[14] != 8:
            raise ValueError("unsupported superblock")
        self.leaf_k, self.internal_k = struct.unpack_from("<HH", b, 16)
        self.eof = struct.unpack_from("<Q", b, 40)[0]
        root_entry = 56
        self.root_header = self.q(root_entry + 8)
        self.root_cache_type = struct.unpack_from("<I", b, root_entry + 16)[0]
        self.links = self._group(self.root_header)

    def q(self, o):
        return struct.unpack_from("<Q", self.b, o)[0]

    def messages(self, addr):
        b = self.b
        ver, _, nmsg, _refc, size = struct.unpack_from("<BBHII", b, addr)
        if ver != 1:
            raise ValueError("object header version %d" % ver)
        todo, out = [(addr + 16, size)], []
        while todo and len(out) < nmsg:
            start, length = todo.pop(0)
            pos = start
            while pos + 8 <= start + length and len(out) < nmsg:
                mtype, msize, mflags = struct.unpack_from("<HHB", b, pos)
                body = b[pos + 8:pos + 8 + msize]
                if len(body) != msize:
                    raise ValueError("message runs past the end of the file")
                if mtype == 0x10:
                    todo.append(struct.unpack_from("<QQ", body, 0))
                out.append((mtype, mflags, body))
                pos += 8 + msize
        return out

    def _group(self, header):
        stab = [body for t, _, body in self.messages(header) if t == 0x11]
        if not stab:
            raise ValueError("root group has no symbol table")
        btree, heap = struct.unpack_from("<QQ", stab[0], 0)
        b = self.b
        if b[heap:heap + 4] != b"HEAP":
            raise ValueError("bad heap")
        seg_size, free_head, seg = struct.unpack_from("<QQQ", b, heap + 8)
        self.heap = dict(size=seg_size, free=free_head, segment=seg)

        def name(off):
            end = b.index(b"\0", seg + off)
            return b[seg + off:end].decode()

        links = {}

        def walk(node):
            if b[node:node + 4] != b"TREE" or b[node + 4] != 0:
                raise ValueError("bad B-tree node")
            level, used = b[node + 5], struct.unpack_from("<H", b, node + 6)[0]
            self.btree = dict(level=level, used=used,
                              keys=[self.q(node + 24 + 16 * i) for i in range(used + 1)])
            for i in range(used):
                child = self.q(node + 32 + 16 * i)
                if level:
                    walk(child)
                    continue
                if b[child:child + 4] != b"SNOD":
                    raise ValueError("bad symbol node")
                count = struct.unpack_from("<H", b, child + 6)[0]
                names = []
                for k in range(count):
                    e = child + 8 + 40 * k
                    nm = name(self.q(e))
                    links[nm] = self.q(e + 8)
                    names.append(nm)
                if names != sorted(names):
                    raise ValueError("symbol node entries out of order")
                self.btree_last_key = name(self.btree["keys"][-1])

        walk(btree)
        return links

    @staticmethod
    def _dtype(body):
        cls, bits, size = body[0] & 15, body[1], struct.unpack_from("<I", body, 4)[0]
        if bits & 1:
            raise ValueError("big-endian")
        if cls == 1:
            return np.dtype("<f%d" % size)
        if cls == 0:
            return np.dtype(("<i%d" if bits & 8 else "<u%d") % size)
        raise ValueError("datatype class %d" % cls)

    @staticmethod
    def _space(body):
        ver, rank = body[0], body[1]
        first = 8 if ver == 1 else 4
        return tuple(struct.unpack_from("<%dQ" % rank, body, first)) if rank else ()

    def _attribute(self, body):
        ver = body[0]
        nlen, tlen, slen = struct.unpack_from("<HHH", body, 2)
        pad = (lambda n: (n + 7) // 8 * 8) if ver == 1 else (lambda n: n)
        p = 8 + (1 if ver == 3 else 0)
        name = body[p:p + nlen].split(b"\0")[0].decode()
        p += pad(nlen)
        dt = self._dtype(body[p:p + tlen])
        p += pad(tlen)
        shape = self._space(body[p:p + slen])
        p += pad(slen)
        n = int(np.prod(shape)) if shape else 1
        val = np.frombuffer(body, dt, n, p)
        return name, (val[0] if not shape else val.reshape(shape))

    def dataset(self, name):
        """(array, attributes, info) of one dataset in the root group."""
        shape = dt = None
        attrs, info, raw = {}, {}, None
        for t, flags, body in self.messages(self.links[name]):
            if t == 0x1:
                shape = self._space(body)
            elif t == 0x3:
                dt = self._dtype(body)
                info["dtype_message"] = bytes(body)
            elif t == 0x8:
                if body[0] != 3:
                    raise ValueError("layout version %d" % body[0])
                if body[1] == 1:
                    addr, size = struct.unpack_from("<QQ", body, 2)
                    info.update(addr=addr, size=size)
                    raw = b"" if size == 0 else self.b[addr:addr + size]
                elif body[1] == 0:
                    size = struct.unpack_from("<H", body, 2)[0]
                    raw = body[4:4 + size]
                else:
                    raise ValueError("chunked layout")
            elif t == 0xC:
                k, v = self._attribute(body)
                attrs[k] = v
        n = int(np.prod(shape))
        arr = np.frombuffer(raw, dt, n).reshape(shape) if n else np.zeros(shape, dt)
        return arr, attrs, info
