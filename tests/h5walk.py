"""A walker of HDF5 files written from the published HDF5 file-format
specification: superblock version 0, version-1 object headers and
symbol-table groups (the B-tree "TREE", the symbol table node "SNOD" and the
local heap "HEAP"), the structures grav_sim's snapshots use.  It shares no
code with the library's own HDF5 reader, so that a file the library writes
is checked by a second, independent reading."""
import numpy as np


def _u(b, o, n):
    return int.from_bytes(b[o:o + n], "little")


def _pad8(n):
    return (n + 7) & ~7


class Walker:
    """A minimal reader of the structures grav_sim's snapshots use."""

    def __init__(self, path):
        self.b = open(path, "rb").read()
        b = self.b
        assert b[:8] == b"\x89HDF\r\n\x1a\n"
        assert b[8] == 0, "superblock version"
        assert b[13] == 8 and b[14] == 8, "offset and length sizes"
        assert _u(b, 40, 8) == len(b), "end-of-file address"
        root = 56   # the root group's symbol table entry
        self.root = _u(b, root + 8, 8)
        assert _u(b, root + 16, 4) == 1
        self.root_cache = (_u(b, root + 24, 8), _u(b, root + 32, 8))

    def messages(self, oh):
        """The (type, body) messages of a version-1 object header, following
        continuation messages (type 0x10) into their blocks."""
        b = self.b
        assert b[oh] == 1, "object header version"
        count = _u(b, oh + 2, 2)
        blocks, out = [(oh + 16, _u(b, oh + 8, 4))], []
        while blocks:
            p, size = blocks.pop(0)
            end = p + size
            while p + 8 <= end:
                t, sz = _u(b, p, 2), _u(b, p + 2, 2)
                if t == 0x10:
                    blocks.append((_u(b, p + 8, 8), _u(b, p + 16, 8)))
                out.append((t, b[p + 8:p + 8 + sz]))
                p += 8 + sz
        assert len(out) == count
        return [(t, d) for t, d in out if t not in (0x00, 0x10)]

    def children(self, oh):
        (bt, heap), = [(_u(d, 0, 8), _u(d, 8, 8)) for t, d in self.messages(oh) if t == 0x11]
        b = self.b
        assert b[heap:heap + 4] == b"HEAP"
        data = _u(b, heap + 24, 8)
        assert b[bt:bt + 4] == b"TREE" and b[bt + 4] == 0 and b[bt + 5] == 0
        names = {}
        for k in range(_u(b, bt + 6, 2)):
            snod = _u(b, bt + 24 + 16 * k + 8, 8)
            assert b[snod:snod + 4] == b"SNOD"
            for e in range(_u(b, snod + 6, 2)):
                eo = snod + 8 + 40 * e
                off = data + _u(b, eo, 8)
                name = b[off:b.index(b"\0", off)].decode()
                names[name] = _u(b, eo + 8, 8)
        assert list(names) == sorted(names), "entries in name order"
        return names

    def lookup(self, path):
        oh = self.root
        for part in path.strip("/").split("/"):
            oh = self.children(oh)[part]
        return oh

    @staticmethod
    def dtype(d):
        cls, size = d[0] & 0x0F, _u(d, 4, 4)
        if cls == 0:
            assert size in (1, 2, 4, 8) and not d[1] & 0x01, "little-endian integer"
            return np.dtype(f"<{'i' if d[1] & 0x08 else 'u'}{size}")
        assert cls == 1 and size in (4, 8)
        return np.dtype("<f4" if size == 4 else "<f8")

    @staticmethod
    def dims(d):
        assert d[0] == 1
        return tuple(_u(d, 8 + 8 * k, 8) for k in range(d[1]))

    def dataset(self, path):
        msgs = dict(self.messages(self.lookup(path)))
        dt, shape, lay = self.dtype(msgs[0x03]), self.dims(msgs[0x01]), msgs[0x08]
        assert lay[0] == 3 and lay[1] == 1, "contiguous layout"
        addr, size = _u(lay, 2, 8), _u(lay, 10, 8)
        assert size == int(np.prod(shape)) * dt.itemsize
        return np.frombuffer(self.b[addr:addr + size], dtype=dt).reshape(shape)

    def attributes(self, path):
        out = {}
        for t, d in self.messages(self.lookup(path)):
            if t != 0x0C:
                continue
            assert d[0] == 1
            nsz, tsz, ssz = _u(d, 2, 2), _u(d, 4, 2), _u(d, 6, 2)
            p = 8
            name = d[p:p + nsz - 1].decode()
            p += _pad8(nsz)
            dt = self.dtype(d[p:p + tsz])
            p += _pad8(tsz)
            shape = self.dims(d[p:p + ssz])
            p += _pad8(ssz)
            count = int(np.prod(shape))
            out[name] = (np.frombuffer(d[p:p + count * dt.itemsize], dtype=dt), shape)
        return out
