"""A minimal HDF5 reader for the reference's small fixture files (test
infrastructure; no HDF5 library is available here).

It reads what the reference's MRS/IOS/src/HDF5_Tools.hpp writes for a matrix
(save_matrix_to_hdf5_file): a dataset in the root group with a version-0
superblock, a version-1 group B-tree with symbol-table nodes and a local heap
for the names, version-1 object headers, a simple dataspace of rank 1 or 2
and a little-endian IEEE float or integer datatype with contiguous or compact
storage.  Anything else raises ValueError.  Layout references: the HDF5 File
Format Specification (version 2.0), sections II.A (superblock), III.A (B-tree
v1), III.B (symbol table node), III.D (local heap), IV.A (object header v1),
IV.A.2 (messages 0x0001 dataspace, 0x0003 datatype, 0x0008 data layout,
0x0010 continuation).

    read_datasets(path) -> {name: numpy array}   (2-D datasets row-major, as
                                                  load_matrix_from_hdf5_file
                                                  fills Matrix(i, j))
"""
import struct

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"


class _File:
    def __init__(self, data):
        self.d = data
        if data[:8] != _SIG:
            raise ValueError("not an HDF5 file")
        if data[8] != 0:
            raise ValueError("superblock version %d is not supported" % data[8])
        self.so, self.sl = data[13], data[14]
        if self.so != 8 or self.sl != 8:
            raise ValueError("only 8-byte offsets and lengths are supported")
        # base, free-space, end-of-file, driver addresses, then the root entry
        p = 24 + 4 * 8
        self.root = self.entry(p)

    def u(self, off, n):
        return int.from_bytes(self.d[off:off + n], "little")

    def entry(self, p):
        """symbol table entry: (name offset, object header address, cache type, scratch)"""
        name_off, hdr = self.u(p, 8), self.u(p + 8, 8)
        cache = self.u(p + 16, 4)
        return name_off, hdr, cache, self.d[p + 24:p + 40]

    def heap_data(self, addr):
        if self.d[addr:addr + 4] != b"HEAP":
            raise ValueError("local heap expected")
        return self.u(addr + 24, 8)

    def name(self, heap_data, off):
        end = self.d.index(b"\0", heap_data + off)
        return self.d[heap_data + off:end].decode()

    def group_entries(self, btree, heap):
        hd = self.heap_data(heap)
        out = []
        stack = [btree]
        while stack:
            a = stack.pop()
            if self.d[a:a + 4] != b"TREE":
                raise ValueError("B-tree node expected")
            ntype, level, used = self.d[a + 4], self.d[a + 5], self.u(a + 6, 2)
            if ntype != 0:
                raise ValueError("group B-tree expected")
            p = a + 8 + 16  # signature, type, level, entries used, two siblings
            for k in range(used):
                child = self.u(p + 8 + k * 16, 8)
                if level > 0:
                    stack.append(child)
                else:
                    out.extend(self.snod(child, hd))
        return out

    def snod(self, a, hd):
        if self.d[a:a + 4] != b"SNOD":
            raise ValueError("symbol table node expected")
        n = self.u(a + 6, 2)
        res = []
        for k in range(n):
            name_off, hdr, _, _ = self.entry(a + 8 + k * 40)
            res.append((self.name(hd, name_off), hdr))
        return res

    def messages(self, addr):
        if self.d[addr] != 1:
            raise ValueError("object header version %d is not supported" % self.d[addr])
        nmsg = self.u(addr + 2, 2)
        blocks = [(addr + 16, self.u(addr + 8, 4))]
        msgs = []
        while blocks and len(msgs) < nmsg:
            p, size = blocks.pop(0)
            end = p + size
            while p + 8 <= end and len(msgs) < nmsg:
                mtype, msize = self.u(p, 2), self.u(p + 2, 2)
                body = p + 8
                if mtype == 0x10:
                    blocks.append((self.u(body, 8), self.u(body + 8, 8)))
                msgs.append((mtype, body, msize))
                p = body + msize
        return msgs

    def dataset(self, addr):
        shape, dtype, raw = None, None, None
        for mtype, p, size in self.messages(addr):
            if mtype == 0x0001:  # dataspace
                ver, rank = self.d[p], self.d[p + 1]
                q = p + (8 if ver == 1 else 4)
                shape = tuple(self.u(q + 8 * k, 8) for k in range(rank))
            elif mtype == 0x0003:  # datatype
                cls, nbytes = self.d[p] & 0x0F, self.u(p + 4, 4)
                if self.d[p + 1] & 1:
                    raise ValueError("big-endian data is not supported")
                if cls == 1:
                    dtype = np.dtype("<f%d" % nbytes)
                elif cls == 0:
                    signed = bool(self.d[p + 1] & 0x08)
                    dtype = np.dtype("<%s%d" % ("i" if signed else "u", nbytes))
                else:
                    raise ValueError("datatype class %d is not supported" % cls)
            elif mtype == 0x0008:  # data layout
                ver = self.d[p]
                if ver != 3:
                    raise ValueError("data layout version %d is not supported" % ver)
                cls = self.d[p + 1]
                if cls == 1:
                    raw = (self.u(p + 2, 8), self.u(p + 10, 8))
                elif cls == 0:
                    raw = (p + 4, self.u(p + 2, 2))
                else:
                    raise ValueError("chunked storage is not supported")
        if shape is None or dtype is None or raw is None:
            raise ValueError("not a simple dataset")
        count = int(np.prod(shape)) if shape else 1
        if raw[0] == (1 << 64) - 1 or count == 0:
            return np.zeros(shape, dtype=dtype)
        a = np.frombuffer(self.d, dtype=dtype, count=count, offset=raw[0])
        return a.reshape(shape).copy()


def read_datasets(path):
    with open(path, "rb") as fh:
        f = _File(fh.read())
    _, hdr, cache, scratch = f.root
    if cache != 1:
        raise ValueError("root group without a symbol table")
    btree, heap = struct.unpack("<QQ", scratch)
    return {name: f.dataset(addr) for name, addr in f.group_entries(btree, heap)}
