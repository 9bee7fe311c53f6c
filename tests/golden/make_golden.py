"""Generate the golden fixtures from the reference's sample data.

Reads ``data/Oil.h5`` (the input the reference ships) and ``data/Oil.out.h5``
(an output file the reference wrote for it: a converged DA-GTM state with
K = 125 (5^3, L = 3), M = 8 (2^3) RBF centres plus bias, N = 1000, D = 12)
from a jychoi-hpc/da-gtm checkout and stores the arrays the parity tests
need in ``oil_golden.npz``; ``oil_input.h5`` and ``oil_output.h5`` are byte
copies of the two files, for the command-line driver's HDF5 reader (the
output file's datasets are chunked and deflate-compressed).  The reference
tree is not available where the GPU tests run, so only these fixtures
travel; this script is kept beside them so they can be regenerated:

    python tests/golden/make_golden.py /path/to/da-gtm/data

No HDF5 library is needed: the two files use the HDF5 1.8 default format
(superblock version 0, version-1 object headers, symbol-table groups), with
contiguous datasets (Oil.h5) and deflate-compressed chunked datasets
(Oil.out.h5).  The small reader below walks exactly those structures.
"""
from __future__ import annotations

import os
import shutil
import struct
import sys
import zlib

import numpy as np


class H5File:
    """Minimal reader: superblock v0, v1 object headers, v1 group B-trees."""

    def __init__(self, path):
        with open(path, "rb") as f:
            self.b = f.read()
        b = self.b
        if b[:8] != b"\x89HDF\r\n\x1a\n":
            raise ValueError("not an HDF5 file")
        if b[8] != 0:
            raise ValueError("only superblock version 0 is supported")
        self.so = b[13]  # size of offsets
        self.sl = b[14]  # size of lengths
        assert self.so == 8 and self.sl == 8
        # superblock v0: 24 bytes of fixed fields, 4 addresses, root symbol table entry
        p = 24 + 4 * 8
        self.root_header = struct.unpack("<Q", b[p + 8:p + 16])[0]
        self.datasets = {}
        self._walk_group(self.root_header)

    def _messages(self, addr):
        b = self.b
        ver = b[addr]
        if ver != 1:
            raise ValueError("only version-1 object headers are supported")
        nmsg = struct.unpack("<H", b[addr + 2:addr + 4])[0]
        hsize = struct.unpack("<I", b[addr + 8:addr + 12])[0]
        blocks = [(addr + 16, hsize)]
        msgs = []
        while blocks and len(msgs) < nmsg:
            start, size = blocks.pop(0)
            p = start
            while p + 8 <= start + size and len(msgs) < nmsg:
                mtype, msize = struct.unpack("<HH", b[p:p + 4])
                body = b[p + 8:p + 8 + msize]
                if mtype == 0x10:  # continuation
                    caddr, clen = struct.unpack("<QQ", body[:16])
                    blocks.append((caddr, clen))
                msgs.append((mtype, body))
                p += 8 + msize
        return msgs

    def _walk_group(self, addr):
        for mtype, body in self._messages(addr):
            if mtype == 0x11:  # symbol table: B-tree address, local heap address
                btree, heap = struct.unpack("<QQ", body[:16])
                names = self._heap(heap)
                for name_off, obj in self._group_btree(btree):
                    name = names[name_off:names.index(b"\0", name_off)].decode()
                    self.datasets[name] = obj

    def _heap(self, addr):
        b = self.b
        assert b[addr:addr + 4] == b"HEAP"
        size, _free, data = struct.unpack("<QQQ", b[addr + 8:addr + 32])
        return b[data:data + size]

    def _group_btree(self, addr):
        b = self.b
        assert b[addr:addr + 4] == b"TREE"
        level = b[addr + 5]
        used = struct.unpack("<H", b[addr + 6:addr + 8])[0]
        p = addr + 24 + 8  # skip header and the first key
        out = []
        for _ in range(used):
            child = struct.unpack("<Q", b[p:p + 8])[0]
            p += 16  # child pointer + next key
            if level > 0:
                out.extend(self._group_btree(child))
            else:
                assert b[child:child + 4] == b"SNOD"
                n = struct.unpack("<H", b[child + 6:child + 8])[0]
                for i in range(n):
                    e = child + 8 + 40 * i
                    out.append(struct.unpack("<QQ", b[e:e + 16]))
        return out

    def read(self, name):
        msgs = dict()
        for mtype, body in self._messages(self.datasets[name]):
            msgs.setdefault(mtype, body)
        ds = msgs[0x1]
        nd = ds[1]
        off = 8 if ds[0] == 1 else 4
        dims = struct.unpack("<%dQ" % nd, ds[off:off + 8 * nd])
        dt = msgs[0x3]
        cls, size = dt[0] & 0x0F, struct.unpack("<I", dt[4:8])[0]
        dtype = {(1, 8): "<f8", (1, 4): "<f4", (0, 4): "<i4", (0, 8): "<i8"}[(cls, size)]
        lay = msgs[0x8]
        if lay[0] != 3:
            raise ValueError("only layout message version 3 is supported")
        if lay[1] == 1:  # contiguous
            addr, size_b = struct.unpack("<QQ", lay[2:18])
            return np.frombuffer(self.b[addr:addr + size_b], dtype=dtype).reshape(dims).copy()
        if lay[1] != 2:
            raise ValueError("unsupported layout class")
        cnd = lay[2]
        btree = struct.unpack("<Q", lay[3:11])[0]
        cdims = struct.unpack("<%dI" % cnd, lay[11:11 + 4 * cnd])[:-1]
        deflate = 0xB in msgs
        arr = np.zeros(dims, dtype=dtype)
        self._chunks(btree, cnd, cdims, dims, dtype, deflate, arr)
        return arr

    def _chunks(self, addr, cnd, cdims, dims, dtype, deflate, arr):
        b = self.b
        assert b[addr:addr + 4] == b"TREE"
        level = b[addr + 5]
        used = struct.unpack("<H", b[addr + 6:addr + 8])[0]
        ks = 8 + 8 * cnd
        p = addr + 24
        for _ in range(used):
            csz, mask = struct.unpack("<II", b[p:p + 8])
            offs = struct.unpack("<%dQ" % cnd, b[p + 8:p + ks])
            child = struct.unpack("<Q", b[p + ks:p + ks + 8])[0]
            p += ks + 8
            if level > 0:
                self._chunks(child, cnd, cdims, dims, dtype, deflate, arr)
                continue
            raw = b[child:child + csz]
            if deflate and mask == 0:
                raw = zlib.decompress(raw)
            chunk = np.frombuffer(raw, dtype=dtype).reshape(cdims)
            sl = tuple(slice(offs[j], min(offs[j] + cdims[j], dims[j])) for j in range(len(dims)))
            arr[sl] = chunk[tuple(slice(0, s.stop - s.start) for s in sl)]


def main(data_dir):
    inp = H5File(os.path.join(data_dir, "Oil.h5"))
    out = H5File(os.path.join(data_dir, "Oil.out.h5"))
    g = {
        "T_in": inp.read("T"),
        "lb_in": inp.read("lb"),
        "id_in": inp.read("id"),
    }
    for name in ("T", "FI", "W", "X", "Y", "M", "beta", "lb"):
        g[name] = out.read(name + ".dat")
    R = out.read("R.dat")
    cols = np.arange(0, R.shape[1], 8)
    g["R_cols"] = cols
    g["R_sub"] = R[:, cols]
    g["R_colsum"] = R.sum(axis=0)
    g["R_rowsum"] = R.sum(axis=1)
    here = os.path.dirname(os.path.abspath(__file__))
    np.savez_compressed(os.path.join(here, "oil_golden.npz"), **g)
    # the input file itself (written by the HDF5 library the reference links),
    # the fixture of the command-line driver's reader
    shutil.copyfile(os.path.join(data_dir, "Oil.h5"), os.path.join(here, "oil_input.h5"))
    shutil.copyfile(os.path.join(data_dir, "Oil.out.h5"), os.path.join(here, "oil_output.h5"))
    for k, v in g.items():
        print(k, v.shape, v.dtype)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <the reference checkout's data directory>")
    main(sys.argv[1])
