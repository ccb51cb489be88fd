"""Extract the POM acceptance tables from the reference's assets (run once;
the committed CSVs are what the package reads).

* assets/pmt_acc.hd5 -> pom_pmt_acceptance.csv (wavelength, acc_pmt_grp_1,
  acc_pmt_grp_2) and pom_pmt_sigma.csv (sigma_grp_1, sigma_grp_2): the
  POMAcceptance inputs (src/pom.jl:16-34).
* assets/PMTAcc.csv -> pom_rel_qe.csv (wavelength, rel_acceptance): the POM's
  InterpQuantumEff table (src/pom.jl:90, src/detection.jl:170-184).

h5py is not available here, so the file is read by a minimal reader of the
HDF5 structures it uses (version-0 superblock, a root group holding link
messages or a symbol table, version-1 object headers with continuations,
float64 datasets stored contiguously or compactly).  Usage: python extract_pom_tables.py [reference_root]
"""
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class H5:
    def __init__(self, path):
        self.d = open(path, "rb").read()
        d = self.d
        if d[:8] != b"\x89HDF\r\n\x1a\n" or d[8] != 0:
            raise ValueError("expected an HDF5 file with a version-0 superblock")
        if d[13] != 8 or d[14] != 8:
            raise ValueError("expected 8-byte offsets and lengths")
        # root symbol-table entry at 56: name offset, object header address
        self.root = struct.unpack_from("<Q", d, 56 + 8)[0]

    def u(self, fmt, off):
        return struct.unpack_from(fmt, self.d, off)

    def heap_name(self, heap, off):
        d = self.d
        if d[heap:heap + 4] != b"HEAP":
            raise ValueError("bad local heap")
        data = self.u("<Q", heap + 24)[0]
        end = d.index(b"\0", data + off)
        return d[data + off:end].decode()

    def group(self):
        """{name: object header address} of the root group: its link messages
        (compact group storage) or, for old-style groups, the symbol table."""
        out = {}
        msgs = self.messages(self.root)
        for mtype, body, _ in msgs:
            if mtype == 0x6:
                name, addr = self._link(body)
                out[name] = addr
        for mtype, body, _ in msgs:
            if mtype == 0x11:
                btree, self.root_heap = self.u("<QQ", body)
                self._walk(btree, out)
        return out

    def _link(self, p):
        d = self.d
        if d[p] != 1:
            raise ValueError("unknown link message version")
        flags = d[p + 1]
        p += 2
        ltype = 0
        if flags & 0x08:
            ltype = d[p]
            p += 1
        if flags & 0x04:
            p += 8  # creation order
        if flags & 0x10:
            p += 1  # character set
        nlen_size = 1 << (flags & 3)
        nlen = int.from_bytes(d[p:p + nlen_size], "little")
        p += nlen_size
        name = d[p:p + nlen].decode()
        p += nlen
        if ltype != 0:
            raise ValueError("only hard links are handled")
        return name, self.u("<Q", p)[0]

    def _walk(self, node, out):
        d = self.d
        if d[node:node + 4] != b"TREE":
            raise ValueError("bad B-tree node")
        ntype, level, used = d[node + 4], d[node + 5], self.u("<H", node + 6)[0]
        if ntype != 0:
            raise ValueError("expected a group B-tree")
        p = node + 24 + 8  # past the first key
        for _ in range(used):
            child = self.u("<Q", p)[0]
            p += 16  # child + next key
            if level > 0:
                self._walk(child, out)
            else:
                self._snod(child, out)

    def _snod(self, node, out):
        d = self.d
        if d[node:node + 4] != b"SNOD":
            raise ValueError("bad symbol table node")
        n = self.u("<H", node + 6)[0]
        for i in range(n):
            e = node + 8 + 40 * i
            name_off, addr = self.u("<QQ", e)
            out[self.heap_name(self.root_heap, name_off)] = addr

    def messages(self, addr):
        d = self.d
        if d[addr] != 1:
            raise ValueError("expected a version-1 object header")
        nmsg = self.u("<H", addr + 2)[0]
        size = self.u("<I", addr + 8)[0]
        blocks = [(addr + 16, size)]
        msgs = []
        while blocks and len(msgs) < nmsg:
            p, n = blocks.pop(0)
            end = p + n
            while p + 8 <= end and len(msgs) < nmsg:
                mtype, msize = self.u("<HH", p)
                body = p + 8
                if mtype == 0x10:  # continuation
                    blocks.append(self.u("<QQ", body))
                msgs.append((mtype, body, msize))
                p = body + msize
        return msgs

    def dataset(self, addr):
        dims, dtype, raw = None, None, None
        for mtype, body, msize in self.messages(addr):
            d = self.d
            if mtype == 0x1:  # dataspace
                ver, rank = d[body], d[body + 1]
                off = body + (8 if ver == 1 else 4)
                dims = [self.u("<Q", off + 8 * i)[0] for i in range(rank)]
            elif mtype == 0x3:  # datatype
                cls = d[body] & 0x0F
                size = self.u("<I", body + 4)[0]
                big = d[body + 1] & 1
                if cls != 1 or size != 8 or big:
                    raise ValueError("expected little-endian float64")
                dtype = "<f8"
            elif mtype == 0x8:  # data layout
                ver = d[body]
                if ver != 3:
                    raise ValueError("expected a version-3 layout message")
                cls = d[body + 1]
                if cls == 0:
                    n = self.u("<H", body + 2)[0]
                    raw = d[body + 4:body + 4 + n]
                elif cls == 1:
                    a, n = self.u("<QQ", body + 2)
                    raw = d[a:a + n]
                else:
                    raise ValueError("chunked datasets are not handled")
        if dtype is None or raw is None or dims is None:
            raise ValueError("incomplete dataset header")
        arr = np.frombuffer(raw, dtype)
        n = int(np.prod(dims)) if dims else 1
        return arr[:n].reshape(dims) if dims else arr[0]


def main(ref):
    h = H5(os.path.join(ref, "assets", "pmt_acc.hd5"))
    g = h.group()
    wl = h.dataset(g["wavelengths"])
    a1 = h.dataset(g["acc_pmt_grp_1"])
    a2 = h.dataset(g["acc_pmt_grp_2"])
    s1 = float(h.dataset(g["sigma_grp_1"]))
    s2 = float(h.dataset(g["sigma_grp_2"]))
    assert wl.shape == a1.shape == a2.shape and np.all(np.diff(wl) > 0)
    with open(os.path.join(HERE, "pom_pmt_acceptance.csv"), "w") as f:
        f.write("wavelength,acc_pmt_grp_1,acc_pmt_grp_2\n")
        for row in zip(wl, a1, a2):
            f.write(",".join(repr(float(v)) for v in row) + "\n")
    with open(os.path.join(HERE, "pom_pmt_sigma.csv"), "w") as f:
        f.write("sigma_grp_1,sigma_grp_2\n%r,%r\n" % (s1, s2))
    src = open(os.path.join(ref, "assets", "PMTAcc.csv")).read().splitlines()
    with open(os.path.join(HERE, "pom_rel_qe.csv"), "w") as f:
        f.write("wavelength,rel_acceptance\n")
        for line in src[1:]:
            if line.strip():
                w, a = (float(v) for v in line.split(","))
                f.write("%r,%r\n" % (w, a))
    print("wavelengths", wl.min(), wl.max(), len(wl), "sigmas", s1, s2)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PP_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: %s <reference checkout> (or set PP_REFERENCE_ROOT)" % sys.argv[0])
    main(root)
