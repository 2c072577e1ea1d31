"""Golden vectors for the Output2HRTF post-processing: the reference's own
SHTF test project (mesh2hrtf tests/resources/SHTF: 2 ear sources, 60
frequencies, evaluation grid FourPointHorPlane_r100cm) and the HRTF / HRIR
SOFA files the reference's output2hrtf wrote for it.

    python tests/golden/make_output2hrtf_golden.py

with MESH2HRTF_REFERENCE set to the root of a Mesh2HRTF checkout.

Writes tests/golden/shtf_output2hrtf.npz: the project's parameters, the grid
nodes, the pEvalGrid text lines of every source and step (as the reference
printed them), and every variable and attribute of the two SOFA files.

The SOFA files are netCDF-4 (HDF5) and no HDF5 library is installed, so this
script carries a small HDF5 reader of its own, restated from the published
HDF5 file format specification (version 3): superblock 2/3, object headers
1/2 with continuation blocks, compact and dense (fractal heap + version 2
B-tree) links and attributes, contiguous, compact and chunked (version 1
B-tree index) layouts with the deflate and shuffle filters, and fixed-point,
floating-point and fixed-length string types.  It reads what these files
hold and refuses anything else.  Test infrastructure only: the library never
imports it.
"""
from __future__ import annotations

import json
import os
import pathlib
import struct
import sys
import zlib

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


class H5:
    def __init__(self, path):
        self.d = pathlib.Path(path).read_bytes()
        d = self.d
        if d[:8] != b"\x89HDF\r\n\x1a\n":
            raise ValueError("not an HDF5 file")
        ver = d[8]
        if ver not in (2, 3):
            raise ValueError("superblock version %d not supported" % ver)
        self.so, self.sl = d[9], d[10]
        if self.so != 8 or self.sl != 8:
            raise ValueError("only 8-byte offsets and lengths")
        self.root = struct.unpack_from("<Q", d, 12 + 24)[0]

    # ---------------------------------------------------------------- helpers
    def u(self, off, n):
        return int.from_bytes(self.d[off:off + n], "little")

    # ------------------------------------------------------------ object header
    def messages(self, addr):
        """[(type, flags, body bytes)] of the object header at addr."""
        d = self.d
        out = []
        if d[addr:addr + 4] == b"OHDR":
            flags = d[addr + 5]
            p = addr + 6
            if flags & 0x20:
                p += 16
            if flags & 0x10:
                p += 4
            nsz = 1 << (flags & 3)
            size0 = self.u(p, nsz)
            p += nsz
            blocks = [(p, size0)]
            crt = bool(flags & 0x04)
            while blocks:
                start, size = blocks.pop(0)
                q, end = start, start + size
                while q + 4 <= end:
                    mt, ms, mf = d[q], self.u(q + 1, 2), d[q + 3]
                    q += 4 + (2 if crt else 0)
                    body = d[q:q + ms]
                    q += ms
                    if mt == 0x10:
                        caddr, clen = struct.unpack_from("<QQ", body)
                        if d[caddr:caddr + 4] != b"OCHK":
                            raise ValueError("bad continuation block")
                        blocks.append((caddr + 4, clen - 8))
                    else:
                        out.append((mt, mf, body))
            return out
        # version 1 object header
        if d[addr] != 1:
            raise ValueError("unknown object header at %d" % addr)
        nmsg = self.u(addr + 2, 2)
        size = self.u(addr + 8, 4)
        blocks = [(addr + 16, size)]
        while blocks and len(out) < nmsg:
            start, size = blocks.pop(0)
            q, end = start, start + size
            while q + 8 <= end:
                mt, ms, mf = self.u(q, 2), self.u(q + 2, 2), d[q + 4]
                body = d[q + 8:q + 8 + ms]
                q += 8 + ms
                if mt == 0x10:
                    caddr, clen = struct.unpack_from("<QQ", body)
                    blocks.append((caddr, clen))
                else:
                    out.append((mt, mf, body))
        return out

    # ------------------------------------------------------------ fractal heap
    def heap(self, addr):
        d = self.d
        if d[addr:addr + 4] != b"FRHP":
            raise ValueError("bad fractal heap")
        p = addr + 5
        idlen, filt_len, flags = self.u(p, 2), self.u(p + 2, 2), d[p + 4]
        if filt_len:
            raise ValueError("filtered fractal heaps not supported")
        p += 5
        max_obj = self.u(p, 4)
        p += 4 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8
        width = self.u(p, 2)
        start_bs, max_dbs = self.u(p + 2, 8), self.u(p + 10, 8)
        max_bits = self.u(p + 18, 2)
        root = self.u(p + 22, 8)
        cur_rows = self.u(p + 30, 2)
        return dict(idlen=idlen, flags=flags, max_obj=max_obj, width=width, start=start_bs,
                    max_dbs=max_dbs, bits=max_bits, root=root, rows=cur_rows, addr=addr)

    def _row_size(self, h, r):
        return h["start"] if r < 2 else h["start"] << (r - 1)

    def _direct_blocks(self, h, iaddr, nrows):
        """[(heap offset, address, size)] of the direct blocks below an
        indirect block (row-major, as the doubling table lays them out)."""
        d = self.d
        if d[iaddr:iaddr + 4] != b"FHIB":
            raise ValueError("bad indirect block")
        offb = (h["bits"] + 7) // 8
        p = iaddr + 5 + 8
        base = self.u(p, offb)
        p += offb
        max_drows = (h["max_dbs"].bit_length() - 1) - (h["start"].bit_length() - 1) + 2
        out, off = [], base
        for r in range(nrows):
            bs = self._row_size(h, r)
            for _ in range(h["width"]):
                a = self.u(p, 8)
                p += 8
                if r < max_drows:
                    if a != UNDEF:
                        out.append((off, a, bs))
                elif a != UNDEF:
                    # child indirect block: rows below it follow from its size
                    sub = (bs * h["width"]).bit_length() - 1
                    sub_rows = sub - (h["start"] * h["width"]).bit_length() + 2
                    out += self._direct_blocks(h, a, sub_rows)
                off += bs
        return out

    def heap_object(self, h, hid):
        t = (hid[0] >> 4) & 3
        if t == 2:                         # tiny: data in the ID
            n = (hid[0] & 0x0F) + 1
            return hid[1:1 + n]
        if t != 0:
            raise ValueError("huge heap objects not supported")
        offb = (h["bits"] + 7) // 8
        lenb = (min(h["max_dbs"], h["max_obj"]).bit_length() + 7) // 8
        off = int.from_bytes(hid[1:1 + offb], "little")
        ln = int.from_bytes(hid[1 + offb:1 + offb + lenb], "little")
        if h["rows"] == 0:
            blocks = [(0, h["root"], h["start"])]
        else:
            blocks = self._direct_blocks(h, h["root"], h["rows"])
        for boff, baddr, bs in blocks:
            if boff <= off < boff + bs:
                if self.d[baddr:baddr + 4] != b"FHDB":
                    raise ValueError("bad direct block")
                a = baddr + (off - boff)
                return self.d[a:a + ln]
        raise ValueError("heap offset %d not found" % off)

    def btree2_records(self, addr):
        d = self.d
        if d[addr:addr + 4] != b"BTHD":
            raise ValueError("bad v2 B-tree")
        rsize = self.u(addr + 10, 2)
        depth = self.u(addr + 12, 2)
        root = self.u(addr + 16, 8)
        nroot = self.u(addr + 24, 2)
        if depth != 0:
            raise ValueError("v2 B-trees deeper than a leaf not supported")
        if d[root:root + 4] != b"BTLF":
            raise ValueError("bad v2 B-tree leaf")
        p = root + 6
        return [d[p + i * rsize:p + (i + 1) * rsize] for i in range(nroot)]

    # ------------------------------------------------------------ links, attrs
    def _link(self, b):
        flags = b[1]
        p = 2
        ltype = 0
        if flags & 0x08:
            ltype = b[p]
            p += 1
        if flags & 0x04:
            p += 8
        if flags & 0x10:
            p += 1
        nb = 1 << (flags & 3)
        n = int.from_bytes(b[p:p + nb], "little")
        p += nb
        name = b[p:p + n].decode()
        p += n
        if ltype != 0:
            return name, None
        return name, int.from_bytes(b[p:p + 8], "little")

    def links(self, addr):
        out = {}
        for mt, mf, b in self.messages(addr):
            if mt == 0x06:
                k, v = self._link(b)
                out[k] = v
            elif mt == 0x02:
                flags = b[1]
                p = 2 + (8 if flags & 1 else 0)
                haddr, naddr = struct.unpack_from("<QQ", b, p)
                if haddr == UNDEF:
                    continue
                h = self.heap(haddr)
                for rec in self.btree2_records(naddr):
                    k, v = self._link(self.heap_object(h, rec[4:4 + h["idlen"]]))
                    out[k] = v
            elif mt == 0x11:
                raise ValueError("version 1 groups (symbol tables) not supported")
        return out

    def _attribute(self, b):
        ver = b[0]
        nlen, tlen, slen = self.u_b(b, 2, 2), self.u_b(b, 4, 2), self.u_b(b, 6, 2)
        if ver == 1:
            p = 8
            pad = lambda x: (x + 7) & ~7
            name = b[p:p + nlen].rstrip(b"\0").decode()
            p += pad(nlen)
            dt = b[p:p + tlen]
            p += pad(tlen)
            ds = b[p:p + slen]
            p += pad(slen)
        else:
            p = 8 + (1 if ver == 3 else 0)
            name = b[p:p + nlen].rstrip(b"\0").decode()
            p += nlen
            dt = b[p:p + tlen]
            p += tlen
            ds = b[p:p + slen]
            p += slen
        shape = self.dataspace(ds)
        return name, self.decode(dt, shape, b[p:])

    @staticmethod
    def u_b(b, off, n):
        return int.from_bytes(b[off:off + n], "little")

    def attributes(self, addr):
        out = {}
        for mt, mf, b in self.messages(addr):
            if mt == 0x0C:
                try:
                    k, v = self._attribute(b)
                    out[k] = v
                except NotImplementedError:
                    pass
            elif mt == 0x15:
                flags = b[1]
                p = 2 + (2 if flags & 1 else 0)
                haddr, naddr = struct.unpack_from("<QQ", b, p)
                if haddr == UNDEF:
                    continue
                h = self.heap(haddr)
                for rec in self.btree2_records(naddr):
                    try:
                        k, v = self._attribute(self.heap_object(h, rec[:8]))
                        out[k] = v
                    except NotImplementedError:
                        pass
        return out

    # ------------------------------------------------------------ types, data
    def dataspace(self, b):
        ver, rank, flags = b[0], b[1], b[2]
        if ver == 1:
            p = 8
        else:
            p = 4
            if b[3] == 2:        # null dataspace
                return None
        return tuple(self.u_b(b, p + 8 * i, 8) for i in range(rank))

    def dtype(self, b):
        cls, ver = b[0] & 0x0F, b[0] >> 4
        bits = b[1] | (b[2] << 8) | (b[3] << 16)
        size = self.u_b(b, 4, 4)
        order = ">" if bits & 1 else "<"
        if cls == 0:
            return np.dtype("%s%s%d" % (order, "i" if bits & 8 else "u", size))
        if cls == 1:
            return np.dtype("%sf%d" % (order, size))
        if cls == 3:
            return ("str", size)
        raise NotImplementedError("datatype class %d" % cls)

    def decode(self, dt, shape, raw):
        t = self.dtype(dt)
        n = 1 if not shape else int(np.prod(shape))
        if isinstance(t, tuple):
            s = raw[:t[1] * n]
            vals = [s[i * t[1]:(i + 1) * t[1]].split(b"\0")[0].decode("utf-8", "replace") for i in range(n)]
            return vals[0] if n == 1 else np.array(vals).reshape(shape)
        a = np.frombuffer(raw[:t.itemsize * n], t).copy()
        return a.reshape(shape) if shape else a[0]

    def dataset(self, addr):
        dt = shape = layout = None
        filters = []
        for mt, mf, b in self.messages(addr):
            if mt == 0x01:
                shape = self.dataspace(b)
            elif mt == 0x03:
                dt = b
            elif mt == 0x08:
                layout = b
            elif mt == 0x0B:
                filters = self.filters(b)
        t = self.dtype(dt)
        if isinstance(t, tuple):
            raise NotImplementedError("string datasets")
        n = int(np.prod(shape)) if shape else 1
        ver, cls = layout[0], layout[1]
        if ver != 3:
            raise NotImplementedError("data layout version %d" % ver)
        if cls == 0:
            sz = self.u_b(layout, 2, 2)
            raw = layout[4:4 + sz]
        elif cls == 1:
            a, sz = struct.unpack_from("<QQ", layout, 2)
            raw = self.d[a:a + sz] if a != UNDEF else bytes(n * t.itemsize)
        elif cls == 2:
            rank1 = layout[2]
            bt = self.u_b(layout, 3, 8)
            cdims = [self.u_b(layout, 11 + 4 * i, 4) for i in range(rank1)]
            return self.chunked(bt, cdims[:-1], shape, t, filters)
        else:
            raise NotImplementedError("layout class %d" % cls)
        return np.frombuffer(raw[:n * t.itemsize], t).reshape(shape).copy()

    def filters(self, b):
        ver, nf = b[0], b[1]
        p = 8 if ver == 1 else 2
        out = []
        for _ in range(nf):
            fid = self.u_b(b, p, 2)
            p += 2
            nlen = 0
            if ver == 1 or fid >= 256:
                nlen = self.u_b(b, p, 2)
                p += 2
            p += 2                              # flags
            ncd = self.u_b(b, p, 2)
            p += 2
            if ver == 1:
                p += (nlen + 7) & ~7
            else:
                p += nlen
            cd = [self.u_b(b, p + 4 * i, 4) for i in range(ncd)]
            p += 4 * ncd
            if ver == 1 and ncd % 2:
                p += 4
            out.append((fid, cd))
        return out

    def chunked(self, bt, cdims, shape, t, filters):
        out = np.zeros(shape, t)
        csize = int(np.prod(cdims)) * t.itemsize
        rank = len(shape)
        if bt == UNDEF:                         # nothing written: fill value (0)
            return out
        for off, mask, size, addr in self._chunks(bt, rank + 1):
            raw = self.d[addr:addr + size]
            for i, (fid, cd) in reversed(list(enumerate(filters))):
                if mask & (1 << i):
                    continue
                if fid == 1:
                    raw = zlib.decompress(raw)
                elif fid == 2:
                    es = cd[0] if cd else t.itemsize
                    m = len(raw) // es
                    raw = np.frombuffer(raw[:m * es], np.uint8).reshape(es, m).T.tobytes()
                else:
                    raise NotImplementedError("filter %d" % fid)
            chunk = np.frombuffer(raw[:csize], t).reshape(cdims)
            sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(off, cdims, shape))
            out[sl] = chunk[tuple(slice(0, x.stop - x.start) for x in sl)]
        return out

    def _chunks(self, addr, ndims):
        d = self.d
        if d[addr:addr + 4] != b"TREE":
            raise ValueError("bad chunk B-tree")
        ntype, level, used = d[addr + 4], d[addr + 5], self.u(addr + 6, 2)
        if ntype != 1:
            raise ValueError("not a chunk B-tree")
        p = addr + 24
        ksize = 8 + 8 * ndims
        out = []
        for i in range(used):
            size, mask = self.u(p, 4), self.u(p + 4, 4)
            off = [self.u(p + 8 + 8 * j, 8) for j in range(ndims - 1)]
            child = self.u(p + ksize, 8)
            if level == 0:
                out.append((off, mask, size, child))
            else:
                out += self._chunks(child, ndims)
            p += ksize + 8
        return out


def read_sofa(path):
    """{name: value} of a SOFA file: global attributes as GLOBAL_<name>,
    variables by name with '.' as '_' (sofar's naming), variable attributes
    as <variable>_<name>."""
    f = H5(path)
    out = {}
    for k, v in f.attributes(f.root).items():
        if not k.startswith("_"):
            out["GLOBAL_" + k] = v
    for name, addr in f.links(f.root).items():
        key = name.replace(".", "_")
        attrs = f.attributes(addr)
        if attrs.get("CLASS") == "DIMENSION_SCALE" and str(attrs.get("NAME", "")).startswith("This is a netCDF dimension"):
            out["_dim_" + name] = f.dataset(addr).shape[0]
            continue
        out[key] = f.dataset(addr)
        for a, v in attrs.items():
            if a in ("DIMENSION_LIST", "_Netcdf4Dimid", "_Netcdf4Coordinates", "CLASS", "NAME", "REFERENCE_LIST"):
                continue
            out[key + "_" + a] = v
    return out


def main(ref_root):
    shtf = os.path.join(ref_root, "tests", "resources", "SHTF")
    params = json.loads(pathlib.Path(os.path.join(shtf, "parameters.json")).read_text())
    grid = params["evaluationGrids"][0]
    nodes = np.loadtxt(os.path.join(shtf, "EvaluationGrids", grid, "Nodes.txt"), skiprows=1, ndmin=2)
    lines = []
    for s in range(params["numSources"]):
        for k in range(params["numFrequencies"]):
            p = os.path.join(shtf, "NumCalc", "source_%d" % (s + 1), "be.out", "be.%d" % (k + 1), "pEvalGrid")
            lines.append(pathlib.Path(p).read_text())
    keep = {"Mesh2HRTF_Version", "speedOfSound", "densityOfMedium", "evaluationGrids", "sourceType",
            "numSources", "sourceCenter", "sourceArea", "reference", "computeHRIRs", "numFrequencies",
            "frequencies"}
    out = {"params_json": json.dumps({k: params[k] for k in keep}),
           "grid_name": grid, "grid_nodes": nodes, "pEvalGrid_text": np.array(lines)}
    for kind in ("HRTF", "HRIR"):
        s = read_sofa(os.path.join(shtf, "Output2HRTF", "%s_%s.sofa" % (kind, grid)))
        for k, v in s.items():
            out["%s__%s" % (kind, k)] = np.asarray(v)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "shtf_output2hrtf.npz")
    np.savez_compressed(dst, **out)
    print("wrote %s (%d arrays)" % (dst, len(out)))
    for k in sorted(out):
        v = np.asarray(out[k])
        if k.endswith("_text") or k == "params_json":
            continue
        print("  %-50s %s %s" % (k, v.dtype, v.shape if v.ndim else repr(v.item())[:60]))


if __name__ == "__main__":
    root = os.environ.get("MESH2HRTF_REFERENCE", "")
    if not os.path.isdir(root):
        sys.exit("set MESH2HRTF_REFERENCE to the root of a Mesh2HRTF checkout")
    main(root)
