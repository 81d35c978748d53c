"""A minimal HDF5 reader and writer for the reference's trajectory files
(src/Saver.cpp:184-427 writes them, src/Loader.cpp:3-267 reads them, both
through libhdf5's C++ API, which is not available here).

Only the subset those files use is implemented, from the published HDF5
file-format specification (version 0 superblock, version 1 object headers):
groups as symbol tables (a version 1 B-tree of SNOD nodes over a local
heap), datasets with contiguous or compact layout, little-endian IEEE
doubles, 32/64-bit integers and compound types of those. The writer emits
the same structures in the same format versions.

    f = read(path)          # {"/Properties/Size": ndarray, "/Steps/Position/Node 0 0/LPOS": ndarray, ...}
    write(path, datasets)   # the same mapping back to a file
"""
from __future__ import annotations

import struct
from typing import Dict

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(ValueError):
    pass


# ---------------------------------------------------------------- reading
class _Reader:
    def __init__(self, data: bytes):
        self.d = data
        if data[:8] != SIGNATURE:
            raise H5Error("not an HDF5 file")
        if data[8] != 0:
            raise H5Error("superblock version %d not supported (only 0)" % data[8])
        self.so, self.sl = data[13], data[14]
        if self.so != 8 or self.sl != 8:
            raise H5Error("only 8-byte offsets and lengths are supported")
        self.root = self.entry(56)

    def u(self, off, n):
        return int.from_bytes(self.d[off:off + n], "little")

    def entry(self, off):
        """symbol table entry: (name offset, object header address, cache type, scratch)"""
        return (self.u(off, 8), self.u(off + 8, 8), self.u(off + 16, 4), self.d[off + 24:off + 40])

    def messages(self, addr):
        """(type, data) of an object header's messages, continuations followed"""
        d = self.d
        if d[addr] != 1:
            raise H5Error("object header version %d not supported (only 1)" % d[addr])
        nmsg = self.u(addr + 2, 2)
        size = self.u(addr + 8, 4)
        blocks = [(addr + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            start, length = blocks.pop(0)
            p = start
            while p + 8 <= start + length and len(out) < nmsg:
                mtype, msize = self.u(p, 2), self.u(p + 2, 2)
                body = d[p + 8:p + 8 + msize]
                if mtype == 0x10:  # continuation
                    blocks.append((self.u(p + 8, 8), self.u(p + 16, 8)))
                out.append((mtype, body))
                p += 8 + msize
        return out

    def heap_name(self, heap, off):
        if self.d[heap:heap + 4] != b"HEAP":
            raise H5Error("bad local heap")
        seg = self.u(heap + 24, 8)
        end = self.d.index(b"\x00", seg + off)
        return self.d[seg + off:end].decode()

    def group(self, btree, heap):
        """{name: object header address} of a symbol-table group"""
        out = {}
        d = self.d
        if d[btree:btree + 4] != b"TREE":
            raise H5Error("bad B-tree node")
        level, used = d[btree + 5], self.u(btree + 6, 2)
        p = btree + 24 + 8  # past the header and key 0
        for _ in range(used):
            child = self.u(p, 8)
            p += 16  # child, next key
            if level > 0:
                out.update(self.group(child, heap))
                continue
            if d[child:child + 4] != b"SNOD":
                raise H5Error("bad symbol node")
            for k in range(self.u(child + 6, 2)):
                name_off, hdr, _, _ = self.entry(child + 8 + 40 * k)
                out[self.heap_name(heap, name_off)] = hdr
        return out

    def walk(self, addr, path, out):
        msgs = self.messages(addr)
        types = {t for t, _ in msgs}
        if 0x11 in types:  # group
            body = next(b for t, b in msgs if t == 0x11)
            btree, heap = struct.unpack_from("<QQ", body)
            for name, hdr in sorted(self.group(btree, heap).items()):
                self.walk(hdr, path.rstrip("/") + "/" + name, out)
        elif 0x08 in types:
            out[path] = self.dataset(msgs)

    def dataset(self, msgs):
        space = next(b for t, b in msgs if t == 0x01)
        dtype = _parse_dtype(next(b for t, b in msgs if t == 0x03))[0]
        layout = next(b for t, b in msgs if t == 0x08)
        ver, nd = space[0], space[1]
        dims = struct.unpack_from("<%dQ" % nd, space, 8 if ver == 1 else 4)
        count = int(np.prod(dims)) if nd else 1
        nbytes = count * dtype.itemsize
        if layout[0] != 3:
            raise H5Error("data layout version %d not supported (only 3)" % layout[0])
        if layout[1] == 0:  # compact
            size = struct.unpack_from("<H", layout, 2)[0]
            raw = layout[4:4 + size]
        elif layout[1] == 1:  # contiguous
            addr, size = struct.unpack_from("<QQ", layout, 2)
            raw = self.d[addr:addr + size] if addr != UNDEF else bytes(nbytes)
        else:
            raise H5Error("chunked datasets are not supported")
        return np.frombuffer(raw[:nbytes], dtype=dtype).reshape(dims).copy()


def _parse_dtype(b):
    """numpy dtype of a datatype message, and its length in bytes"""
    cls, ver = b[0] & 0x0F, b[0] >> 4
    bits = int.from_bytes(b[1:4], "little")
    size = struct.unpack_from("<I", b, 4)[0]
    if cls == 0:  # fixed point
        if bits & 1:
            raise H5Error("big-endian integers not supported")
        return np.dtype(("<i%d" if bits & 8 else "<u%d") % size), 12
    if cls == 1:  # IEEE float
        if bits & 1:
            raise H5Error("big-endian floats not supported")
        return np.dtype("<f%d" % size), 20
    if cls == 6:  # compound
        n = bits & 0xFFFF
        p = 8
        names, formats, offsets = [], [], []
        for _ in range(n):
            end = b.index(b"\x00", p)
            names.append(b[p:end].decode())
            if ver < 3:
                p = p + ((end - p) // 8 + 1) * 8
                off = struct.unpack_from("<I", b, p)[0]
                p += 4
                if ver == 1:
                    p += 28  # dimensionality, permutation, reserved, sizes
            else:
                p = end + 1
                w = max(1, (size.bit_length() + 7) // 8)
                off = int.from_bytes(b[p:p + w], "little")
                p += w
            t, used = _parse_dtype(b[p:])
            formats.append(t)
            offsets.append(off)
            p += used
        return np.dtype(dict(names=names, formats=formats, offsets=offsets, itemsize=size)), p
    raise H5Error("datatype class %d not supported" % cls)


def read(path: str) -> Dict[str, np.ndarray]:
    """Every dataset of the file by its absolute path."""
    with open(path, "rb") as f:
        r = _Reader(f.read())
    out = {}
    r.walk(r.root[1], "/", out)
    return out


# ---------------------------------------------------------------- writing
LEAF_K, INTERNAL_K = 4, 16  # the library defaults the reference's files carry


def _pad8(n):
    return (n + 7) // 8 * 8


def _dtype_message(dt: np.dtype) -> bytes:
    """datatype message body (version 1 encodings, as the reference's files)"""
    if dt.names:
        members = b""
        for name in dt.names:
            sub, off = dt.fields[name][0], dt.fields[name][1]
            nb = name.encode() + b"\x00"
            members += nb + bytes(_pad8(len(nb)) - len(nb)) + struct.pack("<I", off) + bytes(28)
            members += _dtype_message(sub)
        return bytes([0x16]) + struct.pack("<I", len(dt.names))[:3] + struct.pack("<I", dt.itemsize) + members
    if dt.kind == "f" and dt.itemsize in (4, 8):
        if dt.itemsize == 8:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
            return bytes([0x11, 0x20, 0x3F, 0x00]) + struct.pack("<I", 8) + props
        props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
        return bytes([0x11, 0x20, 0x1F, 0x00]) + struct.pack("<I", 4) + props
    if dt.kind in "iu":
        return bytes([0x10, 0x08 if dt.kind == "i" else 0x00, 0, 0]) + struct.pack("<I", dt.itemsize) + \
            struct.pack("<HH", 0, 8 * dt.itemsize)
    raise H5Error("cannot write dtype %s" % dt)


def _msg(mtype, body):
    body = body + bytes(_pad8(len(body)) - len(body))
    return struct.pack("<HHB3x", mtype, len(body), 0) + body


def _object_header(msgs):
    area = b"".join(msgs)
    return struct.pack("<BBHII", 1, 0, len(msgs), 1, len(area)) + bytes(4) + area


class _Writer:
    def __init__(self):
        self.b = bytearray(96)

    def alloc(self, data: bytes) -> int:
        self.b += bytes(_pad8(len(self.b)) - len(self.b))
        a = len(self.b)
        self.b += data
        return a

    def dataset(self, arr: np.ndarray) -> int:
        arr = np.ascontiguousarray(arr)
        dt = arr.dtype.newbyteorder("<") if arr.dtype.byteorder == ">" else arr.dtype
        raw = np.ascontiguousarray(arr, dtype=dt).tobytes()
        addr = self.alloc(raw) if raw else UNDEF
        nd = arr.ndim
        space = struct.pack("<BBB5x", 1, nd, 1) + struct.pack("<%dQ" % nd, *arr.shape) * 2
        # as the reference's saver leaves them: numeric datasets with an explicit
        # zero fill value (its DSetCreatPropList), records with the default
        fill = struct.pack("<BBBBI", 2, 2, 2, 1, 0) if dt.names else \
            struct.pack("<BBBBI", 2, 2, 2, 1, dt.itemsize) + bytes(dt.itemsize)
        layout = struct.pack("<BBQQ", 3, 1, addr, len(raw))
        msgs = [_msg(0x01, space), _msg(0x03, _dtype_message(dt)), _msg(0x05, fill), _msg(0x08, layout)]
        return self.alloc(_object_header(msgs))

    def group(self, tree: dict):
        """writes a group's children, then its heap, symbol nodes and B-tree;
        returns (object header, B-tree, heap) addresses"""
        entries = []
        for name in sorted(tree, key=lambda s: s.encode()):
            node = tree[name]
            if isinstance(node, dict):
                hdr, bt, hp = self.group(node)
                entries.append((name, hdr, 1, struct.pack("<QQ", bt, hp)))
            else:
                entries.append((name, self.dataset(node), 0, bytes(16)))
        heap_data = bytearray(8)  # offset 0: the empty name
        offs = []
        for name, *_ in entries:
            offs.append(len(heap_data))
            nb = name.encode() + b"\x00"
            heap_data += nb + bytes(_pad8(len(nb)) - len(nb))
        seg = self.alloc(bytes(heap_data))
        heap = self.alloc(b"HEAP" + bytes(4) + struct.pack("<QQQ", len(heap_data), 1, seg))
        # symbol nodes of 2 * LEAF_K entries each
        snods = []
        for s in range(0, max(len(entries), 1), 2 * LEAF_K):
            chunk = list(zip(offs, entries))[s:s + 2 * LEAF_K]
            body = b"SNOD" + struct.pack("<BBH", 1, 0, len(chunk))
            for off, (name, hdr, cache, scratch) in chunk:
                body += struct.pack("<QQI4x", off, hdr, cache) + scratch
            body += bytes(8 + 2 * LEAF_K * 40 - len(body))
            snods.append((self.alloc(body), chunk[-1][0] if chunk else 0))
        # B-tree levels of at most 2 * INTERNAL_K children
        level, nodes = 0, snods
        while True:
            parents = []
            for s in range(0, len(nodes), 2 * INTERNAL_K):
                kids = nodes[s:s + 2 * INTERNAL_K]
                body = b"TREE" + struct.pack("<BBH", 0, level, len(kids)) + struct.pack("<QQ", UNDEF, UNDEF)
                body += struct.pack("<Q", 0)
                for addr, last in kids:
                    body += struct.pack("<QQ", addr, last)
                body += bytes(24 + (4 * INTERNAL_K + 1) * 8 - len(body))
                parents.append((self.alloc(body), kids[-1][1]))
            if len(parents) == 1:
                btree = parents[0][0]
                break
            nodes, level = parents, level + 1
        hdr = self.alloc(_object_header([_msg(0x11, struct.pack("<QQ", btree, heap))]))
        return hdr, btree, heap

    def finish(self, root):
        hdr, bt, hp = root
        sb = SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", LEAF_K, INTERNAL_K, 0)
        sb += struct.pack("<QQQQ", 0, UNDEF, len(self.b), UNDEF)
        sb += struct.pack("<QQI4xQQ", 0, hdr, 1, bt, hp)
        self.b[:96] = sb
        return bytes(self.b)


def write(path: str, datasets: Dict[str, np.ndarray]):
    """Writes datasets by absolute path ("/Group/Sub/Name"), groups implied."""
    tree: dict = {}
    for p, arr in datasets.items():
        parts = [s for s in p.split("/") if s]
        node = tree
        for g in parts[:-1]:
            node = node.setdefault(g, {})
        node[parts[-1]] = np.asarray(arr)
    w = _Writer()
    data = w.finish(w.group(tree))
    with open(path, "wb") as f:
        f.write(data)


# ---------------------------------------------------------------- the reference's files
def _node(u, v):
    return "Node %d %d" % (u, v)


def cloth_property_loader(path: str):
    """src/Loader.cpp:3-49: (Size record, Physical properties record) of a
    one-yarn file, as dicts."""
    f = read(path)
    size = f["/Properties/Size"][0]
    phy = f["/Properties/Physical properties"][0]
    return ({k: int(size[k]) for k in size.dtype.names},
            {k: (int(phy[k]) if phy.dtype[k].kind in "iu" else float(phy[k])) for k in phy.dtype.names})


cloth_property_loader_heter = cloth_property_loader  # src/Loader.cpp:51-100: same records, two-yarn fields


def data_loader(path: str, start: int, end: int) -> Dict[str, np.ndarray]:
    """src/Loader.cpp:102-267: steps [start, end) of every node, node index
    u + v W: LPos, LPosFix, LVel [steps, N, 3] and EPos, EPosBar, EVel
    [steps, N, 2]."""
    f = read(path)
    size = f["/Properties/Size"][0]
    W, L = int(size["width"]), int(size["length"])
    names = {"LPos": ("Position", "LPOS"), "LPosFix": ("Position", "LPOSFix"), "LVel": ("Velocity", "LVEL"),
             "EPos": ("Position", "EPOS"), "EPosBar": ("Position", "EPOSBar"), "EVel": ("Velocity", "EVEL")}
    out = {}
    for key, (grp, ds) in names.items():
        out[key] = np.stack([f["/Steps/%s/%s/%s" % (grp, _node(i % W, i // W), ds)][start:end]
                             for i in range(W * L)], axis=1)
    return out


SIZE_DTYPE = np.dtype([("width", "<i4"), ("length", "<i4")])
_PHY_HOMO = ["Gravity", "rho", "R", "L", "Y", "B", "kc", "kf", "df", "mu", "S", "handle_stiff", "wind_velocity_x",
             "wind_velocity_y", "wind_velocity_z", "wind_density", "wind_drag", "woven_pattern"]
_PHY_HETER = ["Gravity", "Yarn1_rho", "Yarn2_rho", "R", "L", "Yarn1_Y", "Yarn2_Y", "Yarn1_B", "Yarn2_B", "kc", "kf",
              "df", "mu", "S", "handle_stiff", "wind_velocity_x", "wind_velocity_y", "wind_velocity_z",
              "wind_density", "wind_drag", "woven_pattern"]


def physical_dtype(heter: bool) -> np.dtype:
    """The Physical properties record (H5Physical / H5PhysicalHeterYarn):
    doubles, then the weave as a 32-bit int, padded to 8 bytes."""
    names = _PHY_HETER if heter else _PHY_HOMO
    return np.dtype(dict(names=names, formats=["<f8"] * (len(names) - 1) + ["<i4"],
                         offsets=[8 * i for i in range(len(names))], itemsize=8 * len(names)))


def save_trajectory(path: str, width: int, length: int, physical: Dict, states: Dict[str, np.ndarray]):
    """The file SaveClothHomoYarn / SaveClothHeterYarn (src/Saver.cpp:
    184-427) leave after a whole run: physical holds the record's fields
    (two-yarn names select the two-yarn record), states the per-step arrays
    as data_loader returns them."""
    heter = "Yarn1_rho" in physical
    pdt = physical_dtype(heter)
    rec = np.zeros(1, pdt)
    for k in pdt.names:
        rec[k] = physical[k]
    ds = {"/Properties/Size": np.array([(width, length)], SIZE_DTYPE), "/Properties/Physical properties": rec}
    names = {"LPos": ("Position", "LPOS"), "LPosFix": ("Position", "LPOSFix"), "LVel": ("Velocity", "LVEL"),
             "EPos": ("Position", "EPOS"), "EPosBar": ("Position", "EPOSBar"), "EVel": ("Velocity", "EVEL")}
    for key, (grp, name) in names.items():
        a = np.asarray(states[key], np.float64)
        for i in range(width * length):
            ds["/Steps/%s/%s/%s" % (grp, _node(i % width, i // width), name)] = a[:, i]
    write(path, ds)
