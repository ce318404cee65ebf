"""Test infrastructure (the oracle): a NumPy reader of the HDF5 subset that the
reference's checkpoints use, and a NumPy writer of the same subset.

Only the tests use this module, to check the library's C++ HDF5 reader and
writer (`ns_3d_staggered_dp_gb300/csrc/ns_h5.cpp`) against a second
implementation.  It follows the published HDF5 File Format Specification
(version 0 superblock, version 1 object headers, symbol-table groups: local
heap, version 1 B-tree, symbol table nodes) for what the reference's HDF5 calls
produce with the library's default property lists:

- `h5ltmake_dataset_double_f` (big_periodic_3D.f90:644-650): a contiguous
  little-endian IEEE double dataset.  The Fortran API reverses the dimensions,
  so the file's dataspace is (nz+2, ny+2, nx+1) for u, and the bytes are the
  Fortran array in memory order;
- `h5ltset_attribute_int_f` / `_double_f` with one value (:637-642): a rank-1,
  one-element attribute of a 32-bit integer or a double;
- `h5ltset_attribute_string_f` (:640): a scalar, null-terminated fixed string
  of strlen + 1 bytes;
- `h5gcreate_f` (:672, :716): a group with a symbol table.

The reading side also follows object header continuations, version 1–3
attribute messages, version 1–2 dataspaces and version 1–3 layouts (compact and
contiguous), which is what other writers of this subset use.  It is pinned on a
file written by the HDF5 library itself: SciPy's MATLAB 7.3 test file
(`testhdf5_7.4_GLNX86.mat`, an HDF5 file after a 512-byte user block), when
SciPy's test data is installed.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(ValueError):
    pass


@dataclass
class Dataset:
    shape: tuple
    dtype: np.dtype
    data: np.ndarray
    attrs: dict = field(default_factory=dict)


@dataclass
class Group:
    members: dict = field(default_factory=dict)  # name -> Group | Dataset
    attrs: dict = field(default_factory=dict)


# --------------------------------------------------------------------------
# reading
# --------------------------------------------------------------------------
class _Reader:
    def __init__(self, buf: bytes):
        self.b = buf
        self.base = None
        for off in (0, 512, 1024, 2048, 4096, 8192):  # user block sizes are powers of two >= 512
            if buf[off:off + 8] == SIG:
                self.base = off
                break
        if self.base is None:
            raise H5Error("no HDF5 signature")
        s = self.base
        ver = buf[s + 8]
        if ver not in (0, 1):
            raise H5Error(f"superblock version {ver} is outside this subset")
        self.so, self.sl = buf[s + 13], buf[s + 14]
        if self.so != 8 or self.sl != 8:
            raise H5Error("offsets and lengths of 8 bytes only")
        p = s + 24 + (4 if ver == 1 else 0)
        base_addr, _fs, self.eof, _drv = struct.unpack_from("<4Q", buf, p)
        self.root_entry = p + 32
        self.base = base_addr  # absolute; every other address is relative to it

    def u(self, fmt, addr):
        return struct.unpack_from("<" + fmt, self.b, self.base + addr)

    def raw(self, addr, n):
        a = self.base + addr
        if a + n > len(self.b):
            raise H5Error("address past the end of the file")
        return self.b[a:a + n]

    # symbol table entry at an absolute file position
    def entry_abs(self, pos):
        name_off, ohdr, cache = struct.unpack_from("<QQI", self.b, pos)
        return name_off, ohdr, cache

    def messages(self, ohdr):
        """(type, flags, payload) of every message of a version 1 object header."""
        ver = self.b[self.base + ohdr]
        if ver != 1:
            raise H5Error(f"object header version {ver} is outside this subset")
        nmsg, _ref, size = self.u("HII", ohdr + 2)
        chunks = [(ohdr + 16, size)]
        out = []
        while chunks and len(out) < nmsg:
            start, length = chunks.pop(0)
            p, end = start, start + length
            while p + 8 <= end and len(out) < nmsg:
                mtype, msize, flags = self.u("HHB", p)
                payload = self.raw(p + 8, msize)
                if mtype == 0x10:  # continuation: offset, length
                    coff, clen = struct.unpack_from("<QQ", payload, 0)
                    chunks.append((coff, clen))
                out.append((mtype, flags, payload))
                p += 8 + msize
        return out

    def heap_name(self, heap, off):
        sig = self.raw(heap, 4)
        if sig != b"HEAP":
            raise H5Error("bad local heap")
        (seg,) = self.u("Q", heap + 24)
        s = bytearray()
        a = seg + off
        while True:
            c = self.raw(a, 1)[0]
            if c == 0:
                break
            s.append(c)
            a += 1
        return s.decode("ascii")

    def group_entries(self, btree, heap):
        out = []
        sig = self.raw(btree, 4)
        if sig != b"TREE":
            raise H5Error("bad B-tree node")
        ntype, level, used = self.u("BBH", btree + 4)
        if ntype != 0:
            raise H5Error("not a group B-tree")
        p = btree + 24
        for i in range(used):
            (child,) = self.u("Q", p + 8 + 16 * i)
            if level > 0:
                out += self.group_entries(child, heap)
            else:
                if self.raw(child, 4) != b"SNOD":
                    raise H5Error("bad symbol table node")
                (nsym,) = self.u("H", child + 6)
                for k in range(nsym):
                    name_off, ohdr, _cache = self.entry_abs(self.base + child + 8 + 40 * k)
                    out.append((self.heap_name(heap, name_off), ohdr))
        return out

    def object(self, ohdr):
        msgs = self.messages(ohdr)
        types = {t for t, _, _ in msgs}
        attrs = {}
        for t, _, pl in msgs:
            if t == 0x0C:
                name, val = self.attribute(pl)
                attrs[name] = val
        if 0x11 in types:
            pl = next(pl for t, _, pl in msgs if t == 0x11)
            btree, heap = struct.unpack_from("<QQ", pl, 0)
            g = Group(attrs=attrs)
            for name, child in self.group_entries(btree, heap):
                g.members[name] = self.object(child)
            return g
        if 0x01 in types and 0x03 in types and 0x08 in types:
            shape = parse_dataspace(next(pl for t, _, pl in msgs if t == 0x01))
            dt = parse_datatype(next(pl for t, _, pl in msgs if t == 0x03))
            lay = next(pl for t, _, pl in msgs if t == 0x08)
            n = int(np.prod(shape)) if shape else 1
            nbytes = n * dt.itemsize
            raw = self.layout_bytes(lay, nbytes)
            data = np.frombuffer(raw, dtype=dt, count=n).reshape(shape)
            return Dataset(shape=tuple(shape), dtype=dt, data=data, attrs=attrs)
        raise H5Error("object is neither a symbol-table group nor a dataset")

    def layout_bytes(self, lay, nbytes):
        ver = lay[0]
        if ver == 3:
            cls = lay[1]
            if cls == 1:
                addr, size = struct.unpack_from("<QQ", lay, 2)
                if addr == UNDEF:
                    return bytes(nbytes)  # never written: the fill value (zero)
                return self.raw(addr, nbytes)
            if cls == 0:
                (size,) = struct.unpack_from("<H", lay, 2)
                return bytes(lay[4:4 + nbytes])
            raise H5Error("chunked layouts are outside this subset")
        if ver in (1, 2):
            rank, cls = lay[1], lay[2]
            if cls == 1:
                (addr,) = struct.unpack_from("<Q", lay, 8)
                return self.raw(addr, nbytes)
            if cls == 0:
                off = 8 + 4 * rank
                (size,) = struct.unpack_from("<I", lay, off)
                return bytes(lay[off + 4:off + 4 + nbytes])
            raise H5Error("chunked layouts are outside this subset")
        raise H5Error(f"layout version {ver} is outside this subset")

    def attribute(self, pl):
        ver = pl[0]
        nlen, tlen, slen = struct.unpack_from("<HHH", pl, 2)
        pad = (lambda n: (n + 7) & ~7) if ver == 1 else (lambda n: n)
        p = 8 if ver < 3 else 9
        name = pl[p:p + nlen].split(b"\0", 1)[0].decode("ascii")
        p += pad(nlen)
        tbytes = pl[p:p + tlen]
        p += pad(tlen)
        sbytes = pl[p:p + slen]
        p += pad(slen)
        shape = parse_dataspace(sbytes)
        if (tbytes[0] & 0x0F) == 3:  # fixed string
            (size,) = struct.unpack_from("<I", tbytes, 4)
            n = int(np.prod(shape)) if shape else 1
            vals = [pl[p + i * size:p + (i + 1) * size].split(b"\0", 1)[0].decode("ascii") for i in range(n)]
            return name, vals[0] if not shape else vals
        dt = parse_datatype(tbytes)
        n = int(np.prod(shape)) if shape else 1
        arr = np.frombuffer(pl[p:p + n * dt.itemsize], dtype=dt, count=n).reshape(shape)
        return name, arr


def parse_dataspace(pl):
    ver = pl[0]
    rank = pl[1]
    flags = pl[2]
    if ver == 1:
        p = 8
    elif ver == 2:
        if pl[3] == 2:  # null dataspace
            return ()
        p = 4
    else:
        raise H5Error(f"dataspace version {ver} is outside this subset")
    return tuple(struct.unpack_from("<%dQ" % rank, pl, p)) if rank else ()


def parse_datatype(pl):
    cls = pl[0] & 0x0F
    bits = pl[1] | (pl[2] << 8) | (pl[3] << 16)
    (size,) = struct.unpack_from("<I", pl, 4)
    order = ">" if bits & 1 else "<"
    if cls == 0:
        signed = bool(bits & 8)
        return np.dtype(f"{order}{'i' if signed else 'u'}{size}")
    if cls == 1:
        if size not in (4, 8):
            raise H5Error("floating point of 4 or 8 bytes only")
        return np.dtype(f"{order}f{size}")
    raise H5Error(f"datatype class {cls} is outside this subset")


def read(path_or_bytes) -> Group:
    """The root group of an HDF5 file of this subset, datasets loaded."""
    buf = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
    r = _Reader(bytes(buf))
    _name, ohdr, _cache = r.entry_abs(r.root_entry)
    root = r.object(ohdr)
    if not isinstance(root, Group):
        raise H5Error("the root object is not a group")
    return root


# --------------------------------------------------------------------------
# writing (a second writer, shaped like a file the HDF5 library grew by
# insertions: half-full symbol table and B-tree nodes, a user block, object
# headers split by a continuation, version 2 and compact layouts)
# --------------------------------------------------------------------------
def _p8(b: bytearray):
    while len(b) % 8:
        b.append(0)


def _dataspace(dims):
    return bytes([1, len(dims), 0, 0, 0, 0, 0, 0]) + b"".join(struct.pack("<Q", d) for d in dims)


_F8 = bytes([0x11, 0x20, 0x3F, 0x00]) + struct.pack("<IHHBBBBI", 8, 0, 64, 52, 11, 0, 52, 1023)
_I4 = bytes([0x10, 0x08, 0x00, 0x00]) + struct.pack("<IHH", 4, 0, 32)


def _attr(name, value):
    if isinstance(value, str):
        raw = value.encode() + b"\0"
        t, s, data = bytes([0x13, 0, 0, 0]) + struct.pack("<I", len(raw)), _dataspace(()), raw
    elif isinstance(value, int):
        t, s, data = _I4, _dataspace((1,)), struct.pack("<i", value)
    else:
        t, s, data = _F8, _dataspace((1,)), struct.pack("<d", value)
    nm = name.encode() + b"\0"
    b = bytearray(struct.pack("<BBHHH", 1, 0, len(nm), len(t), len(s)))
    for part in (nm, t, s):
        b += part
        _p8(b)
    b += data
    return (0x0C, 0, bytes(b))


class _Writer:
    def __init__(self, userblock=512, leaf_fill=4, node_fill=16, split_headers=True):
        self.ub = userblock
        self.buf = bytearray(b"\0" * (userblock + 96))  # user block, superblock
        self.leaf_fill, self.node_fill, self.split = leaf_fill, node_fill, split_headers

    def alloc(self, data: bytes) -> int:
        a = len(self.buf) - self.ub
        self.buf += data
        return a

    def header(self, msgs):
        def chunk(ms):
            b = bytearray()
            for t, fl, d in ms:
                d = bytes(d) + b"\0" * (-len(d) % 8)
                b += struct.pack("<HHB3x", t, len(d), fl) + d
            return bytes(b)
        msgs = list(msgs)
        if self.split and len(msgs) >= 2:
            tail = chunk(msgs[len(msgs) // 2:])
            caddr = self.alloc(tail)
            msgs = msgs[:len(msgs) // 2] + [(0x10, 0, struct.pack("<QQ", caddr, len(tail)))]
            nmsg = len(msgs) + _count(tail)
        else:
            nmsg = len(msgs)
        c0 = chunk(msgs)
        return self.alloc(struct.pack("<BBHII4x", 1, 0, nmsg, 1, len(c0)) + c0)

    def node(self, obj) -> tuple:
        if isinstance(obj, Dataset):
            a = np.ascontiguousarray(obj.data, dtype="<f8")
            raw = a.tobytes()
            if len(raw) <= 64:  # compact, layout version 3
                lay = bytes([3, 0]) + struct.pack("<H", len(raw)) + raw
            else:  # contiguous, layout version 2 (as older libraries wrote)
                addr = self.alloc(raw)
                dims = list(a.shape) + [8]
                lay = struct.pack("<BBB5xQ", 2, len(dims), 1, addr) + b"".join(struct.pack("<I", d) for d in dims)
            msgs = [(0x05, 1, bytes([1, 2, 2, 1, 0, 0, 0, 0])), (0x03, 1, _F8), (0x01, 0, _dataspace(a.shape)),
                    (0x08, 0, lay)] + [_attr(k, v) for k, v in obj.attrs.items()]
            return self.header(msgs), None
        names = sorted(obj.members, key=lambda s: s.encode())
        kids = [self.node(obj.members[n]) for n in names]
        seg = bytearray(b"\0" * 8)
        offs = []
        for n in names:
            offs.append(len(seg))
            seg += n.encode() + b"\0"
            _p8(seg)
        free = len(seg)
        seg += struct.pack("<QQ", 1, 16)
        heap = len(self.buf) - self.ub
        self.alloc(b"HEAP" + bytes(4) + struct.pack("<QQQ", len(seg), free, heap + 32) + bytes(seg))
        child, last = [], []
        for lo in range(0, len(names), self.leaf_fill):
            hi = min(len(names), lo + self.leaf_fill)
            sn = bytearray(b"SNOD" + struct.pack("<BBH", 1, 0, hi - lo))
            for i in range(lo, hi):
                oh, grp = kids[i]
                sn += struct.pack("<QQII", offs[i], oh, 1 if grp else 0, 0)
                sn += struct.pack("<QQ", *grp) if grp else bytes(16)
            sn += bytes(8 + 40 * 8 - len(sn))
            child.append(self.alloc(bytes(sn)))
            last.append(offs[hi - 1])
        level = 0
        size = 24 + 33 * 8 + 32 * 8
        while True:
            nn = max(1, -(-len(child) // self.node_fill))
            first = len(self.buf) - self.ub
            up, up_last = [], []
            for c in range(nn):
                lo, hi = c * self.node_fill, min(len(child), (c + 1) * self.node_fill)
                t = bytearray(b"TREE" + struct.pack("<BBH", 0, level, hi - lo))
                t += struct.pack("<QQ", first + (c - 1) * size if c else UNDEF,
                                 first + (c + 1) * size if c + 1 < nn else UNDEF)
                t += struct.pack("<Q", last[lo - 1] if lo else 0)
                for i in range(lo, hi):
                    t += struct.pack("<QQ", child[i], last[i])
                t += bytes(size - len(t))
                up.append(self.alloc(bytes(t)))
                up_last.append(last[hi - 1] if hi > lo else 0)
            child, last, level = up, up_last, level + 1
            if len(child) == 1:
                break
        stab = (0x11, 1, struct.pack("<QQ", child[0], heap))
        return self.header([stab] + [_attr(k, v) for k, v in obj.attrs.items()]), (child[0], heap)

    def finish(self, root: Group) -> bytes:
        oh, (bt, heap) = self.node(root)
        eof = len(self.buf)
        sb = SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0)
        sb += struct.pack("<QQQQ", self.ub, UNDEF, eof, UNDEF)
        sb += struct.pack("<QQII", 0, oh, 1, 0) + struct.pack("<QQ", bt, heap)
        self.buf[self.ub:self.ub + 96] = sb
        return bytes(self.buf)


def _count(chunk: bytes) -> int:
    n, p = 0, 0
    while p + 8 <= len(chunk):
        (size,) = struct.unpack_from("<H", chunk, p + 2)
        p += 8 + size
        n += 1
    return n


def write(root: Group, **kw) -> bytes:
    """The bytes of an HDF5 file holding root (datasets in file order, C shape)."""
    return _Writer(**kw).finish(root)
