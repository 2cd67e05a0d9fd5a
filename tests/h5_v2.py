"""Test helper: writes small HDF5 files in the newer ("1.8") file format —
superblock version 2, version-2 object headers ("OHDR", optional "OCHK"
continuation blocks, creation-order and time fields), groups of link
messages or dense groups (links in a fractal heap indexed by a version-2
B-tree of name hashes), attribute messages version 3 (also in dense
storage), dataspace version 2, compound
version 3 and array version 3 datatypes, contiguous layout version 3 — so
that the library's reader is tested on a format its writer does not make.
Written from the HDF5 File Format Specification (version 3.0); the metadata
checksum is Bob Jenkins' lookup3 `hashlittle`, pinned in the tests by the
test vectors published with it.
"""
import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
M32 = 0xFFFFFFFF


def lookup3(data, initval=0):
    def rot(x, k):
        return ((x << k) | (x >> (32 - k))) & M32

    n = len(data)
    a = b = c = (0xDEADBEEF + n + initval) & M32
    i = 0
    while n > 12:
        a = (a + int.from_bytes(data[i:i + 4], "little")) & M32
        b = (b + int.from_bytes(data[i + 4:i + 8], "little")) & M32
        c = (c + int.from_bytes(data[i + 8:i + 12], "little")) & M32
        a = (a - c) & M32; a ^= rot(c, 4); c = (c + b) & M32
        b = (b - a) & M32; b ^= rot(a, 6); a = (a + c) & M32
        c = (c - b) & M32; c ^= rot(b, 8); b = (b + a) & M32
        a = (a - c) & M32; a ^= rot(c, 16); c = (c + b) & M32
        b = (b - a) & M32; b ^= rot(a, 19); a = (a + c) & M32
        c = (c - b) & M32; c ^= rot(b, 4); b = (b + a) & M32
        n -= 12
        i += 12
    if n == 0:
        return c
    tail = data[i:i + n] + bytes(12 - n)
    a = (a + int.from_bytes(tail[0:4], "little")) & M32
    b = (b + int.from_bytes(tail[4:8], "little")) & M32
    c = (c + int.from_bytes(tail[8:12], "little")) & M32
    c ^= b; c = (c - rot(b, 14)) & M32
    a ^= c; a = (a - rot(c, 11)) & M32
    b ^= a; b = (b - rot(a, 25)) & M32
    c ^= b; c = (c - rot(b, 16)) & M32
    a ^= c; a = (a - rot(c, 4)) & M32
    b ^= a; b = (b - rot(a, 14)) & M32
    c ^= b; c = (c - rot(b, 24)) & M32
    return c


# ---------------------------------------------------------------- encodings

F64 = bytes([0x11, 0x20, 63, 0]) + struct.pack("<I", 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)


def array_type(base, n):
    return bytes([0x3A, 0, 0, 0]) + struct.pack("<I", 8 * n) + bytes([1]) + struct.pack("<I", n) + base


def string_type(size):
    return bytes([0x13, 0, 0, 0]) + struct.pack("<I", size)


def int_type(size, signed=True):
    return bytes([0x10, 0x08 if signed else 0, 0, 0]) + struct.pack("<I", size) + struct.pack("<HH", 0, 8 * size)


def compound_type(size, members):
    """members: (name, offset, encoded type); version 3 (names not padded)."""
    nb = 1 if size < 256 else 2 if size < 65536 else 3 if size < 1 << 24 else 4
    out = bytes([0x36, len(members) & 0xFF, len(members) >> 8, 0]) + struct.pack("<I", size)
    for name, off, t in members:
        out += name.encode() + b"\0" + off.to_bytes(nb, "little") + t
    return out


def space(dims):
    return bytes([2, len(dims), 0, 1 if dims else 0]) + b"".join(struct.pack("<Q", d) for d in dims)


def attribute(name, dtype, dims, data):
    nm = name.encode() + b"\0"
    ds = space(dims)
    return (bytes([3, 0]) + struct.pack("<HHH", len(nm), len(dtype), len(ds)) + b"\0" + nm + dtype + ds + data)


def link(name, addr):
    nm = name.encode()
    return bytes([1, 0, len(nm)]) + nm + struct.pack("<Q", addr)


LINK_INFO = bytes([0, 0]) + struct.pack("<QQ", UNDEF, UNDEF)
GROUP_INFO = bytes([0, 0])


class Writer:
    """Objects are laid out after the superblock in the order they are
    added; `split` moves every message after the first into an OCHK
    continuation block; `crt_order` / `times` set those header flags."""

    def __init__(self, crt_order=False, times=False, split=False):
        self.crt_order, self.times, self.split = crt_order, times, split
        self.root_msgs = []
        self.sets = []  # (name, msgs without layout, data bytes)

    def attribute(self, name, dtype, dims, data):
        self.root_msgs.append((0x0C, attribute(name, dtype, dims, data)))

    def dataset(self, name, dtype, dims, data):
        self.sets.append((name, [(0x01, space(dims)), (0x03, dtype)], bytes(data)))

    def _msg(self, t, body, k):
        h = bytes([t]) + struct.pack("<H", len(body)) + bytes([0])
        if self.crt_order:
            h += struct.pack("<H", k)
        return h + body

    def _header(self, msgs, at):
        """(OHDR bytes, OCHK bytes or b"") for an object header at `at`; the
        continuation block, if any, follows the header directly."""
        flags = 0x02 | (0x04 if self.crt_order else 0) | (0x20 if self.times else 0)
        first, rest = (msgs[:1], msgs[1:]) if self.split else (msgs, [])
        body = b"".join(self._msg(t, b, k) for k, (t, b) in enumerate(first))
        pre = b"OHDR" + bytes([2, flags]) + (struct.pack("<IIII", 1, 2, 3, 4) if self.times else b"")
        cont = b""
        if rest:
            cbody = b"".join(self._msg(t, b, k + 1) for k, (t, b) in enumerate(rest))
            cont = b"OCHK" + cbody
            cont += struct.pack("<I", lookup3(cont))
        if cont:
            size_now = len(pre) + 4 + len(body) + len(self._msg(0x10, bytes(16), 0)) + 4
            body += self._msg(0x10, struct.pack("<QQ", at + size_now, len(cont)), len(first))
        blk = pre + struct.pack("<I", len(body)) + body
        blk += struct.pack("<I", lookup3(blk))
        return blk, cont

    def _dense(self, at, objects, rtype):
        """Fractal heap (one 512-byte root direct block holding the message
        bodies of `objects`, (name, body) pairs) and a version-2 B-tree (one
        leaf of records of type `rtype`: 5 links, 8 attributes) at `at`:
        returns (bytes, heap address, B-tree address)."""
        start_block, off_size = 512, 4
        len_size = 2 if rtype == 5 else 3  # heap IDs of 7 (links) or 8 (attributes) bytes
        heap_at = at
        hdr_len = 4 + 1 + 2 + 2 + 1 + 4 + 12 * 8 + 3 * 8 + 8 + 4
        dblock_at = heap_at + hdr_len
        objs, recs = b"", []
        head = 4 + 1 + 8 + off_size  # FHDB, version, heap address, block offset
        for k, (name, body) in enumerate(objects):
            hid = bytes([0]) + (head + len(objs)).to_bytes(off_size, "little") + len(body).to_bytes(len_size, "little")
            h = lookup3(name.encode())
            recs.append((h, struct.pack("<I", h) + hid if rtype == 5 else hid + bytes([0]) + struct.pack("<II", k, h)))
            objs += body
        assert head + len(objs) <= start_block
        dblock = b"FHDB" + bytes([0]) + struct.pack("<Q", heap_at) + bytes(off_size) + objs
        dblock += bytes(start_block - len(dblock))
        hdr = b"FRHP" + bytes([0]) + struct.pack("<HHBI", 1 + off_size + len_size, 0, 0, 4096)
        hdr += struct.pack("<QQQQ", 0, UNDEF, start_block - head - len(objs), UNDEF)
        hdr += struct.pack("<QQQQQQQQ", start_block, start_block, start_block, len(objects), 0, 0, 0, 0)
        hdr += struct.pack("<HQQHHQH", 4, start_block, 65536, 8 * off_size, 0, dblock_at, 0)
        hdr += struct.pack("<I", lookup3(hdr))
        assert len(hdr) == hdr_len
        bt_at = dblock_at + len(dblock)
        rec = len(recs[0][1])
        leaf_at = bt_at + 4 + 1 + 1 + 4 + 2 + 2 + 1 + 1 + 8 + 2 + 8 + 4
        bth = b"BTHD" + bytes([0, rtype]) + struct.pack("<IHHBBQHQ", 512, rec, 0, 100, 40, leaf_at, len(recs),
                                                        len(recs))
        bth += struct.pack("<I", lookup3(bth))
        leaf = b"BTLF" + bytes([0, rtype]) + b"".join(r for _h, r in sorted(recs))
        leaf += struct.pack("<I", lookup3(leaf))
        leaf += bytes(512 - len(leaf))
        return hdr + dblock + bth + leaf, heap_at, bt_at

    def write(self, path, root_links_dense=False, dense=False, dense_attrs=False):
        so = 8
        sb_size = 12 + 4 * so + 4
        at = sb_size
        blobs = []
        set_addr = []
        # data first (after the superblock), then dataset headers, then root
        data_at = []
        for _name, _msgs, data in self.sets:
            data_at.append(at)
            blobs.append(data)
            at += len(data)
        for k, (name, msgs, data) in enumerate(self.sets):
            lay = bytes([3, 1]) + struct.pack("<QQ", data_at[k] if data else UNDEF, len(data))
            oh, cont = self._header(msgs + [(0x08, lay)], at)
            set_addr.append(at)
            blobs += [oh, cont]
            at += len(oh) + len(cont)
        links = [(name, set_addr[k]) for k, (name, _m, _d) in enumerate(self.sets)]
        attrs = self.root_msgs
        if dense_attrs:
            # version-3 attribute: 9 bytes of header, then the name and its NUL
            named = [(body[9:9 + struct.unpack("<H", body[2:4])[0] - 1].decode(), body) for _t, body in attrs]
            blob, heap_at, bt_at = self._dense(at, named, 8)
            blobs.append(blob)
            at += len(blob)
            attrs = [(0x15, bytes([0, 0]) + struct.pack("<QQ", heap_at, bt_at))]
        if dense:
            blob, heap_at, bt_at = self._dense(at, [(n, link(n, a)) for n, a in links], 5)
            blobs.append(blob)
            at += len(blob)
            root_msgs = [(0x02, bytes([0, 0]) + struct.pack("<QQ", heap_at, bt_at)), (0x0A, GROUP_INFO)] + attrs
        else:
            linfo = LINK_INFO if not root_links_dense else bytes([0, 0]) + struct.pack("<QQ", 1234, 5678)
            root_msgs = [(0x02, linfo), (0x0A, GROUP_INFO)] + [(0x06, link(n, a)) for n, a in links] + attrs
        oh, cont = self._header(root_msgs, at)
        root = at
        blobs += [oh, cont]
        at += len(oh) + len(cont)
        sb = b"\x89HDF\r\n\x1a\n" + bytes([2, so, 8, 0]) + struct.pack("<QQQQ", 0, UNDEF, at, root)
        sb += struct.pack("<I", lookup3(sb))
        with open(path, "wb") as f:
            f.write(sb + b"".join(blobs))
        return path


def tile_file(path, fluid, rect, names, **kw):
    """A restart tile file of `fluid` over `rect` in the newer format."""
    w = Writer(**kw)
    for n in names:
        a = fluid[n][rect.lo[2]:rect.hi[2] + 1, rect.lo[1]:rect.hi[1] + 1, rect.lo[0]:rect.hi[0] + 1]
        dims = list(a.shape[:3])
        t = F64 if a.ndim == 3 else array_type(F64, a.shape[3])
        w.dataset(n, t, dims, np.ascontiguousarray(a, dtype="<f8").tobytes())
    w.attribute("note", string_type(8), [], b"latest\0\0")
    return w
