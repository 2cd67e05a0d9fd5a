"""Test infrastructure: an independent HDF5 reader (pure Python + numpy) for
the subset of the format that HTR's restart files use.

Only the test suite imports this module.  It is the checker of the restart
writer and reader in the CUDA library (include/htr_restart.h): it restates
the HDF5 File Format Specification (version 3.0) for superblock versions
0/1, version-1 object headers (with continuation blocks), symbol-table
groups (version-1 B-tree of group nodes, symbol table nodes, local heap),
dataspace versions 1/2, datatypes (fixed-point, floating point, string,
compound, array), data layout versions 1-3 (contiguous and compact) and
attribute messages version 1.  Its own correctness is pinned against a file
that libhdf5 wrote (tests/test_restart.py).

The reference writes restarts through libhdf5 (src/Utils/hdf_helper.rg:199-331
tile files, :845-931 master file) and reads them with h5py in its scripts
(scripts/modules/HTRrestart.py:187-760); neither libhdf5 nor h5py is needed
here.
"""
import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(ValueError):
    pass


def _u(b, off, n):
    return int.from_bytes(b[off:off + n], "little")


class File:
    """Parses a whole file held in memory; `datasets` maps a name to
    (numpy array, {attribute: value}), `attrs` holds the root attributes,
    `messages` the raw (type, flags, body) messages of each object."""

    def __init__(self, path):
        with open(path, "rb") as fh:
            self.b = fh.read()
        self.datasets = {}
        self.attrs = {}
        self.messages = {}
        self._superblock()

    # --- structure ---------------------------------------------------------

    def _superblock(self):
        at = 0
        while self.b[at:at + 8] != SIGNATURE:
            at = 512 if at == 0 else 2 * at
            if at + 8 > len(self.b):
                raise H5Error("no HDF5 signature")
        self.sb_at = at
        version = self.b[at + 8]
        if version > 1:
            raise H5Error(f"superblock version {version}")
        self.so, self.sl = self.b[at + 13], self.b[at + 14]
        self.leaf_k, self.internal_k = _u(self.b, at + 16, 2), _u(self.b, at + 18, 2)
        p = at + 24 + (4 if version == 1 else 0)
        self.base = _u(self.b, p, self.so)
        self.eof = _u(self.b, p + 2 * self.so, self.so)
        entry = p + 4 * self.so
        root = _u(self.b, entry + self.so, self.so)
        if self.eof > len(self.b):
            raise H5Error("truncated")
        self._group(root, "")

    def _abs(self, rel):
        return self.base + rel

    def _header(self, rel):
        a = self._abs(rel)
        if self.b[a] != 1:
            raise H5Error(f"object header version {self.b[a]}")
        size = _u(self.b, a + 8, 4)
        msgs = []
        blocks = [(a + 16, size)]
        while blocks:
            start, n = blocks.pop(0)
            p = start
            while p + 8 <= start + n:
                mtype, msize, flags = _u(self.b, p, 2), _u(self.b, p + 2, 2), self.b[p + 4]
                body = self.b[p + 8:p + 8 + msize]
                if len(body) != msize:
                    raise H5Error("message beyond the file")
                if mtype == 0x10:
                    blocks.append((self._abs(_u(body, 0, self.so)), _u(body, self.so, self.sl)))
                msgs.append((mtype, flags, body))
                p += 8 + msize
        return msgs

    def _heap(self, rel):
        a = self._abs(rel)
        if self.b[a:a + 4] != b"HEAP":
            raise H5Error("local heap signature")
        size = _u(self.b, a + 8, self.sl)
        self.heap_free_head = _u(self.b, a + 8 + self.sl, self.sl)
        data = self._abs(_u(self.b, a + 8 + 2 * self.sl, self.so))
        return self.b[data:data + size]

    def _links(self, btree, heap):
        a = self._abs(btree)
        if self.b[a:a + 4] != b"TREE" or self.b[a + 4] != 0:
            raise H5Error("group B-tree node")
        level, used = self.b[a + 5], _u(self.b, a + 6, 2)
        p = a + 8 + 2 * self.so + self.sl
        out = []
        for _ in range(used):
            child = _u(self.b, p, self.so)
            p += self.so + self.sl
            if level:
                out += self._links(child, heap)
                continue
            s = self._abs(child)
            if self.b[s:s + 4] != b"SNOD":
                raise H5Error("symbol table node")
            for k in range(_u(self.b, s + 6, 2)):
                e = s + 8 + k * (2 * self.so + 24)
                off, oh = _u(self.b, e, self.so), _u(self.b, e + self.so, self.so)
                name = heap[off:heap.index(b"\0", off)].decode()
                out.append((name, oh))
        return out

    def _group(self, rel, prefix):
        msgs = self._header(rel)
        self.messages[prefix or "/"] = msgs
        for mtype, _flags, body in msgs:
            if mtype == 0x11:
                bt, hp = _u(body, 0, self.so), _u(body, self.so, self.so)
                self.root_btree, self.root_heap = bt, hp
                for name, oh in self._links(bt, self._heap(hp)):
                    path = f"{prefix}/{name}" if prefix else name
                    sub = self._header(oh)
                    if any(m[0] == 0x11 for m in sub):
                        self._group(oh, path)
                    else:
                        self._dataset(oh, path, sub)
            elif mtype == 0x0C and not prefix:
                name, value = self._attribute(body)
                self.attrs[name] = value

    # --- messages ----------------------------------------------------------

    def _dtype(self, b, p=0):
        """numpy dtype of the datatype at b[p:], and the offset after it."""
        version, cls = b[p] >> 4, b[p] & 15
        bf0, bf1 = b[p + 1], b[p + 2]
        size = _u(b, p + 4, 4)
        q = p + 8
        if cls == 0:
            order = ">" if bf0 & 1 else "<"
            return np.dtype(f"{order}{'i' if bf0 & 8 else 'u'}{size}"), q + 4
        if cls == 1:
            order = ">" if bf0 & 1 else "<"
            return np.dtype(f"{order}f{size}"), q + 12
        if cls == 3:
            return np.dtype(f"S{size}"), q
        if cls == 6:
            names, formats, offsets = [], [], []
            for _ in range(bf0 | bf1 << 8):
                start = q
                end = b.index(b"\0", q)
                names.append(b[start:end].decode())
                if version < 3:
                    # name and its NUL padded to 8 bytes; then the byte
                    # offset, and in version 1 the unused array fields
                    q = start + (end - start + 1 + 7) // 8 * 8
                    offsets.append(_u(b, q, 4))
                    q += 4 + (28 if version == 1 else 0)
                else:
                    q = end + 1
                    nb = 1 if size < 256 else 2 if size < 65536 else 3 if size < 1 << 24 else 4
                    offsets.append(_u(b, q, nb))
                    q += nb
                dt, q = self._dtype(b, q)
                formats.append(dt)
            return np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": size}), q
        if cls == 10:
            rank = b[q]
            q += 4 if version == 2 else 1
            dims = [_u(b, q + 4 * k, 4) for k in range(rank)]
            q += 4 * rank * (2 if version == 2 else 1)
            base, q = self._dtype(b, q)
            return np.dtype((base, tuple(dims))), q
        raise H5Error(f"datatype class {cls}")

    def _space(self, b):
        version, rank, flags = b[0], b[1], b[2]
        p = 8 if version == 1 else 4
        if version == 2 and b[3] == 2:
            return None
        return tuple(_u(b, p + self.sl * k, self.sl) for k in range(rank))

    def _attribute(self, b):
        if b[0] != 1:
            raise H5Error(f"attribute message version {b[0]}")
        nlen, tlen, slen = _u(b, 2, 2), _u(b, 4, 2), _u(b, 6, 2)
        pad = lambda n: (n + 7) // 8 * 8
        p = 8
        name = b[p:p + nlen - 1].decode()
        p += pad(nlen)
        dt, _ = self._dtype(b, p)
        p += pad(tlen)
        shape = self._space(b[p:p + slen])
        p += pad(slen)
        n = int(np.prod(shape)) if shape else 1
        arr = np.frombuffer(b, dtype=dt, count=n, offset=p).reshape(tuple(shape or ()) + dt.shape)
        return name, arr

    def _dataset(self, rel, name, msgs):
        self.messages[name] = msgs
        dt = shape = None
        layout = None
        attrs = {}
        for mtype, _flags, body in msgs:
            if mtype == 0x01:
                shape = self._space(body)
            elif mtype == 0x03:
                dt, _ = self._dtype(body)
            elif mtype == 0x08:
                layout = body
            elif mtype == 0x0B:
                raise H5Error("filtered dataset")
            elif mtype == 0x0C:
                k, v = self._attribute(body)
                attrs[k] = v
        n = int(np.prod(shape)) if shape else 1
        version = layout[0]
        if version in (1, 2):
            rank, cls = layout[1], layout[2]
            addr = _u(layout, 8, self.so) if cls else None
        elif version == 3:
            cls = layout[1]
            addr = _u(layout, 2, self.so) if cls == 1 else None
        else:
            raise H5Error(f"layout version {version}")
        if cls == 1:
            if addr == UNDEF:
                arr = np.zeros(n, dtype=dt)
            else:
                a = self._abs(addr)
                if a + n * dt.itemsize > len(self.b):
                    raise H5Error("data beyond the file")
                arr = np.frombuffer(self.b, dtype=dt, count=n, offset=a)
        elif cls == 0:
            if version == 3:
                size = _u(layout, 2, 2)
                arr = np.frombuffer(layout[4:4 + size], dtype=dt, count=n)
            else:
                raise H5Error("compact layout before version 3")
        else:
            raise H5Error(f"layout class {cls}")
        # an array datatype adds its dimensions after the dataspace's
        self.datasets[name] = (arr.reshape(tuple(shape or ()) + dt.shape), attrs)
