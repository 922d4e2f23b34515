"""Reader and writer for the subset of HDF5 that rubix's files use (h5py is not a
dependency of this package).

rubix keeps its SSP templates (BC03, FSPS; rubix/spectra/ssp/grid.py:304-335) and its
converted galaxies (rubix/galaxy/input_handler/base.py:17-73, read back by
rubix/utils.py:160-200) in HDF5 files written by h5py: groups, numeric datasets and
string attributes ("unit").  This module implements, from the published HDF5 file
format specification:

reading: superblocks 0-3 (with or without a user block), object headers 1 and 2 (with
continuation blocks), old-style groups (symbol-table B-tree + local heap) and compact
new-style groups (link messages), contiguous, compact and chunked data (version-1
B-tree chunk index, deflate and shuffle filters), fixed-point and floating-point
numbers of either byte order, fixed-length strings and variable-length strings (global
heap), scalar and simple dataspaces, compact attributes;

writing: superblock 0 with old-style groups, contiguous datasets of numbers or
fixed-length strings, and fixed-length string or numeric attributes.

Dense (fractal-heap) groups and attributes, compound and reference types and the
newer chunk indexes are refused with an error naming the feature.
"""

from __future__ import annotations

import mmap
import os
import struct
import zlib
from typing import Dict, Iterator, Optional, Union

import numpy as np

__all__ = ["File", "Group", "Dataset", "Chunked", "write_file", "HDF5Error"]

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF


class HDF5Error(ValueError):
    pass


# ---------------------------------------------------------------------- reading
class _Reader:
    def __init__(self, data: bytes):
        self.b = data
        self.base = None
        self.sb_pos = None
        for pos in [0] + [512 << i for i in range(20)]:
            if pos + 8 > len(data):
                break
            if data[pos:pos + 8] == _SIG:
                self.sb_pos = pos
                break
        if self.sb_pos is None:
            raise HDF5Error("not an HDF5 file (no superblock signature)")
        self._superblock()

    # -- primitives
    def u(self, pos: int, n: int) -> int:
        return int.from_bytes(self.b[pos:pos + n], "little")

    def addr(self, pos: int) -> int:
        return self.u(pos, self.O)

    def length(self, pos: int) -> int:
        return self.u(pos, self.L)

    def abs(self, a: int) -> int:
        return self.base + a

    def _superblock(self):
        p = self.sb_pos
        ver = self.b[p + 8]
        if ver in (0, 1):
            self.O, self.L = self.b[p + 13], self.b[p + 14]
            q = p + 24 + (4 if ver == 1 else 0)
            self.base = self.u(q, self.O)
            q += 4 * self.O  # base, free space, end of file, driver info
            # root group symbol table entry: name offset, object header address, ...
            self.root = self.u(q + self.O, self.O)
            cache = self.u(q + 2 * self.O, 4)
            self.root_scratch = None
            if cache == 1:
                s = q + 2 * self.O + 8
                self.root_scratch = (self.u(s, self.O), self.u(s + self.O, self.O))
        elif ver in (2, 3):
            self.O, self.L = self.b[p + 9], self.b[p + 10]
            q = p + 12
            self.base = self.u(q, self.O)
            self.root = self.u(q + 3 * self.O, self.O)
            self.root_scratch = None
        else:
            raise HDF5Error(f"superblock version {ver} is not supported")
        if self.base == _UNDEF:
            self.base = self.sb_pos

    # -- object headers
    def messages(self, oh: int):
        """(type, data bytes) of every message of the object header at oh."""
        pos = self.abs(oh)
        out = []
        if self.b[pos:pos + 4] == b"OHDR":
            ver = self.b[pos + 4]
            if ver != 2:
                raise HDF5Error(f"object header version {ver} is not supported")
            flags = self.b[pos + 5]
            q = pos + 6
            if flags & 0x20:
                q += 16
            if flags & 0x10:
                q += 4
            nsz = 1 << (flags & 3)
            size = self.u(q, nsz)
            q += nsz
            blocks = [(q, size)]
            track_order = bool(flags & 0x04)
            while blocks:
                start, size = blocks.pop(0)
                q, end = start, start + size
                while q + 4 <= end:
                    mtype, msize, _mflags = self.b[q], self.u(q + 1, 2), self.b[q + 3]
                    q += 4 + (2 if track_order else 0)
                    data = self.b[q:q + msize]
                    q += msize
                    if mtype == 0x10:
                        a = int.from_bytes(data[:self.O], "little")
                        ln = int.from_bytes(data[self.O:self.O + self.L], "little")
                        c = self.abs(a)
                        if self.b[c:c + 4] != b"OCHK":
                            raise HDF5Error("bad object header continuation block")
                        blocks.append((c + 4, ln - 8))
                    elif mtype != 0:
                        out.append((mtype, data))
            return out
        ver = self.b[pos]
        if ver != 1:
            raise HDF5Error(f"object header version {ver} is not supported")
        nmsg = self.u(pos + 2, 2)
        size = self.u(pos + 8, 4)
        blocks = [(pos + 16, size)]
        while blocks and len(out) < nmsg + 64:
            start, size = blocks.pop(0)
            q, end = start, start + size
            while q + 8 <= end:
                mtype, msize = self.u(q, 2), self.u(q + 2, 2)
                data = self.b[q + 8:q + 8 + msize]
                q += 8 + msize
                if mtype == 0x10:
                    a = int.from_bytes(data[:self.O], "little")
                    ln = int.from_bytes(data[self.O:self.O + self.L], "little")
                    blocks.append((self.abs(a), ln))
                elif mtype != 0:
                    out.append((mtype, data))
        return out

    # -- datatype / dataspace
    def datatype(self, d: bytes, off: int = 0):
        """(numpy dtype or a descriptor tuple, size) of a datatype message."""
        cv = d[off]
        cls, ver = cv & 0x0F, cv >> 4
        bits = d[off + 1] | (d[off + 2] << 8) | (d[off + 3] << 16)
        size = int.from_bytes(d[off + 4:off + 8], "little")
        order = ">" if bits & 1 else "<"
        if cls == 0:  # fixed point
            kind = "i" if bits & 0x08 else "u"
            return np.dtype(f"{order}{kind}{size}"), size
        if cls == 1:
            if size not in (2, 4, 8):
                raise HDF5Error(f"floating point of {size} bytes is not supported")
            return np.dtype(f"{order}f{size}"), size
        if cls == 3:
            return ("fstr", size), size
        if cls == 9:
            vtype = bits & 0x0F
            if vtype == 1:
                return ("vstr", None), size
            base, _ = self.datatype(d, off + 8)
            return ("vseq", base), size
        if cls == 4:  # bitfield
            return np.dtype(f"{order}u{size}"), size
        raise HDF5Error(f"datatype class {cls} (version {ver}) is not supported")

    def dataspace(self, d: bytes, off: int = 0):
        ver, nd, flags = d[off], d[off + 1], d[off + 2]
        if ver == 1:
            q = off + 8
            kind = 1 if nd > 0 else 0
        elif ver == 2:
            kind = d[off + 3]
            q = off + 4
        else:
            raise HDF5Error(f"dataspace version {ver} is not supported")
        if kind == 2:
            return None  # null dataspace
        dims = tuple(int.from_bytes(d[q + i * self.L:q + (i + 1) * self.L], "little")
                     for i in range(nd))
        return dims

    # -- data
    def decode(self, raw: bytes, dtype, shape):
        n = int(np.prod(shape)) if shape else 1
        if isinstance(dtype, np.dtype):
            a = np.frombuffer(raw, dtype=dtype, count=n).astype(dtype.newbyteorder("="))
            return a.reshape(shape) if shape else a.reshape(())
        kind, arg = dtype
        if kind == "fstr":
            vals = [raw[i * arg:(i + 1) * arg].split(b"\x00", 1)[0].decode("utf-8", "replace")
                    for i in range(n)]
        elif kind == "vstr":
            step = 4 + self.O + 4
            vals = [self.global_object(raw, i * step).decode("utf-8", "replace")
                    for i in range(n)]
        else:
            raise HDF5Error("variable-length sequences are not supported")
        a = np.array(vals, dtype=object)
        return a.reshape(shape) if shape else a.reshape(())

    def global_object(self, raw: bytes, off: int) -> bytes:
        coll = int.from_bytes(raw[off + 4:off + 4 + self.O], "little")
        idx = int.from_bytes(raw[off + 4 + self.O:off + 8 + self.O], "little")
        c = self.abs(coll)
        if self.b[c:c + 4] != b"GCOL":
            raise HDF5Error("bad global heap collection")
        csize = self.length(c + 8)
        q, end = c + 8 + self.L, c + csize
        while q + 8 + self.L <= end:
            hidx = self.u(q, 2)
            osize = self.length(q + 8)
            if hidx == 0:
                break
            if hidx == idx:
                return self.b[q + 8 + self.L:q + 8 + self.L + osize]
            q += 8 + self.L + ((osize + 7) // 8) * 8
        raise HDF5Error("global heap object not found")

    def read_layout(self, d: bytes, dtype, elem: int, shape, filters):
        ver = d[0]
        n = int(np.prod(shape)) if shape else 1
        if ver == 3:
            cls = d[1]
            if cls == 0:
                size = self.u_of(d, 2, 2)
                raw = d[4:4 + size]
            elif cls == 1:
                a = self.u_of(d, 2, self.O)
                size = self.u_of(d, 2 + self.O, self.L)
                raw = b"" if a == _UNDEF else self.b[self.abs(a):self.abs(a) + size]
                if a == _UNDEF:
                    raw = bytes(n * elem)
            elif cls == 2:
                nd = d[2]
                btree = self.u_of(d, 3, self.O)
                cdims = [self.u_of(d, 3 + self.O + 4 * i, 4) for i in range(nd)]
                raw = self.read_chunked(btree, cdims, shape, elem, filters)
            else:
                raise HDF5Error(f"data layout class {cls} is not supported")
        elif ver in (1, 2):
            nd, cls = d[1], d[2]
            q = 8
            a = None
            if cls != 0:
                a = self.u_of(d, q, self.O)
                q += self.O
            cdims = [self.u_of(d, q + 4 * i, 4) for i in range(nd)]
            q += 4 * nd
            if cls == 0:
                size = self.u_of(d, q, 4)
                raw = d[q + 4:q + 4 + size]
            elif cls == 1:
                raw = self.b[self.abs(a):self.abs(a) + n * elem]
            else:
                raw = self.read_chunked(a, cdims, shape, elem, filters)
        else:
            raise HDF5Error(f"data layout version {ver} is not supported (newer chunk "
                            "indexes)")
        return raw

    @staticmethod
    def u_of(d: bytes, off: int, n: int) -> int:
        return int.from_bytes(d[off:off + n], "little")

    def read_chunked(self, btree: int, cdims, shape, elem: int, filters) -> bytes:
        shape = tuple(shape) if shape else ()
        nd = len(shape)
        out = np.zeros(int(np.prod(shape)) * elem if shape else elem, dtype=np.uint8)
        if btree == _UNDEF:
            return out.tobytes()
        cshape = tuple(cdims[:nd])
        full = out.reshape(shape + (elem,)) if shape else out.reshape(1, elem)
        for offs, size, mask, addr in self._chunks(btree, nd + 1):
            raw = self.b[self.abs(addr):self.abs(addr) + size]
            for i, (fid, cd) in reversed(list(enumerate(filters))):
                if (mask >> i) & 1:  # filter i was skipped for this chunk
                    continue
                if fid == 1:
                    raw = zlib.decompress(raw)
                elif fid == 2:
                    es = cd[0] if cd else elem
                    a = np.frombuffer(raw, dtype=np.uint8)
                    m = a.size // es
                    raw = a[:m * es].reshape(es, m).T.tobytes() + a[m * es:].tobytes()
                elif fid == 3:
                    raw = raw[:-4]  # fletcher32 checksum
                else:
                    raise HDF5Error(f"filter {fid} is not supported")
            chunk = np.frombuffer(raw, dtype=np.uint8)
            chunk = chunk[:int(np.prod(cshape)) * elem].reshape(cshape + (elem,))
            sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cshape, shape))
            csl = tuple(slice(0, x.stop - x.start) for x in sl)
            full[sl] = chunk[csl]
        return out.tobytes()

    def _chunks(self, node: int, nk: int) -> Iterator:
        p = self.abs(node)
        if self.b[p:p + 4] != b"TREE" or self.b[p + 4] != 1:
            raise HDF5Error("bad chunk B-tree node")
        level, used = self.b[p + 5], self.u(p + 6, 2)
        q = p + 8 + 2 * self.O
        ksz = 8 + 8 * nk
        for i in range(used):
            k = q + i * (ksz + self.O)
            size, mask = self.u(k, 4), self.u(k + 4, 4)
            offs = [self.u(k + 8 + 8 * j, 8) for j in range(nk - 1)]
            child = self.addr(k + ksz)
            if level == 0:
                yield offs, size, mask, child
            else:
                yield from self._chunks(child, nk)

    # -- groups
    def links(self, oh: int, scratch=None) -> Dict[str, int]:
        msgs = self.messages(oh)
        out: Dict[str, int] = {}
        for mtype, d in msgs:
            if mtype == 0x11:
                bt, heap = self.u_of(d, 0, self.O), self.u_of(d, self.O, self.O)
                out.update(self._symbol_table(bt, heap))
            elif mtype == 0x06:
                name, target = self._link(d)
                if target is not None:
                    out[name] = target
            elif mtype == 0x02:
                fheap = self.u_of(d, 2 + (8 if d[1] & 1 else 0), self.O)
                if fheap != _UNDEF:
                    raise HDF5Error("groups with dense link storage are not supported")
        if not out and scratch is not None:
            out.update(self._symbol_table(*scratch))
        return out

    def _link(self, d: bytes):
        flags = d[1]
        q = 2
        ltype = 0
        if flags & 0x08:
            ltype = d[q]
            q += 1
        if flags & 0x04:
            q += 8
        if flags & 0x10:
            q += 1
        nsz = 1 << (flags & 3)
        nlen = self.u_of(d, q, nsz)
        q += nsz
        name = d[q:q + nlen].decode("utf-8")
        q += nlen
        if ltype != 0:
            return name, None  # soft / external links are not followed
        return name, self.u_of(d, q, self.O)

    def _symbol_table(self, btree: int, heap: int) -> Dict[str, int]:
        h = self.abs(heap)
        if self.b[h:h + 4] != b"HEAP":
            raise HDF5Error("bad local heap")
        seg = self.abs(self.addr(h + 8 + 2 * self.L))
        out: Dict[str, int] = {}

        def name_at(off):
            s = seg + off
            return self.b[s:self.b.find(b"\x00", s)].decode("utf-8")

        def walk(node):
            p = self.abs(node)
            if self.b[p:p + 4] == b"SNOD":
                n = self.u(p + 6, 2)
                q = p + 8
                esz = 2 * self.O + 24
                for i in range(n):
                    e = q + i * esz
                    out[name_at(self.addr(e))] = self.addr(e + self.O)
                return
            if self.b[p:p + 4] != b"TREE" or self.b[p + 4] != 0:
                raise HDF5Error("bad group B-tree node")
            used = self.u(p + 6, 2)
            q = p + 8 + 2 * self.O
            for i in range(used):
                child = self.addr(q + self.L + i * (self.L + self.O))
                walk(child)

        walk(btree)
        return out

    # -- objects
    def is_dataset(self, oh: int) -> bool:
        return any(t == 0x08 for t, _ in self.messages(oh))

    def attributes(self, oh: int) -> Dict[str, object]:
        out = {}
        for mtype, d in self.messages(oh):
            if mtype == 0x15:
                fheap = self.u_of(d, 2 + (2 if d[1] & 1 else 0), self.O)
                if fheap != _UNDEF:
                    raise HDF5Error("dense attribute storage is not supported")
            if mtype != 0x0C:
                continue
            ver = d[0]
            nlen, tlen, slen = self.u_of(d, 2, 2), self.u_of(d, 4, 2), self.u_of(d, 6, 2)
            q = 8 + (1 if ver == 3 else 0)
            pad = (lambda x: (x + 7) // 8 * 8) if ver == 1 else (lambda x: x)
            name = d[q:q + nlen].split(b"\x00", 1)[0].decode("utf-8")
            q += pad(nlen)
            dtype, elem = self.datatype(d, q)
            q += pad(tlen)
            shape = self.dataspace(d, q)
            q += pad(slen)
            if shape is None:
                out[name] = None
                continue
            n = int(np.prod(shape)) if shape else 1
            esz = elem if isinstance(dtype, np.dtype) or dtype[0] == "fstr" else 4 + self.O + 4
            val = self.decode(d[q:q + n * esz], dtype, shape)
            out[name] = val.item() if val.ndim == 0 else val
        return out

    def read_dataset(self, oh: int):
        msgs = self.messages(oh)
        dtype = shape = layout = None
        elem = 0
        filters = []
        for mtype, d in msgs:
            if mtype == 0x03:
                dtype, elem = self.datatype(d)
            elif mtype == 0x01:
                shape = self.dataspace(d)
            elif mtype == 0x08:
                layout = d
            elif mtype == 0x0B:
                filters = self._filters(d)
        if layout is None or dtype is None:
            raise HDF5Error("object is not a dataset")
        if shape is None:
            return None
        esz = elem if isinstance(dtype, np.dtype) or dtype[0] == "fstr" else 4 + self.O + 4
        raw = self.read_layout(layout, dtype, esz, shape, filters)
        return self.decode(raw, dtype, shape)

    def dataset_info(self, oh: int):
        dtype = shape = None
        for mtype, d in self.messages(oh):
            if mtype == 0x03:
                dtype, _ = self.datatype(d)
            elif mtype == 0x01:
                shape = self.dataspace(d)
        return dtype, shape

    def _filters(self, d: bytes):
        ver, n = d[0], d[1]
        q = 8 if ver == 1 else 2
        out = []
        for _ in range(n):
            fid = self.u_of(d, q, 2)
            q += 2
            nlen = 0
            if ver == 1 or fid >= 256:
                nlen = self.u_of(d, q, 2)
                q += 2
            q += 2  # flags
            nv = self.u_of(d, q, 2)
            q += 2
            if ver == 1:
                q += (nlen + 7) // 8 * 8
            else:
                q += nlen
            cd = [self.u_of(d, q + 4 * i, 4) for i in range(nv)]
            q += 4 * nv
            if ver == 1 and nv % 2:
                q += 4
            out.append((fid, cd))
        return out


class Dataset:
    """h5py-like dataset: ``ds[()]`` / ``ds[:]`` read it, ``attrs``, ``shape``, ``dtype``."""

    def __init__(self, r: _Reader, oh: int, name: str):
        self._r, self._oh, self.name = r, oh, name
        dt, shape = r.dataset_info(oh)
        self.shape = shape
        self.dtype = dt if isinstance(dt, np.dtype) else np.dtype(object)

    @property
    def attrs(self) -> Dict[str, object]:
        return self._r.attributes(self._oh)

    def __getitem__(self, key):
        a = self._r.read_dataset(self._oh)
        if key == () or key is Ellipsis:
            return a
        return a[key]

    def __array__(self, dtype=None, copy=None):
        a = np.asarray(self[()])
        return a.astype(dtype) if dtype is not None else a


class Group:
    """h5py-like group: ``g["a/b"]``, ``keys()``, ``items()``, ``in``, ``attrs``."""

    def __init__(self, r: _Reader, oh: int, name: str, scratch=None):
        self._r, self._oh, self.name = r, oh, name
        self._links = r.links(oh, scratch)

    @property
    def attrs(self) -> Dict[str, object]:
        return self._r.attributes(self._oh)

    def keys(self):
        return list(self._links)

    def __iter__(self):
        return iter(self._links)

    def __contains__(self, key) -> bool:
        try:
            self[key]
            return True
        except KeyError:
            return False

    def items(self):
        return [(k, self[k]) for k in self._links]

    def __getitem__(self, key: str) -> Union["Group", Dataset]:
        parts = [p for p in key.split("/") if p]
        g: Union[Group, Dataset] = self
        for i, p in enumerate(parts):
            if not isinstance(g, Group) or p not in g._links:
                raise KeyError(f"{key!r} not found in {self.name!r}")
            oh = g._links[p]
            path = (g.name.rstrip("/") + "/" + p) if g.name != "/" else "/" + p
            g = Dataset(self._r, oh, path) if self._r.is_dataset(oh) else Group(self._r, oh, path)
        return g


class File(Group):
    """Read-only HDF5 file (``mode="r"`` only)."""

    def __init__(self, path: str, mode: str = "r"):
        if mode != "r":
            raise ValueError("hdf5.File reads only; write files with hdf5.write_file")
        # memory-mapped: a dataset read touches only its own bytes
        with open(path, "rb") as f:
            size = os.fstat(f.fileno()).st_size
            self._map = mmap.mmap(f.fileno(), 0, access=mmap.ACCESS_READ) if size else b""
        r = _Reader(self._map)
        super().__init__(r, r.root, "/", r.root_scratch)
        self.filename = path

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False

    def close(self):
        """Datasets already read stay valid (they are copies)."""
        if isinstance(self._map, mmap.mmap) and not self._map.closed:
            self._map.close()


# ---------------------------------------------------------------------- writing
_GROUP_K = 16  # symbol-table node capacity 2K entries per node; superblock leaf K


def _pad8(b: bytes) -> bytes:
    return b + bytes((-len(b)) % 8)


def _dtype_msg(a: np.ndarray) -> bytes:
    dt = a.dtype
    if dt.kind in ("S", "U", "O"):
        raise AssertionError("strings are encoded by _string_dtype_msg")
    order = 1 if dt.byteorder == ">" else 0
    if dt.kind == "f":
        size = dt.itemsize
        if size == 4:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
        elif size == 8:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
        else:
            raise HDF5Error(f"cannot write float{8 * size}")
        # byte order, padding 0, mantissa normalisation 2 (implied msb), sign bit position
        bits0 = order | (2 << 4)
        sign = 8 * size - 1
        return struct.pack("<BBBBI", 0x11, bits0, sign, 0, size) + props
    if dt.kind in ("i", "u", "b"):
        size = dt.itemsize
        bits0 = order | (0x08 if dt.kind == "i" else 0)
        return struct.pack("<BBBBI", 0x10, bits0, 0, 0, size) + struct.pack("<HH", 0, 8 * size)
    raise HDF5Error(f"cannot write arrays of dtype {dt}")


def _string_dtype_msg(size: int) -> bytes:
    # class 3 (string), version 1, null-terminated padding, ASCII
    return struct.pack("<BBBBI", 0x13, 0, 0, 0, size)


def _dataspace_msg(shape) -> bytes:
    nd = len(shape)
    return struct.pack("<BBBB4x", 1, nd, 0, 0) + b"".join(struct.pack("<Q", s) for s in shape)


def _as_strings(value) -> Optional[np.ndarray]:
    a = np.asarray(value)
    if a.dtype.kind in ("U", "S", "O"):
        enc = np.vectorize(lambda s: s.encode("utf-8") if isinstance(s, str) else bytes(s),
                           otypes=[object])(a) if a.size else a.astype(object)
        n = max([len(x) for x in enc.reshape(-1)] + [0]) + 1
        return np.array([x.ljust(n, b"\x00") for x in enc.reshape(-1)],
                        dtype=f"S{n}").reshape(a.shape)
    return None


class Chunked:
    """A dataset to be written in chunks (version-1 B-tree index, one leaf node of at most
    64 chunks), optionally through the shuffle and deflate filters."""

    def __init__(self, data, chunks, gzip: int = 4, shuffle: bool = False, attrs=None):
        self.data = np.asarray(data)
        self.chunks = tuple(int(c) for c in chunks)
        if len(self.chunks) != self.data.ndim or min(self.chunks + (1,)) < 1:
            raise HDF5Error("chunk shape must have one positive extent per dimension")
        self.gzip, self.shuffle, self.attrs = gzip, shuffle, attrs or {}


_ISTORE_K = 32  # chunk B-tree K (the default: superblock 0 does not record it)


class _Writer:
    def __init__(self, vlen_strings: bool = True):
        self.buf = bytearray()
        self.vlen_strings = vlen_strings

    def alloc(self, data: bytes) -> int:
        while len(self.buf) % 8:
            self.buf.append(0)
        a = len(self.buf)
        self.buf += data
        return a

    def reserve(self, n: int) -> int:
        return self.alloc(bytes(n))

    def put(self, a: int, data: bytes):
        self.buf[a:a + len(data)] = data

    @staticmethod
    def message(mtype: int, data: bytes, flags: int = 0) -> bytes:
        data = _pad8(data)
        return struct.pack("<HHB3x", mtype, len(data), flags) + data

    def object_header(self, msgs) -> int:
        body = b"".join(msgs)
        hdr = struct.pack("<BBHII4x", 1, 0, len(msgs), 1, len(body))
        return self.alloc(hdr + body)

    def global_heap(self, objects) -> int:
        """A global heap collection holding ``objects`` (bytes); returns its address."""
        body = bytearray()
        for i, ob in enumerate(objects, start=1):
            body += struct.pack("<HH4xQ", i, 1, len(ob)) + _pad8(ob)
        size = max(4096, 16 + len(body) + 16)
        free = size - 16 - len(body)
        body += struct.pack("<HH4xQ", 0, 0, free - 16)  # free space object
        coll = b"GCOL" + struct.pack("<B3xQ", 1, size) + bytes(body)
        return self.alloc(coll + bytes(size - len(coll)))

    def attribute_msg(self, name: str, value) -> bytes:
        nb = name.encode("utf-8") + b"\x00"
        s = _as_strings(value)
        if s is not None and self.vlen_strings:
            # variable-length UTF-8 strings in a global heap (what h5py writes for str)
            flat = [bytes(x).rstrip(b"\x00") for x in s.reshape(-1)]
            coll = self.global_heap(flat)
            dt = (struct.pack("<BBBBI", 0x19, 0x01, 0x01, 0, 4 + 8 + 4)
                  + struct.pack("<BBBBI", 0x10, 0, 0, 0, 1) + struct.pack("<HH", 0, 8))
            shape = s.shape
            data = b"".join(struct.pack("<IQI", len(x), coll, i + 1) for i, x in enumerate(flat))
        elif s is not None:
            dt = _string_dtype_msg(s.dtype.itemsize)
            shape = s.shape
            data = s.tobytes()
        else:
            a = np.asarray(value)
            if a.dtype.kind == "f":
                a = a.astype(a.dtype.newbyteorder("<"))
            dt = _dtype_msg(a)
            shape = a.shape
            data = np.ascontiguousarray(a).tobytes()
        ds = _dataspace_msg(shape)
        body = (struct.pack("<BBHHH", 1, 0, len(nb), len(dt), len(ds)) + _pad8(nb) + _pad8(dt)
                + _pad8(ds) + data)
        return self.message(0x0C, body)

    def chunked_dataset(self, c: Chunked) -> int:
        a = c.data
        if a.dtype.kind not in ("f", "i", "u"):
            raise HDF5Error("chunked datasets of numbers only")
        a = np.ascontiguousarray(a.astype(a.dtype.newbyteorder("<")))
        es = a.dtype.itemsize
        grid = [range(0, max(n, 1), ch) for n, ch in zip(a.shape, c.chunks)]
        offsets = [()]
        for g in grid:
            offsets = [o + (x,) for o in offsets for x in g]
        if len(offsets) > 2 * _ISTORE_K:
            raise HDF5Error(f"at most {2 * _ISTORE_K} chunks per dataset")
        entries = []
        for off in offsets:
            block = np.zeros(c.chunks, dtype=a.dtype)
            sl = tuple(slice(o, min(o + ch, n)) for o, ch, n in zip(off, c.chunks, a.shape))
            block[tuple(slice(0, x.stop - x.start) for x in sl)] = a[sl]
            raw = block.tobytes()
            if c.shuffle:
                raw = np.frombuffer(raw, np.uint8).reshape(-1, es).T.tobytes()
            if c.gzip is not None:
                raw = zlib.compress(raw, c.gzip)
            entries.append((off, len(raw), self.alloc(raw)))
        nd = a.ndim + 1
        ksz = 8 + 8 * nd

        def key(size, off):
            return struct.pack("<II", size, 0) + b"".join(struct.pack("<Q", o) for o in off) \
                + struct.pack("<Q", 0)

        body = b""
        for off, size, addr in entries:
            body += key(size, off) + struct.pack("<Q", addr)
        end = tuple(-(-n // ch) * ch for n, ch in zip(a.shape, c.chunks))
        body += key(0, end)
        body += bytes((2 * _ISTORE_K - len(entries)) * (ksz + 8))
        bt = self.alloc(b"TREE" + struct.pack("<BBH", 1, 0, len(entries))
                        + struct.pack("<QQ", _UNDEF, _UNDEF) + body)
        filt = b""
        nf = 0
        if c.shuffle:
            filt += struct.pack("<HHHHI4x", 2, 0, 1, 1, es)
            nf += 1
        if c.gzip is not None:
            filt += struct.pack("<HHHHI4x", 1, 0, 0, 1, c.gzip)
            nf += 1
        msgs = [self.message(0x01, _dataspace_msg(a.shape)),
                self.message(0x03, _dtype_msg(a)),
                self.message(0x05, struct.pack("<BBBB", 2, 2, 2, 0))]
        if nf:
            msgs.append(self.message(0x0B, struct.pack("<BB6x", 1, nf) + filt))
        layout = struct.pack("<BBB", 3, 2, nd) + struct.pack("<Q", bt) + b"".join(
            struct.pack("<I", x) for x in c.chunks + (es,))
        msgs.append(self.message(0x08, layout))
        msgs += [self.attribute_msg(k, v) for k, v in c.attrs.items()]
        return self.object_header(msgs)

    def dataset(self, value, attrs) -> int:
        if isinstance(value, Chunked):
            return self.chunked_dataset(value)
        s = _as_strings(value)
        if s is not None:
            a = s
            dt = _string_dtype_msg(s.dtype.itemsize)
        else:
            a = np.asarray(value)
            if a.dtype.byteorder == ">" or (a.dtype.byteorder == "=" and not _little()):
                a = a.astype(a.dtype.newbyteorder("<"))
            if a.dtype.kind == "b":
                a = a.astype(np.uint8)
            dt = _dtype_msg(a)
        raw = np.ascontiguousarray(a).tobytes()
        addr = self.alloc(raw) if raw else _UNDEF
        msgs = [self.message(0x01, _dataspace_msg(a.shape)),
                self.message(0x03, dt),
                # fill value message version 2: allocation late, write never, undefined
                self.message(0x05, struct.pack("<BBBB", 2, 2, 2, 0)),
                self.message(0x08, struct.pack("<BB", 3, 1) + struct.pack("<QQ", addr, len(raw)))]
        msgs += [self.attribute_msg(k, v) for k, v in (attrs or {}).items()]
        return self.object_header(msgs)

    def group(self, children: Dict[str, int], attrs=None):
        """Object header, B-tree, symbol nodes and local heap of a group whose members
        (name -> object header address) are already written.  Returns (object header
        address, B-tree address, heap address)."""
        names = sorted(children)
        heap = bytearray(b"\x00" * 8)  # offset 0: the empty name
        offs = {}
        for n in names:
            offs[n] = len(heap)
            heap += _pad8(n.encode("utf-8") + b"\x00")
        heap_size = max(len(heap), 8)
        data_addr = self.alloc(bytes(heap))
        heap_addr = self.alloc(b"HEAP" + struct.pack("<B3xQQQ", 0, heap_size, _UNDEF, data_addr))
        cap = 2 * _GROUP_K
        chunks = [names[i:i + cap] for i in range(0, len(names), cap)] or [[]]
        snods = []
        for ch in chunks:
            ent = b"".join(struct.pack("<QQII16x", offs[n], children[n], 0, 0) for n in ch)
            ent += bytes((cap - len(ch)) * 40)
            snods.append(self.alloc(b"SNOD" + struct.pack("<BBH", 1, 0, len(ch)) + ent))
        if len(snods) > 2 * _GROUP_K:
            raise HDF5Error(f"groups of more than {cap * 2 * _GROUP_K} members are not "
                            "supported by the writer")
        # one leaf B-tree node: key i = heap offset of the last name of child i-1
        keys = [0] + [offs[ch[-1]] if ch else 0 for ch in chunks]
        body = struct.pack("<Q", keys[0])
        for i, sn in enumerate(snods):
            body += struct.pack("<QQ", sn, keys[i + 1])
        body += bytes((2 * _GROUP_K - len(snods)) * 16)
        bt = self.alloc(b"TREE" + struct.pack("<BBH", 0, 0, len(snods))
                        + struct.pack("<QQ", _UNDEF, _UNDEF) + body)
        msgs = [self.message(0x11, struct.pack("<QQ", bt, heap_addr))]
        msgs += [self.attribute_msg(k, v) for k, v in (attrs or {}).items()]
        return self.object_header(msgs), bt, heap_addr


def _little() -> bool:
    return np.little_endian


def write_file(path: str, tree: dict, attrs: Optional[dict] = None,
               vlen_strings: bool = True) -> None:
    """Write ``tree`` as an HDF5 file: a dict is a group, an array (or scalar, or
    string) a dataset, a ``(value, attrs)`` tuple a dataset with attributes and a
    ``Chunked`` a chunked (optionally compressed) dataset; a ``{"__attrs__": {...}}``
    entry of a dict gives the group's attributes.  ``attrs``: attributes of the root
    group.  String attributes are variable-length UTF-8 strings (as h5py writes str)
    unless ``vlen_strings`` is False."""
    w = _Writer(vlen_strings)
    sb_size = 8 + 16 + 4 * 8 + 40
    w.reserve(sb_size)

    def emit(node, node_attrs=None):
        if isinstance(node, dict):
            kids = {}
            for k, v in node.items():
                if k == "__attrs__":
                    continue
                if "/" in k or not k:
                    raise HDF5Error(f"bad member name {k!r}")
                kids[k] = emit(v)[0]
            return w.group(kids, node.get("__attrs__", node_attrs))
        if isinstance(node, tuple) and len(node) == 2 and isinstance(node[1], dict):
            return w.dataset(node[0], node[1]), None, None
        return w.dataset(node, None), None, None

    root_attrs = dict(tree.get("__attrs__", {})) if isinstance(tree, dict) else {}
    root_attrs.update(attrs or {})
    root, bt, heap = emit(dict(tree, __attrs__=root_attrs))
    while len(w.buf) % 8:
        w.buf.append(0)
    eof = len(w.buf)
    sb = (_SIG + struct.pack("<BBBBBBBBHHI", 0, 0, 0, 0, 0, 8, 8, 0, _GROUP_K, 16, 0)
          + struct.pack("<QQQQ", 0, _UNDEF, eof, _UNDEF)
          + struct.pack("<QQII", 0, root, 1, 0) + struct.pack("<QQ", bt, heap))
    assert len(sb) == sb_size
    w.put(0, sb)
    with open(path, "wb") as f:
        f.write(bytes(w.buf))
