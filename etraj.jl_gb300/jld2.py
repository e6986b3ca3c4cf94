"""Reader for the JLD2 files of the reference's molecule database.

JLD2 (the Julia package, file format "HDF5-based Julia Data Format 0.1")
writes a subset of HDF5: a version-2 superblock after a 512-byte user block,
version-2 object headers ("OHDR"/"OCHK"), links stored in the header, compact
or contiguous data layouts, global heaps ("GCOL") for variable-length data,
and Julia structs as HDF5 compound types that are committed under `_types/`.
This module reads that subset with numpy only (no h5py), following the
published HDF5 File Format Specification (version 3.0): superblock (II.A),
object headers and their messages (IV.A), global heap (III.E).

Julia values come back as Python values: bits arrays as numpy arrays in
Julia's (column-major) shape, structs as dicts of their fields, object
references resolved to the referenced values, `Dict` as dict, `Set` as set,
`Pair` as tuple, `Complex` arrays as numpy complex arrays, `String` as str,
`Nothing` as None.  Only what the molecule files use is supported; anything
else raises ValueError.
"""
import struct

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"


class _Type:
    """A decoded HDF5 datatype."""

    def __init__(self, cls, size, **kw):
        self.cls, self.size = cls, size
        self.__dict__.update(kw)


class JLD2File:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.buf = f.read()
        pos = self.buf.find(_SIG)
        if pos < 0:
            raise ValueError("not an HDF5/JLD2 file: %s" % path)
        b = self.buf
        ver = b[pos + 8]
        if ver not in (2, 3):
            raise ValueError("unsupported superblock version %d" % ver)
        if b[pos + 9] != 8 or b[pos + 10] != 8:
            raise ValueError("only 8-byte offsets and lengths are supported")
        self.base, _ext, _eof, root = struct.unpack_from("<QQQQ", b, pos + 12)
        self.root = root
        self._objs = {}
        self._gheap = {}

    # ---- low level -----------------------------------------------------------
    def _abs(self, addr):
        return self.base + addr

    def _messages(self, addr):
        """The (type, flags, body) messages of the object header at addr."""
        b, p = self.buf, self._abs(addr)
        if b[p:p + 4] != b"OHDR":
            raise ValueError("object header v1 at %#x is not supported" % addr)
        ver, flags = b[p + 4], b[p + 5]
        if ver != 2:
            raise ValueError("object header version %d" % ver)
        q = p + 6
        if flags & 0x20:
            q += 16  # access/modification/change/birth times
        if flags & 0x10:
            q += 4  # attribute phase change values
        szlen = 1 << (flags & 3)
        size = int.from_bytes(b[q:q + szlen], "little")
        q += szlen
        msgs = []
        blocks = [(q, q + size)]
        while blocks:
            s, e = blocks.pop(0)
            while s + 4 <= e:
                mtype = b[s]
                msize = struct.unpack_from("<H", b, s + 1)[0]
                mflags = b[s + 3]
                s += 4
                if flags & 0x04:
                    s += 2  # creation order
                body = b[s:s + msize]
                s += msize
                if mtype == 0x10:  # continuation
                    off, ln = struct.unpack_from("<QQ", body, 0)
                    c = self._abs(off)
                    if b[c:c + 4] != b"OCHK":
                        raise ValueError("bad continuation block")
                    blocks.append((c + 4, c + ln - 4))
                elif mtype != 0:
                    msgs.append((mtype, mflags, body))
        return msgs

    def _dtype(self, body, off=0):
        """Decodes a datatype message starting at body[off]; returns (_Type, length)."""
        cv = body[off]
        cls, ver = cv & 0x0F, cv >> 4
        bits = body[off + 1] | (body[off + 2] << 8) | (body[off + 3] << 16)
        size = struct.unpack_from("<I", body, off + 4)[0]
        p = off + 8
        if cls == 0:  # fixed point
            signed = bool(bits & 0x08)
            return _Type(0, size, signed=signed), 12
        if cls == 1:  # floating point
            if bits & 0x01:
                raise ValueError("big-endian floats")
            return _Type(1, size), 20
        if cls == 3:  # fixed-length string
            return _Type(3, size), 8
        if cls == 5:  # opaque
            taglen = bits & 0xFF
            return _Type(5, size), 8 + taglen
        if cls == 7:  # reference
            return _Type(7, size, rtype=bits & 0x0F), 8
        if cls == 6:  # compound
            nmem = bits & 0xFFFF
            mems = []
            for _ in range(nmem):
                e = body.index(b"\x00", p)
                name = body[p:e].decode()
                if ver < 3:
                    raise ValueError("compound datatype version %d" % ver)
                p = e + 1
                nb = 1 if size < 256 else 2 if size < 65536 else 4 if size < (1 << 24) else 8
                moff = int.from_bytes(body[p:p + nb], "little")
                p += nb
                mt, ml = self._dtype(body, p)
                p += ml
                mems.append((name, moff, mt))
            return _Type(6, size, members=mems), p - off
        if cls == 9:  # variable length
            kind = bits & 0x0F
            bt, bl = self._dtype(body, p)
            return _Type(9, size, vkind=kind, base=bt), 8 + bl
        if cls == 10:  # array
            nd = body[p]
            p += 1
            if ver < 3:
                raise ValueError("array datatype version %d" % ver)
            dims = struct.unpack_from("<%dI" % nd, body, p)
            p += 4 * nd
            bt, bl = self._dtype(body, p)
            return _Type(10, size, dims=dims, base=bt), p + bl - off
        raise ValueError("datatype class %d" % cls)

    def _shared_dtype(self, body):
        """A datatype message stored as a shared (committed) message."""
        ver, typ = body[0], body[1]
        if ver == 3 and typ == 2:
            addr = struct.unpack_from("<Q", body, 2)[0]
        elif ver in (1, 2):
            addr = struct.unpack_from("<Q", body, 8 if ver == 1 else 2)[0]
        else:
            raise ValueError("shared message version %d type %d" % (ver, typ))
        return self._committed(addr)

    def _committed(self, addr):
        key = ("T", addr)
        if key not in self._objs:
            for mtype, mflags, body in self._messages(addr):
                if mtype == 0x03:
                    t = self._shared_dtype(body) if mflags & 0x02 else self._dtype(body)[0]
                    t.committed = addr
                    self._objs[key] = t
                    break
            else:
                raise ValueError("committed datatype without a datatype message")
        return self._objs[key]

    def _dataspace(self, body):
        ver = body[0]
        nd, flags = body[1], body[2]
        if ver == 1:
            p = 8
            typ = 1 if nd > 0 else 0
        else:
            typ = body[3]
            p = 4
        dims = struct.unpack_from("<%dQ" % nd, body, p) if nd else ()
        if typ == 2:
            return None  # null dataspace
        return tuple(dims)

    def _gheap_obj(self, coll, index):
        if coll not in self._gheap:
            b, p = self.buf, self._abs(coll)
            if b[p:p + 4] != b"GCOL":
                raise ValueError("bad global heap collection")
            csize = struct.unpack_from("<Q", b, p + 8)[0]
            objs, q, end = {}, p + 16, p + csize
            while q + 16 <= end:
                idx, _rc = struct.unpack_from("<HH", b, q)
                osize = struct.unpack_from("<Q", b, q + 8)[0]
                if idx == 0:
                    break
                objs[idx] = b[q + 16:q + 16 + osize]
                q += 16 + ((osize + 7) & ~7)
            self._gheap[coll] = objs
        return self._gheap[coll][index]

    # ---- values ------------------------------------------------------------------
    def _decode(self, t, raw, count):
        """count elements of type t from raw bytes -> list or numpy array."""
        if t.cls == 1:
            dt = {8: "<f8", 4: "<f4", 2: "<f2"}[t.size]
            return np.frombuffer(raw, dt, count).copy()
        if t.cls == 0:
            dt = ("<i%d" if t.signed else "<u%d") % t.size
            return np.frombuffer(raw, dt, count).copy()
        if t.cls == 7:
            addrs = np.frombuffer(raw, "<u8", count)
            return [None if a in (0, 0xFFFFFFFFFFFFFFFF) else self.read_object(int(a)) for a in addrs]
        if t.cls == 9:
            out = []
            for i in range(count):
                n, coll, idx = struct.unpack_from("<IQI", raw, i * 16)
                data = self._gheap_obj(coll, idx) if n else b""
                if t.vkind == 1:
                    out.append(data[:n * t.base.size].decode())
                else:
                    out.append(self._decode(t.base, data, n))
            return out
        if t.cls == 3:
            return [raw[i * t.size:(i + 1) * t.size].split(b"\x00")[0].decode() for i in range(count)]
        if t.cls == 5:
            return [raw[i * t.size:(i + 1) * t.size] for i in range(count)]
        if t.cls == 6:
            names = [m[0] for m in t.members]
            if names == ["re", "im"] and all(m[2].cls == 1 for m in t.members):
                dt = {8: "<f8", 4: "<f4"}[t.members[0][2].size]
                v = np.frombuffer(raw, dt, 2 * count)
                return (v[0::2] + 1j * v[1::2]).astype(np.complex128 if dt == "<f8" else np.complex64)
            out = []
            for i in range(count):
                rec = {}
                for name, moff, mt in t.members:
                    s = i * t.size + moff
                    rec[name] = self._decode(mt, raw[s:s + mt.size], 1)[0]
                out.append(self._julia_struct(rec))
            return out
        if t.cls == 10:
            n = int(np.prod(t.dims))
            return [self._decode(t.base, raw[i * t.size:(i + 1) * t.size], n) for i in range(count)]
        raise ValueError("cannot decode datatype class %d" % t.cls)

    @staticmethod
    def _julia_struct(rec):
        """Julia structs that JLD2 serializes with a custom layout."""
        keys = list(rec)
        if keys == ["kvvec"]:  # JLD2.SerializedDict: Vector{Pair}
            kv = rec["kvvec"]
            return {_hashable(k): v for k, v in (kv if isinstance(kv, list) else [])}
        if keys in (["first", "second"], ["first"], ["second"]):  # Core.Pair (a Nothing field is not stored)
            return (rec.get("first"), rec.get("second"))
        if keys and keys == [str(i + 1) for i in range(len(keys))]:  # Tuple{...}: fields "1", "2", ...
            return tuple(_hashable(rec[k]) for k in keys)
        if keys == ["dict"]:  # Base.Set{T}: Dict{T, Nothing}
            return set(rec["dict"].keys()) if isinstance(rec["dict"], dict) else set()
        return rec

    def read_object(self, addr):
        key = ("O", addr)
        if key in self._objs:
            return self._objs[key]
        msgs = self._messages(addr)
        dtype = dspace = layout = pipeline = None
        links = {}
        for mtype, mflags, body in msgs:
            if mtype == 0x0B:
                pipeline = body
            if mtype == 0x03:
                dtype = self._shared_dtype(body) if mflags & 0x02 else self._dtype(body)[0]
            elif mtype == 0x01:
                dspace = self._dataspace(body)
            elif mtype == 0x08:
                layout = body
            elif mtype == 0x06:
                name, target = self._link(body)
                links[name] = target
        if dtype is None:  # a group
            val = {k: self.read_object(a) for k, a in links.items() if k != "_types"}
            self._objs[key] = val
            return val
        if dspace is None:
            val = None if dtype.size == 0 or dtype.cls == 6 and not dtype.members else None
            self._objs[key] = val
            return val
        count = int(np.prod(dspace)) if dspace else 1
        raw = self._layout_data(layout, dtype.size * count, pipeline)
        vals = self._decode(dtype, raw, count)
        if dspace == ():
            val = vals[0]
        elif isinstance(vals, np.ndarray):
            val = vals.reshape(dspace).transpose() if len(dspace) > 1 else vals
        else:
            val = vals
        self._objs[key] = val
        return val

    @staticmethod
    def _filters(body):
        """(id, client data) of a filter pipeline message (version 1 or 2)."""
        ver, n = body[0], body[1]
        p = 8 if ver == 1 else 2
        out = []
        for _ in range(n):
            fid = struct.unpack_from("<H", body, p)[0]
            p += 2
            nlen = 0
            if ver == 1 or fid >= 256:
                nlen = struct.unpack_from("<H", body, p)[0]
                p += 2
            _flags, ncd = struct.unpack_from("<HH", body, p)
            p += 4
            if nlen:
                p += (nlen + 7) // 8 * 8 if ver == 1 else nlen
            cd = struct.unpack_from("<%dI" % ncd, body, p)
            p += 4 * ncd
            if ver == 1 and ncd % 2:
                p += 4
            out.append((fid, cd))
        return out

    def _unfilter(self, data, pipeline):
        """Undoes the filters of a chunk, last first: deflate (1) and byte shuffle (2)."""
        import zlib
        for fid, cd in reversed(self._filters(pipeline)):
            if fid == 1:
                data = zlib.decompress(data)
            elif fid == 2:
                k = cd[0] if cd else 1
                data = np.frombuffer(data, np.uint8).reshape(k, -1).T.tobytes() if k > 1 else data
            else:
                raise ValueError("filter %d is not supported" % fid)
        return data

    def _layout_data(self, body, nbytes, pipeline=None):
        ver = body[0]
        if ver not in (3, 4):
            raise ValueError("data layout version %d" % ver)
        cls = body[1]
        if cls == 0:  # compact
            n = struct.unpack_from("<H", body, 2)[0]
            return body[4:4 + n]
        if cls == 1:  # contiguous
            addr, size = struct.unpack_from("<QQ", body, 2)
            if addr == 0xFFFFFFFFFFFFFFFF:
                return b"\x00" * nbytes
            p = self._abs(addr)
            return self.buf[p:p + size]
        if cls == 2 and ver == 4:  # chunked: the single-chunk index only
            flags, rank, enc = body[2], body[3], body[4]
            p = 5 + rank * enc
            if body[p] != 1:
                raise ValueError("chunk index type %d is not supported" % body[p])
            p += 1
            size = None
            if flags & 0x02:
                size, _mask = struct.unpack_from("<QI", body, p)
                p += 12
            addr = struct.unpack_from("<Q", body, p)[0]
            q = self._abs(addr)
            data = self.buf[q:q + (size if size is not None else nbytes)]
            return self._unfilter(data, pipeline) if pipeline is not None else data
        raise ValueError("this chunked layout is not supported")

    def _link(self, body):
        ver, flags = body[0], body[1]
        if ver != 1:
            raise ValueError("link message version %d" % ver)
        p = 2
        ltype = 0
        if flags & 0x08:
            ltype = body[p]
            p += 1
        if flags & 0x04:
            p += 8
        if flags & 0x10:
            p += 1
        nb = 1 << (flags & 3)
        nlen = int.from_bytes(body[p:p + nb], "little")
        p += nb
        name = body[p:p + nlen].decode()
        p += nlen
        if ltype != 0:
            raise ValueError("soft/external links are not supported")
        return name, struct.unpack_from("<Q", body, p)[0]

    def read(self):
        """Every top-level name of the file -> its value."""
        return self.read_object(self.root)


def _hashable(k):
    if isinstance(k, np.ndarray):
        return tuple(k.tolist())
    if isinstance(k, (np.integer,)):
        return int(k)
    if isinstance(k, dict):
        return tuple(sorted(k.items()))
    if isinstance(k, list):
        return tuple(k)
    return k


def load(path):
    """Reads a JLD2 file into a dict of its top-level names."""
    return JLD2File(path).read()
