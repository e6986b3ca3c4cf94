"""Writer of the reference's output files (TrajectorySimulation.jl:502-546).

`write_output!` stores, at the top level of a JLD2 file (or an HDF5 file
with `output_fmt=:h5`), the datasets info (written when the file is created,
:237), params_text, params (JLD2 only), px, py[, pz], momentum_spec, ion_prob,
ion_prob_uncollected and num_effective_traj.  This module writes the same names
with numpy and zlib only (no libhdf5), as the HDF5 subset JLD2 itself writes
(published HDF5 File Format Specification 3.0):

  - a version-2 superblock; for `.jld2` behind JLD2's 512-byte identification
    block, with the base address after it, as JLD2 does;
  - the root group as a version-2 object header with a Link Info message (no
    fractal heap: links stored in the header), a Group Info message and one
    hard Link message per dataset;
  - each dataset as a version-2 object header with the four messages JLD2
    writes: fill value (version 3, flags 0x09), dataspace (version 2),
    datatype (version 3: IEEE little-endian float64, signed 64-bit integer, or
    null-padded UTF-8 fixed-length strings) and data layout (version 4:
    compact for small data, contiguous otherwise);
  - a compressed dataset (`output_compress`, which the reference applies to
    momentum_spec only) as one chunk: data layout version 4 with the
    single-chunk index and its filtered size, and a version-2 filter pipeline
    message: deflate (filter 1, zlib format) as JLD2's `compress=true`, and for
    :h5 the byte shuffle (filter 2) before deflate at level 6, as HDF5.jl's
    `shuffle=true, deflate=6`;
  - a nested mapping as a group (an object header of links, like the root);
  - every superblock and object header closed by its Jenkins lookup3
    checksum (Bob Jenkins' `hashlittle`, initval 0), as HDF5 requires.

Arrays are written with their dimensions reversed and their data in Julia's
column-major order, so HDF5.jl and JLD2 read back the Julia array.  The
reference's `params` entry is a serialized Julia object (an OrderedDict of
Symbols, tuples and the laser and target structs, whose JLD2 form names Julia
types); here it is a group of plain datasets with the same keys and values
(symbols as strings, tuples as arrays, the laser and target as groups of
their `Serialize` fields), which HDF5 and JLD2 readers open without eTraj.
"""
import struct
import zlib

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
_SIG = b"\x89HDF\r\n\x1a\n"
_COMPACT_MAX = 64  # bytes of data stored inside the object header


def _rot(x, k):
    return ((x << k) | (x >> (32 - k))) & 0xFFFFFFFF


def lookup3(data, initval=0):
    """Bob Jenkins' lookup3 `hashlittle` of a byte string (the HDF5 metadata checksum)."""
    n = len(data)
    a = b = c = (0xDEADBEEF + n + initval) & 0xFFFFFFFF
    k = 0
    while n > 12:
        a = (a + struct.unpack_from("<I", data, k)[0]) & 0xFFFFFFFF
        b = (b + struct.unpack_from("<I", data, k + 4)[0]) & 0xFFFFFFFF
        c = (c + struct.unpack_from("<I", data, k + 8)[0]) & 0xFFFFFFFF
        # mix(a, b, c)
        a = (a - c) & 0xFFFFFFFF; a ^= _rot(c, 4); c = (c + b) & 0xFFFFFFFF
        b = (b - a) & 0xFFFFFFFF; b ^= _rot(a, 6); a = (a + c) & 0xFFFFFFFF
        c = (c - b) & 0xFFFFFFFF; c ^= _rot(b, 8); b = (b + a) & 0xFFFFFFFF
        a = (a - c) & 0xFFFFFFFF; a ^= _rot(c, 16); c = (c + b) & 0xFFFFFFFF
        b = (b - a) & 0xFFFFFFFF; b ^= _rot(a, 19); a = (a + c) & 0xFFFFFFFF
        c = (c - b) & 0xFFFFFFFF; c ^= _rot(b, 4); b = (b + a) & 0xFFFFFFFF
        n -= 12
        k += 12
    if n == 0:
        return c
    tail = data[k:k + n] + b"\x00" * (12 - n)
    a = (a + struct.unpack_from("<I", tail, 0)[0]) & 0xFFFFFFFF
    b = (b + struct.unpack_from("<I", tail, 4)[0]) & 0xFFFFFFFF
    c = (c + struct.unpack_from("<I", tail, 8)[0]) & 0xFFFFFFFF
    # final(a, b, c)
    c ^= b; c = (c - _rot(b, 14)) & 0xFFFFFFFF
    a ^= c; a = (a - _rot(c, 11)) & 0xFFFFFFFF
    b ^= a; b = (b - _rot(a, 25)) & 0xFFFFFFFF
    c ^= b; c = (c - _rot(b, 16)) & 0xFFFFFFFF
    a ^= c; a = (a - _rot(c, 4)) & 0xFFFFFFFF
    b ^= a; b = (b - _rot(a, 14)) & 0xFFFFFFFF
    c ^= b; c = (c - _rot(b, 24)) & 0xFFFFFFFF
    return c


_F64 = bytes.fromhex("31203f00") + struct.pack("<I", 8) + bytes.fromhex("00004000340b0034ff030000")
_I64 = bytes.fromhex("30080000") + struct.pack("<I", 8) + bytes.fromhex("00004000")


def _msg(mtype, body, flags=0):
    return struct.pack("<BHB", mtype, len(body), flags) + body


def _ohdr(messages):
    body = b"".join(messages)
    if len(body) < 256:
        flags, size = 0x00, struct.pack("<B", len(body))
    elif len(body) < 65536:
        flags, size = 0x01, struct.pack("<H", len(body))
    else:
        flags, size = 0x02, struct.pack("<I", len(body))
    head = b"OHDR" + bytes([2, flags]) + size + body
    return head + struct.pack("<I", lookup3(head))


def _strings(vals):
    raw = [v.encode("utf-8") for v in vals]
    n = max([len(r) for r in raw] + [1])
    return bytes([0x33, 0x11, 0x00, 0x00]) + struct.pack("<I", n), b"".join(r.ljust(n, b"\x00") for r in raw)


def _encode(value):
    """(datatype message body, dataspace message body, raw bytes, element size) of a value."""
    if isinstance(value, str):
        dtype, raw = _strings([value])
        return dtype, bytes([2, 0, 0, 0]), raw, len(raw)
    if isinstance(value, (list, tuple)) and value and all(isinstance(v, str) for v in value):
        dtype, raw = _strings(list(value))
        return dtype, bytes([2, 1, 0, 1]) + struct.pack("<Q", len(value)), raw, len(raw) // len(value)
    arr = np.asarray(value)
    if arr.dtype.kind in "iub":
        dtype, arr = _I64, arr.astype("<i8")
    elif arr.dtype.kind == "f":
        dtype, arr = _F64, arr.astype("<f8")
    else:
        raise TypeError("unsupported value type %s" % arr.dtype)
    if arr.ndim == 0:
        space = bytes([2, 0, 0, 0])
    else:
        dims = arr.shape[::-1]  # HDF5's row-major dims of a column-major Julia array
        space = bytes([2, arr.ndim, 0, 1]) + b"".join(struct.pack("<Q", d) for d in dims)
    return dtype, space, arr.ravel(order="F").tobytes(), 8


def _filters(shuffle, esize, level):
    """Filter pipeline message (version 2) body: [shuffle,] deflate."""
    f = []
    if shuffle:
        f.append(struct.pack("<HHH", 2, 0x0001, 1) + struct.pack("<I", esize))
    f.append(struct.pack("<HHH", 1, 0x0001, 1) + struct.pack("<I", level))
    return bytes([2, len(f)]) + b"".join(f)


def _shuffled(raw, esize):
    """HDF5's byte shuffle: byte k of every element, for k = 0 .. esize-1."""
    if esize <= 1:
        return raw
    return np.frombuffer(raw, np.uint8).reshape(-1, esize).T.tobytes()


def write(path, items, jld2=True, compress=()):
    """Writes the (name, value) pairs of `items` as top-level datasets of a new
    file at `path`.  Values: str, int, float, numpy arrays, lists of str, or a
    dict of such values (a group, nested).  Names in `compress` are written as
    one deflated chunk (with the byte shuffle in front for HDF5 files)."""
    block = b""
    if jld2:
        ident = b"HDF5-based Julia Data Format, version 0.1.1\x00 (etraj-gb300)\x00"
        block = ident.ljust(512, b"\x00")
    base = len(block)
    out = bytearray(48)  # superblock, filled at the end

    def here():
        return len(out)

    def dataset(name, value):
        dtype, space, raw, esize = _encode(value)
        msgs = [_msg(0x05, bytes([3, 0x09])), _msg(0x01, space), _msg(0x03, dtype, flags=1)]
        if name in compress and len(raw) > 0 and space[1] > 0:
            packed = zlib.compress(_shuffled(raw, esize) if not jld2 else raw, 6)
            addr = here()
            out.extend(packed)
            rank = space[1]
            dims = struct.unpack_from("<%dQ" % rank, space, 4)
            layout = bytes([4, 2, 0x02, rank + 1, 8]) + b"".join(struct.pack("<Q", d) for d in dims)
            layout += struct.pack("<Q", esize) + bytes([1]) + struct.pack("<QI", len(packed), 0)
            layout += struct.pack("<Q", addr)
            msgs.append(_msg(0x0B, _filters(not jld2, esize, 6), flags=1))
        elif len(raw) <= _COMPACT_MAX:
            layout = bytes([4, 0]) + struct.pack("<H", len(raw)) + raw
        else:
            addr = here()
            out.extend(raw)
            layout = bytes([4, 1]) + struct.pack("<QQ", addr, len(raw))
        msgs.append(_msg(0x08, layout))
        hdr = here()
        out.extend(_ohdr(msgs))
        return hdr

    def group(entries):
        links = []
        for name, value in entries:
            addr = group(list(value.items())) if isinstance(value, dict) else dataset(name, value)
            links.append((name, addr))
        msgs = [_msg(0x02, bytes([0, 0]) + struct.pack("<QQ", UNDEF, UNDEF)), _msg(0x0A, bytes([0, 0]))]
        for name, addr in links:
            nb = name.encode("utf-8")
            if len(nb) > 255:
                raise ValueError("dataset name too long")
            msgs.append(_msg(0x06, bytes([1, 0x10, 0x01, len(nb)]) + nb + struct.pack("<Q", addr)))
        hdr = here()
        out.extend(_ohdr(msgs))
        return hdr

    root = group(list(items))
    eof = len(out)
    sb = _SIG + bytes([2, 8, 8, 0]) + struct.pack("<QQQQ", base, UNDEF, eof, root)
    out[0:48] = sb + struct.pack("<I", lookup3(sb))
    with open(path, "wb") as f:
        f.write(block + bytes(out))
