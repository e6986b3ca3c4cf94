"""Writer of the reference's output files (TrajectorySimulation.jl:502-546).

`write_output!` stores, at the top level of a JLD2 file (or an HDF5 file
with `output_fmt=:h5`), the datasets params_text, px, py[, pz],
momentum_spec, ion_prob, ion_prob_uncollected and num_effective_traj.  This
module writes the same names with numpy only (no libhdf5), as the HDF5 subset
JLD2 itself writes (published HDF5 File Format Specification 3.0):

  - a version-2 superblock; for `.jld2` behind JLD2's 512-byte identification
    block, with the base address after it, as JLD2 does;
  - the root group as a version-2 object header with a Link Info message (no
    fractal heap: links stored in the header), a Group Info message and one
    hard Link message per dataset;
  - each dataset as a version-2 object header with the four messages JLD2
    writes: fill value (version 3, flags 0x09), dataspace (version 2),
    datatype (version 3: IEEE little-endian float64, signed 64-bit integer, or
    a null-padded UTF-8 fixed-length string) and data layout (version 4:
    compact for small data, contiguous otherwise);
  - every superblock and object header closed by its Jenkins lookup3
    checksum (Bob Jenkins' `hashlittle`, initval 0), as HDF5 requires.

Arrays are written with their dimensions reversed and their data in Julia's
column-major order, so HDF5.jl and JLD2 read back the Julia array.  The
reference's `params` entry (a Julia object) has no counterpart here, and the
data is written uncompressed (`output_compress` would need chunked layouts
and a filter pipeline).
"""
import struct

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


def _encode(value):
    """(datatype message body, dataspace message body, raw bytes) of a value."""
    if isinstance(value, str):
        raw = value.encode("utf-8")
        n = max(len(raw), 1)
        dtype = bytes([0x33, 0x11, 0x00, 0x00]) + struct.pack("<I", n)
        return dtype, bytes([2, 0, 0, 0]), raw.ljust(n, b"\x00")
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
    return dtype, space, arr.ravel(order="F").tobytes()


def write(path, items, jld2=True):
    """Writes the (name, value) pairs of `items` (str, int, float or numpy
    arrays) as top-level datasets of a new file at `path`."""
    block = b""
    if jld2:
        ident = b"HDF5-based Julia Data Format, version 0.1.1\x00 (etraj-gb300)\x00"
        block = ident.ljust(512, b"\x00")
    base = len(block)
    out = bytearray(48)  # superblock, filled at the end
    links = []

    def here():
        return len(out)

    for name, value in items:
        dtype, space, raw = _encode(value)
        if len(raw) <= _COMPACT_MAX:
            layout = bytes([4, 0]) + struct.pack("<H", len(raw)) + raw
        else:
            addr = here()
            out += raw
            layout = bytes([4, 1]) + struct.pack("<QQ", addr, len(raw))
        hdr_addr = here()
        out += _ohdr([_msg(0x05, bytes([3, 0x09])), _msg(0x01, space), _msg(0x03, dtype, flags=1),
                      _msg(0x08, layout)])
        links.append((name, hdr_addr))
    msgs = [_msg(0x02, bytes([0, 0]) + struct.pack("<QQ", UNDEF, UNDEF)), _msg(0x0A, bytes([0, 0]))]
    for name, addr in links:
        nb = name.encode("utf-8")
        if len(nb) > 255:
            raise ValueError("dataset name too long")
        msgs.append(_msg(0x06, bytes([1, 0x10, 0x01, len(nb)]) + nb + struct.pack("<Q", addr)))
    root = here()
    out += _ohdr(msgs)
    eof = len(out)
    sb = _SIG + bytes([2, 8, 8, 0]) + struct.pack("<QQQQ", base, UNDEF, eof, root)
    out[0:48] = sb + struct.pack("<I", lookup3(sb))
    with open(path, "wb") as f:
        f.write(block + bytes(out))
