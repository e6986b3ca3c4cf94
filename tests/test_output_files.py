"""The reference's output file (write_output!, TrajectorySimulation.jl:502-546)
written without libhdf5 (h5write.py), checked on the CPU: the metadata
checksum against published test vectors and the reference's own JLD2 files,
and a round trip through the package's reader."""
import os
import re
import struct

import numpy as np
import pytest

from etraj_gb300 import h5write, jld2

from conftest import REFERENCE_DB as REF_DB  # noqa: E402


def test_lookup3_published_vectors():
    # the hashlittle self-test values of Bob Jenkins' lookup3.c
    assert h5write.lookup3(b"") == 0xDEADBEEF
    assert h5write.lookup3(b"", 0xDEADBEEF) == 0xBD5B7DDE
    assert h5write.lookup3(b"Four score and seven years ago") == 0x17770551
    assert h5write.lookup3(b"Four score and seven years ago", 1) == 0xCD628161


@pytest.mark.skipif(not (REF_DB and os.path.isdir(REF_DB)),
                    reason="set ETRAJ_REFERENCE_DIR to a reference checkout (its database files)")
def test_lookup3_reproduces_the_checksums_of_jld2_files():
    for name in ("Molecule_Hydrogen.jld2", "Molecule_Oxygen.jld2"):
        b = open(os.path.join(REF_DB, name), "rb").read()
        p = b.find(b"\x89HDF")
        assert h5write.lookup3(b[p:p + 44]) == struct.unpack_from("<I", b, p + 44)[0]
        n = 0
        for m in re.finditer(rb"OHDR", b):
            q = m.start()
            flags = b[q + 5]
            off = 6 + (16 if flags & 0x20 else 0) + (4 if flags & 0x10 else 0)
            szlen = 1 << (flags & 3)
            end = q + off + szlen + int.from_bytes(b[q + off:q + off + szlen], "little")
            assert h5write.lookup3(b[q:end]) == struct.unpack_from("<I", b, end)[0]
            n += 1
        assert n > 20


def _items():
    spec = np.random.default_rng(1).random((7, 5, 3))
    return [("params_text", "init_cond_method: ADK\nlaser: Cos4Laser\n" * 30), ("px", np.linspace(-2, 2, 7)),
            ("py", np.linspace(-1, 1, 5)), ("pz", np.linspace(-1, 1, 3)), ("momentum_spec", spec),
            ("ion_prob", 0.0123), ("ion_prob_uncollected", 4.5e-5), ("num_effective_traj", 987654321)]


@pytest.mark.parametrize("fmt", ["jld2", "h5"])
def test_written_file_round_trips(tmp_path, fmt):
    path = str(tmp_path / ("out." + fmt))
    items = _items()
    h5write.write(path, items, jld2=(fmt == "jld2"))
    raw = open(path, "rb").read()
    if fmt == "jld2":
        assert raw.startswith(b"HDF5-based Julia Data Format") and raw[512:520] == b"\x89HDF\r\n\x1a\n"
    else:
        assert raw[:8] == b"\x89HDF\r\n\x1a\n"
    d = jld2.load(path)
    assert list(d) == [k for k, _ in items]  # the link order of write_output!
    for k, v in items:
        if isinstance(v, np.ndarray):
            assert d[k].shape == v.shape and np.array_equal(d[k], v)
        else:
            assert d[k] == v
    # every header and the superblock carry a valid checksum
    p = raw.find(b"\x89HDF")
    assert h5write.lookup3(raw[p:p + 44]) == struct.unpack_from("<I", raw, p + 44)[0]
