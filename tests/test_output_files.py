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


@pytest.mark.parametrize("fmt", ["jld2", "h5"])
def test_compressed_file_decodes_to_the_uncompressed_values(tmp_path, fmt):
    """output_compress (TrajectorySimulation.jl:525-541): momentum_spec as one
    deflated chunk (shuffled first for :h5); decoded it equals the data, and the
    chunk is a zlib stream any reader inflates."""
    import zlib
    items = _items()
    spec = items[4][1]
    plain, packed = str(tmp_path / ("a." + fmt)), str(tmp_path / ("b." + fmt))
    big = [(k, np.kron(v, np.ones((40, 40, 1))) if k == "momentum_spec" else v) for k, v in items]
    big_spec = dict(big)["momentum_spec"]
    h5write.write(plain, big, jld2=(fmt == "jld2"))
    h5write.write(packed, big, jld2=(fmt == "jld2"), compress=("momentum_spec",))
    assert os.path.getsize(packed) < os.path.getsize(plain) * 0.6
    a, b = jld2.load(plain), jld2.load(packed)
    assert list(a) == list(b)
    for k in a:
        if isinstance(a[k], np.ndarray):
            assert a[k].shape == b[k].shape and np.array_equal(a[k], b[k]), k
        else:
            assert a[k] == b[k], k
    assert np.array_equal(b["momentum_spec"], big_spec) and spec.shape == (7, 5, 3)
    # the raw chunk: a zlib stream whose inflated bytes are the column-major data
    raw = open(packed, "rb").read()
    p = raw.find(b"\x78\x9c")
    data = zlib.decompressobj().decompress(raw[p:])
    want = big_spec.ravel(order="F").tobytes()
    if fmt == "h5":  # HDF5's byte shuffle: byte k of every element together
        want = np.frombuffer(want, np.uint8).reshape(-1, 8).T.tobytes()
    assert data == want


def test_params_group_round_trips(tmp_path):
    """The params entry as a group: nested laser/target groups, strings, string
    arrays, tuples as arrays, booleans and integers."""
    params = {"init_cond_method": "SPA", "laser": {"type": "BichromaticLaser",
                                                   "laser1": {"type": "Cos4Laser", "peak_int": 5e13},
                                                   "laser2": {"type": "Cos4Laser", "peak_int": 5e13},
                                                   "delay21": 0.0},
              "target": {"type": "GenericMolecule", "atoms": ["H", "H"],
                         "atom_coords": np.array([[0.0, 0.0, -0.37], [0.0, 0.0, 0.37]])},
              "sample_t_intv": (-100.0, 100.0), "sample_monte_carlo": True, "final_p_num": (64, 64, 1),
              "rate_prefix": ["Pre", "Jac"]}
    path = str(tmp_path / "p.jld2")
    h5write.write(path, [("params", params), ("ion_prob", 0.5)])
    d = jld2.load(path)["params"]
    assert list(d) == list(params)
    assert d["init_cond_method"] == "SPA" and d["laser"]["laser2"]["peak_int"] == 5e13
    assert d["target"]["atoms"] == ["H", "H"] and np.array_equal(d["target"]["atom_coords"],
                                                                 params["target"]["atom_coords"])
    assert np.array_equal(d["sample_t_intv"], [-100.0, 100.0]) and d["sample_monte_carlo"] == 1
    assert np.array_equal(d["final_p_num"], [64, 64, 1]) and d["rate_prefix"] == ["Pre", "Jac"]


def test_params_follow_the_reference_order():
    """The effective parameters of TrajectorySimulation.jl:275-296, in order, and
    their YAML text with Julia's float printing."""
    import etraj_gb300 as et
    from etraj_gb300 import simulation as S
    kw = dict(init_cond_method="SPANE", laser=et.Cos2Laser(peak_int=1.2e14, wave_len=800.0, cyc_num=2, ellip=1.0),
              target=et.get_atom("Ar"), dimension=3, sample_t_intv=(-100, 100), sample_t_num=400,
              sample_monte_carlo=True, sample_cutoff_limit=1e-16, traj_phase_method="SCTS", traj_rtol=1e-6,
              traj_t_final=300.0, fmt="jld2", path="run.jld2", final_p_max=(2, 2, 2), final_p_num=(64, 64, 64),
              ss_kd_max=0, ss_kd_num=0, ss_kz_max=0, ss_kz_num=0, mc_kd_max=1.0, mc_kt_num=1000,
              mc_kz_max=1.0, rate_prefix="Full", mol_orbit_ridx=0)
    p = S._params(kw)
    assert list(p) == ["init_cond_method", "laser", "target", "sample_t_intv", "sample_t_num",
                       "sample_monte_carlo", "sample_cutoff_limit", "traj_phase_method", "traj_rtol",
                       "traj_t_final", "output_fmt", "output_path", "final_p_max", "final_p_num",
                       "mc_kd_max", "mc_kt_num", "mc_kz_max", "rate_prefix"]
    assert list(p["laser"]) == ["type", "peak_int", "wave_len", "cyc_num", "ellip", "azi", "cep", "t_shift"]
    assert p["target"]["type"] == "SAEAtom" and list(p["target"])[-1] == "name"
    text = S._yaml(p).splitlines()
    assert text[0] == "init_cond_method: SPANE"
    assert "  peak_int: 1.2e14" in text and "sample_cutoff_limit: 1.0e-16" in text
    i = text.index("sample_t_intv:")
    assert text[i + 1:i + 3] == ["  - -100.0", "  - 100.0"]
    assert "sample_monte_carlo: true" in text
