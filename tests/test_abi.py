"""The C ABI boundary, checked without a GPU: the library loads, exports every
function include/etraj.h declares, and the ctypes mirror matches the C layout."""
import ctypes as C
import os
import re
import subprocess

import pytest

import etraj_gb300 as et
from etraj_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "etraj.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(etraj_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for n in ("etraj_create", "etraj_destroy", "etraj_run", "etraj_sample_batch", "etraj_integrate",
              "etraj_submit", "etraj_poll", "etraj_wait", "etraj_last_error", "etraj_validate"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = abi.load_library()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert {s[0] for s in abi.SIGNATURES} == set(declared_functions())
    assert b"sm_103a" in lib.etraj_version()


def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "probe.c"
    fields = {
        "etraj_mono_laser": [f for f, _ in abi.MonoLaser._fields_],
        "etraj_laser": [f for f, _ in abi.Laser._fields_],
        "etraj_target": [f for f, _ in abi.Target._fields_],
        "etraj_job": [f for f, _ in abi.Job._fields_],
        "etraj_result": [f for f, _ in abi.Result._fields_],
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "etraj.h"', "int main(void){"]
    for st, fs in fields.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (st, st))
        for f in fs:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (st, f, st, f))
    lines.append("return 0;}")
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.split("\n") if l)
    py = {"etraj_mono_laser": abi.MonoLaser, "etraj_laser": abi.Laser, "etraj_target": abi.Target,
          "etraj_job": abi.Job, "etraj_result": abi.Result}
    for st, cls in py.items():
        assert int(out[st]) == C.sizeof(cls), st
        for f in fields[st]:
            assert int(out["%s.%s" % (st, f)]) == getattr(cls, f).offset, (st, f)


def test_validate_without_gpu():
    """etraj_validate is host-only: it answers without touching a device."""
    lib = abi.load_library()
    l = et.Cos4Laser(peak_int=1e14, wave_len=800.0, cyc_num=2, ellip=0.0)
    job = et.make_job(init_cond_method="ADK", laser=l, target=et.get_atom("H"), dimension=2,
                      sample_t_intv=(-100, 100), sample_t_num=10, traj_t_final=300,
                      final_p_max=(1.5, 1.5), final_p_num=(50, 50), ss_kd_max=1.0, ss_kd_num=11)
    buf = C.create_string_buffer(256)
    assert lib.etraj_validate(C.byref(job), buf, 256) == abi.OK
    bad = job.copy()
    bad.traj_t_final = 50.0
    assert lib.etraj_validate(C.byref(bad), buf, 256) == abi.ERR_INVALID_ARGUMENT
    assert b"traj_t_final" in buf.value
    bad = job.copy()
    bad.ss_kd_num = 0
    assert lib.etraj_validate(C.byref(bad), buf, 256) == abi.ERR_INVALID_ARGUMENT
    bad.init_cond_method = abi.SAMPLER_SPANE  # the reference's message names the sampler
    assert lib.etraj_validate(C.byref(bad), buf, 256) == abi.ERR_INVALID_ARGUMENT
    assert buf.value.startswith(b"[SPANESampler] Invalid kd sample number")
    bad = job.copy()
    bad.ss_kd_num = 1  # Julia's range(-1.0, 1.0; length=1) throws: the endpoints differ
    assert lib.etraj_validate(C.byref(bad), buf, 256) == abi.ERR_INVALID_ARGUMENT
    assert b"endpoints differ" in buf.value
    bad = job.copy()
    bad.target.l = 5
    bad.target.m = 0
    assert lib.etraj_validate(C.byref(bad), buf, 256) == abi.ERR_UNSUPPORTED
    # the bulk integrator's FP32 clock covers at most 4096 periods (2^21 intervals of T/512)
    T = 2 * 3.141592653589793 * 800.0 / 45.563352525
    ok = job.copy()
    ok.precision = abi.PRECISION_FP32_BULK
    ok.traj_t_final = -100.0 + 4000 * T
    assert lib.etraj_validate(C.byref(ok), buf, 256) == abi.OK
    ok.traj_t_final = -100.0 + 4100 * T
    assert lib.etraj_validate(C.byref(ok), buf, 256) == abi.ERR_UNSUPPORTED
    assert b"4096" in buf.value
    ok.precision = abi.PRECISION_FP64
    assert lib.etraj_validate(C.byref(ok), buf, 256) == abi.OK


def test_python_mirror_rejects_what_the_reference_rejects():
    l = et.Cos4Laser(peak_int=1e14, wave_len=800.0, cyc_num=2, ellip=0.0)
    kw = dict(init_cond_method="ADK", laser=l, target=et.get_atom("H"), dimension=2,
              sample_t_intv=(-100, 100), sample_t_num=10, traj_t_final=300,
              final_p_max=(1.5, 1.5), final_p_num=(50, 50), ss_kd_max=1.0, ss_kd_num=11)
    with pytest.raises(AssertionError):
        et.make_job(**{**kw, "dimension": 4})
    with pytest.raises(AssertionError):
        et.make_job(**{**kw, "final_p_num": (50, 50, 50)})
    with pytest.raises(ValueError):
        et.make_job(**{**kw, "traj_phase_method": "XYZ"})
    with pytest.raises(TypeError):  # WFATSampler takes molecular targets only (WFATSampler.jl:4)
        et.make_job(**{**kw, "init_cond_method": "WFAT"})
    with pytest.raises(AssertionError):
        et.Cos4Laser(peak_int=1e14, cyc_num=2, ellip=0.0)
    with pytest.raises(AssertionError):
        et.HydrogenLikeAtom(Ip=-0.5, Z=1)
    with pytest.raises(KeyError):
        et.get_atom("Xe", 2)


def test_julia_binding_structs_are_generated_and_match_c(tmp_path):
    """The Julia structs of the ccall binding are the generator's
    output for include/etraj.h, and their layout is the C compiler's."""
    from etraj_gb300 import julia_structs as J

    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    assert J.julia_structs() in text
    layout = J.julia_layout()
    parsed = J.parse_header()
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "etraj.h"', "int main(void){"]
    for st, _ in J.STRUCTS:
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (st, st))
        for f, _, _, _ in parsed[st]:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (st, f, st, f))
    lines.append("return 0;}")
    src = tmp_path / "jprobe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "jprobe"
    subprocess.run(["gcc", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.split("\n") if l)
    for st, _ in J.STRUCTS:
        size, offs = layout[st]
        assert int(out[st]) == size, st
        assert [f for f, _, _, _ in parsed[st]] == list(offs), st
        for f, o in offs.items():
            assert int(out["%s.%s" % (st, f)]) == o, (st, f)
