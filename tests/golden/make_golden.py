"""Extracts the numeric known-answer pins of eTraj.jl's own test suite into
sampler_survivors.json and physics_pins.json.

Run with a checkout of the reference (read as text, nothing is executed):
  python tests/golden/make_golden.py <reference_dir>

Sources:
  test/ElectronSamplers_test.jl:11-50   common parameters of the sampler tests
  test/ElectronSamplers_test.jl:53-320  `f(sp) == (rows, count)` for batch 200
  test/Targets_test.jl:31,56,59         potential values, He asymptotic coefficient
  test/Lasers_test.jl:29-39             getter identities
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_sampler_tests(text):
    """Yield (modifiers, expected) for every `init_sampler(; merge(params, ...)...)` test."""
    cases = []
    pat = re.compile(r"sp = init_sampler\(; (?:merge\(params(?P<mods>(?:, *\w+)*)\)|params)\.\.\.\)\s*\n"
                     r"\s*(?P<check>.*)\n")
    for m in pat.finditer(text):
        mods = [x.strip() for x in (m.group("mods") or "").split(",") if x.strip()]
        check = m.group("check").strip()
        em = re.match(r"f\(sp\) == \((\d+),(\d+)\)", check)
        expected = [int(em.group(1)), int(em.group(2))] if em else None
        line = text[: m.start()].count("\n") + 1
        cases.append({"modifiers": mods, "expected": expected, "line": line})
    return cases


def main(ref):
    path = os.path.join(ref, "test", "ElectronSamplers_test.jl")
    with open(path) as f:
        text = f.read()
    cases = parse_sampler_tests(text)
    out = {
        "source": "test/ElectronSamplers_test.jl",
        "batch_id": 200,
        "common": {
            "target": "get_atom(\"H\")",
            "laser": {"kind": "Cos4Laser", "peak_int": 1e15, "wave_len": 800.0, "cyc_num": 2,
                      "ellip": 1.0},
            "init_cond_method": "ADK", "dimension": 2, "sample_t_intv": [-100, 100],
            "sample_t_num": 400, "sample_cutoff_limit": 1e-14, "sample_monte_carlo": False,
            "traj_phase_method": "CTMC", "rate_prefix": "Full", "ss_kd_max": 2.0,
            "ss_kd_num": 800, "ss_kz_max": 2.0, "ss_kz_num": 0, "mc_kt_num": 800,
            "mc_kd_max": 2.0, "mc_kz_max": 2.0,
        },
        "modifiers": {
            "spane": {"init_cond_method": "SPANE"}, "spa": {"init_cond_method": "SPA"},
            "wfat": {"init_cond_method": "WFAT"},
            "_3d": {"dimension": 3, "ss_kd_num": 30, "ss_kz_num": 30},
            "qtmc": {"traj_phase_method": "QTMC"}, "scts": {"traj_phase_method": "SCTS"},
            "mc2d": {"sample_monte_carlo": True},
            "mc3d": {"sample_monte_carlo": True, "dimension": 3},
            "exp_": {"rate_prefix": "Exp"}, "pre": {"rate_prefix": "Pre"},
            "precc": {"rate_prefix": "PreCC"}, "jac": {"rate_prefix": "Jac"},
            "prejac": {"rate_prefix": ["Pre", "Jac"]},
            "mol": {"target": "get_mol(\"Hydrogen\")"},
            "mol_rot": {"target": "get_mol(\"Hydrogen\"; rot_β=π/2, rot_γ=π/2)"},
        },
        "cases": cases,
    }
    with open(os.path.join(HERE, "sampler_survivors.json"), "w") as f:
        json.dump(out, f, indent=1)

    pins = {
        "source": ["test/Targets_test.jl", "test/Lasers_test.jl"],
        "he_asymp_coeff": {"Z": 1, "Ip": 0.9035698802, "l": 0, "value": 0.9124458182520485,
                           "line": "test/Targets_test.jl:56"},
        "h_potential_111": {"value": -1 / 3 ** 0.5, "line": "test/Targets_test.jl:31"},
        "he_sae": {"Ip": 0.9035698802, "a1": 1.230723, "b1": 0.6620055, "a2": -1.325040,
                   "b2": 1.236224, "a3": -0.2307230, "b3": 0.4804286,
                   "line": "test/Targets_test.jl:41"},
        "gradient_points": [[0, 0, 1], [2, 8, 1], [-1, 2, 1]],
        "laser_derivative_times": [0.0, 10.0],
        "laser_l6": {"peak_int": 4e14, "wave_len": 800.0, "cyc_num": 2.0, "ellip": 1.0,
                     "azi": 3.141592653589793 / 4, "cep": 3.141592653589793, "t_shift": 10.0,
                     "line": "test/Lasers_test.jl:42"},
        "laser_l7": {"peak_int": 4e14, "wave_len": 800.0, "cyc_num": 2.0, "ellip": 1.0,
                     "azi": 0.0, "cep": 3.141592653589793, "t_shift": 10.0,
                     "line": "test/Lasers_test.jl:49"},
    }
    with open(os.path.join(HERE, "physics_pins.json"), "w") as f:
        json.dump(pins, f, indent=1)
    print("wrote %d sampler cases" % len(cases))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference_dir>")
    main(sys.argv[1])
