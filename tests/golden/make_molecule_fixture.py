"""Extracts the Hydrogen molecule of eTraj.jl's molecule database into
molecule_hydrogen.npz, and the numeric molecule pins of its test suite into
molecule_pins.json.

Run with a checkout of the reference (the data file is read with this
package's JLD2 reader; the test file is read as text, nothing is executed):
  python tests/golden/make_molecule_fixture.py <reference_dir>

Sources:
  src/Targets/Database/Molecule_Hydrogen.jld2   the data get_mol("Hydrogen") loads
  test/Targets_test.jl:100-137                  GenericMolecule accessors of that molecule
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def _jld2():
    sys.path.insert(0, ROOT)
    import __graft_entry__
    __graft_entry__.load_package()
    from etraj_gb300 import jld2
    return jld2


def main(ref):
    jld2 = _jld2()
    d = jld2.load(os.path.join(ref, "src", "Targets", "Database", "Molecule_Hydrogen.jld2"))
    assert d["wfat_indices"] == {0} and d["asymp_coeff_indices"] == {0}
    np.savez_compressed(os.path.join(HERE, "molecule_hydrogen.npz"),
                        atoms=np.array(d["atoms"]), atom_coords=d["atom_coords"], charge=d["charge"],
                        spin=d["spin"], name=np.array(d["name"]), energy_levels=d["energy_levels"],
                        orbit_occ=d["orbit_occ"], wfat_intdata_0=d["wfat_intdata"][0],
                        wfat_mu_0=d["wfat_μ"][0], asymp_coeff_0=d["asymp_coeff"][0])

    with open(os.path.join(ref, "test", "Targets_test.jl"), encoding="utf-8") as f:
        lines = f.read().split("\n")

    def num(pattern):
        for i, line in enumerate(lines):
            m = re.search(pattern, line)
            if m:
                return float(m.group(1)), "test/Targets_test.jl:%d" % (i + 1)
        raise KeyError(pattern)

    pins = {"source": "test/Targets_test.jl"}
    fl = r"(-?[0-9.]+(?:e-?[0-9]+)?)"
    for key, pat in [
        ("homo_energy", r"MolEnergyLevels\(m2\)\[1\] ≈ " + fl),
        ("intdata_1111", r"IntData\[1,1,1,1\] ≈ " + fl),
        ("G2_theta0", r"abs2\(MolWFATStructureFactor_G\(m2,0,0,0,0\.0,0\.0\)\) ≈ " + fl),
        ("G2_theta_pi2", r"abs2\(MolWFATStructureFactor_G\(m2,0,0,0,π/2,0\.0\)\) ≈ " + fl),
        ("asymp_coeff_11", r"MolAsympCoeff\(m2, 0\)\[1,1\] ≈ " + fl),
        ("potential_111", r"TargetPotential\(m2\)\(1\.0,1\.0,1\.0\) == " + fl),
    ]:
        v, where = num(pat)
        pins[key] = {"value": v, "line": where}
    _, where = num(r"TargetForce\(m2\)\(1\.0,1\.0,1\.0\) \.== \((-1)/8")
    pins["force_111"] = {"value": [-1 / 8] * 3, "line": where}
    _, where = num(r"AsympNuclCharge\(m2\)\s+== (\d+)")
    pins["asymp_charge"] = {"value": 1, "line": where}
    for i, line in enumerate(lines):
        m = re.search(r'MolExportAtomInfo\(m2\) == "(.*)"', line)
        if m:
            pins["atom_info"] = {"value": m.group(1), "line": "test/Targets_test.jl:%d" % (i + 1)}
        m = re.search(r'TargetName\(m2\)\s+== "(.*)"', line)
        if m and "name" not in pins:
            pins["name"] = {"value": m.group(1), "line": "test/Targets_test.jl:%d" % (i + 1)}
        m = re.search(r'TargetName\(m2\) == "(Oxygen.*)"', line)
        if m:
            pins["oxygen_name"] = {"value": m.group(1), "line": "test/Targets_test.jl:%d" % (i + 1)}
    with open(os.path.join(HERE, "molecule_pins.json"), "w", encoding="utf-8") as f:
        json.dump(pins, f, indent=1, ensure_ascii=False)
    print("wrote molecule_hydrogen.npz and %d pins" % (len(pins) - 1))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_molecule_fixture.py <reference_dir>")
    main(sys.argv[1])
