"""The Hydrogen molecule of the reference's database, from the committed
fixture tests/golden/molecule_hydrogen.npz (made by
tests/golden/make_molecule_fixture.py from src/Targets/Database/Molecule_Hydrogen.jld2)."""
import os

import numpy as np

import etraj_gb300 as et

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def hydrogen(rot_α=0.0, rot_β=0.0, rot_γ=0.0):
    d = np.load(os.path.join(GOLDEN, "molecule_hydrogen.npz"))
    return et.GenericMolecule(atoms=[str(a) for a in d["atoms"]], atom_coords=d["atom_coords"],
                              charge=int(d["charge"]), spin=int(d["spin"]), name=str(d["name"]),
                              rot_α=rot_α, rot_β=rot_β, rot_γ=rot_γ, energy_levels=d["energy_levels"],
                              orbit_occ=d["orbit_occ"], wfat_intdata={0: d["wfat_intdata_0"]},
                              wfat_μ={0: d["wfat_mu_0"]}, asymp_coeff={0: d["asymp_coeff_0"]})
