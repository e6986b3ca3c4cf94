"""GB300-native ensemble-trajectory engine for strong-field ionization.

Host side of the drop-in for eTraj.jl's trajectory-simulation hot path: the
reference's lasers, targets and `perform_traj_simulation` keywords, driving
the sm_103a CUDA library behind include/etraj.h.
"""
from . import h5write, jld2
from .abi import load_library
from .lasers import (Laser, MonochromaticLaser, Cos4Laser, Cos2Laser, GaussianLaser,
                     BichromaticLaser)
from .targets import (Target, SAEAtomBase, HydrogenLikeAtom, SAEAtom, get_atom,
                      get_available_atoms, hartree_asymp_coeff, MoleculeBase, GenericMolecule,
                      LoadMolecule, get_mol, get_available_mols)
from .simulation import (perform_traj_simulation, make_job, rate_prefix_bits, Engine, Server,
                         EtrajError, default_engine)

__all__ = ["load_library", "Laser", "MonochromaticLaser", "Cos4Laser", "Cos2Laser",
           "GaussianLaser", "BichromaticLaser", "Target", "SAEAtomBase", "HydrogenLikeAtom",
           "SAEAtom", "get_atom", "get_available_atoms", "hartree_asymp_coeff", "MoleculeBase",
           "GenericMolecule", "LoadMolecule", "get_mol", "get_available_mols",
           "perform_traj_simulation", "make_job", "rate_prefix_bits", "Engine", "Server",
           "EtrajError", "default_engine"]
