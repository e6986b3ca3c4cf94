"""Targets with the reference's constructors, presets and accessors.

Mirrors src/Targets/HydrogenLikeAtom.jl, SAEAtom.jl, SAEAtomBase_shared.jl,
GenericMolecule.jl and the atom presets of src/Targets/Database/AtomDatabase.jl
(the table values are physical fit parameters and are the same numbers).
Molecules load their orbital data from the reference's JLD2 database files
(jld2.py).  The force, potential and ODE right-hand sides run on the device.
"""
import math
import warnings

import numpy as np

from . import abi


def hartree_asymp_coeff(Z, Ip, l):
    """Hartree formula C_kl = 2^(n*-1)/sqrt(n* G(n*+l+1) G(n*-l)), with the
    l = 0 fallback when n* <= l (SAEAtomBase_shared.jl:3-11)."""
    if Z / math.sqrt(2 * Ip) <= l:
        warnings.warn("[hartree_asymp_coeff] Z/κ<=l, unable to determine the asymptotic coefficient "
                      "using Hartree formula. Using the l=0 case instead.")
        l = 0
    n = Z / math.sqrt(2 * Ip)
    return 2 ** (n - 1) / math.sqrt(n * math.gamma(n + l + 1) * math.gamma(n - l))


class Target:
    """Supertype of all targets."""


class SAEAtomBase(Target):
    def IonPotential(self):
        return self.Ip

    def AsympNuclCharge(self):
        return self.nucl_charge

    def AngularQuantumNumber(self):
        return self.l

    def MagneticQuantumNumber(self):
        return self.m

    def AsympCoeff(self):
        return self.asymp_coeff

    def SoftCore(self):
        return self.soft_core

    def QuantizationAxisOrientaion(self):
        return (self.quan_ax_θ, self.quan_ax_ϕ)

    def TargetName(self):
        return self.name

    def __eq__(self, other):
        return type(self) is type(other) and self.__dict__ == other.__dict__


def _resolve_coeff(name, Z, Ip, l, asymp_coeff):
    assert asymp_coeff == "hartree" or (not isinstance(asymp_coeff, str) and asymp_coeff > 0), \
        "[%s] asymp_coeff should be either `:hartree` or a positive number." % name
    if asymp_coeff == "hartree":
        return hartree_asymp_coeff(Z, Ip, l)
    return float(asymp_coeff)


class HydrogenLikeAtom(SAEAtomBase):
    """Hydrogen-like atom (HydrogenLikeAtom.jl:7-64)."""

    def __init__(self, Ip, Z, l=0, m=0, asymp_coeff="hartree", quan_ax_θ=0.0, quan_ax_ϕ=0.0,
                 soft_core=1e-10, name="[NA]"):
        assert Ip > 0, "[HydrogenLikeAtom] `Ip` should be positive."
        assert l >= 0 and l >= abs(m), "[HydrogenLikeAtom] Invalid (l,m)."
        assert soft_core >= 0, "[HydrogenLikeAtom] `soft_core` should be non-negative."
        self.Ip = float(Ip)
        self.nucl_charge = int(Z)
        self.l = int(l)
        self.m = int(m)
        self.asymp_coeff = _resolve_coeff("HydrogenLikeAtom", Z, Ip, l, asymp_coeff)
        self.quan_ax_θ = float(quan_ax_θ)
        self.quan_ax_ϕ = float(quan_ax_ϕ)
        self.soft_core = float(soft_core)
        self.name = name

    def Serialize(self):
        """The atom's parameters in the order of Serialize (HydrogenLikeAtom.jl:166-180)."""
        return {"type": "HydrogenLikeAtom", "Ip": self.Ip, "nucl_charge": self.nucl_charge, "l": self.l,
                "m": self.m, "asymp_coeff": self.asymp_coeff, "soft_core": self.soft_core,
                "quan_ax_θ": self.quan_ax_θ, "quan_ax_ϕ": self.quan_ax_ϕ, "name": self.name}

    def to_c(self):
        t = abi.Target()
        t.kind = abi.TARGET_HYDROGEN_LIKE
        t.Z, t.l, t.m = self.nucl_charge, self.l, self.m
        t.Ip, t.asymp_coeff = self.Ip, self.asymp_coeff
        t.quan_ax_theta, t.quan_ax_phi = self.quan_ax_θ, self.quan_ax_ϕ
        t.soft_core = self.soft_core
        return t


class SAEAtom(SAEAtomBase):
    """Single-active-electron atom with the Tong-Lin potential (SAEAtom.jl:7-72)."""

    def __init__(self, Ip, Z, l=0, m=0, asymp_coeff="hartree", quan_ax_θ=0.0, quan_ax_ϕ=0.0,
                 a1=0.0, b1=0.0, a2=0.0, b2=0.0, a3=0.0, b3=0.0, soft_core=1e-10, name="[NA]"):
        assert Ip > 0, "[SAEAtom] Ip should be positive."
        assert l >= 0 and l >= abs(m), "[SAEAtom] Invalid (l,m)."
        assert b1 >= 0 and b2 >= 0 and b3 >= 0, "[SAEAtom] b1,b2,b3 should be non-negative."
        assert soft_core > 0, "[SAEAtom] soft_core should be positive."
        self.Ip = float(Ip)
        self.nucl_charge = int(Z)
        self.l = int(l)
        self.m = int(m)
        self.asymp_coeff = _resolve_coeff("SAEAtom", Z, Ip, l, asymp_coeff)
        self.quan_ax_θ = float(quan_ax_θ)
        self.quan_ax_ϕ = float(quan_ax_ϕ)
        self.a1, self.b1, self.a2, self.b2, self.a3, self.b3 = map(float, (a1, b1, a2, b2, a3, b3))
        self.soft_core = float(soft_core)
        self.name = name

    def Serialize(self):
        """The atom's parameters in the order of Serialize (SAEAtom.jl:193-212)."""
        return {"type": "SAEAtom", "Ip": self.Ip, "nucl_charge": self.nucl_charge, "l": self.l, "m": self.m,
                "asymp_coeff": self.asymp_coeff, "quan_ax_θ": self.quan_ax_θ, "quan_ax_ϕ": self.quan_ax_ϕ,
                "a1": self.a1, "b1": self.b1, "a2": self.a2, "b2": self.b2, "a3": self.a3, "b3": self.b3,
                "soft_core": self.soft_core, "name": self.name}

    def to_c(self):
        t = abi.Target()
        t.kind = abi.TARGET_SAE
        t.Z, t.l, t.m = self.nucl_charge, self.l, self.m
        t.Ip, t.asymp_coeff = self.Ip, self.asymp_coeff
        t.quan_ax_theta, t.quan_ax_phi = self.quan_ax_θ, self.quan_ax_ϕ
        t.a1, t.b1, t.a2, t.b2, t.a3, t.b3 = self.a1, self.b1, self.a2, self.b2, self.a3, self.b3
        t.soft_core = self.soft_core
        return t


# Presets of src/Targets/Database/AtomDatabase.jl:54-275 (Tong & Lin,
# J. Phys. B 38, 2593 (2005) fit parameters).
HydLikeAtomData = {
    "H": dict(Ip=0.5, Z=1, name="H"),
    "He1p": dict(Ip=1.0, Z=2, name="He⁺"),
    "Li2p": dict(Ip=1.5, Z=3, name="Li²⁺"),
}

SAEAtomData = {
    "He": dict(Ip=0.9035698802, Z=1, a1=1.230723, b1=0.6620055, a2=-1.325040, b2=1.236224, a3=-0.2307230, b3=0.4804286, l=0, name="He"),
    "Ne": dict(Ip=0.79248225, Z=1, a1=8.069321, b1=2.148149, a2=-3.569610, b2=1.985509, a3=0.9306791, b3=0.6018819, l=1, name="Ne"),
    "Ne1p": dict(Ip=1.505361, Z=2, a1=8.042896, b1=2.714635, a2=0.5064300, b2=0.9818268, a3=-0.04289633, b3=0.4012269, l=1, name="Ne⁺"),
    "Ne2p": dict(Ip=2.3307635, Z=3, a1=7.000000, b1=3.007574, a2=0.6521344, b2=1.048617, a3=0.0, b3=0.0, l=1, name="Ne²⁺"),
    "Ar": dict(Ip=0.579155055, Z=1, a1=16.03862, b1=2.007423, a2=-25.54278, b2=4.524663, a3=0.9613848, b3=0.4426447, l=1, name="Ar"),
    "Ar1p": dict(Ip=1.0153715, Z=2, a1=14.98869, b1=2.217293, a2=-23.60558, b2=4.584761, a3=1.011314, b3=0.5510695, l=1, name="Ar⁺"),
    "Ar2p": dict(Ip=1.497, Z=3, a1=15.00000, b1=3.588835, a2=5.951071, b2=1.692914, a3=0.0, b3=0.0, l=1, name="Ar²⁺"),
    "V": dict(Ip=0.2479178, Z=1, a1=21.27861, b1=1.810071, a2=-30.02658, b2=3.201500, a3=0.7213853, b3=0.4534235, l=2, name="V"),
    "Ni": dict(Ip=0.28076035, Z=1, a1=26.81231, b1=1.937326, a2=-39.55201, b2=3.161884, a3=0.1876890, b3=0.2626299, l=2, name="Ni"),
    "Kr": dict(Ip=1.02895202, Z=1, a1=23.6188, b1=10.8391, a2=109.956, b2=6.55432, a3=11.8312, b3=1.27723, l=1, name="Kr"),
    "Kr1p": dict(Ip=1.790416, Z=2, a1=23.1460, b1=11.0416, a2=110.447, b2=6.67063, a3=10.8540, b3=1.41524, l=1, name="Kr⁺"),
    "Rb": dict(Ip=0.153506625, Z=1, a1=24.02321, b1=11.10663, a2=115.1998, b2=6.629123, a3=11.97679, b3=1.244882, l=0, name="Rb"),
    "Nb": dict(Ip=0.248383, Z=1, a1=4.000000, b1=1.379674, a2=-6.356689, b2=2.245839, a3=0.0, b3=0.0, l=2, name="Nb"),
    "Pd": dict(Ip=0.3063732, Z=1, a1=43.83606, b1=2.395037, a2=-93.35653, b2=4.907321, a3=1.163943, b3=0.3767380, l=2, name="Pd"),
    "Xe": dict(Ip=0.445763535, Z=1, a1=51.35554, b1=2.111554, a2=-99.92747, b2=3.737221, a3=1.644457, b3=0.4306465, l=1, name="Xe"),
    "Xe1p": dict(Ip=0.7708, Z=2, a1=37.49194, b1=9.452474, a2=103.1967, b2=5.305537, a3=14.50806, b3=1.315683, l=1, name="Xe⁺"),
    "Ta": dict(Ip=0.27744165, Z=1, a1=67.70192, b1=2.565180, a2=-135.5191, b2=4.088800, a3=4.298078, b3=0.7303277, l=2, name="Ta"),
}


def get_atom(name, charge=0, **kwargs):
    """Constructs a preset atom by name and charge (AtomDatabase.jl:33-45)."""
    key = name
    if charge > 0:
        key += "%dp" % charge
    elif charge < 0:
        key += "%dn" % (-charge)
    if key in HydLikeAtomData:
        return HydrogenLikeAtom(**{**HydLikeAtomData[key], **kwargs})
    if key in SAEAtomData:
        return SAEAtom(**{**SAEAtomData[key], **kwargs})
    raise KeyError("[get_atom] Atom name key `%s` not found in database." % key)


def get_available_atoms():
    return list(HydLikeAtomData) + list(SAEAtomData)


# ---- molecules (src/Targets/GenericMolecule.jl, Database/MoleculeDatabase.jl) ----------

class MoleculeBase(Target):
    """Supertype of molecular targets."""


def _rotzyz(a, b, g):
    ca, sa, cb, sb, cg, sg = math.cos(a), math.sin(a), math.cos(b), math.sin(b), math.cos(g), math.sin(g)
    return [[ca * cb * cg - sa * sg, -(ca * cb * sg) - sa * cg, ca * sb],
            [sa * cb * cg + ca * sg, -(sa * cb * sg) + ca * cg, sa * sb],
            [-(sb * cg), sb * sg, cb]]


def _wigner_d(j, mp, m, beta):
    """d^j_{m'm}(beta), Wigner's explicit sum."""
    f = math.factorial
    sh, ch = math.sin(beta / 2), math.cos(beta / 2)
    pref = math.sqrt(f(j + mp) * f(j - mp) * f(j + m) * f(j - m))
    s = 0.0
    for k in range(0, 2 * j + 1):
        a1, a3, a4 = j + m - k, mp - m + k, j - mp - k
        if a1 < 0 or a3 < 0 or a4 < 0:
            continue
        s += (-1) ** (mp - m + k) * pref / (f(a1) * f(k) * f(a3) * f(a4)) * ch ** (2 * j + m - mp - 2 * k) \
            * sh ** (mp - m + 2 * k)
    return s


def _last_nonzero(occ):
    """findlast(!iszero, occ) in Julia's column-major order (0-based flat index)."""
    flat = np.asarray(occ).ravel(order="F")
    nz = np.nonzero(flat)[0]
    return int(nz[-1])


class GenericMolecule(MoleculeBase):
    """A molecule with its orbital data (GenericMolecule.jl:7-92).

    The data that the reference computes with its molecular calculator (orbital
    energies, WFAT integrals, asymptotic coefficients) come from the molecule's
    JLD2 data file (LoadMolecule); there is no calculator here."""

    def __init__(self, atoms, atom_coords, charge=0, spin=0, name="[NA]", rot_α=0.0, rot_β=0.0, rot_γ=0.0,
                 energy_levels=None, orbit_occ=None, wfat_intdata=None, wfat_μ=None, asymp_coeff=None):
        assert all(isinstance(a, str) for a in atoms), "[GenericMolecule] Element type of `atoms` must be String."
        atom_coords = np.asarray(atom_coords, dtype=np.float64)
        assert atom_coords.ndim == 2 and atom_coords.shape == (len(atoms), 3), \
            "[GenericMolecule] `atom_coords` should be a Matrix of size N×3."
        assert spin >= 0, "[GenericMolecule] `spin` must be non-negative."
        self.atoms = list(atoms)
        self.atom_coords = atom_coords
        self.charge = int(charge)
        self.spin = spin
        self.name = name
        self.energy_levels = None if energy_levels is None else np.asarray(energy_levels, dtype=np.float64)
        self.orbit_occ = None if orbit_occ is None else np.asarray(orbit_occ, dtype=np.float64)
        self.wfat_intdata = dict(wfat_intdata or {})
        self.wfat_μ = dict(wfat_μ or {})
        self.asymp_coeff = dict(asymp_coeff or {})
        self.rot_α, self.rot_β, self.rot_γ = float(rot_α), float(rot_β), float(rot_γ)

    # -- properties (GenericMolecule.jl:122-340) --
    def MolAtoms(self):
        return self.atoms

    def MolAtomCoords(self):
        return self.atom_coords

    def MolCharge(self):
        return self.charge

    def MolSpin(self):
        return self.spin

    def MolEnergyDataAvailable(self):
        return self.energy_levels is not None and self.energy_levels.size > 0

    def _need_energy(self):
        if not self.MolEnergyDataAvailable():
            raise RuntimeError("[GenericMolecule] The energy data is not available, calculate first.")

    def MolEnergyLevels(self, spin=0):
        self._need_energy()
        if spin == 0 or self.spin == 0:
            return self.energy_levels
        return self.energy_levels[0 if spin == 1 else 1, :]

    def _homo(self, occ):
        return int(np.nonzero(np.asarray(occ))[0][-1])

    def MolEnergyLevel(self, orbit_ridx):
        self._need_energy()
        if self.spin != 0:
            assert isinstance(orbit_ridx, tuple) and len(orbit_ridx) == 2 and orbit_ridx[0] in (1, 2), \
                "[GenericMolecule] For an open-shell molecule, `orbit_ridx` should be a two-element tuple `(spin, ridx)`."
            s = orbit_ridx[0] - 1
            return float(self.energy_levels[s, self._index(self._homo(self.orbit_occ[s, :]) + orbit_ridx[1])])
        assert float(orbit_ridx) == int(orbit_ridx), \
            "[GenericMolecule] For a closed-shell molecule, `orbit_ridx` should be an integer."
        return float(self.energy_levels[self._index(self._homo(self.orbit_occ) + int(orbit_ridx))])

    def _index(self, i):
        if not 0 <= i < self.energy_levels.shape[-1]:
            raise IndexError("[GenericMolecule] orbital index out of the computed levels")
        return i

    def MolOrbitalOccupation(self, spin=0):
        self._need_energy()
        if spin == 0 or self.spin == 0:
            return self.orbit_occ
        return self.orbit_occ[0 if spin == 1 else 1, :]

    def MolHOMOEnergy(self, spin=0):
        self._need_energy()
        if spin == 0:
            # the reference indexes the (possibly 2-row) arrays by the last
            # occupied entry in column-major order
            return float(self.energy_levels.ravel(order="F")[_last_nonzero(self.orbit_occ)])
        if spin in (1, 2):
            s = spin - 1
            return float(self.energy_levels[s, self._homo(self.orbit_occ[s, :])])
        return [self.MolHOMOEnergy(1), self.MolHOMOEnergy(2)]

    def MolWFATAvailableIndices(self):
        return set(self.wfat_intdata)

    def MolWFATData(self, orbit_ridx):
        if not self.MolEnergyDataAvailable() or orbit_ridx not in self.wfat_intdata:
            raise RuntimeError("[GenericMolecule] The WFAT data is not available, calculate first.")
        return self.wfat_μ[orbit_ridx], self.wfat_intdata[orbit_ridx]

    def MolWFATMaxChannels(self, orbit_ridx):
        _, I = self.MolWFATData(orbit_ridx)
        return I.shape[0] - 1, (I.shape[1] - 1) // 2

    def MolWFATStructureFactor_G(self, orbit_ridx, nξ, m, θ, χ):
        """G_{nξ m}(θ, χ) (GenericMolecule.jl:236-259)."""
        μ, I = self.MolWFATData(orbit_ridx)
        assert nξ >= 0, "[GenericMolecule] nξ should be non-negative."
        nξmax, mmax, lmax = I.shape[0] - 1, (I.shape[1] - 1) // 2, I.shape[2] - 1
        if nξ > nξmax or abs(m) > mmax:
            return 0.0
        s = 0j
        for l in range(abs(m), lmax + 1):
            for mp in range(-l, l + 1):
                s += I[nξ, m + mmax, l, mp + l] * _wigner_d(l, m, mp, θ) * complex(math.cos(-mp * χ), math.sin(-mp * χ))
        R = _rotzyz(χ, θ, 0.0)
        μz = R[2][0] * μ[0] + R[2][1] * μ[1] + R[2][2] * μ[2]
        return s * math.exp(-math.sqrt(2 * self.IonPotential(orbit_ridx)) * μz)

    def MolAsympCoeffAvailableIndices(self):
        return set(self.asymp_coeff)

    def MolAsympCoeff(self, orbit_ridx):
        if not self.MolEnergyDataAvailable() or orbit_ridx not in self.asymp_coeff:
            raise RuntimeError("[GenericMolecule] The asymptotic coefficient is not available, calculate first.")
        return self.asymp_coeff[orbit_ridx]

    def MolAsympCoeff_lMax(self, orbit_ridx):
        return self.MolAsympCoeff(orbit_ridx).shape[0] - 1

    def MolRotation(self):
        return (self.rot_α, self.rot_β, self.rot_γ)

    def SetMolRotation(self, α, β=None, γ=None):
        if β is None:
            α, β, γ = α
        self.rot_α, self.rot_β, self.rot_γ = float(α), float(β), float(γ)

    def MolExportAtomInfo(self):
        return "; ".join("%s [%s]" % (a, ", ".join(repr(float(x)) for x in self.atom_coords[i]))
                         for i, a in enumerate(self.atoms))

    # -- Target interface (GenericMolecule.jl:438-446) --
    def IonPotential(self, orbit_ridx=None):
        if orbit_ridx is None:
            h = self.MolHOMOEnergy()
            return -(max(h) if isinstance(h, list) else h)
        return -self.MolEnergyLevel(orbit_ridx)

    def AsympNuclCharge(self):
        return self.charge + 1

    def TargetName(self):
        return self.name

    def TargetPotential(self):
        Z = self.charge + 1
        return lambda x, y, z: -Z * (x * x + y * y + z * z + 1.0) ** -0.5

    def TargetForce(self):
        Z = self.charge + 1
        return lambda x, y, z: tuple(-Z * (x * x + y * y + z * z + 1.0) ** -1.5 * c for c in (x, y, z))

    def to_c(self, orbit_ridx=0, wfat=False):
        """The etraj_target of the ionizing orbital `orbit_ridx`; returns
        (target, arrays the target's pointers refer to)."""
        t = abi.Target()
        t.kind = abi.TARGET_MOLECULE
        t.Z = self.charge + 1
        t.Ip = self.IonPotential(orbit_ridx)
        t.mol_Ip_traj = self.IonPotential()
        t.soft_core = 1.0
        t.mol_rot[0], t.mol_rot[1], t.mol_rot[2] = self.rot_α, self.rot_β, self.rot_γ
        keep = []
        if wfat:
            if orbit_ridx in self.wfat_intdata:
                μ, I = self.MolWFATData(orbit_ridx)
                arr = np.ascontiguousarray(np.asarray(I, dtype=np.complex128).ravel(order="F").view(np.float64))
                keep.append(arr)
                t.wfat_intdata = abi.dptr(arr)
                t.wfat_nxi_max, t.wfat_m_max, t.wfat_lmax = I.shape[0] - 1, (I.shape[1] - 1) // 2, I.shape[2] - 1
                for i in range(3):
                    t.wfat_mu[i] = float(μ[i])
        elif orbit_ridx in self.asymp_coeff:
            Cm = np.asarray(self.asymp_coeff[orbit_ridx], dtype=np.complex128)
            arr = np.ascontiguousarray(Cm.ravel(order="F").view(np.float64))
            keep.append(arr)
            t.asymp_coeff_lm = abi.dptr(arr)
            t.asymp_lmax = Cm.shape[0] - 1
        return t, keep

    def Serialize(self):
        """The molecule's parameters in the order of Serialize (GenericMolecule.jl:620-633)."""
        return {"type": "GenericMolecule", "atoms": list(self.atoms),
                "atom_coords": np.asarray(self.atom_coords, dtype=float), "charge": self.charge,
                "spin": self.spin, "name": self.name, "rot_α": self.rot_α, "rot_β": self.rot_β,
                "rot_γ": self.rot_γ}

    def __repr__(self):
        return "[GenericMolecule] %s" % self.name


def LoadMolecule(ext_data_path, rot_α=0.0, rot_β=0.0, rot_γ=0.0):
    """A GenericMolecule with the data of a JLD2 file (GenericMolecule.jl:78-110)."""
    from .jld2 import load
    d = load(ext_data_path)
    return GenericMolecule(atoms=d["atoms"], atom_coords=d["atom_coords"], charge=int(d["charge"]),
                           spin=d["spin"], name=d["name"], rot_α=rot_α, rot_β=rot_β, rot_γ=rot_γ,
                           energy_levels=d["energy_levels"], orbit_occ=d["orbit_occ"],
                           wfat_intdata=d["wfat_intdata"], wfat_μ=d["wfat_μ"], asymp_coeff=d["asymp_coeff"])


# Names of the molecule database and their data files (MoleculeDatabase.jl:49-64).
MoleculeDataPath = {
    "Hydrogen": "Molecule_Hydrogen.jld2",
    "Nitrogen": "Molecule_Nitrogen.jld2",
    "Oxygen": "Molecule_Oxygen.jld2",
    "Carbon Monoxide": "Molecule_CarbonMonoxide.jld2",
    "Nitric Oxide": "Molecule_NitricOxide.jld2",
    "Hydrochloric Acid": "Molecule_HydrochloricAcid.jld2",
    "Carbon Dioxide": "Molecule_CarbonDioxide.jld2",
    "Water": "Molecule_Water.jld2",
    "Sulfur Dioxide": "Molecule_SulfurDioxide.jld2",
    "Ammonia": "Molecule_Ammonia.jld2",
    "Acetylene": "Molecule_Acetylene.jld2",
    "Methane": "Molecule_Methane.jld2",
    "Benzene": "Molecule_Benzene.jld2",
}


def get_mol(name, rot_α=0.0, rot_β=0.0, rot_γ=0.0, database_dir=None):
    """A molecule of the database by name (MoleculeDatabase.jl:37-43).  The
    data files are those of the reference's src/Targets/Database; pass their
    folder as `database_dir` or set ETRAJ_MOLECULE_DB."""
    import os
    if name not in MoleculeDataPath:
        raise KeyError("[get_mol] Molecule name `%s` not found in database." % name)
    folder = database_dir or os.environ.get("ETRAJ_MOLECULE_DB")
    if not folder:
        raise FileNotFoundError("[get_mol] the molecule data files are not located: pass `database_dir` or set "
                                "ETRAJ_MOLECULE_DB to the folder holding %s" % MoleculeDataPath[name])
    return LoadMolecule(os.path.join(folder, MoleculeDataPath[name]), rot_α=rot_α, rot_β=rot_β, rot_γ=rot_γ)


def get_available_mols():
    return list(MoleculeDataPath)
