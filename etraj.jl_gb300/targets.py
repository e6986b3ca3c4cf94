"""Atomic targets with the reference's constructors and presets.

Mirrors src/Targets/HydrogenLikeAtom.jl, SAEAtom.jl, SAEAtomBase_shared.jl
and the atom presets of src/Targets/Database/AtomDatabase.jl (the table
values are physical fit parameters and are the same numbers).  The force,
potential and ODE right-hand sides run on the device.
"""
import math
import warnings

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

    def to_c(self):
        t = abi.Target()
        t.kind = abi.TARGET_HYDROGEN_LIKE
        t.Z, t.l, t.m = self.nucl_charge, self.l, self.m
        t.Ip, t.asymp_coeff = self.Ip, self.asymp_coeff
        t.quan_ax_theta, t.quan_ax_phi = self.quan_ax_θ, self.quan_ax_ϕ
        t.soft_core = self.soft_core
        return t


class SAEAtom(SAEAtomBase):
    """Single-active-electron atom with the Tong-Lin potential (SAEAtom.jl:187-252)."""

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
