"""Model containers for the structure-factor path (host side).

These mirror the reference's inputs to ``HansenCoppensStructureFactorCalculator``:

* ``Wavefunction`` ~ ``HC_WfnType`` (include/discamb/HC_Model/HC_WfnData.h:120-165):
  Slater-type orbitals with occupancies and a core/valence split, the
  deformation-valence exponent and r-powers n_l, anomalous dispersion;
* ``AtomType`` ~ ``HC_AtomTypeParameters``
  (include/discamb/HC_Model/HC_AtomTypeParameters.h:20-60): P_lm, P_val,
  kappa, kappa';
* ``Structure`` ~ ``Crystal`` + ``HC_ModelParameters`` + local coordinate
  systems + the reflection list of one call.

``density_terms`` restates ``sto_atomic_wfn::atomicStoWfnToSphericalDensity``
(src/HC_Model/HC_WfnData.cpp:11-70) and the valence normalisation applied in
``HansenCoppensStructureFactorCalculator::setModel``
(src/Scattering/HansenCoppensStructureFactorCalculator.cpp:187-218).
"""
from __future__ import annotations

from dataclasses import dataclass, field
import math

import numpy as np

from .crystal import SpaceGroup, frac_to_cart_matrix, reciprocal_matrix


@dataclass
class Orbital:
    powers: list          # r powers k_p
    exponents: list       # alpha_p [1/Angstrom]
    coefficients: list    # d_p (already include the STO normalisation)


@dataclass
class Wavefunction:
    label: str
    atomic_number: int
    orbitals: list
    occupancy: list
    core: list            # orbital indices
    valence: list
    def_val_exp: float    # zeta [1/Angstrom]
    def_val_pow: list     # n_l, one per l (length = number of l available)
    anomalous: complex = 0j


@dataclass
class AtomType:
    plm: np.ndarray       # (25,) P_{l,m} at index l*l + (m + l); density normalised
    n_l: int              # number of l levels present (p_lm.size() in the reference)
    p_val: float
    kappa: float
    kappa_prime: float


def density_terms(wfn: Wavefunction, which: str):
    """Spherical density sum_v c_v r^n_v exp(-z_v r) of the core or valence
    orbitals; the valence density is normalised to one electron."""
    idx = wfn.core if which == "core" else wfn.valence
    coeff, expo, powr = [], [], []
    for k in idx:
        occ = float(wfn.occupancy[k])
        if occ == 0.0:
            continue
        orb = wfn.orbitals[k]
        n = len(orb.coefficients)
        for i in range(n):
            for j in range(i + 1):
                c = orb.coefficients[i] * orb.coefficients[j] * occ / (4 * math.pi)
                if i != j:
                    c *= 2
                coeff.append(c)
                expo.append(orb.exponents[i] + orb.exponents[j])
                powr.append(orb.powers[i] + orb.powers[j])
    if which == "valence":
        tot = sum(float(wfn.occupancy[k]) for k in wfn.valence)
        if tot != 0.0:
            coeff = [c / tot for c in coeff]
    return (np.array(coeff, dtype=np.float64), np.array(expo, dtype=np.float64),
            np.array(powr, dtype=np.int32))


@dataclass
class Structure:
    """One crystal + HC model + reflection set + dTarget/dF of one call."""

    cell: tuple
    sg: SpaceGroup
    xyz: np.ndarray            # (n,3) fractional
    adp: list                  # per atom: [] | [Uiso] | [U11..U23] in adp_convention
    occupancy: np.ndarray      # (n,)
    multiplicity: np.ndarray   # (n,) int
    atom_wfn: np.ndarray       # (n,) int
    atom_type: np.ndarray      # (n,) int
    lcs: np.ndarray            # (n,3,3), columns = local x,y,z in Cartesian frame
    wfns: list                 # [Wavefunction]
    types: list                # [AtomType]
    hkl: np.ndarray            # (m,3) int32
    dtdf: np.ndarray           # (m,) complex128
    anomalous: np.ndarray | None = None   # (n,) complex per atom, else per wfn
    include: np.ndarray | None = None     # (n,) bool
    adp_convention: str = "U_cif"
    xyz_convention: str = "fractional"
    name: str = ""

    @property
    def n_atoms(self):
        return len(self.xyz)

    @property
    def n_hkl(self):
        return len(self.hkl)

    def n_adp(self):
        return np.array([len(a) for a in self.adp], dtype=np.int32)

    def adp_array(self):
        out = np.zeros((self.n_atoms, 6))
        for i, a in enumerate(self.adp):
            out[i, :len(a)] = a
        return out

    def include_mask(self):
        if self.include is None:
            return np.ones(self.n_atoms, dtype=bool)
        return np.asarray(self.include, dtype=bool)

    def frac_to_cart(self):
        return frac_to_cart_matrix(self.cell)

    def reciprocal(self):
        return reciprocal_matrix(self.cell)

    def terms(self):
        """atom x symop x hkl terms, symops counted as point-group order
        without centering."""
        return self.n_atoms * self.sg.point_group_order * self.n_hkl
