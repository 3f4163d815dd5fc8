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

from dataclasses import dataclass, field, replace
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

    def subset(self, idx):
        """The structure of the atoms idx (same cell, symmetry, reflections and
        dT/dF), with its wavefunctions and types renumbered to the ones used."""
        idx = np.asarray(idx, dtype=np.int64)
        used_t = sorted(set(int(t) for t in self.atom_type[idx]))
        used_w = sorted(set(int(w) for w in self.atom_wfn[idx]))
        tmap = {t: i for i, t in enumerate(used_t)}
        wmap = {w: i for i, w in enumerate(used_w)}
        return replace(self, xyz=np.asarray(self.xyz)[idx].copy(), adp=[list(self.adp[i]) for i in idx],
                       occupancy=np.asarray(self.occupancy)[idx].copy(),
                       multiplicity=np.asarray(self.multiplicity)[idx].copy(),
                       atom_wfn=np.array([wmap[int(w)] for w in self.atom_wfn[idx]], dtype=np.int32),
                       atom_type=np.array([tmap[int(t)] for t in self.atom_type[idx]], dtype=np.int32),
                       lcs=np.asarray(self.lcs)[idx].copy(), wfns=[self.wfns[w] for w in used_w],
                       types=[self.types[t] for t in used_t],
                       anomalous=None if self.anomalous is None else np.asarray(self.anomalous)[idx].copy(),
                       include=None if self.include is None else np.asarray(self.include)[idx].copy())

    def frac_to_cart(self):
        return frac_to_cart_matrix(self.cell)

    def reciprocal(self):
        return reciprocal_matrix(self.cell)

    def terms(self):
        """atom x symop x hkl terms, symops counted as point-group order
        without centering."""
        return self.n_atoms * self.sg.point_group_order * self.n_hkl


# ---------------------------------------------------------------------------
# flat-array serialisation (fixtures)
# ---------------------------------------------------------------------------

def structure_to_arrays(st: Structure):
    """All inputs of a Structure as a dict of numpy arrays."""
    out = dict(cell=np.array(st.cell), sg_symbol=np.array(st.sg.symbol), ops="|".join(st.sg.ops_text),
               xyz=st.xyz, adp=st.adp_array(), n_adp=st.n_adp(), occupancy=st.occupancy,
               multiplicity=np.asarray(st.multiplicity), atom_wfn=st.atom_wfn, atom_type=st.atom_type,
               lcs=np.asarray(st.lcs), hkl=st.hkl, dtdf=st.dtdf,
               type_plm=np.array([t.plm for t in st.types]), type_nl=np.array([t.n_l for t in st.types]),
               type_pval=np.array([t.p_val for t in st.types]), type_kappa=np.array([t.kappa for t in st.types]),
               type_kappa_p=np.array([t.kappa_prime for t in st.types]),
               adp_convention=np.array(st.adp_convention), xyz_convention=np.array(st.xyz_convention))
    if st.anomalous is not None:
        out["anomalous"] = np.asarray(st.anomalous)
    if st.include is not None:
        out["include"] = np.asarray(st.include)
    # wavefunctions: orbitals flattened
    wl, wz, wdef, wdpow, wan = [], [], [], [], []
    orb_w, orb_occ, orb_core, sto_o, sto_pow, sto_exp, sto_c = [], [], [], [], [], [], []
    for wi, w in enumerate(st.wfns):
        wl.append(w.label); wz.append(w.atomic_number); wdef.append(w.def_val_exp)
        wdpow.append(list(w.def_val_pow) + [-1] * (5 - len(w.def_val_pow))); wan.append(complex(w.anomalous))
        for k, o in enumerate(w.orbitals):
            oi = len(orb_w)
            orb_w.append(wi); orb_occ.append(w.occupancy[k]); orb_core.append(1 if k in w.core else 0)
            for p_, e_, c_ in zip(o.powers, o.exponents, o.coefficients):
                sto_o.append(oi); sto_pow.append(p_); sto_exp.append(e_); sto_c.append(c_)
    out.update(wfn_label=np.array(wl), wfn_z=np.array(wz), wfn_def_exp=np.array(wdef), wfn_def_pow=np.array(wdpow),
               wfn_anom=np.array(wan), orb_wfn=np.array(orb_w), orb_occ=np.array(orb_occ),
               orb_core=np.array(orb_core), sto_orb=np.array(sto_o), sto_pow=np.array(sto_pow),
               sto_exp=np.array(sto_exp), sto_coeff=np.array(sto_c))
    out["ops"] = np.array(out["ops"])
    out["name"] = np.array(st.name)
    return out


def structure_from_arrays(d):
    from .crystal import SpaceGroup
    ops = str(d["ops"]).split("|")
    sg = SpaceGroup(str(d["sg_symbol"]), ops)
    wfns = []
    for wi in range(len(d["wfn_label"])):
        orbitals, occ, core, val = [], [], [], []
        for oi in np.nonzero(d["orb_wfn"] == wi)[0]:
            sel = d["sto_orb"] == oi
            orbitals.append(Orbital([int(v) for v in d["sto_pow"][sel]], [float(v) for v in d["sto_exp"][sel]],
                                    [float(v) for v in d["sto_coeff"][sel]]))
            occ.append(int(d["orb_occ"][oi]))
            (core if d["orb_core"][oi] else val).append(len(orbitals) - 1)
        dp = [int(v) for v in d["wfn_def_pow"][wi] if v >= 0]
        wfns.append(Wavefunction(str(d["wfn_label"][wi]), int(d["wfn_z"][wi]), orbitals, occ, core, val,
                                 float(d["wfn_def_exp"][wi]), dp, complex(d["wfn_anom"][wi])))
    types = [AtomType(np.array(d["type_plm"][t]), int(d["type_nl"][t]), float(d["type_pval"][t]),
                      float(d["type_kappa"][t]), float(d["type_kappa_p"][t])) for t in range(len(d["type_nl"]))]
    n_adp = d["n_adp"]
    adp = [list(d["adp"][i, :n_adp[i]]) for i in range(len(n_adp))]
    return Structure(cell=tuple(float(v) for v in d["cell"]), sg=sg, xyz=np.array(d["xyz"]), adp=adp,
                     occupancy=np.array(d["occupancy"]), multiplicity=np.array(d["multiplicity"]),
                     atom_wfn=np.array(d["atom_wfn"]), atom_type=np.array(d["atom_type"]), lcs=np.array(d["lcs"]),
                     wfns=wfns, types=types, hkl=np.array(d["hkl"], dtype=np.int32), dtdf=np.array(d["dtdf"]),
                     anomalous=np.array(d["anomalous"]) if "anomalous" in d else None,
                     include=np.array(d["include"]) if "include" in d else None,
                     adp_convention=str(d["adp_convention"]), xyz_convention=str(d["xyz_convention"]),
                     name=str(d["name"]))
