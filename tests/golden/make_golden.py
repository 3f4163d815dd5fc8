"""Writes the golden fixtures of tests/golden/ by running the reference
library's own CPU code (oracle/_ref/libref_driver.so, built from the
reference sources by oracle/Makefile.ref) on seeded synthetic structures.

    python tests/golden/make_golden.py [hc|centering|conventions|lcs|combined|def_val_symm|form_factors|rest ...]
                                                                                  (default: all)

Each fixture (.npz) holds every input of the case (structure_to_arrays) and
the reference outputs: F, d_xyz, d_adp, d_occ in the crystal's conventions.
The multipole fixture adds dT/dP_val, dT/dP_lm, dT/dkappa, dT/dkappa' by
central finite differences of the reference F (F is linear in P_val and
P_lm, so one step is exact to rounding; kappa and kappa' use Richardson
extrapolation over steps h and h/2), because the reference computes no
analytic derivatives for those parameters.
"""
from __future__ import annotations

import copy
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from discamb_gb300 import workloads as W  # noqa: E402
from discamb_gb300.model import structure_to_arrays  # noqa: E402
from oracle import ref as R  # noqa: E402


def hc_cases():
    cases = []
    for i, sg in enumerate(["P1", "P-1", "P21", "P21/c", "P212121", "C2/c", "P43212", "P-1(shift)", "I2/m-like",
                            "P41", "Pbca"]):
        st = W.small_case(sg, n_atoms=5, stol_max=0.55, seed=100 + i, improper_lcs=True)
        cases.append((f"hc_{sg.replace('/', '_').replace('(', '_').replace(')', '')}", st))
    st = W.config0(seed=0)
    cases.append(("hc_config0", st))
    # per-atom anomalous dispersion, an excluded atom, occupancies below one
    st = W.small_case("P21/c", n_atoms=6, stol_max=0.5, seed=201, anomalous_per_atom=True, occupancy=(0.6, 1.0))
    st.include = np.array([1, 1, 0, 1, 1, 1], dtype=bool)
    cases.append(("hc_anomalous_mask", st))
    # isotropic-only, special-position multiplicity, one reflection list with 000
    st = W.small_case("P212121", n_atoms=4, stol_max=0.5, seed=202, aniso=False)
    st.multiplicity = np.array([4, 2, 4, 1], dtype=np.int32)
    st.hkl = np.concatenate([np.zeros((1, 3), dtype=np.int32), st.hkl])
    st.dtdf = np.concatenate([[0.3 - 0.7j], st.dtdf])
    cases.append(("hc_iso_special_000", st))
    # dipole/quadrupole-along-z types only (the engine's pz/dz path)
    st = W.small_case("P-1", n_atoms=4, stol_max=0.5, seed=203, l_max=2)
    for t in st.types:
        t.plm[:] = 0.0
        t.plm[2] = 0.07
        t.plm[6] = -0.03
        t.n_l = 3
    cases.append(("hc_pz_dz", st))
    return cases


def run_hc(name, st):
    r = R.hc(st, n_threads=4)
    out = structure_to_arrays(st)
    nadp = st.n_adp()
    d_adp = np.zeros((st.n_atoms, 6))
    for i, v in enumerate(r["d_adp"]):
        d_adp[i, :nadp[i]] = v
    out.update(ref_f=r["f"], ref_d_xyz=r["d_xyz"], ref_d_adp=d_adp, ref_d_occ=r["d_occ"])
    return out


def target(st):
    r = R.hc(st, n_threads=4)
    return float(np.sum((np.conj(st.dtdf) * r["f"]).real))


def multipole_fd(st):
    """dT/dparam of every type parameter by finite differences of the
    reference F; one type per atom, so these are the per-atom derivatives."""
    n = st.n_atoms
    d_pval, d_kappa, d_kappa_p = np.zeros(n), np.zeros(n), np.zeros(n)
    d_plm = np.zeros((n, 25))

    def diff(mod, h):
        s1 = copy.deepcopy(st); mod(s1, +h)
        s2 = copy.deepcopy(st); mod(s2, -h)
        return (target(s1) - target(s2)) / (2 * h)

    for a in range(n):
        t = st.atom_type[a]

        def set_attr(name):
            def f(s, h):
                setattr(s.types[t], name, getattr(s.types[t], name) + h)
            return f
        d_pval[a] = diff(set_attr("p_val"), 1e-2)
        for name, arr in (("kappa", d_kappa), ("kappa_prime", d_kappa_p)):
            h = 1e-3
            d1 = diff(set_attr(name), h)
            d2 = diff(set_attr(name), h / 2)
            arr[a] = (4 * d2 - d1) / 3
        for q in range(st.types[t].n_l ** 2):
            def fq(s, h, q=q):
                s.types[t].plm[q] += h
            d_plm[a, q] = diff(fq, 1e-2)
    return d_pval, d_plm, d_kappa, d_kappa_p


def write_hc():
    for name, st in hc_cases():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **run_hc(name, st))
        print("wrote", name, st.n_atoms, st.n_hkl)


def write_def_val_symm():
    """The reference's point-group-symmetrised deformation valence engine
    (HansenCoppens_SF_EngineSymm, selected by set_def_val_symm): the same
    structure factors as Engine3, computed per point group (a closed form for
    222, a z-axis shortcut for dipole/quadrupole-only atoms)."""
    for i, sg in enumerate(["P212121", "P21/c", "P43212", "Pbca"]):
        st = W.small_case(sg, n_atoms=5, stol_max=0.55, seed=700 + i, improper_lcs=True)
        if sg == "P212121":  # one dipole/quadrupole-along-z type (the engine's pz/dz branch)
            t = st.types[st.atom_type[0]]
            t.plm[:] = 0.0
            t.plm[2] = 0.05
            t.plm[6] = -0.04
            t.n_l = 3
        name = "dvs_hc_" + sg.replace("/", "_").lower()
        R.lib().ref_set_def_val_symm(1)
        try:
            out = run_hc(name, st)
        finally:
            R.lib().ref_set_def_val_symm(0)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("wrote", name, st.n_atoms, st.n_hkl)


def write_rest():
    # multipole-parameter derivatives
    st = W.small_case("P21/c", n_atoms=3, stol_max=0.45, seed=301)
    out = run_hc("hc_multipole_fd", st)
    d_pval, d_plm, d_k, d_kp = multipole_fd(st)
    out.update(ref_d_pval=d_pval, ref_d_plm=d_plm, ref_d_kappa=d_k, ref_d_kappa_p=d_kp)
    np.savez_compressed(os.path.join(HERE, "hc_multipole_fd.npz"), **out)
    print("wrote hc_multipole_fd")
    # electron scattering (Mott-Bethe inside the engine), F(000) included; f_e(0) per wavefunction from the
    # reference's "electron-IT" table
    for name, sg, seed in (("el_hc_p21c", "P21/c", 501), ("el_hc_p212121", "P212121", 502)):
        st = W.small_case(sg, n_atoms=6, stol_max=0.55, seed=seed, anomalous_per_atom=(seed == 502))
        st.hkl = np.concatenate([np.zeros((1, 3), dtype=np.int32), st.hkl])
        st.dtdf = np.concatenate([[0.4 + 0.2j], st.dtdf])
        f000 = []
        for w in st.wfns:
            a, b, c = R.iam_coefficients(w.label, "electron-IT")
            f000.append(float(np.sum(a) + c))
        R.lib().ref_set_electron(1)
        try:
            out = run_hc(name, st)
        finally:
            R.lib().ref_set_electron(0)
        out.update(electron_f000=np.array(f000))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("wrote", name, st.n_atoms, st.n_hkl)
    # a .tsc file read by the reference's own reader (tsc_io::read_tsc), expanded h' set of all operations
    import tempfile
    from discamb_gb300 import api as A
    st = W.small_case("P21/c", n_atoms=5, stol_max=0.5, seed=601)
    rot, _ = A.all_ops_mod_centering(st.sg)
    keys = sorted({tuple(int(v) for v in h @ r_) for h in st.hkl for r_ in rot})
    rng = np.random.default_rng(602)
    vals = rng.normal(size=(len(keys), st.n_atoms)) + 1j * rng.normal(size=(len(keys), st.n_atoms))
    labels = [f"{st.wfns[w].label}{i + 1}" for i, w in enumerate(st.atom_wfn)]
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "form_factors.tsc")
        A.write_tsc(path, labels, np.array(keys), vals)
        r = R.tsc(st, path)
    out = structure_to_arrays(st)
    nadp = st.n_adp()
    d_adp = np.zeros((st.n_atoms, 6))
    for i, v in enumerate(r["d_adp"]):
        d_adp[i, :nadp[i]] = v
    out.update(tsc_keys=np.array(keys, dtype=np.int32), tsc_values=vals, tsc_labels=np.array(labels),
               ref_f=r["f"], ref_d_xyz=r["d_xyz"], ref_d_adp=d_adp, ref_d_occ=r["d_occ"])
    np.savez_compressed(os.path.join(HERE, "tsc_p21c.npz"), **out)
    print("wrote tsc_p21c", st.n_atoms, st.n_hkl, len(keys))
    # IAM with the reference's IT92 Gaussian table
    st = W.small_case("C2/c", n_atoms=6, stol_max=0.6, seed=401)
    labels = [w.label for w in st.wfns]
    labels_atoms = [st.wfns[w].label for w in st.atom_wfn]
    ng, ga, gb, gc = [], np.zeros((len(labels), 5)), np.zeros((len(labels), 5)), []
    for i, lab in enumerate(labels):
        a, b, c = R.iam_coefficients(lab, "IT92")
        ng.append(len(a)); ga[i, :len(a)] = a; gb[i, :len(b)] = b; gc.append(c)
    st.atom_type = st.atom_wfn.copy()
    r = R.iam(st, labels_atoms, "IT92")
    out = structure_to_arrays(st)
    d_adp = np.zeros((st.n_atoms, 6))
    for i, v in enumerate(r["d_adp"]):
        d_adp[i, :len(v)] = v
    out.update(iam_ngauss=np.array(ng), iam_a=ga, iam_b=gb, iam_c=np.array(gc), ref_f=r["f"], ref_d_xyz=r["d_xyz"],
               ref_d_adp=d_adp, ref_d_occ=r["d_occ"])
    np.savez_compressed(os.path.join(HERE, "iam_it92.npz"), **out)
    print("wrote iam_it92")
    # tabulated form factors: one complex f per (atom, rotated index)
    st = W.small_case("P21/c", n_atoms=4, stol_max=0.5, seed=501)
    rng = np.random.default_rng(502)
    keys = {}
    for h in st.hkl:
        for r_ in st.sg.rot:
            hp = tuple(int(v) for v in (h @ r_))
            if hp not in keys:
                keys[hp] = (rng.normal(2, 1, st.n_atoms) + 1j * rng.normal(0, 0.3, st.n_atoms))
    kk = np.array(list(keys.keys()), dtype=np.int32)
    vv = np.array(list(keys.values()))
    r = R.table(st, kk, vv)
    out = structure_to_arrays(st)
    d_adp = np.zeros((st.n_atoms, 6))
    for i, v in enumerate(r["d_adp"]):
        d_adp[i, :len(v)] = v
    out.update(table_keys=kk, table_values=vv, ref_f=r["f"], ref_d_xyz=r["d_xyz"], ref_d_adp=d_adp,
               ref_d_occ=r["d_occ"])
    np.savez_compressed(os.path.join(HERE, "table_p21c.npz"), **out)
    print("wrote table_p21c")


def write_form_factors():
    """The reference's single-h calculateFormFactors (no anomalous dispersion,
    0 for excluded atoms) at every reflection of a small HC structure (000
    included) and of an IAM structure (IT92)."""
    st = W.small_case("P21/c", n_atoms=5, stol_max=0.5, seed=801, improper_lcs=True)
    st.hkl = np.concatenate([np.zeros((1, 3), dtype=np.int32), st.hkl[:40]])
    st.dtdf = np.concatenate([[1.0 + 0j], st.dtdf[:40]])
    st.include = np.array([1, 1, 0, 1, 1], dtype=bool)
    out = structure_to_arrays(st)
    out.update(ref_ff=R.form_factors(st))
    np.savez_compressed(os.path.join(HERE, "ff_hc_p21c.npz"), **out)
    print("wrote ff_hc_p21c", st.n_atoms, st.n_hkl)
    st = W.small_case("C2/c", n_atoms=6, stol_max=0.6, seed=802)
    st.hkl, st.dtdf = st.hkl[:40], st.dtdf[:40]
    labels = [w.label for w in st.wfns]
    ng, ga, gb, gc = [], np.zeros((len(labels), 5)), np.zeros((len(labels), 5)), []
    for i, lab in enumerate(labels):
        a_, b_, c_ = R.iam_coefficients(lab, "IT92")
        ng.append(len(a_)); ga[i, :len(a_)] = a_; gb[i, :len(b_)] = b_; gc.append(c_)
    st.atom_type = st.atom_wfn.copy()
    out = structure_to_arrays(st)
    out.update(iam_ngauss=np.array(ng), iam_a=ga, iam_b=gb, iam_c=np.array(gc),
               ref_ff=R.form_factors(st, labels=[st.wfns[w].label for w in st.atom_wfn]))
    np.savez_compressed(os.path.join(HERE, "ff_iam_c2c.npz"), **out)
    print("wrote ff_iam_c2c", st.n_atoms, st.n_hkl)


def _with_absences(st, stol_max, seed):
    """The structure's reflections replaced by every unique reflection up to
    stol_max, lattice-centering absences included (the reference multiplies
    those by 0), with a fresh seeded dT/dF."""
    from discamb_gb300.crystal import unique_hkl
    st.hkl = unique_hkl(st.cell, st.sg, stol_max=stol_max, drop_absent=False)
    rng = np.random.default_rng(seed)
    st.dtdf = rng.normal(size=st.n_hkl) + 1j * rng.normal(size=st.n_hkl)
    return st


def write_centering():
    """Rhombohedral (obverse R-3, reverse R3) and face-centred (Fdd2) lattices
    through the reference's HC engine, absences included: pins
    centeringSfMultipliers (scattering_utilities.cpp:103-170), whose reverse
    setting tests (h - k + l) mod 2."""
    for i, sg in enumerate(["R-3", "R3(reverse)", "Fdd2"]):
        st = W.small_case(sg, n_atoms=4, stol_max=0.5, seed=900 + i, improper_lcs=True)
        st = _with_absences(st, 0.5, 950 + i)
        name = "hc_" + sg.replace("(", "_").replace(")", "")
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **run_hc(name, st))
        print("wrote", name, st.n_atoms, st.n_hkl)


def to_conventions(st, xyz, adp):
    """st with its positions and ADPs rewritten in the given conventions
    (xyz "fractional" / "cartesian"; adp "U_cif" / "U_cart" / "U_star";
    isotropic U unchanged)."""
    from discamb_gb300.crystal import convert_adp, frac_to_cart_matrix
    if xyz == "cartesian":
        st.xyz = (frac_to_cart_matrix(st.cell) @ st.xyz.T).T.copy()
    st.adp = [list(convert_adp(st.cell, a, "U_cif", adp)) if len(a) == 6 else list(a) for a in st.adp]
    st.xyz_convention, st.adp_convention = xyz, adp
    return st


def write_conventions():
    """The crystal's xyz and ADP conventions other than fractional / U_cif:
    the reference reads the atoms in them and returns the derivatives in them
    (HansenCoppensStructureFactorCalculator.cpp:69-70, 634-664;
    StructuralParametersConverter.h:90-112).  HC: Cartesian + U_cart (P2_1/c),
    fractional + U_star (P-1), Cartesian + U_cif (P2_1 2_1 2_1); IAM (generic
    engine): Cartesian + U_star (C2/c)."""
    for i, (sg, xyz, adp) in enumerate([("P21/c", "cartesian", "U_cart"), ("P-1", "fractional", "U_star"),
                                         ("P212121", "cartesian", "U_cif")]):
        st = W.small_case(sg, n_atoms=5, stol_max=0.5, seed=1000 + i, improper_lcs=True)
        st = to_conventions(st, xyz, adp)
        name = f"hc_conv_{sg.replace('/', '_')}_{xyz[:4]}_{adp}"
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **run_hc(name, st))
        print("wrote", name, st.n_atoms, st.n_hkl)
    st = W.small_case("C2/c", n_atoms=6, stol_max=0.55, seed=1010)
    labels = [w.label for w in st.wfns]
    ng, ga, gb, gc = [], np.zeros((len(labels), 5)), np.zeros((len(labels), 5)), []
    for i, lab in enumerate(labels):
        a, b, c = R.iam_coefficients(lab, "IT92")
        ng.append(len(a)); ga[i, :len(a)] = a; gb[i, :len(b)] = b; gc.append(c)
    st.atom_type = st.atom_wfn.copy()
    st = to_conventions(st, "cartesian", "U_star")
    r = R.iam(st, [st.wfns[w].label for w in st.atom_wfn], "IT92")
    out = structure_to_arrays(st)
    d_adp = np.zeros((st.n_atoms, 6))
    for i, v in enumerate(r["d_adp"]):
        d_adp[i, :len(v)] = v
    out.update(iam_ngauss=np.array(ng), iam_a=ga, iam_b=gb, iam_c=np.array(gc), ref_f=r["f"], ref_d_xyz=r["d_xyz"],
               ref_d_adp=d_adp, ref_d_occ=r["d_occ"])
    np.savez_compressed(os.path.join(HERE, "iam_conv_c2c_cart_U_star.npz"), **out)
    print("wrote iam_conv_c2c_cart_U_star", st.n_atoms, st.n_hkl)


def lcs_definitions(n, rng):
    """XD-style local coordinate systems for n >= 4 atoms, one per atom: Z (or
    another axis) towards a neighbour, the second axis from a third pair; one
    left-handed system, one point given by two atoms (the reference sums
    their positions) and one by a dummy position."""
    axes = [(3, 1), (1, 2), (-3, 1), (2, -3), (3, -2), (-1, 3)]
    defs = []
    for a in range(n):
        a1, a2 = axes[a % len(axes)]
        q = dict(central=a, point1=[(a + 1) % n], point2_from=[a], point2_to=[(a + 2) % n], axis1=a1, axis2=a2,
                 right=True, dummy=np.zeros((3, 3)))
        defs.append(q)
    defs[1]["right"] = False
    defs[2]["point2_to"] = [(2 + 2) % n, (2 + 3) % n]
    defs[3]["point1"] = []
    defs[3]["dummy"] = np.array([[0.31, 0.62, 0.12], [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]]) + rng.uniform(0, 0.05, (3, 3))
    return defs


def write_lcs():
    """AnyHcCalculator with XD local coordinate systems that are not frozen
    (large-molecule implementation): the calculator is set up on one geometry
    and called with the atoms moved (sigma 0.05 A), so the reference
    recomputes every LCS from the moved atoms before its engine runs
    (AnyHcCalculator.cpp:236-244, 319-329).  The fixture holds both
    geometries, the definitions, the reference's LCS matrices of each
    geometry and the results of the call with the moved atoms."""
    for name, sg, xyz_conv in (("lcs_update_p21c", "P21/c", "fractional"), ("lcs_update_p1_cart", "P1", "cartesian")):
        st = W.small_case(sg, n_atoms=6, stol_max=0.5, seed=1100 + len(name))
        rng = np.random.default_rng(1150 + len(name))
        if xyz_conv == "cartesian":
            st = to_conventions(st, "cartesian", "U_cif")
            moved = st.xyz + rng.normal(scale=0.05, size=st.xyz.shape)
        else:
            from discamb_gb300.crystal import frac_to_cart_matrix
            minv = np.linalg.inv(frac_to_cart_matrix(st.cell))
            moved = st.xyz + (minv @ rng.normal(scale=0.05, size=st.xyz.shape).T).T
        defs = lcs_definitions(st.n_atoms, rng)
        r0 = R.anyhc_lcs(st, st.xyz, defs)  # the set-up geometry: its LCS become st.lcs
        st.lcs = r0["lcs"]
        r = R.anyhc_lcs(st, moved, defs)
        out = structure_to_arrays(st)
        nadp = st.n_adp()
        d_adp = np.zeros((st.n_atoms, 6))
        for i, v in enumerate(r["d_adp"]):
            d_adp[i, :nadp[i]] = v
        ld, la, ldu = R.flatten_lcs(defs)
        out.update(xyz_moved=moved, lcs_def=ld, lcs_atoms=la, lcs_dummy=ldu, ref_lcs_moved=r["lcs"],
                   ref_f=r["f"], ref_d_xyz=r["d_xyz"], ref_d_adp=d_adp, ref_d_occ=r["d_occ"])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("wrote", name, st.n_atoms, st.n_hkl)


def write_combined():
    """The reference's CombinedStructureFactorCalculator with TAAM's split
    (HcAtomBankStructureFactorCalculator.cpp:482-499): the non-H atoms on an
    AnyHcCalculator (XD local coordinate systems), the H atoms on an
    AnyIamCalculator with the IT92 table.  The combined calculator zeroes the
    anomalous dispersion of its parts when it is built.  The fixture adds the
    atom lists, the IT92 coefficients per wavefunction (element) and the
    reference's LCS matrices."""
    st = W.small_case("P21/c", n_atoms=9, stol_max=0.5, seed=1300, improper_lcs=True)
    rng = np.random.default_rng(1301)
    defs = lcs_definitions(st.n_atoms, rng)
    st.lcs = R.anyhc_lcs(st, st.xyz, defs)["lcs"]
    labels = [st.wfns[w].label for w in st.atom_wfn]
    hc_atoms = np.array([i for i, e in enumerate(labels) if e != "H"], dtype=np.int32)
    iam_atoms = np.array([i for i, e in enumerate(labels) if e == "H"], dtype=np.int32)
    r = R.combined(st, hc_atoms, iam_atoms, defs, "IT92")
    ng, ga, gb, gc = [], np.zeros((len(st.wfns), 5)), np.zeros((len(st.wfns), 5)), []
    for i, w in enumerate(st.wfns):
        a, b, c = R.iam_coefficients(w.label, "IT92")
        ng.append(len(a)); ga[i, :len(a)] = a; gb[i, :len(b)] = b; gc.append(c)
    out = structure_to_arrays(st)
    nadp = st.n_adp()
    d_adp = np.zeros((st.n_atoms, 6))
    for i, v in enumerate(r["d_adp"]):
        d_adp[i, :nadp[i]] = v
    ld, la, ldu = R.flatten_lcs(defs)
    out.update(hc_atoms=hc_atoms, iam_atoms=iam_atoms, wfn_iam_ngauss=np.array(ng), wfn_iam_a=ga, wfn_iam_b=gb,
               wfn_iam_c=np.array(gc), lcs_def=ld, lcs_atoms=la, lcs_dummy=ldu,
               ref_f=r["f"], ref_d_xyz=r["d_xyz"], ref_d_adp=d_adp, ref_d_occ=r["d_occ"])
    np.savez_compressed(os.path.join(HERE, "combined_taam_p21c.npz"), **out)
    print("wrote combined_taam_p21c", st.n_atoms, st.n_hkl, len(hc_atoms), len(iam_atoms))


GROUPS = {"hc": write_hc, "lcs": write_lcs, "combined": write_combined, "centering": write_centering, "conventions": write_conventions, "def_val_symm": write_def_val_symm, "form_factors": write_form_factors,
          "rest": write_rest}


def main(groups):
    os.makedirs(HERE, exist_ok=True)
    for g in groups or list(GROUPS):
        GROUPS[g]()


if __name__ == "__main__":
    main(sys.argv[1:])
