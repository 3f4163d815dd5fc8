"""ctypes access to the reference library's own CPU path (TEST INFRASTRUCTURE).

``oracle/_ref/libref_driver.so`` is built from the reference sources by
``oracle/Makefile.ref`` where the reference tree exists (it does not exist on
the GPU host).  Used to pin the oracle restatement and to write the golden
fixtures under tests/golden/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_REPO = os.path.dirname(_HERE)
LIB_PATH = os.path.join(_HERE, "_ref", "libref_driver.so")


def _recipe_tree():
    """The reference tree the build recipe names (its ``REF ?=`` line); the
    environment variable DSF_REFERENCE_TREE overrides it."""
    try:
        with open(os.path.join(_HERE, "Makefile.ref")) as fh:
            for line in fh:
                if line.startswith("REF ?="):
                    return line.split("=", 1)[1].strip()
    except OSError:
        pass
    return ""


REF_TREE = os.environ.get("DSF_REFERENCE_TREE") or _recipe_tree()

_lib = None


def available():
    return os.path.exists(LIB_PATH) or os.path.isdir(os.path.join(REF_TREE, "src", "Scattering"))


def build(jobs=8):
    if not REF_TREE or not os.path.isdir(os.path.join(REF_TREE, "src", "Scattering")):
        raise RuntimeError("reference tree not present (set DSF_REFERENCE_TREE to the reference sources)")
    subprocess.check_call(["make", "-s", "-f", "oracle/Makefile.ref", f"REF={REF_TREE}", f"-j{jobs}"],
                          cwd=_REPO)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        # one helper of the reference library refers to a symbol outside the
        # compiled subset; it is never called, so bind lazily
        _lib = C.CDLL(LIB_PATH, mode=os.RTLD_LAZY)
    return _lib


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(C.c_void_p)


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(C.c_void_p)


_ADP_CONV = {"U_cif": 0, "U_cart": 1, "U_star": 2}


class _Conventions:
    """The structure's xyz and ADP conventions for the reference calls made
    inside the block (the crystal the driver builds takes them)."""

    def __init__(self, st):
        self.xyz = 1 if st.xyz_convention == "cartesian" else 0
        self.adp = _ADP_CONV[st.adp_convention]

    def __enter__(self):
        lib().ref_set_conventions(self.xyz, self.adp)

    def __exit__(self, *a):
        lib().ref_set_conventions(0, 0)


def _common(st):
    cell = np.array(st.cell, dtype=np.float64)
    ops = ";".join(st.sg.ops_text).encode()
    adp = st.adp_array()
    return cell, ops, adp


def _outputs(n_hkl, n):
    return dict(f=np.zeros(2 * n_hkl), d_xyz=np.zeros(3 * n), d_adp=np.zeros(6 * n), d_occ=np.zeros(n))


def _pack(out, st, ms):
    n = st.n_atoms
    nadp = st.n_adp()
    d_adp = out["d_adp"].reshape(n, 6)
    return dict(f=out["f"][0::2] + 1j * out["f"][1::2], d_xyz=out["d_xyz"].reshape(n, 3),
                d_adp=[d_adp[i, :nadp[i]].copy() for i in range(n)], d_occ=out["d_occ"], ms=ms)


def hc(st, n_threads=1):
    """HansenCoppensStructureFactorCalculator with the "CPU" engine."""
    keep = []

    def D(a):
        arr, p = _d(a); keep.append(arr); return p

    def I(a):
        arr, p = _i(a); keep.append(arr); return p

    cell, ops, adp = _common(st)
    n = st.n_atoms
    orb_off, orb_occ, orb_core, sto_off, sto_pow, sto_exp, sto_coeff = [0], [], [], [0], [], [], []
    def_exp, def_npow, def_pow, anom, zs = [], [], [], [], []
    for w in st.wfns:
        for k, o in enumerate(w.orbitals):
            orb_occ.append(w.occupancy[k])
            orb_core.append(1 if k in w.core else 0)
            sto_pow += list(o.powers); sto_exp += list(o.exponents); sto_coeff += list(o.coefficients)
            sto_off.append(len(sto_pow))
        orb_off.append(len(orb_occ))
        def_exp.append(w.def_val_exp)
        def_npow.append(len(w.def_val_pow))
        def_pow += list(w.def_val_pow)[:5] + [0] * (5 - min(5, len(w.def_val_pow)))
        anom += [complex(w.anomalous).real, complex(w.anomalous).imag]
        zs.append(w.atomic_number)
    types = st.types
    out = _outputs(st.n_hkl, n)
    ms = C.c_double(0)
    atom_anom = None
    if st.anomalous is not None:
        atom_anom = D(np.stack([np.real(st.anomalous), np.imag(st.anomalous)], axis=1).reshape(-1))
    with _Conventions(st):
        rc = lib().ref_hc_sf(
            D(cell), C.c_char_p(ops), C.c_int(n), D(st.xyz.reshape(-1)), I(st.n_adp()), D(adp.reshape(-1)),
            D(st.occupancy), I(st.multiplicity), I(st.atom_wfn), I(st.atom_type), D(np.asarray(st.lcs).reshape(-1)),
            C.c_int(len(st.wfns)), I(orb_off), I(orb_occ), I(orb_core), I(sto_off), I(sto_pow), D(sto_exp),
            D(sto_coeff), D(def_exp), I(def_npow), I(def_pow), D(anom), I(zs),
            C.c_int(len(types)), I([t.n_l for t in types]), D(np.array([t.plm for t in types]).reshape(-1)),
            D([t.p_val for t in types]), D([t.kappa for t in types]), D([t.kappa_prime for t in types]),
            C.c_int(st.n_hkl), I(st.hkl.reshape(-1)), D(np.stack([st.dtdf.real, st.dtdf.imag], 1).reshape(-1)),
            atom_anom, I(st.include_mask().astype(np.int32)), C.c_int(n_threads),
            D_out(out["f"]), D_out(out["d_xyz"]), D_out(out["d_adp"]), D_out(out["d_occ"]), C.byref(ms))
    if rc != 0:
        raise RuntimeError("reference HC path raised an exception: " + _err())
    return _pack(out, st, ms.value)


def _err():
    f = lib().ref_last_error
    f.restype = C.c_char_p
    return f().decode()


def D_out(a):
    return a.ctypes.data_as(C.c_void_p)


def iam_coefficients(label, table="IT92"):
    a = np.zeros(5); b = np.zeros(5); c = C.c_double(0); n = C.c_int(0)
    rc = lib().ref_iam_coefficients(label.encode(), table.encode(), D_out(a), D_out(b), C.byref(c), C.byref(n))
    if rc != 0:
        raise KeyError(label)
    return a[: n.value].copy(), b[: n.value].copy(), c.value


def iam(st, labels, table="IT92", n_threads=1):
    cell, ops, adp = _common(st)
    n = st.n_atoms
    out = _outputs(st.n_hkl, n)
    ms = C.c_double(0)
    keep = [np.ascontiguousarray(x) for x in (st.xyz.reshape(-1), adp.reshape(-1))]
    xyz, adpf = keep
    nadp = st.n_adp(); mult = np.asarray(st.multiplicity, dtype=np.int32); occ = np.ascontiguousarray(st.occupancy)
    hkl = np.ascontiguousarray(st.hkl.reshape(-1), dtype=np.int32)
    g = np.ascontiguousarray(np.stack([st.dtdf.real, st.dtdf.imag], 1).reshape(-1))
    with _Conventions(st):
        rc = lib().ref_iam_sf(D_out(cell), C.c_char_p(ops), C.c_char_p(";".join(labels).encode()),
                              C.c_char_p(table.encode()), C.c_int(n), D_out(xyz), D_out(nadp), D_out(adpf),
                              D_out(occ), D_out(mult), C.c_int(st.n_hkl), D_out(hkl), D_out(g), C.c_int(n_threads),
                              D_out(out["f"]), D_out(out["d_xyz"]), D_out(out["d_adp"]), D_out(out["d_occ"]),
                              C.byref(ms))
    if rc != 0:
        raise RuntimeError("reference IAM path raised an exception: " + _err())
    return _pack(out, st, ms.value)


def form_factors(st, labels=None, table="IT92"):
    """The reference's single-h calculateFormFactors at every reflection of st:
    complex [n_hkl][n_atoms] (include mask of st).  HC structures through
    HansenCoppensStructureFactorCalculator; with labels, the IAM path of
    AnyIamCalculator with that n-Gaussian table."""
    ff = np.zeros((st.n_hkl, st.n_atoms, 2))
    lib().ref_set_form_factor_out(ff.ctypes.data_as(C.POINTER(C.c_double)))
    try:
        if labels is None:
            hc(st)
        else:
            iam(st, labels, table)
    finally:
        lib().ref_set_form_factor_out(None)
    return ff[..., 0] + 1j * ff[..., 1]


def table(st, keys, values):
    """keys: (k,3) int Miller indices, values: (k, n_atoms) complex.  The
    generic engine builds a default IAM manager from the atom labels before
    the table manager replaces it, so element labels are passed too."""
    labels = ";".join(st.wfns[w].label for w in st.atom_wfn).encode()
    cell, ops, adp = _common(st)
    n = st.n_atoms
    out = _outputs(st.n_hkl, n)
    ms = C.c_double(0)
    xyz = np.ascontiguousarray(st.xyz.reshape(-1)); adpf = np.ascontiguousarray(adp.reshape(-1))
    nadp = st.n_adp(); mult = np.asarray(st.multiplicity, dtype=np.int32); occ = np.ascontiguousarray(st.occupancy)
    hkl = np.ascontiguousarray(st.hkl.reshape(-1), dtype=np.int32)
    g = np.ascontiguousarray(np.stack([st.dtdf.real, st.dtdf.imag], 1).reshape(-1))
    k = np.ascontiguousarray(np.asarray(keys, dtype=np.int32).reshape(-1))
    v = np.ascontiguousarray(np.stack([np.real(values), np.imag(values)], -1).reshape(-1))
    with _Conventions(st):
        rc = lib().ref_table_sf(D_out(cell), C.c_char_p(ops), C.c_char_p(labels), C.c_int(n), D_out(xyz), D_out(nadp), D_out(adpf),
                                D_out(occ), D_out(mult), C.c_int(len(keys)), D_out(k), D_out(v), C.c_int(st.n_hkl),
                                D_out(hkl), D_out(g), D_out(out["f"]), D_out(out["d_xyz"]), D_out(out["d_adp"]),
                                D_out(out["d_occ"]), C.byref(ms))
    if rc != 0:
        raise RuntimeError("reference tabulated path raised an exception: " + _err())
    return _pack(out, st, ms.value)


def tsc_read_seconds(path):
    """The reference's .tsc reader alone (tsc_io::read_tsc) on a file: (scatterers, rows, seconds of the read)."""
    na, nr, sec = C.c_int(0), C.c_int(0), C.c_double(0.0)
    rc = lib().ref_tsc_read(C.c_char_p(os.fsencode(path)), C.byref(na), C.byref(nr), C.byref(sec))
    if rc != 0:
        raise RuntimeError("reference tsc reader raised an exception: " + _err())
    return na.value, nr.value, sec.value


def tsc(st, path):
    """The tabulated path reading a .tsc file with the reference's own reader
    (tsc_io::read_tsc), columns = the structure's atoms in order."""
    labels = ";".join(st.wfns[w].label for w in st.atom_wfn).encode()
    cell, ops, adp = _common(st)
    n = st.n_atoms
    out = _outputs(st.n_hkl, n)
    xyz = np.ascontiguousarray(st.xyz.reshape(-1)); adpf = np.ascontiguousarray(adp.reshape(-1))
    nadp = st.n_adp(); mult = np.asarray(st.multiplicity, dtype=np.int32); occ = np.ascontiguousarray(st.occupancy)
    hkl = np.ascontiguousarray(st.hkl.reshape(-1), dtype=np.int32)
    g = np.ascontiguousarray(np.stack([st.dtdf.real, st.dtdf.imag], 1).reshape(-1))
    with _Conventions(st):
        rc = lib().ref_tsc_sf(C.c_char_p(os.fsencode(path)), D_out(cell), C.c_char_p(ops), C.c_char_p(labels), C.c_int(n),
                              D_out(xyz), D_out(nadp), D_out(adpf), D_out(occ), D_out(mult), C.c_int(st.n_hkl), D_out(hkl),
                              D_out(g), D_out(out["f"]), D_out(out["d_xyz"]), D_out(out["d_adp"]), D_out(out["d_occ"]))
    if rc != 0:
        raise RuntimeError("reference tsc path raised an exception: " + _err())
    return _pack(out, st, 0.0)


def flatten_lcs(defs):
    """XD-style LCS definitions (dicts: central, point1, point2_from, point2_to
    (atom lists; empty = the dummy), dummy (3 fractional positions), axis1,
    axis2 (+-1..3), right) -> (lcs_def [n][7], lcs_atoms, lcs_dummy [n][9])."""
    d, at, du = [], [], []
    for q in defs:
        d.append([q["central"], q["axis1"], q["axis2"], int(q["right"]), len(q["point1"]), len(q["point2_from"]),
                  len(q["point2_to"])])
        at += list(q["point1"]) + list(q["point2_from"]) + list(q["point2_to"])
        du.append(np.asarray(q.get("dummy", np.zeros((3, 3))), dtype=np.float64).reshape(9))
    return (np.array(d, dtype=np.int32), np.array(at + [0], dtype=np.int32), np.array(du, dtype=np.float64))


def anyhc_lcs(st, xyz_moved, defs, n_threads=1):
    """AnyHcCalculator (large-molecule implementation, LCS not frozen) built on
    st's atoms with XD-style local coordinate systems, called with the atoms
    moved to xyz_moved: F and derivatives, and the reference's LCS matrices of
    the moved geometry ([n][3][3], columns = local x, y, z)."""
    keep = []

    def D(a):
        arr, p = _d(a); keep.append(arr); return p

    def I(a):
        arr, p = _i(a); keep.append(arr); return p

    cell, ops, adp = _common(st)
    n = st.n_atoms
    orb_off, orb_occ, orb_core, sto_off, sto_pow, sto_exp, sto_coeff = [0], [], [], [0], [], [], []
    def_exp, def_npow, def_pow, anom, zs = [], [], [], [], []
    for w in st.wfns:
        for k, o in enumerate(w.orbitals):
            orb_occ.append(w.occupancy[k])
            orb_core.append(1 if k in w.core else 0)
            sto_pow += list(o.powers); sto_exp += list(o.exponents); sto_coeff += list(o.coefficients)
            sto_off.append(len(sto_pow))
        orb_off.append(len(orb_occ))
        def_exp.append(w.def_val_exp)
        def_npow.append(len(w.def_val_pow))
        def_pow += list(w.def_val_pow)[:5] + [0] * (5 - min(5, len(w.def_val_pow)))
        anom += [complex(w.anomalous).real, complex(w.anomalous).imag]
        zs.append(w.atomic_number)
    types = st.types
    ld, la, ldu = flatten_lcs(defs)
    out = _outputs(st.n_hkl, n)
    lcs_out = np.zeros(9 * n)
    with _Conventions(st):
        rc = lib().ref_anyhc_lcs(
            D(cell), C.c_char_p(ops), C.c_int(n), D(st.xyz.reshape(-1)), D(np.asarray(xyz_moved).reshape(-1)),
            I(st.n_adp()), D(adp.reshape(-1)), D(st.occupancy), I(st.multiplicity), I(st.atom_wfn), I(st.atom_type),
            I(ld.reshape(-1)), I(la), D(ldu.reshape(-1)),
            C.c_int(len(st.wfns)), I(orb_off), I(orb_occ), I(orb_core), I(sto_off), I(sto_pow), D(sto_exp),
            D(sto_coeff), D(def_exp), I(def_npow), I(def_pow), D(anom), I(zs),
            C.c_int(len(types)), I([t.n_l for t in types]), D(np.array([t.plm for t in types]).reshape(-1)),
            D([t.p_val for t in types]), D([t.kappa for t in types]), D([t.kappa_prime for t in types]),
            C.c_int(st.n_hkl), I(st.hkl.reshape(-1)), D(np.stack([st.dtdf.real, st.dtdf.imag], 1).reshape(-1)),
            C.c_int(n_threads), D_out(out["f"]), D_out(out["d_xyz"]), D_out(out["d_adp"]), D_out(out["d_occ"]),
            D_out(lcs_out))
    if rc != 0:
        raise RuntimeError("reference AnyHcCalculator path raised an exception: " + _err())
    r = _pack(out, st, 0.0)
    r["lcs"] = lcs_out.reshape(n, 3, 3)
    return r


def _hc_arrays(st):
    """The flat HC-model arrays the driver's HC entries take."""
    orb_off, orb_occ, orb_core, sto_off, sto_pow, sto_exp, sto_coeff = [0], [], [], [0], [], [], []
    def_exp, def_npow, def_pow, anom, zs = [], [], [], [], []
    for w in st.wfns:
        for k, o in enumerate(w.orbitals):
            orb_occ.append(w.occupancy[k])
            orb_core.append(1 if k in w.core else 0)
            sto_pow += list(o.powers); sto_exp += list(o.exponents); sto_coeff += list(o.coefficients)
            sto_off.append(len(sto_pow))
        orb_off.append(len(orb_occ))
        def_exp.append(w.def_val_exp)
        def_npow.append(len(w.def_val_pow))
        def_pow += list(w.def_val_pow)[:5] + [0] * (5 - min(5, len(w.def_val_pow)))
        anom += [complex(w.anomalous).real, complex(w.anomalous).imag]
        zs.append(w.atomic_number)
    types = st.types
    return [("i", orb_off), ("i", orb_occ), ("i", orb_core), ("i", sto_off), ("i", sto_pow), ("d", sto_exp),
            ("d", sto_coeff), ("d", def_exp), ("i", def_npow), ("i", def_pow), ("d", anom), ("i", zs),
            ("n", len(types)), ("i", [t.n_l for t in types]), ("d", np.array([t.plm for t in types]).reshape(-1)),
            ("d", [t.p_val for t in types]), ("d", [t.kappa for t in types]), ("d", [t.kappa_prime for t in types])]


def combined(st, hc_atoms, iam_atoms, defs, table="IT92"):
    """CombinedStructureFactorCalculator over an AnyHcCalculator (XD local
    coordinate systems, large-molecule implementation) for hc_atoms and an
    AnyIamCalculator with the named Gaussian table for iam_atoms, both on the
    whole crystal; F and derivatives of the crystal's atoms."""
    keep = []

    def D(a):
        arr, p = _d(a); keep.append(arr); return p

    def I(a):
        arr, p = _i(a); keep.append(arr); return p

    cell, ops, adp = _common(st)
    n = st.n_atoms
    ld, la, ldu = flatten_lcs(defs)
    model = []
    for kind, v in _hc_arrays(st):
        model.append(C.c_int(v) if kind == "n" else (I(v) if kind == "i" else D(v)))
    out = _outputs(st.n_hkl, n)
    with _Conventions(st):
        rc = lib().ref_combined_sf(
            D(cell), C.c_char_p(ops), C.c_int(n), D(st.xyz.reshape(-1)), I(st.n_adp()), D(adp.reshape(-1)),
            D(st.occupancy), I(st.multiplicity), I(st.atom_wfn), I(st.atom_type), I(ld.reshape(-1)), I(la),
            D(ldu.reshape(-1)), C.c_int(len(hc_atoms)), I(hc_atoms), C.c_int(len(iam_atoms)), I(iam_atoms),
            C.c_char_p(table.encode()), C.c_int(len(st.wfns)), *model,
            C.c_int(st.n_hkl), I(st.hkl.reshape(-1)), D(np.stack([st.dtdf.real, st.dtdf.imag], 1).reshape(-1)),
            D_out(out["f"]), D_out(out["d_xyz"]), D_out(out["d_adp"]), D_out(out["d_occ"]))
    if rc != 0:
        raise RuntimeError("reference combined calculator raised an exception: " + _err())
    return _pack(out, st, 0.0)
