"""Python driver of the CPU oracle (TEST INFRASTRUCTURE).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, as the checker.  It restates the API-level
wrapper of the reference engine around the C core in ``sf_oracle.c``:

* ``HansenCoppensStructureFactorCalculator::calculateStructureFactorsAnd
  Derivatives`` (src/Scattering/HansenCoppensStructureFactorCalculator.cpp:
  380-508): dT/dF conjugated and multiplied by the centering factor, F
  multiplied by it afterwards;
* ``prepareDataForEngine_part`` (same file :897-990): fractional -> Cartesian
  positions, U_cif -> U_cart * 2 pi^2, Cartesian reflection vectors;
* ``setEngineSpecificSpaceGroupRepresentation`` (same file :107-155):
  Cartesian symmetry subset;
* ``convertDerivatives`` (same file :634-664): derivatives back to the
  crystal's conventions;
* the all-operations set-up of ``AnyScattererStructureFactorCalculator``
  (src/Scattering/AnyScattererStructureFactorCalculator.cpp:28-66) for the
  IAM and tabulated models.
"""
from __future__ import annotations

import ctypes as C
import os
import time
import subprocess
import math

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboracle_sf.so")

_P = C.POINTER


class _Problem(C.Structure):
    _fields_ = [
        ("model", C.c_int),
        ("n_wfn", C.c_int),
        ("core_off", _P(C.c_int)), ("core_coeff", _P(C.c_double)), ("core_exp", _P(C.c_double)),
        ("core_pow", _P(C.c_int)),
        ("val_off", _P(C.c_int)), ("val_coeff", _P(C.c_double)), ("val_exp", _P(C.c_double)),
        ("val_pow", _P(C.c_int)),
        ("def_exp", _P(C.c_double)), ("def_npow", _P(C.c_int)), ("def_pow", _P(C.c_int)),
        ("wfn_anom", _P(C.c_double)),
        ("n_types", C.c_int),
        ("type_nl", _P(C.c_int)), ("type_plm", _P(C.c_double)),
        ("type_pval", _P(C.c_double)), ("type_kappa", _P(C.c_double)), ("type_kappa_p", _P(C.c_double)),
        ("iam_ngauss", _P(C.c_int)), ("iam_a", _P(C.c_double)), ("iam_b", _P(C.c_double)),
        ("iam_c", _P(C.c_double)),
        ("table", _P(C.c_double)),
        ("n_atoms", C.c_int),
        ("atom_wfn", _P(C.c_int)), ("atom_type", _P(C.c_int)),
        ("pos", _P(C.c_double)), ("n_adp", _P(C.c_int)), ("adp", _P(C.c_double)),
        ("occ", _P(C.c_double)), ("mult_w", _P(C.c_double)), ("lcs", _P(C.c_double)),
        ("atom_anom", _P(C.c_double)), ("include", _P(C.c_int)),
        ("n_sym", C.c_int), ("rot", _P(C.c_double)), ("trans", _P(C.c_double)),
        ("centro", C.c_int), ("inv_trans", C.c_double * 3),
        ("n_hkl", C.c_int), ("h", _P(C.c_double)), ("dtdf", _P(C.c_double)),
        ("d_xyz", C.c_int), ("d_adp", C.c_int), ("d_occ", C.c_int), ("d_mp", C.c_int),
        ("electron", C.c_int), ("wfn_z", _P(C.c_int)), ("wfn_f000", _P(C.c_double)),
    ]


class _Result(C.Structure):
    _fields_ = [(n, _P(C.c_double)) for n in
                ("f", "d_xyz", "d_adp", "d_occ", "d_pval", "d_plm", "d_kappa", "d_kappa_p")]


def build(force=False, verbose=False):
    src = os.path.join(_HERE, "sf_oracle.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", LIB_PATH, src, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        _lib.sfo_compute.argtypes = [_P(_Problem), _P(_Result), C.c_int]
        _lib.sfo_compute.restype = C.c_int
        _lib.sfo_compute_lines.argtypes = [_P(_Problem), _P(C.c_int), _P(C.c_double), _P(_Result), C.c_int]
        _lib.sfo_compute_lines.restype = C.c_int
        _lib.sfo_g.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double]
        _lib.sfo_g.restype = C.c_double
        _lib.sfo_dlm.argtypes = [_P(C.c_double), _P(C.c_double)]
        _lib.sfo_form_factors.argtypes = [_P(_Problem), _P(C.c_double), _P(C.c_double)]
        _lib.sfo_form_factors.restype = C.c_int
    return _lib


def g_function(l, n, h, z):
    return lib().sfo_g(l, n, h, z)


def dlm(u):
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.zeros(25)
    lib().sfo_dlm(u.ctypes.data_as(_P(C.c_double)), out.ctypes.data_as(_P(C.c_double)))
    return out


def _ptr(a, ct):
    return a.ctypes.data_as(_P(ct))


class _Keep:
    """keeps numpy buffers alive while the C call runs"""

    def __init__(self):
        self.items = []

    def d(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.items.append(a)
        return _ptr(a, C.c_double)

    def i(self, a):
        a = np.ascontiguousarray(a, dtype=np.int32)
        self.items.append(a)
        return _ptr(a, C.c_int)


def hc_model_arrays(st):
    """CSR arrays of the wavefunction density terms and the type table."""
    from discamb_gb300.model import density_terms
    core_off, val_off = [0], [0]
    cc, ce, cp, vc, ve, vp = [], [], [], [], [], []
    def_exp, def_npow, def_pow, anom = [], [], [], []
    for w in st.wfns:
        c, e, p = density_terms(w, "core")
        cc += list(c); ce += list(e); cp += list(p); core_off.append(len(cc))
        c, e, p = density_terms(w, "valence")
        vc += list(c); ve += list(e); vp += list(p); val_off.append(len(vc))
        def_exp.append(w.def_val_exp)
        def_npow.append(len(w.def_val_pow))
        dp = list(w.def_val_pow)[:5] + [0] * (5 - min(5, len(w.def_val_pow)))
        def_pow += dp
        anom += [complex(w.anomalous).real, complex(w.anomalous).imag]
    types = st.types
    return dict(
        core_off=np.array(core_off), core_coeff=np.array(cc + [0.0]), core_exp=np.array(ce + [1.0]),
        core_pow=np.array(cp + [0]), val_off=np.array(val_off), val_coeff=np.array(vc + [0.0]),
        val_exp=np.array(ve + [1.0]), val_pow=np.array(vp + [0]), def_exp=np.array(def_exp),
        def_npow=np.array(def_npow), def_pow=np.array(def_pow), wfn_anom=np.array(anom),
        type_nl=np.array([t.n_l for t in types]),
        type_plm=np.array([t.plm for t in types]).reshape(-1),
        type_pval=np.array([t.p_val for t in types]),
        type_kappa=np.array([t.kappa for t in types]),
        type_kappa_p=np.array([t.kappa_prime for t in types]))


def compute(st, model="hc", n_threads=None, derivatives=("xyz", "adp", "occ"), multipoles=False,
            iam=None, table=None, hkl_subset=None, loop="direct", electron_f000=None, form_factors=False):
    """F and dT/dparam for a Structure at the API level (crystal conventions).

    model: 'hc' (HansenCoppens engine: symmetry subset, inversion and
    centering handled by the engine) or 'iam' / 'table' (generic engine over
    all operations).  ``iam`` = dict(ngauss, a, b, c) per type; ``table`` =
    complex array [hkl][op][atom] over all operations.
    Returns dict with f (complex), d_xyz, d_adp, d_occ and, with multipoles,
    d_pval, d_plm, d_kappa, d_kappa_p.
    loop: 'direct' (every term evaluated directly) or, for the HC model,
    'lines' (the reference engine's line-ordered loop with recurrences: the
    benchmark's CPU baseline).
    electron_f000: per wavefunction, the electron scattering factor at s = 0;
    given, the HC form factors are converted to electron scattering.
    form_factors: instead, the single-h form factors of every atom at every
    reflection (sfo_form_factors: no anomalous dispersion, 0 for excluded
    atoms), complex [n_hkl][n_atoms].
    """
    from discamb_gb300.crystal import (centering_multipliers, convert_adp, convert_adp_gradient,
                                       convert_xyz_gradient)
    if n_threads is None:
        n_threads = os.cpu_count() or 1
    hkl = st.hkl if hkl_subset is None else st.hkl[hkl_subset]
    dtdf = st.dtdf if hkl_subset is None else st.dtdf[hkl_subset]
    cell = st.cell
    m = st.frac_to_cart()
    minv = np.linalg.inv(m)
    bm = st.reciprocal()
    n = st.n_atoms
    sg = st.sg
    keep = _Keep()
    pr = _Problem()
    if model == "hc":
        pr.model = 0
        rot_f, tr_f = sg.subset_rot, sg.subset_trans
        centro = sg.centrosymmetric
        mult = centering_multipliers(sg.centering, sg.obverse, hkl)
    else:
        pr.model = 1 if model == "iam" else 2
        rot_f, tr_f = sg.rot, sg.all_trans()
        centro = False
        mult = np.ones(len(hkl))
    # Cartesian symmetry: R_cart = M R_frac M^-1, t_cart = M t_frac
    rot_c = np.array([m @ r @ minv for r in rot_f])
    tr_c = np.array([m @ t for t in tr_f])
    pr.n_sym = len(rot_c)
    pr.rot = keep.d(rot_c.reshape(-1))
    pr.trans = keep.d(tr_c.reshape(-1))
    pr.centro = int(centro)
    it = m @ sg.inversion_translation if centro else np.zeros(3)
    for k in range(3):
        pr.inv_trans[k] = float(it[k])
    # atoms
    pos = (m @ st.xyz.T).T if st.xyz_convention == "fractional" else st.xyz
    nadp = st.n_adp()
    adp = np.zeros((n, 6))
    i6 = np.flatnonzero(nadp == 6)
    i1 = np.flatnonzero(nadp == 1)
    if len(i6):  # the same conversion for every anisotropic atom, as one batched matrix product
        adp[i6] = convert_adp(cell, np.array([st.adp[i] for i in i6], dtype=np.float64), st.adp_convention,
                              "U_cart") * 2 * math.pi ** 2
    if len(i1):
        adp[i1, 0] = np.array([st.adp[i][0] for i in i1], dtype=np.float64) * 2 * math.pi ** 2
    pr.n_atoms = n
    pr.atom_wfn = keep.i(st.atom_wfn)
    pr.atom_type = keep.i(st.atom_type)
    pr.pos = keep.d(pos.reshape(-1))
    pr.n_adp = keep.i(nadp)
    pr.adp = keep.d(adp.reshape(-1))
    pr.occ = keep.d(st.occupancy)
    pr.mult_w = keep.d(np.asarray(st.multiplicity, dtype=np.float64) / sg.n_total)
    pr.lcs = keep.d(np.asarray(st.lcs).reshape(-1))
    if st.anomalous is not None:
        an = np.stack([np.real(st.anomalous), np.imag(st.anomalous)], axis=1)
        pr.atom_anom = keep.d(an.reshape(-1))
    pr.include = keep.i(st.include_mask().astype(np.int32))
    # model
    if model == "hc":
        arr = hc_model_arrays(st)
        pr.n_wfn = len(st.wfns)
        for k in ("core_coeff", "core_exp", "val_coeff", "val_exp", "def_exp", "wfn_anom",
                  "type_plm", "type_pval", "type_kappa", "type_kappa_p"):
            setattr(pr, k, keep.d(arr[k]))
        for k in ("core_off", "core_pow", "val_off", "val_pow", "def_npow", "def_pow", "type_nl"):
            setattr(pr, k, keep.i(arr[k]))
        pr.n_types = len(st.types)
    elif model == "iam":
        pr.n_types = len(iam["c"])
        pr.iam_ngauss = keep.i(iam["ngauss"])
        pr.iam_a = keep.d(np.asarray(iam["a"]).reshape(-1))
        pr.iam_b = keep.d(np.asarray(iam["b"]).reshape(-1))
        pr.iam_c = keep.d(iam["c"])
    else:
        t = np.asarray(table)
        tt = np.stack([t.real, t.imag], axis=-1)
        pr.table = keep.d(tt.reshape(-1))
    # reflections
    hc = (bm @ hkl.T.astype(np.float64)).T
    g = np.conj(dtdf) * mult
    pr.n_hkl = len(hkl)
    pr.h = keep.d(hc.reshape(-1))
    pr.dtdf = keep.d(np.stack([g.real, g.imag], axis=1).reshape(-1))
    pr.d_xyz = int("xyz" in derivatives)
    pr.d_adp = int("adp" in derivatives)
    pr.d_occ = int("occ" in derivatives)
    pr.d_mp = int(bool(multipoles))
    if electron_f000 is not None and model == "hc":
        pr.electron = 1
        pr.wfn_z = keep.i(np.array([w.atomic_number for w in st.wfns], dtype=np.int32))
        pr.wfn_f000 = keep.d(np.asarray(electron_f000, dtype=np.float64))
    if form_factors:
        ff = np.zeros((len(hkl), n, 2))
        for i in range(len(hkl)):
            hv = np.ascontiguousarray(hc[i], dtype=np.float64)
            if lib().sfo_form_factors(C.byref(pr), hv.ctypes.data_as(_P(C.c_double)),
                                      ff[i].ctypes.data_as(_P(C.c_double))) != 0:
                raise RuntimeError("oracle form factors failed")
        return ff[..., 0] + 1j * ff[..., 1]
    out = dict(f=np.zeros(2 * len(hkl)), d_xyz=np.zeros(3 * n), d_adp=np.zeros(6 * n), d_occ=np.zeros(n),
               d_pval=np.zeros(n), d_plm=np.zeros(25 * n), d_kappa=np.zeros(n), d_kappa_p=np.zeros(n))
    res = _Result()
    for k, v in out.items():
        setattr(res, k, _ptr(v, C.c_double))
    t_c = time.perf_counter()
    if loop == "lines" and model == "hc":
        hk = np.ascontiguousarray(np.asarray(hkl, dtype=np.int32).reshape(-1))
        b3 = np.ascontiguousarray(bm[:, 2], dtype=np.float64)
        rc = lib().sfo_compute_lines(C.byref(pr), hk.ctypes.data_as(_P(C.c_int)), b3.ctypes.data_as(_P(C.c_double)),
                                     C.byref(res), int(n_threads))
    else:
        rc = lib().sfo_compute(C.byref(pr), C.byref(res), int(n_threads))
    t_c = time.perf_counter() - t_c
    if rc != 0:
        raise RuntimeError("oracle failed")
    f = (out["f"][0::2] + 1j * out["f"][1::2]) * mult
    d_xyz = out["d_xyz"].reshape(n, 3)
    if st.xyz_convention == "fractional":
        d_xyz = convert_xyz_gradient(cell, d_xyz, "cartesian", "fractional")
    d_adp = out["d_adp"].reshape(n, 6).copy()
    if len(i6):
        d_adp[i6] = convert_adp_gradient(cell, d_adp[i6], "U_cart", st.adp_convention)
    # c_seconds: the C computation alone (the algorithm's own time, without this wrapper's array set-up)
    res_d = dict(f=f, d_xyz=d_xyz, d_adp=[d_adp[i, :nadp[i]] for i in range(n)], d_occ=out["d_occ"], c_seconds=t_c)
    if multipoles:
        res_d.update(d_pval=out["d_pval"], d_plm=out["d_plm"].reshape(n, 25), d_kappa=out["d_kappa"],
                     d_kappa_p=out["d_kappa_p"])
    return res_d
