"""Python binding of the dsf_gb300 C ABI (include/dsf_gb300.h).

``Engine`` owns one GPU and a stream; ``HcCalculator``, ``IamCalculator`` and
``TabulatedCalculator`` mirror the reference calculators behind
``SfCalculator::calculateStructureFactorsAndDerivatives``
(include/discamb/Scattering/SfCalculator.h:45-67):

* ``HcCalculator`` ~ HansenCoppensStructureFactorCalculator
  (include/discamb/Scattering/HansenCoppensStructureFactorCalculator.h:42-165);
* ``IamCalculator`` ~ AnyIamCalculator (src/Scattering/AnyIamCalculator.cpp);
* ``TabulatedCalculator`` ~ TscFileBasedSfCalculator
  (src/Scattering/TscFileBasedSfCalculator.cpp).

``calculate_structure_factors_and_derivatives`` takes the atoms' current
parameters, dT/dF per reflection and the inclusion mask, and returns F and
the derivatives in the crystal's conventions; errors raise ``DsfError`` with
the engine's message (the reference throws discamb::Exception).  The
library must be built (``discamb_gb300.build.build()``); there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref

import numpy as np

from .build import LIB
from .model import density_terms

_P = C.POINTER

DSF_FP64 = 0
DSF_FP32_BULK = 1
DSF_PENDING = 7
DSF_D_XYZ, DSF_D_ADP, DSF_D_OCC, DSF_D_MULTIPOLE = 1, 2, 4, 8
_ADP = {"U_cif": 0, "U_cart": 1, "U_star": 2}
_XYZ = {"fractional": 0, "cartesian": 1}


class DsfError(RuntimeError):
    pass


class _Sym(C.Structure):
    _fields_ = [("cell", C.c_double * 6), ("n_symops", C.c_int), ("symop_rotation", _P(C.c_int)),
                ("symop_translation", _P(C.c_double)), ("centrosymmetric", C.c_int),
                ("inversion_translation", C.c_double * 3), ("centering", C.c_char), ("obverse", C.c_int),
                ("n_symops_total", C.c_int)]


class _Hc(C.Structure):
    _fields_ = [("n_wfn", C.c_int), ("core_offset", _P(C.c_int)), ("core_coeff", _P(C.c_double)),
                ("core_exp", _P(C.c_double)), ("core_pow", _P(C.c_int)), ("val_offset", _P(C.c_int)),
                ("val_coeff", _P(C.c_double)), ("val_exp", _P(C.c_double)), ("val_pow", _P(C.c_int)),
                ("def_val_exp", _P(C.c_double)), ("def_val_npow", _P(C.c_int)), ("def_val_pow", _P(C.c_int)),
                ("anomalous", _P(C.c_double)), ("n_types", C.c_int), ("type_nl", _P(C.c_int)),
                ("type_plm", _P(C.c_double)), ("type_pval", _P(C.c_double)), ("type_kappa", _P(C.c_double)),
                ("type_kappa_prime", _P(C.c_double))]


class _Iam(C.Structure):
    _fields_ = [("n_types", C.c_int), ("n_gauss", _P(C.c_int)), ("a", _P(C.c_double)), ("b", _P(C.c_double)),
                ("c", _P(C.c_double))]


class _Atoms(C.Structure):
    _fields_ = [("n_atoms", C.c_int), ("atom_wfn", _P(C.c_int)), ("atom_type", _P(C.c_int)),
                ("adp_components", _P(C.c_int)), ("lcs", _P(C.c_double)), ("multiplicity", _P(C.c_double)),
                ("anomalous", _P(C.c_double)), ("xyz_convention", C.c_int), ("adp_convention", C.c_int)]


class _Out(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in
                ("f", "d_xyz", "d_adp", "d_occ", "d_pval", "d_plm", "d_kappa", "d_kappa_prime")]


_lib = None


def library():
    """Loads libdsf_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise DsfError(f"CUDA engine library not built: {LIB} (run discamb_gb300.build.build())")
        _lib = C.CDLL(LIB)
        L = _lib
        L.dsf_engine_create.argtypes = [C.c_int, _P(C.c_void_p)]
        L.dsf_engine_destroy.argtypes = [C.c_void_p]
        L.dsf_last_error.argtypes = [C.c_void_p]
        L.dsf_last_error.restype = C.c_char_p
        L.dsf_structure_create_hc.argtypes = [C.c_void_p, _P(_Sym), _P(_Hc), _P(_Atoms), _P(C.c_void_p)]
        L.dsf_structure_create_iam.argtypes = [C.c_void_p, _P(_Sym), _P(_Iam), _P(_Atoms), _P(C.c_void_p)]
        L.dsf_structure_create_tabulated.argtypes = [C.c_void_p, _P(_Sym), _P(_Atoms), C.c_int, _P(C.c_int),
                                                     _P(C.c_double), C.c_int, _P(C.c_void_p)]
        L.dsf_structure_create_tabulated_device.argtypes = [C.c_void_p, _P(_Sym), _P(_Atoms), C.c_int, _P(C.c_int),
                                                            C.c_void_p, C.c_int, _P(C.c_void_p)]
        L.dsf_structure_destroy.argtypes = [C.c_void_p]
        L.dsf_structure_set_hkl.argtypes = [C.c_void_p, C.c_int, _P(C.c_int)]
        L.dsf_structure_update_atoms.argtypes = [C.c_void_p, _P(C.c_double), _P(C.c_double), _P(C.c_double)]
        L.dsf_structure_update_types.argtypes = [C.c_void_p, _P(C.c_double), _P(C.c_double), _P(C.c_double),
                                                 _P(C.c_double)]
        L.dsf_structure_set_lcs.argtypes = [C.c_void_p, _P(C.c_double)]
        L.dsf_structure_device_bytes.argtypes = [C.c_void_p]
        L.dsf_structure_device_bytes.restype = C.c_int64
        L.dsf_calculate.argtypes = [C.c_void_p, C.c_int, C.c_int, _P(C.c_double), _P(C.c_int), _P(_Out)]
        L.dsf_calculate_atoms.argtypes = [C.c_void_p, C.c_int, C.c_int, _P(C.c_double), _P(C.c_double),
                                          _P(C.c_double), _P(C.c_double), _P(C.c_int), _P(_Out)]
        L.dsf_calculate_device.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, _P(_Out), C.c_void_p]
        L.dsf_calculate_batch_device.argtypes = [_P(C.c_void_p), C.c_int, C.c_int, C.c_int, _P(C.c_void_p),
                                                 _P(_Out), C.c_void_p]
        L.dsf_calculate_batch.argtypes = [_P(C.c_void_p), C.c_int, C.c_int, C.c_int, _P(C.c_void_p),
                                          _P(C.c_void_p), _P(_Out)]
        L.dsf_calculate_batch_atoms.argtypes = [_P(C.c_void_p), C.c_int, C.c_int, C.c_int, _P(C.c_void_p),
                                                _P(C.c_void_p), _P(C.c_void_p), _P(C.c_void_p), _P(C.c_void_p),
                                                _P(_Out)]
        L.dsf_reduce_to_types.argtypes = [C.c_void_p, _P(_Out), _P(_Out), C.c_void_p]
        L.dsf_structure_set_electron.argtypes = [C.c_void_p, C.c_int, _P(C.c_int), _P(C.c_double)]
        L.dsf_structure_create_tsc.argtypes = [C.c_void_p, _P(_Sym), _P(_Atoms), C.c_int, _P(C.c_int), C.c_char_p,
                                               _P(C.c_void_p)]
        L.dsf_tsc_load.argtypes = [C.c_char_p, _P(C.c_int), _P(C.c_int), _P(C.c_int), _P(C.c_double), C.c_int]
        L.dsf_form_factors.argtypes = [C.c_void_p, _P(C.c_int), _P(C.c_int), _P(C.c_double)]
        L.dsf_debug_stall_next_call.argtypes = [C.c_void_p]
        L.dsf_structure_set_anomalous.argtypes = [C.c_void_p, _P(C.c_double)]
        L.dsf_submit.argtypes = [C.c_void_p, C.c_int, C.c_int, _P(C.c_double), _P(C.c_double), _P(C.c_double),
                                 _P(C.c_double), _P(C.c_int), _P(_Out), _P(C.c_void_p)]
        L.dsf_poll.argtypes = [C.c_void_p, C.c_int]
        L.dsf_last_launch_count.argtypes = [C.c_void_p]
        L.dsf_last_kernel_ms.argtypes = [C.c_void_p]
        L.dsf_last_kernel_ms.restype = C.c_double
        L.dsf_autotune.argtypes = [C.c_void_p, C.c_int, C.c_int, _P(C.c_int), _P(C.c_int), _P(C.c_int),
                                   _P(C.c_double)]
        L.dsf_tuning_lookup.argtypes = [C.c_void_p, C.c_int, C.c_int, _P(C.c_int), _P(C.c_int), _P(C.c_int),
                                        _P(C.c_int)]
        L.dsf_tuning_save.argtypes = [C.c_void_p, C.c_char_p]
        L.dsf_tuning_load.argtypes = [C.c_void_p, C.c_char_p]
    return _lib


def _flags(derivatives, multipoles):
    return (DSF_D_XYZ if "xyz" in derivatives else 0) | (DSF_D_ADP if "adp" in derivatives else 0) | \
        (DSF_D_OCC if "occ" in derivatives else 0) | (DSF_D_MULTIPOLE if multipoles else 0)


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_P(C.c_double))


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(_P(C.c_int))


class Ticket:
    """A submitted call (dsf_submit): poll(timeout_ms) returns the result
    dict once the call is done, None while it is pending; it raises DsfError
    if the call failed."""

    def __init__(self, calc, handle, out, multipoles, adp_layout, keep):
        self._calc, self._h, self._out = calc, handle, out
        self._mp, self._layout, self._keep = multipoles, adp_layout, keep
        self.result = None

    def poll(self, timeout_ms=0):
        if self.result is not None:
            return self.result
        rc = self._calc.lib.dsf_poll(self._h, int(timeout_ms))
        if rc == DSF_PENDING:
            return None
        self._keep = None
        self._calc.engine.check(rc, "poll")
        self.result = self._calc._result(self._out, self._mp, self._layout)
        return self.result

    def wait(self):
        while self.poll(1000) is None:
            pass
        return self.result


class Engine:
    """One GPU + stream (dsf_engine)."""

    def __init__(self, device=0):
        self.lib = library()
        self.h = C.c_void_p()
        self._calculators = weakref.WeakSet()
        rc = self.lib.dsf_engine_create(int(device), C.byref(self.h))
        if rc != 0:
            raise DsfError(f"dsf_engine_create failed with status {rc}")

    def check(self, rc, what):
        if rc != 0:
            msg = self.lib.dsf_last_error(self.h)
            raise DsfError(f"{what}: status {rc}: {msg.decode() if msg else ''}")

    def save_tuning(self, path):
        """dsf_tuning_save: the autotuner's shapes of this engine to a text file."""
        self.check(self.lib.dsf_tuning_save(self.h, os.fsencode(path)), "save_tuning")

    def load_tuning(self, path):
        """dsf_tuning_load: shapes of a file written by save_tuning."""
        self.check(self.lib.dsf_tuning_load(self.h, os.fsencode(path)), "load_tuning")

    def calculate_batch(self, calcs, dtdfs, precision=DSF_FP32_BULK, derivatives=("xyz", "adp", "occ"),
                        multipoles=False, includes=None, atoms=None):
        """Several calculators of this engine in one submission
        (dsf_calculate_batch_atoms): host dT/dF per calculator; atoms[i] =
        (xyz, adp, occupancy) of this call or None (the resident ones);
        returns one result dict per calculator (padded [n][6] ADP layout)."""
        n = len(calcs)
        flags = _flags(derivatives, multipoles)
        hs = (C.c_void_p * n)(*[c.h.value for c in calcs])
        keep, gp, ip = [], (C.c_void_p * n)(), (C.c_void_p * n)()
        xp, ap, op = (C.c_void_p * n)(), (C.c_void_p * n)(), (C.c_void_p * n)()
        outs = (_Out * n)()
        res = []
        for i, c in enumerate(calcs):
            if atoms is not None and atoms[i] is not None:
                (x1, p1), (x2, p2), (x3, p3) = c._atom_arrays(*atoms[i])
                keep += [x1, x2, x3]
                xp[i], ap[i], op[i] = x1.ctypes.data, x2.ctypes.data, x3.ctypes.data
            g = np.ascontiguousarray(dtdfs[i], dtype=np.complex128).view(np.float64)
            keep.append(g)
            gp[i] = g.ctypes.data
            if includes is not None and includes[i] is not None:
                inc = np.ascontiguousarray(includes[i], dtype=np.int32)
                keep.append(inc)
                ip[i] = inc.ctypes.data
            r = c._out_arrays(multipoles, flags)
            res.append(r)
            c._fill_out(outs[i], r, multipoles)
        self.check(self.lib.dsf_calculate_batch_atoms(hs, n, int(precision), flags, xp, ap, op, gp,
                                                      ip if includes is not None else None, outs),
                   "calculate_batch")
        return [c._result(r, multipoles, "padded") for c, r in zip(calcs, res)]

    def calculate_batch_device(self, calcs, dtdf_ptrs, outputs, precision=DSF_FP32_BULK,
                               derivatives=("xyz", "adp", "occ"), multipoles=False, stream=0):
        """Device-resident batch (dsf_calculate_batch_device): dtdf_ptrs[i]
        and outputs[i] (dict of device pointers) per calculator."""
        n = len(calcs)
        hs = (C.c_void_p * n)(*[c.h.value for c in calcs])
        gp = (C.c_void_p * n)(*[int(p) for p in dtdf_ptrs])
        outs = (_Out * n)()
        for i, o in enumerate(outputs):
            for k, v in o.items():
                setattr(outs[i], k, v)
        self.check(self.lib.dsf_calculate_batch_device(hs, n, int(precision), _flags(derivatives, multipoles), gp,
                                                       outs, C.c_void_p(stream)), "calculate_batch_device")

    def close(self):
        """Destroys the engine after every structure created on it."""
        for c in list(self._calculators):
            c.close()
        if self.h:
            self.lib.dsf_engine_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def symmetry_desc(st, representation="engine"):
    """dsf_symmetry of a Structure: 'engine' = subset + inversion flag (the
    HansenCoppens CPU engine), 'all' = all operations modulo centering
    (the generic AnyScatterer engine)."""
    sg = st.sg
    keep = []
    if representation == "engine":
        rot, tr = sg.subset_rot, sg.subset_trans
        centro = sg.centrosymmetric
    else:
        # all operations, one per centering coset
        cv = {tuple(t) for r, t in zip(sg.rot, sg.trans12) if np.array_equal(r, np.eye(3, dtype=np.int64))}
        chosen, seen = [], set()
        for r, t in zip(sg.rot, sg.trans12):
            key = (r.tobytes(), tuple(t))
            if key in seen:
                continue
            chosen.append((r, t))
            for c in cv:
                seen.add((r.tobytes(), tuple((np.array(t) + np.array(c)) % 12)))
        rot = np.array([r for r, _ in chosen])
        tr = np.array([t for _, t in chosen], dtype=np.float64) / 12.0
        centro = False
    s = _Sym()
    for k in range(6):
        s.cell[k] = st.cell[k]
    s.n_symops = len(rot)
    a, s.symop_rotation = _i(np.asarray(rot).reshape(-1)); keep.append(a)
    b, s.symop_translation = _d(np.asarray(tr).reshape(-1)); keep.append(b)
    s.centrosymmetric = int(centro)
    for k in range(3):
        s.inversion_translation[k] = float(sg.inversion_translation[k]) if centro else 0.0
    s.centering = sg.centering.encode()
    s.obverse = int(sg.obverse)
    s.n_symops_total = sg.n_total
    return s, keep


def _atoms_desc(st, lcs=True):
    keep = []
    a = _Atoms()
    a.n_atoms = st.n_atoms
    x, a.atom_wfn = _i(st.atom_wfn); keep.append(x)
    x, a.atom_type = _i(st.atom_type); keep.append(x)
    x, a.adp_components = _i(st.n_adp()); keep.append(x)
    if lcs:
        x, a.lcs = _d(np.asarray(st.lcs).reshape(-1)); keep.append(x)
    x, a.multiplicity = _d(np.asarray(st.multiplicity, dtype=np.float64)); keep.append(x)
    if st.anomalous is not None:
        x, a.anomalous = _d(np.stack([np.real(st.anomalous), np.imag(st.anomalous)], 1).reshape(-1)); keep.append(x)
    a.xyz_convention = _XYZ[st.xyz_convention]
    a.adp_convention = _ADP[st.adp_convention]
    return a, keep


def _hc_desc(st):
    keep = []
    m = _Hc()
    core_off, val_off = [0], [0]
    cc, ce, cp, vc, ve, vp, dexp, dnp, dpw, an = [], [], [], [], [], [], [], [], [], []
    for w in st.wfns:
        c, e, p = density_terms(w, "core"); cc += list(c); ce += list(e); cp += list(p); core_off.append(len(cc))
        c, e, p = density_terms(w, "valence"); vc += list(c); ve += list(e); vp += list(p); val_off.append(len(vc))
        dexp.append(w.def_val_exp); dnp.append(min(5, len(w.def_val_pow)))
        dpw += list(w.def_val_pow)[:5] + [0] * (5 - min(5, len(w.def_val_pow)))
        an += [complex(w.anomalous).real, complex(w.anomalous).imag]
    m.n_wfn = len(st.wfns)
    for name, arr, kind in [("core_offset", core_off, "i"), ("core_coeff", cc + [0.0], "d"), ("core_exp", ce + [1.0], "d"),
                            ("core_pow", cp + [0], "i"), ("val_offset", val_off, "i"), ("val_coeff", vc + [0.0], "d"),
                            ("val_exp", ve + [1.0], "d"), ("val_pow", vp + [0], "i"), ("def_val_exp", dexp, "d"),
                            ("def_val_npow", dnp, "i"), ("def_val_pow", dpw, "i"), ("anomalous", an, "d")]:
        x, p = (_i if kind == "i" else _d)(arr)
        keep.append(x)
        setattr(m, name, p)
    types = st.types
    m.n_types = len(types)
    for name, arr, kind in [("type_nl", [t.n_l for t in types], "i"),
                            ("type_plm", np.array([t.plm for t in types]).reshape(-1), "d"),
                            ("type_pval", [t.p_val for t in types], "d"), ("type_kappa", [t.kappa for t in types], "d"),
                            ("type_kappa_prime", [t.kappa_prime for t in types], "d")]:
        x, p = (_i if kind == "i" else _d)(arr)
        keep.append(x)
        setattr(m, name, p)
    return m, keep


class _Calculator:
    model = "hc"

    def __init__(self, engine: Engine, st):
        self.engine = engine
        self.lib = engine.lib
        self.st = st
        self.h = C.c_void_p()
        self.n_atoms = st.n_atoms
        self._n_adp = st.n_adp()
        self.n_hkl = 0
        engine._calculators.add(self)

    def set_hkl(self, hkl):
        hkl = np.ascontiguousarray(hkl, dtype=np.int32)
        x, p = _i(hkl.reshape(-1))
        self.engine.check(self.lib.dsf_structure_set_hkl(self.h, len(hkl), p), "set_hkl")
        self.n_hkl = len(hkl)

    def _atom_arrays(self, xyz, adp, occupancy):
        if isinstance(adp, np.ndarray) and adp.shape == (self.n_atoms, 6):
            adp6 = adp
        else:
            adp6 = np.zeros((self.n_atoms, 6))
            for i, a in enumerate(adp):
                adp6[i, :len(a)] = a
        return _d(np.asarray(xyz).reshape(-1)), _d(adp6.reshape(-1)), _d(occupancy)

    def update_atoms(self, xyz, adp, occupancy):
        (x1, p1), (x2, p2), (x3, p3) = self._atom_arrays(xyz, adp, occupancy)
        self.engine.check(self.lib.dsf_structure_update_atoms(self.h, p1, p2, p3), "update_atoms")

    def calculate_at_hkl(self, hkl, include=None, atoms=None, precision=DSF_FP64):
        """F(h) and the derivatives of F itself at one reflection (complex per
        atom), as calculateStructureFactorsAndDerivatives(hkl, F,
        SfDerivativesAtHkl, mask) (include/discamb/Scattering/SfCalculator.h:82-86):
        two calls on the one reflection with dT/dF = 1 and i give Re and Im of
        dF/dp.  The resident reflection set is restored afterwards."""
        saved = getattr(self, "_hkl_cache", None)
        if saved is None:
            saved = np.asarray(self.st.hkl, dtype=np.int32)
        self.set_hkl(np.asarray(hkl, dtype=np.int32).reshape(1, 3))
        try:
            a = self.calculate(np.array([1.0 + 0j]), precision=precision, include=include, atoms=atoms,
                               adp_layout="padded")
            b = self.calculate(np.array([1j]), precision=precision, include=include, adp_layout="padded")
        finally:
            self.set_hkl(saved)
            self._hkl_cache = saved
        nadp = self._n_adp
        d_adp = a["d_adp"] + 1j * b["d_adp"]
        return dict(f=a["f"][0], d_xyz=a["d_xyz"] + 1j * b["d_xyz"],
                    d_adp=[d_adp[i, :nadp[i]] for i in range(self.n_atoms)], d_occ=a["d_occ"] + 1j * b["d_occ"])

    def set_anomalous(self, anomalous):
        """Per-atom anomalous dispersion f' + i f'' (complex [n_atoms]),
        replacing the values given at creation (SfCalculator::setAnomalous)."""
        a = np.asarray(anomalous, dtype=np.complex128).reshape(-1)
        v, p = _d(np.stack([a.real, a.imag], axis=1).reshape(-1))
        self.engine.check(self.lib.dsf_structure_set_anomalous(self.h, p), "set_anomalous")

    def debug_stall_next_call(self):
        """Test hook of the failure path (dsf_debug_stall_next_call): the
        next call's kernel waits run out and the call raises DsfError
        (DSF_ERR_TIMEOUT) after about 4 s; the engine stays usable."""
        self.engine.check(self.lib.dsf_debug_stall_next_call(self.h), "debug_stall_next_call")

    def form_factors(self, hkl, include=None):
        """The single-h calculateFormFactors of the reference
        (SfCalculator.h:82-93; HansenCoppensStructureFactorCalculator.cpp:
        1277-1304, AnyIamCalculator.cpp:223-233) through dsf_form_factors:
        complex form factors of every atom at one reflection ([n_atoms]) or at
        each of a list ([n][n_atoms]); no anomalous dispersion, 0 for atoms
        with include[a] == 0.  HC and IAM calculators."""
        h = np.asarray(hkl, dtype=np.int32)
        single = h.ndim == 1
        h = np.ascontiguousarray(h.reshape(-1, 3))
        n = self.st.n_atoms
        inc = None
        if include is not None:
            inc_arr, inc = _i(np.asarray(include).astype(np.int32))
        out = np.zeros((len(h), n, 2))
        for i in range(len(h)):
            self.engine.check(self.lib.dsf_form_factors(self.h, h[i].ctypes.data_as(_P(C.c_int)), inc,
                                                        out[i].ctypes.data_as(_P(C.c_double))), "form_factors")
        ff = out[..., 0] + 1j * out[..., 1]
        return ff[0] if single else ff

    def _out_arrays(self, multipoles, flags=DSF_D_XYZ | DSF_D_ADP | DSF_D_OCC):
        """Output arrays of one call: the engine writes F and every requested
        derivative in full (left uninitialised here); the others stay zero."""
        n, m = self.n_atoms, self.n_hkl
        new = lambda k, bit: np.empty(k) if flags & bit else np.zeros(k)
        r = dict(f=np.empty(2 * m), d_xyz=new(3 * n, DSF_D_XYZ), d_adp=new(6 * n, DSF_D_ADP),
                 d_occ=new(n, DSF_D_OCC))
        if multipoles:
            mp = DSF_D_MULTIPOLE if isinstance(self, HcCalculator) else 0
            r.update(d_pval=new(n, mp), d_plm=new(25 * n, mp), d_kappa=new(n, mp), d_kappa_prime=new(n, mp))
        return r

    @staticmethod
    def _fill_out(o, r, multipoles):
        o.f = r["f"].ctypes.data
        o.d_xyz, o.d_adp, o.d_occ = r["d_xyz"].ctypes.data, r["d_adp"].ctypes.data, r["d_occ"].ctypes.data
        if multipoles:
            o.d_pval, o.d_plm = r["d_pval"].ctypes.data, r["d_plm"].ctypes.data
            o.d_kappa, o.d_kappa_prime = r["d_kappa"].ctypes.data, r["d_kappa_prime"].ctypes.data

    def _result(self, r, multipoles, adp_layout):
        n = self.n_atoms
        da = r["d_adp"].reshape(n, 6)
        if adp_layout == "padded":
            d_adp = da
        else:
            nadp = self._n_adp
            d_adp = [da[i, :nadp[i]] for i in range(n)]
        out = dict(f=r["f"].view(np.complex128), d_xyz=r["d_xyz"].reshape(n, 3), d_adp=d_adp, d_occ=r["d_occ"])
        if multipoles:
            out.update(d_pval=r["d_pval"], d_plm=r["d_plm"].reshape(n, 25), d_kappa=r["d_kappa"],
                       d_kappa_p=r["d_kappa_prime"])
        return out

    def calculate(self, dtdf, precision=DSF_FP64, derivatives=("xyz", "adp", "occ"), multipoles=False,
                  include=None, atoms=None, adp_layout="list"):
        """F and dT/dparam in the crystal's conventions (host buffers).
        atoms = (xyz, adp, occupancy) uploads the atoms' parameters in the same
        call (dsf_calculate_atoms); None computes with the resident ones.
        adp_layout "list": d_adp[i] holds the atom's own ADP components (the
        reference's adp_derivatives); "padded": one [n][6] array, zero past
        each atom's component count."""
        flags = _flags(derivatives, multipoles)
        g = np.ascontiguousarray(dtdf, dtype=np.complex128).view(np.float64)
        r = self._out_arrays(multipoles, flags)
        o = _Out()
        self._fill_out(o, r, multipoles)
        inc = None
        if include is not None:
            incarr, inc = _i(np.asarray(include, dtype=np.int32))
        gp = g.ctypes.data_as(_P(C.c_double))
        if atoms is None:
            self.engine.check(self.lib.dsf_calculate(self.h, int(precision), flags, gp, inc, C.byref(o)), "calculate")
        else:
            (x1, p1), (x2, p2), (x3, p3) = self._atom_arrays(*atoms)
            self.engine.check(self.lib.dsf_calculate_atoms(self.h, int(precision), flags, p1, p2, p3, gp, inc,
                                                           C.byref(o)), "calculate")
        return self._result(r, multipoles, adp_layout)

    def submit(self, dtdf, precision=DSF_FP64, derivatives=("xyz", "adp", "occ"), multipoles=False,
               include=None, atoms=None, adp_layout="list"):
        """The same call, asynchronous (dsf_submit): returns a Ticket at once;
        Ticket.poll(timeout_ms) gives the result dict when the call is done
        (None while it is pending).  One pending call per calculator."""
        flags = _flags(derivatives, multipoles)
        g = np.ascontiguousarray(dtdf, dtype=np.complex128).view(np.float64)
        r = self._out_arrays(multipoles, flags)
        o = _Out()
        self._fill_out(o, r, multipoles)
        inc, keep = None, [g]
        if include is not None:
            incarr, inc = _i(np.asarray(include, dtype=np.int32))
            keep.append(incarr)
        ps = (None, None, None)
        if atoms is not None:
            (x1, p1), (x2, p2), (x3, p3) = self._atom_arrays(*atoms)
            keep += [x1, x2, x3]
            ps = (p1, p2, p3)
        t = C.c_void_p()
        self.engine.check(self.lib.dsf_submit(self.h, int(precision), flags, *ps, g.ctypes.data_as(_P(C.c_double)),
                                              inc, C.byref(o), C.byref(t)), "submit")
        return Ticket(self, t, r, multipoles, adp_layout, keep + [o])

    def calculate_structure_factors_and_derivatives(self, xyz, adp, occupancy, hkl, dtdf, include=None,
                                                    precision=DSF_FP64, multipoles=False):
        """Reference-style call: atoms + hkl + dT/dF -> F and derivatives.
        The reflection set stays resident while it does not change."""
        hkl = np.asarray(hkl, dtype=np.int32)
        cached = getattr(self, "_hkl_cache", None)
        if cached is None or cached.shape != hkl.shape or not np.array_equal(cached, hkl):
            self.set_hkl(hkl)
            self._hkl_cache = hkl.copy()
        return self.calculate(dtdf, precision=precision, multipoles=multipoles, include=include,
                              atoms=(xyz, adp, occupancy))

    def device_bytes(self):
        return self.lib.dsf_structure_device_bytes(self.h)

    def last_launch_count(self):
        return self.lib.dsf_last_launch_count(self.h)

    def last_kernel_ms(self):
        return self.lib.dsf_last_kernel_ms(self.h)

    def autotune(self, precision=DSF_FP32_BULK, derivatives=("xyz", "adp", "occ"), multipoles=False):
        """dsf_autotune: times this structure's call over a few tile shapes and
        keeps the fastest for every later call of structures of the same shape
        key.  Returns dict(blocks_per_sm, ht, occupancy, ms) of the chosen
        shape (ht 0: the longest shared-memory sub-tile; occupancy 3: the
        register-capped form, 0: the compiler's registers)."""
        bps, ht, occ, ms = C.c_int(0), C.c_int(0), C.c_int(0), C.c_double(0)
        self.engine.check(self.lib.dsf_autotune(self.h, int(precision), _flags(derivatives, multipoles), C.byref(bps),
                                                C.byref(ht), C.byref(occ), C.byref(ms)), "autotune")
        return dict(blocks_per_sm=bps.value, ht=ht.value, occupancy=occ.value, ms=ms.value)

    def tile_shape(self, precision=DSF_FP32_BULK, derivatives=("xyz", "adp", "occ"), multipoles=False):
        """dsf_tuning_lookup: the tile shape the next call takes and whether it
        is a tuned one."""
        bps, ht, occ, tuned = C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0)
        self.engine.check(self.lib.dsf_tuning_lookup(self.h, int(precision), _flags(derivatives, multipoles),
                                                     C.byref(bps), C.byref(ht), C.byref(occ), C.byref(tuned)),
                          "tile_shape")
        return dict(blocks_per_sm=bps.value, ht=ht.value, occupancy=occ.value, tuned=bool(tuned.value))

    def calculate_device(self, dtdf_ptr, outputs, precision=DSF_FP32_BULK, derivatives=("xyz", "adp", "occ"),
                         multipoles=False, stream=0):
        """Device-resident call: dtdf_ptr = device pointer to [n_hkl][2]
        doubles, outputs = dict of device pointers (f required)."""
        flags = _flags(derivatives, multipoles)
        o = _Out()
        for k, v in outputs.items():
            setattr(o, k, v)
        self.engine.check(self.lib.dsf_calculate_device(self.h, int(precision), flags, C.c_void_p(dtdf_ptr),
                                                        C.byref(o), C.c_void_p(stream)), "calculate_device")

    def close(self):
        if self.h:
            self.lib.dsf_structure_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class HcCalculator(_Calculator):
    """Hansen-Coppens structure factors; symmetry as the HC CPU engine
    (subset + inversion + centering multipliers) by default."""

    def __init__(self, engine, st, representation="engine", upload_atoms=True):
        super().__init__(engine, st)
        self.def_val_symm = False
        sym, k1 = symmetry_desc(st, representation)
        model, k2 = _hc_desc(st)
        atoms, k3 = _atoms_desc(st)
        engine.check(self.lib.dsf_structure_create_hc(engine.h, C.byref(sym), C.byref(model), C.byref(atoms),
                                                      C.byref(self.h)), "create_hc")
        self.set_hkl(st.hkl)
        if upload_atoms:  # else the first call brings the atoms (calculate(..., atoms=...))
            self.update_atoms(st.xyz, st.adp, st.occupancy)

    def set_electron(self, on=True, f000=None):
        """Electron scattering (Mott-Bethe) for every form factor; f000[w]:
        the electron scattering factor at s = 0 of wavefunction w's element."""
        if on:
            z, pz = _i(np.array([w.atomic_number for w in self.st.wfns], dtype=np.int32))
            f0, pf = _d(np.asarray(f000, dtype=np.float64))
        else:
            pz = pf = None
        self.engine.check(self.lib.dsf_structure_set_electron(self.h, int(bool(on)), pz, pf), "set_electron")

    def set_def_val_symm(self, on=True):
        """The reference's point-group-symmetrised deformation valence
        (HansenCoppensStructureFactorCalculator::set_def_val_symm, which
        selects HansenCoppens_SF_EngineSymm: the same F and derivatives as
        Engine3, the harmonics of a point group's operations evaluated once
        per parity class).  The kernels here always take that split where the
        operations have sign-diagonal cosets (the coset form), so the switch
        changes nothing in the result or in the work; it is kept so callers
        that set it run unchanged."""
        self.def_val_symm = bool(on)

    def reduce_to_types(self, per_atom, per_type, stream=0):
        """TAAM types: sum the multipole derivatives of the atoms of each type
        on the device (dsf_reduce_to_types); per_atom / per_type: dicts of
        device pointers (d_pval, d_plm, d_kappa, d_kappa_prime)."""
        a, t = _Out(), _Out()
        for o, d in ((a, per_atom), (t, per_type)):
            for k, v in d.items():
                setattr(o, k, v)
        self.engine.check(self.lib.dsf_reduce_to_types(self.h, C.byref(a), C.byref(t), C.c_void_p(stream)),
                          "reduce_to_types")

    def update_types(self, plm=None, pval=None, kappa=None, kappa_prime=None):
        ps = [None if v is None else _d(np.asarray(v).reshape(-1)) for v in (plm, pval, kappa, kappa_prime)]
        args = [None if p is None else p[1] for p in ps]
        self.engine.check(self.lib.dsf_structure_update_types(self.h, *args), "update_types")

    def set_lcs(self, lcs):
        x, p = _d(np.asarray(lcs).reshape(-1))
        self.engine.check(self.lib.dsf_structure_set_lcs(self.h, p), "set_lcs")


class IamCalculator(_Calculator):
    """IAM with per-type n-Gaussian form factors; all operations modulo
    centering (the AnyScatterer engine's representation) by default, or
    representation="engine": the subset with the inversion and centering
    taken by the engine (the same F and derivatives)."""

    def __init__(self, engine, st, iam, representation="all"):
        super().__init__(engine, st)
        sym, k1 = symmetry_desc(st, representation)
        m = _Iam()
        m.n_types = len(iam["c"])
        keep = []
        for name, arr, kind in [("n_gauss", iam["ngauss"], "i"), ("a", np.asarray(iam["a"]).reshape(-1), "d"),
                                ("b", np.asarray(iam["b"]).reshape(-1), "d"), ("c", iam["c"], "d")]:
            x, p = (_i if kind == "i" else _d)(arr)
            keep.append(x)
            setattr(m, name, p)
        atoms, k3 = _atoms_desc(st, lcs=False)
        engine.check(self.lib.dsf_structure_create_iam(engine.h, C.byref(sym), C.byref(m), C.byref(atoms),
                                                       C.byref(self.h)), "create_iam")
        self.set_hkl(st.hkl)
        self.update_atoms(st.xyz, st.adp, st.occupancy)


class TabulatedCalculator(_Calculator):
    """Tabulated complex form factors per (reflection, operation, atom) over
    all operations modulo centering."""

    def __init__(self, engine, st, table=None, fp32_table=False, table_device=None, table_device_fp64=False,
                 tsc_path=None):
        """table: host complex [n_hkl][n_ops][n_atoms]; or table_device: a
        device pointer to the same layout (complex64, or complex128 with
        table_device_fp64), gathered on the device (FP32 table); or
        tsc_path: a .tsc file whose columns are the structure's atoms."""
        super().__init__(engine, st)
        sym, k1 = symmetry_desc(st, "all")
        atoms, k3 = _atoms_desc(st, lcs=False)
        x, p = _i(np.asarray(st.hkl).reshape(-1))
        if tsc_path is not None:
            engine.check(self.lib.dsf_structure_create_tsc(engine.h, C.byref(sym), C.byref(atoms), len(st.hkl), p,
                                                           os.fsencode(tsc_path), C.byref(self.h)), "create_tsc")
        elif table_device is not None:
            engine.check(self.lib.dsf_structure_create_tabulated_device(
                engine.h, C.byref(sym), C.byref(atoms), len(st.hkl), p, C.c_void_p(int(table_device)),
                int(table_device_fp64), C.byref(self.h)), "create_tabulated_device")
        else:
            t = np.asarray(table)
            tt = np.ascontiguousarray(np.stack([t.real, t.imag], -1).reshape(-1), dtype=np.float64)
            engine.check(self.lib.dsf_structure_create_tabulated(engine.h, C.byref(sym), C.byref(atoms), len(st.hkl),
                                                                 p, tt.ctypes.data_as(_P(C.c_double)),
                                                                 int(fp32_table), C.byref(self.h)), "create_tabulated")
        self.n_hkl = len(st.hkl)
        self.update_atoms(st.xyz, st.adp, st.occupancy)


def all_ops_mod_centering(sg):
    """(rot, trans) of all operations modulo lattice centering, in the
    order symmetry_desc(..., 'all') passes them to the engine."""
    cv = {tuple(t) for r, t in zip(sg.rot, sg.trans12) if np.array_equal(r, np.eye(3, dtype=np.int64))}
    chosen, seen = [], set()
    for r, t in zip(sg.rot, sg.trans12):
        key = (r.tobytes(), tuple(t))
        if key in seen:
            continue
        chosen.append((r, t))
        for c in cv:
            seen.add((r.tobytes(), tuple((np.array(t) + np.array(c)) % 12)))
    return np.array([r for r, _ in chosen]), np.array([t for _, t in chosen], dtype=np.float64) / 12.0


class CombinedCalculator:
    """Atoms split over several calculators, F summed and every atom's
    derivatives taken from its own calculator, as
    CombinedStructureFactorCalculator (include/discamb/Scattering/
    CombinedStructureFactorCalculator.h:14-60; TAAM: multipolar atoms on the
    HC model, the rest IAM, src/Scattering/HcAtomBankStructureFactorCalculator.cpp:482-499).
    Each part is a calculator over its own atoms (no masked-out work); the
    parts run in one batched submission.  As the reference's set()
    (src/Scattering/CombinedStructureFactorCalculator.cpp:19-52), building it
    sets every atom's anomalous dispersion to zero; set_anomalous gives the
    parts new per-atom values."""

    def __init__(self, engine, st, parts):
        """parts: [(make, atom_indices)], make(substructure) -> calculator."""
        self.engine = engine
        self.st = st
        self.parts = []
        seen = np.zeros(st.n_atoms, dtype=int)
        for make, idx in parts:
            idx = np.asarray(idx, dtype=np.int64)
            seen[idx] += 1
            sub = st.subset(idx)
            self.parts.append((make(sub), idx))
        if not np.all(seen == 1):
            raise DsfError("every atom must belong to exactly one part")
        self.set_anomalous(np.zeros(st.n_atoms, dtype=np.complex128))

    def set_anomalous(self, anomalous):
        """Per-atom f' + i f'' in the whole structure's atom order, handed to
        each part for its own atoms (CombinedStructureFactorCalculator::setAnomalous)."""
        a = np.asarray(anomalous, dtype=np.complex128).reshape(-1)
        if len(a) != self.st.n_atoms:
            raise DsfError("anomalous dispersion size differs from the atom count")
        for c, idx in self.parts:
            c.set_anomalous(a[idx])

    def calculate(self, dtdf, precision=DSF_FP64, derivatives=("xyz", "adp", "occ"), atoms=None):
        calcs = [c for c, _ in self.parts]
        at = None
        if atoms is not None:
            xyz, adp, occ = atoms
            xyz = np.asarray(xyz).reshape(-1, 3)
            adp6 = adp if isinstance(adp, np.ndarray) and adp.shape == (self.st.n_atoms, 6) else None
            if adp6 is None:
                adp6 = np.zeros((self.st.n_atoms, 6))
                for i, a in enumerate(adp):
                    adp6[i, :len(a)] = a
            occ = np.asarray(occ)
            at = [(xyz[idx], adp6[idx], occ[idx]) for _, idx in self.parts]
        res = self.engine.calculate_batch(calcs, [dtdf] * len(calcs), precision=precision, derivatives=derivatives,
                                          atoms=at)
        n = self.st.n_atoms
        f = np.zeros(len(self.st.hkl), dtype=np.complex128)
        d_xyz, d_adp, d_occ = np.zeros((n, 3)), np.zeros((n, 6)), np.zeros(n)
        for (c, idx), r in zip(self.parts, res):
            f += r["f"]
            d_xyz[idx] = r["d_xyz"]
            d_adp[idx] = r["d_adp"]
            d_occ[idx] = r["d_occ"]
        nadp = self.st.n_adp()
        return dict(f=f, d_xyz=d_xyz, d_adp=[d_adp[i, :nadp[i]] for i in range(n)], d_occ=d_occ)

    def close(self):
        for c, _ in self.parts:
            c.close()


def tsc_load(path):
    """The rows of a .tsc file: (hkl [n][3] int, form factors [n][n_atoms] complex)."""
    L = library()
    na, nr = C.c_int(0), C.c_int(0)
    rc = L.dsf_tsc_load(os.fsencode(path), C.byref(na), C.byref(nr), None, None, 0)
    if rc != 0:
        raise DsfError(f"dsf_tsc_load failed with status {rc}")
    hkl = np.zeros((nr.value, 3), dtype=np.int32)
    val = np.zeros((nr.value, na.value, 2))
    rc = L.dsf_tsc_load(os.fsencode(path), C.byref(na), C.byref(nr), hkl.ctypes.data_as(_P(C.c_int)),
                        val.ctypes.data_as(_P(C.c_double)), nr.value)
    if rc != 0:
        raise DsfError(f"dsf_tsc_load failed with status {rc}")
    return hkl, val[..., 0] + 1j * val[..., 1]


def write_tsc(path, labels, hkl, ff, title="form factors"):
    """Writes a .tsc file (header, then "h k l re,im ..." per row; full precision)."""
    with open(path, "w") as fh:
        fh.write(f"TITLE: {title}\nAD: FALSE\nSYMM: expanded\nSCATTERERS: {' '.join(labels)}\nDATA:\n")
        for h, row in zip(np.asarray(hkl), np.asarray(ff)):
            fh.write(f"{int(h[0])} {int(h[1])} {int(h[2])} " +
                     " ".join(f"{float(v.real)!r},{float(v.imag)!r}" for v in row) + "\n")
