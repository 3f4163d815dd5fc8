"""The C++ host layer (include/dsf_calculator.hpp): the reference's
SfCalculator calls (whole set, structure factors only, single h, form factors,
setAnomalous, getModelInformation, error on a size mismatch) on a reference fixture, through a small C++ driver
(tests/cpp/calculator_driver.cpp) built with g++ against the engine library."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import REPO, load_fixture, ref_adp_list, rel_f, rel_norm
from discamb_gb300 import api

DRIVER = os.path.join(REPO, "tests", "cpp", "calculator_driver.cpp")
INC = os.path.join(REPO, "include")


def test_header_compiles_standalone():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    subprocess.check_call([gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-I", INC, DRIVER])


@pytest.mark.gpu
def test_cpp_calculator_matches_reference(engine, tmp_path):
    from discamb_gb300.build import LIB
    so = str(tmp_path / "libdrv.so")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I", INC, DRIVER, "-o", so,
                           "-L", os.path.dirname(LIB), "-ldsf_gb300", "-Wl,-rpath," + os.path.dirname(LIB)])
    drv = C.CDLL(so)
    drv.drv_error.restype = C.c_char_p
    st, d = load_fixture("hc_anomalous_mask")  # P2_1/c, per-atom anomalous dispersion, one excluded atom
    sym, k1 = api.symmetry_desc(st)
    model, k2 = api._hc_desc(st)
    atoms, k3 = api._atoms_desc(st)
    n, m = st.n_atoms, st.n_hkl
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    xyz = np.ascontiguousarray(st.xyz, dtype=np.float64)
    adp = np.ascontiguousarray(st.adp_array(), dtype=np.float64)
    occ = np.ascontiguousarray(st.occupancy, dtype=np.float64)
    hkl = np.ascontiguousarray(st.hkl, dtype=np.int32)
    g = np.ascontiguousarray(np.stack([st.dtdf.real, st.dtdf.imag], 1))
    inc = np.ascontiguousarray(st.include_mask().astype(np.int32))
    f, f_only = np.zeros((m, 2)), np.zeros((m, 2))
    dx, da, do = np.zeros((n, 3)), np.zeros((n, 6)), np.zeros(n)
    f1, d1x, d1a, d1o, ff = np.zeros(2), np.zeros((n, 3, 2)), np.zeros((n, 6, 2)), np.zeros((n, 2)), np.zeros((n, 2))
    rc = drv.drv_hc(0, C.byref(sym), C.byref(model), C.byref(atoms), api.DSF_FP64, P(xyz), P(adp), P(occ), m, P(hkl),
                    P(g), P(inc), P(f), P(dx), P(da), P(do), P(f_only), P(f1), P(d1x), P(d1a), P(d1o), P(ff))
    assert rc == 0, drv.drv_error().decode()
    fc = f[:, 0] + 1j * f[:, 1]
    nadp = st.n_adp()
    assert rel_f(fc, d["ref_f"]) < 1e-10
    assert rel_norm(dx, d["ref_d_xyz"]) < 1e-10
    assert rel_norm([da[i, :nadp[i]] for i in range(n)], ref_adp_list(st, d)) < 1e-10
    assert rel_norm(do, d["ref_d_occ"]) < 1e-10
    assert rel_f(f_only[:, 0] + 1j * f_only[:, 1], d["ref_f"]) < 1e-10
    # single h at hkl[0]: F equals the whole-set F there, the complex dF/dp equal the Python binding's single-h call
    assert abs(complex(*f1) - fc[0]) <= 1e-10 * max(1.0, abs(fc[0]))
    calc = api.HcCalculator(engine, st)
    one = calc.calculate_at_hkl(st.hkl[0], include=inc)
    assert np.abs(d1x[..., 0] + 1j * d1x[..., 1] - one["d_xyz"]).max() <= 1e-10 * np.abs(one["d_xyz"]).max()
    assert np.abs(d1o[:, 0] + 1j * d1o[:, 1] - one["d_occ"]).max() <= 1e-10 * np.abs(one["d_occ"]).max()
    ffp = calc.form_factors(st.hkl[1], include=inc)
    assert np.abs(ff[:, 0] + 1j * ff[:, 1] - ffp).max() <= 1e-12 * np.abs(ffp).max()
    calc.close()
