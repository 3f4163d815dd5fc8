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


def _driver(tmp_path):
    from discamb_gb300.build import LIB, build
    build()
    so = str(tmp_path / "libdrv.so")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I", INC, DRIVER, "-o", so,
                           "-L", os.path.dirname(LIB), "-ldsf_gb300", "-Wl,-rpath," + os.path.dirname(LIB)])
    drv = C.CDLL(so)
    drv.drv_error.restype = C.c_char_p
    return drv


LCS = ["lcs_update_p21c", "lcs_update_p1_cart"]


@pytest.mark.parametrize("name", LCS)
def test_lcs_matrices_match_reference(tmp_path, name):
    # host only: the C++ layer's XD local coordinate systems (dsf::lcsMatrix) against the matrices the
    # reference's XdLocalCoordinateSystem computed for the moved geometry, including a left-handed system, a
    # point summed over two atoms and a dummy point
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    drv = _driver(tmp_path)
    st, d = load_fixture(name)
    P = lambda a: np.ascontiguousarray(a).ctypes.data_as(C.c_void_p)  # noqa: E731
    keep = [np.ascontiguousarray(x) for x in (st.cell, d["xyz_moved"], d["lcs_def"], d["lcs_atoms"], d["lcs_dummy"])]
    out = np.zeros((st.n_atoms, 9))
    rc = drv.drv_lcs_matrices(st.n_atoms, P(np.asarray(st.cell, dtype=np.float64)),
                              int(st.xyz_convention == "cartesian"), P(keep[1]), P(keep[2].astype(np.int32)),
                              P(keep[3].astype(np.int32)), P(keep[4]), P(out))
    assert rc == 0, drv.drv_error().decode()
    assert np.abs(out.reshape(-1, 3, 3) - d["ref_lcs_moved"]).max() < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("frozen", [0, 1])
@pytest.mark.parametrize("name", LCS)
def test_cpp_lcs_recomputed_on_update_matches_reference(engine, tmp_path, name, frozen):
    # AnyHcCalculator with local coordinate systems (large-molecule implementation): the calculator is set up on
    # one geometry and called with the atoms moved.  Not frozen, the reference recomputes every LCS from the
    # moved atoms (AnyHcCalculator.cpp:236-244, 319-329); the fixture holds its result.  Frozen, the systems of
    # the set-up geometry stay: checked against the oracle with those systems and the moved atoms.
    from oracle import oracle as O
    drv = _driver(tmp_path)
    st, d = load_fixture(name)
    sym, k1 = api.symmetry_desc(st)
    model, k2 = api._hc_desc(st)
    atoms, k3 = api._atoms_desc(st)
    n, m = st.n_atoms, st.n_hkl
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    arr = dict(xyz=st.xyz, moved=d["xyz_moved"], adp=st.adp_array(), occ=st.occupancy, dummy=d["lcs_dummy"],
               g=np.stack([st.dtdf.real, st.dtdf.imag], 1))
    arr = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in arr.items()}
    ints = dict(defs=d["lcs_def"], list=d["lcs_atoms"], hkl=st.hkl)
    ints = {k: np.ascontiguousarray(v, dtype=np.int32) for k, v in ints.items()}
    f, dx, da, do, lcs = np.zeros((m, 2)), np.zeros((n, 3)), np.zeros((n, 6)), np.zeros(n), np.zeros((n, 9))
    rc = drv.drv_hc_lcs(0, C.byref(sym), C.byref(model), C.byref(atoms), api.DSF_FP64, frozen, P(arr["xyz"]),
                        P(arr["moved"]), P(arr["adp"]), P(arr["occ"]), P(ints["defs"]), P(ints["list"]),
                        P(arr["dummy"]), m, P(ints["hkl"]), P(arr["g"]), P(f), P(dx), P(da), P(do), P(lcs))
    assert rc == 0, drv.drv_error().decode()
    nadp = st.n_adp()
    fc = f[:, 0] + 1j * f[:, 1]
    if frozen:
        assert np.abs(lcs.reshape(-1, 3, 3) - st.lcs).max() < 1e-12
        st.xyz = d["xyz_moved"]
        o = O.compute(st)
        ref = dict(f=o["f"], d_xyz=o["d_xyz"], d_adp=o["d_adp"], d_occ=o["d_occ"])
    else:
        assert np.abs(lcs.reshape(-1, 3, 3) - d["ref_lcs_moved"]).max() < 1e-12
        ref = dict(f=d["ref_f"], d_xyz=d["ref_d_xyz"], d_adp=ref_adp_list(st, d), d_occ=d["ref_d_occ"])
    assert rel_f(fc, ref["f"]) < 1e-10
    assert rel_norm(dx, ref["d_xyz"]) < 1e-10
    assert rel_norm([da[i, :nadp[i]] for i in range(n)], ref["d_adp"]) < 1e-10
    assert rel_norm(do, ref["d_occ"]) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tf,tg", [(api.DSF_FP64, 1e-10, 1e-10), (api.DSF_FP32_BULK, 1e-6, 1e-5)])
def test_cpp_combined_calculator_matches_reference(engine, tmp_path, prec, tf, tg):
    # dsf::CombinedCalculator (HC part + IAM part, one batched submission) against the reference's
    # CombinedStructureFactorCalculator over AnyHcCalculator + AnyIamCalculator (TAAM's split)
    from conftest import combined_parts
    drv = _driver(tmp_path)
    st, d = load_fixture("combined_taam_p21c")
    hc, ia, s1, s2, iam = combined_parts(st, d)
    sym1, k1 = api.symmetry_desc(s1)
    model1, k2 = api._hc_desc(s1)
    atoms1, k3 = api._atoms_desc(s1)
    sym2, k4 = api.symmetry_desc(s2, "all")
    atoms2, k5 = api._atoms_desc(s2, lcs=False)
    model2 = api._Iam()
    model2.n_types = len(iam["c"])
    keep = [np.ascontiguousarray(iam["ngauss"], dtype=np.int32)] + \
           [np.ascontiguousarray(np.asarray(iam[k], dtype=np.float64).reshape(-1)) for k in ("a", "b", "c")]
    model2.n_gauss = keep[0].ctypes.data_as(C.POINTER(C.c_int))
    model2.a, model2.b, model2.c = (x.ctypes.data_as(C.POINTER(C.c_double)) for x in keep[1:])
    n, m = st.n_atoms, st.n_hkl
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    ints = {k: np.ascontiguousarray(v, dtype=np.int32) for k, v in (("hc", hc), ("ia", ia), ("nadp", st.n_adp()),
                                                                     ("hkl", st.hkl))}
    dbl = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in (
        ("xyz", st.xyz), ("adp", st.adp_array()), ("occ", st.occupancy), ("g", np.stack([st.dtdf.real, st.dtdf.imag], 1)))}
    f, dx, da, do = np.zeros((m, 2)), np.zeros((n, 3)), np.zeros((n, 6)), np.zeros(n)
    rc = drv.drv_combined(0, prec, C.byref(sym1), C.byref(model1), C.byref(atoms1), P(ints["hc"]), C.byref(sym2),
                          C.byref(model2), C.byref(atoms2), P(ints["ia"]), n, P(ints["nadp"]), P(dbl["xyz"]),
                          P(dbl["adp"]), P(dbl["occ"]), m, P(ints["hkl"]), P(dbl["g"]), P(f), P(dx), P(da), P(do))
    assert rc == 0, drv.drv_error().decode()
    nadp = st.n_adp()
    assert rel_f(f[:, 0] + 1j * f[:, 1], d["ref_f"]) < tf
    assert rel_norm(dx, d["ref_d_xyz"]) < tg
    assert rel_norm([da[i, :nadp[i]] for i in range(n)], ref_adp_list(st, d)) < tg
    assert rel_norm(do, d["ref_d_occ"]) < tg


def test_reference_side_binding_compiles_against_the_reference_headers(tmp_path):
    # include/reference_binding/GpuSfCalculators.h: the SfCalculator subclasses a maintainer adds to the reference
    # (GpuHcCalculator, GpuIamCalculator, the factory branch), compiled against the reference's own headers
    from oracle import ref
    tree = ref.REF_TREE
    if not tree or not os.path.isdir(os.path.join(tree, "include", "discamb")) or shutil.which("g++") is None:
        pytest.skip("reference tree or g++ absent")
    cfg = tmp_path / "discamb"
    cfg.mkdir()
    # the one header the reference's build generates (three defines; its default configuration)
    (cfg / "discamb_config.h").write_text("#ifndef DISCAMB_DEC_CONFIG_H\n#define DISCAMB_DEC_CONFIG_H\n#endif\n"
                                          "#define HAS_SPH_BESSEL\n")
    src = tmp_path / "use_binding.cpp"
    src.write_text('#include "reference_binding/GpuSfCalculators.h"\n'
                   "discamb::SfCalculator *make(const discamb::Crystal &c, const nlohmann::json &j) {\n"
                   '    return discamb::gb300::createGpuSfCalculator(c, "iam_gb300", j);\n}\n')
    subprocess.check_call(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(tree, "include"),
                           "-I", os.path.join(tree, "third-party"), "-I", str(tmp_path), "-I", INC, str(src)])
