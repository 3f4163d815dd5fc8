"""The allocation-free IAM entry point (dsf_iam_calculate_noalloc).

Some callers cannot allocate device memory: a host program that owns every
device allocation through its own pool, or a refinement loop that must not
allocate (and so must not risk the device-wide synchronisation that
cudaMalloc and cudaFree can bring) inside its per-cycle loop.  The entry
point serves them from a static device array.  These tests call it through
the C ABI and compare it with the allocating entry point (an IAM structure
through dsf_calculate) on the same inputs and the same symmetry descriptor,
on two calls in a row, and with the reference's own result where a fixture
holds one; they also check that a warmed call leaves the device's free
memory unchanged.  The file sorts last so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_fixture, rel_f, rel_norm, ref_adp_list

pytestmark = pytest.mark.gpu

TOL = {0: (1e-10, 1e-10), 1: (1e-6, 1e-5)}


def _iam(d):
    return dict(ngauss=d["iam_ngauss"], a=d["iam_a"], b=d["iam_b"], c=d["iam_c"])


def _entry_point(lib):
    from discamb_gb300 import api
    fn = lib.dsf_iam_calculate_noalloc
    fn.argtypes = [C.POINTER(api._Sym), C.POINTER(api._Iam), C.c_int] + [C.c_void_p] * 7 + \
                  [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.POINTER(api._Out), C.c_void_p,
                   C.c_char_p, C.c_int]
    fn.restype = C.c_int
    return fn


def _model(iam):
    from discamb_gb300 import api
    model = api._Iam()
    model.n_types = len(iam["c"])
    keep = [np.ascontiguousarray(iam["ngauss"], dtype=np.int32), np.ascontiguousarray(iam["a"], dtype=np.float64),
            np.ascontiguousarray(iam["b"], dtype=np.float64), np.ascontiguousarray(iam["c"], dtype=np.float64)]
    model.n_gauss = keep[0].ctypes.data_as(C.POINTER(C.c_int))
    model.a = keep[1].ctypes.data_as(C.POINTER(C.c_double))
    model.b = keep[2].ctypes.data_as(C.POINTER(C.c_double))
    model.c = keep[3].ctypes.data_as(C.POINTER(C.c_double))
    return model, keep


def _device_inputs(torch, st):
    dev = torch.device("cuda", 0)
    t = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=dev)  # noqa: E731
    x = dict(atom_type=t(st.atom_type, torch.int32), adpk=t(st.n_adp(), torch.int32),
             xyz=t(st.xyz, torch.float64), adp=t(st.adp_array(), torch.float64),
             occ=t(st.occupancy, torch.float64), mult=t(np.asarray(st.multiplicity, dtype=np.float64), torch.float64),
             hkl=t(st.hkl, torch.int32), dtdf=t(np.stack([st.dtdf.real, st.dtdf.imag], 1), torch.float64))
    x["anom"] = None
    if st.anomalous is not None:
        x["anom"] = t(np.stack([np.real(st.anomalous), np.imag(st.anomalous)], 1), torch.float64)
    return x


def _shifted_inversion_case():
    """P-1 with the inversion centre at (1/4, 0, 1/4) (the engine form with a
    phase per reflection) and per-atom anomalous dispersion, on the IT92
    coefficients of the iam_it92 fixture (same five elements)."""
    from discamb_gb300 import workloads as W
    st0, d = load_fixture("iam_it92")
    st = W.small_case("P-1(shift)", n_atoms=6, stol_max=0.55, seed=1201, anomalous_per_atom=True)
    assert [w.label for w in st.wfns] == [w.label for w in st0.wfns]
    st.atom_type = st.atom_wfn.copy()
    return st, _iam(d)


def _case(name):
    if name == "shifted_inversion_anomalous":
        st, iam = _shifted_inversion_case()
        return st, iam, None
    st, d = load_fixture("iam_it92")
    return st, _iam(d), d


CASES = [("iam_it92", "all"),                       # the generic engine's operation list (C2/c)
         ("iam_it92", "engine"),                    # subset + inversion at the origin (C2/c)
         ("shifted_inversion_anomalous", "engine")]  # inversion off the origin, anomalous array given


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name,rep", CASES)
def test_noalloc_matches_allocating_entry_point(engine, name, rep, precision):
    torch = pytest.importorskip("torch")
    from discamb_gb300 import api
    st, iam, d = _case(name)
    ref = api.IamCalculator(engine, st, iam, representation=rep).calculate(st.dtdf, precision=precision)
    sym, keep_sym = api.symmetry_desc(st, rep)
    model, keep_model = _model(iam)
    fn = _entry_point(api.library())
    x = _device_inputs(torch, st)
    n, m = st.n_atoms, st.n_hkl
    nadp = st.n_adp()
    tf, tg = TOL[precision]
    # and the reference's own result where the fixture holds one.  The shifted-inversion case has none: with
    # the inversion taken by the engine, anomalous dispersion enters as the reference's centrosymmetric engine
    # takes it (F = U + c conj(U), HansenCoppens_SF_Engine3.cpp:1920-1935), which differs from the sum over
    # all operations by design; the allocating call with the same descriptor is its check
    golds = [ref]
    if d is not None:
        golds.append(dict(f=d["ref_f"], d_xyz=d["ref_d_xyz"], d_adp=ref_adp_list(st, d), d_occ=d["ref_d_occ"]))
    err = C.create_string_buffer(256)
    # outputs allocated before the first call: the second call must leave the device's free memory unchanged
    outs = []
    for call in range(2):
        o = dict(f=torch.zeros(m, 2, dtype=torch.float64, device="cuda"),
                 d_xyz=torch.zeros(n, 3, dtype=torch.float64, device="cuda"),
                 d_adp=torch.zeros(n, 6, dtype=torch.float64, device="cuda"),
                 d_occ=torch.zeros(n, dtype=torch.float64, device="cuda"))
        outs.append(o)
    stream = torch.cuda.current_stream().cuda_stream
    free_before = None
    for call, o in enumerate(outs):
        out = api._Out()
        out.f, out.d_xyz, out.d_adp, out.d_occ = (o[k].data_ptr() for k in ("f", "d_xyz", "d_adp", "d_occ"))
        torch.cuda.synchronize()
        if call == 1:
            free_before = torch.cuda.mem_get_info()[0]
        rc = fn(C.byref(sym), C.byref(model), n, x["atom_type"].data_ptr(), x["adpk"].data_ptr(),
                x["xyz"].data_ptr(), x["adp"].data_ptr(), x["occ"].data_ptr(), x["mult"].data_ptr(),
                None if x["anom"] is None else x["anom"].data_ptr(),
                m, x["hkl"].data_ptr(), x["dtdf"].data_ptr(), precision, 7, C.byref(out), stream, err, 256)
        assert rc == 0, err.value.decode()
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before, "the allocation-free call changed free memory"
        fz = o["f"].cpu().numpy()
        fz = fz[:, 0] + 1j * fz[:, 1]
        gaa = o["d_adp"].cpu().numpy()
        r = dict(f=fz, d_xyz=o["d_xyz"].cpu().numpy(), d_adp=[gaa[i, :nadp[i]] for i in range(n)],
                 d_occ=o["d_occ"].cpu().numpy())
        for against in golds:
            assert rel_f(r["f"], against["f"]) < tf, (call, rel_f(r["f"], against["f"]))
            for k in ("d_xyz", "d_adp", "d_occ"):
                assert rel_norm(r[k], against[k]) < tg, (call, k, rel_norm(r[k], against[k]))


def _call_with(fn, sym, model, err, n_atoms=10_000_000, n_hkl=1_000_000):
    """A call that returns before any device pointer is read: the symmetry
    checks come first and the default sizes are over the scratch limit, so
    the call returns an error either way (the pointers are never
    dereferenced)."""
    from discamb_gb300 import api
    out = api._Out()
    out.f = 1
    dummy = C.c_void_p(1)
    return fn(C.byref(sym), C.byref(model), n_atoms, dummy, dummy, dummy, dummy, dummy, dummy, None,
              n_hkl, dummy, dummy, 0, 7, C.byref(out), None, err, 256)


def test_noalloc_rejects_oversized_problems_and_bad_symmetry(engine):
    from discamb_gb300 import api
    fn = _entry_point(api.library())
    st, d = load_fixture("iam_it92")
    model, keep = _model(_iam(d))
    err = C.create_string_buffer(256)
    sym, keep_sym = api.symmetry_desc(st, "all")
    assert _call_with(fn, sym, model, err) == 1  # DSF_ERR_ARGUMENT
    assert b"scratch" in err.value
    sym.centering = b"H"  # rejected as dsf_structure_create_* rejects it
    assert _call_with(fn, sym, model, err) == 1
    assert b"centering" in err.value
    sym, keep_sym = api.symmetry_desc(st, "engine")
    sym.inversion_translation[0] = 0.01
    assert _call_with(fn, sym, model, err) == 1
    assert b"inversion" in err.value
    sym, keep_sym = api.symmetry_desc(st, "all")
    sym.cell[1] = 0.0
    assert _call_with(fn, sym, model, err) == 1
    assert b"cell" in err.value
