"""The allocation-free IAM entry point (dsf_iam_calculate_noalloc), for
callers that cannot allocate device memory, against the allocating entry
point (dsf_calculate through an IAM structure) on the same inputs, through
the C ABI, on two calls in a row.  Kept in a file of its own that pytest
collects last."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_fixture, rel_f, rel_norm

pytestmark = pytest.mark.gpu

TOL = {0: (1e-10, 1e-10), 1: (1e-6, 1e-5)}


def _iam(d):
    return dict(ngauss=d["iam_ngauss"], a=d["iam_a"], b=d["iam_b"], c=d["iam_c"])


def _device_inputs(torch, st):
    dev = torch.device("cuda", 0)
    t = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=dev)  # noqa: E731
    return dict(
        atom_type=t(st.atom_type, torch.int32), adpk=t(st.n_adp(), torch.int32),
        xyz=t(st.xyz, torch.float64), adp=t(st.adp_array(), torch.float64),
        occ=t(st.occupancy, torch.float64), mult=t(np.asarray(st.multiplicity, dtype=np.float64), torch.float64),
        hkl=t(st.hkl, torch.int32), dtdf=t(np.stack([st.dtdf.real, st.dtdf.imag], 1), torch.float64))


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_matches_allocating_entry_point(engine, precision):
    torch = pytest.importorskip("torch")
    from discamb_gb300 import api
    st, d = load_fixture("iam_it92")
    iam = _iam(d)
    ref = api.IamCalculator(engine, st, iam).calculate(st.dtdf, precision=precision)

    lib = api.library()
    sym, keep_sym = api.symmetry_desc(st, "all")
    model = api._Iam()
    model.n_types = len(iam["c"])
    arrs = [np.ascontiguousarray(iam["ngauss"], dtype=np.int32), np.ascontiguousarray(iam["a"], dtype=np.float64),
            np.ascontiguousarray(iam["b"], dtype=np.float64), np.ascontiguousarray(iam["c"], dtype=np.float64)]
    model.n_gauss = arrs[0].ctypes.data_as(C.POINTER(C.c_int))
    model.a = arrs[1].ctypes.data_as(C.POINTER(C.c_double))
    model.b = arrs[2].ctypes.data_as(C.POINTER(C.c_double))
    model.c = arrs[3].ctypes.data_as(C.POINTER(C.c_double))
    x = _device_inputs(torch, st)
    n, m = st.n_atoms, st.n_hkl
    fn = lib.dsf_iam_calculate_noalloc
    fn.argtypes = [C.POINTER(api._Sym), C.POINTER(api._Iam), C.c_int] + [C.c_void_p] * 7 + \
                  [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.POINTER(api._Out), C.c_void_p,
                   C.c_char_p, C.c_int]
    err = C.create_string_buffer(256)
    for call in range(2):
        f = torch.zeros(m, 2, dtype=torch.float64, device="cuda")
        gx = torch.zeros(n, 3, dtype=torch.float64, device="cuda")
        ga = torch.zeros(n, 6, dtype=torch.float64, device="cuda")
        go = torch.zeros(n, dtype=torch.float64, device="cuda")
        out = api._Out()
        out.f, out.d_xyz, out.d_adp, out.d_occ = f.data_ptr(), gx.data_ptr(), ga.data_ptr(), go.data_ptr()
        rc = fn(C.byref(sym), C.byref(model), n, x["atom_type"].data_ptr(), x["adpk"].data_ptr(),
                x["xyz"].data_ptr(), x["adp"].data_ptr(), x["occ"].data_ptr(), x["mult"].data_ptr(), None,
                m, x["hkl"].data_ptr(), x["dtdf"].data_ptr(), precision, 7, C.byref(out),
                torch.cuda.current_stream().cuda_stream, err, 256)
        assert rc == 0, err.value.decode()
        torch.cuda.synchronize()
        fz = f.cpu().numpy()
        fz = fz[:, 0] + 1j * fz[:, 1]
        nadp = st.n_adp()
        gaa = ga.cpu().numpy()
        tf, tg = TOL[precision]
        assert rel_f(fz, ref["f"]) < tf, (call, rel_f(fz, ref["f"]))
        assert rel_norm(gx.cpu().numpy(), ref["d_xyz"]) < tg
        assert rel_norm([gaa[i, :nadp[i]] for i in range(n)], ref["d_adp"]) < tg
        assert rel_norm(go.cpu().numpy(), ref["d_occ"]) < tg


def test_noalloc_rejects_oversized_problems(engine):
    from discamb_gb300 import api
    lib = api.library()
    st, d = load_fixture("iam_it92")
    sym, keep = api.symmetry_desc(st, "all")
    iam = _iam(d)
    model = api._Iam()
    model.n_types = len(iam["c"])
    ng = np.ascontiguousarray(iam["ngauss"], dtype=np.int32)
    model.n_gauss = ng.ctypes.data_as(C.POINTER(C.c_int))
    fn = lib.dsf_iam_calculate_noalloc
    fn.argtypes = [C.POINTER(api._Sym), C.POINTER(api._Iam), C.c_int] + [C.c_void_p] * 7 + \
                  [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.POINTER(api._Out), C.c_void_p,
                   C.c_char_p, C.c_int]
    out = api._Out()
    out.f = 1  # never dereferenced: the size check comes first
    err = C.create_string_buffer(256)
    dummy = C.c_void_p(1)
    rc = fn(C.byref(sym), C.byref(model), 10_000_000, dummy, dummy, dummy, dummy, dummy, dummy, None,
            1_000_000, dummy, dummy, 0, 7, C.byref(out), None, err, 256)
    assert rc == 1  # DSF_ERR_ARGUMENT
    assert b"scratch" in err.value
