"""Batched submission (dsf_calculate_batch / dsf_calculate_batch_device):
many structures of one engine give the same results as one call each.

FP64: equal to the single calls up to the order of the FP64 atomic sums.
FP32: the batch chooses its own reflection chunks (and so its own line
re-anchoring points), so it is compared with the oracle at the FP32 bar
(sum|dF|/sum|F| <= 1e-6, per-class derivative norm error <= 1e-5)."""
import numpy as np
import pytest

from conftest import rel_f, rel_norm
from discamb_gb300 import api, workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64, FP32 = api.DSF_FP64, api.DSF_FP32_BULK


def mixed_set():
    """HC structures of every kernel shape (operation count, coset form,
    ADP kind), an IAM and a tabulated structure."""
    cases = []
    for i, sg in enumerate(["P1", "P-1", "P21", "P21/c", "P212121", "C2/c", "P41", "P43212", "Pbca"]):
        cases.append(("hc", W.small_case(sg, n_atoms=5 + i, stol_max=0.5, seed=300 + i, aniso=bool(i % 2))))
    return cases


def iam_case():
    st = W.small_case("P21/c", n_atoms=7, stol_max=0.5, seed=351)
    ntype = int(st.atom_type.max()) + 1
    rng = np.random.default_rng(5)
    iam = dict(ngauss=np.full(ntype, 4, np.int32), a=rng.uniform(0.5, 3, (ntype, 5)),
               b=rng.uniform(0.5, 30, (ntype, 5)), c=rng.uniform(0, 0.5, ntype))
    return st, iam


def table_case():
    st = W.small_case("P212121", n_atoms=6, stol_max=0.45, seed=352)
    rot, _ = api.all_ops_mod_centering(st.sg)
    rng = np.random.default_rng(6)
    t = rng.normal(size=(st.n_hkl, len(rot), st.n_atoms)) + 1j * rng.normal(size=(st.n_hkl, len(rot), st.n_atoms))
    return st, t


def make_calcs(engine):
    calcs, oracles = [], []
    for kind, st in mixed_set():
        calcs.append(api.HcCalculator(engine, st))
        oracles.append(lambda st=st, mp=False: O.compute(st, multipoles=mp))
    st, iam = iam_case()
    calcs.append(api.IamCalculator(engine, st, iam))
    oracles.append(lambda st=st, iam=iam, mp=False: O.compute(st, model="iam", iam=iam))
    st, t = table_case()
    calcs.append(api.TabulatedCalculator(engine, st, t))
    oracles.append(lambda st=st, t=t, mp=False: O.compute(st, model="table", table=t))
    return calcs, oracles


@pytest.mark.parametrize("prec", [FP64, FP32])
def test_batch_matches_single_calls(engine, prec):
    calcs, oracles = make_calcs(engine)
    dtdfs = [c.st.dtdf for c in calcs]
    batch = engine.calculate_batch(calcs, dtdfs, precision=prec)
    for c, o, b in zip(calcs, oracles, batch):
        if prec == FP64:
            a = c.calculate(c.st.dtdf, precision=prec, adp_layout="padded")
            assert rel_f(b["f"], a["f"]) < 1e-12
            for k in ("d_xyz", "d_adp", "d_occ"):
                assert rel_norm(b[k], a[k]) < 1e-12, k
        else:
            ref = o()
            nadp = c.st.n_adp()
            adp = [b["d_adp"][i, :nadp[i]] for i in range(c.n_atoms)]
            assert rel_f(b["f"], ref["f"]) < 1e-6
            assert rel_norm(b["d_xyz"], ref["d_xyz"]) < 1e-5
            assert rel_norm(adp, ref["d_adp"]) < 1e-5
            assert rel_norm(b["d_occ"], ref["d_occ"]) < 1e-5
    for c in calcs:
        c.close()


def test_batch_with_multipole_adjoint_and_repeats(engine):
    # HC structures with the multipole adjoint launch per structure inside the batch
    sts = [W.small_case(sg, n_atoms=6, stol_max=0.5, seed=360 + i) for i, sg in enumerate(["P21/c", "P212121", "P1"])]
    calcs = [api.HcCalculator(engine, st) for st in sts]
    for rep in range(2):
        batch = engine.calculate_batch(calcs, [st.dtdf for st in sts], precision=FP32, multipoles=True)
        for st, b in zip(sts, batch):
            o = O.compute(st, multipoles=True)
            assert rel_f(b["f"], o["f"]) < 1e-6
            for k in ("d_pval", "d_plm", "d_kappa", "d_kappa_p"):
                assert rel_norm(b[k], o[k]) < 1e-5, k
    for c in calcs:
        c.close()


def test_batch_larger_than_one_launch(engine):
    # more structures of one kernel shape than one batched launch holds (48)
    sts = [W.small_case("P21/c", n_atoms=3, stol_max=0.3, seed=400 + i) for i in range(53)]
    calcs = [api.HcCalculator(engine, st) for st in sts]
    batch = engine.calculate_batch(calcs, [st.dtdf for st in sts], precision=FP64)
    for c, st, b in zip(calcs, sts, batch):
        a = c.calculate(st.dtdf, precision=FP64)
        assert rel_f(b["f"], a["f"]) < 1e-12
        assert rel_norm(b["d_xyz"], a["d_xyz"]) < 1e-12
    # FP32: all 53 in batched launches (two of them)
    batch = engine.calculate_batch(calcs, [st.dtdf for st in sts], precision=FP32)
    for st, b in zip(sts[::13], batch[::13]):
        o = O.compute(st)
        assert rel_f(b["f"], o["f"]) < 1e-6
        assert rel_norm(b["d_xyz"], o["d_xyz"]) < 1e-5
    for c in calcs:
        c.close()


def test_large_host_batch_in_overlapped_groups(engine):
    # 20 structures of about 130k reflections: more than 64 MB of host inputs and outputs, so the call runs in
    # groups whose host copies overlap the GPU work of the others; the results equal one call each (FP32: at
    # the FP32 bar, since batch and single call re-anchor the line recurrence at different reflections)
    sts = [W.small_case("P21/c", n_atoms=4, stol_max=2.2, seed=500 + i, aniso=bool(i % 2)) for i in range(20)]
    assert sum(32 * st.n_hkl + 8 * 38 * st.n_atoms for st in sts) >= 64 << 20
    calcs = [api.HcCalculator(engine, st) for st in sts]
    for prec, tol_f, tol_d in ((FP64, 1e-12, 1e-12), (FP32, 1e-6, 1e-5)):
        batch = engine.calculate_batch(calcs, [st.dtdf for st in sts], precision=prec)
        for c, st, b in zip(calcs, sts, batch):
            a = c.calculate(st.dtdf, precision=prec, adp_layout="padded")
            assert rel_f(b["f"], a["f"]) < tol_f
            for k in ("d_xyz", "d_adp", "d_occ"):
                assert rel_norm(b[k], a[k]) < tol_d, k
    # derivative outputs the flags leave out are not written
    batch = engine.calculate_batch(calcs, [st.dtdf for st in sts], precision=FP32, derivatives=("xyz",))
    for b in batch:
        assert np.all(b["d_adp"] == 0) and np.all(b["d_occ"] == 0)
        assert np.abs(b["d_xyz"]).max() > 0
    for c in calcs:
        c.close()


def test_batch_rejects_foreign_structures(engine):
    st = W.small_case("P21", n_atoms=3, stol_max=0.3, seed=450)
    other = api.Engine(0)
    try:
        a = api.HcCalculator(engine, st)
        b = api.HcCalculator(other, st)
        with pytest.raises(api.DsfError):
            engine.calculate_batch([a, b], [st.dtdf, st.dtdf])
        a.close()
        b.close()
    finally:
        other.close()


def test_device_table_matches_host_table_and_oracle(engine):
    torch = pytest.importorskip("torch")
    for i, (na, nh) in enumerate([(12, 2100), (40, 2500), (7, 3000)]):
        st = W.config4_crystal(na, nh, seed=5000 + i)
        t = W.config4_table(st, np.random.default_rng(5000 + i))
        dev = torch.device("cuda", 0)
        tt = torch.tensor(np.stack([t.real, t.imag], -1), dtype=torch.float32, device=dev).contiguous()
        torch.cuda.synchronize()  # the engine gathers the table on its own stream
        a = api.TabulatedCalculator(engine, st, table_device=tt.data_ptr())
        del tt
        torch.cuda.synchronize()
        b = api.TabulatedCalculator(engine, st, table=t.astype(np.complex64), fp32_table=True)
        for prec in (FP32, FP64):
            ra = a.calculate(st.dtdf, precision=prec)
            rb = b.calculate(st.dtdf, precision=prec)
            assert rel_f(ra["f"], rb["f"]) < 1e-13
            assert rel_norm(ra["d_xyz"], rb["d_xyz"]) < 1e-12
        o = O.compute(st, model="table", table=t.astype(np.complex64).astype(np.complex128))
        r = a.calculate(st.dtdf, precision=FP32)
        assert rel_f(r["f"], o["f"]) < 1e-6
        assert rel_norm(r["d_xyz"], o["d_xyz"]) < 1e-5 and rel_norm(r["d_adp"], o["d_adp"]) < 1e-5
        # the FP64 form reads the complex64 table widened: FP64 accuracy on those values
        r = a.calculate(st.dtdf, precision=FP64)
        assert rel_f(r["f"], o["f"]) < 1e-10
        a.close()
        b.close()


def test_tabulated_batch_device_path(engine):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    calcs, sts, tabs = [], [], []
    for i, (na, nh) in enumerate([(12, 2100), (40, 2500), (7, 3000), (25, 2200)]):
        st = W.config4_crystal(na, nh, seed=5100 + i)
        t = W.config4_table(st, np.random.default_rng(5100 + i)).astype(np.complex64)
        tt = torch.tensor(np.stack([t.real, t.imag], -1), dtype=torch.float32, device=dev).contiguous()
        torch.cuda.synchronize()
        calcs.append(api.TabulatedCalculator(engine, st, table_device=tt.data_ptr()))
        sts.append(st)
        tabs.append(t.astype(np.complex128))
    dt = [torch.tensor(np.stack([st.dtdf.real, st.dtdf.imag], 1), dtype=torch.float64, device=dev) for st in sts]
    outs = [{"f": torch.zeros(st.n_hkl, 2, dtype=torch.float64, device=dev),
             "d_xyz": torch.zeros(st.n_atoms, 3, dtype=torch.float64, device=dev)} for st in sts]
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.synchronize()
    engine.calculate_batch_device(calcs, [d.data_ptr() for d in dt],
                                  [{k: v.data_ptr() for k, v in o.items()} for o in outs],
                                  precision=FP32, derivatives=("xyz",), stream=stream.cuda_stream)
    stream.synchronize()
    for st, t, o in zip(sts, tabs, outs):
        ref = O.compute(st, model="table", table=t)
        f = o["f"].cpu().numpy()
        assert rel_f(f[:, 0] + 1j * f[:, 1], ref["f"]) < 1e-6
        assert rel_norm(o["d_xyz"].cpu().numpy(), ref["d_xyz"]) < 1e-5
    for c in calcs:
        c.close()


def test_combined_hc_and_iam_atoms(engine):
    # TAAM-style split: multipolar atoms on the HC model, the others IAM
    st = W.small_case("P21/c", n_atoms=9, stol_max=0.5, seed=470)
    hc_idx, iam_idx = [0, 1, 2, 4, 7], [3, 5, 6, 8]
    sub_iam = st.subset(iam_idx)
    ntype = int(sub_iam.atom_type.max()) + 1
    rng = np.random.default_rng(8)
    iam = dict(ngauss=np.full(ntype, 4, np.int32), a=rng.uniform(0.5, 3, (ntype, 5)),
               b=rng.uniform(0.5, 30, (ntype, 5)), c=rng.uniform(0, 0.5, ntype))
    comb = api.CombinedCalculator(engine, st, [(lambda s: api.HcCalculator(engine, s), hc_idx),
                                               (lambda s: api.IamCalculator(engine, s, iam), iam_idx)])
    xyz = st.xyz + 0.002
    for prec, tf, tg in ((FP64, 1e-10, 1e-10), (FP32, 1e-6, 1e-5)):
        r = comb.calculate(st.dtdf, precision=prec, atoms=(xyz, st.adp, st.occupancy))
        s1, s2 = st.subset(hc_idx), st.subset(iam_idx)
        s1.xyz, s2.xyz = xyz[hc_idx], xyz[iam_idx]
        # the combined calculator starts with zero anomalous dispersion, as the reference's does
        s1.anomalous, s2.anomalous = np.zeros(s1.n_atoms, complex), np.zeros(s2.n_atoms, complex)
        o1, o2 = O.compute(s1), O.compute(s2, model="iam", iam=iam)
        assert rel_f(r["f"], o1["f"] + o2["f"]) < tf
        ref_xyz = np.zeros((st.n_atoms, 3))
        ref_xyz[hc_idx], ref_xyz[iam_idx] = o1["d_xyz"], o2["d_xyz"]
        assert rel_norm(r["d_xyz"], ref_xyz) < tg
        ref_adp = [None] * st.n_atoms
        for k, i in enumerate(hc_idx):
            ref_adp[i] = o1["d_adp"][k]
        for k, i in enumerate(iam_idx):
            ref_adp[i] = o2["d_adp"][k]
        assert rel_norm(r["d_adp"], ref_adp) < tg
    comb.close()


def test_multipole_derivatives_reduced_to_types(engine):
    torch = pytest.importorskip("torch")
    st = W.build_structure(cell=(11.0, 12.0, 13.0, 90.0, 101.0, 90.0), sg_symbol="P21/c",
                           elements=["C", "C", "N", "O", "C", "N", "O", "C", "H", "H"],
                           rng=np.random.default_rng(480), n_types=5, stol_max=0.5)
    calc = api.HcCalculator(engine, st)
    dev = torch.device("cuda", 0)
    n, nt = st.n_atoms, len(st.types)
    g = torch.tensor(np.stack([st.dtdf.real, st.dtdf.imag], 1), dtype=torch.float64, device=dev)
    f = torch.zeros(st.n_hkl, 2, dtype=torch.float64, device=dev)
    pa = {k: torch.zeros(n, w, dtype=torch.float64, device=dev)
          for k, w in (("d_pval", 1), ("d_plm", 25), ("d_kappa", 1), ("d_kappa_prime", 1))}
    pt = {k: torch.zeros(nt, w, dtype=torch.float64, device=dev)
          for k, w in (("d_pval", 1), ("d_plm", 25), ("d_kappa", 1), ("d_kappa_prime", 1))}
    torch.cuda.synchronize()
    calc.calculate_device(g.data_ptr(), {"f": f.data_ptr(), **{k: v.data_ptr() for k, v in pa.items()}},
                          precision=FP64, derivatives=(), multipoles=True)
    calc.reduce_to_types({k: v.data_ptr() for k, v in pa.items()}, {k: v.data_ptr() for k, v in pt.items()})
    torch.cuda.synchronize()
    o = O.compute(st, multipoles=True)
    for k, ko in (("d_pval", "d_pval"), ("d_plm", "d_plm"), ("d_kappa", "d_kappa"), ("d_kappa_prime", "d_kappa_p")):
        ref = np.zeros((nt,) + np.asarray(o[ko]).shape[1:])
        np.add.at(ref, st.atom_type, np.asarray(o[ko]))
        got = pt[k].cpu().numpy().reshape(ref.shape)
        assert rel_norm(got, ref) < 1e-10, k
    calc.close()


def test_submit_and_poll(engine):
    # asynchronous calls (dsf_submit / dsf_poll) on two structures at once equal the synchronous ones; a second
    # submit on a structure with a pending call is refused; a failed call (stalled producer) reports through poll
    sts = [W.small_case("P212121", n_atoms=40, stol_max=0.6, seed=91), W.config1(n_atoms=800)]
    calcs = [api.HcCalculator(engine, st) for st in sts]
    want = [c.calculate(st.dtdf, precision=FP32, adp_layout="padded") for c, st in zip(calcs, sts)]
    atoms = [(st.xyz, st.adp_array(), st.occupancy) for st in sts]
    tickets = [c.submit(st.dtdf, precision=FP32, atoms=a, adp_layout="padded") for c, st, a in zip(calcs, sts, atoms)]
    with pytest.raises(api.DsfError, match="pending"):
        calcs[0].submit(sts[0].dtdf, precision=FP32)
    got = [t.wait() for t in tickets]
    for g, w in zip(got, want):
        assert rel_f(g["f"], w["f"]) < 1e-12
        assert rel_norm(g["d_xyz"], w["d_xyz"]) < 1e-12 and rel_norm(g["d_adp"], w["d_adp"]) < 1e-12
    calcs[0].debug_stall_next_call()
    t = calcs[0].submit(sts[0].dtdf, precision=FP32)
    with pytest.raises(api.DsfError, match="ran out"):
        t.wait()
    assert rel_f(calcs[0].calculate(sts[0].dtdf, precision=FP32)["f"], want[0]["f"]) < 1e-12
    for c in calcs:
        c.close()


@pytest.mark.parametrize("prec,tf,tg", [(FP64, 1e-10, 1e-10), (FP32, 1e-6, 1e-5)])
def test_combined_calculator_matches_reference(engine, prec, tf, tg):
    # the reference's CombinedStructureFactorCalculator with TAAM's split: non-H atoms on AnyHcCalculator, H atoms
    # on AnyIamCalculator (IT92), anomalous dispersion zeroed by the combined calculator
    from conftest import combined_parts, load_fixture, ref_adp_list
    st, d = load_fixture("combined_taam_p21c")
    hc, ia, s1, s2, iam = combined_parts(st, d)

    def make_iam(sub):
        sub.atom_type = sub.atom_wfn.copy()
        return api.IamCalculator(engine, sub, iam)

    comb = api.CombinedCalculator(engine, st, [(lambda s: api.HcCalculator(engine, s), hc), (make_iam, ia)])
    r = comb.calculate(st.dtdf, precision=prec)
    assert rel_f(r["f"], d["ref_f"]) < tf, rel_f(r["f"], d["ref_f"])
    assert rel_norm(r["d_xyz"], d["ref_d_xyz"]) < tg
    assert rel_norm(r["d_adp"], ref_adp_list(st, d)) < tg
    assert rel_norm(r["d_occ"], d["ref_d_occ"]) < tg
    comb.close()
