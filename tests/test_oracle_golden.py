"""The CPU oracle against the reference's own outputs (golden fixtures
written by tests/golden/make_golden.py from the reference build)."""
import numpy as np
import pytest

from conftest import fixture_names, load_fixture, rel_f, rel_norm, ref_adp_list
from oracle import oracle as O

# hc_*: Engine3; dvs_*: the def-val-symmetrised EngineSymm (same results by construction)
HC = fixture_names("hc_") + fixture_names("dvs_")


@pytest.mark.parametrize("name", HC)
def test_hc_oracle_matches_reference(name):
    st, d = load_fixture(name)
    r = O.compute(st, n_threads=2)
    assert rel_f(r["f"], d["ref_f"]) < 1e-12
    assert rel_norm(r["d_xyz"], d["ref_d_xyz"]) < 1e-11
    assert rel_norm(r["d_adp"], ref_adp_list(st, d)) < 1e-11
    assert rel_norm(r["d_occ"], d["ref_d_occ"]) < 1e-11


def test_multipole_derivatives_match_reference_finite_differences():
    st, d = load_fixture("hc_multipole_fd")
    r = O.compute(st, n_threads=2, multipoles=True)
    assert rel_norm(r["d_pval"], d["ref_d_pval"]) < 1e-8
    assert rel_norm(r["d_plm"], d["ref_d_plm"]) < 1e-8
    assert rel_norm(r["d_kappa"], d["ref_d_kappa"]) < 1e-6
    assert rel_norm(r["d_kappa_p"], d["ref_d_kappa_p"]) < 1e-6


def iam_dict(d):
    return dict(ngauss=d["iam_ngauss"], a=d["iam_a"], b=d["iam_b"], c=d["iam_c"])


@pytest.mark.parametrize("name", fixture_names("iam_"))
def test_iam_oracle_matches_reference(name):
    st, d = load_fixture(name)
    r = O.compute(st, model="iam", iam=iam_dict(d), n_threads=2)
    assert rel_f(r["f"], d["ref_f"]) < 1e-12
    assert rel_norm(r["d_xyz"], d["ref_d_xyz"]) < 1e-11
    assert rel_norm(r["d_adp"], ref_adp_list(st, d)) < 1e-11
    assert rel_norm(r["d_occ"], d["ref_d_occ"]) < 1e-11


def table_all_ops(st, d):
    """[hkl][op][atom] over all operations from the (rotated index -> f) map"""
    lut = {tuple(k): v for k, v in zip(d["table_keys"], d["table_values"])}
    t = np.zeros((st.n_hkl, st.sg.n_total, st.n_atoms), dtype=complex)
    for i, h in enumerate(st.hkl):
        for s, r_ in enumerate(st.sg.rot):
            t[i, s] = lut[tuple(int(v) for v in h @ r_)]
    return t


def test_tabulated_oracle_matches_reference():
    st, d = load_fixture("table_p21c")
    r = O.compute(st, model="table", table=table_all_ops(st, d), n_threads=2)
    assert rel_f(r["f"], d["ref_f"]) < 1e-12
    assert rel_norm(r["d_xyz"], d["ref_d_xyz"]) < 1e-11
    assert rel_norm(r["d_adp"], ref_adp_list(st, d)) < 1e-11
    assert rel_norm(r["d_occ"], d["ref_d_occ"]) < 1e-11


def test_oracle_is_deterministic_across_thread_counts():
    st, d = load_fixture("hc_config0")
    a = O.compute(st, n_threads=1)
    b = O.compute(st, n_threads=3)
    assert rel_f(a["f"], b["f"]) < 1e-15
    assert rel_norm(a["d_xyz"], b["d_xyz"]) < 1e-13


@pytest.mark.parametrize("name", HC)
def test_line_ordered_loop_matches_the_golden_fixtures(name):
    # the benchmark's CPU baseline (the reference engine's line-ordered loop with recurrences)
    st, d = load_fixture(name)
    o = O.compute(st, multipoles=False, loop="lines")
    assert rel_f(o["f"], d["ref_f"]) < 1e-12
    assert rel_norm(o["d_xyz"], d["ref_d_xyz"]) < 1e-11
    assert rel_norm(o["d_adp"], ref_adp_list(st, d)) < 1e-11
    assert rel_norm(o["d_occ"], d["ref_d_occ"]) < 1e-11


def test_line_ordered_loop_multipole_derivatives():
    st, d = load_fixture("hc_multipole_fd")
    a = O.compute(st, multipoles=True)
    b = O.compute(st, multipoles=True, loop="lines")
    for k in ("d_pval", "d_plm", "d_kappa", "d_kappa_p"):
        assert rel_norm(b[k], a[k]) < 1e-11, k


EL = fixture_names("el_")


@pytest.mark.parametrize("loop", ["direct", "lines"])
@pytest.mark.parametrize("name", EL)
def test_electron_scattering_matches_reference(name, loop):
    st, d = load_fixture(name)
    r = O.compute(st, electron_f000=d["electron_f000"], loop=loop)
    assert rel_f(r["f"], d["ref_f"]) < 1e-12
    assert rel_norm(r["d_xyz"], d["ref_d_xyz"]) < 1e-11
    assert rel_norm(r["d_adp"], ref_adp_list(st, d)) < 1e-11
    assert rel_norm(r["d_occ"], d["ref_d_occ"]) < 1e-11


def test_electron_multipole_derivatives_by_finite_differences():
    # F is linear in P_val and P_lm: one central difference of the oracle's own F
    st, d = load_fixture("el_hc_p21c")
    f000 = d["electron_f000"]
    r = O.compute(st, electron_f000=f000, multipoles=True)

    def target(s):
        return float(np.sum((np.conj(s.dtdf) * O.compute(s, electron_f000=f000)["f"]).real))

    import copy
    for a in (0, 3):
        t = st.atom_type[a]
        for q, h in ((None, 1e-2), (6, 1e-2)):
            s1, s2 = copy.deepcopy(st), copy.deepcopy(st)
            if q is None:
                s1.types[t].p_val += h
                s2.types[t].p_val -= h
                ana = r["d_pval"][a]
            else:
                s1.types[t].plm[q] += h
                s2.types[t].plm[q] -= h
                ana = r["d_plm"][a][q]
            fd = (target(s1) - target(s2)) / (2 * h)
            assert abs(fd - ana) <= 1e-8 * max(1.0, abs(ana)), (a, q, fd, ana)


def test_single_h_form_factors_match_reference():
    # the reference's single-h calculateFormFactors (HC: 000 included, one excluded atom; IAM: IT92)
    st, d = load_fixture("ff_hc_p21c")
    o = O.compute(st, form_factors=True)
    assert np.abs(o - d["ref_ff"]).max() <= 1e-11 * np.abs(d["ref_ff"]).max()
    assert np.all(o[:, ~st.include_mask()] == 0)
    st, d = load_fixture("ff_iam_c2c")
    o = O.compute(st, model="iam", iam=iam_dict(d), form_factors=True)
    assert np.abs(o - d["ref_ff"]).max() <= 1e-13 * np.abs(d["ref_ff"]).max()


@pytest.mark.parametrize("name", ["lcs_update_p21c", "lcs_update_p1_cart"])
def test_reference_recomputed_the_lcs_from_the_moved_atoms(name):
    # the fixture's reference result is that of the moved atoms with the LCS of the moved geometry; with the
    # LCS of the set-up geometry instead it differs (so the fixture pins the recomputation)
    st, d = load_fixture(name)
    st.xyz = d["xyz_moved"]
    kept = st.lcs.copy()
    st.lcs = d["ref_lcs_moved"]
    r = O.compute(st, n_threads=2)
    assert rel_f(r["f"], d["ref_f"]) < 1e-12
    assert rel_norm(r["d_xyz"], d["ref_d_xyz"]) < 1e-11
    st.lcs = kept
    assert rel_f(O.compute(st, n_threads=2)["f"], d["ref_f"]) > 1e-6


def test_combined_calculator_fixture_is_the_sum_of_its_parts():
    # the reference's CombinedStructureFactorCalculator (HC atoms + IAM atoms, anomalous dispersion zeroed by the
    # combined calculator): F is the sum of the parts' F, each atom's derivatives come from its own part
    from conftest import combined_parts
    st, d = load_fixture("combined_taam_p21c")
    hc, ia, s1, s2, iam = combined_parts(st, d)
    o1, o2 = O.compute(s1, n_threads=2), O.compute(s2, model="iam", iam=iam, n_threads=2)
    assert rel_f(o1["f"] + o2["f"], d["ref_f"]) < 1e-12
    ref_xyz = d["ref_d_xyz"]
    assert rel_norm(o1["d_xyz"], ref_xyz[hc]) < 1e-11 and rel_norm(o2["d_xyz"], ref_xyz[ia]) < 1e-11
    ref_adp = ref_adp_list(st, d)
    assert rel_norm(o1["d_adp"], [ref_adp[i] for i in hc]) < 1e-11
    assert rel_norm(o2["d_adp"], [ref_adp[i] for i in ia]) < 1e-11
    assert rel_norm(np.concatenate([o1["d_occ"], o2["d_occ"]]), np.concatenate([d["ref_d_occ"][hc], d["ref_d_occ"][ia]])) < 1e-11
