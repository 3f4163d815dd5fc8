"""The tile-shape autotuner (dsf_autotune, dsf_tuning_lookup/save/load):
it picks one of its candidate shapes, later calls take it, the results stay
those of the rule's shape (parity unchanged: only the order of the
cross-block sums differs), and a saved cache gives another engine the same
shape."""
import numpy as np
import pytest

from conftest import rel_f, rel_norm
from discamb_gb300 import api, workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tf,tg", [(api.DSF_FP64, 1e-12, 1e-12), (api.DSF_FP32_BULK, 1e-6, 1e-5)])
def test_autotuned_shape_keeps_the_results(engine, prec, tf, tg):
    st = W.config1(n_atoms=900, d_min=1.9)
    calc = api.HcCalculator(engine, st)
    before = calc.tile_shape(prec)
    assert before == dict(blocks_per_sm=75, ht=0, occupancy=0, tuned=False)
    r0 = calc.calculate(st.dtdf, precision=prec, adp_layout="padded")
    t = calc.autotune(prec)
    assert t["blocks_per_sm"] in (24, 48, 75, 150) and t["ht"] in (0, 8) and t["ms"] > 0
    after = calc.tile_shape(prec)
    assert after["tuned"] and after["blocks_per_sm"] == t["blocks_per_sm"] and after["ht"] == t["ht"]
    assert after["occupancy"] == t["occupancy"] == 0  # no register-capped form without the multipole adjoint
    r1 = calc.calculate(st.dtdf, precision=prec, adp_layout="padded")
    assert rel_f(r1["f"], r0["f"]) < tf
    for k in ("d_xyz", "d_adp", "d_occ"):
        assert rel_norm(r1[k], r0[k]) < tg, k
    calc.close()


def test_tuning_cache_round_trip(engine, tmp_path):
    st = W.small_case("P212121", n_atoms=300, stol_max=0.6, seed=31)
    calc = api.HcCalculator(engine, st)
    t = calc.autotune(api.DSF_FP32_BULK)
    path = str(tmp_path / "tuning.txt")
    engine.save_tuning(path)
    other = api.Engine(0)
    c2 = api.HcCalculator(other, st)
    assert not c2.tile_shape(api.DSF_FP32_BULK)["tuned"]
    other.load_tuning(path)
    s2 = c2.tile_shape(api.DSF_FP32_BULK)
    assert s2["tuned"] and (s2["blocks_per_sm"], s2["ht"], s2["occupancy"]) == (t["blocks_per_sm"], t["ht"],
                                                                               t["occupancy"])
    # another shape key (FP64) is not affected
    assert not c2.tile_shape(api.DSF_FP64)["tuned"]
    r1 = calc.calculate(st.dtdf, precision=api.DSF_FP32_BULK)
    r2 = c2.calculate(st.dtdf, precision=api.DSF_FP32_BULK)
    assert rel_f(r2["f"], r1["f"]) < 1e-6
    c2.close()
    other.close()
    calc.close()


def test_register_capped_form_keeps_the_results(engine):
    # the multipole-adjoint kernels' register-capped form (three blocks per SM) is one of the tuner's candidates:
    # whichever it keeps, the results are those of the rule's form within the FP32 tolerance, and the oracle's
    from oracle import oracle as O
    prec, tf, tg = api.DSF_FP32_BULK, 1e-6, 1e-5
    st = W.config2(n_atoms=1500, d_min=2.4)
    calc = api.HcCalculator(engine, st)
    r0 = calc.calculate(st.dtdf, precision=prec, multipoles=True, adp_layout="padded")
    t = calc.autotune(prec, multipoles=True)
    assert t["occupancy"] in (0, 3)
    r1 = calc.calculate(st.dtdf, precision=prec, multipoles=True, adp_layout="padded")
    assert rel_f(r1["f"], r0["f"]) < tf
    for k in ("d_xyz", "d_adp", "d_occ", "d_pval", "d_plm", "d_kappa", "d_kappa_p"):
        assert rel_norm(r1[k], r0[k]) < tg, k
    o = O.compute(st, multipoles=True)
    assert rel_f(r1["f"], o["f"]) < tf
    calc.close()
