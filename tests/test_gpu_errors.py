"""Failure paths on the GPU, injected on the host: bad inputs are rejected
with a status and the engine stays usable; a stalled copy producer (the
first sub-tile's copies never issued) makes every bounded wait of the kernel
run out, and the call returns DSF_ERR_TIMEOUT instead of hanging."""
import numpy as np
import pytest

from conftest import rel_f
from discamb_gb300 import api, workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64, FP32 = api.DSF_FP64, api.DSF_FP32_BULK


def test_non_finite_coordinates_rejected_then_engine_usable(engine):
    st = W.small_case("P21", n_atoms=5, stol_max=0.35, seed=81)
    calc = api.HcCalculator(engine, st)
    bad = st.xyz.copy()
    bad[2, 1] = np.nan
    with pytest.raises(api.DsfError, match="non-finite"):
        calc.calculate(st.dtdf, precision=FP64, atoms=(bad, st.adp_array(), st.occupancy), adp_layout="padded")
    r = calc.calculate(st.dtdf, precision=FP64, atoms=(st.xyz, st.adp_array(), st.occupancy), adp_layout="padded")
    assert rel_f(r["f"], O.compute(st)["f"]) < 1e-10
    calc.close()


def test_malformed_inputs_are_rejected(engine):
    st = W.small_case("P21", n_atoms=5, stol_max=0.35, seed=82)
    calc = api.HcCalculator(engine, st)
    with pytest.raises(api.DsfError, match="Miller index"):
        calc.set_hkl(np.array([[1, 2, 1 << 21]], dtype=np.int32))
    with pytest.raises(api.DsfError, match="precision"):
        calc.calculate(st.dtdf, precision=7)
    calc.close()
    bad = W.small_case("P21", n_atoms=5, stol_max=0.35, seed=82)
    bad.atom_type = bad.atom_type.copy()
    bad.atom_type[0] = len(bad.types) + 3  # out-of-range type index
    with pytest.raises(api.DsfError):
        api.HcCalculator(engine, bad)


@pytest.mark.parametrize("prec", [FP32, FP64])
def test_stalled_producer_times_out_and_engine_recovers(engine, prec):
    st = W.small_case("P21", n_atoms=5, stol_max=0.35, seed=83)
    calc = api.HcCalculator(engine, st)
    calc.debug_stall_next_call()
    with pytest.raises(api.DsfError, match="ran out"):
        calc.calculate(st.dtdf, precision=prec)
    # the next call (hook cleared) is correct: the error flag was reset and nothing was left in flight
    r = calc.calculate(st.dtdf, precision=prec)
    assert rel_f(r["f"], O.compute(st)["f"]) < (1e-10 if prec == FP64 else 1e-6)
    calc.close()
