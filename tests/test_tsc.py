"""The .tsc reader (dsf_tsc_load / dsf_structure_create_tsc): the file the
reference's own reader produced the golden outputs from, written again here,
read back exactly; malformed lines skipped as the reference skips them; the
engine built from the file matches the reference."""
import os

import numpy as np
import pytest

from conftest import load_fixture, rel_f, rel_norm, ref_adp_list
from discamb_gb300 import api


def fixture_file(tmp_path):
    st, d = load_fixture("tsc_p21c")
    path = os.path.join(str(tmp_path), "ff.tsc")
    api.write_tsc(path, [str(x) for x in d["tsc_labels"]], d["tsc_keys"], d["tsc_values"])
    return st, d, path


def test_reader_returns_the_file_exactly(tmp_path):
    st, d, path = fixture_file(tmp_path)
    hkl, ff = api.tsc_load(path)
    assert np.array_equal(hkl, d["tsc_keys"])
    assert np.array_equal(ff, d["tsc_values"])


def test_reader_skips_lines_of_another_form(tmp_path):
    path = os.path.join(str(tmp_path), "odd.tsc")
    with open(path, "w") as fh:
        fh.write("TITLE: t\nSCATTERERS: A B\nDATA:\n")
        fh.write("1 0 0 1.5,-2 3,4\n")          # kept
        fh.write("1 1 0 1.5,-2\n")              # one scatterer short: skipped
        fh.write("# comment\n")                 # skipped
        fh.write("  -2 3 1   0.25,0.5 -1e-3,7E2  \r\n")  # kept, blanks and CR
        fh.write("2 0 0 1,2 3,4 5,6\n")         # one too many: skipped
    hkl, ff = api.tsc_load(path)
    assert hkl.tolist() == [[1, 0, 0], [-2, 3, 1]]
    assert np.allclose(ff, [[1.5 - 2j, 3 + 4j], [0.25 + 0.5j, -1e-3 + 700j]], rtol=0, atol=0)


def test_reader_rejects_a_file_without_data(tmp_path):
    path = os.path.join(str(tmp_path), "none.tsc")
    with open(path, "w") as fh:
        fh.write("TITLE: t\nSCATTERERS: A\n")
    with pytest.raises(api.DsfError):
        api.tsc_load(path)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [api.DSF_FP64, api.DSF_FP32_BULK])
def test_engine_from_tsc_matches_reference(engine, tmp_path, prec):
    st, d, path = fixture_file(tmp_path)
    calc = api.TabulatedCalculator(engine, st, tsc_path=path)
    r = calc.calculate(st.dtdf, precision=prec)
    # the file holds complex64-representable values only after the engine's complex64 table: compare at the
    # FP32 bar for both forms of the arithmetic
    assert rel_f(r["f"], d["ref_f"]) < 1e-6
    assert rel_norm(r["d_xyz"], d["ref_d_xyz"]) < 1e-5
    assert rel_norm(r["d_adp"], ref_adp_list(st, d)) < 1e-5
    assert rel_norm(r["d_occ"], d["ref_d_occ"]) < 1e-5
    calc.close()


@pytest.mark.gpu
def test_missing_reflection_is_an_error(engine, tmp_path):
    st, d, path = fixture_file(tmp_path)
    keys, vals = d["tsc_keys"][1:], d["tsc_values"][1:]
    short = os.path.join(str(tmp_path), "short.tsc")
    api.write_tsc(short, [str(x) for x in d["tsc_labels"]], keys, vals)
    used = {tuple(k) for k in d["tsc_keys"][:1]}
    with pytest.raises(api.DsfError, match="no form factors"):
        api.TabulatedCalculator(engine, st, tsc_path=short)
    assert used
