import glob
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")


def load_fixture(name):
    from discamb_gb300.model import structure_from_arrays
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))
    return structure_from_arrays(d), d


def fixture_names(prefix):
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))


def rel_f(a, b):
    """sum |dF| / sum |F|"""
    return float(np.sum(np.abs(np.asarray(a) - np.asarray(b))) / max(np.sum(np.abs(b)), 1e-300))


def rel_norm(a, b):
    """per-class norm error ||dg|| / ||g||"""
    a = np.concatenate([np.ravel(v) for v in a]) if isinstance(a, list) else np.ravel(a)
    b = np.concatenate([np.ravel(v) for v in b]) if isinstance(b, list) else np.ravel(b)
    nb = np.linalg.norm(b)
    if nb == 0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / nb)


def ref_adp_list(st, d):
    nadp = st.n_adp()
    return [d["ref_d_adp"][i, :nadp[i]] for i in range(st.n_atoms)]


@pytest.fixture(scope="session")
def engine():
    from discamb_gb300 import build, api
    build.build()
    eng = api.Engine(0)
    yield eng
    eng.close()


def combined_parts(st, d):
    """The two parts of the combined_taam fixture as the engine's split takes
    them: the HC atoms' structure (anomalous dispersion zero, as the reference's
    combined calculator sets it) and the IAM atoms' structure with its types
    renumbered to its elements, plus that part's IT92 coefficients."""
    hc, ia = np.asarray(d["hc_atoms"]), np.asarray(d["iam_atoms"])
    s1 = st.subset(hc)
    s1.anomalous = np.zeros(s1.n_atoms, dtype=complex)
    used_w = sorted(set(int(w) for w in st.atom_wfn[ia]))
    s2 = st.subset(ia)
    s2.atom_type = s2.atom_wfn.copy()
    s2.anomalous = np.zeros(s2.n_atoms, dtype=complex)
    iam = dict(ngauss=d["wfn_iam_ngauss"][used_w], a=d["wfn_iam_a"][used_w], b=d["wfn_iam_b"][used_w],
               c=d["wfn_iam_c"][used_w])
    return hc, ia, s1, s2, iam
