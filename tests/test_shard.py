"""The reflection-sharded single-structure path (discamb_gb300/shard.py) on
CPU: the partition of a reflection set into line-aligned shares, and the
calculation over world-size 2 and 3 gloo ranks, each rank's calculator
answering from rank-local slices of precomputed per-reflection
contributions (a stand-in for the engine; linear in dT/dF as the real
derivatives are).  The all-reduced derivatives must equal the whole set's
sum on every rank and the gathered F the whole set in the caller's order."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as tmp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

from discamb_gb300 import shard  # noqa: E402
from discamb_gb300 import workloads as W  # noqa: E402


def _reflections(seed=5, stol=0.55):
    st = W.small_case("P21/c", n_atoms=4, stol_max=stol, seed=seed)
    rng = np.random.default_rng(seed)
    return st.hkl[rng.permutation(st.n_hkl)]  # the caller's order need not be line order


@pytest.mark.parametrize("world", [1, 2, 3, 5, 8])
def test_shares_cover_every_reflection_once_and_start_lines(world):
    hkl = _reflections()
    shares = shard.shard_indices(hkl, world)
    assert len(shares) == world
    allidx = np.concatenate(shares)
    assert len(allidx) == len(hkl) and len(set(allidx.tolist())) == len(hkl)
    order = shard.line_order(hkl)
    longest = 1 + max(np.diff(np.flatnonzero(np.r_[True, np.any(np.diff(hkl[order], axis=0) != [0, 0, 1], axis=1),
                                                    True])))
    for s in shares:
        # every share is a contiguous run of the line order that starts a line
        rank_of = np.empty(len(hkl), dtype=int)
        rank_of[order] = np.arange(len(hkl))
        p = np.sort(rank_of[s])
        if len(p):
            assert np.all(np.diff(p) == 1)
            first = hkl[order[p[0]]]
            if p[0] > 0:
                prev = hkl[order[p[0] - 1]]
                assert not (first[0] == prev[0] and first[1] == prev[1] and first[2] == prev[2] + 1)
        # balanced to within a line
        assert abs(len(s) - len(hkl) / world) <= longest + 1


class _Contributions:
    """Per-reflection contributions of a synthetic structure: F_h and complex
    c_h[atom] per derivative class, so that a share's derivatives are
    sum_h Re(conj(dT/dF_h) c_h), linear in dT/dF like the engine's."""

    def __init__(self, hkl, n_atoms, seed=11):
        rng = np.random.default_rng(seed)
        m = len(hkl)
        self.key = {tuple(int(v) for v in h): i for i, h in enumerate(hkl)}
        self.f = rng.normal(size=m) + 1j * rng.normal(size=m)
        self.c = {k: rng.normal(size=(m, n_atoms, w)) + 1j * rng.normal(size=(m, n_atoms, w))
                  for k, w in (("d_xyz", 3), ("d_adp", 6), ("d_occ", 1))}

    def result(self, idx, dtdf):
        g = np.conj(np.asarray(dtdf))[:, None, None]
        out = {"f": self.f[idx]}
        for k, c in self.c.items():
            v = np.sum((g * c[idx]).real, axis=0)
            out[k] = v[:, 0] if v.shape[1] == 1 else v
        return out


class _ShareCalc:
    def __init__(self, contrib, hkl_share):
        self.contrib = contrib
        self.idx = np.array([contrib.key[tuple(int(v) for v in h)] for h in hkl_share], dtype=np.int64)

    def calculate(self, dtdf_share, **kw):
        return self.contrib.result(self.idx, dtdf_share)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        hkl = _reflections()
        n_atoms = 7
        contrib = _Contributions(hkl, n_atoms)
        dtdf = np.random.default_rng(3).normal(size=len(hkl)) + 1j * np.random.default_rng(4).normal(size=len(hkl))
        calc = shard.ShardedCalculator(lambda h: _ShareCalc(contrib, h), hkl, n_atoms)
        r = calc.calculate(dtdf)
        local = calc.calculate(dtdf, gather_f=False)
        q.put((rank, r, local["f_indices"], local["f"]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_calculation_over_gloo_ranks(world):
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    hkl = _reflections()
    contrib = _Contributions(hkl, 7)
    dtdf = np.random.default_rng(3).normal(size=len(hkl)) + 1j * np.random.default_rng(4).normal(size=len(hkl))
    whole = contrib.result(np.arange(len(hkl)), dtdf)
    seen = np.zeros(len(hkl), dtype=int)
    for rank, r, idx, f_local in out:
        assert np.abs(r["f"] - whole["f"]).max() == 0.0  # gathered F: every reflection, caller's order
        for k in ("d_xyz", "d_adp", "d_occ"):
            np.testing.assert_allclose(r[k], whole[k], rtol=1e-12, atol=1e-12)
        assert np.abs(f_local - whole["f"][idx]).max() == 0.0
        seen[idx] += 1
    assert np.all(seen == 1)


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tf,tg", [(0, 1e-10, 1e-10), (1, 1e-6, 1e-5)])
def test_engine_shares_add_up_to_the_whole_set(engine, prec, tf, tg):
    # what every rank of the sharded path runs, on one GPU in turn: the engine over each line-aligned share of
    # a config-1-like structure's reflections; the shares' derivatives summed (the all-reduce) and their F put
    # back in order equal the whole set's call
    from conftest import rel_f, rel_norm
    from discamb_gb300 import api
    st = W.config1(n_atoms=600, d_min=2.2)
    whole = api.HcCalculator(engine, st).calculate(st.dtdf, precision=prec, adp_layout="padded")
    f = np.zeros(st.n_hkl, dtype=complex)
    acc = {k: 0.0 for k in ("d_xyz", "d_adp", "d_occ")}
    for idx in shard.shard_indices(st.hkl, 3):
        sub = st.subset(np.arange(st.n_atoms))
        sub.hkl, sub.dtdf = st.hkl[idx], st.dtdf[idx]
        c = api.HcCalculator(engine, sub)
        r = c.calculate(sub.dtdf, precision=prec, adp_layout="padded")
        c.close()
        f[idx] = r["f"]
        for k in acc:
            acc[k] = acc[k] + r[k]
    assert rel_f(f, whole["f"]) < tf
    for k in acc:
        assert rel_norm(acc[k], whole[k]) < tg, k
