"""Serving loop (discamb_gb300.serve): scheduling, admission by device
memory and continuous batching, with a fake executor on the CPU; the GPU
test checks that a request answered inside a mixed batch equals the same
call made alone."""
import threading
import time

import numpy as np
import pytest

from discamb_gb300 import serve


class FakeCalc:
    def __init__(self, key, nbytes, log):
        self.key, self.nbytes, self.log = key, nbytes, log
        self.closed = False
        log.append(("create", key))

    def device_bytes(self):
        return self.nbytes

    def close(self):
        self.closed = True
        self.log.append(("close", self.key))


def make_server(budget, sizes, max_batch=8, fail=False):
    log, batches = [], []

    def executor(calcs, reqs):
        if fail:
            raise RuntimeError("device error")
        batches.append([c.key for c in calcs])
        return [{"key": c.key, "cycle": r.dtdf} for c, r in zip(calcs, reqs)]

    srv = serve.SfServer(executor, budget, max_batch=max_batch)
    for k, b in sizes.items():
        srv.add_structure(k, lambda k=k, b=b: FakeCalc(k, b, log), b)
    return srv, log, batches


def req(key, cycle):
    return serve.Request(key=key, xyz=None, adp=None, occupancy=None, dtdf=cycle)


def test_one_round_batches_one_request_per_structure():
    srv, log, batches = make_server(100, {"a": 10, "b": 10, "c": 10})
    rs = [srv.submit(req(k, 0)) for k in "abc"] + [srv.submit(req("a", 1))]
    assert srv.step() == 3
    assert sorted(batches[0]) == ["a", "b", "c"]
    assert srv.step() == 1 and batches[1] == ["a"]
    assert srv.step() == 0
    assert all(r.done.is_set() for r in rs)
    # a structure's cycles complete in order
    assert rs[0].t_done <= rs[3].t_done and rs[3].result["cycle"] == 1


def test_admission_by_device_memory_and_lru_eviction():
    srv, log, batches = make_server(25, {"a": 10, "b": 10, "c": 10})
    for k in "ab":
        srv.submit(req(k, 0))
    assert srv.step() == 2
    assert srv.resident_bytes == 20
    srv.retire("a")
    srv.submit(req("c", 0))
    srv.submit(req("b", 1))
    assert srv.step() == 2  # c admitted by evicting the retired, idle a
    assert ("close", "a") in log and srv.evictions == 1
    assert srv.resident_bytes == 20


def test_request_waits_when_nothing_can_be_evicted():
    srv, log, batches = make_server(15, {"a": 10, "b": 10})
    srv.submit(req("a", 0))
    srv.submit(req("a", 1))
    srv.submit(req("b", 0))
    assert srv.step() == 1 and batches[0] == ["a"]   # b does not fit while a has work
    assert srv.step() == 1 and batches[1] == ["a"]
    assert srv.step() == 1 and batches[2] == ["b"]   # a idle: evicted for b
    assert srv.evictions == 1


def test_max_batch_and_arrival_order():
    sizes = {i: 1 for i in range(10)}
    srv, log, batches = make_server(100, sizes, max_batch=4)
    for i in range(10):
        srv.submit(req(i, 0))
        time.sleep(0.001)
    assert srv.step() == 4 and batches[0] == [0, 1, 2, 3]
    assert srv.step() == 4 and batches[1] == [4, 5, 6, 7]
    assert srv.step() == 2


def test_executor_error_reaches_every_request():
    srv, log, batches = make_server(100, {"a": 1, "b": 1}, fail=True)
    rs = [srv.submit(req(k, 0)) for k in "ab"]
    assert srv.step() == 2
    assert all(r.error == "device error" and r.result is None for r in rs)


def test_background_loop_serves_concurrent_clients():
    sizes = {i: 1 for i in range(6)}
    srv, log, batches = make_server(100, sizes)
    srv.start()
    out = []

    def client(k):
        for c in range(5):
            r = srv.submit(req(k, c))
            assert r.done.wait(5.0)
            out.append((k, c, r.result["cycle"]))

    th = [threading.Thread(target=client, args=(k,)) for k in range(6)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    srv.stop()
    assert len(out) == 30 and all(c == rc for _, c, rc in out)
    assert max(len(b) for b in batches) > 1  # clients' cycles shared batches
    srv.close()
    assert all(("close", k) in log for k in range(6))


def test_unknown_structure_is_rejected():
    srv, log, batches = make_server(10, {"a": 1})
    with pytest.raises(KeyError):
        srv.submit(req("zz", 0))


# the same request answered alone and inside a mixed batch: FP64 to rounding (the cross-block sums are FP64
# atomics in varying order), FP32-bulk within the stated tolerance (1e-6 for F, 1e-5 per derivative class; the
# batch runs the batched kernel, the call alone the single-structure kernel)
@pytest.mark.gpu
@pytest.mark.parametrize("precision,tf,tg", [(0, 1e-12, 1e-12), (1, 1e-6, 1e-5)])
def test_request_in_a_mixed_batch_equals_the_call_alone(engine, precision, tf, tg):
    from discamb_gb300 import api, workloads as W
    from conftest import rel_f, rel_norm
    # uneven sizes: 6 to 160 atoms, sin(theta)/lambda up to 0.4-0.6
    sts = {sg: W.small_case(sg, n_atoms=n, stol_max=smax, seed=600 + i)
           for i, (sg, n, smax) in enumerate([("P1", 6, 0.5), ("P-1", 40, 0.45), ("P21", 160, 0.4),
                                              ("P21/c", 12, 0.6), ("P212121", 90, 0.45), ("C2/c", 25, 0.5)])}
    srv = serve.SfServer(serve.batch_executor(engine, precision=precision), 1 << 34)
    for k, st in sts.items():
        srv.add_structure(k, lambda st=st: api.HcCalculator(engine, st),
                          serve.estimate_device_bytes(st.n_atoms, st.n_hkl, len(st.sg.subset_rot), st.n_atoms))
    rng = np.random.default_rng(9)
    cycles, rs = {}, {}
    for k, st in sts.items():
        cycles[k] = (st.xyz + rng.normal(scale=1e-3, size=st.xyz.shape), st.adp, st.occupancy)
        rs[k] = srv.submit(serve.Request(key=k, xyz=cycles[k][0], adp=st.adp, occupancy=st.occupancy,
                                         dtdf=st.dtdf))
    assert srv.step() == len(sts)
    assert srv.batch_sizes == [len(sts)]
    for k, st in sts.items():
        c = api.HcCalculator(engine, st)
        a = c.calculate(st.dtdf, precision=precision, atoms=cycles[k], adp_layout="padded")
        c.close()
        r = rs[k].result
        assert rs[k].error is None
        assert rel_f(r["f"], a["f"]) < tf, (k, rel_f(r["f"], a["f"]))
        for q in ("d_xyz", "d_adp", "d_occ"):
            assert rel_norm(r[q], a[q]) < tg, (k, q, rel_norm(r[q], a[q]))
    srv.close()
