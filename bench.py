#!/usr/bin/env python
"""Benchmark of the structure-factor + derivative path on GB300.

Default workload (config 2 of the benchmark set, the one the FP32-bulk
target is stated on): 50,000 atoms in protein ratios, P4_3 2_1 2
(8 operations), cell 120 x 120 x 140 A, all 315,281 unique reflections
with d >= 1.2 A, anisotropic U for the non-H atoms, Hansen-Coppens
multipoles to l = 4 on 300 shared types; F plus the full derivative set
dT/d(xyz, U, occupancy, P_val, P_lm, kappa, kappa') from a complex N(0,1)
dT/dF.  Seeded synthetic data (no dataset exists).  ``--workload config1``
(5,000 atoms, P2_1 2_1 2_1, 54,704 reflections, isotropic B, dF/d(xyz, B,
occ)), ``config0`` (32 atoms in P2_1/c: a small molecule, latency-bound),
``config3`` (the served stream) and ``config4`` (a batch of tabulated
crystals) run the other configurations.

One step = one SF + derivative pass over that reflection set.  Metric:
atom x symop x hkl terms per second (symops = point-group order without
centering).  ``value`` is the FP32-bulk form with inputs resident in HBM
(device path); ``e2e`` is the same through the host-buffer C ABI call with
the step's inputs (atomic parameters, dT/dF) copied from pinned host memory
and F + derivatives copied back inside the timed region.  The plain FP64
form is timed beside it (``fp64``) over the whole reflection set, and the
FP32-bulk error is stated against it over every reflection.  L2 (129 MB)
is flushed by writing a 256 MB buffer between timed steps (outside the
timed events).  With config 2 the served stream (config 3: p50/p99
latency, requests/s) runs first in a child process of its own and is
attached as ``served_stream``.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload configN]
                    [--electron] [--taam]

``--electron`` (configs 1, 2): electron scattering (Mott-Bethe) instead of
X-rays.  ``--taam`` (config 1): the hydrogen atoms on the IAM model and the
rest on HC through the combined calculator, host-buffer calls.

``--impl reference``: the reference engine's CPU algorithm timed on the
host cores (the reference sources are absent on the GPU host, so the
oracle's C restatement of its line-ordered loop runs, OpenMP over all host
threads), each step a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

# algorithmic flops per term (FMA = 2; sincos and exp counted apart):
#   config1: phase 6 + multipole forward 60 + 1 + f*e*T 8 + accumulate 4 + adjoint 6 + xyz 6 + B 2 + occ 1 = 94
#   config2: forward 91 (with the aniso exponent 12) + full adjoint 104 (xyz 6, U 12, occ 1, Pv 6, kappa 4,
#            kappa' 14, Plm 55, p 6) = 195
#   config0: forward 91 (as config2) + adjoint xyz 6, U 12, occ 1 = 110
WORKLOADS = {
    "config0": dict(seed=0, multipoles=False, flops=110, fp64_steps=5, fp64_warmup=2, cpu_frac=1.0, traffic_key=None,
                    desc="config0: HC multipoles l<=4, 32 atoms (12 C, 12 H, 4 N, 4 O), P21/c, all hkl with "
                         "sin(theta)/lambda<=0.8, aniso U (H iso), dF/d(xyz,U,occ); the small-molecule case"),
    "config1": dict(seed=1, multipoles=False, flops=94, fp64_steps=3, fp64_warmup=1, cpu_frac=0.25,
                    traffic_key="sf_grad_kernel3<float,HC,0,ISO,4,CS4,PAT_D2>@config1",
                    desc="config1: HC multipoles l<=4, 5000 atoms (150 types), P212121, 54704 hkl d>=1.5A, iso B, "
                         "dF/d(xyz,B,occ)"),
    "config4": dict(seed=4, desc="config4: 256 crystals, P21/c, tabulated complex64 form factors per (atom, h'), "
                                 "atoms log-uniform 10-2000, hkl log-uniform 2k-100k, aniso U (H iso), "
                                 "dF/d(xyz,U,occ); one batched submission per step"),
    "config3": dict(seed=3, desc="config3: served stream, Poisson arrivals at 200 req/s, 400 structures x 5 "
                                 "least-squares cycles (xyz sigma 0.01 A, U sigma 5%), atoms log-uniform 20-20000, "
                                 "hkl log-uniform 1k-300k, P1/P-1/P21/P21c/P212121/C2c, HC l<=4, aniso U, "
                                 "dF/d(xyz,U,occ)"),
    "config2": dict(seed=2, multipoles=True, flops=195, fp64_steps=1, fp64_warmup=0, cpu_frac=0.002,
                    traffic_key="sf_grad_kernel3<float,HC,MP,ANISO,8,CS4,PAT_D2>@config2",
                    desc="config2: HC multipoles l<=4, 50000 atoms (300 types), P43212, all hkl d>=1.2A, aniso U "
                         "(H iso), dF/d(xyz,U,occ,Pv,Plm,kappa,kappa')"),
}


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def aggregate_ranks(terms, times_ms, world, device=None):
    """Weak-scaling replicas (every rank runs its own structure; no data
    exchange): the whole job's terms (sum over ranks) and each timing as the
    max over ranks (one all-reduce each; NCCL on GPUs, gloo on CPU).  Returns
    (total_terms, [max times])."""
    import torch
    t = torch.tensor(list(times_ms), dtype=torch.float64, device=device)
    n = torch.tensor([float(terms)], dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return n.item(), t.tolist()


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    mx.append(float(p[2]))
                except ValueError:
                    continue
                for n, v in zip(names, p[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def kernel_traffic(key):
    """DRAM bytes per launch of the FP32 kernel on this workload, from the
    committed ncu summary (dram__bytes_read.sum + dram__bytes_write.sum)."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles", "ncu_traffic.json")) as fh:
            rec = json.load(fh).get(key)
        return rec["dram_bytes_per_launch"] if rec else None
    except (OSError, ValueError, KeyError):
        return None


def measured_peaks():
    try:
        return json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def fp32_peak_tflops(device):
    import ctypes
    from discamb_gb300.build import PEAK_LIB
    lib = ctypes.CDLL(PEAK_LIB)
    out = ctypes.c_double(0)
    if lib.dsf_probe_fp32_tflops(device, ctypes.byref(out)) != 0:
        return None
    return out.value


def cpu_baseline(st, sample_frac, threads, multipoles=False, electron_f000=None):
    """The reference engine's algorithm on the host cores: the oracle's
    line-ordered restatement of its loop (recurrences along reflection lines,
    one contiguous share of the ordered reflections per thread, as the
    reference splits them), which runs at the reference's own speed (same
    3,000 reflections of config 1 on x86: 1.87 s vs 1.90 s single-threaded).

    Only the C computation is timed (not the wrapper's array set-up).  A call
    costs a per-atom set-up (crystal-frame P_lm, rotation blocks) plus a cost
    per reflection; both are measured, from the first m/2 and the first m
    reflections (m = sample_frac of the set), and the rate is that of one call
    over the whole reflection set.  Returns (terms/s, seconds of the m call,
    m, per-reflection seconds, set-up seconds)."""
    from oracle import oracle as O

    def timed(m):
        r = O.compute(st, hkl_subset=np.arange(m), n_threads=threads, multipoles=multipoles, loop="lines",
                      electron_f000=electron_f000)
        return r["c_seconds"]

    m = max(2, int(st.n_hkl * sample_frac))
    t_half, t_full = timed(m // 2), timed(m)
    per_refl = max(1e-12, (t_full - t_half) / (m - m // 2))
    setup = max(0.0, t_full - m * per_refl)
    terms = st.terms()
    return terms / (setup + st.n_hkl * per_refl), t_full, m, per_refl, setup


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from discamb_gb300 import workloads as W
    wl = WORKLOADS[args.workload]
    st = getattr(W, args.workload)(seed=wl["seed"])
    threads = os.cpu_count() or 1
    frac = args.reference_sample if args.workload == "config1" else wl["cpu_frac"]
    vals = []
    for i in range(args.warmup + args.steps):
        v, dt, m, per_refl, setup = cpu_baseline(st, frac, threads, multipoles=wl["multipoles"])
        if i >= args.warmup:
            vals.append((v, dt, per_refl, setup))
    value = statistics.median(v[0] for v in vals)
    ms = statistics.median(v[1] for v in vals) * 1e3
    per_refl = statistics.median(v[2] for v in vals)
    setup = statistics.median(v[3] for v in vals)
    line = {"metric": "atom*symop*hkl terms/s (SF+grad)", "value": value, "unit": "terms/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "impl": "reference",
            "config": {"workload": wl["desc"], "sample": f"first {frac:.1%} of the reflections per step"},
            "cpu_baseline": {"value": value, "unit": "terms/s", "cores": threads, "kind": "port",
                             "sample": f"{args.workload} atoms x first {m // 2} and {m} reflections per step (C "
                                       f"time only): {per_refl * 1e3:.3f} ms per reflection + {setup:.2f} s "
                                       f"set-up, rate of one call over all {st.n_hkl} reflections"},
            "e2e": {"value": value, "unit": "terms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def config4_batch(args, eng, dev, api, W, torch):
    """The config4 crystals on the device: structures created from tables
    drawn on the device (f0 (1 + 0.05 CN(0,1)) per (h, operation, atom)),
    plus per-crystal dT/dF and output buffers."""
    specs = W.config4_specs(args.c4_crystals, seed=WORKLOADS["config4"]["seed"])
    calcs, sts, dtdf, outs, tables_small = [], [], [], [], {}
    for i, (na, nh) in enumerate(specs):
        st = W.config4_crystal(na, nh, seed=4000 + i)
        f0e, el = W.config4_f0_elements(st, W.config4_stol(st))
        f0 = torch.tensor(f0e, dtype=torch.float32, device=dev)[:, torch.tensor(el, device=dev)]  # [nh, na]
        gen = torch.Generator(device=dev)
        gen.manual_seed(4000 + i)
        noise = torch.randn((st.n_hkl, 4, st.n_atoms, 2), generator=gen, device=dev) * (0.05 / math.sqrt(2.0))
        table = torch.empty_like(noise)
        table[..., 0] = f0[:, None, :] * (1.0 + noise[..., 0])
        table[..., 1] = f0[:, None, :] * noise[..., 1]
        del noise
        torch.cuda.synchronize(dev)  # the engine gathers the table on its own stream
        calcs.append(api.TabulatedCalculator(eng, st, table_device=table.data_ptr()))
        if st.n_atoms * st.n_hkl <= 4e6:
            tables_small[i] = table
        del table
        sts.append(st)
        dtdf.append(torch.tensor(np.stack([st.dtdf.real, st.dtdf.imag], 1), dtype=torch.float64,
                                 device=dev).contiguous())
        o = {"f": torch.empty(st.n_hkl, 2, dtype=torch.float64, device=dev)}
        for k, w in (("d_xyz", 3), ("d_adp", 6), ("d_occ", 1)):
            o[k] = torch.empty(st.n_atoms, w, dtype=torch.float64, device=dev)
        outs.append(o)
    return specs, calcs, sts, dtdf, outs, tables_small


def _perturbed_cycle(st, rng):
    """One least-squares cycle's parameters: xyz moved by N(0, 0.01 A) per
    Cartesian axis (as fractional shifts), U scaled by N(1, 0.05)."""
    lengths = np.asarray(st.cell[:3])
    xyz = st.xyz + rng.normal(scale=0.01, size=st.xyz.shape) / lengths
    adp = st.adp_array() * (1.0 + rng.normal(scale=0.05, size=(st.n_atoms, 6)))
    return xyz, adp, st.occupancy


def run_config3(args):
    import multiprocessing as mp
    from discamb_gb300 import workloads as W
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    specs = W.config3_specs(args.c3_structures, seed=WORKLOADS["config3"]["seed"])
    t_gen = time.perf_counter()
    # structures are generated in a process pool before any CUDA use (spawn: no inherited CUDA state)
    with mp.get_context("spawn").Pool(max(1, min(16, os.cpu_count() or 1))) as pool:
        sts = pool.starmap(W.config3_structure, [(a, h, g, 3000 + i) for i, (a, h, g) in enumerate(specs)])
    t_gen = time.perf_counter() - t_gen
    # request r is least-squares cycle r // n of structure r % n: every structure's five cycles are spread
    # over the stream (a client submits its next cycle after solving the previous one)
    n_st = len(sts)
    n_req = 5 * n_st
    rng = np.random.default_rng(33)
    arrivals = np.cumsum(rng.exponential(1.0 / args.c3_rate, n_req))
    cycles = [_perturbed_cycle(sts[r % n_st], rng) for r in range(n_req)]
    terms = [st.n_atoms * st.sg.point_group_order * st.n_hkl for st in sts]
    if args.impl == "reference":
        return run_config3_reference(args, sts, terms)
    import torch
    from discamb_gb300 import api, build, serve
    torch.cuda.set_device(0)
    build.build()
    eng = api.Engine(0)
    budget = int(args.c3_hbm_gb * (1 << 30))
    launches = [0]
    run_batch = serve.batch_executor(eng, precision=api.DSF_FP32_BULK)

    def executor(calcs, batch):
        out = run_batch(calcs, batch)
        launches[0] += calcs[0].last_launch_count()
        return out

    srv = serve.SfServer(executor, budget, max_batch=48)
    admit_ms = []

    def factory(st):
        t0 = time.perf_counter()
        c = api.HcCalculator(eng, st, upload_atoms=False)  # every request brings its cycle's atoms
        admit_ms.append((time.perf_counter() - t0) * 1e3)
        return c

    for i, st in enumerate(sts):
        srv.add_structure(i, lambda st=st: factory(st),
                          serve.estimate_device_bytes(st.n_atoms, st.n_hkl, len(st.sg.subset_rot),
                                                      len(st.types)))
    # warm-up: kernel modules and first-call costs, on structures outside the stream
    warm = [W.small_case(g, n_atoms=40, stol_max=0.6, seed=900 + j) for j, g in enumerate(W.CONFIG3_GROUPS)]
    for j, st in enumerate(warm):
        srv.add_structure(("warm", j), lambda st=st: api.HcCalculator(eng, st), 1 << 24)
    for rep in range(args.warmup):
        ws = [srv.submit(serve.Request(key=("warm", j), xyz=st.xyz, adp=st.adp_array(), occupancy=st.occupancy,
                                       dtdf=st.dtdf)) for j, st in enumerate(warm)]
        while srv.step():
            pass
        assert all(w.done.is_set() and w.error is None for w in ws)
    for j in range(len(warm)):
        srv.retire(("warm", j))
    srv.rounds, srv.batch_sizes, srv.admissions = 0, [], 0
    admit_ms.clear()
    launches[0] = 0
    reqs = []
    with ClockSampler(0) as clk:
        srv.start()
        t0 = time.perf_counter()
        for r in range(n_req):
            dt = t0 + arrivals[r] - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            xyz, adp, occ = cycles[r]
            k = r % n_st
            reqs.append(srv.submit(serve.Request(key=k, xyz=xyz, adp=adp, occupancy=occ, dtdf=sts[k].dtdf)))
            if r // n_st == 4:
                srv.retire(k)
        for q in reqs:
            q.done.wait()
        t_end = time.perf_counter()
        srv.stop()
    clocks = clk.summary()
    errors = [q.error for q in reqs if q.error]
    lat = np.array([q.latency for q in reqs]) * 1e3
    total_terms = sum(terms[r % n_st] for r in range(n_req))
    span = max(q.t_done for q in reqs) - min(q.t_submit for q in reqs)
    value = total_terms / span
    line = {
        "metric": "atom*symop*hkl terms/s (SF+grad)", "value": value, "unit": "terms/s", "n_gpus": 1,
        "steps": 1, "warmup": args.warmup, "ms_per_step": span * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 bulk (integer phase reduction, f64 accumulation)",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOADS["config3"]["desc"], "structures": len(sts), "requests": n_req,
                   "offered_req_per_s": args.c3_rate, "hbm_budget_gb": args.c3_hbm_gb,
                   "generation_s": t_gen, "terms_served": total_terms,
                   "step": "the whole served stream (arrival of the first request to completion of the last)"},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p90": float(np.percentile(lat, 90)),
                       "p99": float(np.percentile(lat, 99)), "mean": float(lat.mean()), "max": float(lat.max())},
        "served": {"req_per_s": n_req / span, "rounds": srv.rounds,
                   "mean_batch": float(np.mean(srv.batch_sizes)) if srv.batch_sizes else 0.0,
                   "max_batch": max(srv.batch_sizes) if srv.batch_sizes else 0, "admissions": srv.admissions,
                   "evictions": srv.evictions, "errors": len(errors),
                   "admission_ms": {"p50": float(np.percentile(admit_ms, 50)) if admit_ms else None,
                                    "max": float(max(admit_ms)) if admit_ms else None}},
        "e2e": {"value": value, "unit": "terms/s",
                "h2d_bytes_per_step": int(sum(16 * sts[r % n_st].n_hkl + 80 * sts[r % n_st].n_atoms
                                              for r in range(n_req))),
                "d2h_bytes_per_step": int(sum(16 * sts[r % n_st].n_hkl + 80 * sts[r % n_st].n_atoms
                                              for r in range(n_req)))},
        "gpu_launches": launches[0],
        "clocks": {"sm_mhz": clocks["sm_mhz"], "sm_max_mhz": clocks["sm_max_mhz"], "reasons": clocks["reasons"]},
        "wall_s_timed_region": t_end - t0,
    }
    srv.close()
    if args.c3_burst > 0:
        line["burst"] = config3_burst(args, eng, api, serve, sts, terms, factory)
    print(json.dumps(line))
    eng.close()
    return 0


def config3_burst(args, eng, api, serve, sts, terms, factory):
    """The served stream's scheduler under pressure: the five cycles of the
    first `--c3-burst` structures submitted at once (all clients arrive
    together) to a server whose device-memory budget (`--c3-burst-hbm-gb`)
    holds only part of them, so requests batch up to 48 per round and idle
    structures are evicted to admit the next."""
    n_st = min(args.c3_burst, len(sts))
    budget = int(args.c3_burst_hbm_gb * (1 << 30))
    run_batch = serve.batch_executor(eng, precision=api.DSF_FP32_BULK)
    srv = serve.SfServer(run_batch, budget, max_batch=48)
    est = [serve.estimate_device_bytes(st.n_atoms, st.n_hkl, len(st.sg.subset_rot), len(st.types))
           for st in sts[:n_st]]
    for i in range(n_st):
        srv.add_structure(i, lambda st=sts[i]: factory(st), est[i])
    rng = np.random.default_rng(44)
    cycles = [[_perturbed_cycle(sts[i], rng) for _ in range(5)] for i in range(n_st)]
    srv.start()
    t0 = time.perf_counter()
    reqs = []
    for c in range(5):
        for i in range(n_st):
            xyz, adp, occ = cycles[i][c]
            reqs.append(srv.submit(serve.Request(key=i, xyz=xyz, adp=adp, occupancy=occ, dtdf=sts[i].dtdf)))
    for q in reqs:
        q.done.wait()
    span = time.perf_counter() - t0
    srv.stop()
    lat = np.array([q.latency for q in reqs]) * 1e3
    out = {"structures": n_st, "requests": len(reqs), "hbm_budget_gb": args.c3_burst_hbm_gb,
           "sum_of_structure_bytes_gb": sum(est) / (1 << 30),
           "value": 5 * sum(terms[:n_st]) / span, "unit": "terms/s", "span_ms": span * 1e3,
           "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "max": float(lat.max())},
           "mean_batch": float(np.mean(srv.batch_sizes)) if srv.batch_sizes else 0.0,
           "max_batch": max(srv.batch_sizes) if srv.batch_sizes else 0, "rounds": srv.rounds,
           "admissions": srv.admissions, "evictions": srv.evictions,
           "errors": sum(1 for q in reqs if q.error)}
    srv.close()
    return out


def run_config3_reference(args, sts, terms):
    """The reference engine's algorithm (oracle port, all host threads) on a
    bounded sample of the served requests: whole calls of structures drawn in
    a seeded random order (each call pays its own set-up, as a served request
    does), skipping those above 2e9 terms (several seconds each on the host),
    about 3 s of C time per step."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    order = [i for i in np.random.default_rng(33).permutation(len(sts)) if terms[i] <= 2e9]
    vals, times = [], []
    for rep in range(args.warmup + args.steps):
        t_cpu, done = 0.0, 0
        for i in order[rep * 7 % len(order):] + order[:rep * 7 % len(order)]:
            t_cpu += O.compute(sts[i], n_threads=threads, loop="lines")["c_seconds"]  # C time only
            done += terms[i]
            if t_cpu > 3.0:
                break
        if rep >= args.warmup:
            vals.append(done / t_cpu)
            times.append(t_cpu)
    value = statistics.median(vals)
    line = {"metric": "atom*symop*hkl terms/s (SF+grad)", "value": value, "unit": "terms/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.median(times) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": WORKLOADS["config3"]["desc"],
                       "sample": "whole calls of served structures in a seeded random order (up to 2e9 terms "
                                 "each), about 3 s of C time per step"},
            "cpu_baseline": {"value": value, "unit": "terms/s", "cores": threads, "kind": "port",
                             "sample": "served structures in a seeded random order, all host threads"},
            "e2e": {"value": value, "unit": "terms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_config4(args):
    import torch
    from discamb_gb300 import api, build, workloads as W
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_config4_reference(args)
    device = local if world > 1 else 0
    torch.cuda.set_device(device)
    build.build()
    dev = torch.device("cuda", device)
    eng = api.Engine(device)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    t_setup = time.perf_counter()
    specs, calcs, sts, dtdf, outs, small = config4_batch(args, eng, dev, api, W, torch)
    torch.cuda.synchronize(dev)
    t_setup = time.perf_counter() - t_setup
    terms = sum(st.n_atoms * 4 * st.n_hkl for st in sts)
    table_bytes = 8 * terms
    io_bytes = sum(32 * st.n_hkl + 8 * 10 * st.n_atoms for st in sts)  # dT/dF in, F out, per-atom outputs
    ptrs = [d.data_ptr() for d in dtdf]
    optrs = [{k: v.data_ptr() for k, v in o.items()} for o in outs]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step():
        eng.calculate_batch_device(calcs, ptrs, optrs, precision=api.DSF_FP32_BULK, stream=sptr)

    for _ in range(args.warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize(dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(device) as clk:
        t0 = time.perf_counter()
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
    clocks = clk.summary()
    launches = calcs[0].last_launch_count()
    ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
    # FP64 form of the same batch (per-structure launches); the FP32 results of the last timed step against it
    r32 = [{k: v.clone() for k, v in o.items()} for o in outs]
    ev64 = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    eng.calculate_batch_device(calcs, ptrs, optrs, precision=api.DSF_FP64, stream=sptr)
    ev64[0].record(stream)
    eng.calculate_batch_device(calcs, ptrs, optrs, precision=api.DSF_FP64, stream=sptr)
    ev64[1].record(stream)
    torch.cuda.synchronize(dev)
    ms64 = ev64[0].elapsed_time(ev64[1])
    err32 = {"f": float(sum((a["f"] - b["f"]).norm(dim=1).sum() for a, b in zip(r32, outs)) /
                        sum(b["f"].norm(dim=1).sum() for b in outs))}
    err_max = {}
    for k in ("d_xyz", "d_adp", "d_occ"):
        dg = torch.cat([(a[k] - b[k]).flatten() for a, b in zip(r32, outs)])
        g64 = torch.cat([b[k].flatten() for b in outs])
        err32[k] = float(dg.norm() / g64.norm())
        err_max[k] = float(dg.abs().max() / g64.abs().max())
    del r32
    # end to end: host dT/dF in, host F and derivatives out, one submission
    hd = [st.dtdf for st in sts]
    for _ in range(2):
        eng.calculate_batch(calcs, hd, precision=api.DSF_FP32_BULK)
    e2e = []
    for _ in range(args.steps):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        eng.calculate_batch(calcs, hd, precision=api.DSF_FP32_BULK)
        e2e.append(time.perf_counter() - t0)
    e2e_ms = statistics.mean(e2e) * 1e3
    mp = measured_peaks()
    peak = mp.get("hbm_gbs")
    achieved = (table_bytes + io_bytes) / (ms * 1e-3) * 1e-9
    # CPU: the generic engine with a tabulated form factor, one thread, on the small crystals
    from oracle import oracle as O
    t_cpu, cpu_terms, used = 0.0, 0, []
    for i in sorted(small, key=lambda j: sts[j].n_atoms * sts[j].n_hkl):
        st = sts[i]
        tb = small[i].cpu().numpy()
        t = tb[..., 0] + 1j * tb[..., 1]
        t_cpu += O.compute(st, model="table", table=t, n_threads=1)["c_seconds"]  # C time only
        cpu_terms += st.n_atoms * 4 * st.n_hkl
        used.append(i)
        if t_cpu > 10.0:
            break
    line = {
        "metric": "atom*symop*hkl terms/s (SF+grad)", "value": terms / (ms * 1e-3), "unit": "terms/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 bulk (complex64 table, f64 accumulation)",
        "data": "synthetic (seeded; tables drawn on the device)",
        "config": {"workload": WORKLOADS["config4"]["desc"], "crystals": len(sts), "terms_per_step": terms,
                   "table_bytes": table_bytes, "setup_s": t_setup,
                   "l2": "inputs larger than L2 (tables); 256 MB flush between steps"},
        "fp64": {"value": terms / (ms64 * 1e-3), "ms_per_step": ms64, "fp32_over_fp64": ms64 / ms,
                 "fp32_error": {**err32, "measure": "sum|dF|/sum|F| over every crystal's reflections; derivatives "
                                                   "per class |dg|/|g| over every crystal's atoms, FP32-bulk "
                                                   "against this FP64 run"},
                 "fp32_error_max": {**err_max, "measure": "per derivative class max|dg| / max|g|"}},
        "e2e": {"value": terms / (e2e_ms * 1e-3), "unit": "terms/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": sum(16 * st.n_hkl for st in sts),
                "d2h_bytes_per_step": sum(16 * st.n_hkl + 80 * st.n_atoms for st in sts)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if peak else None,
                     "traffic": kernel_traffic("sf_grad_batch3<float,TABLE,ISO+ANISO,4>@config4"),
                     "bytes_per_step": table_bytes + io_bytes, "timed": "whole batched step (CUDA events)"},
        "cpu_baseline": {"value": cpu_terms / t_cpu if t_cpu else None, "unit": "terms/s", "cores": 1,
                         "kind": "port",
                         "sample": f"{len(used)} smallest crystals, generic engine with the table, one thread "
                                   f"({t_cpu:.1f} s)"},
        "gpu_launches": launches,
        "clocks": {"sm_mhz": clocks["sm_mhz"], "sm_max_mhz": clocks["sm_max_mhz"], "reasons": clocks["reasons"]},
        "wall_s_timed_region": wall,
    }
    print(json.dumps(line))
    for c in calcs:
        c.close()
    eng.close()
    return 0


def run_config4_reference(args):
    """The generic engine with tabulated form factors on the host, one
    thread (the reference's tabulated path is serial), on the smallest
    crystals of the batch, tables drawn on the host."""
    from discamb_gb300 import workloads as W
    from oracle import oracle as O
    specs = W.config4_specs(args.c4_crystals, seed=WORKLOADS["config4"]["seed"])
    order = sorted(range(len(specs)), key=lambda i: specs[i][0] * specs[i][1])
    vals, times = [], []
    for rep in range(args.warmup + args.steps):
        t_cpu, terms = 0.0, 0
        for i in order:
            st = W.config4_crystal(*specs[i], seed=4000 + i)
            t = W.config4_table(st, np.random.default_rng(4000 + i))
            t_cpu += O.compute(st, model="table", table=t, n_threads=1)["c_seconds"]  # C time only
            terms += st.n_atoms * 4 * st.n_hkl
            if t_cpu > 3.0:
                break
        if rep >= args.warmup:
            vals.append(terms / t_cpu)
            times.append(t_cpu)
    value = statistics.median(vals)
    line = {"metric": "atom*symop*hkl terms/s (SF+grad)", "value": value, "unit": "terms/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.median(times) * 1e3,
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "impl": "reference", "config": {"workload": WORKLOADS["config4"]["desc"],
                                            "sample": "smallest crystals, about 3 s of work per step"},
            "cpu_baseline": {"value": value, "unit": "terms/s", "cores": 1, "kind": "port",
                             "sample": "smallest crystals of the batch, one thread"},
            "e2e": {"value": value, "unit": "terms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_gpu(args, served=None):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    device = local if world > 1 else 0
    torch.cuda.set_device(device)
    from discamb_gb300 import api, build, workloads as W
    build.build()
    wl = WORKLOADS[args.workload]
    kw = {}
    if args.workload == "config2" and args.c2_atoms:  # a cut of config 2 (e.g. for a profile capture)
        kw = dict(n_atoms=args.c2_atoms, d_min=args.c2_dmin)
    st = getattr(W, args.workload)(seed=wl["seed"] + rank, **kw)
    mpd = wl["multipoles"]
    eng = api.Engine(device)
    calc = api.HcCalculator(eng, st)
    # electron scattering (Mott-Bethe), folded into the radial tables; f_e(0) per wavefunction only enters F(000),
    # which no benchmark reflection set holds
    f000 = [float(w.atomic_number) for w in st.wfns] if args.electron else None
    if args.electron:
        calc.set_electron(True, f000)
    n_hkl, n = st.n_hkl, st.n_atoms
    terms = st.terms()
    dev = torch.device("cuda", device)
    # a dedicated stream: the engine launches on it, the CUDA events record on it
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    assert sptr != 0
    dtdf = torch.tensor(np.stack([st.dtdf.real, st.dtdf.imag], 1), dtype=torch.float64, device=dev).contiguous()
    f = torch.empty(n_hkl, 2, dtype=torch.float64, device=dev)
    widths = [("d_xyz", 3), ("d_adp", 6), ("d_occ", 1)]
    if mpd:
        widths += [("d_pval", 1), ("d_plm", 25), ("d_kappa", 1), ("d_kappa_prime", 1)]
    g = {k: torch.empty(n, w, dtype=torch.float64, device=dev) for k, w in widths}
    outs = {"f": f.data_ptr(), **{k: v.data_ptr() for k, v in g.items()}}
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > L2 (129 MB)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def timed_device(prec, steps, warmup, calc_=calc, dtdf_=dtdf, outs_=outs):
        for _ in range(warmup):
            flush.zero_()
            calc_.calculate_device(dtdf_.data_ptr(), outs_, precision=prec, multipoles=mpd, stream=sptr)
        torch.cuda.synchronize(dev)
        barrier()
        torch.cuda.synchronize(dev)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        kern = []
        launches = 0
        t0 = time.perf_counter()
        for i in range(steps):
            flush.zero_()
            ev[i][0].record(stream)
            calc_.calculate_device(dtdf_.data_ptr(), outs_, precision=prec, multipoles=mpd, stream=sptr)
            ev[i][1].record(stream)
            launches += calc_.last_launch_count()
            stream.synchronize()
            kern.append(calc_.last_kernel_ms())
        torch.cuda.synchronize(dev)
        barrier()
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
        step_ms = [a.elapsed_time(b) for a, b in ev]
        return step_ms, kern, launches, wall

    # the tile shape: the autotuner times a few candidates on this structure (set-up, outside the timed region)
    tuned = calc.autotune(api.DSF_FP32_BULK, multipoles=mpd) if args.autotune else None
    shape = calc.tile_shape(api.DSF_FP32_BULK, multipoles=mpd)
    with ClockSampler(device) as clk:
        ms32, kern32, launches32, wall32 = timed_device(api.DSF_FP32_BULK, args.steps, args.warmup)
    clocks = clk.summary()

    def snapshot(m):
        return f[:m].clone(), {k: v.clone() for k, v in g.items()}

    # the plain FP64 form on the whole reflection set (no sample: the FP32 error is measured over every
    # reflection and every atom); the FP32 results of the last timed step against it
    r32 = snapshot(n_hkl)
    ms64, kern64, _, _ = timed_device(api.DSF_FP64, wl["fp64_steps"], wl["fp64_warmup"])
    r64 = snapshot(n_hkl)
    terms64 = terms
    err32 = {"f": float((r32[0] - r64[0]).norm(dim=1).sum() / r64[0].norm(dim=1).sum())}
    err_max = {}
    for k in r64[1]:
        dg = r32[1][k] - r64[1][k]
        err32[k] = float(dg.norm() / r64[1][k].norm())
        err_max[k] = float(dg.abs().max() / r64[1][k].abs().max())

    # end to end through the reference-shaped host call (atoms + dT/dF in, F and
    # derivatives out); the library stages through its own pinned buffer
    xyz_h = st.xyz.copy()
    adp_h = st.adp_array()
    occ_h = st.occupancy.copy()

    def host_call():
        return calc.calculate(st.dtdf, precision=api.DSF_FP32_BULK, atoms=(xyz_h, adp_h, occ_h),
                              adp_layout="padded", multipoles=mpd)

    for _ in range(args.warmup):
        host_call()
    e2e = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        host_call()
        e2e.append(time.perf_counter() - t0)
    h2d = 80 * n + 16 * n_hkl
    d2h = 16 * n_hkl + sum(w for _, w in widths) * 8 * n

    step32 = statistics.mean(ms32)
    step64 = statistics.mean(ms64)
    k32 = statistics.mean(kern32)
    # weak scaling: every rank runs its own replica; max time over ranks
    job_terms, (step32, e2e_ms, k32) = aggregate_ranks(terms, [step32, statistics.mean(e2e) * 1e3, k32], world, dev)
    value = job_terms / (step32 * 1e-3)
    if rank != 0:
        return 0
    achieved = wl["flops"] * terms / (k32 * 1e-3) * 1e-12
    peak = fp32_peak_tflops(device)
    cpu_v, cpu_dt, cpu_m, cpu_pr, cpu_su = cpu_baseline(st, wl["cpu_frac"], os.cpu_count() or 1, multipoles=mpd,
                                                        electron_f000=f000)
    mp = measured_peaks()
    line = {
        "metric": "atom*symop*hkl terms/s (SF+grad)", "value": value, "unit": "terms/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step32, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 bulk (integer phase reduction, f64 accumulation)",
        "data": "synthetic (seeded)",
        "config": {"workload": wl["desc"], "terms_per_step": terms, "l2": "flushed (256 MB write) between timed steps",
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
                   "scattering": "electron (Mott-Bethe)" if args.electron else "X-ray"},
        "fp64": {"value": world * terms64 / (step64 * 1e-3), "ms_per_step": step64,
                 "kernel_ms": statistics.mean(kern64),
                 "fp32_over_fp64": (terms / step32) / (terms64 / step64),
                 "sample": f"all {n_hkl} reflections, {wl['fp64_steps']} timed step(s)",
                 "fp32_error": {**err32, "measure": "sum|dF|/sum|F|; derivatives per class |dg|/|g|, FP32-bulk "
                                                   "against this FP64 run over every reflection"},
                 "fp32_error_max": {**err_max, "measure": "per derivative class max|dg| / max|g|"}},
        "e2e": {"value": job_terms / (e2e_ms * 1e-3), "unit": "terms/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": kernel_traffic(wl["traffic_key"]),
                     "peak_source": "FP32 FMA throughput probe measured in this run (MEASURED_PEAKS.json lists "
                                    "HBM and bf16 tensor peaks only)",
                     "flops_per_term": wl["flops"], "kernel_ms": k32,
                     "hbm_peak_gbs_measured": mp.get("hbm_gbs")},
        "cpu_baseline": {"value": cpu_v, "unit": "terms/s", "cores": os.cpu_count() or 1, "kind": "port",
                         "sample": f"{args.workload} atoms x first {cpu_m // 2} and {cpu_m} reflections (C time "
                                   f"only, {cpu_dt:.1f} s): {cpu_pr * 1e3:.3f} ms per reflection + {cpu_su:.2f} s "
                                   f"set-up, rate of one call over all {st.n_hkl} reflections"},
        "gpu_launches": launches32,
        "clocks": {"sm_mhz": clocks["sm_mhz"], "sm_max_mhz": clocks["sm_max_mhz"], "reasons": clocks["reasons"]},
        "wall_s_timed_region": wall32,
        "tile_shape": {"blocks_per_sm": shape["blocks_per_sm"], "ht": shape["ht"] or "longest",
                       "register_cap_blocks_per_sm": shape["occupancy"] or "compiler's",
                       "source": "autotuner (dsf_autotune at set-up)" if shape["tuned"]
                       else "rule (75 blocks per SM, longest sub-tile)",
                       "tuned_ms": tuned["ms"] if tuned else None},
    }
    calc.close()
    eng.close()
    if served is not None:
        line["served_stream"] = served
    print(json.dumps(line))
    return 0


def run_taam(args):
    """Config 1's structure with the TAAM split: hydrogen atoms on the IAM
    model (seeded four-Gaussian form factors), the rest on HC, through the
    combined calculator (CombinedStructureFactorCalculator's split: F summed,
    every atom's derivatives from its own part, the parts in one batched
    submission).  Host-buffer calls of the combined calculator, timed beside
    the same call with every atom on HC; FP32-bulk against FP64; the CPU port
    of both parts on a sample of the reflections."""
    import torch
    from discamb_gb300 import api, build, workloads as W
    from oracle import oracle as O
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(0)
    build.build()
    wl = WORKLOADS["config1"]
    st = W.config1(seed=wl["seed"])
    z = np.array([st.wfns[w].atomic_number for w in st.atom_wfn])
    h_idx = np.flatnonzero(z == 1)
    hc_idx = np.flatnonzero(z != 1)
    rng = np.random.default_rng(11)
    a = np.zeros((1, 5))
    b = np.zeros((1, 5))
    a[0, :4] = rng.uniform(0.05, 0.5, 4)
    b[0, :4] = rng.uniform(2.0, 50.0, 4)
    iam = dict(ngauss=np.array([4], dtype=np.int32), a=a, b=b, c=np.array([0.002]))
    eng = api.Engine(0)

    def make_iam(sub):
        sub.atom_type = np.zeros(sub.n_atoms, dtype=np.int64)  # one IAM type: hydrogen
        return api.IamCalculator(eng, sub, iam)

    comb = api.CombinedCalculator(eng, st, [(lambda sub: api.HcCalculator(eng, sub), hc_idx), (make_iam, h_idx)])
    hc_all = api.HcCalculator(eng, st)
    terms = st.terms()

    def timed(call, steps):
        for _ in range(args.warmup):
            call()
        out = []
        for _ in range(steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            call()
            out.append(time.perf_counter() - t0)
        return statistics.mean(out) * 1e3

    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        ms = timed(lambda: comb.calculate(st.dtdf, precision=api.DSF_FP32_BULK), args.steps)
        wall = time.perf_counter() - t0
    clocks = clk.summary()
    launches = sum(c.last_launch_count() for c, _ in comb.parts)
    ms_hc = timed(lambda: hc_all.calculate(st.dtdf, precision=api.DSF_FP32_BULK), args.steps)
    r32 = comb.calculate(st.dtdf, precision=api.DSF_FP32_BULK)
    t0 = time.perf_counter()
    r64 = comb.calculate(st.dtdf, precision=api.DSF_FP64)
    ms64 = (time.perf_counter() - t0) * 1e3
    err = {"f": float(np.abs(r32["f"] - r64["f"]).sum() / np.abs(r64["f"]).sum())}
    for k in ("d_xyz", "d_adp", "d_occ"):
        g32 = np.concatenate([np.ravel(v) for v in r32[k]])
        g64 = np.concatenate([np.ravel(v) for v in r64[k]])
        err[k] = float(np.linalg.norm(g32 - g64) / np.linalg.norm(g64))
    # CPU: the port of both parts on the first 5% of the reflections (line-ordered HC engine, generic IAM engine)
    m = max(2, int(st.n_hkl * 0.05))
    threads = os.cpu_count() or 1
    s_hc, s_h = st.subset(hc_idx), st.subset(h_idx)
    s_h.atom_type = np.zeros(s_h.n_atoms, dtype=np.int64)
    t_cpu = O.compute(s_hc, hkl_subset=np.arange(m), n_threads=threads, loop="lines")["c_seconds"]
    t_cpu += O.compute(s_h, model="iam", iam=iam, hkl_subset=np.arange(m), n_threads=threads)["c_seconds"]
    cpu_v = terms * m / st.n_hkl / t_cpu
    line = {
        "metric": "atom*symop*hkl terms/s (SF+grad)", "value": terms / (ms * 1e-3), "unit": "terms/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 bulk (integer phase reduction, f64 accumulation)",
        "data": "synthetic (seeded)",
        "config": {"workload": wl["desc"] + "; TAAM split: " + f"{len(hc_idx)} atoms HC, {len(h_idx)} H atoms IAM "
                                            "(seeded 4-Gaussian f0), combined calculator",
                   "terms_per_step": terms, "timed": "host-buffer calls of the combined calculator (dT/dF in, "
                                                     "F and derivatives out)"},
        "hc_only_ms_per_step": ms_hc,
        "fp64": {"ms_per_step": ms64, "fp32_over_fp64": ms64 / ms,
                 "fp32_error": {**err, "measure": "sum|dF|/sum|F|; derivatives per class |dg|/|g|, FP32-bulk "
                                                 "against FP64 over every reflection"}},
        "e2e": {"value": terms / (ms * 1e-3), "unit": "terms/s", "ms_per_step": ms,
                "h2d_bytes_per_step": 2 * 16 * st.n_hkl,
                "d2h_bytes_per_step": 2 * 16 * st.n_hkl + 80 * st.n_atoms},
        "cpu_baseline": {"value": cpu_v, "unit": "terms/s", "cores": threads, "kind": "port",
                         "sample": f"both parts on the first {m} reflections ({t_cpu:.1f} s, C time only)"},
        "gpu_launches": launches,
        "clocks": {"sm_mhz": clocks["sm_mhz"], "sm_max_mhz": clocks["sm_max_mhz"], "reasons": clocks["reasons"]},
        "wall_s_timed_region": wall,
    }
    print(json.dumps(line))
    hc_all.close()
    for c, _ in comb.parts:
        c.close()
    eng.close()
    return 0


def served_stream(args):
    """The served mixed stream (config 3: 2,000 requests, Poisson arrivals at
    200 req/s) run in a child process of its own before this process touches
    the GPU: its latency percentiles, throughput and batching, as a key of the
    headline line."""
    cmd = [sys.executable, os.path.abspath(__file__), "--workload", "config3", "--warmup", "3",
           "--c3-structures", str(args.c3_structures), "--c3-rate", str(args.c3_rate),
           "--c3-hbm-gb", str(args.c3_hbm_gb)]
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
        rec = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    except Exception as exc:  # the headline stands without it; say why
        return {"error": f"config3 run failed: {exc}"}
    keep = ("value", "unit", "ms_per_step", "latency_ms", "served", "e2e", "clocks", "gpu_launches", "burst")
    out = {k: rec.get(k) for k in keep}
    out["workload"] = rec.get("config", {}).get("workload")
    out["requests"] = rec.get("config", {}).get("requests")
    out["p99_target_ms"] = 50.0
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="config2", choices=sorted(WORKLOADS))
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep the rule's tile shape instead of tuning it at set-up")
    ap.add_argument("--electron", action="store_true",
                    help="config1/config2: electron scattering (Mott-Bethe) instead of X-ray")
    ap.add_argument("--taam", action="store_true",
                    help="config1: the TAAM split (H atoms on IAM, the rest on HC) through the combined calculator")
    ap.add_argument("--no-served", dest="served", action="store_false",
                    help="config2: skip the served stream (config3) attached to the line")
    ap.add_argument("--c4-crystals", type=int, default=256)
    ap.add_argument("--c2-atoms", type=int, default=0, help="config2 cut: atoms (0 = the full 50,000)")
    ap.add_argument("--c2-dmin", type=float, default=1.2)
    ap.add_argument("--c3-structures", type=int, default=400)
    ap.add_argument("--c3-rate", type=float, default=200.0)
    ap.add_argument("--c3-hbm-gb", type=float, default=160.0)
    ap.add_argument("--c3-burst", type=int, default=80,
                    help="config3: structures of the burst phase (all cycles at once, small budget); 0 = none")
    ap.add_argument("--c3-burst-hbm-gb", type=float, default=6.0)
    ap.add_argument("--cpu-sample", type=float, default=0.25)
    ap.add_argument("--reference-sample", type=float, default=0.1)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "config4":
        return run_config4(args)
    if args.workload == "config3":
        return run_config3(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.taam:
        return run_taam(args)
    served = None
    if args.workload == "config2" and args.served and dist_env()[1] == 1:
        served = served_stream(args)
    return run_gpu(args, served)


if __name__ == "__main__":
    sys.exit(main())
