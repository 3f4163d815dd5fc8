"""Times the oracle's line-ordered port (sfo_compute_lines, the CPU arm of
bench.py) against the reference's own Engine3 (HansenCoppensStructureFactor
Calculator, "CPU", built from the reference sources by oracle/Makefile.ref)
on the same inputs and thread counts (TEST INFRASTRUCTURE: it needs the
reference build, which exists only where the reference tree does).

    python oracle/port_speed.py [--threads 1 8] [--reps 3]

Inputs: reflection subsets (the first m in line order, as the bench's CPU
sample takes them, and m at random) of the benchmark's config 1 (5,000 atoms,
P2_1 2_1 2_1, isotropic) and config 2 (a 6,000-atom cut of its generator,
P4_3 2_1 2, anisotropic, multipoles to l = 4; the port without the multipole
adjoint, which the reference does not compute).  Both sides time their own
compute call only (the reference's std::chrono around
calculateStructureFactorsAndDerivatives; the port's C call), median of
--reps calls.  Prints one line per case: seconds of each and the ratio.
"""
from __future__ import annotations

import argparse
import os
import statistics
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[0] = os.path.dirname(HERE)  # the repository, not this directory (whose oracle.py would shadow the package)

from discamb_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle import ref as R  # noqa: E402


def cut(st, m, seed=None):
    """m reflections: the first m of the line-ordered set (whole lines, as the bench's CPU sample takes them), or
    with a seed a random choice (lines broken: every reflection starts one)"""
    sel = np.arange(m) if seed is None else np.sort(np.random.default_rng(seed).choice(st.n_hkl, m, replace=False))
    st.hkl, st.dtdf = st.hkl[sel], st.dtdf[sel]
    return st


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, nargs="+", default=[1, 8])
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    cases = [("config1, first 3,000 reflections", cut(W.config1(), 3000)),
             ("config1, 3,000 random reflections", cut(W.config1(), 3000, 1)),
             ("config2 cut (6,000 atoms), first 600 reflections", cut(W.config2(n_atoms=6000), 600)),
             ("config2 cut (6,000 atoms), 600 random reflections", cut(W.config2(n_atoms=6000), 600, 2))]
    for name, st in cases:
        for t in a.threads:
            ref = statistics.median(R.hc(st, n_threads=t)["ms"] * 1e-3 for _ in range(a.reps))
            port = statistics.median(O.compute(st, n_threads=t, loop="lines")["c_seconds"] for _ in range(a.reps))
            print(f"{name}, {t} thread(s): reference {ref:.3f} s, port {port:.3f} s, port/reference {port / ref:.2f}")


if __name__ == "__main__":
    main()
