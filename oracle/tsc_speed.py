"""Times the engine's .tsc parser (dsf_tsc_load, one pass over the file into
flat arrays) against the reference's own reader (tsc_io::read_tsc, built from
the reference sources by oracle/Makefile.ref) on the same synthetic files
(TEST INFRASTRUCTURE: it needs the reference build, which exists only where
the reference tree does).

    python oracle/tsc_speed.py [--atoms 50 200] [--rows 20000] [--reps 3]

Files: --rows reflections x --atoms scatterers of complex form factors with
full-precision values, written by api.write_tsc into a temporary directory.
Both sides time only their parse (the engine's C call with no output arrays;
the reference's std::chrono around read_tsc), median of --reps.  Prints one
line per file: size, seconds of each, and MB/s.  The engine's parser runs on
up to 16 threads and the reference's reader on one; `taskset -c 0 python
oracle/tsc_speed.py` compares them on one core.
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import statistics
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[0] = os.path.dirname(HERE)  # the repository, not this directory (whose oracle.py would shadow the package)

from discamb_gb300 import api  # noqa: E402
from oracle import ref as R  # noqa: E402


def engine_parse_seconds(path):
    L = api.library()
    na, nr = C.c_int(0), C.c_int(0)
    t0 = time.perf_counter()
    rc = L.dsf_tsc_load(os.fsencode(path), C.byref(na), C.byref(nr), None, None, 0)
    dt = time.perf_counter() - t0
    if rc != 0:
        raise RuntimeError(f"dsf_tsc_load failed with status {rc}")
    return na.value, nr.value, dt


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--atoms", type=int, nargs="+", default=[50, 200])
    ap.add_argument("--rows", type=int, default=20000)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    rng = np.random.default_rng(7)
    with tempfile.TemporaryDirectory() as tmp:
        for na in a.atoms:
            path = os.path.join(tmp, f"ff_{na}.tsc")
            hkl = rng.integers(-40, 41, (a.rows, 3))
            ff = rng.normal(size=(a.rows, na)) + 1j * rng.normal(size=(a.rows, na))
            api.write_tsc(path, [f"A{i}" for i in range(na)], hkl, ff)
            mb = os.path.getsize(path) / 1e6
            ours, ref = [], []
            for _ in range(a.reps):
                n1, r1, t1 = engine_parse_seconds(path)
                n2, r2, t2 = R.tsc_read_seconds(path)
                assert (n1, r1) == (n2, r2) == (na, a.rows), ((n1, r1), (n2, r2))
                ours.append(t1)
                ref.append(t2)
            t_ours, t_ref = statistics.median(ours), statistics.median(ref)
            print(f"{a.rows} rows x {na} scatterers ({mb:.1f} MB): reference read_tsc {t_ref:.3f} s "
                  f"({mb / t_ref:.0f} MB/s), engine parser {t_ours:.3f} s ({mb / t_ours:.0f} MB/s), "
                  f"reference/engine {t_ref / t_ours:.2f}")


if __name__ == "__main__":
    main()
