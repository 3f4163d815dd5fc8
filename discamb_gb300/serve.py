"""Serving loop for structure-factor requests from many refinement clients.

The reference serves one caller per calculator object and has no scheduler
(``SfCalculator::calculateStructureFactorsAndDerivatives``,
include/discamb/Scattering/SfCalculator.h:45-67; callers create one calculator
per thread, src/Scattering/HcAtomBankStructureFactorCalculator.cpp:501-520).
On one GPU many clients share one engine, so this module adds what that
needs:

* a request queue: a request is one least-squares cycle of one structure
  (its atomic parameters and dT/dF);
* admission by device memory: a structure's calculator (model, reflection
  tables) is created when its first request arrives and stays resident while
  it has work; idle structures are evicted, retired ones first, then least
  recently used, when a new one would exceed the device-memory budget;
* continuous batching: every scheduling round takes the oldest pending
  request of each resident structure, up to ``max_batch``, and runs them as one
  batched submission (``Engine.calculate_batch`` with the cycle's atoms), so
  requests that arrive while a batch runs join the next one.  A structure's
  requests complete in order.

With ``start()`` the scheduler thread (batches) and ``admitters`` admission
threads (structure creation and eviction) run, so creating new structures
overlaps the batches of the resident ones (the engine sets structures up on
its own stream, and its C calls release the interpreter lock).  ``step()``
runs one round synchronously, admitting inline.

Latency of a request = completion time - submission time.  The executor and
the calculator factories are injectable, so the scheduling logic is testable
without a GPU.
"""
from __future__ import annotations

import collections
import threading
import time
from dataclasses import dataclass, field

from . import api


@dataclass
class Request:
    key: object                 # structure id
    xyz: object
    adp: object
    occupancy: object
    dtdf: object
    t_submit: float = 0.0
    t_start: float = 0.0
    t_done: float = 0.0
    result: dict = None
    error: str = None
    done: threading.Event = field(default_factory=threading.Event)

    @property
    def latency(self):
        return self.t_done - self.t_submit


@dataclass
class _Entry:
    key: object
    factory: object             # () -> calculator
    est_bytes: int
    calc: object = None
    bytes: int = 0
    admitting: bool = False
    pending: collections.deque = field(default_factory=collections.deque)
    last_used: float = 0.0
    retired: bool = False


def estimate_device_bytes(n_atoms, n_hkl, n_sym, n_types=1, multipoles=False):
    """Device bytes of one structure for FP32 calls: reflection-operation
    records, radial tables per (type, reflection), per-reflection and
    per-atom buffers."""
    n_pad = (n_hkl + 15) // 16 * 16
    rs = n_pad * n_sym * 144
    tr = n_types * n_pad * 8 * 4 * (2 if multipoles else 1)
    per_h = n_pad * (16 * 4 + 8 * 4 + 8 * 6)
    per_atom = n_atoms * (8 * 40 + 8 * 25 * 2 + 165 * 8 + 8 * 30)
    return rs + tr + per_h + per_atom


def batch_executor(engine, precision=api.DSF_FP32_BULK, derivatives=("xyz", "adp", "occ")):
    """The GPU executor: one batched submission with every request's atoms."""
    def run(calcs, requests):
        return engine.calculate_batch(calcs, [r.dtdf for r in requests], precision=precision,
                                      derivatives=derivatives,
                                      atoms=[(r.xyz, r.adp, r.occupancy) for r in requests])
    return run


class SfServer:
    """Request queue + admission + continuous batching over one engine."""

    def __init__(self, executor, hbm_budget_bytes, max_batch=48, clock=time.perf_counter, admitters=2):
        self.executor = executor
        self.n_admitters = max(1, int(admitters))
        self.budget = int(hbm_budget_bytes)
        self.max_batch = max_batch
        self.clock = clock
        self._entries = {}
        self._arrivals = collections.deque()
        self._lock = threading.Lock()
        self._cond = threading.Condition(self._lock)
        self._threads = []
        self._stop = False
        self._busy = set()          # structures of the batch that is running
        self.resident_bytes = 0
        self.reserved_bytes = 0     # structures being created
        self.rounds = 0
        self.evictions = 0
        self.admissions = 0
        self.batch_sizes = []

    # -- client side ---------------------------------------------------------
    def add_structure(self, key, factory, est_bytes):
        with self._lock:
            self._entries[key] = _Entry(key=key, factory=factory, est_bytes=int(est_bytes))

    def submit(self, req: Request):
        req.t_submit = self.clock()
        with self._cond:
            if req.key not in self._entries:
                raise KeyError(f"unknown structure {req.key!r}")
            self._arrivals.append(req)
            self._cond.notify_all()
        return req

    def retire(self, key):
        """The client is done with the structure: evict it first."""
        with self._lock:
            e = self._entries.get(key)
            if e is not None:
                e.retired = True

    # -- admission -------------------------------------------------------------
    def _drain_arrivals(self):
        while self._arrivals:
            r = self._arrivals.popleft()
            self._entries[r.key].pending.append(r)

    def _make_room(self, need):
        """Under the lock: evict idle structures until `need` bytes fit;
        returns the evicted calculators (closed by the caller, unlocked) or
        None when they cannot be made to fit now."""
        victims = []
        while self.resident_bytes + self.reserved_bytes + need > self.budget:
            idle = [x for x in self._entries.values()
                    if x.calc is not None and not x.pending and x.key not in self._busy]
            if not idle:
                for v in victims:  # undo: nothing was closed yet
                    self.resident_bytes += v[1]
                    v[0].calc, v[0].bytes = v[2], v[1]
                return None
            x = min(idle, key=lambda x: (not x.retired, x.last_used))
            victims.append((x, x.bytes, x.calc))
            self.resident_bytes -= x.bytes
            x.calc, x.bytes = None, 0
        self.evictions += len(victims)
        return [v[2] for v in victims]

    def _admit_one(self, e):
        """Creates e's calculator (lock not held); returns True when resident."""
        with self._lock:
            closing = self._make_room(e.est_bytes)
            if closing is None:
                return False
            e.admitting = True
            self.reserved_bytes += e.est_bytes
        for c in closing:
            c.close()
        try:
            calc = e.factory()
            err = None
        except Exception as ex:
            calc, err = None, str(ex)
        with self._cond:
            self.reserved_bytes -= e.est_bytes
            e.admitting = False
            if calc is None:  # the structure cannot be created: fail its requests
                t = self.clock()
                while e.pending:
                    r = e.pending.popleft()
                    r.error, r.t_done = f"structure set-up failed: {err}", t
                    r.done.set()
                self._cond.notify_all()
                return False
            dev = getattr(calc, "device_bytes", None)
            e.bytes = int(dev()) if callable(dev) else e.est_bytes
            e.calc = calc
            self.resident_bytes += e.bytes
            self.admissions += 1
            self._cond.notify_all()
        return True

    def _next_to_admit(self):
        """Under the lock: the structure of the oldest request whose structure is not resident."""
        best = None
        for e in self._entries.values():
            if e.pending and e.calc is None and not e.admitting:
                if best is None or e.pending[0].t_submit < best.pending[0].t_submit:
                    best = e
        return best

    # -- scheduling ------------------------------------------------------------
    def _take_batch(self):
        """Under the lock: the oldest request of each resident structure."""
        ready = sorted((e for e in self._entries.values() if e.pending and e.calc is not None and not e.admitting),
                       key=lambda e: e.pending[0].t_submit)[:self.max_batch]
        self._busy = {e.key for e in ready}
        return [e.pending[0] for e in ready], [e.calc for e in ready]

    def _run(self, batch, calcs):
        t0 = self.clock()
        for r in batch:
            r.t_start = t0
        try:
            results = self.executor(calcs, batch)
            err = None
        except Exception as ex:  # the whole submission failed: report it on every request
            results, err = [None] * len(batch), str(ex)
        t1 = self.clock()
        with self._cond:
            for r, res in zip(batch, results):
                e = self._entries[r.key]
                e.pending.popleft()
                e.last_used = t1
                r.result, r.error, r.t_done = res, err, t1
                r.done.set()
            self._busy = set()
            self.rounds += 1
            self.batch_sizes.append(len(batch))
            self._cond.notify_all()

    def step(self):
        """One synchronous round (admission inline): returns the number of
        requests completed."""
        with self._lock:
            self._drain_arrivals()
            todo = sorted((e for e in self._entries.values() if e.pending and e.calc is None),
                          key=lambda e: e.pending[0].t_submit)
        resident = sum(1 for e in self._entries.values() if e.calc is not None and e.pending)
        for e in todo:
            if resident >= self.max_batch:
                break
            if self._admit_one(e):
                resident += 1
        with self._lock:
            batch, calcs = self._take_batch()
        if not batch:
            return 0
        self._run(batch, calcs)
        return len(batch)

    def pending(self):
        with self._lock:
            return len(self._arrivals) + sum(len(e.pending) for e in self._entries.values())

    # -- background threads ------------------------------------------------------
    def start(self):
        self._stop = False
        self._threads = [threading.Thread(target=self._scheduler, name="sf-scheduler", daemon=True)]
        self._threads += [threading.Thread(target=self._admitter, name=f"sf-admitter-{i}", daemon=True)
                          for i in range(self.n_admitters)]
        for t in self._threads:
            t.start()

    def _scheduler(self):
        while True:
            with self._cond:
                while True:
                    if self._stop:
                        return
                    self._drain_arrivals()
                    batch, calcs = self._take_batch()
                    if batch:
                        break
                    self._cond.wait(0.05)
            self._run(batch, calcs)

    def _admitter(self):
        while True:
            with self._cond:
                while True:
                    if self._stop:
                        return
                    self._drain_arrivals()
                    e = self._next_to_admit()
                    if e is not None:
                        break
                    self._cond.wait(0.05)
            if not self._admit_one(e) and e.calc is None and e.pending:
                with self._cond:  # no room yet: wait for a batch to finish
                    if not self._stop:
                        self._cond.wait(0.01)

    def stop(self):
        with self._cond:
            self._stop = True
            self._cond.notify_all()
        for t in self._threads:
            t.join()
        self._threads = []

    def close(self):
        self.stop()
        for e in self._entries.values():
            if e.calc is not None:
                e.calc.close()
                e.calc = None
        self.resident_bytes = 0
