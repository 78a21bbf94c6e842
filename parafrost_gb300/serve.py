"""Serving loop: simplification requests arrive over time and are answered by
batched sigmify rounds on one GPU.

A request is one formula. Requests go to a lane by size (small and large). A
worker thread of a lane takes every request waiting in the lane when it becomes
free, admits them in arrival order while their estimated device footprint fits
its share of the HBM budget (and the batch's formula cap), and runs one batched
round over them (``pf_sigma_upload_batch`` -> ``pf_sigma_round`` ->
``pf_sigma_batch_download``): each formula gets exactly the result of its own
round. Batched mode runs two workers per lane, each with its own context and
stream: the batches of all workers are on the device at once, one batch's copies
and host work overlap the others' kernels, a request that arrives while batches
run is admitted by the next worker of its lane that frees up, and a small request
never waits behind a large one. In ``plain`` mode one worker runs every request
alone through the single-formula calls instead, the comparison point for
batching. Latency is measured from a request's arrival to the moment its result
is on the host.

There is no counterpart in the reference (ParaFROST simplifies the formula of one
solver object inside ``sigmify()``); the per-formula work is the reference's
round, unchanged.
"""
from __future__ import annotations

import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from .options import Options
from .sigma import Result, Simplifier


def estimate_footprint(num_vars: int, num_clauses: int, num_literals: int) -> int:
    """Device bytes a formula needs inside a context: clause store with growth room
    (headers 16 B + stamps 4 B per clause slot, 1.5x), literals and occurrence refs
    (4 B each, 1.5x), witness room (4 B per literal + 8 B per variable), about 110 B
    of per-variable arrays, and a third more for stage scratch."""
    b = 1.5 * 20 * num_clauses + 1.5 * 8 * num_literals + 4 * num_literals + 118 * num_vars
    return int(b * 4 / 3) + 4096


@dataclass
class Request:
    formula: tuple                # (num_vars, lits, offsets)
    arrival: float                # time.perf_counter() when it arrived
    done: threading.Event = field(default_factory=threading.Event)
    status: int | None = None     # PF_OK / PF_UNSAT, or a negative pf_status
    phases: int = 0
    result: Result | None = None
    error: str | None = None
    finished: float = 0.0
    batch: int = -1               # index of the batch that served it

    @property
    def latency(self) -> float:
        return self.finished - self.arrival

    def wait(self, timeout: float | None = None) -> bool:
        return self.done.wait(timeout)


class Server:
    """One GPU; worker threads, each with its own context and stream, in lanes by
    request size; requests admitted in arrival order within a lane.

    Batched mode has two lanes: requests of up to ``small_clauses`` clauses go to
    the small lane, larger ones to the large lane, each lane with its own queue and
    workers, so a small request never waits behind a multi-million-clause batch. A
    lane's free worker admits every request waiting in its lane (while it fits the
    worker's share of the HBM budget) into its next batched round; the workers'
    rounds overlap on the device. Plain mode has one lane and one worker that runs
    each request alone."""

    def __init__(self, opts: Options | None = None, hbm_budget: int = 64 << 30, max_batch: int = 4096,
                 mode: str = "batched", library: str | None = None, workers: int | None = None,
                 small_clauses: int = 200_000, lanes: int | None = None):
        if mode not in ("batched", "plain"):
            raise ValueError("mode is 'batched' or 'plain'")
        self.opts = opts or Options(all=1)
        self.hbm_budget = int(hbm_budget)
        self.max_batch = int(max_batch)
        self.mode = mode
        self.library = library
        self.lanes = int(lanes) if lanes else (2 if mode == "batched" else 1)
        self.small_clauses = int(small_clauses)
        # workers per lane
        self.per_lane = int(workers) if workers else (2 if mode == "batched" else 1)
        self.workers = self.per_lane * self.lanes
        self.worker_budget = self.hbm_budget // self.workers
        self.queues: list = [queue.Queue() for _ in range(self.lanes)]
        self.q = self.queues[0]
        self.batches: list = []          # (formulas, clauses, estimated bytes, device bytes held after, launches)
        self.max_footprint = 0           # device bytes held by all workers' contexts at once, at most
        self._held: list = [0] * self.workers
        self._lock = threading.Lock()
        self._lane_locks = [threading.Lock() for _ in range(self.lanes)]
        self._stop = threading.Event()
        self._threads: list = []
        self._pending: list = [[] for _ in range(self.lanes)]

    def lane_of(self, formula: tuple) -> int:
        """The lane of a request: 0 (small) or the last (large) by clause count."""
        return 0 if self.lanes == 1 or formula[2].size - 1 <= self.small_clauses else self.lanes - 1

    # ---- client side
    def submit(self, formula: tuple, arrival: float | None = None) -> Request:
        r = Request(formula, time.perf_counter() if arrival is None else arrival)
        nv, lits, off = formula
        if estimate_footprint(nv, off.size - 1, lits.size) > self.worker_budget:
            self._finish(r, -2, error="request larger than the HBM budget")
            return r
        self.queues[self.lane_of(formula)].put(r)
        return r

    def start(self) -> "Server":
        for w in range(self.workers):
            t = threading.Thread(target=self._run, args=(w,), name=f"sigma-server-{w}", daemon=True)
            t.start()
            self._threads.append(t)
        return self

    def stop(self, timeout: float | None = None) -> None:
        self._stop.set()
        for t in self._threads:
            t.join(timeout)

    def __enter__(self):
        return self.start()

    def __exit__(self, *exc):
        self.stop()

    # ---- server side
    def _finish(self, r: Request, status: int, phases: int = 0, result=None, error=None, batch: int = -1):
        r.status, r.phases, r.result, r.error, r.batch = status, phases, result, error, batch
        r.finished = time.perf_counter()
        r.done.set()

    def _admit(self, lane: int) -> list:
        """The next batch of a lane (called under the lane's lock): waiting requests in
        arrival order while they fit one worker's budget; [] once stopped with
        nothing waiting."""
        q = self.queues[lane]
        reqs = self._pending[lane]
        self._pending[lane] = []
        while not reqs:
            if self._stop.is_set() and q.empty():
                return []
            try:
                r = q.get(timeout=0.02)
            except queue.Empty:
                continue
            reqs = [r]
        while True:
            try:
                reqs.append(q.get_nowait())
            except queue.Empty:
                break
        batch, used = [], 0
        for i, r in enumerate(reqs):
            nv, lits, off = r.formula
            need = estimate_footprint(nv, off.size - 1, lits.size)
            if batch and (used + need > self.worker_budget or len(batch) >= self.max_batch):
                self._pending[lane] = reqs[i:]
                break
            batch.append(r)
            used += need
        return batch

    def _run(self, w: int) -> None:
        lane = w % self.lanes
        try:
            ctx = Simplifier(self.opts, library=self.library)
        except Exception as e:  # no context: this worker answers what it admits with the error
            while True:
                with self._lane_locks[lane]:
                    batch = self._admit(lane)
                if not batch:
                    return
                for r in batch:
                    self._finish(r, getattr(e, "status", -4), error=str(e))
        try:
            while True:
                with self._lane_locks[lane]:
                    batch = self._admit(lane)
                with self._lock:
                    bi = len(self.batches)
                    if batch:
                        self.batches.append(None)  # this batch's slot, filled below
                if not batch:
                    break
                launches = 0
                if self.mode == "plain":
                    for r in batch:
                        launches += self._serve_one(ctx, r, bi)
                else:
                    launches = self._serve_batch(ctx, batch, bi)
                fp = ctx.footprint()
                est = sum(estimate_footprint(r.formula[0], r.formula[2].size - 1, r.formula[1].size) for r in batch)
                with self._lock:
                    self._held[w] = fp
                    self.max_footprint = max(self.max_footprint, sum(self._held))
                    self.batches[bi] = (len(batch), int(sum(r.formula[2].size - 1 for r in batch)), est, fp, launches)
        finally:
            ctx.close()

    def _serve_one(self, ctx: Simplifier, r: Request, bi: int) -> int:
        nv, lits, off = r.formula
        try:
            ctx.awaken(nv, lits, off)
            st = ctx.sigmify()
            self._finish(r, st.status, st.phases_run, ctx.result() if st.status == 0 else None, batch=bi)
            return st.kernel_launches
        except Exception as e:  # the request fails, the server goes on
            self._finish(r, getattr(e, "status", -4), error=str(e), batch=bi)
            return 0

    def _serve_batch(self, ctx: Simplifier, batch: list, bi: int) -> int:
        forms = [r.formula for r in batch]
        try:
            ctx.awaken_batch(forms)
            st = ctx.sigmify()
            out = ctx.batch_results()
        except Exception as e:
            for r in batch:
                self._finish(r, getattr(e, "status", -4), error=str(e), batch=bi)
            return 0
        for r, (st_f, ph, res) in zip(batch, out):
            self._finish(r, st_f, ph, res if st_f == 0 else None, batch=bi)
        return st.kernel_launches


def poisson_load(server: Server, pool: list, rate: float, num: int, seed: int = 1) -> list:
    """Open-loop Poisson arrivals at `rate` requests/s: request i (formula
    pool[i % len(pool)]) is submitted at its scheduled time, which is also its
    arrival time (a late submit does not hide queueing). Returns the requests after
    all have finished."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=num)
    t0 = time.perf_counter()
    sched = t0 + np.cumsum(gaps)
    reqs = []
    for i in range(num):
        delay = sched[i] - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        reqs.append(server.submit(pool[i % len(pool)], arrival=float(sched[i])))
    for r in reqs:
        r.wait()
    return reqs


def summarize(reqs: list, server: Server) -> dict:
    lat = np.array([r.latency for r in reqs if r.status is not None and r.status >= 0])
    first = min(r.arrival for r in reqs)
    last = max(r.finished for r in reqs)
    ok = [r for r in reqs if r.status is not None and r.status >= 0]
    return {"requests": len(reqs), "served": len(ok), "failed": len(reqs) - len(ok),
            "formulas_per_s": len(ok) / (last - first) if last > first else None,
            "clauses_per_s": sum(r.formula[2].size - 1 for r in ok) / (last - first) if last > first else None,
            "p50_ms": float(np.percentile(lat, 50) * 1e3) if lat.size else None,
            "p99_ms": float(np.percentile(lat, 99) * 1e3) if lat.size else None,
            "batches": len(server.batches),
            "mean_batch": float(np.mean([b[0] for b in server.batches])) if server.batches else 0.0,
            "gpu_launches": int(sum(b[4] for b in server.batches)),
            "max_footprint_bytes": int(server.max_footprint)}
