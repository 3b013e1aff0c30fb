"""Request loop: many independent ReaxFF jobs on one GPU with continuous
batching.

A request is a periodic system plus either a single-point evaluation
(energies, forces and QEq charges) or a short NVE run of n steps.  Systems
live as segments of handles (independent systems in one set of device
arrays, rg_set_segments), and two kinds of work run side by side, each
handle on its own CUDA stream, driven from worker threads:

* evaluation batches: whenever an evaluation handle is free, every
  admitted request not yet evaluated is loaded into it and evaluated
  together -- single points, and the first QEq + force evaluation of new
  MD requests;
* the MD cohort: the MD requests in flight advance together a few steps at
  a time on one handle.  Between two such chunks the cohort is regrouped on
  the device (rg_regroup_segments): finished trajectories leave, and new
  MD requests join straight from the evaluation handle that evaluated
  them, their positions, velocities, forces and QEq histories copied
  device to device.  No trajectory's state passes through host memory
  between its input and its result, and a trajectory does not depend on
  what it shares the GPU with.

An evaluation batch starts as soon as a handle is free, without waiting for
the MD chunk, and a chunk starts as soon as the previous one is done.
Admission is by device-memory footprint: a request is admitted when its
estimated footprint fits beside the requests on the device; requests that
arrive while others run wait for that.  Latency is completion time minus
arrival time, reported per request kind.
"""
from __future__ import annotations

import concurrent.futures as cf
import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from .api import PREC_MIXED, ReaxGPU

# device bytes per atom of a handle (pair list with H values, bond arrays,
# H-bond partners, work lists, per-atom state) at liquid densities: a
# conservative estimate, used for admission
BYTES_PER_ATOM = {0: 16 << 10, PREC_MIXED: 13 << 10}


@dataclass
class Request:
    rid: int
    system: object                # sw_reaxff_gb300.systems.System
    kind: str                     # "sp" (single point) or "md"
    nsteps: int = 0
    arrival: float = 0.0          # seconds from the start of the stream
    # results
    t_admit: float = math.nan
    t_done: float = math.nan
    q: np.ndarray = None
    f: np.ndarray = None
    energies: dict = None
    x: np.ndarray = None
    v: np.ndarray = None
    steps_done: int = 0

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival


def _pct(lat, p):
    return float(np.percentile(np.array(lat), p) * 1e3) if lat else None


@dataclass
class ServeStats:
    completed: int = 0
    wall: float = 0.0
    eval_batches: int = 0
    md_chunks: int = 0
    rebuilds: int = 0
    max_atoms_on_device: int = 0
    latencies: list = field(default_factory=list)
    latencies_sp: list = field(default_factory=list)
    latencies_md: list = field(default_factory=list)
    last_arrival: float = 0.0

    def summary(self) -> dict:
        return {"completed": self.completed, "wall_s": self.wall,
                "req_per_s": self.completed / self.wall if self.wall > 0 else 0.0,
                "arrivals_end_s": self.last_arrival,
                "p50_ms": _pct(self.latencies, 50), "p99_ms": _pct(self.latencies, 99),
                "single_point": {"count": len(self.latencies_sp),
                                 "p50_ms": _pct(self.latencies_sp, 50),
                                 "p99_ms": _pct(self.latencies_sp, 99)},
                "md": {"count": len(self.latencies_md), "p50_ms": _pct(self.latencies_md, 50),
                       "p99_ms": _pct(self.latencies_md, 99)},
                "eval_batches": self.eval_batches, "md_chunks": self.md_chunks,
                "cohort_regroups": self.rebuilds,
                "max_atoms_on_device": self.max_atoms_on_device}


class ReaxServer:
    def __init__(self, ffield: str, precision: int = PREC_MIXED, hbm_budget: int = 32 << 30,
                 dt: float = 0.25, md_chunk: int = 10, device: int = 0, n_eval: int = 3):
        self.eval_h = [ReaxGPU(ffield, precision=precision, device=device) for _ in range(n_eval)]
        self.md_h = ReaxGPU(ffield, precision=precision, device=device)
        self.bpa = BYTES_PER_ATOM[precision]
        self.budget = hbm_budget
        self.dt = dt
        self.md_chunk = md_chunk
        self.pool = cf.ThreadPoolExecutor(n_eval + 1)
        self.md_active: list = []          # requests of the MD cohort, segment order
        # per evaluation handle: MD requests evaluated there, waiting to join
        # the cohort as (segment, request); the handle is not reused before
        self.hold = [[] for _ in range(n_eval)]

    def close(self):
        self.pool.shutdown()
        for g in self.eval_h:
            g.close()
        self.md_h.close()

    # -- one evaluation batch (worker thread) -------------------------------
    def _evaluate(self, k: int, batch: list):
        g = self.eval_h[k]
        off = g.set_systems([r.system for r in batch])
        q, _, _ = g.qeq()
        f, _ = g.compute()
        es = g.energies()
        for s, r in enumerate(batch):
            sl = slice(off[s], off[s] + r.system.n)
            r.energies = es[s]
            if r.kind == "sp" or r.nsteps == 0:
                r.q, r.f = q[sl].copy(), f[sl].copy()
                if r.kind == "md":
                    r.x, r.v = r.system.x.copy(), r.system.v.copy()
        return batch

    # -- one MD chunk (worker thread) ---------------------------------------
    def _advance(self, k: int):
        self.md_h.run(k, self.dt, energies=False)
        for r in self.md_active:
            r.steps_done += k

    def _regroup(self, stats, finish):
        """Between chunks: finished trajectories leave the cohort (their
        results read back), MD requests held by idle evaluation handles join
        it, all on the device."""
        done = [i for i, r in enumerate(self.md_active) if r.steps_done >= r.nsteps]
        for i in done:
            r = self.md_active[i]
            r.x, r.v, r.q, r.f = self.md_h.segment_atoms(i)
            finish(r)
        keep = [i for i, r in enumerate(self.md_active) if r.steps_done < r.nsteps]
        ready = [k for k in range(len(self.eval_h)) if self.hold[k] and not self.eval_busy[k]]
        if not done and not ready:
            return
        members = [self.md_active[i] for i in keep]
        if ready:
            for j, k in enumerate(ready):
                sel = [s for s, _ in self.hold[k]]
                kp = keep if j == 0 else list(range(len(members)))
                self.md_h.regroup(kp, self.eval_h[k], sel)
                members += [r for _, r in self.hold[k]]
                self.hold[k] = []
        elif keep:
            self.md_h.regroup(keep)
        self.md_active = members
        stats.rebuilds += 1

    # -- the loop -----------------------------------------------------------
    def serve(self, requests: list, realtime: bool = True) -> ServeStats:
        """Run a request stream (arrival times in seconds from the start).
        realtime=False admits every request at once (offline batch)."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        waiting: deque = deque()
        stats = ServeStats()
        stats.last_arrival = pending[-1].arrival if pending else 0.0
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        on_device = [0]          # atoms of admitted, unfinished requests
        fut_eval = {}            # evaluation handle -> future
        fut_md = None
        self.eval_busy = [False] * len(self.eval_h)

        def finish(r):
            r.t_done = now()
            on_device[0] -= r.system.n
            stats.latencies.append(r.latency)
            (stats.latencies_sp if r.kind == "sp" else stats.latencies_md).append(r.latency)
            stats.completed += 1

        while pending or waiting or fut_eval or fut_md is not None or self.md_active or \
                any(self.hold):
            t = now()
            while pending and (not realtime or pending[0].arrival <= t):
                waiting.append(pending.popleft())
            # finished evaluation batches
            for k in [k for k, fu in fut_eval.items() if fu.done()]:
                batch = fut_eval.pop(k).result()
                self.eval_busy[k] = False
                for s, r in enumerate(batch):
                    if r.kind == "sp" or r.nsteps == 0:
                        finish(r)
                    else:
                        self.hold[k].append((s, r))
            # the MD side: regroup between chunks, then the next chunk
            if fut_md is not None and fut_md.done():
                fut_md.result()
                fut_md = None
            if fut_md is None:
                self._regroup(stats, finish)
                if self.md_active:
                    kk = min([self.md_chunk] + [r.nsteps - r.steps_done for r in self.md_active])
                    fut_md = self.pool.submit(self._advance, kk)
                    stats.md_chunks += 1
            # admission into a free evaluation handle
            free = [k for k in range(len(self.eval_h))
                    if not self.eval_busy[k] and not self.hold[k]]
            if free and waiting:
                batch = []
                while waiting and (on_device[0] + waiting[0].system.n) * self.bpa <= self.budget:
                    r = waiting.popleft()
                    r.t_admit = now()
                    on_device[0] += r.system.n
                    batch.append(r)
                if not batch and on_device[0] == 0:
                    # a request larger than the whole budget runs alone
                    r = waiting.popleft()
                    r.t_admit = now()
                    on_device[0] += r.system.n
                    batch.append(r)
                if batch:
                    k = free[0]
                    self.eval_busy[k] = True
                    fut_eval[k] = self.pool.submit(self._evaluate, k, batch)
                    stats.eval_batches += 1
            stats.max_atoms_on_device = max(stats.max_atoms_on_device, on_device[0])
            # wait for a worker or the next arrival
            futs = list(fut_eval.values()) + ([fut_md] if fut_md is not None else [])
            timeout = None
            if realtime and pending:
                timeout = max(0.0, pending[0].arrival - now())
            if futs:
                cf.wait(futs, timeout=timeout, return_when=cf.FIRST_COMPLETED)
            elif timeout is not None:
                time.sleep(timeout)
        stats.wall = now()
        return stats


def sequential(ffield: str, requests: list, dt: float = 0.25, precision: int = 0) -> float:
    """The same requests solved one after another with one plain handle (the
    sequential baseline); returns the wall time."""
    g = ReaxGPU(ffield, precision=precision)
    t0 = time.perf_counter()
    for r in requests:
        g.set_system(r.system)
        if r.kind == "sp":
            g.qeq()
            g.compute()
        else:
            g.run(r.nsteps, dt, energies=False)
            g.get_atoms()
    wall = time.perf_counter() - t0
    g.close()
    return wall


def stream_specs(n: int, rate: float, seed: int = 0, min_atoms: int = 100,
                 max_atoms: int = 20000, md_fraction: float = 0.3, md_steps=(10, 500)):
    """Request specifications of a Poisson stream at `rate` req/s: sizes
    log-uniform in [min_atoms, max_atoms], a random pack of
    H2O/CH4/NH3/CO2/C2H6 at a density uniform in 0.3-1.0 g/cm3 each,
    md_fraction of them NVE runs with a step count uniform in md_steps.
    Each spec: (rid, arrival, size, density, pack_seed, kind, nsteps)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(n):
        t += rng.exponential(1.0 / rate)
        size = int(round(math.exp(rng.uniform(math.log(min_atoms), math.log(max_atoms)))))
        dens = float(rng.uniform(0.3, 1.0))
        pseed = int(rng.integers(1 << 30))
        if rng.uniform() < md_fraction:
            out.append((k, t, size, dens, pseed, "md", int(rng.integers(md_steps[0], md_steps[1] + 1))))
        else:
            out.append((k, t, size, dens, pseed, "sp", 0))
    return out


def make_request(spec) -> Request:
    """Generate the system of one spec (picklable, for process pools)."""
    from . import systems
    rid, t, size, dens, pseed, kind, nsteps = spec
    return Request(rid, systems.small_pack(size, dens, seed=pseed), kind, nsteps, t)


def request_stream(n: int, rate: float, seed: int = 0, pool=None, **kw) -> list:
    """Requests of stream_specs(...), systems generated (in `pool` if given)."""
    specs = stream_specs(n, rate, seed, **kw)
    if pool is not None:
        return list(pool.map(make_request, specs))
    return [make_request(s) for s in specs]
