"""Request loop: many independent ReaxFF jobs on one GPU with continuous
batching.

A request is a periodic system plus either a single-point evaluation
(energies, forces and QEq charges) or a short NVE run of n steps.  The loop
keeps two segment handles (independent systems in one set of device arrays,
rg_set_segments) and drives them concurrently from two host threads, each
handle on its own CUDA stream:

* the evaluation batch: every iteration takes the requests admitted since
  the last one, single points and the first force evaluation of new MD
  requests alike, and evaluates them together;
* the MD cohort: the MD requests in flight advance together a few steps per
  iteration; when requests finish or new ones (evaluated in the previous
  iteration) are ready, the cohort is rebuilt with the state of every
  continuing request carried over exactly (positions, velocities, forces,
  QEq histories), so a trajectory does not depend on what it shares the
  GPU with.

Admission is by device-memory footprint: a request is admitted when its
estimated footprint fits beside the requests on the device; requests that
arrive while others run wait for that.  Latency is completion time minus
arrival time.
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
    # MD state between cohort rebuilds: x, v, f, s_hist, t_hist
    state: tuple = None
    steps_done: int = 0

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival


@dataclass
class ServeStats:
    completed: int = 0
    wall: float = 0.0
    iterations: int = 0
    rebuilds: int = 0
    max_atoms_on_device: int = 0
    latencies: list = field(default_factory=list)

    def summary(self) -> dict:
        lat = np.array(self.latencies) if self.latencies else np.zeros(1)
        return {"completed": self.completed, "wall_s": self.wall,
                "req_per_s": self.completed / self.wall if self.wall > 0 else 0.0,
                "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "iterations": self.iterations, "cohort_rebuilds": self.rebuilds,
                "max_atoms_on_device": self.max_atoms_on_device}


class ReaxServer:
    def __init__(self, ffield: str, precision: int = PREC_MIXED, hbm_budget: int = 32 << 30,
                 dt: float = 0.25, md_chunk: int = 10, device: int = 0):
        self.eval_h = ReaxGPU(ffield, precision=precision, device=device)
        self.md_h = ReaxGPU(ffield, precision=precision, device=device)
        self.bpa = BYTES_PER_ATOM[precision]
        self.budget = hbm_budget
        self.dt = dt
        self.md_chunk = md_chunk
        self.pool = cf.ThreadPoolExecutor(2)
        self.md_active: list = []          # requests in the MD cohort, cohort order
        self.md_ready: list = []           # evaluated, waiting to join the cohort
        self.md_offsets = None

    def close(self):
        self.pool.shutdown()
        self.eval_h.close()
        self.md_h.close()

    # -- one evaluation batch (runs in a worker thread) --------------------
    def _evaluate(self, batch: list):
        g = self.eval_h
        off = g.set_systems([r.system for r in batch])
        q, _, _ = g.qeq()
        f, _ = g.compute()
        es = g.energies()
        s_hist, t_hist = g.get_histories() if any(r.kind == "md" for r in batch) else (None, None)
        for k, r in enumerate(batch):
            sl = slice(off[k], off[k] + r.system.n)
            if r.kind == "sp":
                r.q, r.f, r.energies = q[sl].copy(), f[sl].copy(), es[k]
            else:
                r.state = (r.system.x.copy(), r.system.v.copy(), f[sl].copy(),
                           s_hist[:, sl].copy(), t_hist[:, sl].copy())
                r.energies = es[k]
        return batch

    # -- the MD cohort ------------------------------------------------------
    def _save_cohort(self):
        if not self.md_active:
            return
        g = self.md_h
        x, v, q, f = g.get_atoms()
        s_hist, t_hist = g.get_histories()
        for k, r in enumerate(self.md_active):
            sl = slice(self.md_offsets[k], self.md_offsets[k] + r.system.n)
            r.state = (x[sl].copy(), v[sl].copy(), f[sl].copy(), s_hist[:, sl].copy(),
                       t_hist[:, sl].copy())
            r.q = q[sl].copy()

    def _rebuild_cohort(self, members: list):
        g = self.md_h
        self.md_active = members
        if not members:
            self.md_offsets = None
            return
        systems = [r.system for r in members]
        self.md_offsets = g.set_systems(systems)
        x = np.concatenate([r.state[0] for r in members])
        v = np.concatenate([r.state[1] for r in members])
        f = np.concatenate([r.state[2] for r in members])
        s_hist = np.concatenate([r.state[3] for r in members], axis=1)
        t_hist = np.concatenate([r.state[4] for r in members], axis=1)
        g.set_state(x, v, f)
        g.set_histories(s_hist, t_hist)

    def _advance(self, k: int):
        if self.md_active and k > 0:
            self.md_h.run(k, self.dt, energies=False)
            for r in self.md_active:
                r.steps_done += k

    # -- the loop -----------------------------------------------------------
    def serve(self, requests: list, realtime: bool = True) -> ServeStats:
        """Run a request stream (arrival times in seconds from the start).
        realtime=False admits every request at once (offline batch)."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        waiting: deque = deque()
        stats = ServeStats()
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        on_device = 0          # atoms of admitted, unfinished requests
        while pending or waiting or self.md_active or self.md_ready:
            t = now()
            while pending and (not realtime or pending[0].arrival <= t):
                waiting.append(pending.popleft())
            if not waiting and not self.md_active and not self.md_ready:
                # idle until the next arrival
                time.sleep(max(0.0, pending[0].arrival - now()))
                continue
            batch = []
            while waiting and (on_device + waiting[0].system.n) * self.bpa <= self.budget:
                r = waiting.popleft()
                r.t_admit = now()
                on_device += r.system.n
                batch.append(r)
            if not batch and not self.md_active and not self.md_ready and waiting:
                # a request larger than the whole budget runs alone
                r = waiting.popleft()
                r.t_admit = now()
                on_device += r.system.n
                batch.append(r)
            stats.max_atoms_on_device = max(stats.max_atoms_on_device, on_device)
            # cohort membership changes between iterations only
            done = [r for r in self.md_active if r.steps_done >= r.nsteps]
            if done or self.md_ready:
                self._save_cohort()
                for r in done:
                    r.x, r.v, r.f = r.state[0], r.state[1], r.state[2]
                    r.t_done = now()
                    on_device -= r.system.n
                    stats.latencies.append(r.latency)
                    stats.completed += 1
                keep = [r for r in self.md_active if r.steps_done < r.nsteps]
                self._rebuild_cohort(keep + self.md_ready)
                self.md_ready = []
                stats.rebuilds += 1
            k = min([self.md_chunk] + [r.nsteps - r.steps_done for r in self.md_active]) \
                if self.md_active else 0
            fe = self.pool.submit(self._evaluate, batch) if batch else None
            fm = self.pool.submit(self._advance, k) if k > 0 else None
            if fe is not None:
                for r in fe.result():
                    if r.kind == "sp":
                        r.t_done = now()
                        on_device -= r.system.n
                        stats.latencies.append(r.latency)
                        stats.completed += 1
                    elif r.nsteps == 0:
                        r.x, r.v, r.f = r.state[0], r.state[1], r.state[2]
                        r.t_done = now()
                        on_device -= r.system.n
                        stats.latencies.append(r.latency)
                        stats.completed += 1
                    else:
                        self.md_ready.append(r)
            if fm is not None:
                fm.result()
            stats.iterations += 1
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
