#!/usr/bin/env python3
"""ReaxFF MD throughput on GB300: atom-steps/s of NVE molecular dynamics.

One step = initial_integrate -> QEq (dual pipelined CG) -> full ReaxFF force
step (pair list, bond orders, bonded terms, H-bonds, vdW+Coulomb, dBond
forces) -> final_integrate, on the seeded 1,048,576-atom H2O/CH4/C2H6/NH3
mixture at 0.8 g/cm^3 (synthetic; the reference publishes no dataset), FP64.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  With N>1 (launched under torch.distributed.run) every
rank runs an independent replica of the workload on its own GPU ("replicas
only": the single-GPU path has no cross-GPU exchange) and value is the sum
of atom-steps over the max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "atom-steps/s at 1M atoms (FP64 NVE MD step incl. QEq)"
METRIC_MIXED = "atom-steps/s at 1M atoms (mixed FP32/FP64 NVE MD step incl. QEq)"
UNIT = "atom-steps/s"
DT = 0.25          # fs
SEED = 7

# Per-unit figures of the kernels that can dominate the FP64 step.  FP64
# FLOP (2*dfma + dmul + dadd, SASS thread-instruction counts) and DRAM
# bytes (dram__bytes_read + write) are from one ncu capture of the
# 52,428-atom case of the same mixture (`--scale 0.05`; the nonbonded
# kernel's force-only variant, which the timed steps run); the algorithmic
# bytes are the compulsory traffic of the canonical layout: per unordered
# pair one 4-byte index (+ the 8-byte H value where the kernel produces or
# reads H), plus per-atom position/charge/type reads and result writes; the
# streamed bytes are what the kernel's layout reads per unit (the QEq
# SpMV's full rows: index and FP32-pair H of every directed entry).  Units:
# per directed pair for the pair-list build, per unordered pair for the
# nonbonded kernel, per list entry for one QEq SpMV (both systems).
FP64_PER_UNIT = {
    # phase: (kernel, unit, FP64 FLOP/unit, DRAM bytes/unit, algorithmic
    #         bytes/unit, algorithmic bytes/atom, streamed bytes/unit)
    "pair_list+H": ("k_build_nbrs_tiles", "directed pair", 0.0006, 11.61, 6.0, 64.0, 12.0),
    "nonbonded": ("k_nonbonded", "unordered pair", 5.80, 17.78, 4.0, 60.0, 8.0),
    "qeq_spmv": ("k_spmvp", "list entry", 0.013, 12.79, 6.0, 96.0, 12.0),
}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    p.add_argument("--scale", type=float, default=1.0,
                   help="workload size relative to the 1,048,576-atom mixture")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--form", default="fp64", choices=["fp64", "mixed"],
                   help="precision of the main timed handle (mixed: for profiling the mixed "
                        "kernels alone; the headline metric is the FP64 form)")
    p.add_argument("--no-mixed", action="store_true",
                   help="skip the mixed-precision measurement of the same workload")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cpu-scale", type=float, default=0.02,
                   help="size of the CPU-baseline sample relative to 1M atoms")
    p.add_argument("--no-batched", action="store_true",
                   help="skip the batched single-point measurement (512 small systems)")
    p.add_argument("--no-serve", action="store_true",
                   help="skip the serving-loop measurement (Poisson request stream)")
    p.add_argument("--pair-kernel", type=int, default=0, choices=[0, 1, 2],
                   help="pair-list build: 0 autotuned, 1 warp per atom, 2 per-cell tiles")
    p.add_argument("--no-water", action="store_true",
                   help="skip the 6,000-atom water measurement (2,000 H2O, 100 NVE steps)")
    p.add_argument("--water-cpu", action="store_true",
                   help="also time the oracle on the full 100 steps of the 6,000-atom water "
                        "box (single thread, a few minutes)")
    p.add_argument("--batch-systems", type=int, default=512)
    p.add_argument("--serve-requests", type=int, default=300)
    p.add_argument("--serve-rate", type=float, default=200.0,
                   help="mean arrival rate of the request stream (req/s)")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


class Dist:
    def __init__(self, backend):
        self.rank, self.world, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            td.init_process_group(backend)
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        dev = "cuda" if self.td.get_backend() == "nccl" else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        dev = "cuda" if self.td.get_backend() == "nccl" else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return json.load(open(path))
    except Exception:
        return {}


def cpu_baseline(cpu_scale: float, procs: int = 1, warmup: int = 1, steps: int = 2):
    """The oracle (single-threaded restatement of the reference CPU path,
    its QEq equal bit for bit to the reference's own) on bounded samples of
    the same workload: `procs` processes, each a smaller periodic box of the
    same mixture at the same density (its own seed) running warm NVE steps
    -- setup evaluation and `warmup` steps untimed, then `steps` timed steps
    (initial_integrate, QEq from the extrapolated s/t histories, forces,
    final_integrate).  Returns (atom-steps/s over all processes, processes,
    atoms per process)."""
    import multiprocessing as mp
    jobs = [(cpu_scale, SEED + k, warmup, steps) for k in range(procs)]
    if procs <= 1:
        res = [_cpu_md_sample(jobs[0])]
    else:
        with mp.get_context("spawn").Pool(procs) as pool:
            res = pool.map(_cpu_md_sample, jobs)
    atoms = sum(r[0] for r in res)
    slowest = max(r[1] for r in res)          # the processes run side by side
    return atoms * steps / slowest, procs, res[0][0]


def _cpu_md_sample(arg):
    cpu_scale, seed, warmup, steps = arg
    sys.path.insert(0, ROOT)
    from oracle.pyoracle import Oracle
    from sw_reaxff_gb300 import systems
    from sw_reaxff_gb300.api import DEFAULT_FFIELD
    s = systems.mixture(scale=cpu_scale, seed=seed)
    o = Oracle(DEFAULT_FFIELD)
    o.set_system(s.box, s.x, s.types(["C", "H", "O", "N"]), s.tag, None, s.v)
    o.run_nve(max(warmup, 1), DT)             # setup (cold QEq) + warm-up steps
    t0 = time.perf_counter()
    o.md_steps(steps, DT)
    return s.n, time.perf_counter() - t0


def _gen_batch_system(k):
    """System k of the batched workload: log-uniform 50-3000 atoms, a random
    pack of H2O/CH4/NH3/CO2/C2H6 at a density uniform in 0.3-1.0 g/cm3."""
    import math
    sys.path.insert(0, ROOT)
    from sw_reaxff_gb300 import systems
    rng = np.random.default_rng(1000 + k)
    size = int(round(math.exp(rng.uniform(math.log(50), math.log(3000)))))
    return systems.small_pack(size, float(rng.uniform(0.3, 1.0)), seed=20000 + k)


def _gen_request(spec):
    sys.path.insert(0, ROOT)
    from sw_reaxff_gb300 import serve
    return serve.make_request(spec)


def _spawn_pool():
    import multiprocessing as mp
    return mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1))


def batched_section(args, local):
    """512 independent small systems, one single point each (QEq + energies
    + forces), evaluated together as segments of one handle -- the whole
    step one captured graph launch (rg_single_point) -- in the mixed and the
    FP64 form; against the same systems solved one after another with a
    plain FP64 handle."""
    import torch
    from sw_reaxff_gb300 import ReaxGPU
    from sw_reaxff_gb300.api import DEFAULT_FFIELD, PREC_MIXED
    with _spawn_pool() as pool:
        S = pool.map(_gen_batch_system, range(args.batch_systems))
    natoms = sum(s.n for s in S)
    out = {"workload": f"{len(S)} periodic systems, {natoms} atoms, 50-3000 atoms "
                       "log-uniform, 0.3-1.0 g/cm3, single point (QEq+energies+forces)"}
    for label, prec in (("mixed", PREC_MIXED), ("fp64", 0)):
        g = ReaxGPU(DEFAULT_FFIELD, device=local, precision=prec)
        g.set_systems(S)
        st = torch.cuda.ExternalStream(g.stream())
        times = []
        for it in range(max(args.warmup, 2) + args.steps):
            g.set_histories(None, None)        # fresh single points
            if it == max(args.warmup, 2):
                s0 = g.stats()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            g.single_point()                   # QEq + forces: one graph replay
            e1.record(st)
            g.synchronize()
            if it >= max(args.warmup, 2):
                times.append(e0.elapsed_time(e1) / 1e3)
        s1 = g.stats()
        t_batch = float(np.mean(times))
        out[label] = {"batch_ms": t_batch * 1e3, "req_per_s": len(S) / t_batch,
                      "p50_ms": t_batch * 1e3, "p99_ms": t_batch * 1e3,
                      "atom_evals_per_s": natoms / t_batch,
                      "graph_replays": s1["step_graph_replays"] - s0["step_graph_replays"],
                      "kernels_per_batch": (s1["kernel_launches"] - s0["kernel_launches"])
                      / max(1, args.steps),
                      "cg_iters_s_t": [s1["cg_iters_s"], s1["cg_iters_t"]]}
        g.close()
    # sequential plain FP64 solves (host arrays in and out, one handle), on
    # a sample of the systems
    g = ReaxGPU(DEFAULT_FFIELD, device=local)
    sample = S[:: max(1, len(S) // 64)]
    for s in sample[:3]:
        g.set_system(s); g.qeq(); g.compute()
    lat = []
    for s in sample:
        t0 = time.perf_counter()
        g.set_system(s)
        g.qeq()
        g.compute()
        lat.append(time.perf_counter() - t0)
    g.close()
    out["sequential_fp64"] = {"req_per_s": 1.0 / float(np.mean(lat)),
                              "p50_ms": float(np.percentile(lat, 50) * 1e3),
                              "p99_ms": float(np.percentile(lat, 99) * 1e3),
                              "sample": len(sample)}
    out["speedup_vs_sequential_fp64"] = out["mixed"]["req_per_s"] / out["sequential_fp64"]["req_per_s"]
    return out


def serve_section(args, local):
    """The request loop on a Poisson stream (200 req/s by default; sizes
    100-20,000 atoms log-uniform; 70 % single points, 30 % NVE runs of
    10-500 steps), mixed form, against the same requests solved one after
    another with a plain FP64 handle (all of them)."""
    from sw_reaxff_gb300 import serve
    from sw_reaxff_gb300.api import DEFAULT_FFIELD, PREC_MIXED
    specs = serve.stream_specs(args.serve_requests, rate=args.serve_rate, seed=SEED)
    with _spawn_pool() as pool:
        reqs = pool.map(_gen_request, specs)
    srv = serve.ReaxServer(DEFAULT_FFIELD, precision=PREC_MIXED, device=local)
    warm = serve.request_stream(8, rate=1e6, seed=SEED + 1, max_atoms=2000, md_steps=(5, 10))
    srv.serve(warm, realtime=False)
    st = srv.serve(reqs, realtime=True)
    srv.close()
    out = {"workload": f"{len(reqs)} requests, Poisson {args.serve_rate:g} req/s, 100-20000 "
                       "atoms, 70% single point / 30% NVE 10-500 steps, mixed form",
           "offered_req_per_s": args.serve_rate, **st.summary()}
    work = sum(r.system.n * max(1, r.nsteps) for r in reqs)
    out["atom_steps_per_s"] = work / st.wall
    out["keeps_up"] = bool(out["req_per_s"] >= 0.95 * args.serve_rate)
    wall = serve.sequential(DEFAULT_FFIELD, reqs)
    out["sequential_fp64"] = {"req_per_s": len(reqs) / wall, "requests": len(reqs),
                              "wall_s": wall}
    out["speedup_vs_sequential_fp64"] = out["req_per_s"] / out["sequential_fp64"]["req_per_s"]
    return out


def water_section(args, local):
    """2,000 H2O (6,000 atoms) at 1.0 g/cm3, 300 K, 100 NVE steps of 0.25 fs,
    FP64 (the reference's own CPU-runnable scale): the GPU's 100 steps timed
    with CUDA events after a 5-step warm-up run, and -- with --water-cpu --
    the oracle's 100 steps on one thread (setup excluded)."""
    import torch
    from sw_reaxff_gb300 import ReaxGPU, systems
    from sw_reaxff_gb300.api import DEFAULT_FFIELD
    s = systems.water_box(2000, seed=2024)
    g = ReaxGPU(DEFAULT_FFIELD, device=local)
    g.set_system(s)
    g.run(5, DT, energies=False)
    g.set_system(s)
    g.run(0, DT, energies=False)              # setup: QEq from zero guesses + forces
    st = torch.cuda.ExternalStream(g.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    g.synchronize()
    e0.record(st)
    e = g.run(100, DT)
    e1.record(st)
    g.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    out = {"workload": "2,000 H2O, 6,000 atoms, 1.0 g/cm3, 300 K, 100 NVE steps of 0.25 fs, "
                       "FP64, QEq tol 1e-6",
           "gpu": {"atom_steps_per_s": s.n * 100 / t, "ms_per_step": t * 10.0,
                   "cg_iters_last_step": [g.stats()["cg_iters_s"], g.stats()["cg_iters_t"]],
                   "potential_energy_last": e["eng_vdwl"] + e["eng_coul"]}}
    g.close()
    if args.water_cpu:
        from oracle.pyoracle import Oracle
        o = Oracle(DEFAULT_FFIELD)
        o.set_system(s.box, s.x, s.types(["C", "H", "O", "N"]), s.tag, None, s.v)
        o.run_nve(0, DT)
        t0 = time.perf_counter()
        eo = o.md_steps(100, DT)
        tc = time.perf_counter() - t0
        out["cpu_oracle_1_thread"] = {"atom_steps_per_s": s.n * 100 / tc, "s_per_step": tc / 100,
                                      "potential_energy_last": eo["eng_vdwl"] + eo["eng_coul"]}
        out["speedup_gpu_vs_cpu"] = out["gpu"]["atom_steps_per_s"] / \
            out["cpu_oracle_1_thread"]["atom_steps_per_s"]
    return out


def workload_name(n, mixed=False):
    return (f"H2O/CH4/C2H6/NH3 0.5/0.2/0.2/0.1 mixture, {n} atoms, "
            "0.8 g/cm3, 300 K, NVE dt 0.25 fs, QEq tol 1e-6, "
            + ("mixed FP32/FP64 form" if mixed else "FP64"))


REF_SAMPLE_SCALE = 0.01      # 10,486-atom boxes of the mixture per process


def reference_arm(args):
    """--impl reference: the reference's CPU algorithm on all host cores.
    The reference itself needs LAMMPS and the Sunway toolchain, so this is
    the oracle port (force-step routines checked against the reference's own
    compiled CPU branches, QEq equal bit for bit to the reference's own
    pre_force).  Every process runs one bounded sample of the workload -- a
    10,486-atom box of the same mixture -- through warm NVE steps: setup and
    W warm-up steps untimed, K steps timed."""
    dist = Dist("gloo")
    if dist.rank != 0:
        dist.close()
        return
    procs = os.cpu_count() or 1
    t0 = time.perf_counter()
    value, cores, sample = cpu_baseline(REF_SAMPLE_SCALE, procs, max(args.warmup, 1),
                                        max(1, args.steps))
    total = sample * procs
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "impl": "reference",
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{procs} independent {sample}-atom boxes of the "
                               "H2O/CH4/C2H6/NH3 0.5/0.2/0.2/0.1 mixture, 0.8 g/cm3, 300 K, "
                               "NVE dt 0.25 fs, QEq tol 1e-6, FP64, warm steps",
                   "atoms": total, "parallelism": f"{procs} CPU processes",
                   "sample_atoms_per_process": sample, "processes": procs},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                         "sample": f"{procs} processes x {args.steps} warm NVE steps of a "
                                   f"{sample}-atom box of the same mixture (setup and "
                                   f"{max(args.warmup, 1)} warm-up steps untimed)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.perf_counter() - t0,
    }
    print(json.dumps(line), flush=True)
    dist.close()


def gpu_arm(args):
    import torch
    from sw_reaxff_gb300 import ReaxGPU, systems
    from sw_reaxff_gb300.api import DEFAULT_FFIELD, measure_fp64_peak

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = Dist("nccl")
    s = systems.mixture(scale=args.scale, seed=SEED + rank)
    n = s.n
    from sw_reaxff_gb300.api import PREC_MIXED
    main_mixed = args.form == "mixed"
    if main_mixed:
        args.no_mixed = True          # the main handle is the mixed form itself
    g = ReaxGPU(DEFAULT_FFIELD, device=local, precision=PREC_MIXED if main_mixed else 0,
                pair_kernel=args.pair_kernel)
    g.set_system(s)
    g.run(max(args.warmup, 1), DT, energies=False)          # setup + warm-up steps
    # phase breakdown from a separate, profiled run (events around every
    # kernel group; the CG iterations then run as plain launches)
    psteps = max(1, min(args.steps, 2))
    g.profile(True)
    g.run(psteps, DT, energies=False)
    g.synchronize()
    prof = g.profile_get()
    g.profile(False)
    # the roofline kernel: the step's largest phase among those with
    # per-unit figures (the QEq SpMV included); the timed steps carry events
    # around it alone (for the SpMV the CG iterations then run as plain
    # launches instead of their CUDA graph)
    dom = max(FP64_PER_UNIT, key=lambda k: prof.get(k, (0.0, 0))[0])
    stream = torch.cuda.ExternalStream(g.stream())
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clocks = Clocks(local)
    dist.barrier()
    g.synchronize()
    torch.cuda.synchronize()
    clocks.start()
    st0 = g.stats()
    launches0 = st0["kernel_launches"]
    g.profile(True, phases=[dom])
    ev0.record(stream)
    g.run(args.steps, DT, energies=False)
    ev1.record(stream)
    g.synchronize()
    torch.cuda.synchronize()
    dist.barrier()
    ck = clocks.stop()
    live = g.profile_get()[dom]
    g.profile(False)
    st = g.stats()
    launches = st["kernel_launches"] - launches0
    ms = ev0.elapsed_time(ev1)
    tmax = dist.max(ms / 1e3)
    value = n * args.steps * world / tmax

    # the mixed-precision form on the same workload (FP32 pair/bond arithmetic
    # and QEq SpMV, FP64 accumulation), timed the same way
    mixed = None
    if not args.no_mixed:
        from sw_reaxff_gb300.api import PREC_MIXED
        gm = ReaxGPU(DEFAULT_FFIELD, device=local, precision=PREC_MIXED,
                     pair_kernel=args.pair_kernel)
        gm.set_system(s)
        gm.run(max(args.warmup, 1), DT, energies=False)
        sm = torch.cuda.ExternalStream(gm.stream())
        m0 = torch.cuda.Event(enable_timing=True)
        m1 = torch.cuda.Event(enable_timing=True)
        dist.barrier()
        gm.synchronize()
        m0.record(sm)
        gm.run(args.steps, DT, energies=False)
        m1.record(sm)
        gm.synchronize()
        dist.barrier()
        tm = dist.max(m0.elapsed_time(m1) / 1e3)
        sm0 = gm.stats()
        gm.profile(True)
        gm.run(psteps, DT, energies=False)
        gm.synchronize()
        pm = gm.profile_get()
        gm.profile(False)
        smx = sm1 = gm.stats()
        live_m = pm["qeq_spmv"]
        # the mixed SpMV against HBM: 8 bytes (index + FP32 H) per entry
        # streamed per launch with work, and the half-symmetric algorithmic
        # 4 bytes per directed entry (+ 48 B of vector traffic per atom)
        # (events around every kernel group in the profiled steps)
        passes = sm1["cg_spmv_rows_passes"] - sm0["cg_spmv_rows_passes"]
        ent = sm1["n_pairs"]
        hbm_peak_m = measured_peaks().get("hbm_gbs")
        t_spmv = live_m[0] * 1e-3
        read_b = (8.0 * ent + 48.0 * n) * passes
        alg_b = (4.0 * ent + 48.0 * n) * passes
        mixed_roof = {"kernel": "k_spmv32", "bound": "hbm", "launches_timed": live_m[1],
                      "launches_with_work": passes,
                      "avg_launch_ms": live_m[0] / max(live_m[1], 1),
                      "streamed_gbs": read_b / t_spmv / 1e9 if t_spmv > 0 else None,
                      "algorithmic_gbs": alg_b / t_spmv / 1e9 if t_spmv > 0 else None,
                      "peak_gbs": hbm_peak_m,
                      "frac_streamed": read_b / t_spmv / 1e9 / hbm_peak_m
                      if t_spmv > 0 and hbm_peak_m else None,
                      "frac_algorithmic": alg_b / t_spmv / 1e9 / hbm_peak_m
                      if t_spmv > 0 and hbm_peak_m else None}
        mixed = {"value": n * args.steps * world / tm, "unit": UNIT,
                 "ms_per_step": tm * 1e3 / args.steps, "speedup_vs_fp64": tmax / tm,
                 "phases_ms_per_step": {k: round(v[0] / psteps, 4)
                                        for k, v in pm.items() if v[1] > 0},
                 "autotuned": {"cell_div": smx["cell_div"], "spmv_lanes_per_row": smx["spmv_rows"],
                               "pair_kernel": "cell tiles" if smx["pair_kernel"] == 2
                               else "warp per atom"},
                 "fp64_fallback_items": {"angles": smx["fp64_angles"],
                                         "torsions": smx["fp64_torsions"]},
                 "spmv_roofline": mixed_roof}

    # end to end through the C ABI with host (pinned) buffers: per step the
    # state x, v, f goes host->device, the step runs, x, v, q, f come back
    e2e = None
    if not args.no_e2e:
        pin = lambda shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
        hx, hv, hf, hq = pin((n, 3)), pin((n, 3)), pin((n, 3)), pin((n,))
        g.get_atoms_into(hx, hv, hq, hf)
        dist.barrier()
        g.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            g.set_state(hx, hv, hf)
            g.run(1, DT, energies=False)
            g.get_atoms_into(hx, hv, hq, hf)
        e1.record(stream)
        g.synchronize()
        dist.barrier()
        t_e2e = dist.max(e0.elapsed_time(e1) / 1e3)
        e2e = {"value": n * args.steps * world / t_e2e, "unit": UNIT,
               "h2d_bytes_per_step": int(hx.nbytes + hv.nbytes + hf.nbytes),
               "d2h_bytes_per_step": int(hx.nbytes + hv.nbytes + hq.nbytes + hf.nbytes)}

    # errors of the mixed form against the FP64 form on the same state (the
    # initial configuration, charges from zero initial guesses)
    if mixed is not None:
        g.set_system(s)
        gm.set_system(s)
        q64, _, _ = g.qeq()
        f64, e64 = g.compute()
        q32, its32, itt32 = gm.qeq()
        f32, e32 = gm.compute()
        mixed["errors_vs_fp64"] = {
            "force_rel_rms": float(np.sqrt(((f32 - f64) ** 2).sum() / (f64 ** 2).sum())),
            "charge_max_abs": float(np.abs(q32 - q64).max()),
            "energy_rel_max": max(float(abs(e32[k] - e64[k]) / abs(e64[k]))
                                  for k in e64 if e64[k] != 0.0),
            "qeq_restarts": gm.stats()["qeq_restarts"],
            "bars": {"force_rel_rms": 1e-4, "charge_max_abs": 1e-5}}
        gm.close()

    # roofline of the dominant kernel, its launch time measured with CUDA
    # events in the timed steps: against the FP64 rate (FMA probe run here)
    # and against HBM (MEASURED_PEAKS.json); the binding one is reported
    fp64_peak = measure_fp64_peak(local)
    peaks = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs")
    phases = {k: v for k, v in prof.items() if v[1] > 0}
    tot_ms = sum(v[0] for v in phases.values())
    kname, uname, flop_u, bytes_u, alg_u, alg_atom, stream_u = FP64_PER_UNIT[dom]
    units = st["n_pairs"] / 2 if dom == "nonbonded" else st["n_pairs"]
    avg_ms = live[0] / max(live[1], 1)
    if dom == "qeq_spmv":
        # a CG SpMV launch streams the rows when a system is still
        # iterating (its products and sums run on the FP32 units, as FP32
        # pairs), and a launch with none left returns at once: bytes are
        # summed over the timed region and divided by the summed time
        passes = st["cg_spmv_rows_passes"] - st0["cg_spmv_rows_passes"]
        per = passes / max(live[1], 1)
        fp64_ach = flop_u * units * per / (avg_ms * 1e-3) / 1e12
        alg_bytes = (alg_u * units + alg_atom * n) * per
        stream_bytes = (stream_u * units + 48.0 * n) * per
        flop_note = (f"FP64 instructions per entry from ncu ({flop_u}: the row tails); "
                     f"{passes} of {live[1]} launches had a system to update")
    else:
        fp64_ach = flop_u * units / (avg_ms * 1e-3) / 1e12
        alg_bytes = alg_u * units + alg_atom * n
        stream_bytes = stream_u * units + alg_atom * n
        flop_note = "ncu-counted FP64 FLOP per unit (52,428-atom capture) x units"
    hbm_ach = alg_bytes / (avg_ms * 1e-3) / 1e9
    stream_ach = stream_bytes / (avg_ms * 1e-3) / 1e9
    fp64_frac = fp64_ach / fp64_peak
    hbm_frac = hbm_ach / hbm_peak if hbm_peak else None
    bind_fp64 = hbm_frac is None or fp64_frac >= hbm_frac
    roof = {"kernel": kname, "phase": dom, "share": phases[dom][0] / tot_ms if tot_ms else None,
            "bound": "fp64" if bind_fp64 else "hbm",
            "achieved": fp64_ach if bind_fp64 else hbm_ach,
            "peak": fp64_peak if bind_fp64 else hbm_peak,
            "unit": "TFLOP/s" if bind_fp64 else "GB/s",
            "frac": fp64_frac if bind_fp64 else hbm_frac,
            "traffic": bytes_u * units,
            "fp64": {"achieved_tflops": fp64_ach, "peak_tflops": fp64_peak, "frac": fp64_frac,
                     "flop_count": flop_note,
                     "peak_source": "FP64 FMA probe measured in this run (MEASURED_PEAKS.json "
                                    "has no FP64 figure)"},
            "hbm": {"algorithmic_bytes": alg_bytes, "achieved_gbs": hbm_ach,
                    "peak_gbs": hbm_peak, "frac": hbm_frac,
                    "streamed_bytes": stream_bytes, "streamed_gbs": stream_ach,
                    "streamed_frac": stream_ach / hbm_peak if hbm_peak else None,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"},
            "units_per_launch": units, "unit_of_work": uname, "flop_per_unit": flop_u,
            "avg_launch_ms": avg_ms, "launches_timed": live[1],
            "traffic_source": "ncu DRAM bytes per unit of the 52,428-atom capture x units"}
    if main_mixed:
        roof = None   # the per-unit FP64 counts are the FP64 kernels

    line = {
        "metric": METRIC_MIXED if main_mixed else METRIC, "value": value, "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tmax * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32/f64 mixed" if main_mixed else "f64",
        "data": "synthetic (seeded molecular mixture)",
        "config": {"workload": workload_name(n, main_mixed),
                   "atoms": n, "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (pair list ~GBs)"},
        "e2e": e2e,
        "mixed": mixed,
        "gpu_launches": None,
        "clocks": ck,
        "roofline": roof,
        "phases_ms_per_step": {k: round(v[0] / psteps, 4) for k, v in phases.items()},
        "counts": {"pairs": st["n_pairs"], "bonds": st["n_bonds"], "hbond_pairs": st["n_hbond_pairs"],
                   "cg_iters_s": st["cg_iters_s"], "cg_iters_t": st["cg_iters_t"]},
        "autotuned": {"cell_div": st["cell_div"], "spmv_lanes_per_row": st["spmv_rows"],
                      "pair_kernel": "cell tiles" if st["pair_kernel"] == 2 else "warp per atom"},
        "hbm_peak_gbs": peaks.get("hbm_gbs"),
    }
    line["gpu_launches"] = int(launches)
    if rank == 0 and not args.no_water:
        line["water6k"] = water_section(args, local)
    if rank == 0 and not args.no_batched:
        line["batched"] = batched_section(args, local)
    if rank == 0 and not args.no_serve:
        line["serving"] = serve_section(args, local)
    if rank == 0 and not args.no_cpu:
        v, cores, sample = cpu_baseline(args.cpu_scale, 1, 1, 2)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"2 warm NVE steps (after setup and 1 untimed step) "
                                          f"of a {sample}-atom box of the same mixture, "
                                          "single thread"}
    if mixed is not None:
        # the mixed form's headline figures, last, where a reader of the
        # line's tail sees them
        err = mixed.get("errors_vs_fp64", {})
        line["mixed_summary"] = {"metric": METRIC_MIXED, "value": mixed["value"], "unit": UNIT,
                                 "ms_per_step": mixed["ms_per_step"],
                                 "speedup_vs_fp64": mixed["speedup_vs_fp64"],
                                 "force_rel_rms_vs_fp64": err.get("force_rel_rms"),
                                 "charge_max_abs_vs_fp64": err.get("charge_max_abs")}
    if rank == 0:
        print(json.dumps(line), flush=True)
    g.close()
    dist.close()


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
