#!/usr/bin/env python3
"""Throughput of the GPU Metropolis hot path on the canonical FCC workload
(128 replicas of a 24x24x24 FCC A/B supercell, T in [200, 1200] K x
x_B in {0.25, 0.5}), printed as one JSON line.

A step is one Metropolis pass over every replica of the batch (each pass
proposes about one pair swap per site). The timed region runs K passes in
one persistent launch with occupations resident in shared memory; `value`
is real swap proposals (pairs of different species) per second from CUDA
events on the launching stream. `e2e` runs steps through the C ABI with
host buffers: copy occupations in, one pass, copy occupations out; two
replica batches on two streams alternate so that one batch's copies overlap
the other's pass.

The line also carries `learned_vs_plain`, the headline half of the metric:
effective independent samples per second of the learned group sweep against
the plain sweep on configuration 3 (32 x 48^3 FCC, L1_2 cluster expansion,
x_B = 0.25, T = 0.9 T_c), both continued from one equilibrated state, with
their <E> compared within 2 standard errors (`--no-learned` leaves it out).

--impl reference runs the CPU restatement of the reference loop (one
sequential std::mt19937_64 chain per host thread) on a bounded sample of the
same workload.
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
sys.path.insert(0, ROOT)

WORKLOAD_INDEX = 1
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        return ws, rank, local, dist
    return 1, 0, 0, None


def reduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64,
                     device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64,
                     device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.gpu = gpu_index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p is not None:
            time.sleep(0.3)
            self.p.terminate()
            try:
                self.p.wait(5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self) -> dict:
        self.f.flush()
        rows = []
        try:
            for line in open(self.f.name):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                    rows.append(parts)
        except OSError:
            pass
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(float(r[2]) for r in rows),
                "reasons": sorted(reasons), "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())
                if any(r[3].replace(".", "").isdigit() for r in rows) else None}


def load_workload():
    from casmcode_clexmonte_gb300 import workloads

    return workloads.config(WORKLOAD_INDEX)


def workload_config(w, extra=None) -> dict:
    c = {
        "workload": w.name,
        "replicas": w.n_replicas,
        "sites_per_replica": int(w.n_sites[0]),
        "lattice": "FCC a=4.0 A, 24x24x24 primitive cells",
        "cluster_expansion": "7 functions: empty, point, pairs to NN3, triplets to NN2",
        "ensemble": "canonical (pair swaps)",
        "temperatures_K": [float(w.temperature.min()), float(w.temperature.max())],
        "x_B": sorted(set(float(x) for x in w.x_b)),
        "mode": "parallel (colour classes of non-interacting sites)",
        "step": "one Metropolis pass over every replica",
        "l2": "flushed (256 MiB write) before the timed launch; occupations stay in "
              "shared memory for the whole launch",
    }
    if extra:
        c.update(extra)
    return c


def cpu_baseline(w, n_threads: int, target_s: float = 12.0) -> dict:
    """Oracle (CPU restatement of the reference loop) on a bounded sample."""
    from oracle import oracle

    oracle.build_oracle()
    o = oracle.OracleSystem(w.ce, w.L[0])
    n = min(n_threads, w.n_replicas)
    occ = np.concatenate([w.occupation[i] for i in range(n)]).astype(np.int8)
    temps = w.temperature[:n].copy()
    mus = np.zeros((n, 1))
    secs, steps = o.run_threads(occ.copy(), 1, temps, mus, 7, 1, n)  # probe
    rate = steps / max(secs, 1e-9)
    passes = max(1, int(target_s * rate / (n * int(w.n_sites[0]))))
    secs, steps = o.run_threads(occ.copy(), 1, temps, mus, 11, passes, n)
    # one chain on one core (a bounded sample of about 3 s)
    n1 = int(w.n_sites[0])
    p1 = max(1, int(3.0 * rate / n / n1))
    s1, st1 = o.run_threads(occ[:n1].copy(), 1, temps[:1].copy(), mus[:1].copy(), 13, p1, 1)
    return {
        "value": steps / secs, "unit": "proposals/s", "cores": n, "kind": "port",
        "sample": f"{n} replicas x {passes} passes of the 24^3 canonical workload, one "
                  f"sequential std::mt19937_64 chain per host thread ({secs:.1f} s)",
        "seconds": secs,
        "single_core": {"value": st1 / s1, "unit": "proposals/s",
                        "sample": f"1 replica x {p1} passes on one thread ({s1:.1f} s)"},
    }


def run_reference(args):
    ws, rank, local, dist = dist_init()
    if rank != 0:
        barrier(dist)
        return 0
    w = load_workload()
    from oracle import oracle

    oracle.build_oracle()
    o = oracle.OracleSystem(w.ce, w.L[0])
    cores = os.cpu_count() or 1
    n = min(cores, w.n_replicas)
    occ = np.concatenate([w.occupation[i] for i in range(n)]).astype(np.int8)
    temps = w.temperature[:n].copy()
    mus = np.zeros((n, 1))
    # warm-up steps, then K timed steps; a step = one pass over the sample
    o.run_threads(occ, 1, temps, mus, 3, args.warmup, n)
    secs, steps = o.run_threads(occ, 1, temps, mus, 5, args.steps, n)
    value = steps / secs
    line = {
        "impl": "reference", "metric": "proposals/s", "value": value, "unit": "proposals/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(w, {"sample_replicas": n, "step": "one pass over the sample"}),
        "cpu_baseline": {"value": value, "unit": "proposals/s", "cores": n, "kind": "port",
                         "sample": f"{n} of {w.n_replicas} replicas (one per host thread), "
                                   f"{args.steps} passes; CPU FP64 restatement of "
                                   "occupation_metropolis_v2 (the reference needs "
                                   "libcasm-clexulator/libcasm-monte, absent offline)"},
        "e2e": {"value": value, "unit": "proposals/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    barrier(dist)
    return 0


def run_gb300(args):
    ws, rank, local, dist = dist_init()
    import ctypes as C

    import torch

    from casmcode_clexmonte_gb300 import build as B

    B.build()
    from casmcode_clexmonte_gb300 import _lib
    from casmcode_clexmonte_gb300 import calculator as cm
    from casmcode_clexmonte_gb300.stats import tau_int

    if not torch.cuda.is_available():
        raise RuntimeError("no CUDA device: the GPU path has no CPU fallback")
    torch.cuda.set_device(local)
    w = load_workload()
    sysd = cm.System(w.ce)
    batch = cm.ReplicaBatch(sysd, "canonical", w.L)
    for i in range(w.n_replicas):
        batch.set_conditions(i, float(w.temperature[i]))
        batch.set_seed(i, int(w.seeds[i]) + 7919 * rank)
    packed = np.concatenate(w.occupation).astype(np.int8)
    batch.set_occupation_all(packed)
    lib = _lib.load()
    smem = C.c_double()
    _lib.check(lib.cem_smem_bandwidth(C.byref(smem)))
    smem_gbs = smem.value

    # launch schedule picked by the autotuner (state restored afterwards)
    tuned = batch.autotune(10)
    # warm-up
    batch.run(args.warmup, 0)
    batch.synchronize()
    before = [batch.stats(i) for i in range(w.n_replicas)]
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    flush.fill_(1)
    torch.cuda.synchronize()
    barrier(dist)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        batch.run(args.steps, 0, record_samples=True)
        batch.synchronize()
        t1 = time.perf_counter()
    torch.cuda.synchronize()
    kernel_ms = batch.kernel_ms()
    after = [batch.stats(i) for i in range(w.n_replicas)]
    props = sum(a["n_proposed"] - b["n_proposed"] for a, b in zip(after, before))
    accs = sum(a["n_accepted"] - b["n_accepted"] for a, b in zip(after, before))
    t_dev = reduce_max(dist, kernel_ms / 1e3)
    props_all = reduce_sum(dist, props)
    value = props_all / t_dev
    # effective independent samples of the potential energy: the first tenth
    # of the timed passes is left out as equilibration, and the estimate is
    # reported only where every replica's series holds >= 50 tau_int
    n_eff = n_eff_op = 0.0
    taus = []
    min_ratio = float("inf")
    for i in range(w.n_replicas):
        pot, _ = batch.samples(i, args.steps)
        op = batch.order_samples(i, args.steps)
        pot, op = pot[pot.size // 10:], op[op.size // 10:]
        t = tau_int(pot) if pot.size >= 8 else float("inf")
        t_op = tau_int(op) if op.size >= 8 else float("inf")
        taus.append(t)
        min_ratio = min(min_ratio, pot.size / t, op.size / t_op)
        n_eff += pot.size / (2.0 * t)
        n_eff_op += op.size / (2.0 * t_op)
    n_eff = reduce_sum(dist, n_eff)
    n_eff_op = reduce_sum(dist, n_eff_op)
    eff_ok = min_ratio >= 50.0

    # end-to-end through the C ABI with pinned host buffers: two replica
    # batches (each with its own stream) alternate, so one batch's host <->
    # device copies and launch overhead overlap the other batch's sweep; every
    # step uploads its occupations and reads its result back
    nbytes = int(packed.size)
    batches = [batch, cm.ReplicaBatch(sysd, "canonical", w.L)]
    batches[1].set_option("threads", tuned["threads"])
    batches[1].set_option("cta_order", tuned["cta_order"])
    for i in range(w.n_replicas):
        batches[1].set_conditions(i, float(w.temperature[i]))
        batches[1].set_seed(i, int(w.seeds[i]) + 7919 * rank + 104729)
    hosts = []
    for b in batches:
        hosts.append(b.pinned_buffer())
        batch.get_occupation_all(hosts[-1])
    for b, h in zip(batches, hosts):  # capture each batch's step graph
        b.step_async(h, h, 1)
        b.synchronize()
    e2e_steps = max(4, min(args.steps, 400))

    def n_proposed():
        return sum(b.stats(i)["n_proposed"] for b in batches for i in range(w.n_replicas))

    e_before = n_proposed()
    barrier(dist)
    t2 = time.perf_counter()
    for s in range(e2e_steps):
        b, h = batches[s % 2], hosts[s % 2]
        if s >= 2:
            b.synchronize()  # step s - 2 has written its result to h
        b.step_async(h, h, 1)  # graph: h -> device, one pass, device -> h
    for b in batches:
        b.synchronize()
    t3 = time.perf_counter()
    e2e_props = reduce_sum(dist, n_proposed() - e_before)
    e2e_time = reduce_max(dist, t3 - t2)

    # drift of the running energy (integer delta-count bookkeeping) against a
    # fresh full recompute of the final states
    drift = 0.0
    for i in range(0, w.n_replicas, max(1, w.n_replicas // 8)):
        e_run = batch.stats(i)["energy"]
        e_fresh, _ = batch.energy(i)
        drift = max(drift, abs(e_run - e_fresh) / max(abs(e_fresh), 1e-300))
    p_acc = accs / max(props, 1)
    z = 42  # distinct flower sites of an FCC site (12 + 6 + 24)
    bytes_per_prop = 2 * (1 + z) + 2 * p_acc
    achieved = props * bytes_per_prop / (kernel_ms / 1e3) / 1e9
    clocks = clk.summary()
    # DRAM bytes of one k_sweep launch from the committed ncu capture (the
    # replica stays in shared memory: only the staging read reaches DRAM)
    traffic = None
    prof = os.path.join(ROOT, "profiles", "k_sweep_fcc24_canonical_ncu.md")
    if os.path.exists(prof):
        import re

        m = re.search(r"^dram_bytes_per_launch: (\d+)$", open(prof).read(), re.M)
        traffic = int(m.group(1)) if m else None
    line = {
        "metric": "proposals/s", "value": value, "unit": "proposals/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": workload_config(w, {
            "arithmetic": "int8 occupations; integer cluster-count changes; energy change = "
                          "exact int32 sum of integer multiples of a power-of-two quantum plus "
                          "one f32 FMA chain of the weight remainders; f32 acceptance; f64 "
                          "running energy from integer counts",
            "parallelism": f"replicas only, {w.n_replicas} per GPU",
            "schedule": {"threads_per_replica": tuned["threads"],
                         "cta_order": "largest first" if tuned["cta_order"] else "replica order",
                         "picked_by": "autotuner (10 timed trial passes per candidate)"},
        }),
        "proposals": int(props_all), "acceptance": p_acc,
        "proposals_per_s_per_replica": value / (w.n_replicas * ws),
        "effective_samples_per_s": n_eff / t_dev if eff_ok else None,
        "effective_samples_per_s_order_parameter": n_eff_op / t_dev if eff_ok else None,
        "effective_samples_note": ("timed passes after the first tenth; every replica's series "
                                   f"holds >= {min_ratio:.0f} tau_int") if eff_ok else
                                  (f"not reported: the timed run holds only {min_ratio:.1f} "
                                   "tau_int per replica (< 50)"),
        "running_energy_rel_drift_vs_recompute": drift,
        "tau_int_potential_median": float(np.median(taus)) if eff_ok else None,
        "host_wall_s": t1 - t0,
        "e2e": {"value": e2e_props / e2e_time, "unit": "proposals/s",
                "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": e2e_steps,
                "pipeline": "two replica batches on two streams alternate; each step = one "
                            "CUDA graph: upload occupations, one pass, read occupations back"},
        "roofline": {"bound": "smem", "achieved": achieved, "peak": smem_gbs, "unit": "GB/s",
                     "frac": achieved / smem_gbs, "traffic": traffic,
                     "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one "
                                       "k_sweep launch of this workload, ncu capture "
                                       "summarised in profiles/k_sweep_fcc24_canonical_ncu.md",
                     "peak_source": "measured in this run by cem_smem_bandwidth "
                                    "(16-byte shared loads, all SMs)",
                     "bytes_per_proposal": bytes_per_prop,
                     "kernel": "k_sweep<2>", "kernel_ms": kernel_ms},
        "gpu_launches": 1,
        "clocks": clocks,
    }
    if rank == 0 and not args.no_learned:
        # the headline half of the metric: learned vs plain GPU Metropolis in
        # effective independent samples per second (configuration 3)
        line["learned_vs_plain"] = learned_vs_plain(cm, 0.9 * T_C_CONFIG3_K)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, os.cpu_count() or 1)
    if rank == 0:
        print(json.dumps(line), flush=True)
    barrier(dist)
    return 0


def _plain_batch(cm, w, rank=0):
    sysd = cm.System(w.ce)
    batch = cm.ReplicaBatch(sysd, w.ensemble, w.L)
    for i in range(w.n_replicas):
        mu = w.param_chem_pot[i] if w.ensemble == "semigrand_canonical" else None
        batch.set_conditions(i, float(w.temperature[i]), mu)
        batch.set_seed(i, int(w.seeds[i]) + 7919 * rank)
    batch.set_occupation_all(np.concatenate(w.occupation).astype(np.int8))
    return sysd, batch


def run_other_workload(args):
    """Throughput line of configurations 0, 2 and 4 (plain parallel sampler)."""
    import torch

    from casmcode_clexmonte_gb300 import build as B

    B.build()
    from casmcode_clexmonte_gb300 import calculator as cm
    from casmcode_clexmonte_gb300 import workloads

    w = workloads.config(args.workload)
    notes = {}
    groups = [w]
    if args.workload == 4:
        # two batches on their own streams, run concurrently: 512 x 32^3 in
        # shared memory and 4 x 96^3 HBM-streamed (one kernel per sub-step)
        def subset(keep):
            import copy

            v = copy.copy(w)
            v.L = [w.L[i] for i in keep]
            v.temperature = w.temperature[keep]
            v.param_chem_pot = w.param_chem_pot[keep]
            v.x_b = w.x_b[keep]
            v.occupation = [w.occupation[i] for i in keep]
            v.seeds = w.seeds[keep]
            return v

        groups = [subset([i for i, l in enumerate(w.L) if l[0] == 32]),
                  subset([i for i, l in enumerate(w.L) if l[0] == 96])]
    batches = [_plain_batch(cm, g)[1] for g in groups]
    tuned = [b.autotune(5) for b in batches]
    notes["schedules"] = [{"threads": t["threads"], "cta_order": t["cta_order"]} for t in tuned]
    for b in batches:
        b.run(args.warmup, 0)
    for b in batches:
        b.synchronize()
    before = [sum(b.stats(i)["n_proposed"] for i in range(b.n)) for b in batches]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for b in batches:
        b.run(args.steps, 0)
    for b in batches:
        b.synchronize()
    wall = time.perf_counter() - t0
    ms = [b.kernel_ms() for b in batches]
    after = [sum(b.stats(i)["n_proposed"] for i in range(b.n)) for b in batches]
    props = [a - bb for a, bb in zip(after, before)]
    parts = []
    for g, b, p_, m in zip(groups, batches, props, ms):
        parts.append({"replicas": b.n, "sites": int(g.n_sites[0]), "streamed": b.get_option("streamed"),
                      "pitch": b.get_option("pitch"), "device_ms": m,
                      "proposals_per_s": p_ / (m / 1e3)})
    value = sum(props) / (max(ms) / 1e3) if len(batches) > 1 else props[0] / (ms[0] / 1e3)
    line = {
        "metric": "proposals/s", "value": value, "unit": "proposals/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": max(ms) / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": w.name, "replicas": w.n_replicas,
                   "sites": [int(x) for x in sorted(set(w.n_sites))][:4],
                   "ensemble": w.ensemble, "batches": parts, "wall_s_all_batches": wall,
                   "colour_classes": batches[0].get_option("colour_classes"), **notes},
        "gpu_launches": "1 per shared-memory batch; 25 per pass for a streamed batch (CUDA graph)",
    }
    print(json.dumps(line), flush=True)
    return 0


T_C_CONFIG3_K = 100.0  # heat-capacity maximum of a plain-sweep temperature scan (--tc-scan)


def _l12_state(L: int, k: int) -> np.ndarray:
    """Perfect L1_2 order on an L^3 FCC supercell: B on simple-cubic
    sublattice k (site index x + L (y + L z), primitive-cell coordinates)."""
    x, y, z = np.meshgrid(np.arange(L), np.arange(L), np.arange(L), indexing="ij")
    x, y, z = (a.transpose(2, 1, 0).ravel() for a in (x, y, z))
    return ((((y + z) & 1) | (((x + z) & 1) << 1)) == k).astype(np.int8)


def tc_scan(cm, ce):
    """T_c of an L1_2 cluster expansion: heat-capacity maximum of the plain
    sweep over 20..320 K (24^3, x_B = 0.25, 3000 + 3000 passes)."""
    from casmcode_clexmonte_gb300 import workloads

    sysd = cm.System(ce)
    temps = np.linspace(20.0, 320.0, 31)
    scan = cm.ReplicaBatch(sysd, "canonical", [(24, 24, 24)] * len(temps))
    rng = np.random.default_rng(3)
    for i, t in enumerate(temps):
        scan.set_conditions(i, float(t))
        scan.set_seed(i, 300 + i)
        scan.set_occupation(i, workloads.fixed_composition(rng, 24 ** 3, 0.25))
    scan.run(6000, 3000)
    cv = np.array([scan.stats(i)["var_potential"] * 24 ** 3 / (8.617333262e-5 * t * t)
                   for i, t in enumerate(temps)])
    inner = slice(1, len(temps) - 1)  # a maximum at the scan's edge is no transition
    return float(temps[inner][int(np.argmax(cv[inner]))]), temps, cv


def learned_vs_plain(cm, T: float, plain_passes: int = 60000, learned_passes: int = 6000,
                     equil_passes: int = 5000, rounds: int = 2, local_substeps: int = 4,
                     weights=("network",)) -> dict:
    """Configuration 3 (32 x 48^3 FCC, L1_2 cluster expansion, canonical
    x_B = 0.25) at temperature T: plain GPU Metropolis (the colour-class
    sweep, each replica on a cluster of 4 CTAs) against the learned group
    sweep (also 4 CTAs per replica), both continued from one common state
    equilibrated by the plain sweep from perfect L1_2 order.

    Per sampler: integrated autocorrelation times of E and of the L1_2 order
    parameter per replica (Sokal window; the run must hold >= 50 tau_int),
    effective independent samples per second = sum over replicas of
    n / (2 tau_int) / device seconds, and <E> with the standard error of the
    replica means (32 independent chains). The network is trained on the GPU
    on 10^6 environments of the equilibrated plain states."""
    from casmcode_clexmonte_gb300 import workloads
    from casmcode_clexmonte_gb300.stats import tau_int

    w = workloads.config(3)
    sysd = cm.System(w.ce)
    L = w.L[0][0]
    n_rep = w.n_replicas

    def batch():
        b = cm.ReplicaBatch(sysd, "canonical", w.L)
        for i in range(n_rep):
            b.set_conditions(i, T)
            b.set_seed(i, 1000 + i)
        return b

    def summary(e_series, op_series, seconds, props, accs, passes):
        te = np.array([tau_int(e) for e in e_series])
        to = np.array([tau_int(o) for o in op_series])
        means = np.array([e.mean() for e in e_series])
        n = len(e_series[0])
        return {
            "passes": passes, "device_s": seconds, "ms_per_pass": 1e3 * seconds / passes,
            "proposals_per_s": props / seconds, "acceptance": accs / max(1, props),
            "tau_int_E_median": float(np.median(te)), "tau_int_E_max": float(te.max()),
            "tau_int_order_median": float(np.median(to)),
            "samples_over_tau_min": float(n / max(te.max(), to.max())),
            "eff_samples_per_s_E": float(np.sum(n / (2.0 * te)) / seconds),
            "eff_samples_per_s_order": float(np.sum(n / (2.0 * to)) / seconds),
            "mean_E": float(means.mean()), "mean_E_sigma": float(means.std(ddof=1) / np.sqrt(n_rep)),
        }

    plain = batch()
    for i in range(n_rep):
        plain.set_occupation(i, _l12_state(L, i % 4))
    plain.run(equil_passes, 0)
    plain.synchronize()
    common = plain.get_occupation_all()
    st0 = [plain.stats(i) for i in range(n_rep)]
    plain.run(plain_passes, 0, record_samples=True)
    plain.synchronize()
    t_plain = plain.kernel_ms() / 1e3
    st1 = [plain.stats(i) for i in range(n_rep)]
    e_p = [plain.samples(i, plain_passes)[0] for i in range(n_rep)]
    o_p = [plain.order_samples(i, plain_passes) for i in range(n_rep)]
    out = {"workload": w.name, "temperature_K": T, "T_c_K": T_C_CONFIG3_K,
           "start": f"one state: perfect L1_2 order + {equil_passes} plain passes",
           "plain": summary(e_p, o_p, t_plain,
                            sum(b["n_proposed"] - a["n_proposed"] for a, b in zip(st0, st1)),
                            sum(b["n_accepted"] - a["n_accepted"] for a, b in zip(st0, st1)),
                            plain_passes)}
    # both samplers spread a replica over a cluster of CTAs when that pays
    out["plain"]["cluster_ctas_per_replica"] = plain.get_option("sweep_cluster")
    # network trained on the equilibrated plain states (10^6 environments)
    eq = batch()
    eq.set_occupation_all(common)
    X, t = [], []
    for i in range(n_rep):
        x_i, t_i = eq.learned_features(i)
        X.append(x_i)
        t.append(t_i)
    X = np.concatenate(X)[:1_000_000]
    t = np.concatenate(t)[:1_000_000]
    net = cm.LearnedProposal(seed=11)
    t0 = time.perf_counter()
    losses = net.train(X, t, epochs=4, batch=4096, lr=2e-3, seed=5)
    out["network"] = {"train_s": time.perf_counter() - t0, "environments": int(len(X)),
                      "loss_per_epoch": [float(v) for v in losses]}
    for wname in weights:
        b = batch()
        b.set_occupation_all(common)
        prop = net if wname == "network" else None
        b.learned_group_run(prop, learned_passes, 0, record_samples=True, weights=wname,
                            rounds=rounds, local_substeps=local_substeps)
        b.synchronize()
        t_l = b.kernel_ms() / 1e3
        st1 = [b.stats(i) for i in range(n_rep)]
        e_l = [b.learned_samples(i, learned_passes)[0] for i in range(n_rep)]
        o_l = [b.learned_samples(i, learned_passes)[1] for i in range(n_rep)]
        r = summary(e_l, o_l, t_l, sum(y["n_proposed"] for y in st1),
                    sum(y["n_accepted"] for y in st1), learned_passes)
        r.update(weights=wname, rounds=rounds, local_substeps=local_substeps,
                 cluster_ctas_per_replica=b.get_option("group_cluster"))
        key = "learned" if wname == "network" else f"informed_{wname}"
        out[key] = r
        sig = float(np.hypot(out["plain"]["mean_E_sigma"], r["mean_E_sigma"]))
        z = abs(r["mean_E"] - out["plain"]["mean_E"]) / sig if sig > 0 else float("inf")
        sfx = "" if wname == "network" else f"_{wname}"
        out[f"ratio_learned_over_plain_E{sfx}"] = r["eff_samples_per_s_E"] / out["plain"]["eff_samples_per_s_E"]
        out[f"ratio_learned_over_plain_order{sfx}"] = (r["eff_samples_per_s_order"] /
                                                       out["plain"]["eff_samples_per_s_order"])
        out[f"E_difference_over_sigma{sfx}"] = z
        out[f"same_E_within_2sigma{sfx}"] = bool(z <= 2.0)
    # the headline comparison needs >= 50 tau_int in both the plain and the
    # network-weighted runs (the other weightings are diagnostics)
    out["runs_hold_50_tau"] = bool(out["plain"]["samples_over_tau_min"] >= 50 and
                                   out.get("learned", out["plain"])["samples_over_tau_min"] >= 50)
    return out


def run_learned_comparison(args):
    """Configuration 3: plain vs learned-proposal effective independent
    samples per second of the energy and the L1_2 order parameter at
    T = 0.9 T_c (48^3, x_B = 0.25), from one common equilibrated state."""
    from casmcode_clexmonte_gb300 import build as B

    B.build()
    from casmcode_clexmonte_gb300 import calculator as cm
    from casmcode_clexmonte_gb300 import workloads

    tc = T_C_CONFIG3_K
    scan = None
    if args.tc_scan:
        tc, temps, cv = tc_scan(cm, workloads.config(3).ce)
        scan = {"T_K": [float(x) for x in temps], "C_per_uc": [float(x) for x in cv]}
    res = learned_vs_plain(cm, 0.9 * tc, plain_passes=args.plain_passes,
                           learned_passes=args.learned_passes, equil_passes=args.equil_passes,
                           rounds=args.rounds, weights=("network", "exact", "uniform"))
    res["T_c_K"] = tc
    if scan:
        res["heat_capacity_scan"] = scan
    line = {"metric": "effective samples/s (learned vs plain GPU Metropolis, same <E>)", **res}
    print(json.dumps(line), flush=True)
    return 0


def run_nfold_comparison(args):
    """n-fold way against the plain Metropolis sweep on one semi-grand
    canonical batch (128 replicas of 24^3 FCC A/B, configuration 0's CE) at a
    low temperature, where most Metropolis proposals are rejected: events/s of
    the n-fold kernel, its Metropolis-equivalent trials/s (sum of residence
    weights / time) and the sweep's proposals/s on the same states."""
    import torch

    from casmcode_clexmonte_gb300 import build as B

    B.build()
    from casmcode_clexmonte_gb300 import calculator as cm
    from casmcode_clexmonte_gb300 import workloads

    w = workloads.config(0)
    sysd = cm.System(w.ce)
    n, L, T = 128, (24, 24, 24), args.nfold_temperature
    rng = np.random.default_rng(5)
    b = cm.ReplicaBatch(sysd, "semigrand_canonical", [L] * n)
    for i in range(n):
        b.set_conditions(i, T, np.array([0.0]))
        b.set_seed(i, 4242 + i)
        b.set_occupation(i, rng.integers(0, 2, 24 ** 3).astype(np.int8))
    b.run(200, 0)  # equilibrate with the sweep
    b.synchronize()
    st0 = [b.stats(i) for i in range(n)]
    b.run(args.steps, 0)
    b.synchronize()
    sweep_ms = b.kernel_ms()
    st = [b.stats(i) for i in range(n)]
    props = sum(s["n_proposed"] - s0["n_proposed"] for s, s0 in zip(st, st0))
    accs = sum(s["n_accepted"] - s0["n_accepted"] for s, s0 in zip(st, st0))
    acc = accs / max(1, props)
    sweep_rate = props / (sweep_ms / 1e3)
    b.nfold_run(200, 0)  # warm-up
    torch.cuda.synchronize()
    n_ev = args.nfold_events
    b.nfold_run(n_ev, 0)
    nf_ms = b.kernel_ms()
    weight = sum(b.stats(i)["n_samples"] for i in range(n))
    line = {
        "metric": "events/s", "value": n * n_ev / (nf_ms / 1e3), "unit": "events/s",
        "n_gpus": 1, "steps": n_ev, "warmup": 200, "higher_is_better": True,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": "fcc_binary_24I_sgc_x128_nfold", "replicas": n,
                   "temperature_K": T, "param_chem_pot": 0.0},
        "metropolis_equivalent_trials_per_s": weight / (nf_ms / 1e3),
        "sweep_proposals_per_s": sweep_rate, "sweep_acceptance": acc,
        "sweep_accepted_per_s": sweep_rate * acc,
        "gpu_launches": 1,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_zro(args):
    """A real CASM basis set on the GPU: the reference's Clex_ZrO_Occ system
    (hcp Zr, O/Va on the octahedral sites; 73 orbits, 1591 clusters per O
    site), semi-grand canonical, 152 replicas of 12 x 12 x 8 prim cells
    (2304 O/Va sites each) over a temperature x chemical-potential grid.
    Proposals/s of the orbit-at-a-time sweep kernel, and the oracle (CPU
    restatement of the reference loop) on the same system beside it."""
    import torch

    from casmcode_clexmonte_gb300 import build as B

    B.build()
    from casmcode_clexmonte_gb300 import calculator as cm
    from tests.zro_fixture import zro_ce

    ce = zro_ce()
    n, L = 152, (12, 12, 8)
    temps = np.linspace(1000.0, 2500.0, n)
    mus = np.linspace(-1.0, 0.0, n)[np.random.default_rng(3).permutation(n)]
    rng = np.random.default_rng(17)
    n_sites = 2 * int(np.prod(L))
    occ = [(rng.random(n_sites) < 0.5).astype(np.int8) for _ in range(n)]
    sysd = cm.System(ce)

    def measure(walk, passes):
        b = cm.ReplicaBatch(sysd, "semigrand_canonical", [L] * n)
        if walk:
            b.set_option("orbit_walk", walk)
        for i in range(n):
            b.set_conditions(i, float(temps[i]), np.array([mus[i]]))
            b.set_seed(i, 5150 + i)
        b.set_occupation_all(np.concatenate(occ))
        b.run(args.warmup, 0)
        b.synchronize()
        st0 = [b.stats(i) for i in range(n)]
        torch.cuda.synchronize()
        b.run(passes, 0)
        b.synchronize()
        ms = b.kernel_ms()
        st = [b.stats(i) for i in range(n)]
        props = sum(s["n_proposed"] - s0["n_proposed"] for s, s0 in zip(st, st0))
        accs = sum(s["n_accepted"] - s0["n_accepted"] for s, s0 in zip(st, st0))
        drift = max(abs(b.stats(i)["energy"] - b.energy(i)[0]) / max(1.0, abs(b.energy(i)[0]))
                    for i in range(0, n, 19))
        return b, props, accs, ms, drift

    b, props, accs, ms, drift = measure(0, args.zro_passes)
    value = props / (ms / 1e3)
    _, props1, _, ms1, _ = measure(1, max(2, args.zro_passes // 8))
    line = {
        "metric": "proposals/s", "value": value, "unit": "proposals/s", "n_gpus": 1,
        "steps": args.zro_passes, "warmup": args.warmup, "ms_per_step": ms / args.zro_passes,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "reference basis set and ECI (Clex_ZrO_Occ); seeded random initial states",
        "config": {"workload": "zro_hcp_12x12x8_sgc_x152", "replicas": n, "sites_per_replica": n_sites,
                   "orbits": len(ce.orbits), "clusters_per_site": len(ce.flowers[0]),
                   "pitch": b.get_option("pitch"), "colour_classes": b.get_option("colour_classes"),
                   "smem_bytes": b.get_option("smem_bytes"),
                   "temperatures_K": [1000.0, 2500.0], "param_chem_pot": [-1.0, 0.0]},
        "acceptance": accs / max(1, props),
        "running_energy_rel_drift_vs_recompute": drift,
        "thread_per_site_orbit_walk_proposals_per_s": props1 / (ms1 / 1e3),
        "gpu_launches": 1,
    }
    if not args.no_cpu_baseline:
        from oracle import oracle

        oracle.build_oracle()
        o = oracle.OracleSystem(ce, L)
        nt = min(os.cpu_count() or 1, n)
        occ_s = np.concatenate(occ[:nt]).astype(np.int8)
        secs, steps = o.run_threads(occ_s.copy(), 0, temps[:nt].copy(), mus[:nt, None].copy(), 7, 1, nt)
        passes = max(1, int(12.0 * (steps / max(secs, 1e-9)) / (nt * n_sites)))
        secs, steps = o.run_threads(occ_s.copy(), 0, temps[:nt].copy(), mus[:nt, None].copy(), 9,
                                    passes, nt)
        line["cpu_baseline"] = {
            "value": steps / secs, "unit": "proposals/s", "cores": nt, "kind": "port",
            "sample": f"{nt} replicas x {passes} passes of the same system, one sequential "
                      f"std::mt19937_64 chain per host thread ({secs:.1f} s)"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", type=int, default=WORKLOAD_INDEX, choices=[0, 1, 2, 3, 4])
    ap.add_argument("--learned-passes", type=int, default=6000)
    ap.add_argument("--plain-passes", type=int, default=60000)
    ap.add_argument("--equil-passes", type=int, default=5000,
                    help="workload 3: plain passes that equilibrate the common state")
    ap.add_argument("--rounds", type=int, default=2,
                    help="workload 3: swap rounds per group of the learned group sweep")
    ap.add_argument("--tc-scan", action="store_true",
                    help="workload 3: locate T_c by a heat-capacity scan first")
    ap.add_argument("--no-learned", action="store_true",
                    help="leave the learned-vs-plain comparison out of the default line")
    ap.add_argument("--nfold", action="store_true",
                    help="n-fold way vs Metropolis sweep (semi-grand canonical, low T)")
    ap.add_argument("--nfold-temperature", type=float, default=150.0)
    ap.add_argument("--nfold-events", type=int, default=20000)
    ap.add_argument("--zro", action="store_true",
                    help="the reference's Clex_ZrO_Occ basis set (73 orbits), semi-grand canonical")
    ap.add_argument("--zro-passes", type=int, default=40)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.nfold:
        return run_nfold_comparison(args)
    if args.zro:
        return run_zro(args)
    if args.workload == 3:
        return run_learned_comparison(args)
    if args.workload != WORKLOAD_INDEX:
        return run_other_workload(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
