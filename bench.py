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
    # effective independent samples of the potential energy per pass
    n_eff = n_eff_op = 0.0
    taus = []
    for i in range(w.n_replicas):
        pot, _ = batch.samples(i, args.steps)
        op = batch.order_samples(i, args.steps)
        t = tau_int(pot) if pot.size > 16 else float("nan")
        t_op = tau_int(op) if op.size > 16 else float("nan")
        taus.append(t)
        if np.isfinite(t):
            n_eff += pot.size / (2.0 * t)
        if np.isfinite(t_op):
            n_eff_op += op.size / (2.0 * t_op)
    n_eff = reduce_sum(dist, n_eff)
    n_eff_op = reduce_sum(dist, n_eff_op)

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
            "arithmetic": "int8 occupations, integer delta correlations, float-float "
                          "(2 x f32) ECI dot, f32 acceptance, f64 running energy",
            "parallelism": f"replicas only, {w.n_replicas} per GPU",
            "schedule": {"threads_per_replica": tuned["threads"],
                         "cta_order": "largest first" if tuned["cta_order"] else "replica order",
                         "picked_by": "autotuner (10 timed trial passes per candidate)"},
        }),
        "proposals": int(props_all), "acceptance": p_acc,
        "proposals_per_s_per_replica": value / (w.n_replicas * ws),
        "effective_samples_per_s": n_eff / t_dev,
        "effective_samples_per_s_order_parameter": n_eff_op / t_dev,
        "running_energy_rel_drift_vs_recompute": drift,
        "tau_int_potential_median": float(np.nanmedian(taus)),
        "host_wall_s": t1 - t0,
        "e2e": {"value": e2e_props / e2e_time, "unit": "proposals/s",
                "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": e2e_steps,
                "pipeline": "two replica batches on two streams alternate; each step = one "
                            "CUDA graph: upload occupations, one pass, read occupations back"},
        "roofline": {"bound": "smem", "achieved": achieved, "peak": smem_gbs, "unit": "GB/s",
                     "frac": achieved / smem_gbs, "traffic": traffic,
                     "peak_source": "measured in this run by cem_smem_bandwidth "
                                    "(16-byte shared loads, all SMs)",
                     "bytes_per_proposal": bytes_per_prop,
                     "kernel": "k_sweep<2>", "kernel_ms": kernel_ms},
        "gpu_launches": 1,
        "clocks": clocks,
    }
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


def run_learned_comparison(args):
    """Configuration 3: T_c from a temperature scan of the plain sampler, then
    plain vs learned-proposal effective independent samples per second of the
    energy and the L1_2 order parameter at T = 0.9 T_c (48^3, x_B = 0.25)."""
    from casmcode_clexmonte_gb300 import build as B

    B.build()
    from casmcode_clexmonte_gb300 import calculator as cm
    from casmcode_clexmonte_gb300 import workloads
    from casmcode_clexmonte_gb300.stats import tau_int

    w = workloads.config(3)
    ce = w.ce
    sysd = cm.System(ce)
    # 1. temperature scan (24^3, plain sampler): heat capacity peak
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
    tc = float(temps[inner][int(np.argmax(cv[inner]))])
    T = 0.9 * tc
    # 2. plain sampler, 32 x 48^3
    n_rep = w.n_replicas
    plain = cm.ReplicaBatch(sysd, "canonical", w.L)
    for i in range(n_rep):
        plain.set_conditions(i, T)
        plain.set_seed(i, 1000 + i)
        plain.set_occupation(i, w.occupation[i])
    plain.run(args.warmup * 50, 0)
    plain.run(args.steps, 0, record_samples=True)
    plain.synchronize()
    t_plain = plain.kernel_ms() / 1e3
    prop_plain = sum(plain.stats(i)["n_proposed"] for i in range(n_rep))
    neff_e = neff_op = 0.0
    taus_p = []
    for i in range(n_rep):
        e, _ = plain.samples(i, args.steps)
        op = plain.order_samples(i, args.steps)
        te, to = tau_int(e), tau_int(op)
        taus_p.append((te, to))
        neff_e += e.size / (2 * te)
        neff_op += op.size / (2 * to)
    e_rep_plain = np.array([plain.stats(i)["mean_potential"] for i in range(n_rep)])
    mean_e_plain = float(e_rep_plain.mean())
    sig_plain = float(e_rep_plain.std(ddof=1) / np.sqrt(n_rep))
    # 3. train the proposal network on plain-sampler snapshots (1e6 environments)
    X, t = [], []
    for i in range(n_rep):
        x_i, t_i = plain.learned_features(i)
        X.append(x_i)
        t.append(t_i)
    X = np.concatenate(X)[:1_000_000]
    t = np.concatenate(t)[:1_000_000]
    net = cm.LearnedProposal(seed=11)
    t0 = time.perf_counter()
    losses = net.train(X, t, epochs=4, batch=4096, lr=2e-3, seed=5)
    train_s = time.perf_counter() - t0
    # 4. learned-proposal sampler from the equilibrated plain states
    lp = args.learned_passes
    plain.learned_run(net, lp, lp // 5, record_samples=True)
    plain.synchronize()
    t_learned = plain.kernel_ms() / 1e3
    neff_e_l = neff_op_l = 0.0
    taus_l = []
    acc_l = []
    for i in range(n_rep):
        e, op = plain.learned_samples(i, lp)
        te, to = tau_int(e), tau_int(op)
        taus_l.append((te, to))
        neff_e_l += e.size / (2 * te)
        neff_op_l += op.size / (2 * to)
    e_rep_learned = np.array([plain.learned_samples(i, lp)[0].mean() for i in range(n_rep)])
    mean_e_learned = float(e_rep_learned.mean())
    sig_learned = float(e_rep_learned.std(ddof=1) / np.sqrt(n_rep))
    sig_diff = float(np.hypot(sig_plain, sig_learned))
    # 5. the plain sampler again, from the learned chain's final states (its global
    # swaps have removed the antiphase boundaries the plain chain was still
    # coarsening): both chains then sample the same equilibrium state
    plain.run(args.steps, 0, record_samples=True)
    plain.synchronize()
    e_rep_plain2 = np.array([plain.stats(i)["mean_potential"] for i in range(n_rep)])
    mean_e_plain2 = float(e_rep_plain2.mean())
    sig_plain2 = float(e_rep_plain2.std(ddof=1) / np.sqrt(n_rep))
    sig_diff2 = float(np.hypot(sig_plain2, sig_learned))
    line = {
        "metric": "effective samples/s (learned vs plain GPU Metropolis, same <E>)",
        "workload": w.name, "T_c_scan_K": tc, "temperature_K": T,
        "heat_capacity_scan": {"T_K": [float(x) for x in temps], "C_per_uc": [float(x) for x in cv]},
        "plain": {"passes": args.steps, "seconds": t_plain, "proposals_per_s": prop_plain / t_plain,
                  "tau_int_E_median": float(np.median([a for a, _ in taus_p])),
                  "tau_int_order_median": float(np.median([b for _, b in taus_p])),
                  "eff_samples_per_s_E": neff_e / t_plain,
                  "eff_samples_per_s_order": neff_op / t_plain, "mean_E": mean_e_plain,
                  "mean_E_sigma": sig_plain},
        "learned": {"passes": lp, "seconds": t_learned,
                    "proposals_per_s": n_rep * lp * int(w.n_sites[0]) / t_learned,
                    "tau_int_E_median": float(np.median([a for a, _ in taus_l])),
                    "tau_int_order_median": float(np.median([b for _, b in taus_l])),
                    "eff_samples_per_s_E": neff_e_l / t_learned,
                    "eff_samples_per_s_order": neff_op_l / t_learned, "mean_E": mean_e_learned,
                    "mean_E_sigma": sig_learned,
                    "train_seconds": train_s, "train_loss": [float(x) for x in losses]},
        "ratio_learned_over_plain_E": (neff_e_l / t_learned) / (neff_e / t_plain),
        "ratio_learned_over_plain_order": (neff_op_l / t_learned) / (neff_op / t_plain),
        "same_E_within_2sigma": bool(abs(mean_e_learned - mean_e_plain) <= 2 * sig_diff),
        "E_difference_over_sigma": abs(mean_e_learned - mean_e_plain) / sig_diff if sig_diff > 0 else None,
        "plain_from_learned_states": {
            "passes": args.steps, "mean_E": mean_e_plain2, "mean_E_sigma": sig_plain2,
            "same_E_within_2sigma": bool(abs(mean_e_learned - mean_e_plain2) <= 2 * sig_diff2),
            "E_difference_over_sigma": abs(mean_e_learned - mean_e_plain2) / sig_diff2
            if sig_diff2 > 0 else None},
    }
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
    ap.add_argument("--learned-passes", type=int, default=40)
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
