"""Benchmark: Metropolis site-attempts/s, plain FCC 64^3 binary cluster expansion.

Workload (one "step" = one Metropolis pass over every site of every chain): binary FCC
cluster expansion (empty, point, pairs 1-4NN, 3 smallest triplets, NN tetrahedron;
occupation basis; ECI N(0, 0.03 eV)/size^2 from seed 1), 64^3 primitive-cell supercell
(262,144 sites), 50 % B placed by a seeded shuffle, semi-grand canonical at 8
temperatures linspace(300, 2000, 8) K, mu = 0.  The 8 chains are independent; with
N GPUs every rank runs its own 8 chains (weak scaling, no collective).

value   device throughput of the sweep: attempts / sum over runs of the CUDA-event time of
        each run (first launch to last; a rotated run is several launches on the batch's
        streams, seven chains on 16-CTA clusters and one in turn on a 12-CTA cluster), inputs
        resident in HBM, L2 flushed between runs (outside the events).
e2e     the same job through the public C-ABI with host buffers: create the batch
        (H2D of occupations and parameters), run the passes returning per-pass samples to
        the host (D2H), read the final occupations (D2H); wall clock.
full_config
        the same chains as one job of the configuration's 2000 passes (--config-passes):
        device time of one run call (long runs rotate) and the same job end to end from
        pinned host buffers.
batched the batched-chains workload (4096 binary FCC chains, L uniform in {8,12,16,24,32,48},
        T in [300,2000] K, mu in [-0.3,0.3] eV, 500 passes, one persistent launch per CTA
        class and layout) as converged-or-finished jobs/s, beside the same jobs one launch per
        job on a sample; chains shard by rank.
serving a Poisson stream of binary/ternary FCC jobs (L uniform in 16..128, pass budget
        100..5000, stop at 1e-4 eV/site by the reference's rule) served with continuous
        batching: converged jobs/s and p50/p99 latency, beside the same kind of jobs one at a
        time; jobs shard by rank (job i on rank i mod N).
--impl reference: the reference's CPU path (random-site SGC Metropolis, mt19937_64,
        FP64 cluster-expansion dE; the oracle restatement) on all host cores, one chain
        per process, each step a bounded sample.
--gpus N without a torchrun environment starts its own N ranks (one process per GPU,
        127.0.0.1 rendezvous) and prints rank 0's line.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L = 64
N_CHAINS = 8
BYTES_PER_ATTEMPT = 56  # (1 own read + 54 neighbour reads + 1 write) x int8
METRIC = "Metropolis site-attempts/s (FCC 64^3 CE)"
WORKLOAD = "fcc64_binary_ce_sgc_8T"


def launch_ranks(n: int, argv: list) -> int:
    """Start ``n`` ranks of this script (one process per GPU, RANK/LOCAL_RANK/WORLD_SIZE and a
    127.0.0.1 rendezvous in their environment), forward rank 0's output and return the
    largest exit code: ``--gpus N`` outside torchrun never silently runs one rank."""
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, os.path.abspath(__file__), *argv], env=env,
                                      stdout=None if r == 0 else subprocess.DEVNULL))
    return max(p.wait() for p in procs)


def _env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(x: float, dist_mod, device: str) -> float:
    """The largest of the ranks' values of x: the slowest rank sets a whole-job time."""
    if dist_mod is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist_mod.all_reduce(t, op=dist_mod.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, world: int, ms: float) -> float:
    """Whole-job throughput: the units all ranks processed over the (slowest) time."""
    return units_per_rank * world / (ms * 1e-3)


def make_inputs(rank: int):
    from casmcode_monte_gb300 import clex

    eci = clex.make_eci("fcc_binary", 1)
    rng = np.random.default_rng(1000 + rank)
    n = L**3
    occ = np.stack([clex.random_occupation(2, n, rng) for _ in range(N_CHAINS)])
    T = np.linspace(300.0, 2000.0, N_CHAINS)
    mu = np.zeros((N_CHAINS, 1))
    seeds = (np.arange(N_CHAINS, dtype=np.uint64) + np.uint64(1 + 1000 * rank)) * np.uint64(0x9E3779B97F4A7C15 % (2**63))
    return eci, occ, T, mu, seeds


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def flush_l2(buf):
    import torch

    buf.add_(1)  # writes 256 MB, larger than the 129 MB L2


def cpu_baseline_sample(seconds_target: float = 10.0) -> dict:
    """The oracle's random-site reference loop on one host core, one 64^3 chain."""
    from casmcode_monte_gb300 import clex
    from tests import oracle_lib

    eci, occ, T, mu, seeds = make_inputs(0)
    orc = oracle_lib.OracleCE((L, L, L), 2, eci)
    o = occ[0].astype(np.int32)
    # calibrate then run a bounded sample
    _, _, t = orc.random_site_run(o, float(T[3]), mu[3], 7, 20000)
    rate = 20000 / max(t, 1e-9)
    n = int(min(max(rate * seconds_target, 1e5), 5e8))
    _, _, t = orc.random_site_run(o, float(T[3]), mu[3], 8, n)
    return {"value": n / t, "unit": "site-attempts/s", "cores": 1, "kind": "port",
            "sample": f"{n} random-site attempts on one 64^3 chain at T={T[3]:.0f} K (oracle restatement, g++ -O2)"}


_REF_STATE = {}


def _ref_init():
    """Worker set-up (pool initializer): the model and the chains' initial occupations."""
    if "model" not in _REF_STATE:
        from tests import oracle_lib

        eci, occ, T, mu, seeds = make_inputs(0)
        _REF_STATE["model"] = oracle_lib.OracleCE((L, L, L), 2, eci)
        _REF_STATE["inputs"] = (occ.astype(np.int32), T, mu)


def _ref_worker(args):
    """One bounded sample of the reference loop.  The model (the same cluster expansion for
    every chain) and the chains' initial occupations are built once per worker process and
    reused across steps, whichever chain a step hands the worker."""
    chain, n_steps, step = args
    _ref_init()
    orc = _REF_STATE["model"]
    occ, T, mu = _REF_STATE["inputs"]
    _, _, t = orc.random_site_run(occ[chain], float(T[chain]), mu[chain], 100 + 1000 * step + chain, n_steps)
    return n_steps, t


def run_reference(args) -> None:
    rank, world, _ = _env_rank()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    n_proc = cores  # one independent chain per host core (chain c % 8 of the workload)
    # each step is a bounded sample: about two minutes for the whole run at ~0.8 M
    # attempts/s per process, at most --ref-steps-per-sample attempts per process
    steps_per_chain = int(min(args.ref_steps_per_sample, max(2e4, 0.8e6 * 120.0 / (args.steps + args.warmup))))
    ctx = mp.get_context("spawn")
    vals, walls = [], []
    with ctx.Pool(n_proc, initializer=_ref_init) as pool:
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            res = pool.map(_ref_worker, [(c % N_CHAINS, steps_per_chain, i) for c in range(n_proc)], chunksize=1)
            wall = time.perf_counter() - t0
            if i >= args.warmup:
                vals.append(sum(r[0] for r in res) / wall)
                walls.append(wall)
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "site-attempts/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(walls),
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "supercell": [L, L, L], "chains": N_CHAINS,
                       "sample_steps_per_process": steps_per_chain, "processes": n_proc},
            "cpu_baseline": {"value": value, "unit": "site-attempts/s", "cores": n_proc, "kind": "port",
                             "sample": f"{steps_per_chain} random-site attempts per process, {n_proc} processes"},
            "e2e": {"value": value, "unit": "site-attempts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _gather(obj, dist_mod):
    """Every rank's ``obj`` as a list (just [obj] on one rank)."""
    if dist_mod is None:
        return [obj]
    out = [None] * dist_mod.get_world_size()
    dist_mod.all_gather_object(out, obj)
    return out


def run_batched_extra(rank: int, world: int, dist_mod, n_chains: int = 4096, n_passes: int = 500,
                      plain_sample: int = 48) -> dict:
    """Batched chains (this rank's share: chain c on rank c mod N) in one persistent launch per
    CTA class and layout, end to end through the pool API (admission H2D, the run, the
    per-pass outputs and final occupations back to the host), against the same jobs one
    ChainBatch per job (create, run, read back) on a sample."""
    import torch

    from casmcode_monte_gb300 import clex, workloads

    model, jobs = workloads.batched_jobs(n_chains, seed=0)
    mine = [j for j in jobs if j["id"] % world == rank]
    total_sites = sum(j["L"] ** 3 for j in mine)
    pool = clex.ChainPool(model, arena_bytes=total_sites + 16 * len(mine), max_chains=len(mine))
    for L in workloads.BATCHED_L:  # geometry of every shape built once, as a long-lived pool has it
        pool.prepare((L, L, L))
    # per-pass outputs into pinned host memory allocated ahead, as a server keeps it
    out_t = torch.empty((len(mine), n_passes, model.n_classes + 2), dtype=torch.int64, pin_memory=True)
    out = out_t.numpy()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    slots = pool.add_many([(j["L"],) * 3 for j in mine], [j["occ"] for j in mine], [j["T"] for j in mine],
                          np.stack([j["mu"] for j in mine]), [j["seed"] for j in mine], [j["id"] for j in mine])
    pool.run(slots, n_passes, out=out)
    finals = [pool.occupation(s) for s in slots[:: max(1, len(slots) // 64)]]
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    kernel_ms = pool.last_kernel_ms()
    launches = pool.last_launches()
    pool.close()
    rng = np.random.default_rng(1)
    sample = [mine[int(i)] for i in rng.choice(len(mine), size=min(plain_sample, len(mine)), replace=False)]
    for L in workloads.BATCHED_L:  # per-shape host geometry cached before the clock, as for the pool
        clex.color_supercell("fcc_binary", (L, L, L))
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for j in sample:
        b = clex.ChainBatch(model, (j["L"],) * 3, j["occ"][None, :], [j["T"]], j["mu"][None, :], [j["seed"]],
                            chain_ids=[j["id"]])
        b.run(n_passes, want_output=True)
        b.occupation()
        b.close()
    torch.cuda.synchronize()
    plain_wall = time.perf_counter() - t1
    per = _gather({"wall": wall, "kernel_ms": kernel_ms, "sites": total_sites, "n": len(mine),
                   "plain_wall": plain_wall, "plain_n": len(sample),
                   "accept": float(out[:, :, 0].sum())}, dist_mod)
    wall_max = max(p["wall"] for p in per)
    kms = max(p["kernel_ms"] for p in per)
    n_all = sum(p["n"] for p in per)
    sites_all = sum(p["sites"] for p in per)
    plain_rate = sum(p["plain_n"] for p in per) / max(p["plain_wall"] for p in per)
    jobs_per_s = n_all / wall_max
    return {"workload": f"batched_fcc_binary_{n_chains}_chains", "chains": n_all, "passes": n_passes,
            "jobs_per_s": jobs_per_s, "unit": "jobs/s",
            "timed": "end to end: admission of every chain in one add_many call (H2D), one run of all passes "
                     "with per-pass outputs back into pinned host memory, final occupations of a sample read back",
            "kernel_ms": kms, "site_attempts_per_s_kernel": sites_all * n_passes / (kms * 1e-3),
            "launches": launches,
            "plain_jobs_per_s": plain_rate, "plain_sample_jobs": sum(p["plain_n"] for p in per),
            "plain": "one ChainBatch per job: create (H2D), run with per-pass outputs, read the occupation",
            "speedup_vs_plain": jobs_per_s / plain_rate,
            "mean_acceptance": sum(p["accept"] for p in per) / (sites_all * n_passes)}


def run_serving_extra(rank: int, world: int, dist_mod, n_jobs: int = 2000, rate: float = 200.0,
                      plain_sample: int = 24) -> dict:
    """A Poisson stream of jobs served with continuous batching (this rank's share: job i on
    rank i mod N, arrival times kept), against the same kind of jobs run one at a time."""
    from casmcode_monte_gb300 import clex, serving

    models = {k: clex.ClexModel(k, clex.make_eci(k, 1)) for k in ("fcc_binary", "fcc_ternary")}
    jobs = serving.poisson_jobs(n_jobs, rate, models, seed=0)
    mine = [j for j in jobs if j.id % world == rank]
    eng = serving.ServingEngine(models, arena_bytes=16 << 30, max_chains=4096, precision="fp32")
    t_prep = eng.prepare(sorted({j.L for j in mine}))
    st = eng.run(mine, realtime=True)
    plain_jobs = [j for j in serving.poisson_jobs(plain_sample * world, rate, models, seed=1) if j.id % world == rank]
    pst = serving.run_plain(plain_jobs, models, precision="fp32", prepare=True)
    per = _gather({"lat": [j.latency for j in st.jobs], "conv": sum(1 for j in st.jobs if j.converged),
                   "n": len(st.jobs), "wall": st.wall_s, "gpu_s": st.gpu_ms * 1e-3,
                   "plain_conv": sum(1 for j in pst.jobs if j.converged), "plain_wall": pst.wall_s,
                   "plain_n": len(pst.jobs), "prep": t_prep}, dist_mod)
    lat = np.concatenate([np.asarray(p["lat"], dtype=np.float64) for p in per])
    wall = max(p["wall"] for p in per)
    conv = sum(p["conv"] for p in per)
    plain_rate = sum(p["plain_conv"] for p in per) / max(p["plain_wall"] for p in per)
    return {"workload": "serving_fcc_ce_poisson", "jobs": sum(p["n"] for p in per), "rate_per_s": rate,
            "precision": "fp32 decisions (fp64 energies)", "converged_jobs": conv,
            "converged_jobs_per_s": conv / wall, "unit": "converged jobs/s",
            "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
            "wall_s": wall, "gpu_busy_s": max(p["gpu_s"] for p in per),
            "geometry_prepare_s": max(p["prep"] for p in per),
            "plain_converged_jobs_per_s": plain_rate, "plain_sample_jobs": sum(p["plain_n"] for p in per),
            "plain": "the same kind of jobs one at a time, one launch per 100-pass chunk per job",
            "speedup_vs_plain": (conv / wall) / max(plain_rate, 1e-12)}


def run_full_config_extra(rank: int, world: int, dist_mod, model, occ, T, mu, seeds, passes: int = 2000,
                          peak: float = 6800.0) -> dict:
    """The workload as the configuration names it: the same 8 chains of 64^3, ``passes`` passes
    as one job.  Device time: one run call on a fresh batch (the library's own choice of
    launches; long runs rotate the chains over two cluster sizes), L2 flushed before it.  End to
    end: the same job from pinned host buffers (create the batch, initial correlations, the
    passes with per-pass outputs, final occupations), median of three; max over ranks."""
    import torch

    from casmcode_monte_gb300 import clex

    attempts = N_CHAINS * L**3 * passes
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    b = clex.ChainBatch(model, (L, L, L), occ, T, mu, seeds)
    flush_l2(flush)
    torch.cuda.synchronize()
    b.run(passes, want_output=False)
    torch.cuda.synchronize()
    dev_ms = max_over_ranks(b.last_kernel_ms(), dist_mod, "cuda")
    launches = b.last_launches()
    b.close()
    del flush

    def pinned(a):
        t = torch.empty(a.shape, dtype={np.dtype(np.int8): torch.int8, np.dtype(np.int64): torch.int64}[a.dtype],
                        pin_memory=True)
        t.numpy()[...] = a
        return t

    occ_h = pinned(occ)
    out_h = pinned(np.zeros((passes, N_CHAINS, model.n_classes + 2), dtype=np.int64))
    final_h = pinned(np.zeros_like(occ))
    walls = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b = clex.ChainBatch(model, (L, L, L), occ_h.numpy(), T, mu, seeds)
        b.corr()
        b.run(passes, out=out_h.numpy())
        b.occupation(out=final_h.numpy())
        torch.cuda.synchronize()
        walls.append((time.perf_counter() - t0) * 1e3)
        b.close()
    e2e_ms = max_over_ranks(statistics.median(walls), dist_mod, "cuda")
    value = job_throughput(attempts, world, dev_ms)
    achieved = BYTES_PER_ATTEMPT * attempts / (dev_ms * 1e-3) / 1e9
    return {"workload": f"{WORKLOAD}, {passes} passes as one job", "passes": passes,
            "value": value, "unit": "site-attempts/s", "ms": dev_ms, "gpu_launches": launches,
            "roofline_frac": achieved / peak, "achieved_gbs": achieved,
            "e2e": {"value": job_throughput(attempts, world, e2e_ms), "unit": "site-attempts/s", "ms": e2e_ms,
                    "h2d_bytes": int(occ.nbytes + T.nbytes + mu.nbytes + seeds.nbytes),
                    "d2h_bytes": int(out_h.numel() * 8 + occ.nbytes)}}


def run_gpu(args) -> None:
    import torch

    rank, world, local = _env_rank()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from casmcode_monte_gb300 import clex

    eci, occ, T, mu, seeds = make_inputs(rank)
    model = clex.ClexModel("fcc_binary", eci)
    batch = clex.ChainBatch(model, (L, L, L), occ, T, mu, seeds, ctas_per_chain=args.ctas_per_chain)
    attempts_per_step = N_CHAINS * L**3
    ppl = max(1, int(args.passes_per_launch))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    # warmup
    left = args.warmup
    while left > 0:
        n = min(ppl, left)
        batch.run(n, want_output=False)
        left -= n
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    kernel_ms = 0.0
    launches = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    left = args.steps
    while left > 0:
        n = min(ppl, left)
        flush_l2(flush)
        torch.cuda.synchronize()
        batch.run(n, want_output=False)
        kernel_ms += batch.last_kernel_ms()
        launches += batch.last_launches()
        left -= n
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    kernel_ms = max_over_ranks(kernel_ms, dist, "cuda")
    if dist:
        dist.barrier()
    value = job_throughput(attempts_per_step * args.steps, world, kernel_ms)

    # ---- e2e through the C-ABI with host buffers: the inputs (occupations, temperatures,
    # exchange potentials, seeds) copied from pinned host memory, per-pass outputs and the final
    # occupations read back into pinned host memory
    def pinned(a):
        t = torch.empty(a.shape, dtype={np.dtype(np.int8): torch.int8, np.dtype(np.int64): torch.int64,
                                        np.dtype(np.float64): torch.float64}[a.dtype], pin_memory=True)
        v = t.numpy()
        v[...] = a
        return t, v

    _pin_keep = []
    occ_h = pinned(occ)
    _pin_keep.append(occ_h[0])
    out_h = pinned(np.zeros((args.steps, N_CHAINS, model.n_classes + 2), dtype=np.int64))
    final_h = pinned(np.zeros_like(occ))
    _pin_keep += [out_h[0], final_h[0]]
    e2e_ms = []
    h2d = occ.nbytes + T.nbytes + mu.nbytes + seeds.nbytes
    d2h_per_step = N_CHAINS * (model.n_classes + 2) * 8
    for rep in range(5):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        b2 = clex.ChainBatch(model, (L, L, L), occ_h[1], T, mu, seeds, ctas_per_chain=args.ctas_per_chain)
        corr0 = b2.corr()
        left, done = args.steps, 0
        while left > 0:
            n = min(ppl, left)
            b2.run(n, out=out_h[1][done:done + n])
            left -= n
            done += n
        b2.occupation(out=final_h[1])
        torch.cuda.synchronize()
        e2e_ms.append((time.perf_counter() - t1) * 1e3)
        b2.close()
    chunks = [out_h[1].copy()]
    e2e_best_ms = max_over_ranks(statistics.median(e2e_ms), dist, "cuda")
    e2e_value = job_throughput(attempts_per_step * args.steps, world, e2e_best_ms)
    samples = clex.accumulate(model, corr0, np.concatenate(chunks, axis=0), mu, L**3)

    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            peak = float(json.load(f)["hbm_gbs"])
        peak_src = "measured"
    achieved = BYTES_PER_ATTEMPT * attempts_per_step * args.steps / (kernel_ms * 1e-3) / 1e9
    traffic, traffic_source = None, None
    tp = os.path.join(ROOT, "profiles", "ce_sweep_fcc64_binary_traffic.json")
    last_launch_passes = min(ppl, args.steps)
    if os.path.exists(tp) and launches > 0:
        with open(tp) as f:
            tj = json.load(f)
        # DRAM bytes per pass from an ncu capture of the same kernel and workload, scaled to
        # the passes of one launch of this run (traffic per launch grows with its passes:
        # the lattice stays in shared memory for the launch, so per pass it is nearly flat)
        traffic = tj["dram_bytes_per_pass"] * args.steps / launches
        traffic_source = (f"{os.path.relpath(tp, ROOT)}: {tj['source']}; scaled to {args.steps / launches:g} "
                          "passes per launch")
    rotation = batch.rotation()
    extras = {}
    if not args.no_extras:
        extras["full_config"] = run_full_config_extra(rank, world, dist, model, occ, T, mu, seeds,
                                                      passes=args.config_passes, peak=peak)
        extras["batched"] = run_batched_extra(rank, world, dist, n_chains=args.batched_chains)
        extras["serving"] = run_serving_extra(rank, world, dist, n_jobs=args.serving_jobs)
    if rank == 0:
        cpu = cpu_baseline_sample(args.cpu_seconds) if args.cpu_seconds > 0 else None
        line = {
            "metric": METRIC, "value": value, "unit": "site-attempts/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": kernel_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "i8/i32+f32 (f64 exact decisions)",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "supercell": [L, L, L], "chains_per_gpu": N_CHAINS,
                       "temperatures_K": T.tolist(), "passes_per_launch": ppl,
                       "ctas_per_chain": batch.ctas_per_chain, "rotation": rotation,
                       "rotated_launches": launches > (args.steps + ppl - 1) // ppl, "colors": batch.n_colors,
                       "threads_per_cta": batch.threads, "l2": "flushed between launches (256 MB write)",
                       "attempts_per_step": attempts_per_step},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_source,
                         "peak_source": peak_src, "bytes_per_attempt": BYTES_PER_ATTEMPT,
                         "attempts_per_launch": attempts_per_step * args.steps / max(launches, 1)},
            "e2e": {"value": e2e_value, "unit": "site-attempts/s", "h2d_bytes_per_step": h2d / args.steps,
                    "d2h_bytes_per_step": d2h_per_step + occ.nbytes / args.steps, "ms": e2e_best_ms,
                    "timed": "median of 5 jobs: create the batch from pinned host inputs (H2D), initial "
                             "correlations (D2H), the passes with per-pass outputs and the final occupations "
                             "read into pinned host memory (D2H)"},
            "gpu_launches": launches,
            "clocks": clk,
            "wall_s_timed": wall,
            "check": {"mean_potential_energy_last_pass_eV": samples.potential_energy[-1].tolist(),
                      "acceptance_last_pass": (samples.n_accept[-1] / L**3).tolist()},
        }
        if cpu is not None:
            line["cpu_baseline"] = cpu
        line.update(extras)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


CANON_L = 48
CANON_METRIC = "canonical Metropolis site-attempts/s (FCC 48^3 CE, fixed composition)"


def run_canonical(args) -> None:
    """Canonical (fixed-composition) sweep: one chain per SM of binary FCC 48^3 (110,592
    sites, exactly 50 % B by a seeded shuffle), T linspace(300, 2000), exchanges of matched
    same-colour pairs.  A site-attempt is one site of a proposed pair (every site of a pass is
    in one pair or a fixed point: N per chain and pass); the reference's step proposes one
    pair (2 site-attempts).  value: attempts / CUDA-event time, L2 flushed between runs;
    cpu_baseline: the reference's canonical dynamics (random pairs of different occupants)
    restated in the oracle, on one host core."""
    import torch

    from casmcode_monte_gb300 import clex

    rank, world, local = _env_rank()
    torch.cuda.set_device(local)
    n_chains = torch.cuda.get_device_properties(local).multi_processor_count
    eci = clex.make_eci("fcc_binary", 1)
    model = clex.ClexModel("fcc_binary", eci)
    rng = np.random.default_rng(2000 + rank)
    n = CANON_L**3
    occ = np.stack([clex.random_occupation(2, n, rng) for _ in range(n_chains)])
    T = np.linspace(300.0, 2000.0, n_chains)
    seeds = np.arange(1, n_chains + 1, dtype=np.uint64) * np.uint64(0x9E3779B1) + np.uint64(rank)
    batch = clex.CanonicalBatch(model, (CANON_L,) * 3, occ, T, seeds)
    ppl = max(1, int(args.passes_per_launch))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    left = args.warmup
    while left > 0:
        m = min(ppl, left)
        batch.run(m, want_output=False)
        left -= m
    torch.cuda.synchronize()
    kernel_ms, launches, left = 0.0, 0, args.steps
    while left > 0:
        m = min(ppl, left)
        flush_l2(flush)
        torch.cuda.synchronize()
        batch.run(m, want_output=False)
        kernel_ms += batch.last_kernel_ms()
        launches += 1
        left -= m
    attempts = n_chains * n * args.steps
    value = attempts / (kernel_ms * 1e-3)
    # end to end: create (H2D), run with per-pass outputs (D2H), read the occupations
    t1 = time.perf_counter()
    b2 = clex.CanonicalBatch(model, (CANON_L,) * 3, occ, T, seeds)
    left = args.steps
    while left > 0:
        m = min(ppl, left)
        b2.run(m)
        left -= m
    final = b2.occupation()
    e2e_s = time.perf_counter() - t1
    assert np.array_equal(np.bincount(final[0], minlength=2), np.bincount(occ[0], minlength=2))
    line = {"metric": CANON_METRIC, "value": value, "unit": "site-attempts/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": kernel_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "i8/i32+f32 (f64 exact decisions)", "data": "synthetic",
            "config": {"workload": "fcc48_binary_ce_canonical", "supercell": [CANON_L] * 3, "chains": n_chains,
                       "composition_B": 0.5, "passes_per_launch": ppl, "colors": list(batch.n_colors),
                       "threads_per_cta": batch.threads, "l2": "flushed between launches (256 MB write)"},
            "e2e": {"value": attempts / e2e_s, "unit": "site-attempts/s", "h2d_bytes_per_step": occ.nbytes / args.steps,
                    "d2h_bytes_per_step": n_chains * batch.n_slots * 8 + occ.nbytes / args.steps},
            "gpu_launches": launches}
    if rank == 0 and args.cpu_seconds > 0:
        from tests import oracle_lib

        orc = oracle_lib.OracleCE((CANON_L,) * 3, 2, eci)
        o = occ[0].astype(np.int32)
        t0 = time.perf_counter()
        orc.canonical_samples(o, float(T[n_chains // 2]), 5, 1)
        per_pass = time.perf_counter() - t0
        passes = max(1, int(args.cpu_seconds / max(per_pass, 1e-9)))
        t0 = time.perf_counter()
        orc.canonical_samples(o, float(T[n_chains // 2]), 6, passes)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": 2.0 * n * passes / dt, "unit": "site-attempts/s", "cores": 1, "kind": "port",
                                "sample": f"{passes} passes of {n} random canonical swaps on one 48^3 chain at "
                                          f"T={T[n_chains // 2]:.0f} K (oracle restatement, g++ -O2)"}
    if rank == 0:
        print(json.dumps(line), flush=True)


ISING_METRIC = "serial-replay Metropolis site-attempts/s (2-D Ising 25x25)"


def run_ising(args) -> None:
    """The plain method at CPU scale: 2-D square Ising, 25x25 periodic, occupation +-1 drawn
    uniformly from seed 1, J = 0.1 eV, T = 2000 K, mu = 0, 1000 passes, one sample of energy and
    composition per pass.  A step is one site-attempt.  The GPU path is the bit-exact serial
    replay (one warp, the reference's mt19937_64 draws) behind the reference's calculator
    interface (ising_cpp.semigrand_canonical.SemiGrandCanonicalCalculator.run); value: device
    time of the replay kernels; e2e: the calculator's run end to end (host state in and out);
    cpu_baseline: the reference's loop restated in the oracle on one host core."""
    import casmcode_monte_gb300 as monte
    import casmcode_monte_gb300.ising_cpp as ising
    import casmcode_monte_gb300.ising_cpp.semigrand_canonical as sgc
    import casmcode_monte_gb300.sampling as sampling

    rows = cols = 25
    n_pass = 1000
    rng = np.random.default_rng(1)
    occ0 = rng.choice(np.array([-1, 1], dtype=np.int32), size=rows * cols)

    def one_run():
        calc = sgc.SemiGrandCanonicalCalculator(ising.IsingSystem(ising.IsingFormationEnergy(J=0.1),
                                                                  ising.IsingParamComposition()))
        cfg = ising.IsingConfiguration((rows, cols))
        cfg.set_occupation(occ0)
        state = ising.IsingState(cfg, monte.ValueMap.from_dict({"temperature": 2000.0, "exchange_potential": [0.0]}))
        p = sampling.CompletionCheckParams()
        p.cutoff_params.max_count = n_pass
        engine = monte.RandomNumberEngine()
        engine.seed(1)
        t0 = time.perf_counter()
        data = calc.run(state, calc.default_sampling_functions(), {}, p, sgc.SemiGrandCanonicalEventGenerator(),
                        method_log=monte.MethodLog(None, None), random_engine=engine,
                        write_status_f=lambda c, l: None)
        return time.perf_counter() - t0, calc.last_kernel_ms, data

    for _ in range(args.warmup):
        one_run()
    walls, kms = [], []
    for _ in range(args.steps):
        w, k, data = one_run()
        walls.append(w)
        kms.append(k)
    attempts = rows * cols * n_pass
    kernel_ms = statistics.median(kms)
    line = {"metric": ISING_METRIC, "value": attempts / (kernel_ms * 1e-3), "unit": "site-attempts/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": kernel_ms, "higher_is_better": True,
            "scaling": "none (one chain)", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "ising25x25_sgc_1000_passes", "J": 0.1, "T": 2000.0, "mu": 0.0, "passes": n_pass,
                       "step": "one 1000-pass run of the calculator"},
            "e2e": {"value": attempts / statistics.median(walls), "unit": "site-attempts/s",
                    "h2d_bytes_per_step": rows * cols * 4 + 6700, "d2h_bytes_per_step": rows * cols * 4 + 6700 + n_pass * 8 * 52},
            "gpu_launches": None, "n_accept": int(data.n_accept)}
    if args.cpu_seconds > 0:
        from tests import oracle_lib

        t0 = time.perf_counter()
        reps = 0
        while time.perf_counter() - t0 < min(args.cpu_seconds, 5.0) or reps == 0:
            oracle_lib.ising_run(rows, cols, 0.1, True, 2000.0, 0.0, occ0, oracle_lib.make_cc_params(max_count=n_pass),
                                 1, oracle_lib.engine_state(1))
            reps += 1
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": attempts * reps / dt, "unit": "site-attempts/s", "cores": 1, "kind": "port",
                                "sample": f"{reps} runs of the reference loop (oracle restatement, g++ -O2, samples "
                                          "and completion checks included)"}
    print(json.dumps(line), flush=True)


NFOLD_METRIC = "rejection-free (N-fold way) events/s (FCC binary CE)"


def run_nfold(args) -> None:
    """Rejection-free semi-grand canonical dynamics of binary FCC L^3 chains (--nfold-size L,
    default 32: 32,768 sites, one chain per SM; up to 8192 sites four chains per SM), 50 % B
    by a seeded shuffle, T linspace(300, 2000), mu = 0; a step is one event (a selected flip
    with its rate updates) of every chain.  value: events / CUDA-event
    time; cpu_baseline: the same dynamics on the CPU (oracle: FP64 rates, Fenwick selection)
    on one host core."""
    import torch

    from casmcode_monte_gb300 import clex

    rank, world, local = _env_rank()
    torch.cuda.set_device(local)
    L_n = int(args.nfold_size)
    n = L_n**3
    eci = clex.make_eci("fcc_binary", 1)
    model = clex.ClexModel("fcc_binary", eci)
    # chains resident per SM for this size (4 up to 8192 sites), one chain per resident slot
    probe = clex.NfoldBatch(model, (L_n,) * 3, np.zeros((1, n), dtype=np.int8), [1000.0], [[0.0]], [1])
    n_chains = torch.cuda.get_device_properties(local).multi_processor_count * probe.chains_per_sm
    probe.close()
    rng = np.random.default_rng(3000 + rank)
    occ = np.stack([clex.random_occupation(2, n, rng) for _ in range(n_chains)])
    T = np.linspace(300.0, 2000.0, n_chains)
    mu = np.zeros((n_chains, 1))
    seeds = np.arange(1, n_chains + 1, dtype=np.uint64) * np.uint64(0x2545F491) + np.uint64(rank)
    batch = clex.NfoldBatch(model, (L_n,) * 3, occ, T, mu, seeds)
    warm = max(1, args.warmup // n)  # passes of N events
    batch.run(warm)
    passes = max(1, args.steps // n)
    kernel_ms = 0.0
    for _ in range(passes):
        batch.run(1)
        kernel_ms += batch.last_kernel_ms()
    events = n_chains * n * passes
    assert np.array_equal(batch.corr(), batch.corr(recompute=True))
    line = {"metric": NFOLD_METRIC, "value": events / (kernel_ms * 1e-3), "unit": "events/s", "n_gpus": world,
            "steps": passes * n, "warmup": warm * n, "ms_per_step": kernel_ms / (passes * n),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 rates, i64 correlations",
            "data": "synthetic",
            "config": {"workload": f"fcc{L_n}_binary_ce_nfold", "supercell": [L_n] * 3, "chains": n_chains,
                       "chains_per_sm": batch.chains_per_sm, "threads_per_cta": batch.threads,
                       "events_per_pass": n, "passes": passes},
            "gpu_launches": passes}
    if rank == 0 and args.cpu_seconds > 0:
        from tests import oracle_lib

        orc = oracle_lib.OracleCE((L_n,) * 3, 2, eci)
        o = occ[0].astype(np.int32)
        _, secs, _ = orc.nfold_run(o, float(T[n_chains // 2]), mu[0], 5, 2000)
        n_ev = int(max(2000, 2000 * args.cpu_seconds / max(secs, 1e-9)))
        _, secs, _ = orc.nfold_run(o, float(T[n_chains // 2]), mu[0], 6, n_ev)
        line["cpu_baseline"] = {"value": n_ev / secs, "unit": "events/s", "cores": 1, "kind": "port",
                                "sample": f"{n_ev} events on one {L_n}^3 chain at T={T[n_chains // 2]:.0f} K "
                                          "(oracle: FP64 rates, Fenwick selection, g++ -O2)"}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--passes-per-launch", type=int, default=100)
    ap.add_argument("--ctas-per-chain", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-steps-per-sample", type=float, default=2e6)
    ap.add_argument("--nfold-size", type=int, default=32, help="supercell edge of the nfold workload")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched and serving workloads")
    ap.add_argument("--config-passes", type=int, default=2000,
                    help="passes of the full-configuration job reported beside the headline")
    ap.add_argument("--batched-chains", type=int, default=4096)
    ap.add_argument("--serving-jobs", type=int, default=2000)
    ap.add_argument("--workload", default="fcc64_sgc", choices=["fcc64_sgc", "canonical", "nfold", "ising"],
                    help="fcc64_sgc: the headline semi-grand canonical pass; canonical: fixed-composition "
                         "sweeps of 48^3 chains; nfold: rejection-free dynamics of 32^3 chains; ising: the 25x25 "
                         "Ising serial replay")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_ranks(args.gpus, sys.argv[1:]))
    if args.gpus != int(os.environ.get("WORLD_SIZE", "1")):
        ap.error(f"--gpus {args.gpus} but WORLD_SIZE={os.environ.get('WORLD_SIZE', '1')}")
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "canonical":
        run_canonical(args)
    elif args.workload == "nfold":
        run_nfold(args)
    elif args.workload == "ising":
        run_ising(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
