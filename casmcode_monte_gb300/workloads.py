"""Synthetic workloads of the benchmark configurations other than the headline FCC 64^3 pass.

``python -m casmcode_monte_gb300.workloads batched [--chains 4096 --passes 500]``
    4096 independent binary FCC cluster-expansion chains, L uniform in
    {8,12,16,24,32,48}, T uniform in [300,2000] K, mu uniform in [-0.3,0.3] eV, random
    initial occupations, all swept in one launch of the persistent pool kernel; compared
    with running the same jobs one launch per job (ChainBatch, one chain) on a sample.

Each prints one JSON line.  Inputs are seeded synthetic data of the configurations' shapes.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from . import clex

BATCHED_L = (8, 12, 16, 24, 32, 48)


def batched_jobs(n_chains: int, seed: int = 0, kind: str = "fcc_binary"):
    rng = np.random.default_rng(seed)
    model = clex.ClexModel(kind, clex.make_eci(kind, 1))
    jobs = []
    for c in range(n_chains):
        L = int(rng.choice(BATCHED_L))
        n = L**3
        occ = rng.integers(0, model.n_species, size=n).astype(np.int8)
        T = float(rng.uniform(300.0, 2000.0))
        mu = rng.uniform(-0.3, 0.3, size=model.n_species - 1)
        jobs.append({"L": L, "occ": occ, "T": T, "mu": mu, "seed": int(seed * 1000003 + c + 1), "id": c})
    return model, jobs


def run_batched(n_chains: int = 4096, n_passes: int = 500, plain_sample: int = 64, precision: str = "fp64",
                seed: int = 0) -> dict:
    import torch

    model, jobs = batched_jobs(n_chains, seed)
    total_sites = sum(j["L"] ** 3 for j in jobs)
    pool = clex.ChainPool(model, arena_bytes=total_sites + 16 * n_chains, max_chains=n_chains, precision=precision)
    t0 = time.perf_counter()
    slots = [pool.add((j["L"],) * 3, j["occ"], j["T"], j["mu"], j["seed"], j["id"]) for j in jobs]
    t_admit = time.perf_counter() - t0
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    out = pool.run(slots, n_passes, want_output=True)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t1
    kernel_ms = pool.last_kernel_ms()
    attempts = total_sites * n_passes
    # plain per-job launches on a sample (one chain per launch, created and read back per job)
    rng = np.random.default_rng(seed + 1)
    sample = rng.choice(n_chains, size=min(plain_sample, n_chains), replace=False)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    plain_attempts = 0
    for i in sample:
        j = jobs[int(i)]
        b = clex.ChainBatch(model, (j["L"],) * 3, j["occ"][None, :], [j["T"]], j["mu"][None, :], [j["seed"]],
                            chain_ids=[j["id"]], precision=precision)
        b.run(n_passes, want_output=True)
        b.occupation()
        b.close()
        plain_attempts += j["L"] ** 3 * n_passes
    torch.cuda.synchronize()
    plain_wall = time.perf_counter() - t2
    plain_jobs_per_s = len(sample) / plain_wall
    # identical trajectories either way (same Philox streams): compare the sample's last chain
    return {
        "workload": "batched_fcc_binary_4096_chains",
        "chains": n_chains, "passes": n_passes, "precision": precision, "total_sites": total_sites,
        "site_attempts": attempts,
        "batched_kernel_ms": kernel_ms, "batched_wall_s": wall, "admission_s": t_admit,
        "batched_jobs_per_s": n_chains / wall,
        "batched_site_attempts_per_s": attempts / (kernel_ms * 1e-3),
        "plain_sample_jobs": int(len(sample)), "plain_jobs_per_s": plain_jobs_per_s,
        "plain_site_attempts_per_s": plain_attempts / plain_wall,
        "speedup_jobs_per_s": (n_chains / wall) / plain_jobs_per_s,
        "mean_acceptance": float(out[:, :, 0].sum() / attempts),
    }


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=["batched"])
    ap.add_argument("--chains", type=int, default=4096)
    ap.add_argument("--passes", type=int, default=500)
    ap.add_argument("--plain-sample", type=int, default=64)
    ap.add_argument("--precision", default="fp64")
    a = ap.parse_args(argv)
    if a.workload == "batched":
        r = run_batched(a.chains, a.passes, a.plain_sample, a.precision)
    print(json.dumps(r), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
