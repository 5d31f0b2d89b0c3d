"""Synthetic workloads of the benchmark configurations other than the headline FCC 64^3 pass.

``python -m casmcode_monte_gb300.workloads precision``
    ternary FCC cluster expansion, 96^3, 5000 passes at 600 K, FP32 decisions against
    FP64 decisions from the same start; FP64 full recompute every 50 passes; <E>, <x>,
    C_v with error bars and the count of decisions FP32 flipped.

``python -m casmcode_monte_gb300.workloads serving [--jobs 20000 --rate 200]``
    Poisson stream of binary/ternary FCC cluster-expansion jobs (L uniform in 16..128,
    random T and mu, pass budget 100..5000, convergence of the potential energy to
    1e-4 eV/site by the reference's rule) served with continuous batching; jobs/s, p50/p99
    latency, and the same kind of jobs run one at a time for comparison.

``python -m casmcode_monte_gb300.workloads batched [--chains 4096 --passes 500]``
    4096 independent binary FCC cluster-expansion chains, L uniform in
    {8,12,16,24,32,48}, T uniform in [300,2000] K, mu uniform in [-0.3,0.3] eV, random
    initial occupations, all swept in one launch of the persistent pool kernel; compared
    with running the same jobs one launch per job (ChainBatch, one chain) on a sample.

``python -m casmcode_monte_gb300.workloads sweep --kind fcc_ternary --L 64 --chains 8 --passes 20``
    one chain batch of L^3 chains (seeded occupations, T spread over 600..1500 K, mu = 0)
    on the layout the library chooses or ``--layout byte|word|grid``: 3 warm-up passes,
    then three runs of --passes passes with L2 flushed before each; µs per pass and
    site-attempts/s of the median run (device time of the run).

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
    slots = pool.add_many([(j["L"],) * 3 for j in jobs], [j["occ"] for j in jobs], [j["T"] for j in jobs],
                          np.stack([j["mu"] for j in jobs]), [j["seed"] for j in jobs], [j["id"] for j in jobs])
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


def _stats(x: np.ndarray) -> dict:
    """Mean and precision of the mean (reference BasicStatisticsCalculator, 95 %)."""
    from .sampling import BasicStatisticsCalculator

    st = BasicStatisticsCalculator()(np.ascontiguousarray(x, dtype=np.float64))
    return {"mean": st.mean, "precision": st.calculated_precision}


def run_precision(L: int = 96, n_passes: int = 5000, T: float = 600.0, recompute_every: int = 50,
                  discard: int = 1000, seed: int = 4) -> dict:
    """Ternary FCC chain: FP32 decisions against FP64 decisions from the same start.

    Energies are exact integer correlation sums on the device (FP64 only when turned into
    energies), checked against a full FP64 recompute every ``recompute_every`` passes.
    Averages use the passes after ``discard``; error bars are the reference's
    autocorrelation-corrected precision of the mean (95 %).
    """
    kind = "fcc_ternary"
    model = clex.ClexModel(kind, clex.make_eci(kind, seed))
    rng = np.random.default_rng(seed)
    n = L**3
    occ = clex.random_occupation(3, n, rng)[None, :]
    mu = np.zeros((1, 2))
    result = {"workload": "precision_fcc_ternary_96", "L": L, "passes": n_passes, "T": T,
              "recompute_every": recompute_every, "discard": discard}
    series = {}
    for prec in ("fp64", "fp32"):
        b = clex.ChainBatch(model, (L, L, L), occ, [T], mu, [seed * 7919 + 1], precision=prec)
        corr = b.corr()[0]
        e_pot, x_b, x_c = [], [], []
        mismatches = 0
        kernel_ms = 0.0
        n_exact = n_flip = n_acc = 0
        for chunk in range(0, n_passes, recompute_every):
            m = min(recompute_every, n_passes - chunk)
            out = b.run(m)
            kernel_ms += b.last_kernel_ms()
            s = clex.accumulate(model, corr[None, :], out, mu, n)
            corr = s.int_corr[-1, 0].copy()
            full = b.corr()[0]
            mismatches += int(not np.array_equal(full, corr))
            e_pot.append(s.potential_energy[:, 0])
            x_b.append(s.param_composition[:, 0, 0])
            x_c.append(s.param_composition[:, 0, 1])
            n_exact += int(s.n_exact.sum())
            n_flip += int(s.n_flipped.sum())
            n_acc += int(s.n_accept.sum())
        e = np.concatenate(e_pot)[discard:]
        xb = np.concatenate(x_b)[discard:]
        xc = np.concatenate(x_c)[discard:]
        kB = clex.KB
        # heat capacity per site in units of kB: N * Var(e) / (kB T)^2, with the precision of
        # the mean of its per-pass terms N (e - <e>)^2 / (kB T)^2
        cv = n * float(np.var(e)) / (kB * T) ** 2
        cv_terms = _stats(n * (e - e.mean()) ** 2 / (kB * T) ** 2)
        series[prec] = e
        result[prec] = {
            "E_per_site": _stats(e), "x_B": _stats(xb), "x_C": _stats(xc), "Cv_per_site_kB": cv,
            "Cv_precision": cv_terms["precision"],
            "acceptance": n_acc / (n * n_passes), "fp64_redecisions": n_exact,
            "fp32_flipped_decisions": n_flip, "recompute_mismatches": mismatches,
            "kernel_s": kernel_ms * 1e-3, "site_attempts_per_s": n * n_passes / (kernel_ms * 1e-3),
            "ctas_per_chain": b.ctas_per_chain,
        }
        b.close()
    d64, d32 = result["fp64"], result["fp32"]
    result["fp32_minus_fp64"] = {
        k: {"diff": d32[k]["mean"] - d64[k]["mean"],
            "combined_error_bar": (d32[k]["precision"] ** 2 + d64[k]["precision"] ** 2) ** 0.5}
        for k in ("E_per_site", "x_B", "x_C")}
    result["fp32_minus_fp64"]["Cv_rel"] = d32["Cv_per_site_kB"] / d64["Cv_per_site_kB"] - 1.0
    result["fp32_minus_fp64"]["Cv"] = {"diff": d32["Cv_per_site_kB"] - d64["Cv_per_site_kB"],
                                       "combined_error_bar": (d32["Cv_precision"] ** 2 + d64["Cv_precision"] ** 2) ** 0.5}
    return result


def run_serving(n_jobs: int = 20000, rate: float = 200.0, plain_sample: int = 100, precision: str = "fp32",
                arena_gb: float = 16.0, seed: int = 0) -> dict:
    """Poisson stream of binary/ternary FCC jobs (L in 16..128, budget 100..5000 passes,
    convergence to 1e-4 eV/site) served with continuous batching; compared with the same
    kind of jobs run one at a time (one launch per chunk per job) on a sample."""
    from . import serving

    models = {k: clex.ClexModel(k, clex.make_eci(k, 1)) for k in ("fcc_binary", "fcc_ternary")}
    jobs = serving.poisson_jobs(n_jobs, rate, models, seed=seed)
    eng = serving.ServingEngine(models, arena_bytes=int(arena_gb * (1 << 30)), max_chains=4096, precision=precision)
    t_prep = eng.prepare(sorted({j.L for j in jobs}))
    st = eng.run(jobs, realtime=True)
    served = st.summary()
    served["geometry_prepare_s"] = t_prep
    plain_jobs = serving.poisson_jobs(plain_sample, rate, models, seed=seed + 1)
    pst = serving.run_plain(plain_jobs, models, precision=precision, prepare=True)
    plain = pst.summary()
    return {"workload": "serving_fcc_ce_poisson", "n_jobs": n_jobs, "rate_per_s": rate, "precision": precision,
            "served": served, "plain_one_job_at_a_time": plain,
            "converged_jobs_per_s_ratio": served["converged_jobs_per_s"] / max(plain["converged_jobs_per_s"], 1e-12),
            "mean_passes": float(np.mean([j.n_pass for j in st.jobs])) if st.jobs else 0.0}


def run_sweep(kind: str = "fcc_ternary", L: int = 64, n_chains: int = 8, n_passes: int = 20,
              layout: str = "auto", seed: int = 4) -> dict:
    import torch

    model = clex.ClexModel(kind, clex.make_eci(kind, seed))
    rng = np.random.default_rng(1)
    occ = np.stack([clex.random_occupation(model.n_species, L**3, rng) for _ in range(n_chains)])
    T = np.linspace(600.0, 1500.0, n_chains)
    mu = np.zeros((n_chains, model.n_species - 1))
    seeds = np.arange(1, n_chains + 1, dtype=np.uint64)
    b = clex.ChainBatch(model, (L, L, L), occ, T, mu, seeds)
    if layout != "auto":
        b.set_layout(layout)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    b.run(3, want_output=False)
    ms = []
    for _ in range(3):
        flush.add_(1)  # 256 MB written: L2 flushed
        torch.cuda.synchronize()
        b.run(n_passes, want_output=False)
        ms.append(b.last_kernel_ms())
    m = float(np.median(ms))
    r = {"workload": f"sweep_{kind}_{L}^3_x{n_chains}", "layout": b.layout, "ctas_per_chain": b.ctas_per_chain,
         "threads": b.threads, "colors": b.n_colors, "passes": n_passes, "ms": ms,
         "us_per_pass": 1e3 * m / n_passes, "site_attempts_per_s": n_chains * L**3 * n_passes / (m * 1e-3)}
    b.close()
    return r


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=["batched", "precision", "serving", "sweep"])
    ap.add_argument("--kind", default="fcc_ternary", choices=["fcc_binary", "fcc_ternary"])
    ap.add_argument("--L", type=int, default=64)
    ap.add_argument("--layout", default="auto", choices=["auto", "byte", "word", "word_pipelined",
                                                         "word_specialised", "grid"])
    ap.add_argument("--jobs", type=int, default=20000)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--chains", type=int, default=4096)
    ap.add_argument("--passes", type=int, default=500)
    ap.add_argument("--plain-sample", type=int, default=64)
    ap.add_argument("--precision", default="fp64")
    a = ap.parse_args(argv)
    if a.workload == "batched":
        r = run_batched(a.chains, a.passes, a.plain_sample, a.precision)
    elif a.workload == "precision":
        r = run_precision(n_passes=a.passes if a.passes != 500 else 5000)
    elif a.workload == "serving":
        r = run_serving(a.jobs, a.rate, a.plain_sample, precision="fp32" if a.precision == "fp64" else a.precision)
    elif a.workload == "sweep":
        r = run_sweep(a.kind, a.L, a.chains if a.chains != 4096 else 8, a.passes if a.passes != 500 else 20, a.layout)
    print(json.dumps(r), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
