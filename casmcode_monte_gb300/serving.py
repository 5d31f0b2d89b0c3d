"""Serving loop: continuous batching of semi-grand canonical Monte Carlo jobs on one GPU.

A job is one run of the reference's semi-grand canonical calculator (one thermodynamic
state of one supercell, ``SemiGrandCanonicalCalculator.run`` in
include/casm/monte/ising_cpp/basic_semigrand_canonical.hh:416-470) on an FCC cluster
expansion: supercell L^3, temperature, exchange potential, a pass budget (the completion
check's ``max_count``) and a requested absolute precision of the potential energy per
site.  The engine

* admits arriving jobs into chain pools (binary and ternary) while their occupation fits
  in the pool's HBM arena and a slot is free (jobs wait in arrival order otherwise);
* advances every admitted job by one chunk of passes per tick in one launch per pool
  (jobs that arrive while others run join at the next tick: continuous batching);
* keeps occupation, Philox pass counters, integer correlation sums and the per-pass
  potential-energy series on the device between ticks;
* runs the reference's completion rule: a convergence check (equilibration, then the
  autocorrelation-corrected precision of the mean, on the device) whenever the number of
  samples reaches check_begin + check_period * n (CompletionCheck.hh:57-67, linear
  spacing), completion when converged or when the pass budget is reached;
* records, per job, arrival, start and finish times and the converged statistics.

Because each chain's random numbers depend only on (seed, chain id, pass), a job's result
is identical whether it runs alone or mixed with others.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import clex


@dataclass
class Job:
    id: int
    kind: str
    L: int
    temperature: float
    mu: np.ndarray
    pass_budget: int
    abs_precision: float
    seed: int
    occ: Optional[np.ndarray] = None  # None: drawn from the seed at admission
    arrival: float = 0.0
    # results
    start: Optional[float] = None
    finish: Optional[float] = None
    n_pass: int = 0
    converged: bool = False
    equilibrated: bool = False
    n_equilibration: int = 0
    mean: float = float("nan")
    precision: float = float("inf")
    slot: int = -1
    n_checks: int = 0
    final_occ: Optional[np.ndarray] = None

    def initial_occupation(self, n_species: int) -> np.ndarray:
        if self.occ is not None:
            return self.occ
        rng = np.random.default_rng([self.seed, self.id])
        return rng.integers(0, n_species, size=self.L**3).astype(np.int8)

    @property
    def latency(self) -> float:
        return self.finish - self.arrival


@dataclass
class ServingStats:
    jobs: list = field(default_factory=list)
    wall_s: float = 0.0
    ticks: int = 0
    gpu_ms: float = 0.0
    site_attempts: int = 0

    def summary(self) -> dict:
        lat = np.array([j.latency for j in self.jobs]) if self.jobs else np.zeros(1)
        conv = sum(1 for j in self.jobs if j.converged)
        return {
            "jobs": len(self.jobs), "converged_jobs": conv, "wall_s": self.wall_s,
            "jobs_per_s": len(self.jobs) / self.wall_s if self.wall_s else 0.0,
            "converged_jobs_per_s": conv / self.wall_s if self.wall_s else 0.0,
            "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
            "latency_max_s": float(lat.max()), "ticks": self.ticks, "gpu_s": self.gpu_ms * 1e-3,
            "site_attempts": self.site_attempts,
            "site_attempts_per_s": self.site_attempts / self.wall_s if self.wall_s else 0.0,
        }


class ServingEngine:
    """Continuous-batching engine over one chain pool per basis set."""

    def __init__(self, models: dict, arena_bytes: int = 8 << 30, max_chains: int = 2048, chunk: int = 100,
                 max_passes: int = 5000, precision: str = "fp32", check_begin: int = 100, check_period: int = 100,
                 confidence: float = 0.95, keep_occupation: bool = False):
        self.models = models
        self.keep_occupation = keep_occupation
        self.chunk = int(chunk)
        self.check_begin = int(check_begin)
        self.check_period = int(check_period)
        self.confidence = float(confidence)
        self.pools = {}
        for kind, model in models.items():
            pool = clex.ChainPool(model, arena_bytes=arena_bytes // len(models), max_chains=max_chains,
                                  precision=precision)
            pool.enable_series(max_passes)
            self.pools[kind] = pool
        self.queue: list[Job] = []
        self.active: dict = {k: [] for k in models}
        self.stats = ServingStats()

    def submit(self, job: Job) -> None:
        self.queue.append(job)

    def prepare(self, L_values) -> float:
        """Build the geometry of every cubic supercell L^3 in ``L_values`` for every pool
        (done once per shape; a server keeps them across jobs).  Returns seconds taken."""
        t0 = time.perf_counter()
        for pool in self.pools.values():
            for L in L_values:
                pool.prepare((L, L, L))
        return time.perf_counter() - t0

    def _admit(self, now: float) -> None:
        while self.queue and self.queue[0].arrival <= now:
            job = self.queue[0]
            pool = self.pools[job.kind]
            try:
                occ = job.initial_occupation(self.models[job.kind].n_species)
                job.slot = pool.add((job.L,) * 3, occ, job.temperature, job.mu, job.seed, job.id)
            except clex.PoolFull:
                return  # wait for memory/slots to free up (arrival order is kept)
            job.start = time.perf_counter() - self._t0
            self.active[job.kind].append(job)
            self.queue.pop(0)

    def _check_due(self, job: Job) -> bool:
        return job.n_pass >= self.check_begin + self.check_period * job.n_checks

    def tick(self) -> int:
        """Advance every active job by one chunk; returns the number of active jobs."""
        n_active = 0
        for kind, jobs in self.active.items():
            if not jobs:
                continue
            pool = self.pools[kind]
            n_active += len(jobs)
            groups: dict = {}
            for j in jobs:
                p = min(self.chunk, j.pass_budget - j.n_pass)
                groups.setdefault(p, []).append(j)
            for p, js in groups.items():
                pool.run([j.slot for j in js], p, want_output=False)
                self.stats.gpu_ms += pool.last_kernel_ms()
                for j in js:
                    j.n_pass += p
                    self.stats.site_attempts += p * j.L**3
            due = [j for j in jobs if self._check_due(j) or j.n_pass >= j.pass_budget]
            done = []
            if due:
                # one device check per distinct precision request
                by_prec: dict = {}
                for j in due:
                    by_prec.setdefault(j.abs_precision, []).append(j)
                for prec, js in by_prec.items():
                    res = pool.check([j.slot for j in js], prec, self.confidence)
                    for j, r in zip(js, res):
                        if self._check_due(j):
                            j.n_checks += 1
                        j.equilibrated = bool(r[0])
                        j.n_equilibration = int(r[1])
                        j.mean = float(r[3])
                        j.precision = float(r[4])
                        j.converged = bool(r[5])
                        if j.converged or j.n_pass >= j.pass_budget:
                            done.append(j)
            now = time.perf_counter() - self._t0
            for j in done:
                j.finish = now
                if self.keep_occupation:
                    j.final_occ = pool.occupation(j.slot)
                pool.remove(j.slot)
                jobs.remove(j)
                self.stats.jobs.append(j)
        self.stats.ticks += 1
        return n_active

    def run(self, jobs: list, realtime: bool = True, timeout_s: float = 1e9) -> ServingStats:
        """Serve ``jobs`` (sorted by arrival time, seconds from start)."""
        for j in sorted(jobs, key=lambda j: j.arrival):
            self.submit(j)
        total = len(jobs)
        self._t0 = time.perf_counter()
        while len(self.stats.jobs) < total:
            elapsed = time.perf_counter() - self._t0
            if elapsed > timeout_s:
                break
            now = elapsed if realtime else float("inf")
            self._admit(now)
            n = self.tick()
            if n == 0 and self.queue:
                wait = self.queue[0].arrival - (time.perf_counter() - self._t0)
                if wait > 0:
                    time.sleep(min(wait, 0.01))
        self.stats.wall_s = time.perf_counter() - self._t0
        return self.stats


def poisson_jobs(n_jobs: int, rate: float, models: dict, seed: int = 0, L_range=(16, 128), budget=(100, 5000),
                 abs_precision: float = 1e-4) -> list:
    """Synthetic job stream: Poisson arrivals, binary or ternary CE, L uniform, random T and mu."""
    rng = np.random.default_rng(seed)
    t = 0.0
    jobs = []
    kinds = sorted(models)
    for i in range(n_jobs):
        t += rng.exponential(1.0 / rate)
        kind = kinds[int(rng.integers(0, len(kinds)))]
        ns = models[kind].n_species
        L = int(rng.integers(L_range[0], L_range[1] + 1))
        jobs.append(Job(id=i, kind=kind, L=L, temperature=float(rng.uniform(300.0, 2000.0)),
                        mu=rng.uniform(-0.3, 0.3, size=ns - 1), pass_budget=int(rng.integers(budget[0], budget[1] + 1)),
                        abs_precision=abs_precision, seed=int(rng.integers(1, 2**63)), arrival=t))
    return jobs


def run_plain(jobs: list, models: dict, chunk: int = 100, check_begin: int = 100, check_period: int = 100,
              confidence: float = 0.95, precision: str = "fp32", prepare: bool = False) -> ServingStats:
    """Baseline: the same jobs one at a time, one launch per chunk per job (no batching).

    With ``prepare`` each job's geometry is built before the clock starts, as the served
    engine's is."""
    stats = ServingStats()
    pools = []
    for job in jobs:
        pool = clex.ChainPool(models[job.kind], arena_bytes=job.L**3 + 64, max_chains=1, precision=precision)
        pool.enable_series(job.pass_budget)
        if prepare:
            pool.prepare((job.L,) * 3)
        pools.append(pool)
    t0 = time.perf_counter()
    for job, pool in zip(jobs, pools):
        slot = pool.add((job.L,) * 3, job.initial_occupation(models[job.kind].n_species), job.temperature, job.mu,
                        job.seed, job.id)
        job.start = time.perf_counter() - t0
        while True:
            p = min(chunk, job.pass_budget - job.n_pass)
            pool.run([slot], p, want_output=False)
            stats.gpu_ms += pool.last_kernel_ms()
            stats.site_attempts += p * job.L**3
            job.n_pass += p
            due = job.n_pass >= check_begin + check_period * job.n_checks
            if due or job.n_pass >= job.pass_budget:
                r = pool.check([slot], job.abs_precision, confidence)[0]
                if due:
                    job.n_checks += 1
                job.equilibrated, job.n_equilibration = bool(r[0]), int(r[1])
                job.mean, job.precision, job.converged = float(r[3]), float(r[4]), bool(r[5])
                if job.converged or job.n_pass >= job.pass_budget:
                    break
        job.finish = time.perf_counter() - t0
        job.arrival = job.start
        stats.jobs.append(job)
        pool.remove(slot)
    stats.wall_s = time.perf_counter() - t0
    for pool in pools:
        pool.close()
    return stats
