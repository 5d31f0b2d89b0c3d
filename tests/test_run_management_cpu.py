"""Run management (include/casm/monte/run_management, sampling/SamplingParams.hh) and the
generic occupation Metropolis loop (methods/occupation_metropolis.hh:90-154): sampling
schedules, counters, and a run whose trajectory is the oracle's run of the reference's
semi-grand canonical dynamics (OccLocation proposals, the same random numbers), with the
reference's JSON results files."""
import json
import math
import os

import numpy as np
import pytest

import casmcode_monte_gb300 as monte
import casmcode_monte_gb300.clex.semigrand_canonical as csgc
import casmcode_monte_gb300.events as ev
import casmcode_monte_gb300.methods as methods
import casmcode_monte_gb300.run_management as rm
import casmcode_monte_gb300.sampling as sampling
from tests import oracle_lib


def test_sample_at_schedules():
    s = rm.SamplingParams()
    assert [rm.sample_at(i, s) for i in range(3)] == [1.0, 2.0, 3.0]
    s = rm.SamplingParams(sample_method=sampling.SAMPLE_METHOD.LOG, begin=0.0, base=2.0, shift=1.0)
    assert [rm.sample_at(i, s) for i in range(3)] == [2.0, 4.0, 8.0]
    s = rm.SamplingParams(sample_method=sampling.SAMPLE_METHOD.CUSTOM, custom_sample_at=lambda n: 5.0 * n * n)
    assert rm.sample_at(3, s) == 45.0
    with pytest.raises(RuntimeError):
        rm.sample_at(0, rm.SamplingParams(sample_method=sampling.SAMPLE_METHOD.CUSTOM))
    # stochastic interval: the number of trials to the first success of probability rate
    engine = monte.RandomNumberEngine()
    engine.seed(3)
    rng = monte.RandomNumberGenerator(engine)
    steps = [rm.stochastic_count_step(0.25, rng) for _ in range(4000)]
    assert min(steps) >= 1 and abs(np.mean(steps) - 4.0) < 0.3


def test_counter_by_step_and_by_pass():
    c = rm.MonteCounter()
    c.reset(sampling.SAMPLE_MODE.BY_PASS, 3)
    for _ in range(7):
        c.increment_step()
    assert (c.step, c.pass_count, c.count) == (1, 2, 2)
    c.reset(sampling.SAMPLE_MODE.BY_STEP, 3)
    for _ in range(7):
        c.increment_step()
    assert (c.step, c.pass_count, c.count) == (1, 2, 7)


class OraclePotential:
    """Semi-grand canonical potential of the oracle's cluster expansion (test support)."""

    def __init__(self, orc, state, mu):
        self.orc, self.state, self.mu = orc, state, np.asarray(mu, dtype=float)

    def per_supercell(self) -> float:
        occ = self.state.configuration.occupation().astype(np.int32)
        return self.orc.formation(occ) - float(self.mu[0]) * float(np.count_nonzero(occ == 1))

    def occ_delta_per_supercell(self, sites, new_occ) -> float:
        occ = self.state.configuration.occupation().astype(np.int32)
        return self.orc.delta_e(occ, int(sites[0]), int(new_occ[0]), self.mu)


def _run(tmp_path, state, orc, mu, seed, n_pass, run_index):
    convert = ev.Conversions(ev.Prim.fcc(4.0, ["A", "B"]), np.eye(3, dtype=int) * 4)
    cands = ev.OccCandidateList(convert)
    swaps = ev.make_semigrand_canonical_swaps(convert, cands)
    loc = ev.OccLocation(convert, cands)
    loc.initialize(state.configuration.occupation().copy())
    fmap = sampling.StateSamplingFunctionMap()
    fmap["potential_energy"] = sampling.StateSamplingFunction(
        "potential_energy", "", [], lambda: np.array([state.properties.scalar_values["potential_energy"]]))
    fmap["x"] = sampling.StateSamplingFunction(
        "x", "B fraction", [1], lambda: np.array([np.count_nonzero(state.configuration.occupation() == 1) / 64.0]))
    jmap = sampling.jsonStateSamplingFunctionMap()
    cc = sampling.CompletionCheckParams()
    cc.cutoff_params.max_count = n_pass
    sp = rm.SamplingParams(sampler_names=["potential_energy", "x"], do_sample_trajectory=True)
    io = rm.jsonResultsIO(str(tmp_path / "results"), write_trajectory=True, write_observations=True)
    fx = rm.SamplingFixtureParams("thermo", fmap, jmap, {}, sp, cc, results_io=io,
                                  method_log=monte.MethodLog(str(tmp_path / "status.json"), None))
    engine = monte.RandomNumberEngine()
    engine.seed(seed)
    manager = rm.RunManager(engine, [fx])
    manager.run_index = run_index
    potential = OraclePotential(orc, state, mu)
    methods.occupation_metropolis(state, loc, potential, swaps, ev.propose_semigrand_canonical_event,
                                  monte.RandomNumberGenerator(engine), manager)
    return manager.sampling_fixtures[0]


def test_occupation_metropolis_matches_reference_dynamics_and_writes_results(tmp_path):
    from casmcode_monte_gb300 import clex

    eci = clex.make_eci("fcc_binary", 4)
    orc = oracle_lib.OracleCE((4, 4, 4), 2, eci)
    occ0 = np.random.default_rng(9).integers(0, 2, size=64).astype(np.int8)
    T, mu, n_pass = 1500.0, [0.02], 30
    for run_index, seed in ((0, 41), (1, 42)):
        state = csgc.ClexState(csgc.ClexConfiguration((4, 4, 4), occ0),
                               monte.ValueMap.from_dict({"temperature": T, "exchange_potential": mu}))
        fx = _run(tmp_path, state, orc, mu, seed, n_pass, run_index)
        e_ref, x_ref, nacc = orc.sgc_samples(occ0.astype(np.int32), T, np.array(mu), seed, n_pass)
        r = fx.results()
        assert r.sample_count == list(range(1, n_pass + 1))
        assert r.n_accept == nacc and r.n_accept + r.n_reject == 64 * n_pass
        assert np.allclose(r.samplers["potential_energy"].component(0), e_ref, rtol=0, atol=1e-12)
        assert np.array_equal(r.samplers["x"].component(0), x_ref[:, 0])
    # results files: one summary entry per run, observations and trajectory per run
    with open(tmp_path / "results" / "summary.json") as f:
        summary = json.load(f)
    assert summary["conditions"]["temperature"] == {"shape": [], "value": [T, T]}
    assert summary["conditions"]["exchange_potential"]["0"] == [0.02, 0.02]
    st = summary["statistics"]["potential_energy"]
    assert st["shape"] == [] and len(st["value"]["mean"]) == 2 and len(st["value"]["calculated_precision"]) == 2
    assert summary["statistics"]["x"]["component_names"] == ["0"]
    ccr = summary["completion_check_results"]
    assert ccr["N_samples"] == [n_pass, n_pass] and ccr["count"] == [n_pass, n_pass]
    assert "all_converged" not in ccr  # no requested precision
    with open(tmp_path / "results" / "run.1" / "observations.json") as f:
        obs = json.load(f)
    assert obs["count"] == list(range(1, n_pass + 1))
    assert np.allclose(obs["potential_energy"]["value"], r.samplers["potential_energy"].component(0))
    with open(tmp_path / "results" / "run.1" / "trajectory.json") as f:
        traj = json.load(f)
    assert len(traj) == n_pass and traj[-1]["occupation"] == [int(v) for v in state.configuration.occupation()]
    assert os.path.exists(tmp_path / "status.json")


def test_global_cutoff_and_break_points(tmp_path):
    """Two fixtures: with global_cutoff the run ends when the first completes."""
    fmap = sampling.StateSamplingFunctionMap()
    fmap["c"] = sampling.StateSamplingFunction("c", "", [], lambda: np.array([1.0]))
    fixtures = []
    for label, max_count in (("short", 5), ("long", 50)):
        cc = sampling.CompletionCheckParams()
        cc.cutoff_params.max_count = max_count
        fixtures.append(rm.SamplingFixtureParams(label, fmap, {}, {}, rm.SamplingParams(sampler_names=["c"]), cc))
    for global_cutoff, expect in ((True, 5), (False, 50)):
        m = rm.RunManager(monte.RandomNumberEngine(), fixtures, global_cutoff=global_cutoff)
        hits = []
        m.break_point_checks["short"] = lambda f, s: hits.append(f.counter().count) or f.counter().count == 3
        m.initialize(2)
        steps = 0
        while not m.is_complete():
            m.increment_step()
            steps += 1
            m.sample_data_by_count_if_due(None)
        assert m.sampling_fixtures[0].counter().count == expect and steps == 2 * expect
        assert hits[:3] == [1, 2, 3]
