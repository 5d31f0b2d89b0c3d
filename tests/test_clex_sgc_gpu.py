"""The cluster-expansion semi-grand canonical calculator (the reference's calculator
interface, basic_semigrand_canonical.hh:324-470, with the CE model as its system) on the
GPU: a run to convergence by the reference's completion check whose averages agree with the
reference's dynamics in the oracle; exact default samples; custom sampling functions that
read the host state; determinism from the caller's engine; per-state queries."""
import numpy as np
import pytest

import casmcode_monte_gb300 as monte
import casmcode_monte_gb300.clex as clex
import casmcode_monte_gb300.clex.semigrand_canonical as sgc
import casmcode_monte_gb300.sampling as sampling
from casmcode_monte_gb300.sampling import BasicStatisticsCalculator
from tests.oracle_lib import OracleCE

pytestmark = pytest.mark.gpu


def _setup(kind="fcc_binary", L=(8, 8, 8), T=1200.0, mu=(0.02,), seed=3):
    model = clex.ClexModel(kind, clex.make_eci(kind, 3))
    calc = sgc.SemiGrandCanonicalCalculator(sgc.ClexSystem(sgc.ClexFormationEnergy(model),
                                                           sgc.ClexParamComposition(model)))
    n = L[0] * L[1] * L[2]
    occ = clex.random_occupation(model.n_species, n, np.random.default_rng(seed))
    state = sgc.ClexState(sgc.ClexConfiguration(L, occ),
                          monte.ValueMap.from_dict({"temperature": T, "exchange_potential": list(mu)}))
    return model, calc, state, occ


def _params(max_count=None, reqs=(), min_sample=100, check_begin=100, check_period=100):
    p = sampling.CompletionCheckParams()
    p.cutoff_params.min_sample = min_sample
    p.cutoff_params.max_count = max_count
    p.log_spacing = False
    p.check_begin = check_begin
    p.check_period = check_period
    return p


def _quiet(c, log):
    pass


def test_run_to_convergence_matches_reference_dynamics(gpu_lib, tmp_path):
    model, calc, state, occ0 = _setup()
    sf = calc.default_sampling_functions()
    p = _params()
    sampling.converge(sf, p).set_precision("potential_energy", abs=2e-4)
    engine = monte.RandomNumberEngine()
    engine.seed(5)
    calc.run(state, sf, {}, p, sgc.SemiGrandCanonicalEventGenerator(), sample_period=1,
             method_log=monte.MethodLog(str(tmp_path / "status.json"), log_frequency=None), random_engine=engine,
             write_status_f=_quiet)
    r = calc.data.completion_check.results()
    assert r.is_complete and r.convergence_check_results.all_converged
    e = calc.data.samplers["potential_energy"].component(0)
    assert e.size == calc.data.n_pass >= 100
    assert calc.data.n_accept + calc.data.n_reject == calc.data.n_pass * 512
    # the final state is the chain's, and the last sample is its potential energy
    assert np.isclose(calc.potential.per_unitcell(), e[-1], rtol=0, atol=1e-12)
    # averages over the equilibrated part against the reference's random-site dynamics
    n_eq = r.equilibration_check_results.N_samples_for_all_to_equilibrate
    orc = OracleCE((8, 8, 8), 2, model.eci)
    e_ref, _, _ = orc.sgc_samples(occ0, 1200.0, np.array([0.02]), 777, 6000)
    e_ref = e_ref[1000:]
    sg = BasicStatisticsCalculator(confidence=0.95)(np.ascontiguousarray(e[n_eq:]))
    sr = BasicStatisticsCalculator(confidence=0.95)(np.ascontiguousarray(e_ref))
    assert abs(sg.mean - sr.mean) <= 2.0 * np.hypot(sg.calculated_precision, sr.calculated_precision)


def test_custom_sampling_function_and_determinism(gpu_lib, tmp_path):
    runs = []
    for _ in range(2):
        model, calc, state, _ = _setup(T=900.0)
        sf = calc.default_sampling_functions()
        sf["x_host"] = sampling.StateSamplingFunction(
            "x_host", "B fraction read from the host state", [1],
            lambda st=state: np.array([np.count_nonzero(st.configuration.occupation() == 1) / 512.0]))
        engine = monte.RandomNumberEngine()
        engine.seed(11)
        calc.run(state, sf, calc.default_json_sampling_functions(), _params(max_count=40, min_sample=None), None,
                 sample_period=3,
                 method_log=monte.MethodLog(str(tmp_path / "s.json"), log_frequency=None), random_engine=engine,
                 write_status_f=_quiet)
        d = calc.data
        assert d.n_pass == 40 and d.samplers["x_host"].n_samples() == 13
        assert np.array_equal(d.samplers["x_host"].component(0), d.samplers["param_composition"].component(0))
        assert len(d.json_samplers["configuration"].values) == 13
        # samples at passes 3, 6, ..., 39: the B fraction of each JSON configuration is the
        # sampled composition
        xs = [np.count_nonzero(np.asarray(c["occupation"]) == 1) / 512.0 for c in d.json_samplers["configuration"].values]
        assert np.array_equal(np.asarray(xs), d.samplers["param_composition"].component(0))
        runs.append((d.samplers["potential_energy"].component(0).copy(), state.configuration.occupation().copy(),
                     engine.dump()))
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])
    assert runs[0][2] == runs[1][2]


def test_ternary_run_and_state_queries(gpu_lib, tmp_path):
    model, calc, state, _ = _setup("fcc_ternary", T=1500.0, mu=(0.02, -0.01))
    sf = calc.default_sampling_functions()
    engine = monte.RandomNumberEngine()
    engine.seed(2)
    calc.run(state, sf, {}, _params(max_count=60, min_sample=None), None, sample_period=1,
             method_log=monte.MethodLog(str(tmp_path / "t.json"), log_frequency=None), random_engine=engine,
             write_status_f=_quiet)
    pe = calc.data.samplers["potential_energy"].component(0)
    assert pe.size == 60
    # the device's tracked sums against a recompute from the final occupation
    assert calc.potential.per_unitcell() == pe[-1]
    x = calc.data.samplers["param_composition"]
    assert np.allclose(np.array([x.component(0)[-1], x.component(1)[-1]]),
                       calc.param_composition_calculator.per_unitcell(), rtol=0, atol=1e-15)
    # energy changes of one and two sites against differences of energies
    fe = calc.formation_energy_calculator
    e0 = fe.per_supercell()
    cfg = state.configuration
    l1, l2 = 5, 77
    n1, n2 = (cfg.occ(l1) + 1) % 3, (cfg.occ(l2) + 2) % 3
    d2 = fe.occ_delta_per_supercell([l1, l2], [n1, n2])
    cfg.set_occ(l1, n1)
    cfg.set_occ(l2, n2)
    assert abs((fe.per_supercell() - e0) - d2) <= 1e-10 * max(1.0, abs(e0))


def test_run_fixtures_with_run_manager(gpu_lib, tmp_path):
    """GPU sweeps driven by the reference's run management: a converging fixture with its
    results files and a second fixture with a count cutoff (all fixtures must complete)."""
    import json

    import casmcode_monte_gb300.run_management as rm

    model, calc, state, _ = _setup(T=1200.0)
    fmap = calc.default_sampling_functions()
    fmap["pe_tracked"] = sampling.StateSamplingFunction(
        "pe_tracked", "tracked potential energy per unit cell", [],
        lambda: np.array([state.properties.scalar_values["potential_energy"]]))
    cc = _params()
    sampling.converge(fmap, cc).set_precision("pe_tracked", abs=3e-4)
    thermo = rm.SamplingFixtureParams(
        "thermo", fmap, {}, {}, rm.SamplingParams(sampler_names=["pe_tracked", "potential_energy", "param_composition"]),
        cc, results_io=rm.jsonResultsIO(str(tmp_path / "thermo"), write_observations=True))
    cc2 = _params(max_count=150, min_sample=None)
    traj = rm.SamplingFixtureParams(
        "traj", fmap, {}, {}, rm.SamplingParams(sampler_names=["param_composition"], period=10.0, begin=10.0,
                                               do_sample_trajectory=True),
        cc2, results_io=rm.jsonResultsIO(str(tmp_path / "traj"), write_trajectory=True))
    engine = monte.RandomNumberEngine()
    engine.seed(8)
    manager = rm.RunManager(engine, [thermo, traj], global_cutoff=False)
    calc.run_fixtures(state, manager)
    t, tr = manager.sampling_fixtures
    assert t.completion_check_results().convergence_check_results.all_converged
    assert tr.counter().count >= 150 and tr.results().sample_count[:3] == [10, 20, 30]
    rt = t.results()
    # the tracked energy is the device's exact sums; the default function recomputes it
    assert np.allclose(rt.samplers["pe_tracked"].component(0), rt.samplers["potential_energy"].component(0),
                       rtol=0, atol=1e-12)
    assert rt.n_accept + rt.n_reject == 512 * t.counter().count
    with open(tmp_path / "thermo" / "summary.json") as f:
        summary = json.load(f)
    assert summary["completion_check_results"]["all_converged"] == [True]
    assert summary["statistics"]["pe_tracked"]["value"]["is_converged"] == [True]
    with open(tmp_path / "traj" / "run.0" / "trajectory.json") as f:
        assert len(json.load(f)) == len(tr.results().sample_count)
