"""GPU serial replay of the reference's Ising semi-grand canonical run: bit-exact
against the oracle (occupations, every sample, counters, final engine state), plus the
reference's own convergence scenario (python/tests/ising_cpp/
test_ising_semigrand_canonical_cpp.py:12-100)."""
import json

import numpy as np
import pytest

import casmcode_monte_gb300 as monte
import casmcode_monte_gb300.ising_cpp as ising
import casmcode_monte_gb300.ising_cpp.semigrand_canonical as sgc
import casmcode_monte_gb300.sampling as sampling
from tests import oracle_lib

pytestmark = pytest.mark.gpu


def _make(J=0.1, use_nlist=True, shape=(25, 25), T=2000.0, mu=0.0, occ=None):
    calc = sgc.SemiGrandCanonicalCalculator(
        system=ising.IsingSystem(
            formation_energy_calculator=ising.IsingFormationEnergy(J=J, lattice_type=1, use_nlist=use_nlist),
            param_composition_calculator=ising.IsingParamComposition(),
        )
    )
    state = ising.IsingState(
        configuration=ising.IsingConfiguration(shape=shape),
        conditions=monte.ValueMap.from_dict({"temperature": T, "exchange_potential": [mu]}),
    )
    if occ is not None:
        state.configuration.set_occupation(occ)
    return calc, state


def _params(min_sample=None, max_sample=None, max_count=None, check_begin=100, check_period=10, reqs=()):
    p = sampling.CompletionCheckParams()
    p.cutoff_params.min_sample = min_sample
    p.cutoff_params.max_sample = max_sample
    p.cutoff_params.max_count = max_count
    p.log_spacing = False
    p.check_begin = check_begin
    p.check_period = check_period
    return p


def _quiet(calc, log):
    pass


@pytest.mark.parametrize("use_nlist", [True, False])
@pytest.mark.parametrize("seed,T,mu,shape,occ_seed", [(1, 2000.0, 0.0, (25, 25), 1), (7, 1500.0, 0.05, (16, 12), 3),
                                                        (11, 800.0, -0.1, (9, 13), 5)])
def test_replay_fixed_passes_bit_exact(gpu_lib, tmp_path, use_nlist, seed, T, mu, shape, occ_seed):
    rng = np.random.default_rng(occ_seed)
    N = shape[0] * shape[1]
    occ = rng.choice(np.array([-1, 1], dtype=np.int32), size=N)
    calc, state = _make(use_nlist=use_nlist, shape=shape, T=T, mu=mu, occ=occ)
    p = _params(max_count=1000)
    engine = monte.RandomNumberEngine()
    engine.seed(seed)
    state0 = engine.dump()
    sf = calc.default_sampling_functions()
    log = monte.MethodLog(str(tmp_path / "status.json"), log_frequency=None)
    calc.run(state, sf, {}, p, sgc.SemiGrandCanonicalEventGenerator(), sample_period=1, method_log=log,
             random_engine=engine, write_status_f=_quiet)
    ref = oracle_lib.ising_run(shape[0], shape[1], 0.1, use_nlist, T, mu, occ,
                               oracle_lib.make_cc_params(max_count=1000), 1, state0)
    assert ref["out"].n_pass == 1000
    assert np.array_equal(state.configuration.occupation(), ref["occ"])
    for name in ("formation_energy", "param_composition", "potential_energy"):
        got = calc.data.samplers[name].component(0)
        assert got.shape == ref[name].shape
        assert np.array_equal(got, ref[name]), name  # bit-exact FP64 samples
    assert calc.data.n_accept == ref["out"].n_accept
    assert calc.data.n_reject == ref["out"].n_reject
    assert engine.dump() == ref["engine"]


def test_replay_convergence_scenario_matches_oracle(gpu_lib, tmp_path):
    """The reference's test scenario (25x25, J=0.1, T=2000, mu=0, min_sample=100,
    linear checks begin=100 period=10, abs precision 0.001 on potential_energy and
    param_composition), with a seeded engine so that it can be compared with the oracle."""
    calc, state = _make()
    for l in range(state.configuration.n_sites):
        state.configuration.set_occ(l, 1)
    sf = calc.default_sampling_functions()
    jsf = calc.default_json_sampling_functions()
    p = _params(min_sample=100)
    sampling.converge(sf, p).set_precision("potential_energy", abs=0.001).set_precision("param_composition", abs=0.001)
    engine = monte.RandomNumberEngine()
    engine.seed(12345)
    state0 = engine.dump()
    log = monte.MethodLog(str(tmp_path / "status.json"), log_frequency=0.2)
    calc.run(state, sf, jsf, p, sgc.SemiGrandCanonicalEventGenerator(), sample_period=1, method_log=log,
             random_engine=engine, write_status_f=_quiet)
    results = calc.data.completion_check.results()
    # the reference test's own assertions
    assert sampling.get_n_samples(calc.data.samplers) >= 100
    assert results.is_complete
    assert results.equilibration_check_results.all_equilibrated
    assert len(results.equilibration_check_results.individual_results) == 2
    assert results.convergence_check_results.all_converged
    assert len(results.convergence_check_results.individual_results) == 2
    for key, req in p.requested_precision.items():
        assert results.convergence_check_results.individual_results[key].stats.calculated_precision < req.abs_precision
    # and exact agreement with the oracle run of the reference loop
    ref = oracle_lib.ising_run(25, 25, 0.1, True, 2000.0, 0.0, np.ones(625, dtype=np.int32),
                               oracle_lib.make_cc_params(min_sample=100, check_begin=100, check_period=10,
                                                         reqs=[(1, 0.001), (2, 0.001)]), 1, state0)
    assert calc.data.n_pass == ref["out"].n_pass
    assert sampling.get_n_samples(calc.data.samplers) == ref["out"].n_samples
    assert np.array_equal(state.configuration.occupation(), ref["occ"])
    assert np.array_equal(calc.data.samplers["potential_energy"].component(0), ref["potential_energy"])
    key_pe = sampling.SamplerComponent("potential_energy", 0, "0")
    st = results.convergence_check_results.individual_results[key_pe].stats
    assert st.mean == ref["out"].mean[1]
    assert st.calculated_precision == ref["out"].calculated_precision[1]
    assert engine.dump() == ref["engine"]
    # JSON configuration samples were taken every pass and the final one is the state
    assert len(calc.data.json_samplers["configuration"].values) == calc.data.n_pass
    assert calc.data.json_samplers["configuration"].values[-1]["occupation"] == state.configuration.occupation().tolist()
    json.dumps(results.to_dict())


def test_replay_sample_period_and_max_sample(gpu_lib, tmp_path):
    calc, state = _make(shape=(12, 10), T=1200.0, mu=0.02)
    p = _params(max_sample=37)
    engine = monte.RandomNumberEngine()
    engine.seed(99)
    state0 = engine.dump()
    log = monte.MethodLog(str(tmp_path / "s.json"), None)
    calc.run(state, calc.default_sampling_functions(), {}, p, sgc.SemiGrandCanonicalEventGenerator(),
             sample_period=3, method_log=log, random_engine=engine, write_status_f=_quiet)
    ref = oracle_lib.ising_run(12, 10, 0.1, True, 1200.0, 0.02, np.ones(120, dtype=np.int32),
                               oracle_lib.make_cc_params(max_sample=37), 3, state0)
    assert calc.data.n_pass == ref["out"].n_pass == 111
    assert np.array_equal(calc.data.samplers["formation_energy"].component(0), ref["formation_energy"])
    assert engine.dump() == ref["engine"]


def test_replay_custom_sampling_function_sees_state(gpu_lib, tmp_path):
    """Python sampling functions are called with the host state brought up to date
    (the reference calls them per sample, test_ising_cpp_custom_functions.py:121-225)."""
    calc, state = _make(shape=(10, 10))
    seen = []

    def magnetization():
        m = float(np.mean(state.configuration.occupation()))
        seen.append(m)
        return [m]

    sf = calc.default_sampling_functions()
    sf["m"] = sampling.StateSamplingFunction("m", "magnetization", [], magnetization)
    engine = monte.RandomNumberEngine()
    engine.seed(5)
    log = monte.MethodLog(str(tmp_path / "s.json"), None)
    calc.run(state, sf, {}, _params(max_count=20), sgc.SemiGrandCanonicalEventGenerator(), method_log=log,
             random_engine=engine, write_status_f=_quiet)
    x = calc.data.samplers["param_composition"].component(0)
    assert np.allclose(np.array(seen), 2.0 * x - 1.0, atol=1e-12)
