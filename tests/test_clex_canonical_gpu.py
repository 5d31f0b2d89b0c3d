"""The cluster-expansion canonical calculator (the calculator interface of the semi-grand
canonical module at fixed composition; the reference's canonical event made parallel) on the
GPU: a run by the reference's completion check keeps the composition, samples formation and
potential energy alike, follows the chain CanonicalBatch runs from the same Philox key (drawn
from the caller's engine), and converges to the averages of the reference's canonical
dynamics; the calculator also runs sampling fixtures of a RunManager."""
import numpy as np
import pytest

import casmcode_monte_gb300 as monte
import casmcode_monte_gb300.clex as clex
import casmcode_monte_gb300.clex.canonical as can
import casmcode_monte_gb300.run_management as rm
import casmcode_monte_gb300.sampling as sampling
from tests.oracle_lib import OracleCE

pytestmark = pytest.mark.gpu


def _setup(kind="fcc_binary", L=(8, 8, 8), T=1200.0, seed=3):
    model = clex.ClexModel(kind, clex.make_eci(kind, 3))
    calc = can.CanonicalCalculator(can.ClexSystem(can.ClexFormationEnergy(model), can.ClexParamComposition(model)))
    n = L[0] * L[1] * L[2]
    occ = clex.random_occupation(model.n_species, n, np.random.default_rng(seed))
    state = can.ClexState(can.ClexConfiguration(L, occ), monte.ValueMap.from_dict({"temperature": T}))
    return model, calc, state, occ


def _quiet(c, log):
    pass


def test_canonical_calculator_follows_the_batch(gpu_lib):
    model, calc, state, occ0 = _setup(kind="fcc_ternary")
    p = sampling.CompletionCheckParams()
    p.cutoff_params.max_count = 150
    engine = monte.RandomNumberEngine()
    engine.seed(5)
    st0 = engine.dump()
    data = calc.run(state, calc.default_sampling_functions(), {}, p, method_log=monte.MethodLog(None, None),
                    random_engine=engine, write_status_f=_quiet)
    assert data.n_pass == 150
    final = state.configuration.occupation()
    assert np.array_equal(np.bincount(final, minlength=3), np.bincount(occ0, minlength=3))
    x = data.samplers["param_composition"]
    for i in range(2):
        assert np.all(x.component(i) == x.component(i)[0])
    ef = data.samplers["formation_energy"].component(0)
    assert np.array_equal(ef, data.samplers["potential_energy"].component(0))
    # the same chain through CanonicalBatch, keyed as the calculator keys it
    e2 = monte.RandomNumberEngine()
    e2.load(st0)
    seed = monte.RandomNumberGenerator(e2).random_int(2**63 - 1)
    b = clex.CanonicalBatch(model, (8, 8, 8), occ0[None, :], [1200.0], [seed])
    corr = b.corr()
    s = clex.accumulate(model, corr, b.run(150), np.zeros((1, 2)), 512)
    assert np.allclose(ef, s.formation_energy[:, 0], rtol=0, atol=1e-12)
    assert np.array_equal(final, b.occupation()[0])


def test_canonical_calculator_converges_to_reference_dynamics(gpu_lib, tmp_path):
    model, calc, state, occ0 = _setup(T=1500.0, seed=8)
    sf = calc.default_sampling_functions()
    p = sampling.CompletionCheckParams()
    p.cutoff_params.min_sample = 100
    p.log_spacing = False
    p.check_begin = 100
    p.check_period = 100
    sampling.converge(sf, p).set_precision("formation_energy", abs=3e-4)
    engine = monte.RandomNumberEngine()
    engine.seed(9)
    calc.run(state, sf, {}, p, can.CanonicalEventGenerator(),
             method_log=monte.MethodLog(str(tmp_path / "status.json"), log_frequency=None), random_engine=engine,
             write_status_f=_quiet)
    r = calc.data.completion_check.results()
    assert r.is_complete and r.convergence_check_results.all_converged
    conv = r.convergence_check_results.individual_results
    mean_gpu = next(v for k, v in conv.items() if k.sampler_name == "formation_energy").stats.mean
    e_ref, _ = OracleCE((8, 8, 8), 2, model.eci).canonical_samples(occ0, 1500.0, 77, 6000)
    e_ref = e_ref[1000:]
    st = sampling.BasicStatisticsCalculator(confidence=0.95)(np.ascontiguousarray(e_ref))
    assert abs(mean_gpu - st.mean) <= 2.0 * np.hypot(3e-4, st.calculated_precision), (mean_gpu, st.mean)


def test_canonical_calculator_runs_sampling_fixtures(gpu_lib, tmp_path):
    model, calc, state, occ0 = _setup(T=1000.0, seed=4)
    fmap = calc.default_sampling_functions()
    cc = sampling.CompletionCheckParams()
    cc.cutoff_params.max_count = 60
    sp = rm.SamplingParams(sampler_names=["formation_energy", "potential_energy"])
    fx = rm.SamplingFixtureParams("thermo", fmap, sampling.jsonStateSamplingFunctionMap(), {}, sp, cc)
    engine = monte.RandomNumberEngine()
    engine.seed(12)
    manager = rm.RunManager(engine, [fx])
    calc.run_fixtures(state, manager)
    res = manager.sampling_fixtures[0].results()
    assert res.sample_count == list(range(1, 61))
    assert np.array_equal(np.bincount(state.configuration.occupation(), minlength=2), np.bincount(occ0, minlength=2))
    assert np.array_equal(res.samplers["formation_energy"].component(0), res.samplers["potential_energy"].component(0))
