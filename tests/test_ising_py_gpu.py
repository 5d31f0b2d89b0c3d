"""``ising_py.semigrand_canonical`` on the GPU: the reference's two scenarios
(python/tests/ising_py/test_ising_semigrand_canonical_py.py:14-100,
test_ising_semigrand_canonical_mixed.py:11-100), and bit-exact parity of the GPU loop with
the oracle and with the reference's Python loop (the host loop of a user-supplied
generator) for this model's composition change."""
import pathlib

import numpy as np
import pytest

import casmcode_monte_gb300 as monte
import casmcode_monte_gb300.ising_cpp as ising_cpp
import casmcode_monte_gb300.ising_py as ising
import casmcode_monte_gb300.ising_py.semigrand_canonical as sgc
import casmcode_monte_gb300.sampling as sampling
from tests import oracle_lib

pytestmark = pytest.mark.gpu


def _sampling_functions(calc):
    sf = sampling.StateSamplingFunctionMap()
    for f in (sgc.make_param_composition_f(calc), sgc.make_formation_energy_f(calc),
              sgc.make_potential_energy_f(calc)):
        sf[f.name] = f
    return sf


def _scenario(models, tmp_path):
    calc = sgc.SemiGrandCanonicalCalculator(
        system=models.IsingSystem(
            formation_energy_calculator=models.IsingFormationEnergy(J=0.1, lattice_type=1),
            param_composition_calculator=models.IsingParamComposition()))
    sf = _sampling_functions(calc)
    state = models.IsingState(
        configuration=models.IsingConfiguration(shape=(25, 25)),
        conditions=monte.ValueMap.from_dict({"temperature": 2000.0, "exchange_potential": [0.0]}))
    for l in range(state.configuration.n_sites):
        state.configuration.set_occ(l, 1)
    p = sampling.CompletionCheckParams()
    p.cutoff_params.min_sample = 100
    p.log_spacing = False
    p.check_begin = 100
    p.check_period = 10
    sampling.converge(sf, p).set_precision("potential_energy", abs=0.001).set_precision("param_composition",
                                                                                         abs=0.001)
    log = monte.MethodLog(logfile_path=str(pathlib.Path(tmp_path) / "status.json"), log_frequency=0.2)
    calc.run(state=state, sampling_functions=sf, completion_check_params=p,
             event_generator=sgc.SemiGrandCanonicalEventGenerator(), sample_period=1, method_log=log,
             random_engine=None)
    results = calc.data.completion_check.results()
    assert sampling.get_n_samples(calc.data.samplers) >= 100
    assert results.is_complete
    assert results.equilibration_check_results.all_equilibrated
    assert len(results.equilibration_check_results.individual_results) == 2
    assert results.convergence_check_results.all_converged
    assert len(results.convergence_check_results.individual_results) == 2
    converge = results.convergence_check_results.individual_results
    for key, req in p.requested_precision.items():
        assert converge[key].stats.calculated_precision < req.abs_precision


def test_ising_semigrand_canonical_py(gpu_lib, tmp_path):
    _scenario(ising, tmp_path)


def test_ising_semigrand_canonical_mixed(gpu_lib, tmp_path):
    """The C++-mirroring models of ``ising_cpp`` in the Python-style calculator."""
    _scenario(ising_cpp, tmp_path)


class _UserGenerator(sgc.SemiGrandCanonicalEventGenerator):
    """Same proposal, but a user type: the run takes the reference's host loop."""


def _fixed_run(shape, T, mu, occ, seed, n_pass, generator, tmp_path):
    state = ising.IsingState(
        configuration=ising.IsingConfiguration(shape=shape),
        conditions=monte.ValueMap.from_dict({"temperature": T, "exchange_potential": [mu]}))
    state.configuration.set_occupation(occ.reshape(shape, order="F"))
    calc = sgc.SemiGrandCanonicalCalculator(ising.IsingSystem(ising.IsingFormationEnergy(J=0.1),
                                                              ising.IsingParamComposition()))
    p = sampling.CompletionCheckParams()
    p.cutoff_params.max_count = n_pass
    p.log_spacing = False
    engine = monte.RandomNumberEngine()
    engine.seed(seed)
    calc.run(state, _sampling_functions(calc), p, generator, sample_period=1,
             method_log=monte.MethodLog(str(tmp_path / "status.json"), log_frequency=None), random_engine=engine,
             write_status_f=lambda c, log: None)
    return calc, state, engine


@pytest.mark.parametrize("shape,T,mu,seed", [((16, 12), 1500.0, 0.05, 7), ((9, 13), 800.0, -0.1, 11)])
def test_gpu_loop_matches_oracle_and_host_loop(gpu_lib, tmp_path, shape, T, mu, seed):
    rng = np.random.default_rng(seed)
    occ = rng.choice(np.array([-1, 1], dtype=np.int32), size=shape[0] * shape[1])
    e0 = monte.RandomNumberEngine()
    e0.seed(seed)
    state0 = e0.dump()
    gpu, gstate, gengine = _fixed_run(shape, T, mu, occ, seed, 400, sgc.SemiGrandCanonicalEventGenerator(), tmp_path)
    host, hstate, hengine = _fixed_run(shape, T, mu, occ, seed, 400, _UserGenerator(), tmp_path)
    ref = oracle_lib.ising_run(shape[0], shape[1], 0.1, False, T, 2.0 * mu, occ,
                               oracle_lib.make_cc_params(max_count=400), 1, state0)
    assert np.array_equal(gstate.configuration.occupation(), hstate.configuration.occupation())
    assert np.array_equal(gstate.configuration.occupation().flatten(order="F"), ref["occ"])
    for name in ("formation_energy", "param_composition", "potential_energy"):
        assert np.array_equal(gpu.data.samplers[name].component(0), host.data.samplers[name].component(0)), name
    assert np.array_equal(gpu.data.samplers["formation_energy"].component(0), ref["formation_energy"])
    assert (gpu.data.n_accept, gpu.data.n_reject) == (host.data.n_accept, host.data.n_reject)
    assert gpu.data.n_accept == ref["out"].n_accept
    assert gengine.dump() == hengine.dump() == ref["engine"]
