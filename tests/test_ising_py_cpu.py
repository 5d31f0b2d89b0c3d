"""The numpy Ising model of ``ising_py`` (python/libcasm/monte/ising_py): the reference's
known-answer values (tests/unit/monte/Ising_basic_semigrand_canonical_test.cpp:113-267,
with this model's composition change, sum (new - old), python/libcasm/monte/ising_py/
_model.py:380-393), and its Python loop for a user-supplied event generator against the
oracle's run of the same dynamics."""
import numpy as np

import casmcode_monte_gb300 as monte
import casmcode_monte_gb300.ising_py as ising
import casmcode_monte_gb300.ising_py.semigrand_canonical as sgc
import casmcode_monte_gb300.sampling as sampling
from tests import oracle_lib


def _state(shape=(25, 25), T=2000.0, mu=0.0):
    return ising.IsingState(
        configuration=ising.IsingConfiguration(shape=shape),
        conditions=monte.ValueMap.from_dict({"temperature": T, "exchange_potential": [mu]}))


def test_known_answers():
    state = _state(mu=2.0)
    fe = ising.IsingFormationEnergy(J=0.1, lattice_type=1, state=state)
    x = ising.IsingParamComposition(state=state)
    assert fe.per_supercell() == -125.0
    assert fe.per_unitcell() == -0.2
    assert fe.occ_delta_per_supercell([0], [-1]) == 0.8
    assert x.per_supercell()[0] == 625.0
    assert x.occ_delta_per_supercell([0], [-1])[0] == -2.0  # sum (new - old) in this model
    pot = sgc.SemiGrandCanonicalPotential(ising.IsingSystem(fe, x))
    pot.set_state(state, sgc.SemiGrandCanonicalConditions.from_values(state.conditions))
    assert pot.per_supercell() == -1375.0
    assert pot.occ_delta_per_supercell([0], [-1]) == 0.8 - 2.0 * (-2.0)
    # multi-site change: sequential apply and undo
    assert fe.occ_delta_per_supercell([0, 1], [-1, -1]) == 0.8 + 0.4
    assert fe.per_supercell() == -125.0


def test_configuration_indexing():
    cfg = ising.IsingConfiguration(shape=(4, 3))
    cfg.set_occ(5, -1)  # l = i + 4 j -> (1, 1)
    assert cfg.occupation()[1, 1] == -1 and cfg.occ(5) == -1
    assert cfg.to_linear_site_index((1, 1)) == 5
    d = cfg.to_dict()
    assert ising.IsingConfiguration.from_dict(d).to_dict() == d
    assert not cfg.occupation().flags.writeable


class CustomGenerator(sgc.SemiGrandCanonicalEventGenerator):
    """A user-supplied generator (same proposal): the run uses the host loop."""


def test_host_loop_matches_oracle(tmp_path):
    shape, T, mu = (8, 6), 1500.0, 0.03
    rng = np.random.default_rng(4)
    occ = rng.choice(np.array([-1, 1], dtype=np.int32), size=shape[0] * shape[1])
    state = _state(shape=shape, T=T, mu=mu)
    state.configuration.set_occupation(occ.reshape(shape, order="F"))
    calc = sgc.SemiGrandCanonicalCalculator(ising.IsingSystem(ising.IsingFormationEnergy(J=0.1),
                                                              ising.IsingParamComposition()))
    sf = sampling.StateSamplingFunctionMap()
    for f in (sgc.make_param_composition_f(calc), sgc.make_formation_energy_f(calc),
              sgc.make_potential_energy_f(calc)):
        sf[f.name] = f
    p = sampling.CompletionCheckParams()
    p.cutoff_params.max_count = 60
    p.log_spacing = False
    engine = monte.RandomNumberEngine()
    engine.seed(12)
    state0 = engine.dump()
    calc.run(state, sf, p, CustomGenerator(), sample_period=1,
             method_log=monte.MethodLog(str(tmp_path / "status.json"), log_frequency=None), random_engine=engine,
             write_status_f=lambda c, log: None)
    # the oracle runs the reference's C++ loop, whose N dx is (new - old) / 2: twice mu gives
    # this model's dE = dE_f - mu (new - old)
    ref = oracle_lib.ising_run(shape[0], shape[1], 0.1, False, T, 2.0 * mu, occ,
                               oracle_lib.make_cc_params(max_count=60), 1, state0)
    assert np.array_equal(state.configuration.occupation().flatten(order="F"), ref["occ"])
    assert np.array_equal(calc.data.samplers["formation_energy"].component(0), ref["formation_energy"])
    assert np.array_equal(calc.data.samplers["param_composition"].component(0), ref["param_composition"])
    assert calc.data.n_accept == ref["out"].n_accept and calc.data.n_reject == ref["out"].n_reject
    assert engine.dump() == ref["engine"]
    ef = calc.data.samplers["formation_energy"].component(0)
    x = calc.data.samplers["param_composition"].component(0)
    # (E_f - mu N x) / N against e_f - mu x: equal up to rounding
    assert np.allclose(calc.data.samplers["potential_energy"].component(0), ef - mu * x, rtol=1e-12, atol=1e-15)
