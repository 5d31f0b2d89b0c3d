"""Rejection-free and kinetic loops with run management (methods/nfold.hh:48-149,
methods/kinetic_monte_carlo.hh:108-224) on a 4x4x4 binary FCC cluster expansion, driven by
a test event selector over single-site flips with Metropolis rates (the reference ships the
loops; selectors come from the calling code).

* nfold: every selected event is applied; a sample by count carries the time increment of
  the step it is taken at as its weight and sees total_rate / n_events_possible as the
  expected acceptance rate; time-weighted averages agree with the reference's Metropolis
  dynamics.
* kinetic_monte_carlo: samples by time at the scheduled times, with kmc_data's time, total
  rate, previous sample time and atom positions as the reference sets them.
"""
import math

import numpy as np

import casmcode_monte_gb300 as monte
import casmcode_monte_gb300.clex.semigrand_canonical as csgc
import casmcode_monte_gb300.events as ev
import casmcode_monte_gb300.methods as methods
import casmcode_monte_gb300.run_management as rm
import casmcode_monte_gb300.sampling as sampling
from casmcode_monte_gb300 import clex
from tests import oracle_lib

KB = 8.6173303e-05
L = (4, 4, 4)
N = 64


class FlipSelector:
    """Single-site flips of a semi-grand canonical binary CE, selected with probability
    proportional to the Metropolis rate min(1, exp(-beta dE)); time increment -ln(1-u) /
    total rate (test support).  Rates are recomputed from the state at each selection."""

    def __init__(self, orc, state, T, mu, rng):
        self.orc, self.state, self.beta, self.mu, self.rng = orc, state, 1.0 / (KB * T), np.asarray(mu), rng
        self.log = []  # (total_rate, time_increment) per selection
        self._total = None
        self._occ_at_total = None

    def _rates(self):
        occ = self.state.configuration.occupation().astype(np.int32)
        dE = np.array([self.orc.delta_e(occ, l, 1 - int(occ[l]), self.mu) for l in range(N)])
        return np.minimum(1.0, np.exp(-self.beta * dE))

    def total_rate(self):
        # the total of the current state (nfold reads it before selecting, kinetic Monte
        # Carlo after): the last selection's total when the state has not changed since
        occ = self.state.configuration.occupation()
        if self._total is None or not np.array_equal(occ, self._occ_at_total):
            self._total = float(self._rates().sum())
            self._occ_at_total = occ.copy()
        return self._total

    def select_event(self):
        r = self._rates()
        total = float(r.sum())
        x = self.rng.random_real(total)
        l = int(np.searchsorted(np.cumsum(r), x, side="right"))
        dt = -math.log(1.0 - self.rng.random_real(1.0)) / total
        self._total = total
        self._occ_at_total = self.state.configuration.occupation().copy()
        self.log.append((total, dt))
        return min(l, N - 1), dt


def _setup(occ0, T, mu, update_atoms=False):
    eci = clex.make_eci("fcc_binary", 4)
    orc = oracle_lib.OracleCE(L, 2, eci)
    state = csgc.ClexState(csgc.ClexConfiguration(L, occ0.copy()),
                           monte.ValueMap.from_dict({"temperature": T, "exchange_potential": mu}))
    convert = ev.Conversions(ev.Prim.fcc(4.0, ["A", "B"]), np.eye(3, dtype=int) * 4)
    cands = ev.OccCandidateList(convert)
    loc = ev.OccLocation(convert, cands, update_atoms=update_atoms)
    loc.initialize(state.configuration.occupation().copy())

    def get_event(l):
        mol = loc.mol(loc.l_to_mol_id(l))
        to = 1 - mol.species_index
        t = ev.OccTransform(l=l, mol_id=mol.id, asym=mol.asym, from_species=mol.species_index, to_species=to)
        return ev.OccEvent(linear_site_index=[l], new_occ=[convert.occ_index(mol.asym, to)], occ_transform=[t],
                           atom_traj=[])

    return orc, state, loc, get_event


def _potential(orc, state, mu):
    occ = state.configuration.occupation().astype(np.int32)
    return (orc.formation(occ) - mu[0] * np.count_nonzero(occ == 1)) / N


def test_nfold_weights_rates_and_counts():
    mu = [0.01]
    occ0 = np.random.default_rng(1).integers(0, 2, size=N).astype(np.int8)
    orc, state, loc, get_event = _setup(occ0, 1200.0, mu)
    engine = monte.RandomNumberEngine()
    engine.seed(5)
    sel = FlipSelector(orc, state, 1200.0, mu, monte.RandomNumberGenerator(engine))
    data = methods.NfoldData(n_events_possible=N)
    fmap = sampling.StateSamplingFunctionMap()
    fmap["expected_acceptance_rate"] = sampling.StateSamplingFunction(
        "expected_acceptance_rate", "", [], lambda: np.array([data.expected_acceptance_rate]))
    fmap["potential_energy"] = sampling.StateSamplingFunction(
        "potential_energy", "", [], lambda: np.array([_potential(orc, state, mu)]))
    cc = sampling.CompletionCheckParams()
    cc.cutoff_params.max_count = 12
    sp = rm.SamplingParams(sampler_names=["expected_acceptance_rate", "potential_energy"])
    fx = rm.SamplingFixtureParams("thermo", fmap, sampling.jsonStateSamplingFunctionMap(), {}, sp, cc)
    manager = rm.RunManager(engine, [fx])
    methods.nfold(state, loc, data, sel, get_event, manager)
    r = manager.sampling_fixtures[0].results()
    # a sample is taken after the step's selection and before its count: the run ends when
    # the count reaches 12 passes, before the sample of pass 12
    assert r.sample_count == list(range(1, 12))
    assert r.n_accept == len(sel.log) == 12 * N and r.n_reject == 0
    # samples by pass are taken at steps 64 k, after that step's selection
    w = r.sample_weight.component(0)
    acc = r.samplers["expected_acceptance_rate"].component(0)
    for k in range(1, 12):
        total, dt = sel.log[64 * k]
        assert w[k - 1] == dt and acc[k - 1] == total / N
    # the tracked occupation and the lists agree
    occ = state.configuration.occupation()
    assert all(loc.mol(loc.l_to_mol_id(l)).species_index == occ[l] for l in range(N))


def _block_mean(x, w, n_blocks=10):
    m = len(x) // n_blocks
    means = [np.average(x[i * m:(i + 1) * m], weights=w[i * m:(i + 1) * m]) for i in range(n_blocks)]
    return float(np.average(x, weights=w)), float(np.std(means, ddof=1) / math.sqrt(n_blocks))


def test_nfold_time_weighted_average_matches_metropolis():
    mu = [0.0]
    T = 2000.0
    occ0 = np.random.default_rng(2).integers(0, 2, size=N).astype(np.int8)
    orc, state, loc, get_event = _setup(occ0, T, mu)
    engine = monte.RandomNumberEngine()
    engine.seed(7)
    sel = FlipSelector(orc, state, T, mu, monte.RandomNumberGenerator(engine))
    data = methods.NfoldData(n_events_possible=N)
    fmap = sampling.StateSamplingFunctionMap()
    fmap["potential_energy"] = sampling.StateSamplingFunction(
        "potential_energy", "", [], lambda: np.array([_potential(orc, state, mu)]))
    cc = sampling.CompletionCheckParams()
    cc.cutoff_params.max_count = 3000
    sp = rm.SamplingParams(sampler_names=["potential_energy"], sample_mode=sampling.SAMPLE_MODE.BY_STEP,
                           period=8.0, begin=8.0)
    fx = rm.SamplingFixtureParams("thermo", fmap, sampling.jsonStateSamplingFunctionMap(), {}, sp, cc)
    manager = rm.RunManager(engine, [fx])
    methods.nfold(state, loc, data, sel, get_event, manager)
    r = manager.sampling_fixtures[0].results()
    e = r.samplers["potential_energy"].component(0)[300:]
    w = r.sample_weight.component(0)[300:]
    m_nfold, s_nfold = _block_mean(e, w)
    e_ref, _, _ = orc.sgc_samples(occ0.astype(np.int32), T, np.array(mu), 99, 3000)
    e_ref = e_ref[300:]
    m_ref, s_ref = _block_mean(e_ref, np.ones_like(e_ref))
    assert abs(m_nfold - m_ref) <= 4.0 * math.hypot(s_nfold, s_ref), (m_nfold, m_ref, s_nfold, s_ref)


def test_kinetic_monte_carlo_samples_by_time():
    mu = [0.0]
    occ0 = np.random.default_rng(3).integers(0, 2, size=N).astype(np.int8)
    orc, state, loc, get_event = _setup(occ0, 1500.0, mu, update_atoms=True)
    engine = monte.RandomNumberEngine()
    engine.seed(11)
    sel = FlipSelector(orc, state, 1500.0, mu, monte.RandomNumberGenerator(engine))
    kmc = methods.KMCData()
    seen = []
    fmap = sampling.StateSamplingFunctionMap()
    fmap["t"] = sampling.StateSamplingFunction(
        "t", "", [], lambda: seen.append((kmc.time, kmc.total_rate, kmc.prev_time["kinetics"],
                                          kmc.atom_positions_cart.shape, kmc.sampling_fixture_label))
        or np.array([kmc.time]))
    cc = sampling.CompletionCheckParams()
    cc.cutoff_params.max_time = 20.0
    sp = rm.SamplingParams(sampler_names=["t"], sample_mode=sampling.SAMPLE_MODE.BY_TIME, period=2.0, begin=2.0,
                           do_sample_time=True)
    fx = rm.SamplingFixtureParams("kinetics", fmap, sampling.jsonStateSamplingFunctionMap(), {}, sp, cc)
    manager = rm.RunManager(engine, [fx])
    methods.kinetic_monte_carlo(state, loc, kmc, sel, get_event, manager)
    r = manager.sampling_fixtures[0].results()
    times = list(r.sample_time)
    assert len(times) >= 9 and times == [2.0 * (i + 1) for i in range(len(times))]
    for i, (t, total, prev, shape, label) in enumerate(seen):
        assert t == times[i] and label == "kinetics" and shape == (3, loc.atom_size()) and total > 0
        assert prev == (times[i - 1] if i > 0 else 0.0)
    assert kmc.prev_time["kinetics"] == times[-1]
    assert r.n_accept == len(sel.log)
