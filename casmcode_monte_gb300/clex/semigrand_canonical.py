"""Semi-grand canonical Monte Carlo of an FCC cluster expansion behind the reference's
calculator interface.

The reference's calculator pattern (include/casm/monte/ising_cpp/basic_semigrand_canonical.hh:
36-627, python/src/monte_ising_cpp_semigrand_canonical.cpp:453-576) with the CE model as
its ``SystemType``: ``SemiGrandCanonicalCalculator(system).run(state, sampling_functions,
json_sampling_functions, completion_check_params, event_generator, sample_period,
method_log, random_engine, write_status_f)``.

``run`` sweeps the chain on the GPU (coloured Metropolis sweeps, ``ChainBatch``): a pass
proposes every site once, so the dynamics are the reference's in distribution, not step
for step.  Samples and the pass count change only at pass boundaries, so the completion
check the reference evaluates before every step (basic_occupation_metropolis.hh:381) is
evaluated at each pass boundary, with the calls in between applied to its check schedule;
chunks of passes end at the first boundary where it could finish the run or check
convergence.  The default sampling functions read the exact integer correlation sums the
GPU tracks; other sampling functions are called on the host after the occupation has been
brought back.  The Philox key of the sweep is drawn from the caller's random engine.
"""
from __future__ import annotations

import os
import sys
from typing import Callable, Optional

import numpy as np

from .. import MethodLog, RandomNumberEngine, RandomNumberGenerator, ValueMap
from ..sampling import (CompletionCheck, CompletionCheckParams, Sampler, StateSamplingFunction,
                        StateSamplingFunctionMap, get_n_samples, jsonSampler, jsonSamplerMap,
                        jsonStateSamplingFunction, jsonStateSamplingFunctionMap)
from . import ChainBatch, ClexModel, accumulate

KB = 8.6173303e-05  # eV/K (libcasm-global's KB)


class ClexConfiguration:
    """Occupant indices of an L0 x L1 x L2 FCC supercell (diagonal transformation matrix),
    linear site index l = i + L0 (j + L1 k)."""

    def __init__(self, shape=(8, 8, 8), occupation=None):
        self.shape = tuple(int(x) for x in shape)
        if len(self.shape) != 3 or min(self.shape) < 1:
            raise RuntimeError("Error in ClexConfiguration: shape must be three positive integers")
        n = self.shape[0] * self.shape[1] * self.shape[2]
        self._occ = np.zeros(n, dtype=np.int8)
        if occupation is not None:
            self.set_occupation(occupation)

    @property
    def n_sites(self) -> int:
        return int(self._occ.size)

    @property
    def n_variable_sites(self) -> int:
        return int(self._occ.size)

    @property
    def n_unitcells(self) -> int:
        return int(self._occ.size)

    def occupation(self) -> np.ndarray:
        v = self._occ.view()
        v.flags.writeable = False
        return v

    def set_occupation(self, occupation) -> None:
        o = np.asarray(occupation).reshape(-1)
        if o.size != self._occ.size:
            raise RuntimeError("Error in ClexConfiguration::set_occupation: size mismatch")
        self._occ[:] = o.astype(np.int8)

    def occ(self, linear_site_index: int) -> int:
        return int(self._occ[int(linear_site_index)])

    def set_occ(self, linear_site_index: int, new_occ: int) -> None:
        self._occ[int(linear_site_index)] = new_occ

    def to_dict(self) -> dict:
        return {"shape": list(self.shape), "occupation": [int(x) for x in self._occ]}

    @staticmethod
    def from_dict(data: dict) -> "ClexConfiguration":
        return ClexConfiguration(tuple(data["shape"]), np.asarray(data["occupation"], dtype=np.int8))


class ClexState:
    """Configuration, conditions and calculated properties."""

    def __init__(self, configuration: ClexConfiguration, conditions: ValueMap,
                 properties: Optional[ValueMap] = None):
        self.configuration = configuration
        self.conditions = conditions
        self.properties = properties if properties is not None else ValueMap()


class _DeviceQuery:
    """A one-chain batch holding a copy of a state's occupation for per-state queries
    (correlation sums, single-site energy changes) on the GPU."""

    def __init__(self, model: ClexModel, cfg: ClexConfiguration, mu):
        self.batch = ChainBatch(model, cfg.shape, cfg.occupation()[None, :], [1000.0],
                                np.asarray(mu, dtype=float).reshape(1, -1), [1])

    def load(self, cfg: ClexConfiguration) -> None:
        self.batch.set_occupation(cfg.occupation()[None, :])


def _delta_sequential(query: _DeviceQuery, cfg: ClexConfiguration, linear_site_index, new_occ) -> float:
    """Energy change of changing several sites: each change on the state left by the
    previous ones (as the reference's occ_delta_per_supercell), then restored."""
    sites = [int(x) for x in linear_site_index]
    new = [int(x) for x in new_occ]
    query.load(cfg)
    if len(sites) == 1:
        return float(query.batch.delta_e([0], sites, new)[0])
    tmp = ClexConfiguration(cfg.shape, cfg.occupation())
    dE = 0.0
    for l, v in zip(sites, new):
        dE += float(query.batch.delta_e([0], [l], [v])[0])
        tmp.set_occ(l, v)
        query.load(tmp)
    return dE


class ClexFormationEnergy:
    """Formation energy of a cluster expansion: E_f = sum_f w_f IntCorr_f (per supercell),
    from the GPU's integer correlation sums."""

    def __init__(self, model: ClexModel, state: Optional[ClexState] = None):
        self.model = model
        self.state: Optional[ClexState] = None
        self._query: Optional[_DeviceQuery] = None
        if state is not None:
            self.set_state(state)

    def set_state(self, state: ClexState) -> None:
        if state is None:
            raise RuntimeError("Error in ClexFormationEnergy::set_state: state==nullptr")
        self.state = state
        self._query = None

    def _q(self) -> _DeviceQuery:
        if self._query is None:
            self._query = _DeviceQuery(self.model, self.state.configuration, np.zeros(self.model.n_species - 1))
        return self._query

    def int_corr(self) -> np.ndarray:
        q = self._q()
        q.load(self.state.configuration)
        return q.batch.corr()[0]

    def per_supercell(self) -> float:
        return float(self.model.formation_per_supercell(self.int_corr()))

    def per_unitcell(self) -> float:
        return self.per_supercell() / self.state.configuration.n_unitcells

    def occ_delta_per_supercell(self, linear_site_index, new_occ) -> float:
        return _delta_sequential(self._q(), self.state.configuration, linear_site_index, new_occ)

    def __deepcopy__(self, memo):
        return ClexFormationEnergy(self.model)


class ClexParamComposition:
    """Parametric composition: binary x = n_B / N; ternary (x_B, x_C) = (n_B, n_C) / N."""

    def __init__(self, model: ClexModel, state: Optional[ClexState] = None):
        self.model = model
        self.state: Optional[ClexState] = None
        if state is not None:
            self.set_state(state)

    def set_state(self, state: ClexState) -> None:
        if state is None:
            raise RuntimeError("Error in ClexParamComposition::set_state: state==nullptr")
        self.state = state

    def n_independent_compositions(self) -> int:
        return self.model.n_species - 1

    def per_supercell(self) -> np.ndarray:
        o = self.state.configuration.occupation()
        return np.array([float(np.count_nonzero(o == s)) for s in range(1, self.model.n_species)])

    def per_unitcell(self) -> np.ndarray:
        return self.per_supercell() / self.state.configuration.n_unitcells

    def occ_delta_per_supercell(self, linear_site_index, new_occ) -> np.ndarray:
        cfg = self.state.configuration
        d = np.zeros(self.model.n_species - 1)
        for l, v in zip(linear_site_index, new_occ):
            old = cfg.occ(l)
            if int(v) >= 1:
                d[int(v) - 1] += 1.0
            if old >= 1:
                d[old - 1] -= 1.0
        return d

    def __deepcopy__(self, memo):
        return ClexParamComposition(self.model)


class ClexSystem:
    """Holds the formation energy and parametric composition calculators."""

    def __init__(self, formation_energy_calculator: ClexFormationEnergy,
                 param_composition_calculator: ClexParamComposition):
        if formation_energy_calculator.model is not param_composition_calculator.model:
            raise RuntimeError("Error in ClexSystem: the calculators must share one ClexModel")
        self.formation_energy_calculator = formation_energy_calculator
        self.param_composition_calculator = param_composition_calculator

    @property
    def model(self) -> ClexModel:
        return self.formation_energy_calculator.model


class SemiGrandCanonicalConditions:
    """Temperature and exchange potential (basic_semigrand_canonical.hh:36-80)."""

    def __init__(self, temperature: float = 0.0, exchange_potential=None):
        self.temperature = float(temperature)
        self.exchange_potential = np.asarray(exchange_potential if exchange_potential is not None else [],
                                             dtype=float).reshape(-1)

    @staticmethod
    def from_values(values: ValueMap) -> "SemiGrandCanonicalConditions":
        if "temperature" not in values.scalar_values:
            raise RuntimeError('Error in SemiGrandCanonicalConditions: missing "temperature"')
        if "exchange_potential" not in values.vector_values:
            raise RuntimeError('Error in SemiGrandCanonicalConditions: missing "exchange_potential"')
        return SemiGrandCanonicalConditions(values.scalar_values["temperature"], values.vector_values["exchange_potential"])

    def to_values(self) -> ValueMap:
        v = ValueMap()
        v.scalar_values["temperature"] = self.temperature
        v.vector_values["exchange_potential"] = self.exchange_potential.copy()
        return v

    def to_dict(self) -> dict:
        return self.to_values().to_dict()

    @staticmethod
    def from_dict(data: dict) -> "SemiGrandCanonicalConditions":
        return SemiGrandCanonicalConditions.from_values(ValueMap.from_dict(data))


class SemiGrandCanonicalPotential:
    """E_sgc = E_f - mu . N x and its change (basic_semigrand_canonical.hh:104-199)."""

    def __init__(self, system: ClexSystem):
        self.system = system
        self.formation_energy_calculator = ClexFormationEnergy(system.model)
        self.param_composition_calculator = ClexParamComposition(system.model)
        self.state: Optional[ClexState] = None
        self.conditions: Optional[SemiGrandCanonicalConditions] = None
        self._query: Optional[_DeviceQuery] = None

    def set_state(self, state: ClexState, conditions: SemiGrandCanonicalConditions) -> None:
        if conditions.exchange_potential.size != self.system.model.n_species - 1:
            raise RuntimeError("Error in SemiGrandCanonicalPotential::set_state: exchange_potential size must be "
                               "the number of independent compositions")
        self.state = state
        self.conditions = conditions
        self.formation_energy_calculator.set_state(state)
        self.param_composition_calculator.set_state(state)
        self._query = None

    def per_supercell(self) -> float:
        nx = self.param_composition_calculator.per_supercell()
        return self.formation_energy_calculator.per_supercell() - float(np.dot(self.conditions.exchange_potential, nx))

    def per_unitcell(self) -> float:
        return self.per_supercell() / self.state.configuration.n_unitcells

    def occ_delta_per_supercell(self, linear_site_index, new_occ) -> float:
        if self._query is None:
            self._query = _DeviceQuery(self.system.model, self.state.configuration, self.conditions.exchange_potential)
        return _delta_sequential(self._query, self.state.configuration, linear_site_index, new_occ)


class SemiGrandCanonicalEventGenerator:
    """The proposals of the GPU sweep: every site once per pass, colour by colour, a new
    occupant chosen uniformly among the others (binary: the other species)."""

    def __init__(self):
        self.state: Optional[ClexState] = None

    def set_state(self, state: ClexState) -> None:
        if state is None:
            raise RuntimeError("Error in SemiGrandCanonicalEventGenerator::set_state: state==nullptr")
        self.state = state


class SemiGrandCanonicalData:
    """Run data (BasicOccupationMetropolisData, basic_occupation_metropolis.hh:18-115)."""

    def __init__(self, sampling_functions, json_sampling_functions, n_steps_per_pass: int,
                 completion_check_params: CompletionCheckParams):
        self.sampling_functions = sampling_functions
        self.json_sampling_functions = json_sampling_functions
        self.samplers = {f.name: Sampler(f.shape, f.component_names) for f in sampling_functions.values()}
        self.json_samplers = jsonSamplerMap({f.name: jsonSampler() for f in json_sampling_functions.values()})
        self.sample_weight = Sampler([])
        self.n_pass = 0
        self.n_steps_per_pass = int(n_steps_per_pass)
        self.n_accept = 0
        self.n_reject = 0
        self.completion_check = CompletionCheck(completion_check_params)

    def acceptance_rate(self) -> float:
        return self.n_accept / (self.n_accept + self.n_reject)

    def rejection_rate(self) -> float:
        return self.n_reject / (self.n_accept + self.n_reject)

    def to_dict(self) -> dict:
        tot = self.n_accept + self.n_reject
        return {"completion_check_results": self.completion_check.results().to_dict(), "n_pass": self.n_pass,
                "n_steps_per_pass": self.n_steps_per_pass, "n_accept": self.n_accept,
                "n_reject": self.n_reject, "acceptance_rate": self.n_accept / tot if tot else float("nan"),
                "rejection_rate": self.n_reject / tot if tot else float("nan")}


class _DeviceSampled:
    """A default sampling function: during ``run`` its values come from the GPU's exact
    integer correlation sums; outside ``run`` it evaluates the calculators."""

    def __init__(self, calc: "SemiGrandCanonicalCalculator", kind: str):
        self.calc = calc
        self.kind = kind

    def __call__(self):
        c = self.calc
        if self.kind == "param_composition":
            return c.param_composition_calculator.per_unitcell()
        if self.kind == "formation_energy":
            return np.array([c.formation_energy_calculator.per_unitcell()])
        if self.kind == "corr":
            return c._corr_per_unitcell(c.formation_energy_calculator.int_corr())
        return np.array([c.potential.per_unitcell()])


def default_write_status(mc_calculator, method_log: MethodLog) -> None:
    """Status to stdout and completion-check results to the log file."""
    data = mc_calculator.data
    n_samples = get_n_samples(data.samplers)
    steps = float(data.n_pass) * float(data.n_steps_per_pass)
    t = method_log.time_s()
    print(f"Passes={data.n_pass}, Samples={n_samples}, ClockTime(s)={t}, "
          f"Steps/Second={steps / t if t > 0 else float('inf')}, Seconds/Step={t / steps if steps else 0.0}")
    results = data.completion_check.results()
    print(f"  AllEquilibrated={int(results.equilibration_check_results.all_equilibrated)}")
    if results.equilibration_check_results.all_equilibrated:
        print(f"  AllConverged={int(results.convergence_check_results.all_converged)}")
    sys.stdout.flush()
    if method_log.logfile_path():
        method_log.reset()
        method_log.write_json(results.to_dict())
    method_log.begin_lap()


class SemiGrandCanonicalCalculator:
    """Semi-grand canonical Monte Carlo calculator for a cluster-expansion system."""

    def __init__(self, system: ClexSystem, precision: str = "fp64"):
        if system is None:
            raise RuntimeError("Error constructing SemiGrandCanonicalCalculator: system==nullptr")
        self.system = system
        self.precision = precision
        self.state: Optional[ClexState] = None
        self.conditions: Optional[SemiGrandCanonicalConditions] = None
        self.potential = SemiGrandCanonicalPotential(system)
        self.formation_energy_calculator = self.potential.formation_energy_calculator
        self.param_composition_calculator = self.potential.param_composition_calculator
        self.data: Optional[SemiGrandCanonicalData] = None
        #: upper bound on passes per kernel launch
        self.max_passes_per_launch = 500
        #: device time of the sweep kernels in the last run (ms)
        self.last_kernel_ms = 0.0

    # construction steps a calculator of another ensemble replaces (clex.canonical)
    def _conditions_from(self, values: ValueMap) -> SemiGrandCanonicalConditions:
        return SemiGrandCanonicalConditions.from_values(values)

    def _default_event_generator(self):
        return SemiGrandCanonicalEventGenerator()

    def _make_batch(self, state: ClexState, mu: np.ndarray, seed: int):
        return ChainBatch(self.system.model, state.configuration.shape, state.configuration.occupation()[None, :],
                          [self.conditions.temperature], mu, np.array([seed], dtype=np.uint64),
                          precision=self.precision)

    def default_sampling_functions(self) -> StateSamplingFunctionMap:
        m = StateSamplingFunctionMap()
        model = self.system.model
        m["param_composition"] = StateSamplingFunction(
            "param_composition", "Parametric composition", [model.n_species - 1],
            _DeviceSampled(self, "param_composition"))
        m["formation_energy"] = StateSamplingFunction(
            "formation_energy", "Intensive formation energy", [], _DeviceSampled(self, "formation_energy"))
        m["potential_energy"] = StateSamplingFunction(
            "potential_energy", "Intensive potential energy", [], _DeviceSampled(self, "potential_energy"))
        m["corr"] = StateSamplingFunction(
            "corr", "Correlations per unit cell (one per cluster class)", [model.n_classes],
            _DeviceSampled(self, "corr"))
        return m

    def default_json_sampling_functions(self) -> jsonStateSamplingFunctionMap:
        m = jsonStateSamplingFunctionMap()
        m["configuration"] = jsonStateSamplingFunction(
            "configuration", "Configuration values", lambda: self.state.configuration.to_dict())
        return m

    def _corr_per_unitcell(self, int_corr) -> np.ndarray:
        model = self.system.model
        return np.asarray(int_corr, dtype=float) * model.scale / model.multiplicity / self.state.configuration.n_unitcells

    def run(self, state: ClexState, sampling_functions, json_sampling_functions,
            completion_check_params: CompletionCheckParams,
            event_generator: Optional[SemiGrandCanonicalEventGenerator] = None, sample_period: int = 1,
            method_log: Optional[MethodLog] = None, random_engine: Optional[RandomNumberEngine] = None,
            write_status_f: Optional[Callable] = None) -> SemiGrandCanonicalData:
        """Run at one thermodynamic state; ``state`` is modified in place."""
        if write_status_f is None:
            write_status_f = default_write_status
        if sample_period < 1:
            raise RuntimeError("Error in SemiGrandCanonicalCalculator::run: sample_period must be >= 1")
        self.state = state
        self.conditions = self._conditions_from(state.conditions)
        self.potential.set_state(state, self.conditions)
        if event_generator is None:
            event_generator = self._default_event_generator()
        event_generator.set_state(state)
        N = state.configuration.n_variable_sites
        self.data = data = SemiGrandCanonicalData(sampling_functions, json_sampling_functions, N,
                                                  completion_check_params)
        if random_engine is None:
            random_engine = RandomNumberEngine()
        if method_log is None:
            method_log = MethodLog(os.path.join(os.getcwd(), "status.json"), 600.0)
        method_log.restart_clock()
        method_log.begin_lap()
        # the sweep's Philox key, drawn from the caller's engine
        seed = RandomNumberGenerator(random_engine).random_int(2**63 - 1)
        model = self.system.model
        mu = self.conditions.exchange_potential.reshape(1, -1)
        batch = self._make_batch(state, mu, seed)
        self.last_kernel_ms = 0.0
        try:
            self._main_loop(batch, data, N, mu, sample_period, method_log, write_status_f, completion_check_params)
        finally:
            state.configuration.set_occupation(batch.occupation()[0])
            batch.close()
        write_status_f(self, method_log)
        return data

    def _main_loop(self, batch, data, N, mu, sample_period, method_log, write_status_f, params) -> None:
        model = self.system.model
        cc = data.completion_check
        funcs = data.sampling_functions
        device_only = all(isinstance(f.function, _DeviceSampled) and f.function.calc is self
                          for f in funcs.values()) and len(data.json_sampling_functions) == 0
        max_chunk = max(1, int(self.max_passes_per_launch))
        if params.cutoff_params.max_clocktime is not None:
            max_chunk = min(max_chunk, sample_period)
        corr = batch.corr()
        n_samples = 0

        def check():
            return cc.count_check(data.samplers, data.sample_weight, data.n_pass, method_log)

        complete = check()
        while not complete:
            cc._repeat_calls(N - 1)
            # the chunk ends at the first pass boundary where the check could act
            k, ns = 0, n_samples
            limit = max_chunk if device_only else max(1, sample_period - (data.n_pass % sample_period))
            limit = min(limit, max_chunk)
            while k < limit:
                k += 1
                p = data.n_pass + k
                if p % sample_period == 0:
                    ns += 1
                if cc._could_complete_at(ns, p):
                    break
            out = batch.run(k)
            self.last_kernel_ms += batch.last_kernel_ms()
            s = accumulate(model, corr, out, mu, N)
            corr = s.int_corr[-1]
            for b in range(k):
                data.n_pass += 1
                acc = int(out[b, 0, 0])
                data.n_accept += acc
                data.n_reject += N - acc
                if data.n_pass % sample_period == 0:
                    self._push_sample(batch, data, s, b, device_only)
                    n_samples += 1
                    lf = method_log.log_frequency()
                    if lf is not None and method_log.lap_time() >= lf:
                        write_status_f(self, method_log)
                complete = check()
                if complete:
                    if b != k - 1:
                        raise RuntimeError("internal error: completion inside a planned chunk")
                    break
                if b < k - 1:
                    cc._repeat_calls(N - 1)

    def run_fixtures(self, state: ClexState, run_manager) -> None:
        """Run with the sampling fixtures of a ``run_management.RunManager`` (as
        occupation_metropolis.hh:90-154 does on the host), sweeping on the GPU.

        Fixtures must sample by pass.  Every pass counts N steps; the accepted flips of a
        pass come from the device, and ``state.properties.scalar_values["potential_energy"]``
        (per unit cell) follows the device's exact integer sums.  Chunks of passes end at
        the next pass where a fixture samples or where its completion check could finish or
        check convergence; before each sample the occupation is brought back to ``state``.
        The fixtures are finalized (results written) with the final state.
        """
        from ..sampling import SAMPLE_MODE

        for f in run_manager.sampling_fixtures:
            if f.params().sampling_params.sample_mode != SAMPLE_MODE.BY_PASS:
                raise RuntimeError("Error in SemiGrandCanonicalCalculator::run_fixtures: the GPU sweep proposes whole "
                                   "passes; sampling fixtures must sample by pass")
        self.state = state
        self.conditions = self._conditions_from(state.conditions)
        self.potential.set_state(state, self.conditions)
        model = self.system.model
        N = state.configuration.n_variable_sites
        mu = self.conditions.exchange_potential.reshape(1, -1)
        seed = RandomNumberGenerator(run_manager.engine).random_int(2**63 - 1)
        batch = self._make_batch(state, mu, seed)
        fixtures = run_manager.sampling_fixtures
        self.last_kernel_ms = 0.0
        try:
            run_manager.initialize(N)
            corr = batch.corr()
            ef = float(model.formation_per_supercell(corr[0]))
            nx = model.n_x(corr[0], N)
            state.properties.scalar_values["potential_energy"] = (ef - float(np.dot(mu[0], nx))) / N
            run_manager.sample_data_by_count_if_due(state)
            while not run_manager.is_complete():
                run_manager.write_status_if_due()
                for f in fixtures:
                    f._completion_check._repeat_calls(N - 1)
                # plan the chunk
                k = max(1, min(int(self.max_passes_per_launch), *[max(1, _fixture_passes_to_sample(f)) for f in fixtures]))
                for p in range(1, k + 1):
                    if any(f._completion_check._could_complete_at(
                            get_n_samples(f.results().samplers) + (1 if f.next_sample_count() <= f.counter().count + p
                                                                   else 0), f.counter().count + p) for f in fixtures):
                        k = p
                        break
                out = batch.run(k)
                self.last_kernel_ms += batch.last_kernel_ms()
                s = accumulate(model, corr, out, mu, N)
                corr = s.int_corr[-1]
                for b in range(k):
                    acc = int(out[b, 0, 0])
                    for f in fixtures:
                        c = f.counter()
                        c.pass_ += 1
                        c.count += 1
                        c.n_accept += acc
                        c.n_reject += N - acc
                    state.properties.scalar_values["potential_energy"] = float(s.potential_energy[b, 0])
                    if any(f.counter().count == f.next_sample_count() for f in fixtures):
                        # a chunk ends at the first pass where a fixture samples
                        state.configuration.set_occupation(batch.occupation()[0])
                        run_manager.sample_data_by_count_if_due(state)
                    if b < k - 1:
                        if run_manager.is_complete():
                            raise RuntimeError("internal error: completion inside a planned chunk")
                        for f in fixtures:
                            f._completion_check._repeat_calls(N - 1)
        finally:
            state.configuration.set_occupation(batch.occupation()[0])
            batch.close()
        run_manager.finalize(state)

    def _push_sample(self, batch, data, s, b, device_only) -> None:
        values = {
            "param_composition": np.asarray(s.param_composition[b, 0], dtype=float),
            "formation_energy": np.array([float(s.formation_energy[b, 0])]),
            "potential_energy": np.array([float(s.potential_energy[b, 0])]),
            "corr": self._corr_per_unitcell(s.int_corr[b, 0]),
        }
        if not device_only:
            # other functions read the host state: bring the occupation back first (the
            # device state is the one after the last pass of the chunk, which is this pass
            # whenever a chunk may end at a sample)
            self.state.configuration.set_occupation(batch.occupation()[0])
        for name in sorted(data.sampling_functions):
            f = data.sampling_functions[name]
            if isinstance(f.function, _DeviceSampled) and f.function.calc is self:
                data.samplers[name].append(values[f.function.kind])
            else:
                data.samplers[name].append(f())
        for name in sorted(data.json_sampling_functions):
            data.json_samplers[name].values.append(data.json_sampling_functions[name]())


def _fixture_passes_to_sample(f) -> int:
    return f.next_sample_count() - f.counter().count


__all__ = ["ClexConfiguration", "ClexFormationEnergy", "ClexParamComposition", "ClexState", "ClexSystem",
           "SemiGrandCanonicalCalculator", "SemiGrandCanonicalConditions", "SemiGrandCanonicalData",
           "SemiGrandCanonicalEventGenerator", "SemiGrandCanonicalPotential", "default_write_status"]
