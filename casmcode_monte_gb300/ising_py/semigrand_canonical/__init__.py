"""Semi-grand canonical Monte Carlo of the numpy Ising model (mirrors
``libcasm.monte.ising_py.semigrand_canonical``,
python/libcasm/monte/ising_py/semigrand_canonical/_methods.py).

The reference runs this calculator as a Python loop (_methods.py:552-724): propose a
random site, ``dE = dE_f - mu . N dx`` from the potential, Metropolis acceptance, apply,
count passes, sample every ``sample_period`` passes, with the completion check before
every step.  Here ``SemiGrandCanonicalCalculator.run`` executes the same loop on the GPU
(the serial replay of ``ising_cpp.semigrand_canonical``), consuming the caller's
``RandomNumberEngine`` exactly as the Python loop would: the same sites, the same
acceptances, the same samples (the sampling functions are called on the host with the
state brought back after each sampled pass) and the same final engine state.  The
system may hold this package's numpy calculators or the ``ising_cpp`` ones, as in the
reference.  An event generator other than ``SemiGrandCanonicalEventGenerator`` runs its
``propose``/``apply`` callbacks in the reference's loop on the host (user code cannot
run on the GPU).
"""
from __future__ import annotations

import copy
import json
import math
import os
from typing import Any, Callable, Optional

import numpy as np

from ... import MethodLog, RandomNumberEngine, RandomNumberGenerator, ValueMap
from ...events import OccEvent
from ...ising_cpp.semigrand_canonical import _ReplayDriver
from ...sampling import (CompletionCheck, CompletionCheckParams, Sampler, StateSamplingFunction,
                         StateSamplingFunctionMap, get_n_samples, jsonSamplerMap, jsonStateSamplingFunctionMap,
                         scalar_as_vector)
from .. import IsingFormationEnergy, IsingParamComposition, IsingState, IsingSystem

KB = 8.6173303e-05  # eV/K (libcasm-global's KB)


class SemiGrandCanonicalConditions:
    """Temperature and exchange potential (_methods.py:37-92)."""

    def __init__(self, temperature: float, exchange_potential: np.ndarray):
        self.temperature: float = temperature
        self.exchange_potential: np.ndarray = exchange_potential

    @staticmethod
    def from_values(values: ValueMap) -> "SemiGrandCanonicalConditions":
        if "temperature" not in values.scalar_values:
            raise Exception('Missing required condition: "temperature"')
        if "exchange_potential" not in values.vector_values:
            raise Exception('Missing required condition: "exchange_potential"')
        return SemiGrandCanonicalConditions(temperature=values.scalar_values["temperature"],
                                            exchange_potential=values.vector_values["exchange_potential"])

    def to_values(self) -> ValueMap:
        values = ValueMap()
        values.scalar_values["temperature"] = self.temperature
        values.vector_values["exchange_potential"] = self.exchange_potential
        return values

    @staticmethod
    def from_dict(data: dict) -> "SemiGrandCanonicalConditions":
        return SemiGrandCanonicalConditions.from_values(ValueMap.from_dict(data))

    def to_dict(self) -> dict:
        return self.to_values().to_dict()


class SemiGrandCanonicalPotential:
    """E_sgc = E_f - mu . N x and its change (_methods.py:95-194)."""

    def __init__(self, system: IsingSystem):
        self.system = system
        self.formation_energy_calculator = copy.deepcopy(system.formation_energy_calculator)
        self.param_composition_calculator = copy.deepcopy(system.param_composition_calculator)
        self.state: Optional[IsingState] = None
        self.conditions: Optional[SemiGrandCanonicalConditions] = None

    def set_state(self, state: IsingState, conditions: SemiGrandCanonicalConditions) -> None:
        self.state = state
        self.conditions = conditions
        self.formation_energy_calculator.set_state(state)
        self.param_composition_calculator.set_state(state)

    def per_supercell(self) -> float:
        mu_exchange = self.conditions.exchange_potential
        E_f = self.formation_energy_calculator.per_supercell()
        Nx = self.param_composition_calculator.per_supercell()
        return E_f - mu_exchange @ Nx

    def per_unitcell(self) -> float:
        return self.per_supercell() / self.state.configuration.n_unitcells

    def occ_delta_per_supercell(self, linear_site_index, new_occ) -> float:
        dE_f = self.formation_energy_calculator.occ_delta_per_supercell(linear_site_index, new_occ)
        mu_exchange = self.conditions.exchange_potential
        Ndx = self.param_composition_calculator.occ_delta_per_supercell(linear_site_index, new_occ)
        return dE_f - mu_exchange @ Ndx


class SemiGrandCanonicalData:
    """Samplers, counters and completion check of a run (_methods.py:197-299)."""

    def __init__(self, sampling_functions: StateSamplingFunctionMap, n_steps_per_pass: int,
                 completion_check_params: CompletionCheckParams):
        self.sampling_functions = sampling_functions
        self.samplers = {f.name: Sampler(f.shape, f.component_names) for f in sampling_functions.values()}
        self.sample_weight = Sampler([])
        self.n_pass: int = 0
        self.n_steps_per_pass: int = int(n_steps_per_pass)
        self.n_accept: int = 0
        self.n_reject: int = 0
        self.completion_check = CompletionCheck(completion_check_params)
        # no JSON samplers in this calculator (the GPU loop shares its code with ising_cpp)
        self.json_sampling_functions = jsonStateSamplingFunctionMap()
        self.json_samplers = jsonSamplerMap()

    def acceptance_rate(self) -> float:
        return float(self.n_accept) / (float(self.n_accept) + float(self.n_reject))

    def rejection_rate(self) -> float:
        return float(self.n_reject) / (float(self.n_accept) + float(self.n_reject))

    def reset(self) -> None:
        for sampler in self.samplers.values():
            sampler.clear()
        self.sample_weight.clear()
        self.n_pass = 0
        self.n_accept = 0
        self.n_reject = 0
        self.completion_check.reset()

    def to_dict(self) -> dict:
        return {"completion_check_results": self.completion_check.results().to_dict(), "n_pass": self.n_pass,
                "n_steps_per_pass": self.n_steps_per_pass, "n_accept": self.n_accept, "n_reject": self.n_reject,
                "acceptance_rate": self.acceptance_rate(), "rejection_rate": self.rejection_rate()}


def default_write_status(mc_calculator: Any, method_log: MethodLog) -> None:
    """Passes, timing and current properties to stdout; completion-check results to the
    method log (_methods.py:302-405)."""
    data = mc_calculator.data
    completion_check = data.completion_check
    n_pass = data.n_pass
    n_samples = get_n_samples(data.samplers)
    n_variable_sites = mc_calculator.state.configuration.n_variable_sites
    np_formatter = {"float_kind": lambda x: f"{x:.4f}"}
    steps = n_pass * n_variable_sites
    time_s = method_log.time_s()
    print(f"Passes={n_pass}, Samples={n_samples}, ClockTime(s)={time_s:.2f}, "
          f"Steps/Second={steps / time_s:.2e}, Seconds/Step={time_s / steps:.2e}")
    x_str = np.array2string(mc_calculator.param_composition_calculator.per_unitcell(), formatter=np_formatter)
    ef = mc_calculator.formation_energy_calculator.per_unitcell()
    print(f"  ParametricComposition={x_str}, FormationEnergy={ef:.4e}")
    results = completion_check.results()

    def finish():
        method_log.reset()
        method_log.print(json.dumps(results.to_dict(), sort_keys=True, indent=2))
        method_log.begin_lap()

    all_equilibrated = results.equilibration_check_results.all_equilibrated
    print(f"  AllEquilibrated={all_equilibrated}")
    if not all_equilibrated:
        finish()
        return
    all_converged = results.convergence_check_results.all_converged
    print(f"  AllConverged={all_converged}")
    if all_converged:
        finish()
        return
    converge_results = results.convergence_check_results.individual_results
    for key, req in completion_check.params().requested_precision.items():
        stats = converge_results[key].stats
        abs_prec = stats.calculated_precision
        rel_prec = math.fabs(abs_prec / stats.mean)
        if req.abs_convergence_is_required:
            print(f"  - {key.sampler_name}({key.component_index}): mean={stats.mean:.4e}, "
                  f"abs_prec={abs_prec:.4e} < requested={req.abs_precision:.4e} == {abs_prec < req.abs_precision}")
        if req.rel_convergence_is_required:
            print(f"  - {key.sampler_name}({key.component_index}): mean={stats.mean:.4e}, "
                  f"rel_prec={rel_prec:.4e} < requested={req.rel_precision:.4e} == {rel_prec < req.rel_precision}")
    finish()


class SemiGrandCanonicalEventGenerator:
    """Random single-site flip (_methods.py:408-491): site ``random_int(N - 1)``, new
    value minus the current one."""

    def __init__(self, state: Optional[IsingState] = None):
        e = OccEvent()
        e.linear_site_index = [0]
        e.new_occ = [1]
        self.occ_event = e
        self.state: Optional[IsingState] = None
        if state is not None:
            self.set_state(state)

    def set_state(self, state: IsingState) -> None:
        self.state = state
        self._max_linear_site_index = self.state.configuration.n_variable_sites - 1

    def propose(self, random_number_generator: RandomNumberGenerator) -> OccEvent:
        self.occ_event.linear_site_index[0] = random_number_generator.random_int(self._max_linear_site_index)
        self.occ_event.new_occ[0] = -self.state.configuration.occ(self.occ_event.linear_site_index[0])
        return self.occ_event

    def apply(self, occ_event: OccEvent) -> None:
        self.state.configuration.set_occ(occ_event.linear_site_index[0], occ_event.new_occ[0])


def _composition_scale(param_composition_calculator) -> float:
    """Change of N x for one flip of +1 -> -1 in units of the replay kernel's
    (new - old) / 2: 2 for this module's calculator (its change is new - old), 1 for the
    ``ising_cpp`` one."""
    return 2.0 if isinstance(param_composition_calculator, IsingParamComposition) else 1.0


class SemiGrandCanonicalCalculator(_ReplayDriver):
    """Semi-grand canonical Monte Carlo calculator (_methods.py:494-724)."""

    def __init__(self, system: IsingSystem):
        self.system = system
        self.potential: Optional[SemiGrandCanonicalPotential] = None
        self.formation_energy_calculator = None
        self.param_composition_calculator = None
        self.data: Optional[SemiGrandCanonicalData] = None
        self.state: Optional[IsingState] = None
        self.conditions: Optional[SemiGrandCanonicalConditions] = None

    def run(self, state: IsingState, sampling_functions: StateSamplingFunctionMap,
            completion_check_params: CompletionCheckParams, event_generator: SemiGrandCanonicalEventGenerator,
            sample_period: int = 1, method_log: Optional[MethodLog] = None,
            random_engine: Optional[RandomNumberEngine] = None, write_status_f: Optional[Callable] = None) -> None:
        """Run at one thermodynamic state; ``state`` is modified in place and the results
        are in :attr:`data`."""
        self.state = state
        self.conditions = SemiGrandCanonicalConditions.from_values(self.state.conditions)
        temperature = self.conditions.temperature
        n_steps_per_pass = self.state.configuration.n_variable_sites
        self.potential = SemiGrandCanonicalPotential(system=self.system)
        self.potential.set_state(self.state, self.conditions)
        self.formation_energy_calculator = self.potential.formation_energy_calculator
        self.param_composition_calculator = self.potential.param_composition_calculator
        event_generator = copy.deepcopy(event_generator)
        event_generator.set_state(state=self.state)
        self.data = data = SemiGrandCanonicalData(sampling_functions, n_steps_per_pass, completion_check_params)
        if random_engine is None:
            random_engine = RandomNumberEngine()
        if method_log is None:
            method_log = MethodLog(logfile_path=os.path.join(os.getcwd(), "status.json"), log_frequency=600)
        method_log.restart_clock()
        method_log.begin_lap()
        if write_status_f is None:
            write_status_f = default_write_status

        if type(event_generator) is SemiGrandCanonicalEventGenerator:
            mu = np.asarray(self.conditions.exchange_potential, dtype=float).reshape(-1)
            if mu.size != 1:
                raise Exception("Error in SemiGrandCanonicalCalculator.run: exchange_potential must have size 1")
            fe = self.formation_energy_calculator
            mu_kernel = float(mu[0]) * _composition_scale(self.param_composition_calculator)
            self._replay(data, float(fe.J), mu_kernel, float(temperature), bool(getattr(fe, "use_nlist", False)),
                         sample_period, method_log, random_engine, write_status_f, completion_check_params)
        else:
            self._host_loop(event_generator, temperature, sample_period, method_log, random_engine, write_status_f)
        write_status_f(self, method_log)

    def _host_loop(self, event_generator, temperature, sample_period, method_log, random_engine, write_status_f):
        """The reference's loop (_methods.py:660-720) for user-supplied event generators."""
        data = self.data
        beta = 1.0 / (KB * temperature)
        rng = RandomNumberGenerator(random_engine)
        n_pass_next_sample = sample_period
        n_step = 0
        while not data.completion_check.count_check(samplers=data.samplers, sample_weight=data.sample_weight,
                                                    count=data.n_pass, method_log=method_log):
            event = event_generator.propose(rng)
            dE = self.potential.occ_delta_per_supercell(event.linear_site_index, event.new_occ)
            if dE < 0.0:
                accept = True
            else:
                accept = rng.random_real(1.0) < math.exp(-dE * beta)
            if accept:
                data.n_accept += 1
                event_generator.apply(event)
            else:
                data.n_reject += 1
            n_step += 1
            if n_step == data.n_steps_per_pass:
                n_step = 0
                data.n_pass += 1
            if data.n_pass == n_pass_next_sample:
                n_pass_next_sample += sample_period
                for name, f in data.sampling_functions.items():
                    data.samplers[name].append(f())
                if method_log.log_frequency() is not None and method_log.lap_time() >= method_log.log_frequency():
                    write_status_f(self, method_log)


def make_param_composition_f(mc_calculator) -> StateSamplingFunction:
    """"param_composition": ``mc_calculator.param_composition_calculator.per_unitcell()``."""
    def f():
        return mc_calculator.param_composition_calculator.per_unitcell()

    return StateSamplingFunction(
        name="param_composition", description="Parametric composition",
        shape=[mc_calculator.system.param_composition_calculator.n_independent_compositions()], function=f)


def make_formation_energy_f(mc_calculator) -> StateSamplingFunction:
    """"formation_energy": ``mc_calculator.formation_energy_calculator.per_unitcell()``."""
    def f():
        return scalar_as_vector(mc_calculator.formation_energy_calculator.per_unitcell())

    return StateSamplingFunction(name="formation_energy", description="Intensive formation energy", shape=[],
                                 function=f)


def make_potential_energy_f(mc_calculator) -> StateSamplingFunction:
    """"potential_energy": ``mc_calculator.potential.per_unitcell()``."""
    def f():
        return scalar_as_vector(mc_calculator.potential.per_unitcell())

    return StateSamplingFunction(name="potential_energy", description="Intensive potential energy", shape=[],
                                 function=f)


__all__ = ["SemiGrandCanonicalCalculator", "SemiGrandCanonicalConditions", "SemiGrandCanonicalData",
           "SemiGrandCanonicalEventGenerator", "SemiGrandCanonicalPotential", "default_write_status",
           "make_formation_energy_f", "make_param_composition_f", "make_potential_energy_f"]
