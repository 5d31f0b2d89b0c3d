"""Monte Carlo methods (libcasm.monte.methods, python/libcasm/monte/methods/__init__.py:3-9).

* ``metropolis_acceptance`` (python/libcasm/monte/methods/_metropolis.py:6-48,
  include/casm/monte/methods/metropolis.hh:26-35): accept if dE < 0 without drawing,
  else accept if ``random_real(1.0) < exp(-dE * beta)``.
* ``occupation_metropolis`` (include/casm/monte/methods/occupation_metropolis.hh:90-154):
  the same loop over an ``OccLocation`` with a proposal function over possible swaps,
  tracking the potential energy per unit cell in ``state.properties`` and sampling through
  a ``run_management.RunManager`` (sampling fixtures, completion checks, results files).
* ``BasicOccupationMetropolisData`` and ``basic_occupation_metropolis``
  (include/casm/monte/methods/basic_occupation_metropolis.hh:18-115, 354-425): the
  reference's generic Metropolis loop, parameterised by caller-supplied functions for the
  potential change, the proposal and the application of an event.  Because those
  functions are the caller's (any system, any event type), this loop is driven from the
  host and calls them once per step, as the reference's Python binding does through
  std::function (python/src/monte_methods.cpp).  The built-in systems run their loops on
  the GPU instead: ``casmcode_monte_gb300.ising_cpp.semigrand_canonical`` (serial replay
  of the reference's trajectory) and ``casmcode_monte_gb300.clex`` (coloured sweeps).
"""
from __future__ import annotations

import math
import sys
from typing import Callable, Optional

import numpy as np

from .. import MethodLog, RandomNumberEngine, RandomNumberGenerator, __version__  # noqa: F401
from ..events import OccEvent
from ..sampling import (CompletionCheck, CompletionCheckParams, Sampler, get_n_samples, jsonSampler,
                        jsonStateSamplingFunctionMap, StateSamplingFunctionMap)

__all__ = ["KB", "BasicOccupationMetropolisData", "basic_occupation_metropolis", "default_write_status",
           "metropolis_acceptance", "occupation_metropolis", "write_no_status", "NfoldData", "nfold", "KMCData",
           "kinetic_monte_carlo"]

KB = 8.6173303e-05  # eV/K (the reference's libcasm-global constant)


def metropolis_acceptance(delta_potential_energy: float, beta: float, random_number_generator) -> bool:
    """Metropolis acceptance (metropolis.hh:26-35): no random number is drawn for a
    decrease of the potential."""
    if delta_potential_energy < 0.0:
        return True
    return random_number_generator.random_real(1.0) < math.exp(-delta_potential_energy * beta)


class BasicOccupationMetropolisData:
    """Samplers, counters and completion check of a basic occupation Metropolis run
    (basic_occupation_metropolis.hh:18-115)."""

    def __init__(self, sampling_functions: StateSamplingFunctionMap,
                 json_sampling_functions: jsonStateSamplingFunctionMap, n_steps_per_pass: int,
                 completion_check_params: CompletionCheckParams):
        self.sampling_functions = sampling_functions
        self.json_sampling_functions = json_sampling_functions
        self.samplers = {f.name: Sampler(f.shape, f.component_names) for f in sampling_functions.values()}
        self.json_samplers = {f.name: jsonSampler() for f in json_sampling_functions.values()}
        self.sample_weight = Sampler([])
        self.n_pass = 0
        self.n_steps_per_pass = int(n_steps_per_pass)
        self.n_accept = 0
        self.n_reject = 0
        self.completion_check = CompletionCheck(completion_check_params)

    def acceptance_rate(self) -> float:
        total = float(self.n_accept) + float(self.n_reject)
        return float(self.n_accept) / total if total else float("nan")

    def rejection_rate(self) -> float:
        total = float(self.n_accept) + float(self.n_reject)
        return float(self.n_reject) / total if total else float("nan")

    def reset(self) -> None:
        for s in self.samplers.values():
            s.clear()
        for s in self.json_samplers.values():
            s.values.clear()
        self.sample_weight.clear()
        self.n_pass = 0
        self.n_accept = 0
        self.n_reject = 0
        self.completion_check.reset()

    def to_dict(self) -> dict:
        return {"completion_check_results": self.completion_check.results().to_dict(), "n_pass": self.n_pass,
                "n_steps_per_pass": self.n_steps_per_pass, "n_accept": int(self.n_accept),
                "n_reject": int(self.n_reject), "acceptance_rate": self.acceptance_rate(),
                "rejection_rate": self.rejection_rate()}


def write_no_status(data: BasicOccupationMetropolisData, method_log: MethodLog) -> None:
    method_log.begin_lap()


def default_write_status(data: BasicOccupationMetropolisData, method_log: MethodLog) -> None:
    """Run status (passes, samples, clock time, steps per second) and the latest
    completion-check results to stdout; the results to the method log's file."""
    n_samples = get_n_samples(data.samplers)
    t = method_log.time_s()
    steps = float(data.n_pass) * float(data.n_steps_per_pass)
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


def basic_occupation_metropolis(data: BasicOccupationMetropolisData, temperature: float,
                                potential_occ_delta_per_supercell_f: Callable, propose_event_f: Callable,
                                apply_event_f: Callable, sample_period: int = 1,
                                method_log: Optional[MethodLog] = None,
                                random_engine: Optional[RandomNumberEngine] = None,
                                write_status_f: Optional[Callable] = None) -> None:
    """Occupation Metropolis loop (basic_occupation_metropolis.hh:354-425).

    Until the completion check (with count = passes, checked before every step): propose an
    event with ``propose_event_f(rng)``, compute ``potential_occ_delta_per_supercell_f(e)``,
    accept by ``metropolis_acceptance`` and apply with ``apply_event_f(e)``; every
    ``n_steps_per_pass`` steps is a pass, and every ``sample_period`` passes each
    sampling function is sampled (status written when the method log's frequency is due).
    """
    beta = 1.0 / (KB * temperature)
    rng = RandomNumberGenerator(random_engine if random_engine is not None else RandomNumberEngine())
    if write_status_f is None:
        write_status_f = default_write_status
    if method_log is None:
        method_log = MethodLog(logfile_path="status.json", log_frequency=600.0)
    method_log.restart_clock()
    method_log.begin_lap()
    n_pass_next_sample = sample_period
    n_step = 0
    cc = data.completion_check
    while not cc.count_check(data.samplers, data.sample_weight, data.n_pass, method_log):
        event = propose_event_f(rng)
        dE = potential_occ_delta_per_supercell_f(event)
        if metropolis_acceptance(dE, beta, rng):
            data.n_accept += 1
            apply_event_f(event)
        else:
            data.n_reject += 1
        n_step += 1
        if n_step == data.n_steps_per_pass:
            n_step = 0
            data.n_pass += 1
        if data.n_pass == n_pass_next_sample:
            n_pass_next_sample += sample_period
            for f in data.sampling_functions.values():
                data.samplers[f.name].push_back(f())
            for f in data.json_sampling_functions.values():
                data.json_samplers[f.name].values.append(f())
            freq = method_log.log_frequency()
            if freq is not None and method_log.lap_time() >= freq:
                write_status_f(data, method_log)
    write_status_f(data, method_log)


def _occupation_array(state) -> np.ndarray:
    """The state's occupation as a writable array (the configurations of this package
    keep it in ``_occ`` or ``_occupation``; a plain array is used as it is)."""
    cfg = state.configuration
    for attr in ("_occ", "_occupation"):
        a = getattr(cfg, attr, None)
        if isinstance(a, np.ndarray):
            return a.reshape(-1, order="F") if a.ndim > 1 else a
    return cfg.occupation()


def occupation_metropolis(state, occ_location, potential, possible_swaps, propose_event_f: Callable,
                          random_number_generator, run_manager) -> None:
    """Occupation Metropolis Monte Carlo with run management (occupation_metropolis.hh:90-154).

    Until ``run_manager.is_complete()``: write status if due; propose an event with
    ``propose_event_f(event, occ_location, possible_swaps, random_number_generator)`` (an
    exception ends the run); ``dE = potential.occ_delta_per_supercell(sites, new_occ)``;
    Metropolis acceptance; an accepted event updates ``occ_location`` and the occupation
    and adds dE / n_unitcells to ``state.properties.scalar_values["potential_energy"]``;
    count the step; sample if due.  The run manager is initialized with
    ``occ_location.mol_size()`` steps per pass and finalized with the final state.
    """
    if getattr(potential, "state", None) is not state:
        raise RuntimeError("Error in monte::occupation_metropolis: potential not set to correct state")
    n_unitcells = float(state.configuration.n_unitcells)
    state.properties.scalar_values["potential_energy"] = potential.per_supercell() / n_unitcells
    beta = 1.0 / (KB * state.conditions.scalar_values["temperature"])
    occupation = _occupation_array(state)
    event = OccEvent()
    run_manager.initialize(occ_location.mol_size())
    run_manager.sample_data_by_count_if_due(state)
    while not run_manager.is_complete():
        run_manager.write_status_if_due()
        try:
            propose_event_f(event, occ_location, possible_swaps, random_number_generator)
        except Exception as e:  # the reference logs the error and ends the run
            sys.stderr.write(f"\nError proposing event: {e}\n")
            break
        dE = potential.occ_delta_per_supercell(event.linear_site_index, event.new_occ)
        if metropolis_acceptance(dE, beta, random_number_generator):
            run_manager.increment_n_accept()
            occ_location.apply(event, occupation)
            state.properties.scalar_values["potential_energy"] += dE / n_unitcells
        else:
            run_manager.increment_n_reject()
        run_manager.increment_step()
        run_manager.sample_data_by_count_if_due(state)
    run_manager.finalize(state)



# ---- rejection-free and kinetic loops (methods/nfold.hh, methods/kinetic_monte_carlo.hh)

def _member_copy(self, memo=None):
    """A copy whose members are the same objects (samplers, functions), as the reference's
    copy constructor copies shared pointers."""
    c = object.__new__(type(self))
    c.__dict__.update(self.__dict__)
    return c


BasicOccupationMetropolisData.__copy__ = _member_copy
BasicOccupationMetropolisData.__deepcopy__ = _member_copy


class NfoldData:
    """Data sampling functions can use during an N-fold way run (nfold.hh:24-44)."""

    def __init__(self, n_events_possible: float = 0.0):
        #: set to the current sampling fixture's label before it samples
        self.sampling_fixture_label = ""
        #: set to the sampling fixture before it samples
        self.sampling_fixture = None
        #: total number of events that could be selected at any time (set before running)
        self.n_events_possible = float(n_events_possible)
        #: total_rate / n_events_possible: the Metropolis acceptance rate the current
        #: event acceptance probabilities imply
        self.expected_acceptance_rate = 0.0


def _sample_mode_is_time(fixture) -> bool:
    from ..sampling import SAMPLE_MODE

    return fixture.params().sampling_params.sample_mode == SAMPLE_MODE.BY_TIME


def nfold(state, occ_location, nfold_data: NfoldData, event_selector, get_event_f: Callable, run_manager) -> None:
    """N-fold way occupation Monte Carlo with run management (nfold.hh:48-149).

    ``event_selector.total_rate()`` and ``event_selector.select_event() -> (event_id,
    time_increment)`` choose the next event without rejection (the selector updates the rates
    the last event changed); ``get_event_f(event_id) -> OccEvent`` gives the event to apply.
    Each step: write status if due; total rate, then selection; sample if due by count and by
    time (the samples' weight is the time increment, or 1.0 for fixtures that sample by
    time, whose time is then set to the sample time); apply the event (every selected event
    is accepted); advance time; count the step.  The run manager is initialized with
    ``occ_location.mol_size()`` steps per pass and finalized with the final state.
    """
    loop = {"total_rate": 0.0, "time": 0.0, "time_increment": 0.0}

    def pre_sample_action(fixture, state_):
        nfold_data.sampling_fixture_label = fixture.label()
        nfold_data.sampling_fixture = fixture
        nfold_data.expected_acceptance_rate = loop["total_rate"] / nfold_data.n_events_possible
        if _sample_mode_is_time(fixture):
            fixture.push_back_sample_weight(1.0)
            loop["time"] = fixture.next_sample_time()
        else:
            fixture.push_back_sample_weight(loop["time_increment"])

    occupation = _occupation_array(state)
    run_manager.initialize(occ_location.mol_size())
    run_manager.update_next_sampling_fixture()
    while not run_manager.is_complete():
        run_manager.write_status_if_due()
        loop["total_rate"] = event_selector.total_rate()
        selected_event_id, loop["time_increment"] = event_selector.select_event()
        event_time = loop["time"] + loop["time_increment"]
        run_manager.sample_data_by_count_if_due(state, pre_sample_action, None)
        run_manager.sample_data_by_time_if_due(event_time, state, pre_sample_action, None)
        run_manager.increment_n_accept()
        occ_location.apply(get_event_f(selected_event_id), occupation)
        loop["time"] = event_time
        run_manager.set_time(event_time)
        run_manager.increment_step()
    run_manager.finalize(state)


class KMCData:
    """Data sampling functions can use during a kinetic Monte Carlo run
    (kinetic_monte_carlo.hh:25-98): the total rate and time at sampling, the previous sample
    time per fixture, and atom positions now and at each fixture's previous sample (shape
    (3, n_atoms), Cartesian, following atoms across periodic boundaries)."""

    def __init__(self):
        self.sampling_fixture_label = ""
        self.sampling_fixture = None
        self.total_rate = 0.0
        self.time = 0.0
        self.prev_time: dict = {}
        self.unique_atom_id: list = []
        self.prev_unique_atom_id: dict = {}
        #: atom name index of each column of the position matrices (set by the caller)
        self.atom_name_index_list: list = []
        self.atom_positions_cart = np.zeros((3, 0))
        self.prev_atom_positions_cart: dict = {}


def kinetic_monte_carlo(state, occ_location, kmc_data: KMCData, event_selector, get_event_f: Callable,
                        run_manager) -> None:
    """Kinetic Monte Carlo with run management (kinetic_monte_carlo.hh:108-224).

    As ``nfold`` but the event is selected before the total rate is read (the selector
    updates rates after the last event, then chooses), and sampling functions see
    ``kmc_data``: before a sample its label, fixture, current atom positions, total rate and,
    for fixtures that sample by time, the sample time; after it the fixture's previous time
    and positions.  ``occ_location`` must track atoms (``update_atoms=True``).
    """
    kmc_data.time = 0.0
    kmc_data.atom_positions_cart = occ_location.atom_positions_cart()
    kmc_data.prev_atom_positions_cart = {}
    for fixture in run_manager.sampling_fixtures:
        kmc_data.prev_time.setdefault(fixture.label(), kmc_data.time)
        kmc_data.prev_atom_positions_cart.setdefault(fixture.label(), kmc_data.atom_positions_cart.copy())
    loop = {"total_rate": 0.0}

    def pre_sample_action(fixture, state_):
        kmc_data.sampling_fixture_label = fixture.label()
        kmc_data.sampling_fixture = fixture
        kmc_data.atom_positions_cart = occ_location.atom_positions_cart()
        kmc_data.total_rate = loop["total_rate"]
        if _sample_mode_is_time(fixture):
            kmc_data.time = fixture.next_sample_time()

    def post_sample_action(fixture, state_):
        kmc_data.prev_time[fixture.label()] = kmc_data.time
        kmc_data.prev_atom_positions_cart[fixture.label()] = kmc_data.atom_positions_cart.copy()

    occupation = _occupation_array(state)
    run_manager.initialize(occ_location.mol_size())
    run_manager.update_next_sampling_fixture()
    while not run_manager.is_complete():
        run_manager.write_status_if_due()
        selected_event_id, time_increment = event_selector.select_event()
        loop["total_rate"] = event_selector.total_rate()
        event_time = kmc_data.time + time_increment
        run_manager.sample_data_by_count_if_due(state, pre_sample_action, post_sample_action)
        run_manager.sample_data_by_time_if_due(event_time, state, pre_sample_action, post_sample_action)
        run_manager.increment_n_accept()
        occ_location.apply(get_event_f(selected_event_id), occupation)
        kmc_data.time = event_time
        run_manager.set_time(event_time)
        run_manager.increment_step()
    run_manager.finalize(state)
