"""Run management: sampling fixtures, run manager, results and their JSON files.

Mirrors include/casm/monte/run_management (RunManager.hh:19-241, SamplingFixture.hh:22-649,
Results.hh:14-355, ResultsAnalysisFunction.hh:20-141) and sampling/SamplingParams.hh:1-278,
with the JSON results writer of run_management/io/json/jsonResultsIO_impl.hh:1-555:

* ``SamplingParams`` / ``sample_at`` / ``stochastic_sample_at``: when the i-th sample of a
  fixture is taken (by step, pass or time; linear, logarithmic or custom spacing; optionally
  at stochastic intervals with the given mean rate)
* ``SamplingFixture``: one set of sampling functions with its counters, sample schedule,
  completion check, results, status log and results writer
* ``RunManager``: the fixtures of one run (complete when all are, or when any is with
  ``global_cutoff``), driven by a Monte Carlo loop such as
  ``methods.occupation_metropolis``
* ``jsonResultsIO``: ``summary.json`` (conditions, statistics, completion-check results and
  analysis, one entry appended per run) and ``run.<i>/trajectory.json`` /
  ``run.<i>/observations.json``
"""
from __future__ import annotations

import copy
import json
import math
import os
from typing import Callable, Optional

import numpy as np

from .. import MethodLog, RandomNumberEngine, RandomNumberGenerator, ValueMap
from ..sampling import (SAMPLE_METHOD, SAMPLE_MODE, CompletionCheck, CompletionCheckParams, Sampler,
                        SamplerComponent, SamplingParams, default_component_names, get_n_samples, jsonSampler)

__all__ = ["SamplingParams", "sample_at", "stochastic_count_step", "stochastic_time_step", "stochastic_sample_at",
           "MonteCounter", "ResultsAnalysisFunction", "make_analysis", "Results", "SamplingFixtureParams",
           "SamplingFixture", "RunManager", "jsonResultsIO", "memory_used_MiB"]


# ---- sampling schedule (SamplingParams.hh)

def sample_at(sample_index: int, s: SamplingParams) -> float:
    """Count or time of the sample_index-th sample (SamplingParams.hh:164-181)."""
    n = float(sample_index)
    if s.sample_method == SAMPLE_METHOD.LINEAR:
        return s.begin + s.period * n
    if s.sample_method == SAMPLE_METHOD.LOG:
        return s.begin + math.pow(s.base, n + s.shift)
    if s.custom_sample_at is None:
        raise RuntimeError("Error in sample_at: sample_method==SAMPLE_METHOD::CUSTOM and !custom_sample_at")
    return s.custom_sample_at(n)


def stochastic_count_step(sample_rate: float, random_number_generator) -> int:
    """Steps or passes to the next sample: each one sampled with probability sample_rate
    (SamplingParams.hh:194-206)."""
    dn = 1
    while True:
        if random_number_generator.random_real(1.0) < sample_rate:
            return dn
        dn += 1


def stochastic_time_step(sample_rate: float, random_number_generator) -> float:
    """-ln(R) / sample_rate (SamplingParams.hh:215-221)."""
    return -math.log(random_number_generator.random_real(1.0)) / sample_rate


def stochastic_sample_at(sample_index: int, s: SamplingParams, random_number_generator, sample_count,
                         sample_time) -> float:
    """Next sample at a stochastic interval with the schedule's local rate
    (SamplingParams.hh:241-273)."""
    if sample_index == 0:
        return s.begin
    n = float(sample_index)
    if s.sample_method == SAMPLE_METHOD.LINEAR:
        rate = 1.0 / s.period
    elif s.sample_method == SAMPLE_METHOD.LOG:
        rate = 1.0 / (math.log(s.base) * math.pow(s.base, n + s.shift))
    else:
        # the reference's branch for custom spacing repeats its LOG test and so is never
        # taken, leaving the rate unset; the rate implied by custom_sample_at is used here
        if s.custom_sample_at is None:
            raise RuntimeError("Error in stochastic_sample_at: sample_method==SAMPLE_METHOD::CUSTOM and "
                               "!custom_sample_at")
        rate = 1.0 / (s.custom_sample_at(n + 1) - s.custom_sample_at(n))
    if s.sample_mode == SAMPLE_MODE.BY_TIME:
        return sample_time[-1] + stochastic_time_step(rate, random_number_generator)
    return sample_count[-1] + stochastic_count_step(rate, random_number_generator)


def memory_used_MiB() -> Optional[float]:
    """Resident set size of the process (Linux /proc), or None."""
    try:
        with open("/proc/self/status") as f:
            for line in f:
                if line.startswith("VmRSS:"):
                    return float(line.split()[1]) / 1024.0
    except OSError:
        pass
    return None


# ---- counters, results, analysis

class MonteCounter:
    """Step / pass / count / time counters (SamplingFixture.hh:95-166)."""

    def __init__(self):
        self.reset(SAMPLE_MODE.BY_PASS, 1)

    def reset(self, sample_mode: SAMPLE_MODE, steps_per_pass: int) -> None:
        self.sample_mode = sample_mode
        self.steps_per_pass = int(steps_per_pass)
        self.step = 0
        self.pass_ = 0
        self.count = 0
        self.time = 0.0
        self.n_accept = 0
        self.n_reject = 0

    @property
    def pass_count(self) -> int:
        return self.pass_

    def increment_n_accept(self) -> None:
        self.n_accept += 1

    def increment_n_reject(self) -> None:
        self.n_reject += 1

    def increment_step(self) -> None:
        self.step += 1
        if self.sample_mode == SAMPLE_MODE.BY_STEP:
            self.count += 1
        if self.step == self.steps_per_pass:
            self.pass_ += 1
            if self.sample_mode != SAMPLE_MODE.BY_STEP:
                self.count += 1
            self.step = 0

    def set_time(self, event_time: float) -> None:
        self.time = float(event_time)


class ResultsAnalysisFunction:
    """A function of the results evaluated when a run finishes (ResultsAnalysisFunction.hh:20-104)."""

    def __init__(self, name: str, description: str, shape, function: Callable, component_names=None):
        self.name = name
        self.description = description
        self.shape = list(shape)
        self.component_names = list(component_names) if component_names is not None else \
            default_component_names(self.shape)
        self.function = function

    def __call__(self, results: "Results") -> np.ndarray:
        return np.asarray(self.function(results), dtype=float).reshape(-1)


def make_analysis(results: "Results", analysis_functions: dict, analysis_names) -> dict:
    """Evaluate the named analysis functions; a failing one gives NaNs
    (ResultsAnalysisFunction.hh:111-138)."""
    analysis = {}
    for name in analysis_names:
        f = analysis_functions.get(name)
        if f is None:
            continue
        try:
            analysis[f.name] = f(results)
        except Exception:
            analysis[f.name] = np.full(len(f.component_names), np.nan)
    return analysis


class Results:
    """Sampled data and run summary of one sampling fixture (Results.hh:14-160)."""

    def __init__(self, sampler_names, sampling_functions, json_sampler_names, json_sampling_functions,
                 analysis_functions):
        self.sampler_names = list(sampler_names)
        self.sampling_functions = sampling_functions
        self.json_sampler_names = list(json_sampler_names)
        self.json_sampling_functions = json_sampling_functions
        self.analysis_functions = analysis_functions
        self.reset()

    def reset(self) -> None:
        self.initial_memory_used_MiB: Optional[float] = None
        self.final_memory_used_MiB: Optional[float] = None
        self.elapsed_clocktime: Optional[float] = None
        self.samplers: dict = {}
        self.json_samplers: dict = {}
        self.analysis: dict = {}
        self.sample_count: list = []
        self.sample_time: list = []
        self.sample_weight = Sampler([])
        self.sample_clocktime: list = []
        self.sample_trajectory: list = []
        self.completion_check_results = None
        self.n_accept = 0
        self.n_reject = 0
        for name in self.sampler_names:
            if name not in self.sampling_functions:
                raise RuntimeError(f"Results::reset error.\nFailed to find sampling function '{name}'.")
            f = self.sampling_functions[name]
            self.samplers[f.name] = Sampler(f.shape, f.component_names)
        for name in self.json_sampler_names:
            if name not in self.json_sampling_functions:
                raise RuntimeError(f"Results::reset error.\nFailed to find json sampling function '{name}'.")
            self.json_samplers[self.json_sampling_functions[name].name] = jsonSampler()


def _is_auto_converge_mode(results: Results) -> bool:
    return len(results.completion_check_results.params.requested_precision) != 0


def _N_samples_for_statistics(results: Results) -> int:
    if _is_auto_converge_mode(results):
        return results.completion_check_results.convergence_check_results.N_samples_for_statistics
    return get_n_samples(results.samplers)


def _acceptance_rate(results: Results) -> float:
    tot = float(results.n_accept) + float(results.n_reject)
    return float(results.n_accept) / tot if tot else float("nan")


def _quantity_stats(name: str, sampler: Sampler, results: Results):
    """Per component: (is_converged or None, statistics or None) (Results.hh:244-322)."""
    ccr = results.completion_check_results
    calc = ccr.params.calc_statistics_f
    if calc is None:
        raise RuntimeError("Error in QuantityStats: calc_statistics_f == nullptr")
    out = []
    weight = results.sample_weight
    for i, cname in enumerate(sampler.component_names()):
        key = SamplerComponent(name, i, cname)
        requested = key in ccr.params.requested_precision
        if _is_auto_converge_mode(results):
            n_stats = _N_samples_for_statistics(results)
            if n_stats == 0:
                out.append((False if requested else None, None))
            elif requested:
                r = ccr.convergence_check_results.individual_results[key]
                out.append((r.is_converged, r.stats))
            else:
                obs = sampler.component(i)[-n_stats:]
                w = weight.component(0)[-n_stats:] if weight.n_samples() else np.zeros(0)
                out.append((None, calc(obs, w)))
        else:
            obs = sampler.component(i)
            w = weight.component(0) if weight.n_samples() else np.zeros(0)
            out.append((None, calc(obs, w)))
    return out


# ---- sampling fixture

class SamplingFixtureParams:
    """Parameters of one sampling fixture (SamplingFixture.hh:22-93)."""

    def __init__(self, label: str, sampling_functions, json_sampling_functions, analysis_functions,
                 sampling_params: SamplingParams, completion_check_params: CompletionCheckParams,
                 analysis_names=None, results_io: Optional["jsonResultsIO"] = None,
                 method_log: Optional[MethodLog] = None):
        self.label = label
        self.sampling_functions = sampling_functions
        self.json_sampling_functions = json_sampling_functions
        self.analysis_functions = analysis_functions if analysis_functions is not None else {}
        self.sampling_params = sampling_params
        self.completion_check_params = completion_check_params
        self.analysis_names = list(analysis_names or [])
        self.results_io = results_io
        self.method_log = method_log if method_log is not None else MethodLog()
        for name in sampling_params.sampler_names:
            if name not in sampling_functions:
                raise RuntimeError(f"SamplingFixtureParams constructor error: No sampling function for '{name}'")
        for name in sampling_params.json_sampler_names:
            if name not in json_sampling_functions:
                raise RuntimeError(f"SamplingFixtureParams constructor error: No sampling function for '{name}'")


class SamplingFixture:
    """Counters, sample schedule, completion check and results of one set of sampling
    functions (SamplingFixture.hh:168-649)."""

    def __init__(self, params: SamplingFixtureParams, engine: RandomNumberEngine):
        self._params = params
        self._rng = RandomNumberGenerator(engine)
        self._n_samples = 0
        self._count = 0
        self._is_complete = False
        self._counter = MonteCounter()
        self._completion_check = CompletionCheck(params.completion_check_params)
        self._results = Results(params.sampling_params.sampler_names, params.sampling_functions,
                                params.sampling_params.json_sampler_names, params.json_sampling_functions,
                                params.analysis_functions)
        self._next_sample_count = 0
        self._next_sample_time = 0.0
        self.sampling_functions: dict = {}
        self.json_sampling_functions: dict = {}

    def label(self) -> str:
        return self._params.label

    def params(self) -> SamplingFixtureParams:
        return self._params

    def counter(self) -> MonteCounter:
        return self._counter

    def results(self) -> Results:
        return self._results

    def initialize(self, steps_per_pass: int) -> None:
        p = self._params
        sp = p.sampling_params
        self._n_samples = 0
        self._count = 0
        self._is_complete = False
        self._counter.reset(sp.sample_mode, steps_per_pass)
        self._completion_check.reset()
        self._results.reset()
        self._results.initial_memory_used_MiB = memory_used_MiB()
        if sp.sample_mode == SAMPLE_MODE.BY_TIME:
            self._next_sample_count = 0
            self._next_sample_time = self.sample_at(len(self._results.sample_time))
            if self._next_sample_time < 0.0:
                raise RuntimeError("Error: sampling period parameter error, next_sample_time < 0.0")
        else:
            self._next_sample_time = 0.0
            self._next_sample_count = _round_count(self.sample_at(len(self._results.sample_count)))
            if self._next_sample_count < 0:
                raise RuntimeError("Error: sampling period parameter error, next_sample_count < 0")
        self.sampling_functions = {}
        for name in sp.sampler_names:
            if name not in p.sampling_functions:
                raise RuntimeError(f"Sampling parameters error: No sampling function for '{name}'")
            self.sampling_functions[name] = p.sampling_functions[name]
        self.json_sampling_functions = {}
        for name in sp.json_sampler_names:
            if name not in p.json_sampling_functions:
                raise RuntimeError(f"Sampling parameters error: No json sampling function for '{name}'")
            self.json_sampling_functions[name] = p.json_sampling_functions[name]
        p.method_log.restart_clock()
        p.method_log.begin_lap()

    def is_complete(self) -> bool:
        if self._is_complete:
            return True
        r = self._results
        log = self._params.method_log
        if self._params.sampling_params.do_sample_time:
            self._is_complete = self._completion_check.count_and_time_check(
                r.samplers, r.sample_weight, self._counter.count, self._counter.time, log)
        else:
            self._is_complete = self._completion_check.count_check(r.samplers, r.sample_weight, self._counter.count,
                                                                   log)
        return self._is_complete

    def completion_check_results(self):
        return self._completion_check.results()

    def write_status(self, run_index: int) -> None:
        log = self._params.method_log
        if not log.logfile_path():
            return
        log.reset()
        log.write_json({"run_index": run_index, "time": log.time_s(),
                        "completion_check_results": self._completion_check.results().to_dict()})
        log.begin_lap()

    def write_status_if_due(self, run_index: int) -> None:
        log = self._params.method_log
        freq = log.log_frequency()
        if freq is None:
            return
        n = get_n_samples(self._results.samplers)
        if self._n_samples != n or self._count != self._counter.count:
            self._n_samples = n
            self._count = self._counter.count
            if log.lap_time() > freq:
                self.write_status(run_index)

    def increment_n_accept(self) -> None:
        self._counter.increment_n_accept()

    def increment_n_reject(self) -> None:
        self._counter.increment_n_reject()

    def increment_step(self) -> None:
        self._counter.increment_step()

    def set_time(self, event_time: float) -> None:
        self._counter.set_time(event_time)

    def push_back_sample_weight(self, weight: float) -> None:
        self._results.sample_weight.append(np.array([float(weight)]))

    def next_sample_count(self) -> int:
        return self._next_sample_count

    def next_sample_time(self) -> float:
        return self._next_sample_time

    def sample_data(self, state) -> None:
        r = self._results
        sp = self._params.sampling_params
        c = self._counter
        r.sample_count.append(c.count)
        if sp.do_sample_time:
            r.sample_time.append(c.time)
        r.sample_clocktime.append(self._params.method_log.time_s())
        if sp.do_sample_trajectory:
            r.sample_trajectory.append(copy.deepcopy(state.configuration))
        for name in sp.sampler_names:
            if name not in self.sampling_functions:
                raise RuntimeError(f"Error in SamplingFixture::sample_data: did not find sampling function '{name}'")
            r.samplers[name].append(self.sampling_functions[name]())
        for name in sp.json_sampler_names:
            if name not in self.json_sampling_functions:
                raise RuntimeError("Error in SamplingFixture::sample_data: did not find json sampling "
                                   f"function'{name}'")
            r.json_samplers[name].values.append(self.json_sampling_functions[name]())
        if sp.sample_mode == SAMPLE_MODE.BY_TIME:
            self._next_sample_time = self.sample_at(len(r.sample_time))
            if self._next_sample_time <= c.time:
                raise RuntimeError("Error: state sampling period parameter error, next_sample_time <= current time")
        else:
            self._next_sample_count = _round_count(self.sample_at(len(r.sample_count)))
            if self._next_sample_count <= c.count:
                raise RuntimeError("Error: state sampling period parameter error, next_sample_count <= current count")

    def sample_data_by_count_if_due(self, state) -> None:
        if self._params.sampling_params.sample_mode != SAMPLE_MODE.BY_TIME and \
                self._counter.count == self._next_sample_count:
            self.sample_data(state)

    def sample_at(self, sample_index: int) -> float:
        sp = self._params.sampling_params
        if sp.stochastic_sample_period:
            return stochastic_sample_at(sample_index, sp, self._rng, self._results.sample_count,
                                        self._results.sample_time)
        return sample_at(sample_index, sp)

    def finalize(self, state, run_index: int) -> None:
        r = self._results
        r.final_memory_used_MiB = memory_used_MiB()
        r.elapsed_clocktime = self._params.method_log.time_s()
        r.completion_check_results = self._completion_check.results()
        r.analysis = make_analysis(r, self._params.analysis_functions, self._params.analysis_names)
        r.n_accept = self._counter.n_accept
        r.n_reject = self._counter.n_reject
        if self._params.results_io is not None:
            self._params.results_io.write(r, state.conditions, run_index)
        self.write_status(run_index)


def _round_count(x: float) -> int:
    """std::round to an integer count (halfway cases away from zero)."""
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


# ---- run manager

class RunManager:
    """Sampling fixtures of one run (RunManager.hh:19-238)."""

    def __init__(self, engine: RandomNumberEngine, sampling_fixture_params, global_cutoff: bool = True):
        if engine is None:
            raise RuntimeError("Error constructing RunManager: engine==nullptr")
        self.run_index = 0
        self.engine = engine
        self.sampling_fixtures = [SamplingFixture(p, engine) for p in sampling_fixture_params]
        self.global_cutoff = bool(global_cutoff)
        self.next_sampling_fixture: Optional[SamplingFixture] = None
        self.next_sample_time = 0.0
        #: label -> f(fixture, state) -> bool: a true value sets a break point
        self.break_point_checks: dict = {}
        self.break_point_set = False

    def initialize(self, steps_per_pass: int) -> None:
        for f in self.sampling_fixtures:
            f.initialize(steps_per_pass)
        self.break_point_set = False

    def is_break_point(self) -> bool:
        return self.break_point_set

    def is_complete(self) -> bool:
        # every fixture is checked (status files then carry the latest results)
        all_complete, any_complete = True, False
        for f in self.sampling_fixtures:
            if f.is_complete():
                any_complete = True
            else:
                all_complete = False
        if self.global_cutoff and any_complete:
            return True
        return all_complete

    def write_status_if_due(self) -> None:
        for f in self.sampling_fixtures:
            f.write_status_if_due(self.run_index)

    def increment_n_accept(self) -> None:
        for f in self.sampling_fixtures:
            f.increment_n_accept()

    def increment_n_reject(self) -> None:
        for f in self.sampling_fixtures:
            f.increment_n_reject()

    def increment_step(self) -> None:
        for f in self.sampling_fixtures:
            f.increment_step()

    def set_time(self, event_time: float) -> None:
        for f in self.sampling_fixtures:
            f.set_time(event_time)

    def sample_data_by_count_if_due(self, state, pre_sample_f: Optional[Callable] = None,
                                    post_sample_f: Optional[Callable] = None) -> None:
        for f in self.sampling_fixtures:
            if f.params().sampling_params.sample_mode != SAMPLE_MODE.BY_TIME and \
                    f.counter().count == f.next_sample_count():
                if pre_sample_f is not None:
                    pre_sample_f(f, state)
                f.sample_data(state)
                if post_sample_f is not None:
                    post_sample_f(f, state)
                check = self.break_point_checks.get(f.label())
                if check is not None:
                    self.break_point_set = bool(check(f, state))

    def sample_data_by_time_if_due(self, event_time: float, state, pre_sample_f: Optional[Callable] = None,
                                   post_sample_f: Optional[Callable] = None) -> None:
        while self.next_sampling_fixture is not None and event_time >= self.next_sample_time:
            f = self.next_sampling_fixture
            if pre_sample_f is not None:
                pre_sample_f(f, state)
            f.set_time(self.next_sample_time)
            f.sample_data(state)
            if post_sample_f is not None:
                post_sample_f(f, state)
            check = self.break_point_checks.get(f.label())
            if check is not None:
                self.break_point_set = bool(check(f, state))
            self.update_next_sampling_fixture()

    def update_next_sampling_fixture(self) -> None:
        self.next_sampling_fixture = None
        for f in self.sampling_fixtures:
            if f.params().sampling_params.sample_mode == SAMPLE_MODE.BY_TIME:
                if self.next_sampling_fixture is None or f.next_sample_time() < self.next_sample_time:
                    self.next_sample_time = f.next_sample_time()
                    self.next_sampling_fixture = f

    def finalize(self, final_state) -> None:
        for f in self.sampling_fixtures:
            f.finalize(final_state, self.run_index)


# ---- JSON results files (jsonResultsIO_impl.hh)

def _component_names_for(name: str, shape: list, sampling_functions) -> list:
    """Component names of a condition from the sampling function of the same name, else
    the defaults (StateSamplingFunction.hh:130-205)."""
    f = sampling_functions.get(name) if sampling_functions is not None else None
    n = 1
    for d in shape:
        n *= d
    if f is None:
        return default_component_names(shape)
    if len(f.component_names) != n:
        raise RuntimeError(f'Error in get_component_names: Dimension of "{name}" ({n}) does not match the '
                           "corresponding sampling function.")
    return list(f.component_names)


def _append_condition(name: str, value: np.ndarray, shape: list, component_names: list, js: dict) -> None:
    j = js.setdefault(name, {})
    j["shape"] = list(shape)
    if len(shape) == 0:
        j.setdefault("value", []).append(float(value[0]))
    else:
        j["component_names"] = list(component_names)
        for i, cname in enumerate(component_names):
            j.setdefault(cname, []).append(float(value[i]))


def _stats_arrays(stats, js: dict) -> None:
    js.setdefault("mean", [])
    js.setdefault("calculated_precision", [])
    if stats is None:
        js["mean"].append(None)
        js["calculated_precision"].append(None)
    else:
        js["mean"].append(float(stats.mean))
        js["calculated_precision"].append(float(stats.calculated_precision))


def _json_value(x):
    if isinstance(x, float) and not math.isfinite(x):
        return None
    return x


class jsonResultsIO:
    """Results writer: ``summary.json`` in ``output_dir`` (one entry per run, appended)
    and ``run.<i>/trajectory.json`` / ``run.<i>/observations.json``."""

    def __init__(self, output_dir: str, write_trajectory: bool = False, write_observations: bool = False):
        self.output_dir = str(output_dir)
        self.write_trajectory_ = bool(write_trajectory)
        self.write_observations_ = bool(write_observations)

    def to_dict(self) -> dict:
        return {"method": "json", "kwargs": {"output_dir": self.output_dir, "write_trajectory": self.write_trajectory_,
                                             "write_observations": self.write_observations_}}

    def write(self, results: Results, conditions: ValueMap, run_index: int) -> None:
        self.write_summary(results, conditions)
        if self.write_trajectory_:
            self.write_trajectory(results, run_index)
        if self.write_observations_:
            self.write_observations(results, run_index)

    def read_summary(self) -> dict:
        path = os.path.join(self.output_dir, "summary.json")
        if not os.path.exists(path):
            return {"conditions": {}, "statistics": {}, "completion_check_results": {}}
        with open(path) as f:
            return json.load(f)

    def run_dir(self, run_index: int) -> str:
        d = os.path.join(self.output_dir, f"run.{run_index}")
        os.makedirs(d, exist_ok=True)
        return d

    def write_summary(self, results: Results, conditions: ValueMap) -> None:
        js = self.read_summary()
        for key in ("conditions", "statistics", "completion_check_results", "analysis"):
            if key not in js:
                js[key] = {}
            elif not isinstance(js[key], dict):
                raise RuntimeError(f'JSON Error: "{key}" is expected to be an object.')
        sf = results.sampling_functions
        for name in sorted(conditions.scalar_values):
            v = conditions.scalar_values[name]
            _append_condition(name, np.array([v]), [], _component_names_for(name, [], sf), js["conditions"])
        for name in sorted(conditions.vector_values):
            v = np.asarray(conditions.vector_values[name], dtype=float).reshape(-1)
            _append_condition(name, v, [v.size], _component_names_for(name, [v.size], sf), js["conditions"])
        for name in sorted(getattr(conditions, "matrix_values", {})):
            m = np.asarray(conditions.matrix_values[name], dtype=float)
            shape = list(m.shape)
            _append_condition(name, m.reshape(-1, order="F"), shape, _component_names_for(name, shape, sf),
                              js["conditions"])
        # statistics of every sampled quantity
        for name in sorted(results.samplers):
            sampler = results.samplers[name]
            qj = js["statistics"].setdefault(name, {})
            qj["shape"] = list(sampler.shape())
            comp = _quantity_stats(name, sampler, results)
            if len(sampler.shape()) == 0:
                vj = qj.setdefault("value", {})
                conv, st = comp[0]
                _stats_arrays(st, vj)
                if conv is not None:
                    vj.setdefault("is_converged", []).append(bool(conv))
            else:
                qj["component_names"] = list(sampler.component_names())
                for i, cname in enumerate(sampler.component_names()):
                    cj = qj.setdefault(cname, {})
                    conv, st = comp[i]
                    _stats_arrays(st, cj)
                    if conv is not None:
                        cj.setdefault("is_converged", []).append(bool(conv))
        # completion check results
        cj = js["completion_check_results"]
        ccr = results.completion_check_results
        if _is_auto_converge_mode(results):
            eq = ccr.equilibration_check_results
            cj.setdefault("all_equilibrated", []).append(bool(eq.all_equilibrated))
            cj.setdefault("all_converged", []).append(bool(ccr.convergence_check_results.all_converged))
            cj.setdefault("N_samples_for_all_to_equilibrate", []).append(
                int(eq.N_samples_for_all_to_equilibrate) if eq.all_equilibrated else "did_not_equilibrate")
        cj.setdefault("N_samples", []).append(get_n_samples(results.samplers))
        cj.setdefault("N_samples_for_statistics", []).append(_N_samples_for_statistics(results))
        cj.setdefault("acceptance_rate", []).append(_json_value(_acceptance_rate(results)))
        cj.setdefault("initial_memory_used_MiB", []).append(results.initial_memory_used_MiB)
        cj.setdefault("final_memory_used_MiB", []).append(results.final_memory_used_MiB)
        cj.setdefault("elapsed_clocktime", []).append(results.elapsed_clocktime)
        cj.setdefault("count", []).append(results.sample_count[-1] if results.sample_count else None)
        if results.sample_time:
            cj.setdefault("time", []).append(results.sample_time[-1])
        # analysis
        aj = js["analysis"]
        not_eq = _is_auto_converge_mode(results) and not ccr.equilibration_check_results.all_equilibrated
        for name in sorted(results.analysis):
            value = results.analysis[name]
            f = results.analysis_functions.get(name)
            if f is None:
                raise RuntimeError(f"Error in append_results_analysis_to_json: No matching analysis function found "
                                   f"for '{name}'.")
            vj = aj.setdefault(name, {})
            vj["shape"] = list(f.shape)
            if len(f.shape) == 0:
                vj.setdefault("value", []).append("did_not_equilibrate" if not_eq else _json_value(float(value[0])))
            else:
                vj["component_names"] = list(f.component_names)
                for i, cname in enumerate(f.component_names):
                    vj.setdefault(cname, []).append("did_not_equilibrate" if not_eq else _json_value(float(value[i])))
        os.makedirs(self.output_dir, exist_ok=True)
        path = os.path.join(self.output_dir, "summary.json")
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(js, f)
        os.replace(tmp, path)

    def write_trajectory(self, results: Results, run_index: int) -> None:
        with open(os.path.join(self.run_dir(run_index), "trajectory.json"), "w") as f:
            json.dump([c.to_dict() for c in results.sample_trajectory], f)

    def write_observations(self, results: Results, run_index: int) -> None:
        js: dict = {}
        if results.sample_count:
            js["count"] = [int(x) for x in results.sample_count]
        if results.sample_time:
            js["time"] = [float(x) for x in results.sample_time]
        if results.sample_weight.n_samples():
            js["weight"] = results.sample_weight.component(0).tolist()
        if results.sample_clocktime:
            js["clocktime"] = [float(x) for x in results.sample_clocktime]
        for name in sorted(results.samplers):
            s = results.samplers[name]
            j = js.setdefault(name, {})
            j["shape"] = list(s.shape())
            if len(s.shape()) == 0:
                j["value"] = s.component(0).tolist()
            else:
                j["component_names"] = list(s.component_names())
                j["value"] = s.values().tolist()
        for name in sorted(results.json_samplers):
            js.setdefault(name, {})["value"] = results.json_samplers[name].values
        with open(os.path.join(self.run_dir(run_index), "observations.json"), "w") as f:
            json.dump(js, f)
