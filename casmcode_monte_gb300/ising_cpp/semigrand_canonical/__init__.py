"""Semi-grand canonical Metropolis for the Ising model, run on the GPU.

Mirrors ``libcasm.monte.ising_cpp.semigrand_canonical``
(python/src/monte_ising_cpp_semigrand_canonical.cpp:65-599) and the C++ classes of
include/casm/monte/ising_cpp/basic_semigrand_canonical.hh:36-627.

``SemiGrandCanonicalCalculator.run`` executes the reference's main loop
(methods/basic_occupation_metropolis.hh:354-425) as a serial replay on the GPU: the
kernel consumes the caller's mt19937_64 engine exactly as the reference does (site draw,
acceptance draw only for dE >= 0), so occupations, samples, acceptance counts and the
final engine state are identical to the reference's.  The host drives the kernel in
chunks of whole passes and reproduces, call for call, the completion check the
reference evaluates before every step: samples and counts change only at pass
boundaries, so a chunk ends at the first pass boundary where that check could finish
the run or run a convergence check.
"""
from __future__ import annotations

import copy
import ctypes as C
import os
import sys
from typing import Callable, Optional

import numpy as np

from ... import MethodLog, RandomNumberEngine, ValueMap, __version__  # noqa: F401
from ... import _lib
from ...sampling import (CompletionCheck, CompletionCheckParams, Sampler, StateSamplingFunction,
                         StateSamplingFunctionMap, jsonSampler, jsonSamplerMap, jsonStateSamplingFunction,
                         jsonStateSamplingFunctionMap, get_n_samples)
from .. import IsingConfiguration, IsingFormationEnergy, IsingParamComposition, IsingState, IsingSystem

KB = 8.6173303e-05  # eV/K, CASM's Boltzmann constant (libcasm-global)

ENGINE_STATE_LEN = 16384


class SemiGrandCanonicalConditions:
    """Temperature and exchange potential (basic_semigrand_canonical.hh:36-80)."""

    def __init__(self, temperature: float = 0.0, exchange_potential=None):
        self.temperature = float(temperature)
        self.exchange_potential = np.asarray(exchange_potential if exchange_potential is not None else [],
                                             dtype=float)

    @staticmethod
    def from_values(values: ValueMap) -> "SemiGrandCanonicalConditions":
        if "temperature" not in values.scalar_values:
            raise RuntimeError('Missing required condition: "temperature"')
        if "exchange_potential" not in values.vector_values:
            raise RuntimeError('Missing required condition: "exchange_potential"')
        return SemiGrandCanonicalConditions(values.scalar_values["temperature"],
                                            values.vector_values["exchange_potential"])

    def to_values(self) -> ValueMap:
        v = ValueMap()
        v.scalar_values["temperature"] = self.temperature
        v.vector_values["exchange_potential"] = np.array(self.exchange_potential)
        return v

    def to_dict(self) -> dict:
        return self.to_values().to_dict()

    @staticmethod
    def from_dict(data: dict) -> "SemiGrandCanonicalConditions":
        return SemiGrandCanonicalConditions.from_values(ValueMap.from_dict(data))


class SemiGrandCanonicalPotential:
    """E_sgc = E_f - N mu . x (basic_semigrand_canonical.hh:104-199)."""

    def __init__(self, system: IsingSystem):
        if system is None:
            raise RuntimeError("Error constructing SemiGrandCanonicalPotential: _system==nullptr")
        self.system = system
        self.state: Optional[IsingState] = None
        self.conditions: Optional[SemiGrandCanonicalConditions] = None
        f = system.formation_energy_calculator
        self.formation_energy_calculator = IsingFormationEnergy(f.J, f.lattice_type, f.use_nlist)
        self.param_composition_calculator = IsingParamComposition()

    def set_state(self, state: IsingState, conditions: SemiGrandCanonicalConditions) -> None:
        if state is None:
            raise RuntimeError("Error in SemiGrandCanonicalPotential::set_state: _state is nullptr")
        if conditions is None:
            raise RuntimeError("Error in SemiGrandCanonicalPotential::set_state: _conditions is nullptr")
        self.state = state
        self.conditions = conditions
        self.formation_energy_calculator.set_state(state)
        self.param_composition_calculator.set_state(state)

    def per_supercell(self) -> float:
        mu = self.conditions.exchange_potential
        Nx = self.param_composition_calculator.per_supercell()
        return self.formation_energy_calculator.per_supercell() - _dot(mu, Nx)

    def per_unitcell(self) -> float:
        return self.per_supercell() / self.state.configuration.n_unitcells

    def occ_delta_per_supercell(self, linear_site_index, new_occ) -> float:
        dEf = self.formation_energy_calculator.occ_delta_per_supercell(linear_site_index, new_occ)
        Ndx = self.param_composition_calculator.occ_delta_per_supercell(linear_site_index, new_occ)
        return dEf - _dot(self.conditions.exchange_potential, Ndx)


def _occ_event_delta_per_supercell(self, occ_event) -> float:
    """The change of E_sgc for an OccEvent (its linear_site_index and new_occ)."""
    return self.occ_delta_per_supercell(occ_event.linear_site_index, occ_event.new_occ)


SemiGrandCanonicalPotential.occ_event_delta_per_supercell = _occ_event_delta_per_supercell


def _dot(a, b) -> float:
    r = 0.0
    for i, (x, y) in enumerate(zip(a, b)):
        r = float(x) * float(y) if i == 0 else r + float(x) * float(y)
    return r


class OccEventLite:
    def __init__(self):
        self.linear_site_index = [0]
        self.new_occ = [1]


class SemiGrandCanonicalEventGenerator:
    """Random single-site flip proposal (basic_semigrand_canonical.hh:268-321).

    On the GPU path the proposal is executed by the replay kernel; ``propose``/``apply``
    remain available for host use with a ``RandomNumberGenerator``.
    """

    def __init__(self):
        self.state: Optional[IsingState] = None
        self.occ_event = OccEventLite()
        self._max_l = 0

    def set_state(self, state: IsingState) -> None:
        if state is None:
            raise RuntimeError("Error in SemiGrandCanonicalEventGenerator::set_state: _state==nullptr")
        self.state = state
        self._max_l = state.configuration.n_sites - 1

    def propose(self, random_number_generator):
        l = random_number_generator.random_int(self._max_l)
        self.occ_event.linear_site_index[0] = l
        self.occ_event.new_occ[0] = -self.state.configuration.occ(l)
        return self.occ_event

    def apply(self, e) -> None:
        self.state.configuration.set_occ(e.linear_site_index[0], e.new_occ[0])


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
        tot = self.n_accept + self.n_reject
        return {"completion_check_results": self.completion_check.results().to_dict(), "n_pass": self.n_pass,
                "n_steps_per_pass": self.n_steps_per_pass, "n_accept": self.n_accept,
                "n_reject": self.n_reject, "acceptance_rate": self.n_accept / tot if tot else float("nan"),
                "rejection_rate": self.n_reject / tot if tot else float("nan")}


class _DeviceSampled:
    """A default sampling function; during ``run`` its values come from the GPU's exact
    integer sums, outside ``run`` it evaluates the host calculators."""

    def __init__(self, calc: "SemiGrandCanonicalCalculator", kind: str):
        self.calc = calc
        self.kind = kind

    def __call__(self):
        c = self.calc
        if self.kind == "param_composition":
            return c.param_composition_calculator.per_unitcell()
        if self.kind == "formation_energy":
            return np.array([c.formation_energy_calculator.per_unitcell()])
        return np.array([c.potential.per_unitcell()])


def default_write_status(mc_calculator, method_log: MethodLog) -> None:
    """Status to stdout and completion-check results to the log file (default_write_status)."""
    data = mc_calculator.data
    n_pass = data.n_pass
    n_samples = get_n_samples(data.samplers)
    steps = float(n_pass) * float(data.n_steps_per_pass)
    t = method_log.time_s()
    rate = steps / t if t > 0 else float("inf")
    print(f"Passes={n_pass}, Samples={n_samples}, ClockTime(s)={t}, Steps/Second={rate}, "
          f"Seconds/Step={t / steps if steps else 0.0}")
    x = mc_calculator.param_composition_calculator.per_unitcell()
    ef = mc_calculator.formation_energy_calculator.per_unitcell()
    print(f"  ParametricComposition={x}, FormationEnergy={ef}")
    results = data.completion_check.results()
    print(f"  AllEquilibrated={int(results.equilibration_check_results.all_equilibrated)}")
    if results.equilibration_check_results.all_equilibrated:
        print(f"  AllConverged={int(results.convergence_check_results.all_converged)}")
    sys.stdout.flush()
    if method_log.logfile_path():
        method_log.reset()
        method_log.write_json(results.to_dict())
    method_log.begin_lap()


def _flat_occupation(cfg) -> np.ndarray:
    """Occupation in linear-site-index order (column-major), int32, for either
    configuration type (this package's 1-D one or the numpy 2-D one of ``ising_py``)."""
    o = np.asarray(cfg.occupation())
    if o.ndim == 2:
        o = o.flatten(order="F")
    return np.ascontiguousarray(o, dtype=np.int32)


def _set_flat_occupation(cfg, occ: np.ndarray) -> None:
    if np.asarray(cfg.occupation()).ndim == 2:
        cfg.set_occupation(occ.reshape(tuple(cfg.shape), order="F"))
    else:
        cfg.set_occupation(occ)


class _ReplayDriver:
    """The main loop of basic_occupation_metropolis.hh:354-425 for the random single-site
    flip of a 2-D Ising model, executed as a serial replay on the GPU: the kernel consumes
    the caller's mt19937_64 engine exactly as the reference does (site draw, acceptance
    draw only for dE >= 0).  The host drives it in chunks of whole passes and reproduces,
    call for call, the completion check evaluated before every step: samples and counts
    change only at pass boundaries, so a chunk ends at the first pass boundary where that
    check could finish the run or run a convergence check."""

    #: upper bound on passes per kernel launch
    max_passes_per_launch = 4096
    #: device time of the replay kernels in the last run (ms)
    last_kernel_ms = 0.0

    def _replay(self, data, J: float, mu: float, T: float, use_nlist: bool, sample_period: int,
                method_log: MethodLog, random_engine: RandomNumberEngine, write_status_f: Callable,
                completion_check_params: CompletionCheckParams) -> None:
        """Run ``self.state`` with ``dE = dE_f - mu (new - old) / 2`` until complete; the
        occupation, the engine and the acceptance counts are synchronised at the end."""
        cfg = self.state.configuration
        N = cfg.n_variable_sites
        rows, cols = int(cfg.shape[0]), int(cfg.shape[1])
        L = _lib.lib()
        h = C.c_void_p()
        occ = _flat_occupation(cfg)
        states = (C.c_char_p * 1)(random_engine.dump().encode())
        _lib.check(L.mg_ising_replay_create(
            rows, cols, 1, 1 if use_nlist else 0, _lib.ptr(np.array([J], dtype=float), C.c_double),
            _lib.ptr(np.array([T], dtype=float), C.c_double), _lib.ptr(np.array([mu], dtype=float), C.c_double),
            _lib.ptr(occ, C.c_int32), states, C.byref(h)))
        self.last_kernel_ms = 0.0
        try:
            self._main_loop(h, data, N, rows, cols, J, mu, use_nlist, sample_period, method_log,
                            write_status_f, completion_check_params)
        finally:
            self._sync_state(h, random_engine, data)
            L.mg_ising_replay_destroy(h)

    # -- internals
    def _sync_state(self, h, random_engine, data) -> None:
        L = _lib.lib()
        cfg = self.state.configuration
        occ = np.zeros(cfg.n_sites, dtype=np.int32)
        buf = C.create_string_buffer(ENGINE_STATE_LEN)
        bufs = (C.c_char_p * 1)(C.cast(buf, C.c_char_p))
        acc, rej = C.c_ulonglong(), C.c_ulonglong()
        _lib.check(L.mg_ising_replay_get_state(h, _lib.ptr(occ, C.c_int32), bufs, ENGINE_STATE_LEN,
                                               C.byref(acc), C.byref(rej)))
        _set_flat_occupation(cfg, occ)
        random_engine.load(buf.value.decode())
        data.n_accept = int(acc.value)
        data.n_reject = int(rej.value)

    def _main_loop(self, h, data, N, rows, cols, J, mu, use_nlist, sample_period, method_log,
                   write_status_f, params) -> None:
        L = _lib.lib()
        cc = data.completion_check
        samplers = data.samplers
        funcs = data.sampling_functions
        device_only = all(isinstance(f.function, _DeviceSampled) and f.function.calc is self
                          for f in funcs.values()) and len(data.json_sampling_functions) == 0
        max_chunk = max(1, int(self.max_passes_per_launch))
        if params.cutoff_params.max_clocktime is not None:
            max_chunk = min(max_chunk, sample_period)
        stride = 2 + rows + cols
        n_samples_now = 0

        def first_call():
            return cc.count_check(samplers, data.sample_weight, data.n_pass, method_log)

        complete = first_call()
        while not complete:
            cc._repeat_calls(N - 1)
            # plan the chunk: first pass boundary where the check could act
            k = 0
            ns = n_samples_now
            limit = max_chunk if device_only else max(1, sample_period - (data.n_pass % sample_period))
            limit = min(limit, max_chunk)
            while k < limit:
                k += 1
                p = data.n_pass + k
                if p % sample_period == 0:
                    ns += 1
                if cc._could_complete_at(ns, p):
                    break
            expected = (data.n_pass + k) // sample_period - data.n_pass // sample_period
            buf = np.zeros((1, max(expected, 1), stride), dtype=np.int64)
            n_written = C.c_int()
            _lib.check(L.mg_ising_replay_run(h, k, sample_period, _lib.ptr(buf, C.c_longlong), max(expected, 1),
                                             C.byref(n_written)))
            ms = C.c_float()
            L.mg_ising_replay_last_kernel_ms(h, C.byref(ms))
            self.last_kernel_ms += ms.value
            si = 0
            for b in range(k):
                data.n_pass += 1
                if data.n_pass % sample_period == 0:
                    row = buf[0, si]
                    si += 1
                    self._push_sample(h, data, row, N, rows, cols, J, mu, use_nlist, device_only)
                    n_samples_now += 1
                    lf = method_log.log_frequency()
                    if lf is not None and method_log.lap_time() >= lf:
                        write_status_f(self, method_log)
                complete = first_call()
                if complete:
                    if b != k - 1:
                        raise RuntimeError("internal error: completion inside a planned chunk")
                    break
                if b < k - 1:
                    cc._repeat_calls(N - 1)

    def _push_sample(self, h, data, row, N, rows, cols, J, mu, use_nlist, device_only) -> None:
        spin_sum, bond_sum = int(row[0]), int(row[1])
        Nx = float(N + spin_sum) / 2.0
        if use_nlist:
            ef = float(bond_sum)
            ef *= -J
        else:
            ef = 0.0
            for i in range(rows):
                ef += -J * float(int(row[2 + i]))
            for j in range(cols):
                ef += -J * float(int(row[2 + rows + j]))
        values = {
            "param_composition": np.array([Nx / N]),
            "formation_energy": np.array([ef / N]),
            "potential_energy": np.array([(ef - mu * Nx) / N]),
        }
        if not device_only:
            # custom functions read the host state: bring the occupation back first
            occ = np.zeros(N, dtype=np.int32)
            _lib.check(_lib.lib().mg_ising_replay_get_state(h, _lib.ptr(occ, C.c_int32), None, 0, None, None))
            _set_flat_occupation(self.state.configuration, occ)
        for name in sorted(data.sampling_functions):
            f = data.sampling_functions[name]
            if isinstance(f.function, _DeviceSampled) and f.function.calc is self:
                data.samplers[name].append(values[f.function.kind])
            else:
                data.samplers[name].append(f())
        for name in sorted(data.json_sampling_functions):
            data.json_samplers[name].values.append(data.json_sampling_functions[name]())


def _member_copy(self):
    """A copy whose members are the same objects (system, state, samplers), as the
    reference's copy constructors copy shared pointers."""
    c = object.__new__(type(self))
    c.__dict__.update(self.__dict__)
    return c


def _value_copy(self, memo=None):
    c = object.__new__(type(self))
    c.__dict__.update(copy.deepcopy(self.__dict__, memo))
    return c


SemiGrandCanonicalConditions.__copy__ = _value_copy
SemiGrandCanonicalConditions.__deepcopy__ = _value_copy
for _cls in (SemiGrandCanonicalPotential, SemiGrandCanonicalEventGenerator, SemiGrandCanonicalData):
    _cls.__copy__ = _member_copy
    _cls.__deepcopy__ = lambda self, memo=None: _member_copy(self)


class SemiGrandCanonicalCalculator(_ReplayDriver):
    """Semi-grand canonical Monte Carlo calculator (basic_semigrand_canonical.hh:324-470)."""

    def __init__(self, system: IsingSystem):
        if system is None:
            raise RuntimeError("Error constructing SemiGrandCanonicalCalculator: _system==nullptr")
        self.system = system
        self.state: Optional[IsingState] = None
        self.conditions: Optional[SemiGrandCanonicalConditions] = None
        self.potential = SemiGrandCanonicalPotential(system)
        self.formation_energy_calculator = self.potential.formation_energy_calculator
        self.param_composition_calculator = self.potential.param_composition_calculator
        self.data: Optional[SemiGrandCanonicalData] = None

    def default_sampling_functions(self) -> StateSamplingFunctionMap:
        m = StateSamplingFunctionMap()
        n = self.system.param_composition_calculator.n_independent_compositions()
        m["param_composition"] = StateSamplingFunction(
            "param_composition", "Parametric composition", [n], _DeviceSampled(self, "param_composition"))
        m["formation_energy"] = StateSamplingFunction(
            "formation_energy", "Intensive formation energy", [], _DeviceSampled(self, "formation_energy"))
        m["potential_energy"] = StateSamplingFunction(
            "potential_energy", "Intensive potential energy", [], _DeviceSampled(self, "potential_energy"))
        return m

    def default_json_sampling_functions(self) -> jsonStateSamplingFunctionMap:
        m = jsonStateSamplingFunctionMap()
        m["configuration"] = jsonStateSamplingFunction(
            "configuration", "Configuration values", lambda: self.state.configuration.to_dict())
        return m

    def run(self, state: IsingState, sampling_functions, json_sampling_functions,
            completion_check_params: CompletionCheckParams, event_generator: SemiGrandCanonicalEventGenerator,
            sample_period: int = 1, method_log: Optional[MethodLog] = None,
            random_engine: Optional[RandomNumberEngine] = None,
            write_status_f: Optional[Callable] = None) -> SemiGrandCanonicalData:
        """Run at one thermodynamic state; ``state`` is modified in place."""
        if write_status_f is None:
            write_status_f = default_write_status
        self.state = state
        self.conditions = SemiGrandCanonicalConditions.from_values(state.conditions)
        if self.conditions.exchange_potential.size != 1:
            raise RuntimeError("Error in SemiGrandCanonicalCalculator::run: exchange_potential must have size 1")
        T = self.conditions.temperature
        cfg = state.configuration
        N = cfg.n_variable_sites
        self.potential.set_state(state, self.conditions)
        event_generator.set_state(state)
        self.data = data = SemiGrandCanonicalData(sampling_functions, json_sampling_functions, N,
                                                  completion_check_params)
        if random_engine is None:
            random_engine = RandomNumberEngine()
        if method_log is None:
            method_log = MethodLog(os.path.join(os.getcwd(), "status.json"), 600.0)
        method_log.restart_clock()
        method_log.begin_lap()

        J = self.system.formation_energy_calculator.J
        use_nlist = self.system.formation_energy_calculator.use_nlist
        mu = float(self.conditions.exchange_potential[0])
        self._replay(data, J, mu, T, use_nlist, sample_period, method_log, random_engine, write_status_f,
                     completion_check_params)
        write_status_f(self, method_log)
        return data


__all__ = ["SemiGrandCanonicalCalculator", "SemiGrandCanonicalConditions", "SemiGrandCanonicalData",
           "SemiGrandCanonicalEventGenerator", "SemiGrandCanonicalPotential", "default_write_status"]
