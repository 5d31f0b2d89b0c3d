"""Sampling, completion, equilibration and convergence checks.

Mirrors ``libcasm.monte.sampling`` (python/libcasm/monte/sampling/__init__.py:4-61).
Semantics follow:

* ``Sampler``                    include/casm/monte/sampling/Sampler.hh:30-326
* ``CutoffCheckParams`` & co.    include/casm/monte/checks/CutoffCheck.hh:14-94
* ``CompletionCheck``            include/casm/monte/checks/CompletionCheck.hh:19-376
* equilibration                  src/casm/monte/checks/EquilibrationCheck.cc:50-225
* convergence                    include/casm/monte/checks/ConvergenceCheck.hh:74-184
* ``BasicStatisticsCalculator``  src/casm/monte/BasicStatistics.cc:24-188
* ``converge``                   python/libcasm/monte/sampling/_requested_precision_constructor.py
* selected-event data and histograms: ``_selected_event`` (SelectedEventFunctions.hh/.cc)

The per-component numerics (equilibration scan, autocorrelation, precision of the
mean) run natively in libmontegpu (the same functions the device convergence kernel
uses); the bookkeeping around them is plain Python.
"""
from __future__ import annotations

import ctypes as C
import enum
import math
from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np

from .. import __version__, _lib  # noqa: F401


class SAMPLE_MODE(enum.Enum):
    BY_STEP = 0
    BY_PASS = 1
    BY_TIME = 2


class SAMPLE_METHOD(enum.Enum):
    LINEAR = 0
    LOG = 1
    CUSTOM = 2


class SamplingParams:
    """What to sample and when (sampling/SamplingParams.hh:14-153)."""

    def __init__(self, sampler_names=None, json_sampler_names=None, sample_mode: SAMPLE_MODE = SAMPLE_MODE.BY_PASS,
                 sample_method: SAMPLE_METHOD = SAMPLE_METHOD.LINEAR, period: float = 1.0, begin: float = 1.0,
                 base: float = 10.0 ** (1.0 / 10.0), shift: float = 10.0,
                 custom_sample_at: Optional[Callable[[float], float]] = None, stochastic_sample_period: bool = False,
                 do_sample_trajectory: bool = False, do_sample_time: bool = False):
        self.sampler_names = list(sampler_names or [])
        self.json_sampler_names = list(json_sampler_names or [])
        self.sample_mode = sample_mode
        self.sample_method = sample_method
        self.period = float(period)
        self.begin = float(begin)
        self.base = float(base)
        self.shift = float(shift)
        self.custom_sample_at = custom_sample_at
        self.stochastic_sample_period = bool(stochastic_sample_period)
        self.do_sample_trajectory = bool(do_sample_trajectory)
        self.do_sample_time = bool(do_sample_time)


def _list_helpers(attr: str):
    def append(self, name: str) -> None:
        getattr(self, attr).append(name)

    def remove(self, name: str) -> None:
        names = getattr(self, attr)
        if name in names:
            names.remove(name)

    def extend(self, names) -> None:
        getattr(self, attr).extend(names)
    return append, remove, extend


# monte_sampling.cpp:652-720: the first occurrence is removed; a missing name is ignored
(SamplingParams.append_to_sampler_names, SamplingParams.remove_from_sampler_names,
 SamplingParams.extend_sampler_names) = _list_helpers("sampler_names")
(SamplingParams.append_to_json_sampler_names, SamplingParams.remove_from_json_sampler_names,
 SamplingParams.extend_json_sampler_names) = _list_helpers("json_sampler_names")


def default_component_names(shape: list[int]) -> list[str]:
    """Sampler.hh:333-349: [] -> ["0"]; [n] -> ["0".."n-1"]; [m,n] -> column-major "i,j"."""
    if len(shape) == 0:
        return ["0"]
    if len(shape) == 1:
        return [str(i) for i in range(shape[0])]
    if len(shape) == 2:
        return colmajor_component_names(shape[0], shape[1])
    raise RuntimeError("Error constructing sampler component names: >2 dimensions is not supported")


def colmajor_component_names(n_rows: int, n_cols: int) -> list[str]:
    return [f"{j},{i}" for i in range(n_cols) for j in range(n_rows)]


def scalar_as_vector(value: float) -> np.ndarray:
    return np.array([float(value)])


def matrix_as_vector(value) -> np.ndarray:
    return np.asarray(value, dtype=float).reshape(-1, order="F")


class Sampler:
    """Stores vector-valued samples; component-major storage, grown in increments."""

    def __init__(self, shape: list[int], component_names: Optional[list[str]] = None,
                 capacity_increment: int = 1000):
        self._shape = list(shape)
        self._names = list(component_names) if component_names is not None else default_component_names(shape)
        self._inc = int(capacity_increment)
        self._data = np.zeros((len(self._names), self._inc), dtype=np.float64)
        self._n = 0

    def append(self, vector) -> None:
        v = np.asarray(vector, dtype=np.float64).reshape(-1)
        if v.size != self._data.shape[0]:
            raise RuntimeError("Error in Sampler::push_back: sample size mismatch")
        if self._n == self._data.shape[1]:
            self._grow(self._data.shape[1] + self._inc)
        self._data[:, self._n] = v
        self._n += 1

    push_back = append

    def append_many(self, rows: np.ndarray) -> None:
        """Append several samples at once (rows = samples)."""
        rows = np.asarray(rows, dtype=np.float64).reshape(-1, self._data.shape[0])
        need = self._n + rows.shape[0]
        if need > self._data.shape[1]:
            cap = self._data.shape[1]
            while cap < need:
                cap += self._inc
            self._grow(cap)
        self._data[:, self._n:need] = rows.T
        self._n = need

    def _grow(self, cap: int) -> None:
        d = np.zeros((self._data.shape[0], cap), dtype=np.float64)
        d[:, : self._n] = self._data[:, : self._n]
        self._data = d

    def set_values(self, values) -> None:
        v = np.asarray(values, dtype=np.float64)
        self._data = np.ascontiguousarray(v.T.copy())
        self._n = v.shape[0]

    def clear(self) -> None:
        """n_samples = 0; the buffer and its capacity are kept, so ``sample(i)`` still
        reads what was stored there, as the reference's Sampler::clear leaves it."""
        self._n = 0

    def set_sample_capacity(self, capacity: int) -> None:
        self._grow(max(capacity, self._n))

    def set_capacity_increment(self, inc: int) -> None:
        self._inc = int(inc)

    def component_names(self) -> list[str]:
        return list(self._names)

    def shape(self) -> list[int]:
        return list(self._shape)

    def n_components(self) -> int:
        return self._data.shape[0]

    def n_samples(self) -> int:
        return self._n

    def sample_capacity(self) -> int:
        return self._data.shape[1]

    def values(self) -> np.ndarray:
        """n_samples x n_components (a copy)."""
        return self._data[:, : self._n].T.copy()

    def component(self, component_index: int) -> np.ndarray:
        """All samples of one component (a contiguous view)."""
        return self._data[component_index, : self._n]

    def sample(self, sample_index: int) -> np.ndarray:
        return self._data[:, sample_index].copy()


class SamplerMap(dict):
    """name -> Sampler (std::map: iterated in name order)."""


def get_n_samples(samplers: dict) -> int:
    """n_samples of the first sampler in name order, else 0 (Sampler.hh:410-416)."""
    if len(samplers) == 0:
        return 0
    return samplers[min(samplers)].n_samples()


@dataclass(frozen=True)
class SamplerComponent:
    sampler_name: str = ""
    component_index: int = 0
    component_name: str = ""

    def _key(self):
        return (self.sampler_name, self.component_index)

    def __lt__(self, other: "SamplerComponent") -> bool:
        return self._key() < other._key()

    def __eq__(self, other) -> bool:
        return isinstance(other, SamplerComponent) and self._key() == other._key()

    def __hash__(self) -> int:
        return hash(self._key())


class RequestedPrecision:
    """Sampler.hh:151-180."""

    def __init__(self, abs: Optional[float] = None, rel: Optional[float] = None):
        self.abs_convergence_is_required = abs is not None
        self.abs_precision = float(abs) if abs is not None else 0.0
        self.rel_convergence_is_required = rel is not None
        self.rel_precision = float(rel) if rel is not None else 0.0

    def to_dict(self) -> dict:
        """Sampler_json_io.cc:39-52."""
        d = {}
        if self.abs_convergence_is_required:
            d["abs_precision"] = self.abs_precision
        if self.rel_convergence_is_required:
            d["rel_precision"] = self.rel_precision
        return d

    @staticmethod
    def from_dict(data: dict) -> "RequestedPrecision":
        """"abs_precision" (or the older "precision") and "rel_precision", each optional
        (Sampler_json_io.cc:70-95)."""
        a = data.get("abs_precision", data.get("precision"))
        r = data.get("rel_precision")
        return RequestedPrecision(abs=None if a is None else float(a), rel=None if r is None else float(r))


class RequestedPrecisionMap(dict):
    """SamplerComponent -> RequestedPrecision (iterated in key order)."""


class StateSamplingFunction:
    """A named function sampled once per sample (StateSamplingFunction.hh:20-54)."""

    def __init__(self, name: str, description: str, shape: list[int], function: Callable,
                 component_names: Optional[list[str]] = None):
        self.name = name
        self.description = description
        self.shape = list(shape)
        self.function = function
        self.component_names = (list(component_names) if component_names is not None
                                else default_component_names(self.shape))

    def __call__(self) -> np.ndarray:
        return np.asarray(self.function(), dtype=float).reshape(-1)


class StateSamplingFunctionMap(dict):
    pass


class jsonStateSamplingFunction:
    def __init__(self, name: str, description: str, function: Callable):
        self.name = name
        self.description = description
        self.function = function

    def __call__(self):
        return self.function()


class jsonStateSamplingFunctionMap(dict):
    pass


class _SampleList(list):
    """The samples of a jsonSampler: a list that, called, returns them as a new list (the
    binding's ``values()``)."""

    def __call__(self) -> list:
        return list(self)


class jsonSampler:
    """Sampled dict-like data for JSON output (monte_sampling.cpp:900-1010)."""

    def __init__(self):
        self.values = _SampleList()
        self._capacity = 0

    values = property(lambda self: self.__dict__["_values"],
                      lambda self, v: self.__dict__.__setitem__("_values", _SampleList(v)))

    def append(self, data) -> None:
        self.values.append(data)

    def set_values(self, values) -> None:
        self.values = values

    def clear(self) -> None:
        self.values.clear()

    def set_sample_capacity(self, sample_capacity: int) -> None:
        self._capacity = max(self._capacity, int(sample_capacity))

    def n_samples(self) -> int:
        return len(self.values)

    def sample_capacity(self) -> int:
        return max(self._capacity, len(self.values))

    def sample(self, sample_index: int):
        if not 0 <= int(sample_index) < len(self.values):
            raise IndexError(f"jsonSampler.sample: index {sample_index} out of range")
        return self.values[int(sample_index)]

    def __len__(self) -> int:
        return len(self.values)

    def __iter__(self):
        return iter(self.values)

    def to_list(self) -> list:
        return list(self.values)


class jsonSamplerMap(dict):
    pass


@dataclass
class CutoffCheckParams:
    """CutoffCheck.hh:14-34; None = not set."""

    min_count: Optional[int] = None
    min_time: Optional[float] = None
    min_sample: Optional[int] = None
    min_clocktime: Optional[float] = None
    max_count: Optional[int] = None
    max_time: Optional[float] = None
    max_sample: Optional[int] = None
    max_clocktime: Optional[float] = None

    _KINDS = (("count", int), ("time", float), ("sample", int), ("clocktime", float))

    def to_dict(self) -> dict:
        """{"count": {"min": .., "max": ..}, "time": .., "sample": .., "clocktime": ..}, set
        values only (CutoffCheck_json_io.cc:9-48)."""
        d = {}
        for kind, _ in self._KINDS:
            sub = {k: getattr(self, f"{k}_{kind}") for k in ("min", "max") if getattr(self, f"{k}_{kind}") is not None}
            if sub:
                d[kind] = sub
        return d

    @staticmethod
    def from_dict(data: dict) -> "CutoffCheckParams":
        p = CutoffCheckParams()
        for kind, typ in CutoffCheckParams._KINDS:
            for k, v in (data.get(kind) or {}).items():
                if k not in ("min", "max"):
                    raise RuntimeError(f"Error in CutoffCheckParams.from_dict: unknown option '{kind}/{k}'")
                setattr(p, f"{k}_{kind}", None if v is None else typ(v))
        return p


def all_minimums_met(cutoff_params: CutoffCheckParams, count: Optional[int], time: Optional[float],
                     n_samples: int, clocktime: float) -> bool:
    p = cutoff_params
    if p.min_sample is not None and n_samples < p.min_sample:
        return False
    if p.min_count is not None and count is not None and count < p.min_count:
        return False
    if p.min_time is not None and time is not None and time < p.min_time:
        return False
    if p.min_clocktime is not None and clocktime < p.min_clocktime:
        return False
    return True


def any_maximum_met(cutoff_params: CutoffCheckParams, count: Optional[int], time: Optional[float],
                    n_samples: int, clocktime: float) -> bool:
    p = cutoff_params
    if p.max_sample is not None and n_samples >= p.max_sample:
        return True
    if p.max_count is not None and count is not None and count >= p.max_count:
        return True
    if p.max_time is not None and time is not None and time >= p.max_time:
        return True
    if p.max_clocktime is not None and clocktime >= p.max_clocktime:
        return True
    return False


@dataclass
class BasicStatistics:
    mean: float = 0.0
    calculated_precision: float = float(np.finfo(np.float64).max)

    def to_dict(self) -> dict:
        return {"mean": self.mean, "calculated_precision": self.calculated_precision}

    def relative_precision(self) -> float:
        """|calculated_precision / mean| (BasicStatistics.hh:42-44)."""
        with np.errstate(divide="ignore", invalid="ignore"):
            return float(abs(np.float64(self.calculated_precision) / np.float64(self.mean)))


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


class BasicStatisticsCalculator:
    """Mean and precision of the mean with autocorrelation (BasicStatistics.cc:114-188)."""

    def __init__(self, confidence: float = 0.95, method: int = 1, n_resamples: int = 10000):
        self.confidence = float(confidence)
        self.method = int(method)
        self.n_resamples = int(n_resamples)

    weighted_observations_method = property(lambda self: self.method,
                                            lambda self, v: setattr(self, "method", int(v)))

    def calculate(self, observations, sample_weight) -> "BasicStatistics":
        return self(observations, sample_weight)

    def to_dict(self) -> dict:
        return {"confidence": self.confidence, "weighted_observations_method": self.method,
                "n_resamples": self.n_resamples}

    @staticmethod
    def from_dict(data: dict) -> "BasicStatisticsCalculator":
        return BasicStatisticsCalculator(data.get("confidence", 0.95), data.get("weighted_observations_method", 1),
                                         data.get("n_resamples", 10000))

    def __call__(self, observations, sample_weight=None) -> BasicStatistics:
        x = _f64(observations)
        if x.size == 0:
            raise RuntimeError("Error in BasicStatisticsCalculator: observations.size()==0")
        w = _f64(sample_weight) if sample_weight is not None else np.zeros(0)
        mean, prec = C.c_double(), C.c_double()
        wp = _lib.ptr(w, C.c_double) if w.size else None
        _lib.check(_lib.lib().mg_basic_statistics(_lib.ptr(x, C.c_double), x.size, wp, w.size, self.confidence,
                                                  self.method, self.n_resamples, C.byref(mean), C.byref(prec)))
        return BasicStatistics(mean.value, prec.value)


def autocorrelation_factor(observations, increment: float = 1.0) -> float:
    x = _f64(observations)
    out = C.c_double()
    _lib.check(_lib.lib().mg_autocorrelation_factor(_lib.ptr(x, C.c_double), x.size, float(increment), C.byref(out)))
    return out.value


@dataclass
class IndividualEquilibrationResult:
    is_equilibrated: bool = False
    N_samples_for_equilibration: int = 0

    def to_dict(self) -> dict:
        return {"is_equilibrated": self.is_equilibrated,
                "N_samples_for_equilibration": self.N_samples_for_equilibration}


def default_equilibration_check(observations, sample_weight, requested_precision: RequestedPrecision
                                ) -> IndividualEquilibrationResult:
    """EquilibrationCheck.cc:119-162."""
    x = _f64(observations)
    if requested_precision.abs_convergence_is_required:
        prec = requested_precision.abs_precision
    elif requested_precision.rel_convergence_is_required:
        prec = abs(float(np.sum(x)) / x.size * requested_precision.rel_precision) if x.size else 0.0
    else:
        return IndividualEquilibrationResult(True, 0)
    if x.size == 0:
        raise RuntimeError("Error in equilibration_check: observations.size()==0")
    w = _f64(sample_weight) if sample_weight is not None else np.zeros(0)
    if w.size:
        if w.size != x.size:
            raise RuntimeError("Error in equilibration_check: sample_weight.size() != observations.size()")
        W = 0.0
        for v in w:
            W += v
        x = x * ((x.size / W) * w)
    is_eq, n_eq = C.c_int(), C.c_long()
    _lib.check(_lib.lib().mg_equilibration_check(_lib.ptr(x, C.c_double), x.size, float(prec), C.byref(is_eq),
                                                 C.byref(n_eq)))
    return IndividualEquilibrationResult(bool(is_eq.value), int(n_eq.value))


@dataclass
class EquilibrationCheckResults:
    all_equilibrated: bool = False
    N_samples_for_all_to_equilibrate: int = 0
    individual_results: dict = field(default_factory=dict)

    def to_dict(self) -> dict:
        return {"all_equilibrated": self.all_equilibrated,
                "N_samples_for_all_to_equilibrate": self.N_samples_for_all_to_equilibrate,
                "individual_results": {f"{k.sampler_name}({k.component_index})": v.to_dict()
                                       for k, v in sorted(self.individual_results.items())}}


class EquilibrationResultMap(dict):
    pass


@dataclass
class IndividualConvergenceResult:
    is_converged: bool = False
    requested_precision: Optional[RequestedPrecision] = None
    stats: BasicStatistics = field(default_factory=BasicStatistics)

    def to_dict(self) -> dict:
        return {"is_converged": self.is_converged, **self.stats.to_dict()}


@dataclass
class ConvergenceCheckResults:
    all_converged: bool = False
    N_samples_for_statistics: int = 0
    individual_results: dict = field(default_factory=dict)

    def to_dict(self) -> dict:
        return {"all_converged": self.all_converged,
                "N_samples_for_statistics": self.N_samples_for_statistics,
                "individual_results": {f"{k.sampler_name}({k.component_index})": v.to_dict()
                                       for k, v in sorted(self.individual_results.items())}}


class ConvergenceResultMap(dict):
    pass


def _find_component(samplers: dict, key: SamplerComponent) -> np.ndarray:
    if key.sampler_name not in samplers:
        raise RuntimeError(f"Error finding sampler component: Sampler '{key.sampler_name}' not found.\n")
    s = samplers[key.sampler_name]
    if key.component_index >= s.n_components():
        raise RuntimeError(
            f"Error finding sampler component: Requested component index {key.component_index}, but "
            f"'{key.sampler_name}' has {s.n_components()}components.\n")
    return s.component(key.component_index)


def equilibration_check(equilibration_check_f, requested_precision: dict, samplers: dict,
                        sample_weight: Sampler, check_all: bool) -> EquilibrationCheckResults:
    """EquilibrationCheck.cc:180-225."""
    results = EquilibrationCheckResults()
    if len(requested_precision) == 0:
        return results
    results.all_equilibrated = True
    w = sample_weight.component(0) if sample_weight.n_samples() else None
    for key in sorted(requested_precision):
        obs = _find_component(samplers, key)
        cur = equilibration_check_f(obs, w, requested_precision[key])
        results.N_samples_for_all_to_equilibrate = max(results.N_samples_for_all_to_equilibrate,
                                                       cur.N_samples_for_equilibration)
        results.all_equilibrated = results.all_equilibrated and cur.is_equilibrated
        results.individual_results[key] = cur
        if not check_all and not results.all_equilibrated:
            break
    return results


def component_convergence_check(sampler: Sampler, sample_weight: Sampler, key: SamplerComponent,
                                requested_precision: RequestedPrecision, N_samples_for_statistics: int,
                                calc_statistics_f) -> IndividualConvergenceResult:
    """ConvergenceCheck.hh:94-119, 74-90."""
    obs = sampler.component(key.component_index)[-N_samples_for_statistics:]
    if sample_weight.n_samples() != 0:
        stats = calc_statistics_f(obs, sample_weight.component(0)[-N_samples_for_statistics:])
    else:
        stats = calc_statistics_f(obs, None)
    r = IndividualConvergenceResult(True, requested_precision, stats)
    if requested_precision.abs_convergence_is_required:
        r.is_converged = r.is_converged and stats.calculated_precision < requested_precision.abs_precision
    if requested_precision.rel_convergence_is_required:
        rel = abs(stats.calculated_precision / stats.mean) if stats.mean != 0.0 else math.inf
        r.is_converged = r.is_converged and rel < requested_precision.rel_precision
    return r


def convergence_check(samplers: dict, sample_weight: Sampler, requested_precision: dict,
                      N_samples_for_equilibration: int, calc_statistics_f) -> ConvergenceCheckResults:
    """ConvergenceCheck.hh:139-184."""
    results = ConvergenceCheckResults()
    N = get_n_samples(samplers)
    if len(requested_precision) == 0:
        results.N_samples_for_statistics = N
        return results
    if N_samples_for_equilibration >= N:
        return results
    results.N_samples_for_statistics = N - N_samples_for_equilibration
    results.all_converged = True
    for key in sorted(requested_precision):
        _find_component(samplers, key)
        cur = component_convergence_check(samplers[key.sampler_name], sample_weight, key,
                                          requested_precision[key], results.N_samples_for_statistics,
                                          calc_statistics_f)
        results.all_converged = results.all_converged and cur.is_converged
        results.individual_results[key] = cur
    return results


class CompletionCheckParams:
    """CompletionCheck.hh:19-100."""

    def __init__(self):
        self.cutoff_params = CutoffCheckParams()
        self.equilibration_check_f = default_equilibration_check
        self.calc_statistics_f = BasicStatisticsCalculator()
        self.requested_precision = RequestedPrecisionMap()
        self.log_spacing = False
        self.check_begin = 100
        self.check_period = 100
        self.check_base = 10.0
        self.check_shift = 2.0
        self.check_period_max = 10000

    def sample_check_linear(self, n: int) -> int:
        return self.check_begin + self.check_period * n

    def to_dict(self) -> dict:
        """CompletionCheck_json_io.hh:388-420 (statistics parameters not written, as there)."""
        conv = []
        for key, rp in sorted(self.requested_precision.items()):
            conv.append({"quantity": key.sampler_name, "component_index": [key.component_index],
                         "component_name": [key.component_name], **rp.to_dict()})
        d = {"cutoff": self.cutoff_params.to_dict(), "convergence": conv}
        if not self.log_spacing:
            d.update(spacing="linear", begin=self.check_begin, period=self.check_period)
        else:
            d.update(spacing="log", begin=self.check_begin, base=self.check_base, shift=self.check_shift,
                     period_max=self.check_period_max)
        return d

    @staticmethod
    def from_dict(data: dict, sampling_functions: dict) -> "CompletionCheckParams":
        """CompletionCheck_json_io.hh:295-386: "cutoff", "convergence" (per entry a
        "quantity" naming a sampling function, its precision, and "component_index" and/or
        "component_name", else every component), "spacing" ("linear": begin 100, period
        100; "log": begin 0, base 10, shift 2, period_max 10000), overrides "begin",
        "period", "base", "shift", "period_max"; "confidence",
        "weighted_observations_method", "n_resamples" for the statistics."""
        errors = []
        p = CompletionCheckParams()
        p.calc_statistics_f = BasicStatisticsCalculator.from_dict(data)
        p.cutoff_params = CutoffCheckParams.from_dict(data.get("cutoff") or {})
        conv = data.get("convergence", [])
        if not isinstance(conv, list):
            errors.append('"convergence" must be an array')
            conv = []
        for i, c in enumerate(conv):
            q = c.get("quantity")
            if q is None:
                errors.append(f"convergence/{i}/quantity is required")
                continue
            f = next((g for g in sampling_functions.values() if g.name == q), None) if q not in sampling_functions \
                else sampling_functions[q]
            if f is None:
                errors.append(f'"{q}" is not a sampling option.')
                continue
            rp = RequestedPrecision.from_dict(c)
            names = list(f.component_names)
            has_i, has_n = "component_index" in c, "component_name" in c
            for index in c.get("component_index", []):
                if not 0 <= int(index) < len(names):
                    errors.append(f'For "{f.name}", component index {index} is out of range. Valid range is '
                                  f'[0,{len(names)}).')
                    continue
                p.requested_precision.setdefault(SamplerComponent(f.name, int(index), names[int(index)]), rp)
            for name in c.get("component_name", []):
                if name not in names:
                    errors.append(f'For "{f.name}", component name {name} is not valid.')
                    continue
                p.requested_precision.setdefault(SamplerComponent(f.name, names.index(name), name), rp)
            if not has_i and not has_n:
                for index, name in enumerate(names):
                    p.requested_precision.setdefault(SamplerComponent(f.name, index, name), rp)
        spacing = data.get("spacing", "linear")
        if spacing == "linear":
            p.log_spacing, p.check_begin, p.check_period = False, 100, 100
        elif spacing == "log":
            p.log_spacing, p.check_begin, p.check_base, p.check_shift, p.check_period_max = True, 0, 10.0, 2.0, 10000
        else:
            errors.append('"spacing" must be one of "linear", "log".')
        p.check_begin = int(data.get("begin", p.check_begin))
        p.check_period = int(data.get("period", p.check_period))
        if p.check_period <= 1:  # the reference's own bound
            errors.append('"period" must > 0.')
        p.check_base = float(data.get("base", p.check_base))
        p.check_shift = float(data.get("shift", p.check_shift))
        p.check_period_max = int(data.get("period_max", p.check_period_max))
        if p.check_base <= 1.0:
            errors.append('"base" must > 1.0')
        if errors:
            raise RuntimeError("Error in libcasm.monte.sampling.CompletionCheckParams.from_dict: " + "; ".join(errors))
        return p

    def _sample_check_log(self, n: int) -> int:
        return self.check_begin + int(_round_half_away(math.pow(self.check_base, n + self.check_shift)))

    def find_n_begin_linear(self) -> int:
        n = 0
        while self._sample_check_log(n + 1) - self._sample_check_log(n) <= self.check_period_max:
            n += 1
        return n

    def sample_check_log(self, n: int, n_begin_linear: Optional[int] = None) -> int:
        if n_begin_linear is None:
            return self._sample_check_log(n)
        if n <= n_begin_linear:
            return self._sample_check_log(n)
        return self._sample_check_log(n_begin_linear) + self.check_period_max * (n - n_begin_linear)


def _round_half_away(x: float) -> float:
    """std::round semantics (halfway cases away from zero)."""
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)


class CompletionCheckResults:
    def __init__(self, params: Optional[CompletionCheckParams] = None):
        self.params = params
        self.count: Optional[int] = None
        self.time: Optional[float] = None
        self.clocktime = 0.0
        self.n_samples = 0
        self.has_all_minimums_met = False
        self.has_any_maximum_met = False
        self.n_samples_at_convergence_check: Optional[int] = None
        self.equilibration_check_results = EquilibrationCheckResults()
        self.convergence_check_results = ConvergenceCheckResults()
        self.is_complete = False

    def partial_reset(self, count=None, time=None, clocktime=0.0, n_samples=0) -> None:
        self.count = count
        self.time = time
        self.clocktime = clocktime
        self.n_samples = n_samples
        self.has_all_minimums_met = False
        self.has_any_maximum_met = False
        self.is_complete = False

    def full_reset(self, count=None, time=None, clocktime=0.0, n_samples=0) -> None:
        self.partial_reset(count, time, clocktime, n_samples)
        self.n_samples_at_convergence_check = None
        self.equilibration_check_results = EquilibrationCheckResults()
        self.convergence_check_results = ConvergenceCheckResults()

    def to_dict(self) -> dict:
        return {
            "count": self.count, "time": self.time, "clocktime": self.clocktime,
            "n_samples": self.n_samples, "has_all_minimums_met": self.has_all_minimums_met,
            "has_any_maximum_met": self.has_any_maximum_met,
            "n_samples_at_convergence_check": self.n_samples_at_convergence_check,
            "equilibration_check_results": self.equilibration_check_results.to_dict(),
            "convergence_check_results": self.convergence_check_results.to_dict(),
            "is_complete": self.is_complete,
        }


class CompletionCheck:
    """Cutoff + scheduled equilibration/convergence completion check (CompletionCheck.hh:175-376)."""

    def __init__(self, params: CompletionCheckParams):
        if params.equilibration_check_f is None:
            raise RuntimeError("Error constructing CompletionCheck: params.equilibration_check_f == nullptr")
        if params.calc_statistics_f is None:
            raise RuntimeError("Error constructing CompletionCheck: params.calc_statistics_f == nullptr")
        self._params = params
        self._results = CompletionCheckResults(params)
        self._n_checks = 0
        self._n_begin_linear = params.find_n_begin_linear()
        self._last_n_samples = 0
        self._last_clocktime = 0.0

    def params(self) -> CompletionCheckParams:
        return self._params

    def results(self) -> CompletionCheckResults:
        return self._results

    def reset(self) -> None:
        self._results.full_reset()
        self._n_checks = 0
        self._last_n_samples = 0
        self._last_clocktime = 0.0

    # -- public variants (monte_sampling.cpp:2993-3080)
    def is_complete(self, samplers, sample_weight, method_log) -> bool:
        return self._is_complete(samplers, sample_weight, None, None, method_log)

    def check(self, samplers, sample_weight, method_log) -> bool:
        """The completion check without count or time cutoffs (monte_sampling.cpp:3235-3242)."""
        return self.is_complete(samplers, sample_weight, method_log)

    def count_check(self, samplers, sample_weight, count, method_log) -> bool:
        return self._is_complete(samplers, sample_weight, int(count), None, method_log)

    def time_check(self, samplers, sample_weight, time, method_log) -> bool:
        return self._is_complete(samplers, sample_weight, None, float(time), method_log)

    def count_and_time_check(self, samplers, sample_weight, count, time, method_log) -> bool:
        return self._is_complete(samplers, sample_weight, int(count), float(time), method_log)

    def _check_at(self) -> int:
        p = self._params
        if p.log_spacing:
            return p.sample_check_log(self._n_checks, self._n_begin_linear)
        return p.sample_check_linear(self._n_checks)

    def _is_complete(self, samplers, sample_weight, count, time, method_log) -> bool:
        n_samples = get_n_samples(samplers)
        clocktime = self._last_clocktime
        if n_samples != self._last_n_samples:
            clocktime = method_log.time_s() if method_log is not None else 0.0
            self._last_n_samples = n_samples
            self._last_clocktime = clocktime
        r = self._results
        r.partial_reset(count, time, clocktime, n_samples)
        cp = self._params.cutoff_params
        r.has_all_minimums_met = all_minimums_met(cp, count, time, n_samples, clocktime)
        if not r.has_all_minimums_met:
            return False
        r.has_any_maximum_met = any_maximum_met(cp, count, time, n_samples, clocktime)
        if r.has_any_maximum_met:
            r.is_complete = True
            if n_samples != r.n_samples_at_convergence_check:
                self._check_convergence(samplers, sample_weight, n_samples)
            return True
        if n_samples >= self._check_at():
            self._n_checks += 1
            self._check_convergence(samplers, sample_weight, n_samples)
        if r.convergence_check_results.all_converged:
            r.is_complete = True
        return r.is_complete

    def _repeat_calls(self, n_calls: int) -> None:
        """Effect of ``n_calls`` further calls whose inputs equal the previous call's.

        In the reference loop the check runs before every step, but samples and counts
        change only at pass boundaries; repeated calls within a pass can only advance the
        check schedule (each re-running an identical convergence check).
        """
        r = self._results
        if not r.has_all_minimums_met or r.has_any_maximum_met or r.is_complete:
            return
        while n_calls > 0 and r.n_samples >= self._check_at():
            self._n_checks += 1
            n_calls -= 1

    def _could_complete_at(self, n_samples: int, count: Optional[int]) -> bool:
        """Whether a call with these inputs could return True or run a convergence check
        (clock-time minimums are assumed met)."""
        cp = self._params.cutoff_params
        if not all_minimums_met(cp, count, None, n_samples, 1e300 if cp.min_clocktime is not None else 0.0):
            return False
        if any_maximum_met(cp, count, None, n_samples, 0.0):
            return True
        return n_samples >= self._check_at()

    def _check_convergence(self, samplers, sample_weight, n_samples) -> None:
        p = self._params
        if len(p.requested_precision):
            r = self._results
            r.n_samples_at_convergence_check = n_samples
            r.equilibration_check_results = equilibration_check(
                p.equilibration_check_f, p.requested_precision, samplers, sample_weight, False)
            if r.equilibration_check_results.all_equilibrated:
                r.convergence_check_results = convergence_check(
                    samplers, sample_weight, p.requested_precision,
                    r.equilibration_check_results.N_samples_for_all_to_equilibrate, p.calc_statistics_f)
            else:
                r.convergence_check_results = ConvergenceCheckResults()


class RequestedPrecisionConstructor:
    """Sets requested precision for equilibration and convergence (reference helper)."""

    def __init__(self, sampling_functions: dict, completion_check_params: CompletionCheckParams):
        self.sampling_functions = sampling_functions
        self.completion_check_params = completion_check_params

    def set_precision(self, quantity: str, abs: Optional[float] = None, rel: Optional[float] = None,
                      component_name: Optional[list[str]] = None,
                      component_index: Optional[list[int]] = None) -> "RequestedPrecisionConstructor":
        if quantity not in self.sampling_functions:
            raise Exception(f"{quantity} is not in sampling_functions")
        f = self.sampling_functions[quantity]
        if rel is None and abs is None:
            raise Exception("No abs or rel precision specified")
        idx = list(component_index) if component_index is not None else []
        if component_name is not None:
            for n in component_name:
                if n not in f.component_names:
                    raise Exception(f"{n} is not a component of {quantity}")
                idx.append(f.component_names.index(n))
        idx = sorted(set(idx))
        if len(idx) == 0:
            idx = list(range(len(f.component_names)))
        for i in idx:
            key = SamplerComponent(sampler_name=quantity, component_name=f.component_names[i], component_index=i)
            self.completion_check_params.requested_precision[key] = RequestedPrecision(abs=abs, rel=rel)
        return self


from . import _selected_event  # noqa: E402
from ._selected_event import *  # noqa: E402,F401,F403


def converge(sampling_functions: dict, completion_check_params: CompletionCheckParams
             ) -> RequestedPrecisionConstructor:
    return RequestedPrecisionConstructor(sampling_functions, completion_check_params)


__all__ = [
    "SAMPLE_MODE", "SAMPLE_METHOD", "SamplingParams", "BasicStatistics", "BasicStatisticsCalculator", "CompletionCheck",
    "CompletionCheckParams", "CompletionCheckResults", "ConvergenceCheckResults", "ConvergenceResultMap",
    "CutoffCheckParams", "EquilibrationCheckResults", "EquilibrationResultMap", "IndividualConvergenceResult",
    "IndividualEquilibrationResult", "RequestedPrecision", "RequestedPrecisionMap", "Sampler",
    "SamplerComponent", "SamplerMap", "StateSamplingFunction", "StateSamplingFunctionMap", "all_minimums_met",
    "any_maximum_met", "autocorrelation_factor", "colmajor_component_names", "component_convergence_check",
    "convergence_check", "default_component_names", "default_equilibration_check", "equilibration_check",
    "get_n_samples", "jsonSampler", "jsonSamplerMap", "jsonStateSamplingFunction",
    "jsonStateSamplingFunctionMap", "matrix_as_vector", "scalar_as_vector", "RequestedPrecisionConstructor",
    "converge",
] + _selected_event.__all__
