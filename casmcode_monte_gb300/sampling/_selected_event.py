"""Selected-event data: hop correlations, discrete and continuous histograms.

Mirrors the selected-event part of ``libcasm.monte.sampling``
(python/libcasm/monte/sampling/__init__.py:13-41, bindings in
python/src/monte_sampling.cpp:1279-1960 and 3267-4420). Semantics follow:

* ``CorrelationsDataParams`` / ``CorrelationsData``
      include/casm/monte/sampling/SelectedEventFunctions.hh (struct definitions),
      src/casm/monte/sampling/SelectedEventFunctions.cc:9-72
* ``DiscreteVectorIntHistogram`` / ``DiscreteVectorFloatHistogram``
      src/casm/monte/sampling/SelectedEventFunctions.cc:76-200
* ``Histogram1D`` (growing bins, log spacing, merge) and ``combine``
      src/casm/monte/sampling/SelectedEventFunctions.cc:204-410
* ``PartitionedHistogram1D``   SelectedEventFunctions.hh:395-458, .cc:413-438
* ``VectorIntHistogramFunction`` & co.   include/casm/monte/sampling/HistogramFunction.hh
* ``SelectedEventFunctions`` / ``SelectedEventFunctionParams`` / ``SelectedEventData``
      SelectedEventFunctions.hh:470-640
* ``SelectedEventDataCollector``   SelectedEventFunctions.cc:440-732
* dict forms   src/casm/monte/sampling/io/json/SelectedEventFunctions_json_io.cc

These are host-side bookkeeping structures for methods that record per-event data
(kinetic Monte Carlo); the semi-grand canonical sweep does not produce selected
events, so nothing here touches the device.
"""
from __future__ import annotations

import copy
import math
from typing import Callable, Optional

import numpy as np

# CASM::TOL of libcasm-global (>= 2.2.0, the reference's pinned dependency): 1e-5.
_CASM_TOL = 1e-5


def _default_component_names(shape):
    from . import default_component_names
    return default_component_names(list(shape))


# -- Hop correlations ---------------------------------------------------------

class CorrelationsDataParams:
    """Parameters for collecting hop correlations (SelectedEventFunctions.hh;
    constructor defaults from monte_sampling.cpp:3272-3295)."""

    def __init__(self, jumps_per_position_sample: int = 1, max_n_position_samples: int = 100,
                 output_incomplete_samples: bool = False, stop_run_when_complete: bool = False):
        self.jumps_per_position_sample = int(jumps_per_position_sample)
        self.max_n_position_samples = int(max_n_position_samples)
        self.output_incomplete_samples = bool(output_incomplete_samples)
        self.stop_run_when_complete = bool(stop_run_when_complete)

    def copy(self) -> "CorrelationsDataParams":
        return self.__copy__()

    def __copy__(self) -> "CorrelationsDataParams":
        return CorrelationsDataParams(self.jumps_per_position_sample, self.max_n_position_samples,
                                      self.output_incomplete_samples, self.stop_run_when_complete)

    def __deepcopy__(self, memo):
        return self.__copy__()

    def to_dict(self) -> dict:
        """SelectedEventFunctions_json_io.cc: to_json(CorrelationsDataParams)."""
        return {
            "jumps_per_position_sample": self.jumps_per_position_sample,
            "max_n_position_samples": self.max_n_position_samples,
            "output_incomplete_samples": self.output_incomplete_samples,
            "stop_run_when_complete": self.stop_run_when_complete,
        }

    @staticmethod
    def from_dict(data: dict) -> "CorrelationsDataParams":
        """SelectedEventFunctions_json_io.cc: parse(InputParser<CorrelationsDataParams>),
        every key optional with the constructor's default."""
        try:
            return CorrelationsDataParams(
                jumps_per_position_sample=int(data.get("jumps_per_position_sample", 1)),
                max_n_position_samples=int(data.get("max_n_position_samples", 100)),
                output_incomplete_samples=bool(data.get("output_incomplete_samples", False)),
                stop_run_when_complete=bool(data.get("stop_run_when_complete", False)))
        except (TypeError, ValueError, AttributeError) as e:
            raise RuntimeError("Error in libcasm.monte.sampling.CorrelationsDataParams.from_dict") from e

    def __repr__(self) -> str:
        return repr(self.to_dict())


class CorrelationsData:
    """Atom positions stored every ``jumps_per_position_sample`` jumps of each atom
    (SelectedEventFunctions.cc:9-72)."""

    def __init__(self):
        self.jumps_per_position_sample = 1
        self.max_n_position_samples = 0
        self.output_incomplete_samples = False
        self.stop_run_when_complete = False
        self.n_position_samples: list[int] = []
        self.n_complete_samples = 0
        self.step = np.zeros((0, 0), dtype=np.int64)
        self.pass_ = np.zeros((0, 0), dtype=np.int64)
        self.time = np.zeros((0, 0), dtype=np.float64)
        self.atom_positions_cart: list[np.ndarray] = []

    # ``pass`` is a Python keyword; the reference exposes the matrix under that name.
    def __getattr__(self, name):
        if name == "pass":
            return self.pass_
        raise AttributeError(name)

    def initialize(self, n_atoms: int, jumps_per_position_sample: int, max_n_position_samples: int,
                   output_incomplete_samples: bool) -> None:
        """SelectedEventFunctions.cc:9-27: zeroed (max_n_position_samples x n_atoms) matrices."""
        self.jumps_per_position_sample = int(jumps_per_position_sample)
        self.max_n_position_samples = int(max_n_position_samples)
        self.output_incomplete_samples = bool(output_incomplete_samples)
        self.n_position_samples = [0] * int(n_atoms)
        self.n_complete_samples = 0
        shape = (self.max_n_position_samples, int(n_atoms))
        self.step = np.zeros(shape, dtype=np.int64)
        self.pass_ = np.zeros(shape, dtype=np.int64)
        self.time = np.zeros(shape, dtype=np.float64)
        self.atom_positions_cart = [np.zeros((3, int(n_atoms))) for _ in range(self.max_n_position_samples)]

    def insert(self, atom_id: int, n_jumps: int, position_cart, step: int, pass_: int = None,
               time: float = 0.0, **kwargs) -> None:
        """SelectedEventFunctions.cc:29-53: store on every ``jumps_per_position_sample``-th
        jump while the atom has room, then advance ``n_complete_samples``."""
        if pass_ is None:
            pass_ = kwargs.pop("pass")
        if int(n_jumps) % self.jumps_per_position_sample != 0:
            return
        n_samples = self.n_position_samples[atom_id]
        if n_samples >= self.max_n_position_samples:
            return
        self.step[n_samples, atom_id] = step
        self.pass_[n_samples, atom_id] = pass_
        self.time[n_samples, atom_id] = time
        self.atom_positions_cart[n_samples][:, atom_id] = np.asarray(position_cart, dtype=np.float64)
        self.n_position_samples[atom_id] += 1
        # SelectedEventFunctions.cc:55-65
        if n_samples == self.n_complete_samples:
            if all(x != self.n_complete_samples for x in self.n_position_samples):
                self.n_complete_samples += 1

    def indices_after_pass(self, pass_: int = None, **kwargs) -> list[int]:
        """monte_sampling.cpp:3470-3497: rows j < n_complete_samples whose largest pass is
        at least ``pass``."""
        if pass_ is None:
            pass_ = kwargs.pop("pass")
        if self.n_complete_samples >= self.pass_.shape[0]:
            raise RuntimeError("Error in monte.sampling.CorrelationsData.indices_after_pass: "
                               "n_complete_samples >= pass.rows()")
        return [j for j in range(self.n_complete_samples) if int(self.pass_[j].max()) >= pass_]

    def indices_after_time(self, time: int) -> list[int]:
        """monte_sampling.cpp:3498-3525: the row maximum is truncated to an integer before
        the comparison, as the reference does."""
        if self.n_complete_samples >= self.time.shape[0]:
            raise RuntimeError("Error in monte.sampling.CorrelationsData.indices_after_time: "
                               "n_complete_samples >= time.rows()")
        return [j for j in range(self.n_complete_samples) if int(self.time[j].max()) >= time]

    def to_dict(self) -> dict:
        """SelectedEventFunctions_json_io.cc: to_json(CorrelationsData); matrices as lists
        of rows, only complete rows unless ``output_incomplete_samples``."""
        n = self.step.shape[0] if self.output_incomplete_samples else self.n_complete_samples
        return {
            "jumps_per_position_sample": self.jumps_per_position_sample,
            "max_n_position_samples": self.max_n_position_samples,
            "output_incomplete_samples": self.output_incomplete_samples,
            "n_position_samples": list(self.n_position_samples),
            "n_complete_samples": self.n_complete_samples,
            "step": self.step[:n].tolist(),
            "pass": self.pass_[:n].tolist(),
            "time": self.time[:n].tolist(),
            "atom_positions_cart": [self.atom_positions_cart[i].tolist() for i in range(n)],
        }

    def __repr__(self) -> str:
        return repr({"n_complete_samples": self.n_complete_samples,
                     "jumps_per_position_sample": self.jumps_per_position_sample,
                     "max_n_complete_samples": self.max_n_position_samples,
                     "n_atoms": self.step.shape[1]})


# -- Discrete vector histograms ----------------------------------------------

def _float_lex_less(a, b, tol: float) -> bool:
    """Lexicographical order with a tolerance (libcasm-global's
    float_lexicographical_compare, used by FloatLexicographicalCompare in
    include/casm/monte/misc/LexicographicalCompare.hh): the first pair that differs by
    more than ``tol`` decides; otherwise the shorter vector is less."""
    for x, y in zip(a, b):
        if x < y - tol:
            return True
        if y < x - tol:
            return False
    return len(a) < len(b)


class _DiscreteHistogram:
    """Count per distinct vector value, kept in key order like the reference's
    std::map, with at most ``max_size`` distinct values (SelectedEventFunctions.cc:76-200)."""

    _dtype = np.int64

    def __init__(self, component_names, shape, max_size: int = 10000, value_labels=None):
        self._shape = [int(x) for x in shape]
        self._component_names = list(component_names)
        self._max_size = int(max_size)
        self._max_size_exceeded = False
        self._out_of_range_count = 0.0
        self._keys: list[tuple] = []
        self._counts: list[float] = []
        self._value_labels = None if value_labels is None else list(value_labels)

    def _less(self, a: tuple, b: tuple) -> bool:
        return a < b

    def _key(self, value) -> tuple:
        return tuple(self._dtype(x).item() for x in np.atleast_1d(np.asarray(value)))

    def _find(self, key: tuple):
        lo, hi = 0, len(self._keys)
        while lo < hi:
            mid = (lo + hi) // 2
            if self._less(self._keys[mid], key):
                lo = mid + 1
            else:
                hi = mid
        found = lo < len(self._keys) and not self._less(key, self._keys[lo])
        return lo, found

    def shape(self) -> list[int]:
        return list(self._shape)

    def component_names(self) -> list[str]:
        return list(self._component_names)

    def size(self) -> int:
        return len(self._keys)

    def max_size(self) -> int:
        return self._max_size

    def max_size_exceeded(self) -> bool:
        return self._max_size_exceeded

    def insert(self, value, weight: float = 1.0) -> None:
        key = self._key(value)
        pos, found = self._find(key)
        if not found:
            if len(self._keys) == self._max_size:
                self._max_size_exceeded = True
                self._out_of_range_count += weight
                return
            self._keys.insert(pos, key)
            self._counts.insert(pos, 0.0)
        self._counts[pos] += weight

    def sum(self) -> float:
        s = self._out_of_range_count
        for c in self._counts:
            s += c
        return s

    def values(self) -> list[np.ndarray]:
        return [np.array(k, dtype=self._dtype) for k in self._keys]

    def count(self) -> list[float]:
        return list(self._counts)

    def out_of_range_count(self) -> float:
        return self._out_of_range_count

    def fraction(self) -> list[float]:
        s = self.sum()
        return [c / s for c in self._counts]

    def value_counts(self) -> list[tuple[np.ndarray, float]]:
        return [(np.array(k, dtype=self._dtype), c) for k, c in zip(self._keys, self._counts)]

    def value_labels(self):
        return self._value_labels

    def _label_for(self, key: tuple):
        for v, label in self._value_labels:
            k = self._key(v)
            if not self._less(k, key) and not self._less(key, k):
                return label
        return None

    def to_dict(self) -> dict:
        """SelectedEventFunctions_json_io.cc: _discrete_histogram_to_json."""
        scalar = len(self._shape) == 0
        d = {"shape": self.shape(), "max_size": self._max_size, "max_size_exceeded": self._max_size_exceeded,
             "size": self.size(), "sum": self.sum()}
        if not scalar:
            d["component_names"] = self.component_names()
        if self._value_labels is not None:
            labels = []
            for k in self._keys:
                label = self._label_for(k)
                labels.append(label if label is not None else (k[0] if scalar else list(k)))
            d["labels"] = labels
        d["values"] = [k[0] for k in self._keys] if scalar else [list(k) for k in self._keys]
        d["count"] = self.count()
        d["fraction"] = self.fraction()
        d["out_of_range_count"] = self._out_of_range_count
        return d

    def __repr__(self) -> str:
        return repr({"size": self.size(), "sum": self.sum()})


class DiscreteVectorIntHistogram(_DiscreteHistogram):
    """Histogram of integer vector values (SelectedEventFunctions.cc:76-136)."""


class DiscreteVectorFloatHistogram(_DiscreteHistogram):
    """Histogram of float vector values; values within ``tol`` (component-wise, in
    lexicographical order) share a bin (SelectedEventFunctions.cc:140-200)."""

    _dtype = np.float64

    def __init__(self, component_names, shape, tol: float = _CASM_TOL, max_size: int = 10000, value_labels=None):
        super().__init__(component_names, shape, max_size, value_labels)
        self._tol = float(tol)

    def _less(self, a: tuple, b: tuple) -> bool:
        return _float_lex_less(a, b, self._tol)

    def tol(self) -> float:
        return self._tol


class DiscreteVectorIntHistogramMap(dict):
    pass


class DiscreteVectorFloatHistogramMap(dict):
    pass


# -- Continuous 1D histograms -------------------------------------------------

class Histogram1D:
    """1D histogram with bins of fixed width that grow in either direction up to
    ``max_size`` bins (SelectedEventFunctions.cc:204-392). With ``is_log`` the bins are
    in log10 space."""

    def __init__(self, initial_begin: float = 0.0, bin_width: float = 1.0, is_log: bool = False,
                 max_size: int = 10000):
        self._initial_begin = float(initial_begin)
        self._bin_width = float(bin_width)
        self._is_log = bool(is_log)
        self._max_size = int(max_size)
        self._max_size_exceeded = False
        self._begin = float(initial_begin)
        self._count: list[float] = []
        self._out_of_range_count = 0.0

    def bin_width(self) -> float:
        return self._bin_width

    def is_log(self) -> bool:
        return self._is_log

    def initial_begin(self) -> float:
        return self._initial_begin

    def size(self) -> int:
        return len(self._count)

    def max_size(self) -> int:
        return self._max_size

    def max_size_exceeded(self) -> bool:
        return self._max_size_exceeded

    def begin(self) -> float:
        return self._begin

    def count(self) -> list[float]:
        return list(self._count)

    def out_of_range_count(self) -> float:
        return self._out_of_range_count

    def insert(self, value: float, weight: float = 1.0) -> None:
        """Insert ``value`` (its log10 when ``is_log``) with ``weight``."""
        if self._is_log:
            self._insert(math.log10(value) if value > 0 else (-math.inf if value == 0 else math.nan), weight)
        else:
            self._insert(float(value), weight)

    def insert_log_value(self, log_value: float, weight: float = 1.0) -> None:
        if not self._is_log:
            raise RuntimeError("Error in Histogram1D::insert_log_value: histogram is not in log space")
        self._insert(float(log_value), weight)

    def bin_coords(self) -> list[float]:
        return [self._begin + i * self._bin_width for i in range(len(self._count))]

    def sum(self) -> float:
        s = self._out_of_range_count
        for c in self._count:
            s += c
        return s

    def density(self) -> list[float]:
        s = self.sum()
        return [c / (s * self._bin_width) for c in self._count]

    def merge(self, other: "Histogram1D") -> None:
        """SelectedEventFunctions.cc:264-293: re-insert each of ``other``'s bins at its
        lower edge."""
        if self._is_log != other._is_log:
            raise RuntimeError("Error in Histogram1D::merge: cannot merge histograms with different log settings")
        if self._bin_width != other._bin_width:
            raise RuntimeError("Error in Histogram1D::merge: cannot merge histograms with different bin_width values")
        if self._initial_begin != other._initial_begin:
            raise RuntimeError(
                "Error in Histogram1D::merge: cannot merge histograms with different initial_begin values")
        coords = other.bin_coords()
        counts = list(other._count)
        for x, c in zip(coords, counts):
            if self._is_log:
                self.insert_log_value(x, c)
            else:
                self.insert(x, c)
        self._out_of_range_count += other._out_of_range_count

    def _insert(self, value: float, weight: float) -> None:
        # SelectedEventFunctions.cc:315-345
        if value < self._begin or not self._count:
            self._reset_bins(value)
        if value < self._begin and self._max_size_exceeded:
            self._out_of_range_count += weight
            return
        b = math.floor((value - self._begin) / self._bin_width + 1e-10)
        while b >= len(self._count):
            if len(self._count) == self._max_size:
                self._max_size_exceeded = True
                self._out_of_range_count += weight
                return
            self._count.append(0.0)
        self._count[b] += weight

    def _reset_bins(self, value: float) -> None:
        # SelectedEventFunctions.cc:353-384
        if not math.isfinite(value):
            raise RuntimeError(f"Error in Histogram1D::_reset_bins: value (={value}) is not finite.")
        if not self._count:
            while value < self._begin:
                self._begin -= self._bin_width
            while value > self._begin + self._bin_width:
                self._begin += self._bin_width
            return
        n_prepend = 0
        while value < self._begin:
            if n_prepend + len(self._count) == self._max_size:
                self._max_size_exceeded = True
                break
            self._begin -= self._bin_width
            n_prepend += 1
        if n_prepend:
            self._count = [0.0] * n_prepend + self._count

    def to_dict(self) -> dict:
        """SelectedEventFunctions_json_io.cc: to_json(Histogram1D)."""
        return {"max_size": self._max_size, "max_size_exceeded": self._max_size_exceeded, "is_log": self._is_log,
                "begin": self._begin, "bin_width": self._bin_width, "count": self.count(),
                "bin_coords": self.bin_coords(), "sum": self.sum(), "density": self.density(),
                "out_of_range_count": self._out_of_range_count}

    def __repr__(self) -> str:
        return repr({"size": self.size(), "sum": self.sum()})


class Histogram1DVector(list):
    pass


def combine(histograms) -> Histogram1D:
    """SelectedEventFunctions.cc:396-410: merge every histogram into a copy of the first."""
    if len(histograms) == 0:
        raise RuntimeError("Error in combine: cannot combine empty vector of histograms")
    combined = copy.deepcopy(histograms[0])
    for h in histograms[1:]:
        combined.merge(h)
    return combined


class PartitionedHistogram1D:
    """One Histogram1D per partition (e.g. per event type) plus their combination
    (SelectedEventFunctions.hh:395-458, .cc:413-438)."""

    def __init__(self, partition_names, initial_begin: float = 0.0, bin_width: float = 1.0, is_log: bool = False,
                 max_size: int = 10000):
        self._partition_names = list(partition_names)
        self._histograms = [Histogram1D(initial_begin, bin_width, is_log, max_size)
                            for _ in self._partition_names]
        self._up_to_date = False
        self._combined: Optional[Histogram1D] = None

    def partition_names(self) -> list[str]:
        return list(self._partition_names)

    def insert(self, partition_name: int, value: float, weight: float = 1.0) -> None:
        partition = int(partition_name)
        self._up_to_date = False
        if partition < 0 or partition >= len(self._histograms):
            raise RuntimeError("Partition index out of range")
        if not math.isfinite(value):
            raise RuntimeError(f'Error in PartitionedHistogram1D::insert: for partition='
                               f'"{self._partition_names[partition]}" value (={value}) is not finite.')
        self._histograms[partition].insert(value, weight)

    def _make_combined_histogram(self) -> None:
        # Align every partition to the combined bins with zero-weight inserts at the
        # first and last combined bin (SelectedEventFunctions.cc:422-438).
        self._combined = combine(self._histograms)
        coords = self._combined.bin_coords()
        if coords:
            for h in self._histograms:
                if self._combined.is_log():
                    h.insert_log_value(coords[0], 0.0)
                    h.insert_log_value(coords[-1], 0.0)
                else:
                    h.insert(coords[0], 0.0)
                    h.insert(coords[-1], 0.0)
        self._up_to_date = True

    def histograms(self) -> Histogram1DVector:
        if len(self._histograms) != 1 and not self._up_to_date:
            self._make_combined_histogram()
        return Histogram1DVector(self._histograms)

    def combined_histogram(self) -> Histogram1D:
        if len(self._histograms) == 1:
            return self._histograms[0]
        if not self._up_to_date:
            self._make_combined_histogram()
        return self._combined

    def to_dict(self) -> dict:
        """SelectedEventFunctions_json_io.cc: to_json(PartitionedHistogram1D)."""
        if len(self._partition_names) == 1:
            return self.histograms()[0].to_dict()
        combined = self.combined_histogram()
        d = {"combined": combined.to_dict(), "partition_names": self.partition_names(), "partitions": []}
        for name, h in zip(self._partition_names, self.histograms()):
            frac = h.sum() / combined.sum()
            t = h.to_dict()
            t["partition_name"] = name
            t["partition_fraction"] = frac
            t["partial_density"] = [x * frac for x in h.density()]
            d["partitions"].append(t)
        return d

    def __repr__(self) -> str:
        return repr({"partition_names": self._partition_names})


class PartitionedHistogram1DMap(dict):
    pass


# -- Selected-event functions -------------------------------------------------

def _always_true() -> bool:
    return True


class _VectorHistogramFunction:
    """HistogramFunction.hh: a named vector-valued function with its histogram settings."""

    def __init__(self, name: str, description: str, shape, requires_event_state: bool, function: Callable,
                 has_value_function: Optional[Callable] = None, component_names=None, max_size: int = 10000):
        if function is None:
            raise RuntimeError(f"Error constructing {type(self).__name__}: function == nullptr")
        self.name = name
        self.description = description
        self.shape = [int(x) for x in shape]
        self.component_names = (list(component_names) if component_names is not None
                                else _default_component_names(self.shape))
        self.requires_event_state = bool(requires_event_state)
        self.function = function
        self.has_value_function = has_value_function if has_value_function is not None else _always_true
        self.max_size = int(max_size)
        self._value_labels = None

    def __call__(self):
        return self.function()

    def has_value(self) -> bool:
        return bool(self.has_value_function())

    def value_labels(self):
        """Optional list of (value, label) (monte_sampling.cpp:1415-1430)."""
        return self._value_labels

    def set_value_labels(self, value_labels) -> None:
        self._value_labels = None if value_labels is None else [(np.asarray(v), str(s)) for v, s in value_labels]


class VectorIntHistogramFunction(_VectorHistogramFunction):
    """monte_sampling.cpp:151-167, 1279-1458."""


class VectorFloatHistogramFunction(_VectorHistogramFunction):
    """monte_sampling.cpp:169-185, 1470-1659."""

    def __init__(self, name: str, description: str, shape, requires_event_state: bool, function: Callable,
                 has_value_function: Optional[Callable] = None, component_names=None, max_size: int = 10000,
                 tol: float = _CASM_TOL):
        super().__init__(name, description, shape, requires_event_state, function, has_value_function,
                         component_names, max_size)
        self.tol = float(tol)


class VectorIntHistogramFunctionMap(dict):
    pass


class VectorFloatHistogramFunctionMap(dict):
    pass


class PartitionedHistogramFunction:
    """A scalar function whose values are binned per partition
    (HistogramFunction.hh: PartitionedHistogramFunction; monte_sampling.cpp:187-204)."""

    def __init__(self, name: str, description: str, requires_event_state: bool, function: Callable,
                 partition_names, get_partition_function: Callable, is_log: bool = False,
                 initial_begin: float = 0.0, bin_width: float = 1.0, max_size: int = 10000):
        if function is None:
            raise RuntimeError("PartitionedHistogramFunction: function is empty")
        if get_partition_function is None:
            raise RuntimeError("PartitionedHistogramFunction: get_partition is empty")
        self.name = name
        self.description = description
        self.requires_event_state = bool(requires_event_state)
        self.function = function
        self.partition_names = list(partition_names)
        self.get_partition_function = get_partition_function
        self.is_log = bool(is_log)
        self.initial_begin = float(initial_begin)
        self.bin_width = float(bin_width)
        self.max_size = int(max_size)

    def __call__(self) -> float:
        return self.function()

    def partition(self) -> int:
        return int(self.get_partition_function())


class PartitionedHistogramFunctionMap(dict):
    pass


class GenericSelectedEventFunction:
    """A function evaluated after selected events, in ``order`` then name order
    (SelectedEventFunctions.cc:440-452; monte_sampling.cpp:206-220)."""

    def __init__(self, name: str, description: str, requires_event_state: bool, function: Callable,
                 has_value_function: Optional[Callable] = None, order: int = 0):
        if function is None:
            raise RuntimeError("Error constructing GenericSelectedEventFunction: function == nullptr")
        self.name = name
        self.description = description
        self.requires_event_state = bool(requires_event_state)
        self.function = function
        self.has_value_function = has_value_function if has_value_function is not None else _always_true
        self.order = int(order)

    def __call__(self) -> None:
        self.function()

    def has_value(self) -> bool:
        return bool(self.has_value_function())


class GenericSelectedEventFunctionMap(dict):
    pass


class SelectedEventFunctions:
    """The functions a method offers, by kind (SelectedEventFunctions.hh:490-520)."""

    def __init__(self):
        self.generic_functions = GenericSelectedEventFunctionMap()
        self.discrete_vector_int_functions = VectorIntHistogramFunctionMap()
        self.discrete_vector_float_functions = VectorFloatHistogramFunctionMap()
        self.continuous_1d_functions = PartitionedHistogramFunctionMap()

    def insert(self, f) -> None:
        """Add ``f`` under its name unless the name is taken (std::map::emplace)."""
        if isinstance(f, GenericSelectedEventFunction):
            self.generic_functions.setdefault(f.name, f)
        elif isinstance(f, VectorIntHistogramFunction):
            self.discrete_vector_int_functions.setdefault(f.name, f)
        elif isinstance(f, VectorFloatHistogramFunction):
            self.discrete_vector_float_functions.setdefault(f.name, f)
        elif isinstance(f, PartitionedHistogramFunction):
            self.continuous_1d_functions.setdefault(f.name, f)
        else:
            raise TypeError(f"SelectedEventFunctions.insert: unsupported function type {type(f).__name__}")

    def reset(self) -> None:
        self.generic_functions.clear()
        self.discrete_vector_int_functions.clear()
        self.discrete_vector_float_functions.clear()
        self.continuous_1d_functions.clear()


class SelectedEventFunctionParams:
    """Which selected-event quantities to collect, and per-quantity overrides of their
    histogram settings (SelectedEventFunctions.hh:523-628)."""

    def __init__(self):
        self._correlations_data_params: Optional[CorrelationsDataParams] = None
        self._function_names: list[str] = []
        self.order: dict[str, int] = {}
        self.tol: dict[str, float] = {}
        self.bin_width: dict[str, float] = {}
        self.initial_begin: dict[str, float] = {}
        self.is_log: dict[str, bool] = {}
        self.max_size: dict[str, int] = {}

    @property
    def correlations_data_params(self) -> Optional[CorrelationsDataParams]:
        return self._correlations_data_params

    def __copy__(self) -> "SelectedEventFunctionParams":
        return copy.deepcopy(self)

    def __deepcopy__(self, memo) -> "SelectedEventFunctionParams":
        c = SelectedEventFunctionParams()
        c._correlations_data_params = (None if self._correlations_data_params is None
                                       else self._correlations_data_params.__copy__())
        c._function_names = list(self._function_names)
        for k in ("order", "tol", "bin_width", "initial_begin", "is_log", "max_size"):
            setattr(c, k, dict(getattr(self, k)))
        return c

    @property
    def function_names(self) -> list[str]:
        return list(self._function_names)

    def collect_hop_correlations(self, jumps_per_position_sample: int = 1, max_n_position_samples: int = 100,
                                 output_incomplete_samples: bool = False,
                                 stop_run_when_complete: bool = False) -> "SelectedEventFunctionParams":
        self._correlations_data_params = CorrelationsDataParams(
            jumps_per_position_sample, max_n_position_samples, output_incomplete_samples, stop_run_when_complete)
        return self

    def do_not_collect_hop_correlations(self) -> "SelectedEventFunctionParams":
        self._correlations_data_params = None
        return self

    def evaluate(self, name: str, order: Optional[int] = None) -> "SelectedEventFunctionParams":
        self._function_names.append(name)
        if order is not None:
            self.order[name] = int(order)
        return self

    def collect(self, name: str, tol: Optional[float] = None, bin_width: Optional[float] = None,
                initial_begin: Optional[float] = None, spacing: Optional[str] = None,
                max_size: Optional[int] = None) -> "SelectedEventFunctionParams":
        self._function_names.append(name)
        if tol is not None:
            self.tol[name] = float(tol)
        if bin_width is not None:
            self.bin_width[name] = float(bin_width)
        if initial_begin is not None:
            self.initial_begin[name] = float(initial_begin)
        if spacing is not None:
            if spacing == "log":
                self.is_log[name] = True
            elif spacing == "linear":
                self.is_log[name] = False
            else:
                raise RuntimeError("Error in SelectedEventFunctionParams::set: spacing must be 'log' or 'linear'")
        if max_size is not None:
            self.max_size[name] = int(max_size)
        return self

    def do_not_collect(self, name: str) -> "SelectedEventFunctionParams":
        self._function_names = [x for x in self._function_names if x != name]
        for m in (self.order, self.tol, self.bin_width, self.initial_begin, self.is_log, self.max_size):
            m.pop(name, None)
        return self

    def get_parameters(self, name: str) -> dict:
        """monte_sampling.cpp:4219-4240."""
        d = {}
        if name in self.tol:
            d["tol"] = self.tol[name]
        if name in self.bin_width:
            d["bin_width"] = self.bin_width[name]
        if name in self.initial_begin:
            d["initial_begin"] = self.initial_begin[name]
        if name in self.is_log:
            d["spacing"] = "log" if self.is_log[name] else "linear"
        if name in self.max_size:
            d["max_size"] = self.max_size[name]
        return d

    def reset(self) -> None:
        self._correlations_data_params = None
        self._function_names.clear()
        for m in (self.order, self.tol, self.bin_width, self.initial_begin, self.is_log, self.max_size):
            m.clear()

    def copy(self) -> "SelectedEventFunctionParams":
        return copy.deepcopy(self)

    def to_dict(self) -> dict:
        """SelectedEventFunctions_json_io.cc: to_json(SelectedEventFunctionParams); the
        override maps are written only when non-empty, keys in sorted order."""
        d = {}
        if self._correlations_data_params is not None:
            d["correlations_data_params"] = self._correlations_data_params.to_dict()
        d["quantities"] = list(self._function_names)
        for key, m in (("tol", self.tol), ("bin_width", self.bin_width), ("initial_begin", self.initial_begin)):
            if m:
                d[key] = {k: m[k] for k in sorted(m)}
        if self.is_log:
            d["spacing"] = {k: ("log" if self.is_log[k] else "linear") for k in sorted(self.is_log)}
        if self.max_size:
            d["max_size"] = {k: self.max_size[k] for k in sorted(self.max_size)}
        return d

    @staticmethod
    def from_dict(data: dict) -> "SelectedEventFunctionParams":
        """SelectedEventFunctions_json_io.cc: parse(InputParser<SelectedEventFunctionParams>);
        per-quantity settings are read only for names listed in "quantities"."""
        err = RuntimeError("Error in libcasm.monte.sampling.SelectedEventFunctionParams.from_dict")
        p = SelectedEventFunctionParams()
        try:
            if data.get("correlations_data_params") is not None:
                p._correlations_data_params = CorrelationsDataParams.from_dict(data["correlations_data_params"])
            p._function_names = [str(x) for x in data.get("quantities", [])]
            for name in p._function_names:
                if name in data.get("tol", {}):
                    p.tol[name] = float(data["tol"][name])
                if name in data.get("bin_width", {}):
                    p.bin_width[name] = float(data["bin_width"][name])
                if name in data.get("initial_begin", {}):
                    p.initial_begin[name] = float(data["initial_begin"][name])
                if name in data.get("spacing", {}):
                    spacing = data["spacing"][name]
                    if spacing == "log":
                        p.is_log[name] = True
                    elif spacing == "linear":
                        p.is_log[name] = False
                    else:
                        raise ValueError(f'"{spacing}" is not a valid spacing option for "{name}".')
                if name in data.get("max_size", {}):
                    p.max_size[name] = int(data["max_size"][name])
        except (TypeError, ValueError, AttributeError, RuntimeError) as e:
            raise err from e
        return p

    def __repr__(self) -> str:
        return repr(self.to_dict())


class SelectedEventData:
    """Collected hop correlations and histograms (SelectedEventFunctions.hh:630-650)."""

    def __init__(self):
        self.correlations_data: Optional[CorrelationsData] = None
        self.discrete_vector_int_histograms = DiscreteVectorIntHistogramMap()
        self.discrete_vector_float_histograms = DiscreteVectorFloatHistogramMap()
        self.continuous_1d_histograms = PartitionedHistogram1DMap()

    def reset(self) -> None:
        self.correlations_data = None
        self.discrete_vector_int_histograms.clear()
        self.discrete_vector_float_histograms.clear()
        self.continuous_1d_histograms.clear()

    def to_dict(self) -> dict:
        """SelectedEventFunctions_json_io.cc: to_json(SelectedEventData)."""
        d = {}
        if self.correlations_data is not None:
            d["correlations_data"] = self.correlations_data.to_dict()
        hists = {}
        for m in (self.discrete_vector_int_histograms, self.discrete_vector_float_histograms,
                  self.continuous_1d_histograms):
            for name in sorted(m):
                hists[name] = m[name].to_dict()
        if hists:
            d["histograms"] = hists
        return d


class SelectedEventDataCollector:
    """Builds the histograms a params object asks for and fills them after each selected
    event (SelectedEventFunctions.cc:455-732)."""

    def __init__(self, functions: SelectedEventFunctions, params: SelectedEventFunctionParams,
                 data: SelectedEventData):
        if data is None:
            raise RuntimeError("Error in SelectedEventDataCollector: null selected_event_data")
        self.data = data
        self.requires_event_state = False
        self.discrete_vector_int_f, self.discrete_vector_int_hist = [], []
        self.discrete_vector_float_f, self.discrete_vector_float_hist = [], []
        self.continuous_1d_f, self.continuous_1d_hist = [], []
        data.reset()
        ordered_generic = {}
        for name in params.function_names:
            if name in functions.generic_functions:
                f = copy.copy(functions.generic_functions[name])
                if name in params.order:
                    f.order = params.order[name]
                ordered_generic.setdefault((f.order, f.name), f)
                self.requires_event_state |= f.requires_event_state
            elif name in functions.discrete_vector_int_functions:
                f = copy.copy(functions.discrete_vector_int_functions[name])
                self.requires_event_state |= f.requires_event_state
                if name in params.max_size:
                    f.max_size = params.max_size[name]
                h = data.discrete_vector_int_histograms.setdefault(
                    name, DiscreteVectorIntHistogram(f.component_names, f.shape, f.max_size, f.value_labels()))
                self.discrete_vector_int_f.append(f)
                self.discrete_vector_int_hist.append(h)
            elif name in functions.discrete_vector_float_functions:
                f = copy.copy(functions.discrete_vector_float_functions[name])
                self.requires_event_state |= f.requires_event_state
                if name in params.tol:
                    f.tol = params.tol[name]
                if name in params.max_size:
                    f.max_size = params.max_size[name]
                h = data.discrete_vector_float_histograms.setdefault(
                    name, DiscreteVectorFloatHistogram(f.component_names, f.shape, f.tol, f.max_size,
                                                       f.value_labels()))
                self.discrete_vector_float_f.append(f)
                self.discrete_vector_float_hist.append(h)
            elif name in functions.continuous_1d_functions:
                f = copy.copy(functions.continuous_1d_functions[name])
                self.requires_event_state |= f.requires_event_state
                if name in params.initial_begin:
                    f.initial_begin = params.initial_begin[name]
                if name in params.bin_width:
                    f.bin_width = params.bin_width[name]
                if name in params.is_log:
                    f.is_log = params.is_log[name]
                if name in params.max_size:
                    f.max_size = params.max_size[name]
                h = data.continuous_1d_histograms.setdefault(
                    name, PartitionedHistogram1D(f.partition_names, f.initial_begin, f.bin_width, f.is_log,
                                                 f.max_size))
                self.continuous_1d_f.append(f)
                self.continuous_1d_hist.append(h)
            else:
                raise RuntimeError("Error in SelectedEventDataCollector: unknown quantity in "
                                   "selected_event_data_params: " + name)
        self.generic_f = [ordered_generic[k] for k in sorted(ordered_generic)]

    def collect_vector_int_data(self) -> None:
        for f, h in zip(self.discrete_vector_int_f, self.discrete_vector_int_hist):
            if f.has_value():
                h.insert(f.function(), 1.0)

    def collect_vector_float_data(self) -> None:
        for f, h in zip(self.discrete_vector_float_f, self.discrete_vector_float_hist):
            if f.has_value():
                h.insert(f.function(), 1.0)

    def collect_continuous_1d_data(self) -> None:
        """SelectedEventFunctions.cc:670-715, with the reference's validation messages."""
        for f, h in zip(self.continuous_1d_f, self.continuous_1d_hist):
            partition = f.partition()
            value = f.function()
            if partition < 0 or partition >= len(f.partition_names):
                raise RuntimeError(f'Error in PartitionedHistogram1D::insert: function (name="{f.name}") returned '
                                   f'a partition index (={partition}) that is out of range.')
            pname = f.partition_names[partition]
            if f.is_log:
                log_value = math.log10(value) if value > 0 else (-math.inf if value == 0 else math.nan)
                if not math.isfinite(log_value):
                    raise RuntimeError(f'Error in PartitionedHistogram1D::insert: function (name="{f.name}", '
                                       f'partition="{pname}") returned a value (={value}) with log10(value) '
                                       f'(={log_value}) that is not finite.')
            elif not math.isfinite(value):
                raise RuntimeError(f'Error in PartitionedHistogram1D::insert: function (name="{f.name}", '
                                   f'partition="{pname}")  returned a value (={value}) that is not finite.')
            h.insert(partition, value, 1.0)

    def evaluate_generic_functions(self) -> None:
        for f in self.generic_f:
            f.function()

    def collect(self) -> None:
        self.evaluate_generic_functions()
        self.collect_vector_int_data()
        self.collect_vector_float_data()
        self.collect_continuous_1d_data()


__all__ = [
    "CorrelationsData", "CorrelationsDataParams", "DiscreteVectorFloatHistogram", "DiscreteVectorFloatHistogramMap",
    "DiscreteVectorIntHistogram", "DiscreteVectorIntHistogramMap", "GenericSelectedEventFunction",
    "GenericSelectedEventFunctionMap", "Histogram1D", "Histogram1DVector", "PartitionedHistogram1D",
    "PartitionedHistogram1DMap", "PartitionedHistogramFunction", "PartitionedHistogramFunctionMap",
    "SelectedEventData", "SelectedEventDataCollector", "SelectedEventFunctionParams", "SelectedEventFunctions",
    "VectorFloatHistogramFunction", "VectorFloatHistogramFunctionMap", "VectorIntHistogramFunction",
    "VectorIntHistogramFunctionMap", "combine",
]
