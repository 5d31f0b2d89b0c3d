"""GB300-native lattice Metropolis Monte Carlo with libcasm-monte's API.

Module layout mirrors ``libcasm.monte`` (python/libcasm/monte/__init__.py:3-8):

* ``casmcode_monte_gb300``            MethodLog, RandomNumberEngine, RandomNumberGenerator, ValueMap
* ``casmcode_monte_gb300.sampling``   samplers, completion/equilibration/convergence checks
* ``casmcode_monte_gb300.methods``    metropolis_acceptance, basic_occupation_metropolis
* ``casmcode_monte_gb300.events``     Conversions, OccCandidate/OccSwap/OccEvent/OccLocation
* ``casmcode_monte_gb300.ising_cpp``  the 2-D Ising model
* ``casmcode_monte_gb300.ising_cpp.semigrand_canonical``  SGC calculator (GPU serial replay)
* ``casmcode_monte_gb300.clex``       FCC cluster-expansion model and GPU coloured sweeps

The Metropolis loops run in ``libmontegpu.so`` (hand-written sm_103a kernels behind the
C-ABI in ``include/montegpu.h``); there is no CPU fallback.
"""
from __future__ import annotations

import copy
import ctypes as C
import json
import os
import sys
import time
from typing import Optional

import numpy as np

from . import _lib

__version__ = "1.0.0"


class RandomNumberEngine:
    """A pseudo-random number engine, std::mt19937_64 (monte.cpp:469-513).

    The default constructor seeds from std::random_device, as the reference does.
    """

    def __init__(self):
        h = C.c_void_p()
        _lib.check(_lib.lib().mg_engine_create(1, C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.mg_engine_destroy(h)
            self._h = None

    def seed(self, value: int) -> None:
        _lib.check(_lib.lib().mg_engine_seed(self._h, C.c_uint64(int(value) & (2**64 - 1))))

    def seed_seq(self, values: list[int]) -> None:
        a = np.ascontiguousarray(np.asarray(values, dtype=np.uint64))
        _lib.check(_lib.lib().mg_engine_seed_seq(self._h, _lib.ptr(a, C.c_uint64), a.size))

    def dump(self) -> str:
        buf = C.create_string_buffer(16384)
        _lib.check(_lib.lib().mg_engine_dump(self._h, buf, len(buf)))
        return buf.value.decode()

    def load(self, state: str) -> None:
        _lib.check(_lib.lib().mg_engine_load(self._h, state.encode()))

    def __copy__(self):
        e = RandomNumberEngine()
        e.load(self.dump())
        return e

    def __deepcopy__(self, memo):
        return self.__copy__()


class RandomNumberGenerator:
    """Uniform integers/reals from a shared RandomNumberEngine (RandomNumberGenerator.hh:15-42)."""

    def __init__(self, engine: Optional[RandomNumberEngine] = None):
        self._engine = engine if engine is not None else RandomNumberEngine()

    def engine(self) -> RandomNumberEngine:
        """The shared engine the draws come from."""
        return self._engine

    def random_int(self, maximum_value: int) -> int:
        """Uniformly distributed integer in [0, maximum_value]."""
        out = C.c_uint64()
        _lib.check(_lib.lib().mg_engine_random_int(self._engine._h, C.c_uint64(int(maximum_value)), C.byref(out)))
        return int(out.value)

    def random_real(self, maximum_value: float) -> float:
        """Uniformly distributed float in [0, maximum_value)."""
        out = C.c_double()
        _lib.check(_lib.lib().mg_engine_random_real(self._engine._h, float(maximum_value), C.byref(out)))
        return float(out.value)


class _TypedValueMap(dict):
    """A str-keyed dict that converts each value it stores (the bound std::map types of
    monte.cpp:106-109)."""

    def __init__(self, data=None):
        super().__init__()
        if data is not None:
            self.update(data)

    @staticmethod
    def _convert(value):
        return value

    def __setitem__(self, key: str, value) -> None:
        super().__setitem__(str(key), self._convert(value))

    def update(self, other=(), **kw) -> None:
        for k, v in dict(other, **kw).items():
            self[k] = v

    def setdefault(self, key: str, default=None):
        if key not in self:
            self[key] = default
        return self[key]

    def __deepcopy__(self, memo):
        return type(self)({k: copy.deepcopy(v, memo) for k, v in self.items()})


class BooleanValueMap(_TypedValueMap):
    """std::map<std::string, bool>."""

    @staticmethod
    def _convert(value):
        return bool(value)


class ScalarValueMap(_TypedValueMap):
    """std::map<std::string, double>."""

    @staticmethod
    def _convert(value):
        return float(value)


class VectorValueMap(_TypedValueMap):
    """std::map<std::string, Eigen::VectorXd>: values are 1-d float64 arrays."""

    @staticmethod
    def _convert(value):
        a = np.array(value, dtype=np.float64)
        if a.ndim == 2 and 1 in a.shape:
            a = a.reshape(-1)
        if a.ndim != 1:
            raise ValueError(f"VectorValueMap: expected a vector, got shape {a.shape}")
        return a


class MatrixValueMap(_TypedValueMap):
    """std::map<std::string, Eigen::MatrixXd>: values are 2-d float64 arrays."""

    @staticmethod
    def _convert(value):
        a = np.array(value, dtype=np.float64)
        if a.ndim != 2:
            raise ValueError(f"MatrixValueMap: expected a matrix, got shape {a.shape}")
        return a


class ValueMap:
    """Named boolean, scalar, vector and matrix values (ValueMap.hh:14-19).  The four
    attributes are the typed maps above; assigning a plain dict converts it, as the
    reference's read-write members do (monte.cpp:411-426)."""

    def __init__(self, data: Optional[dict] = None):
        self.boolean_values = BooleanValueMap()
        self.scalar_values = ScalarValueMap()
        self.vector_values = VectorValueMap()
        self.matrix_values = MatrixValueMap()
        if data is not None:
            v = ValueMap.from_dict(data)
            self.__dict__.update(v.__dict__)

    def _get(name):
        return property(lambda self: self.__dict__[name],
                        lambda self, value: self.__dict__.__setitem__(name, _MAP_TYPES[name](value)))

    boolean_values = _get("boolean_values")
    scalar_values = _get("scalar_values")
    vector_values = _get("vector_values")
    matrix_values = _get("matrix_values")
    del _get

    @staticmethod
    def from_dict(data: dict) -> "ValueMap":
        v = ValueMap()
        for k, x in data.items():
            if isinstance(x, bool):
                v.boolean_values[k] = x
            elif isinstance(x, (int, float)):
                v.scalar_values[k] = float(x)
            elif isinstance(x, str):
                raise ValueError(f"Error reading ValueMap from dict: unsupported type for '{k}'")
            else:
                a = np.asarray(x, dtype=float)
                if a.ndim == 1:
                    v.vector_values[k] = a
                elif a.ndim == 2:
                    v.matrix_values[k] = a
                else:
                    raise ValueError(f"Error reading ValueMap from dict: unsupported shape for '{k}'")
        return v

    def to_dict(self) -> dict:
        d: dict = {}
        d.update(self.boolean_values)
        d.update(self.scalar_values)
        d.update({k: v.tolist() for k, v in self.vector_values.items()})
        d.update({k: v.tolist() for k, v in self.matrix_values.items()})
        return d

    def is_mismatched(self, other: "ValueMap") -> bool:
        for a, b in ((self.boolean_values, other.boolean_values), (self.scalar_values, other.scalar_values),
                     (self.vector_values, other.vector_values), (self.matrix_values, other.matrix_values)):
            if set(a) != set(b):
                return True
        for k in self.vector_values:
            if self.vector_values[k].shape != other.vector_values[k].shape:
                return True
        for k in self.matrix_values:
            if self.matrix_values[k].shape != other.matrix_values[k].shape:
                return True
        return False

    def make_incremented_values(self, increment: "ValueMap", n_increment: float) -> "ValueMap":
        v = copy.deepcopy(self)
        for k, x in increment.scalar_values.items():
            v.scalar_values[k] = v.scalar_values.get(k, 0.0) + x * n_increment
        for k, x in increment.vector_values.items():
            v.vector_values[k] = v.vector_values.get(k, 0 * x) + x * n_increment
        for k, x in increment.matrix_values.items():
            v.matrix_values[k] = v.matrix_values.get(k, 0 * x) + x * n_increment
        return v

    def __copy__(self):
        return copy.deepcopy(self)

    def __deepcopy__(self, memo):
        v = ValueMap()
        v.boolean_values = self.boolean_values
        v.scalar_values = self.scalar_values
        v.vector_values = self.vector_values
        v.matrix_values = self.matrix_values
        return v


_MAP_TYPES = {"boolean_values": BooleanValueMap, "scalar_values": ScalarValueMap, "vector_values": VectorValueMap,
              "matrix_values": MatrixValueMap}


class MethodLog:
    """Status logger with a clock and laps (MethodLog.hh:13-38; monte.cpp:111-384)."""

    def __init__(self, logfile_path: Optional[str] = None, log_frequency: Optional[float] = None):
        self._logfile_path = logfile_path
        self._log_frequency = log_frequency
        self._t0 = time.perf_counter()
        self._lap = self._t0

    def logfile_path(self) -> Optional[str]:
        return self._logfile_path

    def log_frequency(self) -> Optional[float]:
        return self._log_frequency

    def restart_clock(self) -> None:
        self._t0 = time.perf_counter()

    def begin_lap(self) -> None:
        self._lap = time.perf_counter()

    def time_s(self) -> float:
        return time.perf_counter() - self._t0

    def lap_time(self) -> float:
        return time.perf_counter() - self._lap

    def reset(self) -> None:
        """Truncate the log file (status files are rewritten on each update)."""
        if self._logfile_path:
            os.makedirs(os.path.dirname(os.path.abspath(self._logfile_path)) or ".", exist_ok=True)
            open(self._logfile_path, "w").close()

    def reset_to_stdout(self) -> None:
        self._logfile_path = None

    def print(self, text: str) -> None:
        self._emit(text)

    def write_json(self, data) -> None:
        self.print(json.dumps(data, indent=2) + "\n")

    # -- verbosity, sections and formatted text (monte.cpp:150-384; the Log of
    # libcasm-global, restated): a section begun at a level prints only while the
    # verbosity is at least that level; text outside sections always prints.
    _LEVELS = {"quiet": 0, "standard": 1, "verbose": 2, "debug": 3}

    def _fmt_state(self) -> dict:
        st = self.__dict__.get("_fmt")
        if st is None:
            st = self.__dict__["_fmt"] = {"verbosity": 1, "sections": [], "indent": 0, "indent_space": 2,
                                          "initial_indent": 0, "clock": False, "width": 100,
                                          "justification": "left"}
        return st

    def _printing(self) -> bool:
        st = self._fmt_state()
        return not st["sections"] or st["sections"][-1] <= st["verbosity"]

    def _emit(self, text: str) -> None:
        if self._printing():
            if self._logfile_path:
                with open(self._logfile_path, "a") as f:
                    f.write(text)
            else:
                sys.stdout.write(text)

    def set_quiet(self) -> None:
        self._fmt_state()["verbosity"] = 0

    def set_standard(self) -> None:
        self._fmt_state()["verbosity"] = 1

    def set_verbose(self) -> None:
        self._fmt_state()["verbosity"] = 2

    def set_debug(self) -> None:
        self._fmt_state()["verbosity"] = 3

    def _begin(self, level: int) -> None:
        self._fmt_state()["sections"].append(level)

    def begin_section_print_always(self) -> None:
        self._begin(-1)

    def begin_section_print_if_quiet(self) -> None:
        self._begin(0)

    def begin_section_print_if_standard(self) -> None:
        self._begin(1)

    def begin_section_print_if_verbose(self) -> None:
        self._begin(2)

    def begin_section_print_if_debug(self) -> None:
        self._begin(3)

    def end_section(self) -> None:
        st = self._fmt_state()
        if st["sections"]:
            st["sections"].pop()

    def show_clock(self) -> None:
        self._fmt_state()["clock"] = True

    def hide_clock(self) -> None:
        self._fmt_state()["clock"] = False

    def increase_indent(self) -> None:
        self._fmt_state()["indent"] += 1

    def decrease_indent(self) -> None:
        st = self._fmt_state()
        st["indent"] = max(0, st["indent"] - 1)

    def set_indent_space(self, indent_space: int) -> None:
        self._fmt_state()["indent_space"] = int(indent_space)

    def set_initial_indent_space(self, initial_indent_space: int) -> None:
        self._fmt_state()["initial_indent"] = int(initial_indent_space)

    def indent_str(self) -> str:
        st = self._fmt_state()
        return " " * (st["initial_indent"] + st["indent"] * st["indent_space"])

    def set_paragraph_width(self, width: int) -> None:
        self._fmt_state()["width"] = int(width)

    def paragraph_width(self) -> int:
        return self._fmt_state()["width"]

    def set_paragraph_justification(self, justification_type: str) -> None:
        if justification_type not in ("left", "right", "center", "full"):
            raise ValueError(f"Error in MethodLog.set_paragraph_justification: invalid '{justification_type}'")
        self._fmt_state()["justification"] = justification_type

    def paragraph_justification(self) -> str:
        return self._fmt_state()["justification"]

    def section(self, what: str, show_clock: bool = False) -> None:
        """A heading "-- what -- ", with the elapsed time when asked or when the clock is shown."""
        text = self.indent_str() + "-- " + what + " -- "
        if show_clock or self._fmt_state()["clock"]:
            text += f"Time: {self.time_s()} (s)"
        self._emit(text + "\n")

    def paragraph(self, text: str) -> None:
        """Indented, wrapped to the paragraph width and justified."""
        import textwrap
        st = self._fmt_state()
        ind = self.indent_str()
        width = max(1, st["width"] - len(ind))
        lines = textwrap.wrap(" ".join(text.split()), width) or [""]
        out = []
        for i, line in enumerate(lines):
            j = st["justification"]
            if j == "right":
                line = line.rjust(width)
            elif j == "center":
                line = line.center(width).rstrip()
            elif j == "full" and i < len(lines) - 1 and " " in line:
                words, gaps = line.split(" "), line.count(" ")
                extra = width - len(line)
                q, r = divmod(extra, gaps)
                line = "".join(w + (" " * (1 + q + (k < r)) if k < gaps else "") for k, w in enumerate(words))
            out.append(ind + line)
        self._emit("\n".join(out) + "\n")

    def verbatim(self, text: str, indent_first_line: bool = True) -> None:
        """Each line indented, not re-wrapped or justified."""
        ind = self.indent_str()
        lines = text.split("\n")
        self._emit("\n".join((ind if (k or indent_first_line) else "") + line for k, line in enumerate(lines)) + "\n")


__all__ = ["BooleanValueMap", "MatrixValueMap", "MethodLog", "RandomNumberEngine", "RandomNumberGenerator",
           "ScalarValueMap", "ValueMap", "VectorValueMap"]

from . import _monte  # noqa: E402,F401  (the names at libcasm.monte._monte)
