"""2-D square-lattice Ising model (mirrors ``libcasm.monte.ising_cpp``).

Classes and arithmetic follow include/casm/monte/ising_cpp/model.hh:19-452:

* ``IsingConfiguration``  periodic 2-D supercell, column-major ``l = shape[0]*j + i``,
  occupation values +1/-1 (n_sites = n_variable_sites = n_unitcells)
* ``IsingFormationEnergy`` E = -J sum_l s_l (s_{i+1,j} + s_{i,j+1}); single-site change
  -J (new - old) (sum of the 4 neighbours); ``use_nlist`` selects the reference's two
  summation orders for E (both give the same value up to rounding)
* ``IsingParamComposition`` N x = (N + sum s) / 2 and N dx = sum (new - old) / 2

These host-side calculators answer the API's per-state queries; the Metropolis loop
itself runs on the GPU (``ising_cpp.semigrand_canonical``).
"""
from __future__ import annotations

import copy
from typing import Optional

import numpy as np

from .. import ValueMap, __version__  # noqa: F401


class IsingConfiguration:
    """Ising configuration on a 2-D periodic supercell (model.hh:19-110)."""

    def __init__(self, shape=(10, 10), fill_value: int = 1):
        shape = np.asarray(shape, dtype=np.int64).reshape(-1)
        if shape.size != 2:
            raise RuntimeError("IsingConfiguration only supports 2d")
        self.shape = shape
        self._occ = np.full(int(shape[0] * shape[1]), int(fill_value), dtype=np.int32)

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
        return self._occ

    def set_occupation(self, occupation) -> None:
        o = np.asarray(occupation, dtype=np.int32).reshape(-1)
        if o.size != self._occ.size:
            raise RuntimeError("Error in set_occupation: size mismatch")
        self._occ = o.copy()

    def occ(self, linear_site_index: int) -> int:
        return int(self._occ[linear_site_index])

    def set_occ(self, linear_site_index: int, new_occ: int) -> None:
        self._occ[linear_site_index] = new_occ

    def within(self, index: int, dim: int) -> int:
        s = int(self.shape[dim])
        r = int(index) % s  # Python modulo is already non-negative
        return r

    def from_linear_site_index(self, linear_site_index: int) -> np.ndarray:
        return np.array([linear_site_index % int(self.shape[0]), linear_site_index // int(self.shape[0])],
                        dtype=np.int64)

    def to_linear_site_index(self, multi_index) -> int:
        return int(self.shape[0] * multi_index[1] + multi_index[0])

    def to_dict(self) -> dict:
        return {"shape": self.shape.tolist(), "occupation": self._occ.tolist()}

    @staticmethod
    def from_dict(data: dict) -> "IsingConfiguration":
        if "shape" not in data:
            raise RuntimeError("Error reading IsingConfiguration from JSON: no 'shape'")
        if "occupation" not in data:
            raise RuntimeError("Error reading IsingConfiguration from JSON: no 'occupation'")
        c = IsingConfiguration(data["shape"])
        c.set_occupation(data["occupation"])
        return c

    def __copy__(self):
        return copy.deepcopy(self)

    def __deepcopy__(self, memo):
        c = IsingConfiguration(self.shape.copy())
        c._occ = self._occ.copy()
        return c


class IsingState:
    """Configuration, conditions and properties (model.hh:139-157)."""

    def __init__(self, configuration: IsingConfiguration, conditions: ValueMap,
                 properties: Optional[ValueMap] = None):
        self.configuration = configuration
        self.conditions = conditions
        self.properties = properties if properties is not None else ValueMap()

    def to_dict(self) -> dict:
        return {"configuration": self.configuration.to_dict(), "conditions": self.conditions.to_dict(),
                "properties": self.properties.to_dict()}

    @staticmethod
    def from_dict(data: dict) -> "IsingState":
        return IsingState(IsingConfiguration.from_dict(data["configuration"]),
                          ValueMap.from_dict(data.get("conditions", {})),
                          ValueMap.from_dict(data.get("properties", {})))

    def __copy__(self):
        return copy.deepcopy(self)

    def __deepcopy__(self, memo):
        return IsingState(copy.deepcopy(self.configuration), copy.deepcopy(self.conditions),
                          copy.deepcopy(self.properties))


def _nbr_sums(cfg: IsingConfiguration):
    rows, cols = int(cfg.shape[0]), int(cfg.shape[1])
    s = cfg.occupation().reshape(cols, rows).astype(np.int64)  # s[j, i]
    return rows, cols, s


class IsingFormationEnergy:
    """Ising model formation energy (model.hh:164-380)."""

    def __init__(self, J: float = 1.0, lattice_type: int = 1, use_nlist: bool = True,
                 state: Optional[IsingState] = None):
        if lattice_type != 1:
            raise RuntimeError("Unsupported lattice_type")
        self.J = float(J)
        self.lattice_type = lattice_type
        self.use_nlist = bool(use_nlist)
        self.state: Optional[IsingState] = None
        if state is not None:
            self.set_state(state)

    def set_state(self, state: IsingState) -> None:
        if state is None:
            raise RuntimeError("Error in IsingFormationEnergy::set_state: _state==nullptr")
        self.state = state

    def per_supercell(self) -> float:
        rows, cols, s = _nbr_sums(self.state.configuration)
        if self.use_nlist:
            bond = int(np.sum(s * (np.roll(s, -1, axis=1) + np.roll(s, -1, axis=0))))
            e = float(bond)
            e *= -self.J
            return e
        e = 0.0
        for i in range(rows):
            e += -self.J * float(int(np.dot(s[:, i], s[:, (i + 1) % rows])))
        for j in range(cols):
            e += -self.J * float(int(np.dot(s[j, :], s[(j + 1) % cols, :])))
        return e

    def per_unitcell(self) -> float:
        return self.per_supercell() / self.state.configuration.n_unitcells

    def _single_occ_delta_per_supercell(self, linear_site_index: int, new_occ: int) -> float:
        cfg = self.state.configuration
        rows, cols = int(cfg.shape[0]), int(cfg.shape[1])
        l = int(linear_site_index)
        i, j = l % rows, l // rows
        o = cfg.occupation()
        s4 = (int(o[(i + 1) % rows + rows * j]) + int(o[i + rows * ((j + 1) % cols)])
              + int(o[(i - 1) % rows + rows * j]) + int(o[i + rows * ((j - 1) % cols)]))
        return (-self.J * float(int(new_occ) - int(o[l]))) * float(s4)

    def occ_delta_per_supercell(self, linear_site_index, new_occ) -> float:
        idx = list(linear_site_index)
        new = list(new_occ)
        if len(idx) == 1:
            return self._single_occ_delta_per_supercell(idx[0], new[0])
        cfg = self.state.configuration
        dE = 0.0
        orig = []
        for l, v in zip(idx, new):
            dE += self._single_occ_delta_per_supercell(l, v)
            orig.append(cfg.occ(l))
            cfg.set_occ(l, v)
        for l, v in zip(idx, orig):
            cfg.set_occ(l, v)
        return dE

    def __copy__(self):
        return IsingFormationEnergy(self.J, self.lattice_type, self.use_nlist, self.state)

    def __deepcopy__(self, memo):
        return self.__copy__()


class IsingParamComposition:
    """Parametric composition x = 1 (all +1) .. 0 (all -1) (model.hh:388-436)."""

    def __init__(self, state: Optional[IsingState] = None):
        self.state: Optional[IsingState] = None
        if state is not None:
            self.set_state(state)

    def set_state(self, state: IsingState) -> None:
        if state is None:
            raise RuntimeError("Error in IsingParamComposition::set_state: _state==nullptr")
        self.state = state

    def n_independent_compositions(self) -> int:
        return 1

    def per_supercell(self) -> np.ndarray:
        o = self.state.configuration.occupation()
        return np.array([float(int(o.size) + int(np.sum(o, dtype=np.int64))) / 2.0])

    def per_unitcell(self) -> np.ndarray:
        return self.per_supercell() / self.state.configuration.n_unitcells

    def occ_delta_per_supercell(self, linear_site_index, new_occ) -> np.ndarray:
        cfg = self.state.configuration
        ndx = 0.0
        for l, v in zip(linear_site_index, new_occ):
            ndx += (int(v) - cfg.occ(l)) / 2.0
        return np.array([ndx])

    def __copy__(self):
        return IsingParamComposition(self.state)

    def __deepcopy__(self, memo):
        return self.__copy__()


class IsingSystem:
    """Holds the formation energy and parametric composition calculators (model.hh:439-452)."""

    def __init__(self, formation_energy_calculator: IsingFormationEnergy,
                 param_composition_calculator: IsingParamComposition):
        self.formation_energy_calculator = formation_energy_calculator
        self.param_composition_calculator = param_composition_calculator


__all__ = ["IsingConfiguration", "IsingFormationEnergy", "IsingParamComposition", "IsingState", "IsingSystem"]
