"""2-D square-lattice Ising model with numpy calculators (mirrors
``libcasm.monte.ising_py``, python/libcasm/monte/ising_py/_model.py).

The reference's Python example model, kept with its own arithmetic:

* ``IsingConfiguration`` a 2-D ``int32`` array in column-major (Fortran) order, linear
  site index ``l = i + shape[0] * j`` (_model.py:12-120)
* ``IsingFormationEnergy`` E = -J (sum over i of s[i, :] . s[i+1, :] + sum over j of
  s[:, j] . s[:, j+1]), accumulated in that order; single-site change
  -J (new - s[i, j]) (s[i, j-1] + s[i, j+1] + s[i-1, j] + s[i+1, j]) (_model.py:151-300)
* ``IsingParamComposition`` N x = (N + sum s) / 2; its change is sum (new - old), as in
  the reference (_model.py:303-393)

These calculators answer per-state queries on the host; the Metropolis loop of
``ising_py.semigrand_canonical`` runs on the GPU.
"""
from __future__ import annotations

import copy
from typing import Optional

import numpy as np

from .. import ValueMap


class IsingConfiguration:
    """Ising model configuration on a periodic 2-D supercell (_model.py:12-120)."""

    def __init__(self, shape: tuple = (10, 10), fill_value: int = 1):
        self.shape: tuple = tuple(int(x) for x in shape)
        self._occupation = np.full(shape=self.shape, fill_value=fill_value, dtype=np.int32, order="F")
        self.n_sites: int = int(self._occupation.size)
        self.n_variable_sites: int = int(self._occupation.size)
        self.n_unitcells: int = int(self._occupation.size)

    def occupation(self) -> np.ndarray:
        """The current occupation (a read-only view)."""
        v = self._occupation.view()
        v.flags.writeable = False
        return v

    def set_occupation(self, occupation: np.ndarray) -> None:
        if self._occupation.shape != np.shape(occupation):
            raise Exception("Error in set_occupation: shape mismatch")
        self._occupation[:] = occupation

    def occ(self, linear_site_index: int) -> np.int32:
        return self._occupation[np.unravel_index(int(linear_site_index), self.shape, order="F")]

    def set_occ(self, linear_site_index: int, new_occ: int) -> None:
        self._occupation[np.unravel_index(int(linear_site_index), self.shape, order="F")] = new_occ

    @staticmethod
    def from_dict(data: dict) -> "IsingConfiguration":
        config = IsingConfiguration(shape=tuple(data["shape"]))
        occ = np.array(data["occupation"], dtype=np.int32)
        config.set_occupation(occ.reshape(config.shape, order="F"))
        return config

    def to_dict(self) -> dict:
        return {"shape": list(self.occupation().shape),
                "occupation": [int(x) for x in self.occupation().flatten(order="F")]}

    def within(self, index: int, dim: int) -> int:
        """Index of the periodic image inside the array along ``dim``."""
        return index % self.shape[dim]

    def from_linear_site_index(self, linear_site_index: int):
        return np.unravel_index(linear_site_index, self.shape, order="F")

    def to_linear_site_index(self, multi_index: tuple):
        return np.ravel_multi_index(multi_index, self.shape, order="F")


class IsingState:
    """Configuration, conditions and calculated properties (_model.py:123-148)."""

    def __init__(self, configuration: IsingConfiguration, conditions: ValueMap):
        self.configuration = configuration
        self.conditions = conditions
        self.properties = ValueMap()


class IsingFormationEnergy:
    """Ising model formation energy, square lattice (_model.py:151-300)."""

    def __init__(self, J: float = 1.0, lattice_type: int = 1, state: Optional[IsingState] = None):
        self.J: float = J
        if lattice_type not in [1]:
            raise Exception("Unsupported lattice_type")
        self.lattice_type: int = lattice_type
        self.state: Optional[IsingState] = None
        if state is not None:
            self.set_state(state)

    def set_state(self, state: IsingState) -> None:
        if self.lattice_type == 1 and not isinstance(state.configuration, IsingConfiguration):
            raise Exception("IsingConfiguration is required for lattice_type == 1")
        self.state = state

    def per_supercell(self) -> float:
        config = self.state.configuration
        sites = config.occupation()
        e_formation = 0.0
        for i in range(sites.shape[0]):
            e_formation += -self.J * np.dot(sites[i, :], sites[config.within(i + 1, dim=0), :])
        for j in range(sites.shape[1]):
            e_formation += -self.J * np.dot(sites[:, j], sites[:, config.within(j + 1, dim=1)])
        return e_formation

    def per_unitcell(self) -> float:
        return self.per_supercell() / self.state.configuration.n_unitcells

    def _single_occ_delta_per_supercell(self, linear_site_index: int, new_occ: int) -> float:
        config = self.state.configuration
        sites = config.occupation()
        i, j = config.from_linear_site_index(linear_site_index)
        ds = new_occ - sites[i, j]
        return -self.J * ds * (sites[i, config.within(j - 1, dim=1)] + sites[i, config.within(j + 1, dim=1)]
                               + sites[config.within(i - 1, dim=0), j] + sites[config.within(i + 1, dim=0), j])

    def occ_delta_per_supercell(self, linear_site_index, new_occ) -> float:
        config = self.state.configuration
        if len(linear_site_index) == 1:
            return self._single_occ_delta_per_supercell(linear_site_index[0], new_occ[0])
        # sequential apply of each flip, then undo
        dE = 0.0
        original = []
        for index, value in zip(linear_site_index, new_occ):
            dE += self._single_occ_delta_per_supercell(index, value)
            original.append(config.occ(index))
            config.set_occ(index, value)
        for index, value in zip(linear_site_index, original):
            config.set_occ(index, value)
        return dE

    def __deepcopy__(self, memo):
        return IsingFormationEnergy(J=copy.deepcopy(self.J), lattice_type=copy.deepcopy(self.lattice_type))


class IsingParamComposition:
    """Parametric composition, x = 1 for all +1 and x = 0 for all -1 (_model.py:303-393)."""

    def __init__(self, state: Optional[IsingState] = None):
        self.state = None
        if state is not None:
            self.set_state(state)

    def set_state(self, state: IsingState) -> None:
        self.state = state
        if not isinstance(state.configuration, IsingConfiguration):
            raise Exception("IsingConfiguration is required for IsingParamComposition")

    def n_independent_compositions(self) -> int:
        return 1

    def per_supercell(self) -> np.ndarray:
        config = self.state.configuration
        return np.array([(config.n_variable_sites + np.sum(config.occupation())) / 2.0], dtype=np.double)

    def per_unitcell(self) -> np.ndarray:
        return self.per_supercell() / self.state.configuration.n_unitcells

    def occ_delta_per_supercell(self, linear_site_index, new_occ) -> np.ndarray:
        config = self.state.configuration
        Ndx = np.array([0.0], dtype=np.double)
        for index, value in zip(linear_site_index, new_occ):
            Ndx[0] += value - config.occ(index)
        return Ndx


class IsingSystem:
    """Formation energy and parametric composition calculators (_model.py:396-414)."""

    def __init__(self, formation_energy_calculator: IsingFormationEnergy,
                 param_composition_calculator: Optional[IsingParamComposition] = None):
        self.formation_energy_calculator = formation_energy_calculator
        self.param_composition_calculator = param_composition_calculator


__all__ = ["IsingConfiguration", "IsingFormationEnergy", "IsingParamComposition", "IsingState", "IsingSystem"]
