"""Canonical (fixed-composition) Monte Carlo of an FCC cluster expansion behind the
calculator interface of the semi-grand canonical module.

The reference's canonical event (events/OccEventProposal.hh:108-237,
``propose_canonical_event``: the occupants of two sites of different species exchanged)
accepted by metropolis.hh:26-35, run with the calculator pattern of
include/casm/monte/ising_cpp/basic_semigrand_canonical.hh:416-470:
``CanonicalCalculator(system).run(state, sampling_functions, json_sampling_functions,
completion_check_params, event_generator, sample_period, method_log, random_engine,
write_status_f)`` and ``run_fixtures(state, run_manager)``.  Conditions are the
temperature; the composition is the state's own and never changes.  The potential is the
formation energy.

``run`` sweeps the chain on the GPU (``CanonicalBatch``): each pass proposes, colour class
by colour class, a perfect matching of the class's sites and exchanges the occupants of each
pair by Metropolis, passes alternating between two colourings whose classes connect every
site.  The dynamics therefore equal the reference's in distribution (the canonical ensemble
at the state's composition), not step for step.  Completion checks, sampling and the default
sampling functions behave as in ``semigrand_canonical``.
"""
from __future__ import annotations

import numpy as np

from .. import ValueMap
from . import CanonicalBatch
from .semigrand_canonical import (ClexConfiguration, ClexFormationEnergy, ClexParamComposition, ClexState,
                                  ClexSystem, SemiGrandCanonicalCalculator, SemiGrandCanonicalConditions,
                                  SemiGrandCanonicalData, default_write_status)

__all__ = ["CanonicalConditions", "CanonicalEventGenerator", "CanonicalCalculator", "CanonicalData",
           "ClexConfiguration", "ClexState", "ClexSystem", "ClexFormationEnergy", "ClexParamComposition",
           "default_write_status"]

#: run data: the semi-grand canonical calculator's (samples, counts, completion check)
CanonicalData = SemiGrandCanonicalData


class CanonicalConditions:
    """Thermodynamic conditions at fixed composition: the temperature (K)."""

    def __init__(self, temperature: float = 0.0):
        self.temperature = float(temperature)

    @staticmethod
    def from_values(values: ValueMap) -> "CanonicalConditions":
        if "temperature" not in values.scalar_values:
            raise RuntimeError('Error in CanonicalConditions: missing "temperature"')
        return CanonicalConditions(values.scalar_values["temperature"])

    def to_values(self) -> ValueMap:
        v = ValueMap()
        v.scalar_values["temperature"] = self.temperature
        return v

    def to_dict(self) -> dict:
        return {"temperature": self.temperature}

    @staticmethod
    def from_dict(data: dict) -> "CanonicalConditions":
        return CanonicalConditions(data["temperature"])


class CanonicalEventGenerator:
    """The proposals of the GPU sweep: per colour class a perfect matching of its sites (a
    state-independent involution), the occupants of each pair of different species exchanged."""

    def __init__(self):
        self.state = None

    def set_state(self, state: ClexState) -> None:
        if state is None:
            raise RuntimeError("Error in CanonicalEventGenerator::set_state: state==nullptr")
        self.state = state


class CanonicalCalculator(SemiGrandCanonicalCalculator):
    """Canonical Monte Carlo calculator for a cluster-expansion system (the semi-grand
    canonical calculator with no exchange potential and pair exchanges instead of flips)."""

    def __init__(self, system: ClexSystem, precision: str = "fp64"):
        if system is None:
            raise RuntimeError("Error constructing CanonicalCalculator: system==nullptr")
        super().__init__(system, precision)
        #: the run's conditions as given (temperature)
        self.canonical_conditions = None

    def _conditions_from(self, values: ValueMap) -> SemiGrandCanonicalConditions:
        # no exchange potential: the potential of the run is the formation energy
        self.canonical_conditions = CanonicalConditions.from_values(values)
        n = self.system.model.n_species - 1
        return SemiGrandCanonicalConditions(self.canonical_conditions.temperature, np.zeros(n))

    def _default_event_generator(self):
        return CanonicalEventGenerator()

    def _make_batch(self, state: ClexState, mu: np.ndarray, seed: int):
        return CanonicalBatch(self.system.model, state.configuration.shape, state.configuration.occupation()[None, :],
                              [self.conditions.temperature], np.array([seed], dtype=np.uint64),
                              precision=self.precision)
