"""Monte Carlo events and occupant tracking (libcasm.monte.events).

Mirrors python/libcasm/monte/events/__init__.py:3-39 and the C++ it binds:

* ``Conversions`` (include/casm/monte/Conversions.hh:44-137, src/casm/monte/
  Conversions.cc:14-321): linear site index l <-> (b, i, j, k), b-major (l = b * N_uc +
  unit-cell index), asymmetric unit (sites equivalent by the prim factor group *and* with
  occupants listed in the same order), occupant index <-> species index.
* ``OccCandidate``, ``OccSwap``, ``MultiOccSwap``, ``OccCandidateList`` and the swap
  builders (include/casm/monte/events/OccCandidate.hh:19-218,
  src/casm/monte/events/OccCandidate.cc:9-212).
* ``Mol``, ``Atom``, ``OccTransform``, ``AtomLocation``, ``AtomTraj``, ``OccEvent``
  (include/casm/monte/events/OccEvent.hh:10-73).
* ``OccLocation`` (include/casm/monte/events/OccLocation.hh:44-385,
  src/casm/monte/events/OccLocation.cc:14-548): per variable site a Mol, per candidate
  the list of Mol ids, O(1) updates by swap-remove; atoms (optionally with unique ids and
  initial/final records) moving within the supercell and to or from a reservoir.
* the proposal functions of include/casm/monte/events/OccEventProposal.hh:74-484: a swap
  type is chosen with probability proportional to its number of possible events
  (``random_real(total)`` against the running sums), then the site(s) with
  ``random_int(cand_size - 1)``; both draws come from the caller's
  ``RandomNumberGenerator`` (std::mt19937_64 with libstdc++'s distributions), so a
  sequence of proposals is the reference's draw for draw.

The crystal structure comes from ``Prim`` (a lattice, fractional basis coordinates and
per-site occupant lists, with optional multi-atom occupants), standing in for
libcasm.xtal.Prim.  Unit cells of a supercell T are indexed i + n0 (j + n1 k) for a
diagonal T = diag(n0, n1, n2) (the ordering of the GPU sweeps); otherwise by the Smith
normal form S = U T V of T: (a0, a1, a2) = U (i, j, k) mod diag(S), index a0 + s0 (a1 +
s1 a2).  These are host data structures (set-up and per-event bookkeeping); the GPU
sweeps of ``casmcode_monte_gb300.clex`` do not need them.
"""
from __future__ import annotations

import copy
import itertools
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from .. import __version__  # noqa: F401  (the module version, as each bound module has)

__all__ = [
    "Atom", "AtomInfo", "AtomInfoMap", "AtomLocation", "AtomTraj", "AtomTrajVector", "AtomVector", "Conversions",
    "IntVector", "IntegralSiteCoordinate", "LongVector", "Mol", "MolVector", "OccSwapCountMap", "OccTransformVector",
    "MultiOccSwap", "OccCandidate", "OccCandidateList", "OccEvent", "OccLocation", "OccSwap", "OccTransform",
    "Occupant", "Prim", "choose_canonical_swap", "choose_semigrand_canonical_multiswap",
    "choose_semigrand_canonical_swap", "is_allowed_canonical_swap", "is_allowed_semigrand_canonical_swap",
    "make_canonical_swaps", "make_multiswaps", "make_semigrand_canonical_swaps", "propose_canonical_event",
    "propose_canonical_event_from_swap", "propose_semigrand_canonical_event",
    "propose_semigrand_canonical_event_from_multiswap", "propose_semigrand_canonical_event_from_swap",
    "propose_semigrand_canonical_multiswap_event", "swaps_allowed_per_unitcell",
]

_TOL = 1e-5


class _Vector(list):
    """The reference's bound ``std::vector`` types (python/src/monte_events.cpp): a list
    with the vector's ``push_back``."""

    def push_back(self, value) -> None:
        self.append(value)


class IntVector(_Vector):
    """std::vector<int>."""


class LongVector(_Vector):
    """std::vector<Index>."""


class AtomVector(_Vector):
    """std::vector<Atom>."""


class MolVector(_Vector):
    """std::vector<Mol>."""


class OccTransformVector(_Vector):
    """std::vector<OccTransform>."""


class AtomTrajVector(_Vector):
    """std::vector<AtomTraj>."""


class OccSwapCountMap(dict):
    """std::map<OccSwap, int>: swap counts of a multi-swap."""


class AtomInfoMap(dict):
    """std::map<std::string, std::vector<AtomInfo>>."""


# ---------------------------------------------------------------- structure


@dataclass
class Occupant:
    """An occupant (atom or molecule): name and atoms (name, Cartesian coordinate
    relative to the site)."""

    name: str
    atoms: list = field(default_factory=list)  # [(atom_name, np.array(3))]

    @staticmethod
    def atom(name: str) -> "Occupant":
        return Occupant(name, [(name, np.zeros(3))])

    def transformed(self, R: np.ndarray) -> list:
        return sorted((a, tuple(np.round(R @ np.asarray(x, dtype=float), 6))) for a, x in self.atoms)

    def key(self) -> list:
        return self.transformed(np.eye(3))


class Prim:
    """Primitive crystal structure: lattice column vectors, fractional basis coordinates
    [3, n_basis] and the allowed occupants of each basis site (``occ_dof``).  Occupant names
    not in ``occupants`` are single atoms of that name."""

    def __init__(self, lattice_column_vector_matrix, coordinate_frac, occ_dof: Sequence[Sequence[str]],
                 occupants: Optional[dict] = None):
        self.L = np.asarray(lattice_column_vector_matrix, dtype=float).reshape(3, 3)
        self.frac = np.asarray(coordinate_frac, dtype=float).reshape(3, -1)
        self.occ_dof = [list(x) for x in occ_dof]
        if len(self.occ_dof) != self.frac.shape[1]:
            raise ValueError("Error in Prim: occ_dof must have one list per basis site")
        occupants = dict(occupants or {})
        for names in self.occ_dof:
            for n in names:
                occupants.setdefault(n, Occupant.atom(n))
        self.occupants = occupants

    @property
    def n_basis(self) -> int:
        return self.frac.shape[1]

    @staticmethod
    def cubic(a: float = 1.0, occ_dof=("A", "B")) -> "Prim":
        return Prim(a * np.eye(3), np.zeros((3, 1)), [list(occ_dof)])

    @staticmethod
    def fcc(a: float = 4.0, occ_dof=("A", "B")) -> "Prim":
        """FCC primitive cell with columns (0, a/2, a/2), (a/2, 0, a/2), (a/2, a/2, 0)."""
        h = a / 2.0
        return Prim(np.array([[0, h, h], [h, 0, h], [h, h, 0]], dtype=float).T, np.zeros((3, 1)), [list(occ_dof)])


def _species_list(prim: Prim) -> tuple[list, list]:
    """Distinct occupants in order of first appearance over the basis sites' occupant
    lists (each orientation of a molecule is its own species): (names, Occupants)."""
    names, occs, keys = [], [], []
    for site in prim.occ_dof:
        for n in site:
            k = (prim.occupants[n].key(), n.split(".")[0])
            if k not in keys:
                keys.append(k)
                names.append(n)
                occs.append(prim.occupants[n])
    return names, occs


def _lattice_point_group(L: np.ndarray) -> list:
    """Integer matrices M (fractional coordinates, entries in {-1, 0, 1}) with
    M^T G M = G, G = L^T L."""
    G = L.T @ L
    scale = max(1.0, float(np.abs(G).max()))
    ops = []
    for e in itertools.product((-1, 0, 1), repeat=9):
        M = np.array(e, dtype=float).reshape(3, 3)
        if abs(abs(np.linalg.det(M)) - 1.0) > 1e-9:
            continue
        if np.abs(M.T @ G @ M - G).max() <= _TOL * scale:
            ops.append(M)
    return ops


def _factor_group_site_maps(prim: Prim) -> list:
    """Site permutations b -> b' of the prim's factor group (point operations with a
    translation mapping every basis site onto a basis site with the same occupants,
    molecules rotated by the operation)."""
    species_names, species = _species_list(prim)
    skey = [s.key() for s in species]
    site_species = [frozenset(species_names.index(n) for n in site) for site in prim.occ_dof]
    Linv = np.linalg.inv(prim.L)
    f = prim.frac
    nb = prim.n_basis
    maps = []
    for M in _lattice_point_group(prim.L):
        R = prim.L @ M @ Linv
        # species images under R
        img = []
        for s in species:
            k = s.transformed(R)
            img.append(skey.index(k) if k in skey else -1)
        for b1 in range(nb):
            tau = f[:, b1] - M @ f[:, 0]
            perm = []
            for b in range(nb):
                x = M @ f[:, b] + tau
                hit = -1
                for b2 in range(nb):
                    d = x - f[:, b2]
                    if np.abs(d - np.round(d)).max() < _TOL:
                        hit = b2
                        break
                if hit < 0:
                    break
                mapped = frozenset(img[s] for s in site_species[b])
                if -1 in mapped or mapped != site_species[hit]:
                    hit = -1
                    break
                perm.append(hit)
            if len(perm) == nb:
                maps.append(tuple(perm))
    return maps


def _b_to_asym(prim: Prim, species_names: list) -> list:
    """Conversions.cc:14-45: orbits of basis sites under the factor group (ordered as
    sorted sets), split by the order of their occupants (occupant index -> species)."""
    nb = prim.n_basis
    orbits = set()
    maps = _factor_group_site_maps(prim)
    for b in range(nb):
        orbits.add(tuple(sorted({m[b] for m in maps} | {b})))
    keyed: dict = {}
    for orbit_index, orbit in enumerate(sorted(orbits)):
        for b in orbit:
            occ_to_species = tuple(species_names.index(_canonical_name(prim, n, species_names))
                                   for n in prim.occ_dof[b])
            keyed.setdefault((orbit_index, occ_to_species), []).append(b)
    out = [0] * nb
    for asym, key in enumerate(sorted(keyed)):
        for b in keyed[key]:
            out[b] = asym
    return out


def _canonical_name(prim: Prim, n: str, species_names: list) -> str:
    """The species name (first-appearance representative) of occupant name n."""
    if n in species_names:
        return n
    k = (prim.occupants[n].key(), n.split(".")[0])
    for s in species_names:
        if (prim.occupants[s].key(), s.split(".")[0]) == k:
            return s
    raise KeyError(n)


def _smith(T: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Smith normal form of a 3x3 integer matrix: (U, s) with U unimodular and
    U T V = diag(s) for some unimodular V, s[0] | s[1] | s[2], s > 0."""
    A = np.array(T, dtype=np.int64)
    U = np.eye(3, dtype=np.int64)
    V = np.eye(3, dtype=np.int64)
    for t in range(3):
        while True:
            nz = [(abs(A[i, j]), i, j) for i in range(t, 3) for j in range(t, 3) if A[i, j] != 0]
            if not nz:
                break
            _, i, j = min(nz)
            A[[t, i]] = A[[i, t]]
            U[[t, i]] = U[[i, t]]
            A[:, [t, j]] = A[:, [j, t]]
            V[:, [t, j]] = V[:, [j, t]]
            done = True
            for i in range(t + 1, 3):
                q = A[i, t] // A[t, t]
                A[i] -= q * A[t]
                U[i] -= q * U[t]
                if A[i, t] != 0:
                    done = False
            for j in range(t + 1, 3):
                q = A[t, j] // A[t, t]
                A[:, j] -= q * A[:, t]
                V[:, j] -= q * V[:, t]
                if A[t, j] != 0:
                    done = False
            if done:
                bad = [(i, j) for i in range(t + 1, 3) for j in range(t + 1, 3) if A[i, j] % A[t, t] != 0]
                if not bad:
                    break
                i, _ = bad[0]
                A[t] += A[i]
                U[t] += U[i]
        if A[t, t] < 0:
            A[t] = -A[t]
            U[t] = -U[t]
    return U, np.array([A[0, 0], A[1, 1], A[2, 2]], dtype=np.int64)


class IntegralSiteCoordinate:
    """(b, i, j, k): basis site index and unit-cell translation."""

    def __init__(self, sublattice: int, unitcell):
        self._b = int(sublattice)
        self._ijk = np.asarray(unitcell, dtype=np.int64).reshape(3).copy()

    @staticmethod
    def from_list(x) -> "IntegralSiteCoordinate":
        return IntegralSiteCoordinate(x[0], x[1:4])

    def sublattice(self) -> int:
        return self._b

    def unitcell(self) -> np.ndarray:
        return self._ijk.copy()

    def to_list(self) -> list:
        return [self._b] + [int(v) for v in self._ijk]

    def __add__(self, translation) -> "IntegralSiteCoordinate":
        return IntegralSiteCoordinate(self._b, self._ijk + np.asarray(translation, dtype=np.int64))

    def __sub__(self, translation) -> "IntegralSiteCoordinate":
        return IntegralSiteCoordinate(self._b, self._ijk - np.asarray(translation, dtype=np.int64))

    def __eq__(self, other) -> bool:
        return isinstance(other, IntegralSiteCoordinate) and self.to_list() == other.to_list()

    def __hash__(self):
        return hash(tuple(self.to_list()))

    def __repr__(self):
        return f"IntegralSiteCoordinate({self.to_list()})"


def _as_bijk(x) -> IntegralSiteCoordinate:
    return x if isinstance(x, IntegralSiteCoordinate) else IntegralSiteCoordinate.from_list(list(x))


class UnitCellIndexConverter:
    """Unit cell (i, j, k) <-> linear unit cell index within a supercell (the unit cell
    part of the site index conversion)."""

    def __init__(self, transformation_matrix_to_super):
        self._c = UnitCellCoordIndexConverter(transformation_matrix_to_super, 1)

    def total_unitcells(self) -> int:
        return self._c.n_uc

    def linear_unitcell_index(self, unitcell) -> int:
        return self._c.unitcell_index(unitcell)

    def unitcell(self, unitcell_index: int) -> np.ndarray:
        return self._c.unitcell(unitcell_index)


class UnitCellCoordIndexConverter:
    """Linear site index <-> (b, i, j, k) within a supercell, b-major."""

    def __init__(self, T, n_basis: int):
        self.T = np.asarray(T, dtype=np.int64).reshape(3, 3)
        self.n_basis = int(n_basis)
        self.n_uc = int(round(abs(np.linalg.det(self.T))))
        if self.n_uc == 0:
            raise ValueError("Error in UnitCellCoordIndexConverter: singular transformation matrix")
        self.diagonal = bool(np.all(self.T == np.diag(np.diag(self.T)))) and np.all(np.diag(self.T) > 0)
        if self.diagonal:
            self._n = np.diag(self.T).copy()
            self._U = np.eye(3, dtype=np.int64)
        else:
            self._U, self._n = _smith(self.T)
        self._Uinv = np.round(np.linalg.inv(self._U)).astype(np.int64)
        self._Tinv = np.linalg.inv(self.T.astype(float))

    def total_sites(self) -> int:
        return self.n_basis * self.n_uc

    def unitcell_index(self, ijk) -> int:
        a = (self._U @ np.asarray(ijk, dtype=np.int64)) % self._n
        return int(a[0] + self._n[0] * (a[1] + self._n[1] * a[2]))

    def unitcell(self, index: int) -> np.ndarray:
        """The unit cell with this index, brought within the supercell (fractional
        supercell coordinates in [0, 1))."""
        i = int(index)
        a = np.array([i % self._n[0], (i // self._n[0]) % self._n[1], i // (self._n[0] * self._n[1])], dtype=np.int64)
        ijk = self._Uinv @ a
        sf = self._Tinv @ ijk
        return (ijk - self.T @ np.floor(sf + 1e-9).astype(np.int64)).astype(np.int64)

    def linear_site_index(self, bijk) -> int:
        bijk = _as_bijk(bijk)
        return bijk.sublattice() * self.n_uc + self.unitcell_index(bijk.unitcell())

    def __call__(self, x):
        if isinstance(x, (int, np.integer)):
            return self.bijk(int(x))
        return self.linear_site_index(x)

    def bijk(self, l: int) -> IntegralSiteCoordinate:
        if l < 0 or l >= self.total_sites():
            raise IndexError(f"Error in UnitCellCoordIndexConverter: linear site index {l} out of range")
        return IntegralSiteCoordinate(l // self.n_uc, self.unitcell(l % self.n_uc))


class Conversions:
    """Site index, asymmetric unit and occupant/species conversions for a supercell of
    ``xtal_prim`` (Conversions.hh:44-137)."""

    def __init__(self, xtal_prim: Prim, transformation_matrix_to_super, b_to_asym: Optional[Sequence[int]] = None):
        names, species = _species_list(xtal_prim)
        if b_to_asym is None:
            b_to_asym = _b_to_asym(xtal_prim, names)
        if len(b_to_asym) != xtal_prim.n_basis:
            raise ValueError("Error in Conversions: b_to_asym must have one entry per basis site")
        self._setup(xtal_prim, names, species, transformation_matrix_to_super, np.eye(3, dtype=np.int64), b_to_asym)

    @staticmethod
    def make_with_custom_asym(xtal_prim: Prim, transformation_matrix_to_super, b_to_asym) -> "Conversions":
        """An asymmetric unit of lower symmetry than the prim's factor group, one index per
        basis site (Conversions.cc:79-84)."""
        return Conversions(xtal_prim, transformation_matrix_to_super, b_to_asym)

    @staticmethod
    def make_with_custom_unitcell(xtal_prim: Prim, species_list: Sequence[Occupant], transformation_matrix_to_super,
                                  unit_transformation_matrix_to_super, unitl_to_asym) -> "Conversions":
        """An asymmetric unit that does not fit in the primitive cell: ``unitl_to_asym``
        gives the asymmetric unit index of every site of the sub-supercell U = P T_unit,
        which must tile the supercell (Conversions.cc:114-174).  ``species_list`` lists
        every distinct occupant (each orientation its own)."""
        T = np.asarray(transformation_matrix_to_super, dtype=np.int64).reshape(3, 3)
        Tu = np.asarray(unit_transformation_matrix_to_super, dtype=np.int64).reshape(3, 3)
        tiling = np.linalg.solve(Tu.astype(float), T.astype(float))
        if np.abs(tiling - np.round(tiling)).max() > 1e-9:
            raise ValueError("Error in Conversions: the unit supercell does not tile the supercell")
        n_unitl = int(round(abs(np.linalg.det(Tu)))) * xtal_prim.n_basis
        if len(unitl_to_asym) != n_unitl:
            raise ValueError("Error in Conversions: unitl_to_asym must have one entry per unit supercell site")
        c = Conversions.__new__(Conversions)
        c._setup(xtal_prim, [o.name for o in species_list], list(species_list), T, Tu, unitl_to_asym)
        return c

    def _setup(self, xtal_prim, names, species, T, T_unit, unitl_to_asym) -> None:
        self.prim = xtal_prim
        self._T = np.asarray(T, dtype=np.int64).reshape(3, 3)
        self._T_unit = np.asarray(T_unit, dtype=np.int64).reshape(3, 3)
        self._conv = UnitCellCoordIndexConverter(self._T, xtal_prim.n_basis)
        self._unit_conv = UnitCellCoordIndexConverter(self._T_unit, xtal_prim.n_basis)
        self._unit_is_prim = bool(np.array_equal(self._T_unit, np.eye(3, dtype=np.int64)))
        self._species_names, self._species = list(names), list(species)
        self._unitl_to_asym = [int(x) for x in unitl_to_asym]
        self._b_to_asym = self._unitl_to_asym if self._unit_is_prim else None
        self._n_asym = max(self._unitl_to_asym) + 1
        self._asym_to_unitl = [set() for _ in range(self._n_asym)]
        self._asym_to_b = [set() for _ in range(self._n_asym)]
        for unitl, a in enumerate(self._unitl_to_asym):
            self._asym_to_unitl[a].add(unitl)
            self._asym_to_b[a].add(self.unitl_to_b(unitl))
        skeys = [(o.key(), n.split(".")[0]) for n, o in zip(self._species_names, self._species)]
        ns = len(self._species_names)
        self._occ_to_species, self._species_to_occ = [], []
        for a in range(self._n_asym):
            b = min(self._asym_to_b[a])
            o2s = [skeys.index((xtal_prim.occupants[n].key(), n.split(".")[0])) for n in xtal_prim.occ_dof[b]]
            s2o = [len(o2s)] * ns
            for o, s in enumerate(o2s):
                s2o[s] = o
            self._occ_to_species.append(o2s)
            self._species_to_occ.append(s2o)

    # -- sites
    def lat_column_mat(self) -> np.ndarray:
        return self.prim.L.copy()

    def transformation_matrix_to_super(self) -> np.ndarray:
        return self._T.copy()

    def l_size(self) -> int:
        return self._conv.total_sites()

    def l_to_b(self, l: int) -> int:
        return int(l) // self._conv.n_uc

    def l_to_ijk(self, l: int) -> np.ndarray:
        return self._conv.bijk(int(l)).unitcell()

    def l_to_bijk(self, l: int) -> IntegralSiteCoordinate:
        return self._conv.bijk(int(l))

    def bijk_to_l(self, bijk) -> int:
        return self._conv.linear_site_index(bijk)

    def l_to_asym(self, l: int) -> int:
        if self._unit_is_prim:
            return self._b_to_asym[self.l_to_b(l)]
        return self._unitl_to_asym[self.l_to_unitl(l)]

    def bijk_to_asym(self, bijk) -> int:
        if self._unit_is_prim:
            return self._b_to_asym[_as_bijk(bijk).sublattice()]
        return self._unitl_to_asym[self.bijk_to_unitl(bijk)]

    def l_to_unitl(self, l: int) -> int:
        if self._unit_is_prim:
            return self.l_to_b(l)
        return self._unit_conv.linear_site_index(self.l_to_bijk(l))

    def bijk_to_unitl(self, bijk) -> int:
        """Site index within the (possibly non-primitive) unit cell."""
        return self._unit_conv.linear_site_index(bijk)

    def unitl_size(self) -> int:
        return self._unit_conv.total_sites()

    def unitl_to_b(self, unitl: int) -> int:
        return int(unitl) // self._unit_conv.n_uc

    def unitl_to_bijk(self, unitl: int) -> IntegralSiteCoordinate:
        """(b, i, j, k) of a unit-cell site (the reference's binding of this name returns
        unitl_to_b; this returns what its documentation states)."""
        return self._unit_conv.bijk(int(unitl))

    def unitl_to_asym(self, unitl: int) -> int:
        return self._unitl_to_asym[int(unitl)]

    def unit_transformation_matrix_to_super(self) -> np.ndarray:
        return self._T_unit.copy()

    def unitcell_index_converter(self) -> "UnitCellIndexConverter":
        return UnitCellIndexConverter(self._T)

    def l_to_frac(self, l: int) -> np.ndarray:
        bijk = self.l_to_bijk(l)
        return self.prim.frac[:, bijk.sublattice()] + bijk.unitcell()

    def l_to_cart(self, l: int) -> np.ndarray:
        return self.prim.L @ self.l_to_frac(l)

    def l_to_basis_frac(self, l: int) -> np.ndarray:
        return self.prim.frac[:, self.l_to_b(l)].copy()

    def l_to_basis_cart(self, l: int) -> np.ndarray:
        return self.prim.L @ self.l_to_basis_frac(l)

    def site_index_converter(self) -> UnitCellCoordIndexConverter:
        return self._conv

    def index_converter(self) -> UnitCellCoordIndexConverter:
        return self._conv

    def unit_site_index_converter(self) -> UnitCellCoordIndexConverter:
        return self._unit_conv

    # -- asymmetric unit
    def asym_size(self) -> int:
        return self._n_asym

    def asym_to_b(self, asym: int) -> set:
        return set(self._asym_to_b[asym])

    def asym_to_unitl(self, asym: int) -> set:
        return set(self._asym_to_unitl[asym])

    # -- occupants and species
    def occ_size(self, asym: int) -> int:
        return len(self._occ_to_species[asym])

    def species_index(self, asym_or_name, occ_index: Optional[int] = None) -> int:
        """species_index(asym, occ_index), or species_index(name) (-1... species_size if absent)."""
        if occ_index is None:
            name = asym_or_name
            return self._species_names.index(name) if name in self._species_names else len(self._species_names)
        return self._occ_to_species[asym_or_name][occ_index]

    def occ_index(self, asym: int, species_index: int) -> int:
        """Occupant index of the species on the asym site, occ_size(asym) if not allowed."""
        return self._species_to_occ[asym][species_index]

    def species_allowed(self, asym: int, species_index: int) -> bool:
        return self.occ_index(asym, species_index) != self.occ_size(asym)

    def species_size(self) -> int:
        return len(self._species_names)

    def species_name(self, species_index: int) -> str:
        return self._species_names[species_index]

    def species_list(self) -> list:
        return list(self._species)

    def species_to_mol(self, species_index: int) -> Occupant:
        return self._species[species_index]

    # -- names of the reference's Python binding (python/src/monte_events.cpp:360-433)
    def occ_to_species_index(self, asym: int, occ_index: int) -> int:
        return self.species_index(asym, occ_index)

    def species_to_occ_index(self, asym: int, species_index: int) -> int:
        return self.occ_index(asym, species_index)

    def species_name_to_index(self, species_name: str) -> int:
        return self.species_index(species_name)

    def species_index_to_occupant(self, species_index: int) -> Occupant:
        return self.species_to_mol(species_index)

    def species_index_to_name(self, species_index: int) -> str:
        return self.species_name(species_index)

    def species_index_to_atoms_size(self, species_index: int) -> int:
        """Number of atoms of the occupant (the reference's binding of this name returns the
        species name; this returns what its documentation states)."""
        return self.components_size(species_index)

    def components_size(self, species_index: int) -> int:
        return len(self._species[species_index].atoms)


# ---------------------------------------------------------------- candidates and swaps


@dataclass(frozen=True, order=True)
class OccCandidate:
    """(asymmetric unit index, species index), ordered lexicographically (OccCandidate.hh:19-43)."""

    asym: int
    species_index: int

    asymmetric_unit_index = property(lambda self: self.asym,
                                     lambda self, v: object.__setattr__(self, "asym", int(v)))

    def is_valid(self, convert: "Conversions") -> bool:
        """Indices in range and the species allowed on the asymmetric unit."""
        return _is_valid(convert, self)

    def __copy__(self) -> "OccCandidate":
        return OccCandidate(self.asym, self.species_index)

    def __deepcopy__(self, memo) -> "OccCandidate":
        return self.__copy__()

    def to_dict(self, convert: "Conversions") -> dict:
        """{"asym": a, "spec": species name} (OccCandidate_json_io.cc:40-46)."""
        return {"asym": int(self.asym), "spec": convert.species_name(self.species_index)}

    @staticmethod
    def from_dict(data: dict, convert: "Conversions") -> "OccCandidate":
        try:
            asym, name = int(data["asym"]), data["spec"]
        except (KeyError, TypeError, ValueError):
            raise RuntimeError("Error: Invalid monte::OccCandidate object")
        species_index = convert.species_index(name)
        if species_index == convert.species_size():
            raise RuntimeError(f"Error: Invalid monte::OccCandidate object: species name '{name}' is not a valid "
                               "option")
        return OccCandidate(asym, species_index)


@dataclass(frozen=True, order=True)
class OccSwap:
    """cand_a -> cand_b (OccCandidate.hh:55-93)."""

    cand_a: OccCandidate
    cand_b: OccCandidate

    first = property(lambda self: self.cand_a, lambda self, v: object.__setattr__(self, "cand_a", v))
    second = property(lambda self: self.cand_b, lambda self, v: object.__setattr__(self, "cand_b", v))

    def reversed(self) -> "OccSwap":
        return OccSwap(self.cand_b, self.cand_a)

    def sorted(self) -> "OccSwap":
        r = self.reversed()
        return r if r < self else self

    def reverse(self) -> None:
        """Exchange first and second in place (a swap used as a dict key is copied into
        the dict, so changing this object leaves the dict intact)."""
        a, b = self.cand_a, self.cand_b
        object.__setattr__(self, "cand_a", b)
        object.__setattr__(self, "cand_b", a)

    def sort(self) -> None:
        """Make (first, second) <= (second, first) in place."""
        if self.reversed() < self:
            self.reverse()

    def is_valid(self, convert: "Conversions") -> bool:
        return _is_valid(convert, self.cand_a) and _is_valid(convert, self.cand_b)

    def __copy__(self) -> "OccSwap":
        return OccSwap(copy.copy(self.cand_a), copy.copy(self.cand_b))

    def __deepcopy__(self, memo) -> "OccSwap":
        return self.__copy__()

    def to_dict(self, convert: "Conversions") -> list:
        """[first.to_dict(), second.to_dict()] (OccCandidate_json_io.cc:73-80)."""
        return [self.cand_a.to_dict(convert), self.cand_b.to_dict(convert)]

    @staticmethod
    def from_dict(data, convert: "Conversions") -> "OccSwap":
        if not isinstance(data, (list, tuple)) or len(data) != 2:
            raise RuntimeError("Error: Invalid monte::OccSwap object")
        return OccSwap(OccCandidate.from_dict(data[0], convert), OccCandidate.from_dict(data[1], convert))


class MultiOccSwap:
    """Several swaps with counts (OccCandidate.hh:99-147)."""

    def __init__(self, swaps: dict):
        if not swaps:
            raise ValueError("Error constructing MultiOccSwap: Empty multi-occ swap.")
        self.swaps = OccSwapCountMap(sorted((copy.copy(k), int(v)) for k, v in swaps.items()))
        self.total_count = sum(self.swaps.values())

    def _key(self):
        return tuple(self.swaps.items())

    def __lt__(self, other):
        return self._key() < other._key()

    def __eq__(self, other):
        return isinstance(other, MultiOccSwap) and self._key() == other._key()

    def __hash__(self):
        return hash(self._key())

    def reversed(self) -> "MultiOccSwap":
        return MultiOccSwap({s.reversed(): n for s, n in self.swaps.items()})

    def sorted(self) -> "MultiOccSwap":
        r = self.reversed()
        return r if r < self else self

    def reverse(self) -> None:
        """Reverse every swap in place."""
        self.swaps = self.reversed().swaps

    def sort(self) -> None:
        """Make self <= its reverse in place."""
        self.swaps = self.sorted().swaps

    def __copy__(self) -> "MultiOccSwap":
        return MultiOccSwap(self.swaps)

    def __deepcopy__(self, memo) -> "MultiOccSwap":
        return self.__copy__()

    def to_dict(self, convert: "Conversions") -> list:
        """[{"swap": swap.to_dict(), "count": n}, ...] (OccCandidate_json_io.cc:122-131)."""
        return [{"swap": s.to_dict(convert), "count": int(n)} for s, n in self.swaps.items()]

    @staticmethod
    def from_dict(data, convert: "Conversions") -> "MultiOccSwap":
        if not isinstance(data, (list, tuple)):
            raise RuntimeError("Error: Invalid monte::MultiOccSwap object: not an array")
        try:
            return MultiOccSwap({OccSwap.from_dict(x["swap"], convert): int(x["count"]) for x in data})
        except (KeyError, TypeError, ValueError):
            raise RuntimeError("Error: Invalid monte::MultiOccSwap object")


class OccCandidateList:
    """Candidates with lookup (asym, species) -> index (OccCandidate.cc:9-56); by default
    every (asym, species) of asymmetric units with more than one allowed occupant."""

    def __init__(self, convert: Conversions, candidates: Optional[Sequence[OccCandidate]] = None):
        if candidates is None:
            candidates = []
            for asym in range(convert.asym_size()):
                if convert.occ_size(asym) < 2:
                    continue
                for i in range(convert.occ_size(asym)):
                    candidates.append(OccCandidate(asym, convert.species_index(asym, i)))
        self._cand = list(candidates)
        self._end = len(self._cand)
        self._index = [[self._end] * convert.species_size() for _ in range(convert.asym_size())]
        for i, c in enumerate(self._cand):
            self._index[c.asym][c.species_index] = i

    def index(self, cand_or_asym, species_index: Optional[int] = None) -> int:
        if species_index is None:
            return self._index[cand_or_asym.asym][cand_or_asym.species_index]
        return self._index[cand_or_asym][species_index]

    def __getitem__(self, i: int) -> OccCandidate:
        return self._cand[i]

    def __iter__(self):
        return iter(self._cand)

    def __len__(self) -> int:
        return self._end

    def size(self) -> int:
        return self._end

    def matching_index(self, asymmetric_unit_index: int, species_index: int) -> int:
        """Index of the candidate (asym, species), len(self) if not in the list."""
        return self._index[asymmetric_unit_index][species_index]

    def to_dict(self, convert: "Conversions") -> dict:
        """The candidates and the canonical and semi-grand canonical swaps made from them
        (OccCandidate_json_io.cc:187-209)."""
        return {"candidate": [c.to_dict(convert) for c in self._cand],
                "canonical_swaps": [x.to_dict(convert) for x in make_canonical_swaps(convert, self)],
                "grand_canonical_swaps": [x.to_dict(convert) for x in make_semigrand_canonical_swaps(convert, self)]}

    @staticmethod
    def from_dict(data, convert: "Conversions") -> "OccCandidateList":
        """From a list of candidates or a dict with a "candidate" list
        (OccCandidate_json_io.cc:134-184)."""
        if isinstance(data, dict) and isinstance(data.get("candidate"), list):
            data = data["candidate"]
        if not isinstance(data, list):
            raise RuntimeError('Error: Invalid monte::OccCandidateList object: not an array or an object with a '
                               '"candidate" array.')
        return OccCandidateList(convert, [OccCandidate.from_dict(x, convert) for x in data])


def _is_valid(convert: Conversions, cand: OccCandidate) -> bool:
    return (0 <= cand.asym < convert.asym_size() and 0 <= cand.species_index < convert.species_size()
            and convert.species_allowed(cand.asym, cand.species_index))


def is_allowed_canonical_swap(convert: Conversions, cand_a: OccCandidate, cand_b: OccCandidate) -> bool:
    """OccCandidate.cc:79-87."""
    return (_is_valid(convert, cand_a) and _is_valid(convert, cand_b) and cand_a.species_index != cand_b.species_index
            and convert.species_allowed(cand_a.asym, cand_b.species_index)
            and convert.species_allowed(cand_b.asym, cand_a.species_index))


def is_allowed_semigrand_canonical_swap(convert: Conversions, cand_a: OccCandidate, cand_b: OccCandidate) -> bool:
    """OccCandidate.cc:115-122."""
    return (_is_valid(convert, cand_a) and _is_valid(convert, cand_b) and cand_a.asym == cand_b.asym
            and cand_a.species_index != cand_b.species_index
            and convert.species_allowed(cand_a.asym, cand_b.species_index))


def make_canonical_swaps(convert: Conversions, occ_candidate_list: OccCandidateList) -> list:
    """Pairs cand_a < cand_b that may exchange species (OccCandidate.cc:90-106)."""
    return [OccSwap(a, b) for a in occ_candidate_list for b in occ_candidate_list
            if a < b and is_allowed_canonical_swap(convert, a, b)]


def make_semigrand_canonical_swaps(convert: Conversions, occ_candidate_list: OccCandidateList) -> list:
    """All a -> b on one asymmetric unit, both directions (OccCandidate.cc:125-140)."""
    return [OccSwap(a, b) for a in occ_candidate_list for b in occ_candidate_list
            if is_allowed_semigrand_canonical_swap(convert, a, b)]


def swaps_allowed_per_unitcell(convert: Conversions, semigrand_canonical_swaps: Sequence[OccSwap]) -> int:
    """Number of events possible at once per unit cell (OccCandidate.cc:144-163)."""
    n_swaps = {a: 0 for a in range(convert.asym_size())}
    for s in semigrand_canonical_swaps:
        n_swaps[s.cand_a.asym] += 1
    return sum((n - 1) * len(convert.asym_to_b(a)) for a, n in sorted(n_swaps.items()) if n > 0)


def make_multiswaps(single_swaps: Sequence[OccSwap], max_total_count: int) -> list:
    """Distinct MultiOccSwap with 1..max_total_count single swaps (OccCandidate.cc:166-199)."""
    multis = {MultiOccSwap({s: 1}) for s in single_swaps}
    last = set(multis)
    for _ in range(1, max_total_count):
        nxt = set()
        for base in last:
            for s in single_swaps:
                sw = dict(base.swaps)
                sw[s] = sw.get(s, 0) + 1
                nxt.add(MultiOccSwap(sw))
        last = nxt
        multis |= nxt
    return sorted(multis)


# ---------------------------------------------------------------- events


@dataclass
class Atom:
    translation: np.ndarray = field(default_factory=lambda: np.zeros(3, dtype=np.int64))
    n_jumps: int = 0


@dataclass
class AtomInfo:
    atom: Atom
    species_index: int
    position_index: int
    time: float


@dataclass
class Mol:
    """A variable site's occupant (OccEvent.hh:22-32)."""

    id: int = 0
    l: int = 0
    asym: int = 0
    species_index: int = 0
    component: list = field(default_factory=list)
    loc: int = 0


Mol.component_id = property(lambda self: self.component, lambda self, v: setattr(self, "component", list(v)))
Mol.linear_site_index = property(lambda self: self.l, lambda self, v: setattr(self, "l", int(v)))
Mol.asymmetric_unit_index = property(lambda self: self.asym, lambda self, v: setattr(self, "asym", int(v)))
Mol.mol_location_index = property(lambda self: self.loc, lambda self, v: setattr(self, "loc", int(v)))


@dataclass
class OccTransform:
    l: int = 0
    mol_id: int = 0
    asym: int = 0
    from_species: int = 0
    to_species: int = 0


@dataclass
class AtomLocation:
    l: int = 0
    mol_id: int = 0
    mol_comp: int = 0


@dataclass
class AtomTraj:
    from_: AtomLocation = field(default_factory=AtomLocation)
    to: AtomLocation = field(default_factory=AtomLocation)
    delta_ijk: np.ndarray = field(default_factory=lambda: np.zeros(3, dtype=np.int64))


OccTransform.linear_site_index = property(lambda self: self.l, lambda self, v: setattr(self, "l", int(v)))
AtomLocation.linear_site_index = property(lambda self: self.l, lambda self, v: setattr(self, "l", int(v)))
# ``from`` is a Python keyword: reached as getattr(traj, "from"), as with the reference's binding
setattr(AtomTraj, "from", property(lambda self: self.from_, lambda self, v: setattr(self, "from_", v)))


@dataclass
class OccEvent:
    """Sites, new occupant indices, occupant transforms, atom trajectories (OccEvent.hh:55-71)."""

    linear_site_index: list = field(default_factory=list)
    new_occ: list = field(default_factory=list)
    occ_transform: list = field(default_factory=list)
    atom_traj: list = field(default_factory=list)

    def __copy__(self) -> "OccEvent":
        return copy.deepcopy(self)

    def __deepcopy__(self, memo) -> "OccEvent":
        return OccEvent(list(self.linear_site_index), list(self.new_occ),
                        [copy.copy(t) for t in self.occ_transform],
                        [AtomTraj(copy.copy(t.from_), copy.copy(t.to), np.array(t.delta_ijk)) for t in self.atom_traj])


class OccLocation:
    """Occupant locations by candidate type (OccLocation.hh:44-385): ``mol(i)`` per
    variable site, ``mol_id(cand, loc)`` lists per candidate, swap-remove updates."""

    def __init__(self, convert: Conversions, candidate_list: OccCandidateList, update_atoms: bool = False,
                 track_unique_atoms: bool = False, save_atom_info: bool = False):
        """OccLocation.cc:14-29: ``update_atoms`` tracks atom trajectories through
        ``apply``; ``track_unique_atoms`` gives every atom that enters the supercell a
        unique id (atoms may come from or go to a reservoir); ``save_atom_info`` keeps the
        initial and final position, species and time of atoms added and removed."""
        self._convert = convert
        self._cand_list = candidate_list
        self._loc = [[] for _ in range(len(candidate_list))]
        self._mol: list = []
        self._l_to_mol: list = []
        self._atoms: list = []
        self._update_atoms = bool(update_atoms)
        self._track_unique_atoms = bool(track_unique_atoms)
        self._save_atom_info = bool(save_atom_info)
        self._initial_atom_species_index: list = []
        self._initial_atom_position_index: list = []
        self._available_atom_id: set = set()
        self._next_unique_atom_id = 0
        self._unique_atom_id: list = []
        self._atom_info_initial: dict = {}
        self._atom_info_final: dict = {}

    def initialize(self, occupation, time: Optional[float] = None) -> None:
        """OccLocation.cc:37-108 (with ``save_atom_info`` and a time, the initial atom
        info of every atom is stored with that time)."""
        occupation = np.asarray(occupation)
        conv, cl = self._convert, self._cand_list
        self._mol, self._atoms = [], []
        self._initial_atom_species_index, self._initial_atom_position_index = [], []
        self._loc = [[] for _ in range(len(cl))]
        if self._update_atoms and self._track_unique_atoms:
            self._available_atom_id = set()
            self._next_unique_atom_id = 0
            self._unique_atom_id = []
            if self._save_atom_info:
                self._atom_info_initial, self._atom_info_final = {}, {}
        n = occupation.size
        variable = [conv.occ_size(conv.l_to_asym(l)) > 1 for l in range(n)]
        n_mut = sum(variable)
        self._l_to_mol = []
        for l in range(n):
            if not variable[l]:
                self._l_to_mol.append(n_mut)
                continue
            asym = conv.l_to_asym(l)
            sp = conv.species_index(asym, int(occupation[l]))
            ci = cl.index(asym, sp)
            mol = Mol(id=len(self._mol), l=l, asym=asym, species_index=sp, loc=len(self._loc[ci]))
            if self._update_atoms:
                for atom_index in range(conv.components_size(sp)):
                    mol.component.append(len(self._atoms))
                    atom = Atom(translation=conv.l_to_ijk(l), n_jumps=0)
                    self._atoms.append(atom)
                    if self._track_unique_atoms:
                        self._unique_atom_id.append(self._next_unique_atom_id)
                        if self._save_atom_info and time is not None:
                            self._atom_info_initial.setdefault(
                                self._next_unique_atom_id, AtomInfo(copy.deepcopy(atom), sp, atom_index, float(time)))
                        self._next_unique_atom_id += 1
                    self._initial_atom_species_index.append(sp)
                    self._initial_atom_position_index.append(atom_index)
            self._loc[ci].append(mol.id)
            self._l_to_mol.append(mol.id)
            self._mol.append(mol)

    def apply(self, e: OccEvent, occupation: np.ndarray, time: Optional[float] = None) -> None:
        """Update the occupation vector (in place), the lists and the atoms for event e
        (OccLocation.cc:212-366).  An atom trajectory from or to position l == -1 is a move
        from or to the reservoir (whose mol_id is the species index); with
        ``track_unique_atoms`` an atom leaving frees its atom id (the smallest free id is
        reused first) and an entering atom gets the next unique id, its species index taken
        from ``to.mol_id`` as the reference does; with ``save_atom_info`` and a time the
        final (leaving) and initial (entering) atom info is stored."""
        conv, cl = self._convert, self._cand_list
        moving = []
        if self._update_atoms:
            for t in e.atom_traj:
                if t.from_.l == -1:
                    moving.append(-1)  # from the reservoir: a new atom
                    continue
                mol = self._mol[t.from_.mol_id]
                atom_id = mol.component[t.from_.mol_comp]
                if self._track_unique_atoms and t.to.l == -1 and self._save_atom_info and time is not None:
                    self._atom_info_final.setdefault(
                        self._unique_atom_id[atom_id],
                        AtomInfo(copy.deepcopy(self._atoms[atom_id]), mol.species_index, t.from_.mol_comp,
                                 float(time)))
                moving.append(atom_id)
        for t in e.occ_transform:
            mol = self._mol[t.mol_id]
            if mol.species_index != t.from_species:
                raise RuntimeError("Error in OccLocation::apply: species mismatch")
            occupation[mol.l] = conv.occ_index(mol.asym, t.to_species)
            ci = cl.index(mol.asym, mol.species_index)
            back = self._loc[ci][-1]
            self._loc[ci][mol.loc] = back
            self._mol[back].loc = mol.loc
            self._loc[ci].pop()
            mol.species_index = t.to_species
            if self._update_atoms:
                size = conv.components_size(mol.species_index)
                mol.component = (mol.component + [0] * size)[:size]
            ci = cl.index(mol.asym, mol.species_index)
            mol.loc = len(self._loc[ci])
            self._loc[ci].append(mol.id)
        if not self._update_atoms:
            return
        if self._track_unique_atoms:
            lmin = np.iinfo(np.int64).min
            for atom_id, t in zip(moving, e.atom_traj):
                if t.to.l == -1 and t.from_.l != -1:  # to the reservoir
                    self._atoms[atom_id].translation = np.array([lmin, lmin, lmin], dtype=np.int64)
                    self._atoms[atom_id].n_jumps = lmin
                    self._unique_atom_id[atom_id] = -1
                    self._initial_atom_species_index[atom_id] = -1
                    self._initial_atom_position_index[atom_id] = -1
                    self._available_atom_id.add(atom_id)
            for t in e.atom_traj:
                if t.to.l != -1 and t.from_.l == -1:  # from the reservoir
                    atom = Atom(translation=conv.l_to_ijk(t.to.l), n_jumps=0)
                    species_index, position_index = t.to.mol_id, t.to.mol_comp
                    if self._available_atom_id:
                        atom_id = min(self._available_atom_id)
                        self._available_atom_id.remove(atom_id)
                        self._atoms[atom_id] = atom
                        self._unique_atom_id[atom_id] = self._next_unique_atom_id
                        self._initial_atom_species_index[atom_id] = species_index
                        self._initial_atom_position_index[atom_id] = position_index
                    else:
                        atom_id = len(self._atoms)
                        self._atoms.append(atom)
                        self._unique_atom_id.append(self._next_unique_atom_id)
                        self._initial_atom_species_index.append(species_index)
                        self._initial_atom_position_index.append(position_index)
                    if self._save_atom_info and time is not None:
                        self._atom_info_initial.setdefault(
                            self._next_unique_atom_id,
                            AtomInfo(copy.deepcopy(atom), species_index, position_index, float(time)))
                    self._mol[t.to.mol_id].component[t.to.mol_comp] = atom_id
                    self._next_unique_atom_id += 1
        for atom_id, t in zip(moving, e.atom_traj):
            if t.to.l != -1 and t.from_.l != -1:  # within the supercell
                self._mol[t.to.mol_id].component[t.to.mol_comp] = atom_id
                self._atoms[atom_id].translation = self._atoms[atom_id].translation + np.asarray(t.delta_ijk)
                self._atoms[atom_id].n_jumps += 1

    def choose_mol(self, cand, random_number_generator, exclude: Optional[set] = None) -> Mol:
        """Uniform Mol of a candidate: random_int(cand_size - 1), redrawn while in
        ``exclude`` (OccLocation.hh:232-263)."""
        ci = cand if isinstance(cand, (int, np.integer)) else self._cand_list.index(cand)
        locs = self._loc[ci]
        while True:
            loc = random_number_generator.random_int(len(locs) - 1)
            if not exclude or loc not in exclude:
                return self._mol[locs[loc]]

    def mol_size(self) -> int:
        return len(self._mol)

    def mol(self, mol_id: int) -> Mol:
        return self._mol[mol_id]

    def atom_size(self) -> int:
        return len(self._atoms)

    def initial_atom_species_index(self) -> list:
        """Initial species index of each atom (-1 for an atom id freed by a move to the
        reservoir)."""
        return self._initial_atom_species_index

    def initial_atom_position_index(self) -> list:
        return self._initial_atom_position_index

    def current_atom_names(self) -> list:
        """Current atom name of each atom ("UK" when it is no longer in the supercell)."""
        names = ["UK"] * len(self._atoms)
        for mol in self._mol:
            molecule = self._convert.species_to_mol(mol.species_index)
            for k, atom_id in enumerate(mol.component):
                names[atom_id] = molecule.atoms[k][0]
        return names

    def current_atom_species_index(self) -> list:
        out = [-1] * len(self._atoms)
        for mol in self._mol:
            for atom_id in mol.component:
                out[atom_id] = mol.species_index
        return out

    def current_atom_position_index(self) -> list:
        out = [-1] * len(self._atoms)
        for mol in self._mol:
            for k, atom_id in enumerate(mol.component):
                out[atom_id] = k
        return out

    def current_atom_n_jumps(self) -> list:
        return [a.n_jumps for a in self._atoms]

    def unique_atom_id(self) -> list:
        return self._unique_atom_id

    def atom_info_initial(self) -> dict:
        """unique atom id -> AtomInfo when the atom entered the supercell (save_atom_info)."""
        return self._atom_info_initial

    def atom_info_final(self) -> dict:
        """unique atom id -> AtomInfo when the atom left the supercell (save_atom_info)."""
        return self._atom_info_final

    def clear_atom_info_final(self) -> None:
        self._atom_info_final = {}

    def replace_mol(self, l: int, occ: int, atom_id, atom) -> None:
        """Put occupant ``occ`` on site l with the given atom ids and atoms, for restoring a
        saved state (OccLocation.cc:506-548); not with unique atom tracking."""
        if self._track_unique_atoms:
            raise RuntimeError("Error in OccLocation::replace_mol: `replace_mol` is not supported when tracking "
                               "unique atoms")
        conv, cl = self._convert, self._cand_list
        mol = self._mol[self.l_to_mol_id(l)]
        ci = cl.index(mol.asym, mol.species_index)
        back = self._loc[ci][-1]
        self._loc[ci][mol.loc] = back
        self._mol[back].loc = mol.loc
        self._loc[ci].pop()
        mol.species_index = conv.species_index(mol.asym, int(occ))
        ci = cl.index(mol.asym, mol.species_index)
        mol.loc = len(self._loc[ci])
        self._loc[ci].append(mol.id)
        mol.component = []
        for aid, a in zip(atom_id, atom):
            mol.component.append(int(aid))
            self._atoms[int(aid)] = a

    def atom_positions_cart(self) -> np.ndarray:
        """Current atom positions, shape (3, n_atoms), following atoms across periodic
        boundaries: site basis position + the atom's position in its molecule + lattice
        translation of the atom (OccLocation.cc:385-405).  Needs ``update_atoms``."""
        conv = self._convert
        L = conv.lat_column_mat()
        R = np.zeros((3, len(self._atoms)))
        for mol in self._mol:
            basis = conv.l_to_basis_cart(mol.l)
            molecule = conv.species_to_mol(mol.species_index)
            for k, atom_id in enumerate(mol.component):
                R[:, atom_id] = basis + np.asarray(molecule.atoms[k][1], dtype=float) + \
                    L @ np.asarray(self._atoms[atom_id].translation, dtype=float)
        return R

    def atom_positions_cart_within(self) -> np.ndarray:
        """Current atom positions, shape (3, n_atoms), within the periodic supercell: site
        position + the atom's position in its molecule (OccLocation.cc:412-429)."""
        conv = self._convert
        R = np.zeros((3, len(self._atoms)))
        for mol in self._mol:
            site = conv.l_to_cart(mol.l)
            molecule = conv.species_to_mol(mol.species_index)
            for k, atom_id in enumerate(mol.component):
                R[:, atom_id] = site + np.asarray(molecule.atoms[k][1], dtype=float)
        return R

    def atom(self, atom_id: int) -> Atom:
        return self._atoms[atom_id]

    def candidate_list(self) -> OccCandidateList:
        return self._cand_list

    def cand_size(self, cand) -> int:
        ci = cand if isinstance(cand, (int, np.integer)) else self._cand_list.index(cand)
        return len(self._loc[ci])

    def mol_id(self, cand, loc: int) -> int:
        ci = cand if isinstance(cand, (int, np.integer)) else self._cand_list.index(cand)
        return self._loc[ci][loc]

    def cand_size_by_candidate_index(self, candidate_index: int) -> int:
        return len(self._loc[candidate_index])

    def mol_id_by_candidate_index(self, candidate_index: int, location_index: int) -> int:
        return self._loc[candidate_index][location_index]

    def choose_mol_by_candidate_index(self, candidate_index: int, random_number_generator) -> Mol:
        return self.choose_mol(int(candidate_index), random_number_generator)

    def linear_site_index_to_mol_id(self, linear_site_index: int) -> int:
        return self.l_to_mol_id(linear_site_index)

    def l_to_mol_id(self, l: int) -> int:
        return self._l_to_mol[l]

    def convert(self) -> Conversions:
        return self._convert


# ---------------------------------------------------------------- proposals


def _choose(weights: list, random_number_generator, what: str):
    tsum = [0.0]
    for w in weights:
        tsum.append(tsum[-1] + float(w))
    if tsum[-1] == 0.0:
        raise RuntimeError(f"Error in {what}: No events possible.")
    r = random_number_generator.random_real(tsum[-1])
    for i in range(len(weights)):
        if r < tsum[i + 1]:
            return i
    raise RuntimeError(f"Error in {what}")


def choose_canonical_swap(occ_location: OccLocation, canonical_swaps: Sequence[OccSwap], random_number_generator):
    """Swap type with probability cand_size(a) * cand_size(b) / total (OccEventProposal.hh:74-115)."""
    w = [float(occ_location.cand_size(s.cand_a)) * float(occ_location.cand_size(s.cand_b)) for s in canonical_swaps]
    return canonical_swaps[_choose(w, random_number_generator, "choose_canonical_swap")]


def propose_canonical_event_from_swap(e: OccEvent, occ_location: OccLocation, swap: OccSwap,
                                      random_number_generator) -> OccEvent:
    """OccEventProposal.hh:117-155."""
    conv = occ_location.convert()
    e.occ_transform, e.atom_traj = [], []
    for ca, cb in ((swap.cand_a, swap.cand_b), (swap.cand_b, swap.cand_a)):
        mol = occ_location.choose_mol(ca, random_number_generator)
        e.occ_transform.append(OccTransform(l=mol.l, mol_id=mol.id, asym=ca.asym, from_species=ca.species_index,
                                            to_species=cb.species_index))
    e.linear_site_index = [t.l for t in e.occ_transform]
    e.new_occ = [conv.occ_index(t.asym, t.to_species) for t in e.occ_transform]
    return e


def propose_canonical_event(e: OccEvent, occ_location: OccLocation, canonical_swaps: Sequence[OccSwap],
                            random_number_generator) -> OccEvent:
    swap = choose_canonical_swap(occ_location, canonical_swaps, random_number_generator)
    return propose_canonical_event_from_swap(e, occ_location, swap, random_number_generator)


def choose_semigrand_canonical_swap(occ_location: OccLocation, semigrand_canonical_swaps: Sequence[OccSwap],
                                    random_number_generator):
    """Swap type with probability cand_size(a) / total (OccEventProposal.hh:168-208)."""
    w = [float(occ_location.cand_size(s.cand_a)) for s in semigrand_canonical_swaps]
    return semigrand_canonical_swaps[_choose(w, random_number_generator, "choose_semigrand_canonical_swap")]


def propose_semigrand_canonical_event_from_swap(e: OccEvent, occ_location: OccLocation, swap: OccSwap,
                                                random_number_generator) -> OccEvent:
    """OccEventProposal.hh:210-235."""
    mol = occ_location.choose_mol(swap.cand_a, random_number_generator)
    t = OccTransform(l=mol.l, mol_id=mol.id, asym=swap.cand_a.asym, from_species=swap.cand_a.species_index,
                     to_species=swap.cand_b.species_index)
    e.occ_transform, e.atom_traj = [t], []
    e.linear_site_index = [t.l]
    e.new_occ = [occ_location.convert().occ_index(t.asym, t.to_species)]
    return e


def propose_semigrand_canonical_event(e: OccEvent, occ_location: OccLocation,
                                      semigrand_canonical_swaps: Sequence[OccSwap],
                                      random_number_generator) -> OccEvent:
    """OccEventProposal.hh:237-247."""
    swap = choose_semigrand_canonical_swap(occ_location, semigrand_canonical_swaps, random_number_generator)
    return propose_semigrand_canonical_event_from_swap(e, occ_location, swap, random_number_generator)


def choose_semigrand_canonical_multiswap(occ_location: OccLocation, multiswaps: Sequence[MultiOccSwap],
                                         random_number_generator):
    """Multiswap with probability prod over swaps of falling factorials of cand_size
    (OccEventProposal.hh:250-306)."""
    w = []
    for m in multiswaps:
        p = 1.0
        for s, n in m.swaps.items():
            for j in range(n):
                p *= float(occ_location.cand_size(s.cand_a) - j)
        w.append(p)
    return multiswaps[_choose(w, random_number_generator, "choose_semigrand_canonical_multiswap")]


def propose_semigrand_canonical_event_from_multiswap(e: OccEvent, occ_location: OccLocation, multiswap: MultiOccSwap,
                                                     random_number_generator) -> OccEvent:
    """Distinct sites per candidate, drawn with exclusion of locations already chosen
    (OccEventProposal.hh:308-343; the exclusion set holds list positions)."""
    conv = occ_location.convert()
    e.occ_transform, e.atom_traj = [], []
    exclude: set = set()
    for swap, n in multiswap.swaps.items():
        for _ in range(n):
            mol = occ_location.choose_mol(swap.cand_a, random_number_generator, exclude)
            exclude.add(mol.loc)
            e.occ_transform.append(OccTransform(l=mol.l, mol_id=mol.id, asym=swap.cand_a.asym,
                                                from_species=swap.cand_a.species_index,
                                                to_species=swap.cand_b.species_index))
    e.linear_site_index = [t.l for t in e.occ_transform]
    e.new_occ = [conv.occ_index(t.asym, t.to_species) for t in e.occ_transform]
    return e


def propose_semigrand_canonical_multiswap_event(e: OccEvent, occ_location: OccLocation,
                                                multiswaps: Sequence[MultiOccSwap],
                                                random_number_generator) -> OccEvent:
    m = choose_semigrand_canonical_multiswap(occ_location, multiswaps, random_number_generator)
    return propose_semigrand_canonical_event_from_multiswap(e, occ_location, m, random_number_generator)
