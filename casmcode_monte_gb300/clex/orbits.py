"""Cluster orbits and symmetrised cluster functions of the FCC lattice.

The reference toolkit does not ship a cluster-expansion evaluator: real CASM runs plug
one in through the ``formation_energy_f_type`` slot of a system
(``ising_cpp/basic_semigrand_canonical.hh:104-111``) and the functions are generated by
the external libcasm-clexulator (the only in-tree pattern is the generated fixture
``tests/unit/monte/data/OccClexulatorZrOTest/.../ZrO_Clexulator.cc:4478-4501``, whose
``_calc_delta_point_corr`` evaluates a change of correlations as
``(phi(new) - phi(old)) * sum over clusters of products of the other sites' phi``).

This module enumerates, from the crystal geometry alone, everything a GPU sweep needs:

* the FCC point group (the 48 signed permutation matrices in Cartesian coordinates);
* cluster orbits (empty, point, pairs 1-4NN, the three smallest triplets, the NN
  tetrahedron) and, for multi-function site bases, the orbits of *decorated* clusters
  (cluster + basis-function index on each site), which are the symmetrised cluster
  functions;
* for a site ``l`` that changes occupant, the local "feature" sums
  ``F[k] = sum over decorated clusters of class f containing l, with basis index b at l,
  of prod_{j != l} psi_{b_j}(occ_j)``;
* for the full-energy reduction, the decorated clusters anchored at a site (each cluster
  counted once, at its lexicographically smallest member).

Conventions (fixed here because no in-tree reference pins them):

* Lattice: FCC primitive vectors (0,2,2), (2,0,2), (2,2,0) as columns (conventional
  a = 4, as ``tests/unit/teststructures.hh:68-88``).  Cartesian coordinates of sites are
  integers; primitive coordinates are obtained with the inverse lattice matrix.
* Site basis functions are ``phi_b(o) = a_b * psi_b(o)`` with integer ``psi``:
  - binary "occupation" basis: ``psi_1 = (0, 1)`` (A, B), ``a_1 = 1``;
  - ternary Chebyshev basis (orthonormal under the uniform measure on 3 occupants):
    ``psi_1 = (-1, 0, 1)``, ``a_1 = sqrt(3/2)``; ``psi_2 = (1, -2, 1)``, ``a_2 = 1/sqrt(2)``.
* Class order: number of sites, then the ascending tuple of squared pair distances,
  then the canonical decorated form.  Multiplicity ``M_f`` = decorated clusters of the
  class per primitive cell.  Energy per supercell
  ``E = sum_f (V_f / M_f) * C_f * sum_{(c,d) in f} prod psi`` with ``C_f = prod a_{d_i}``.
"""
from __future__ import annotations

import itertools
import math
from dataclasses import dataclass, field

import numpy as np

#: primitive lattice vectors (columns), Cartesian, conventional cubic a = 4
FCC_LATTICE = np.array([[0, 2, 2], [2, 0, 2], [2, 2, 0]], dtype=np.int64).T
_FCC_LATTICE_INV = np.linalg.inv(FCC_LATTICE.astype(float))

#: squared lengths of the 1st..4th neighbour shells (Cartesian, a = 4)
FCC_SHELL_D2 = (8, 16, 24, 32)


def cart_to_prim(v) -> tuple[int, int, int]:
    n = _FCC_LATTICE_INV @ np.asarray(v, dtype=float)
    r = np.rint(n).astype(np.int64)
    assert np.allclose(n, r), v
    return tuple(int(x) for x in r)


def point_group_cubic() -> list[np.ndarray]:
    """The 48 operations of m-3m as signed 3x3 permutation matrices."""
    ops = []
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product((1, -1), repeat=3):
            m = np.zeros((3, 3), dtype=np.int64)
            for r, c in enumerate(perm):
                m[r, c] = signs[r]
            ops.append(m)
    return ops


_OPS = point_group_cubic()


def _is_site(v) -> bool:
    x, y, z = (int(t) for t in v)
    return x % 2 == 0 and y % 2 == 0 and z % 2 == 0 and ((x + y + z) // 2) % 2 == 0


def neighbour_shells(n_shells: int = 4) -> list[list[tuple[int, int, int]]]:
    """Cartesian vectors of the first ``n_shells`` neighbour shells (sorted)."""
    d2max = FCC_SHELL_D2[n_shells - 1]
    R = int(math.isqrt(d2max)) + 2
    pts = []
    for v in itertools.product(range(-R, R + 1), repeat=3):
        if v == (0, 0, 0) or not _is_site(v):
            continue
        d2 = v[0] ** 2 + v[1] ** 2 + v[2] ** 2
        if d2 <= d2max:
            pts.append((d2, v))
    shells = []
    for d2 in FCC_SHELL_D2[:n_shells]:
        shells.append(sorted(v for (dd, v) in pts if dd == d2))
    return shells


def _d2(a, b) -> int:
    return int(sum((int(x) - int(y)) ** 2 for x, y in zip(a, b)))


def _canon(sites, decor=None):
    """Canonical form of a (decorated) cluster under the FCC space group."""
    best = None
    arr = np.array(sites, dtype=np.int64)
    for g in _OPS:
        t = arr @ g.T
        rows = [tuple(int(x) for x in r) for r in t]
        if decor is None:
            items = sorted(rows)
            o = items[0]
            key = tuple(tuple(x - y for x, y in zip(r, o)) for r in items)
        else:
            items = sorted(zip(rows, decor))
            o = items[0][0]
            key = tuple((tuple(x - y for x, y in zip(r, o)), b) for r, b in items)
        if best is None or key < best:
            best = key
    return best


def _sorted_d2(sites) -> tuple[int, ...]:
    return tuple(sorted(_d2(a, b) for a, b in itertools.combinations(sites, 2)))


@dataclass
class ClusterOrbit:
    """A cluster orbit: prototype (canonical) and all clusters containing the origin."""

    size: int
    d2: tuple  # ascending squared pair distances
    canon: tuple
    clusters_at_origin: list = field(default_factory=list)  # tuples of Cartesian sites

    @property
    def multiplicity(self) -> int:
        """Clusters per primitive cell."""
        if self.size == 0:
            return 1
        assert len(self.clusters_at_origin) % self.size == 0
        return len(self.clusters_at_origin) // self.size


def fcc_cluster_orbits(n_pair_shells: int = 4, n_triplets: int = 3, n_quads: int = 1):
    """Orbits: empty, point, pairs (1..n_pair_shells NN), smallest triplets, smallest quads.

    Triplets and quadruplets are drawn from sites within the pair cutoff; "smallest" is
    ordered by the ascending tuple of squared pair distances, then canonical form.
    """
    shells = neighbour_shells(n_pair_shells)
    nbrs = [v for s in shells for v in s]
    d2max = FCC_SHELL_D2[n_pair_shells - 1]
    origin = (0, 0, 0)
    orbits: list[ClusterOrbit] = []
    orbits.append(ClusterOrbit(0, (), (), [()]))
    orbits.append(ClusterOrbit(1, (), _canon([origin]), [(origin,)]))
    for s in shells:
        cl = [(origin, v) for v in s]
        orbits.append(ClusterOrbit(2, _sorted_d2(cl[0]), _canon(cl[0]), cl))

    def multi(k, n_keep):
        groups: dict = {}
        for combo in itertools.combinations(nbrs, k - 1):
            sites = (origin,) + combo
            if any(_d2(a, b) > d2max for a, b in itertools.combinations(sites, 2)):
                continue
            key = _canon(sites)
            groups.setdefault(key, []).append(sites)
        keyed = sorted(groups.items(), key=lambda kv: (_sorted_d2(kv[1][0]), kv[0]))
        out = []
        for key, cls in keyed[:n_keep]:
            out.append(ClusterOrbit(k, _sorted_d2(cls[0]), key, cls))
        return out

    if n_triplets:
        orbits += multi(3, n_triplets)
    if n_quads:
        orbits += multi(4, n_quads)
    return orbits


@dataclass
class SiteBasis:
    """Integer-valued site functions ``psi[b][o]`` and scale factors ``a[b]``."""

    name: str
    n_species: int
    psi: list  # psi[b][o], b = 0 .. n_functions-1 (index b+1 in the docs)
    scale: list  # a[b]

    @property
    def n_functions(self) -> int:
        return len(self.psi)


OCCUPATION_BINARY = SiteBasis("occupation", 2, [[0, 1]], [1.0])
CHEBYSHEV_TERNARY = SiteBasis(
    "chebyshev", 3, [[-1, 0, 1], [1, -2, 1]], [math.sqrt(1.5), 1.0 / math.sqrt(2.0)]
)


@dataclass
class FunctionClass:
    """A symmetrised cluster function: an orbit of decorated clusters."""

    orbit_index: int
    size: int
    d2: tuple
    canon: tuple
    # decorated clusters containing the origin: list of (sites, decoration)
    members_at_origin: list = field(default_factory=list)

    @property
    def multiplicity(self) -> int:
        if self.size == 0:
            return 1
        return len(self.members_at_origin) // self.size

    def decoration_multiset(self) -> tuple:
        if self.size == 0:
            return ()
        return tuple(sorted(self.members_at_origin[0][1]))


def function_classes(orbits, basis: SiteBasis) -> list[FunctionClass]:
    """Split each cluster orbit into decorated-cluster orbits (symmetrised functions)."""
    nb = basis.n_functions
    out: list[FunctionClass] = []
    for oi, orb in enumerate(orbits):
        if orb.size == 0:
            out.append(FunctionClass(oi, 0, (), (), [((), ())]))
            continue
        groups: dict = {}
        for sites in orb.clusters_at_origin:
            for decor in itertools.product(range(nb), repeat=orb.size):
                key = _canon(sites, decor)
                groups.setdefault(key, []).append((sites, decor))
        for key in sorted(groups):
            out.append(FunctionClass(oi, orb.size, orb.d2, key, groups[key]))
    return out


@dataclass
class Feature:
    """Local sum F[k] for one (class, basis index at the changing site)."""

    class_index: int
    b_site: int
    # terms: list of tuples of (prim offset (3,), basis index) for the other sites
    terms: list


def local_features(classes: list[FunctionClass]) -> list[Feature]:
    feats: list[Feature] = []
    for ci, fc in enumerate(classes):
        if fc.size == 0:
            continue
        by_b: dict = {}
        for sites, decor in fc.members_at_origin:
            idx = sites.index((0, 0, 0))
            b_l = decor[idx]
            others = []
            for s, b in zip(sites, decor):
                if s == (0, 0, 0):
                    continue
                others.append((cart_to_prim(s), b))
            others.sort()
            by_b.setdefault(b_l, []).append(tuple(others))
        for b_l in sorted(by_b):
            feats.append(Feature(ci, b_l, sorted(by_b[b_l])))
    return feats


def anchored_terms(classes: list[FunctionClass]) -> list[list[tuple]]:
    """Per class: decorated clusters whose lexicographically smallest site is the origin.

    Each entry is a tuple of (prim offset, basis index) over all sites of the cluster.
    Summing these products over all sites of a supercell counts every decorated cluster
    exactly once.
    """
    out = []
    for fc in classes:
        if fc.size == 0:
            out.append([()])
            continue
        seen = set()
        lst = []
        for sites, decor in fc.members_at_origin:
            m = min(sites)
            shifted = tuple(
                (tuple(a - b for a, b in zip(s, m)), d) for s, d in sorted(zip(sites, decor))
            )
            if shifted in seen:
                continue
            seen.add(shifted)
            lst.append(tuple(sorted((cart_to_prim(s), d) for s, d in shifted)))
        assert len(lst) == fc.multiplicity, (len(lst), fc.multiplicity)
        out.append(sorted(lst))
    return out


@dataclass
class ClexBasisSet:
    """Everything the sweep kernels and host code need for one basis set."""

    name: str
    basis: SiteBasis
    orbits: list
    classes: list
    features: list
    anchored: list

    @property
    def n_classes(self) -> int:
        return len(self.classes)

    @property
    def n_features(self) -> int:
        return len(self.features)

    def neighbour_offsets(self) -> list[tuple[int, int, int]]:
        offs = set()
        for f in self.features:
            for t in f.terms:
                for o, _ in t:
                    offs.add(o)
        return sorted(offs)

    def class_scale(self, ci: int) -> float:
        """C_f = product of a_b over a decoration (multiplied in ascending-b order)."""
        c = 1.0
        for b in self.classes[ci].decoration_multiset():
            c = c * self.basis.scale[b]
        return c

    def max_abs_feature(self, k: int) -> int:
        """Upper bound on |F_k| given |psi| bounds."""
        pmax = [max(abs(x) for x in row) for row in self.basis.psi]
        tot = 0
        for t in self.features[k].terms:
            p = 1
            for _, b in t:
                p *= pmax[b]
            tot += p
        return tot


def make_basis_set(kind: str) -> ClexBasisSet:
    """``kind`` is ``"fcc_binary"`` (occupation basis) or ``"fcc_ternary"`` (Chebyshev)."""
    if kind == "fcc_binary":
        basis = OCCUPATION_BINARY
    elif kind == "fcc_ternary":
        basis = CHEBYSHEV_TERNARY
    else:
        raise ValueError(f"Error in make_basis_set: unknown basis set '{kind}'")
    orbits = fcc_cluster_orbits()
    classes = function_classes(orbits, basis)
    feats = local_features(classes)
    anch = anchored_terms(classes)
    return ClexBasisSet(kind, basis, orbits, classes, feats, anch)
