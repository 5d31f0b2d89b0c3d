"""Events and methods modules on the CPU.

* Conversions: the reference's own cases (python/tests/events/test_Conversions.py:8-72):
  site counts, the b-major linear index, translations, the asymmetric unit with
  molecule orientations and occupant order.
* OccLocation: the invariants the reference checks after every proposal and application
  (tests/unit/monte/OccLocation_test.cpp:16-104), for FCC ternary random and dilute
  configurations with canonical and semi-grand canonical proposals.
* Semi-grand canonical proposals: draw-for-draw equal to the oracle's restatement of
  OccEventProposal.hh:168-247 with std::mt19937_64 and libstdc++'s distributions.
* basic_occupation_metropolis driving the Ising model through user functions: the same
  trajectory, counters and samples as the oracle's Ising semi-grand canonical run.
* OccLocation with atoms moving to and from a reservoir (vacancies as occupants with no
  atoms): atom ids freed and reused, unique atom ids, initial and final atom info with
  times; ``replace_mol``.
"""
import numpy as np
import pytest

import casmcode_monte_gb300 as monte
import casmcode_monte_gb300.events as ev
import casmcode_monte_gb300.methods as methods
import casmcode_monte_gb300.sampling as sampling
from tests import oracle_lib


def bijk(b, i, j, k):
    return ev.IntegralSiteCoordinate.from_list([b, i, j, k])


def test_conversions_cubic():
    convert = ev.Conversions(ev.Prim.cubic(1.0, ["A", "B"]), np.eye(3, dtype=int) * 3)
    assert convert.l_size() == 27
    assert convert.asym_size() == 1
    assert convert.occ_size(0) == 2 and convert.species_size() == 2


def test_conversions_two_sites():
    prim = ev.Prim(np.eye(3), np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.5]]).T, [["A", "B"], ["B", "C"]])
    convert = ev.Conversions(prim, np.eye(3, dtype=int) * 3)
    assert convert.l_size() == 54
    f = convert.site_index_converter()
    assert f.total_sites() == 54
    assert f.linear_site_index(bijk(1, 0, 0, 0)) == 27
    assert convert.bijk_to_l(bijk(1, 0, 0, 0)) == 27
    assert convert.l_to_bijk(27) == bijk(1, 0, 0, 0)
    assert convert.bijk_to_l(bijk(1, 0, 0, 0) + np.array([1, 0, 0])) == convert.bijk_to_l(bijk(1, 1, 0, 0))
    # periodic images and round trips
    assert convert.bijk_to_l(bijk(0, 3, -3, 6)) == 0
    for l in range(convert.l_size()):
        assert convert.bijk_to_l(convert.l_to_bijk(l)) == l
    # sites differ in occupants: two asymmetric units; species A, B, C
    assert convert.asym_size() == 2
    assert [convert.species_name(i) for i in range(convert.species_size())] == ["A", "B", "C"]
    assert convert.species_index(1, 0) == 1 and convert.occ_index(1, 2) == 1
    assert not convert.species_allowed(0, 2) and convert.occ_index(0, 2) == convert.occ_size(0)


def _mol_prim(orders):
    occupants = {"A": ev.Occupant.atom("A")}
    for axis, name in enumerate(("mol.x", "mol.y", "mol.z")):
        d = np.zeros(3)
        d[axis] = 0.1
        occupants[name] = ev.Occupant("mol", [("B", -d), ("B", d)])
    coords = np.array([[0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]]).T
    return ev.Prim(np.eye(3), coords, orders, occupants)


def test_conversions_molecules_and_occupant_order():
    full = ["A", "mol.x", "mol.y", "mol.z"]
    convert = ev.Conversions(_mol_prim([["A"], full, full, full]), np.eye(3, dtype=int) * 3)
    assert convert.l_size() == 27 * 4
    assert convert.asym_size() == 2
    shuffled = ["mol.x", "mol.y", "mol.z", "A"]
    convert = ev.Conversions(_mol_prim([["A"], full, shuffled, full]), np.eye(3, dtype=int) * 3)
    assert convert.l_size() == 27 * 4
    assert convert.asym_size() == 3


def test_nondiagonal_supercell_indexing():
    T = np.array([[1, 1, 0], [-1, 1, 0], [0, 0, 2]])
    convert = ev.Conversions(ev.Prim.fcc(4.0, ["A", "B"]), T)
    assert convert.l_size() == 4
    seen = {convert.bijk_to_l(convert.l_to_bijk(l)) for l in range(4)}
    assert seen == {0, 1, 2, 3}
    # translations by supercell lattice vectors map a site onto itself
    for l in range(4):
        x = convert.l_to_bijk(l)
        for n in np.eye(3, dtype=int):
            assert convert.bijk_to_l(x + T @ n) == l


def test_swaps():
    convert = ev.Conversions(ev.Prim.fcc(4.0, ["A", "B", "C"]), np.eye(3, dtype=int) * 2)
    cands = ev.OccCandidateList(convert)
    assert len(cands) == 3 and [cands.index(c) for c in cands] == [0, 1, 2]
    sgc = ev.make_semigrand_canonical_swaps(convert, cands)
    assert [(s.cand_a.species_index, s.cand_b.species_index) for s in sgc] == [(0, 1), (0, 2), (1, 0), (1, 2),
                                                                               (2, 0), (2, 1)]
    can = ev.make_canonical_swaps(convert, cands)
    assert [(s.cand_a.species_index, s.cand_b.species_index) for s in can] == [(0, 1), (0, 2), (1, 2)]
    assert ev.swaps_allowed_per_unitcell(convert, sgc) == 5
    binary = ev.Conversions(ev.Prim.fcc(4.0, ["A", "B"]), np.eye(3, dtype=int) * 2)
    assert ev.swaps_allowed_per_unitcell(binary, ev.make_semigrand_canonical_swaps(binary,
                                                                                    ev.OccCandidateList(binary))) == 1
    multis = ev.make_multiswaps(sgc, 2)
    assert len(multis) == 6 + 21  # one swap, or a multiset of two of the six
    assert all(m.total_count in (1, 2) for m in multis)
    assert ev.OccSwap(cands[1], cands[0]).sorted() == ev.OccSwap(cands[0], cands[1])


def _check_init(occ, loc, convert, cands):
    for mol_id in range(loc.mol_size()):
        assert loc.mol(mol_id).id == mol_id
    for l in range(occ.size):
        mol_id = loc.l_to_mol_id(l)
        if mol_id == loc.mol_size():
            continue
        mol = loc.mol(mol_id)
        assert mol.l == l and mol.id == mol_id
        asym = convert.l_to_asym(l)
        assert asym == mol.asym
        assert occ[l] == convert.occ_index(asym, mol.species_index)
        assert convert.species_index(asym, int(occ[l])) == mol.species_index
        assert loc.mol_id(cands.index(mol.asym, mol.species_index), mol.loc) == mol.id


def _check_event(occ, e, loc, convert, cands):
    for t in e.occ_transform:
        mol_id = loc.l_to_mol_id(t.l)
        mol = loc.mol(mol_id)
        assert mol.l == t.l and mol.id == mol_id and t.mol_id == mol_id
        asym = convert.l_to_asym(t.l)
        assert asym == mol.asym
        assert occ[t.l] == convert.occ_index(asym, mol.species_index)
        assert loc.mol_id(cands.index(mol.asym, mol.species_index), mol.loc) == mol.id


@pytest.mark.parametrize("dilute", [False, True])
@pytest.mark.parametrize("kind", ["canonical", "semigrand_canonical"])
def test_occ_location_invariants(dilute, kind):
    convert = ev.Conversions(ev.Prim.fcc(4.0, ["A", "B", "C"]), np.eye(3, dtype=int) * 9)
    n = convert.l_size()
    rng_np = np.random.default_rng(7)
    occ = np.zeros(n, dtype=np.int32) if dilute else rng_np.integers(0, 3, size=n).astype(np.int32)
    if dilute:
        occ[rng_np.choice(n, size=3, replace=False)] = [1, 2, 1]
    cands = ev.OccCandidateList(convert)
    swaps = (ev.make_canonical_swaps if kind == "canonical" else ev.make_semigrand_canonical_swaps)(convert, cands)
    propose = ev.propose_canonical_event if kind == "canonical" else ev.propose_semigrand_canonical_event
    loc = ev.OccLocation(convert, cands)
    loc.initialize(occ)
    _check_init(occ, loc, convert, cands)
    engine = monte.RandomNumberEngine()
    engine.seed(11)
    rng = monte.RandomNumberGenerator(engine)
    e = ev.OccEvent()
    counts0 = np.bincount(occ, minlength=3)
    for _ in range(3000):
        propose(e, loc, swaps, rng)
        _check_event(occ, e, loc, convert, cands)
        loc.apply(e, occ)
        _check_event(occ, e, loc, convert, cands)
    _check_init(occ, loc, convert, cands)
    if kind == "canonical":
        assert np.array_equal(np.bincount(occ, minlength=3), counts0)


def test_semigrand_canonical_proposals_match_oracle(oracle):
    convert = ev.Conversions(ev.Prim.fcc(4.0, ["A", "B", "C"]), np.eye(3, dtype=int) * 6)
    n = convert.l_size()
    occ = np.random.default_rng(3).integers(0, 3, size=n).astype(np.int32)
    ref_l, ref_o = oracle_lib.sgc_proposals(occ, 3, 2024, 4000, apply=True)
    cands = ev.OccCandidateList(convert)
    swaps = ev.make_semigrand_canonical_swaps(convert, cands)
    loc = ev.OccLocation(convert, cands)
    work = occ.copy()
    loc.initialize(work)
    engine = monte.RandomNumberEngine()
    engine.seed(2024)
    rng = monte.RandomNumberGenerator(engine)
    e = ev.OccEvent()
    got_l, got_o = [], []
    for _ in range(4000):
        ev.propose_semigrand_canonical_event(e, loc, swaps, rng)
        got_l.append(e.linear_site_index[0])
        got_o.append(e.new_occ[0])
        loc.apply(e, work)
    assert got_l == ref_l.tolist()
    assert got_o == ref_o.tolist()


def test_metropolis_acceptance_draws_only_uphill():
    engine = monte.RandomNumberEngine()
    engine.seed(5)
    rng = monte.RandomNumberGenerator(engine)
    s0 = engine.dump()
    assert methods.metropolis_acceptance(-1e-3, 10.0, rng)
    assert engine.dump() == s0
    methods.metropolis_acceptance(1e-3, 10.0, rng)
    assert engine.dump() != s0


def test_basic_occupation_metropolis_matches_oracle(oracle):
    import casmcode_monte_gb300.ising_cpp as ising
    import casmcode_monte_gb300.ising_cpp.semigrand_canonical as sgc

    rows = cols = 8
    J, T, mu, n_pass = 0.1, 2000.0, 0.0, 25
    system = ising.IsingSystem(formation_energy_calculator=ising.IsingFormationEnergy(J=J, lattice_type=1,
                                                                                      use_nlist=True),
                               param_composition_calculator=ising.IsingParamComposition())
    state = ising.IsingState(configuration=ising.IsingConfiguration(shape=(rows, cols)),
                             conditions=monte.ValueMap.from_dict({"temperature": T, "exchange_potential": [mu]}))
    occ0 = state.configuration.occupation().copy()
    potential = sgc.SemiGrandCanonicalPotential(system)
    potential.set_state(state, sgc.SemiGrandCanonicalConditions.from_values(state.conditions))
    N = rows * cols

    def propose(rng):
        e = ev.OccEvent()
        l = rng.random_int(N - 1)
        e.linear_site_index = [l]
        e.new_occ = [-state.configuration.occ(l)]
        return e

    def delta(e):
        return potential.occ_delta_per_supercell(e.linear_site_index, e.new_occ)

    def apply(e):
        state.configuration.set_occ(e.linear_site_index[0], e.new_occ[0])

    fmap = sampling.StateSamplingFunctionMap()
    fmap["potential_energy"] = sampling.StateSamplingFunction(
        "potential_energy", "", [], lambda: np.array([potential.per_unitcell()]))
    params = sampling.CompletionCheckParams()
    params.cutoff_params.max_count = n_pass
    data = methods.BasicOccupationMetropolisData(fmap, sampling.jsonStateSamplingFunctionMap(), N, params)
    engine = monte.RandomNumberEngine()
    engine.seed(77)
    methods.basic_occupation_metropolis(data, T, delta, propose, apply, sample_period=1,
                                        method_log=monte.MethodLog(None, None), random_engine=engine,
                                        write_status_f=methods.write_no_status)
    ref = oracle_lib.ising_run(rows, cols, J, True, T, mu, occ0, oracle_lib.make_cc_params(max_count=n_pass), 1,
                               oracle_lib.engine_state(77))
    assert data.n_pass == n_pass
    assert data.n_accept == ref["out"].n_accept and data.n_reject == ref["out"].n_reject
    assert state.configuration.occupation().tolist() == ref["occ"].tolist()
    pe = data.samplers["potential_energy"].component(0)
    assert [float.hex(float(x)) for x in pe] == [float.hex(float(x)) for x in ref["potential_energy"]]
    assert engine.dump() == ref["engine"]


def _reservoir_setup(**kw):
    prim = ev.Prim(np.eye(3), np.zeros((3, 1)), [["A", "B", "Va"]], occupants={"Va": ev.Occupant("Va", [])})
    convert = ev.Conversions(prim, np.eye(3, dtype=int) * 2)
    occ = np.array([0, 1, 2, 0, 1, 2, 0, 0], dtype=np.int32)
    loc = ev.OccLocation(convert, ev.OccCandidateList(convert), update_atoms=True, **kw)
    return convert, occ, loc


def _flip(loc, l, to_species):
    mol = loc.mol(loc.l_to_mol_id(l))
    return ev.OccTransform(l=l, mol_id=mol.id, asym=mol.asym, from_species=mol.species_index, to_species=to_species)


def test_occ_location_reservoir_moves_and_unique_atoms():
    """Atoms to and from a reservoir (OccLocation.cc:216-366): a leaving atom frees its atom
    id (translation and n_jumps set to LONG_MIN, unique id -1), an entering atom takes the
    smallest free id with the next unique id, final and initial atom info carry the time."""
    convert, occ, loc = _reservoir_setup(track_unique_atoms=True, save_atom_info=True)
    A, B, Va = (convert.species_index(0, i) for i in range(3))
    loc.initialize(occ, time=0.0)
    assert loc.atom_size() == 6 and loc.unique_atom_id() == list(range(6))
    assert loc.current_atom_names() == ["A", "B", "A", "B", "A", "A"]
    assert sorted(loc.atom_info_initial()) == list(range(6))
    assert all(i.time == 0.0 for i in loc.atom_info_initial().values())

    # site 3 (atom id 2) leaves to the reservoir at t = 1.5
    e = ev.OccEvent()
    e.occ_transform = [_flip(loc, 3, Va)]
    e.atom_traj = [ev.AtomTraj(ev.AtomLocation(3, loc.l_to_mol_id(3), 0), ev.AtomLocation(-1, A, 0))]
    loc.apply(e, occ, time=1.5)
    lmin = np.iinfo(np.int64).min
    assert occ[3] == 2 and loc.cand_size(loc.candidate_list().index(0, Va)) == 3
    assert loc.atom(2).n_jumps == lmin and list(loc.atom(2).translation) == [lmin] * 3
    assert loc.unique_atom_id()[2] == -1 and loc.initial_atom_species_index()[2] == -1
    assert loc.current_atom_names()[2] == "UK" and loc.current_atom_species_index()[2] == -1
    info = loc.atom_info_final()[2]
    assert (info.species_index, info.position_index, info.time) == (A, 0, 1.5)

    # a B atom enters on site 2 at t = 2.5: it reuses atom id 2 with unique id 6; its
    # species index is recorded from the trajectory's to.mol_id, as the reference does
    m2 = loc.l_to_mol_id(2)
    e.occ_transform = [_flip(loc, 2, B)]
    e.atom_traj = [ev.AtomTraj(ev.AtomLocation(-1, B, 0), ev.AtomLocation(2, m2, 0))]
    loc.apply(e, occ, time=2.5)
    assert occ[2] == 1 and loc.atom_size() == 6 and loc.unique_atom_id()[2] == 6
    assert loc.mol(m2).component == [2] and loc.atom(2).n_jumps == 0
    assert list(loc.atom(2).translation) == list(convert.l_to_ijk(2))
    assert loc.initial_atom_species_index()[2] == m2
    assert loc.current_atom_names()[2] == "B" and loc.current_atom_species_index()[2] == B
    assert loc.atom_info_initial()[6].time == 2.5

    # another enters with no free id: appended as atom id 6, unique id 7
    e.occ_transform = [_flip(loc, 5, A)]
    e.atom_traj = [ev.AtomTraj(ev.AtomLocation(-1, A, 0), ev.AtomLocation(5, loc.l_to_mol_id(5), 0))]
    loc.apply(e, occ, time=3.0)
    assert loc.atom_size() == 7 and loc.unique_atom_id()[6] == 7
    # a jump within the supercell: site 0 -> site 3 (vacant), one lattice translation
    e.occ_transform = [_flip(loc, 0, Va), _flip(loc, 3, A)]
    e.atom_traj = [ev.AtomTraj(ev.AtomLocation(0, loc.l_to_mol_id(0), 0), ev.AtomLocation(3, loc.l_to_mol_id(3), 0),
                               np.array([1, 0, 0]))]
    loc.apply(e, occ, time=4.0)
    assert loc.mol(loc.l_to_mol_id(3)).component == [0] and loc.current_atom_n_jumps()[0] == 1
    assert list(loc.atom(0).translation) == [1, 0, 0] and loc.unique_atom_id()[0] == 0
    assert sorted(loc.atom_info_final()) == [2]
    loc.clear_atom_info_final()
    assert loc.atom_info_final() == {}
    # re-initialising (one atom left, two entered) renumbers and resets the records
    loc.initialize(occ, time=5.0)
    assert loc.unique_atom_id() == list(range(7)) and loc.atom_info_final() == {}
    assert len(loc.initial_atom_species_index()) == 7 and sorted(loc.atom_info_initial()) == list(range(7))


def test_occ_location_replace_mol():
    """replace_mol puts an occupant with given atoms on a site (OccLocation.cc:506-548);
    refused while tracking unique atoms."""
    convert, occ, loc = _reservoir_setup()
    A, B, Va = (convert.species_index(0, i) for i in range(3))
    loc.initialize(occ)
    a = ev.Atom(translation=np.array([0, 1, 0]), n_jumps=4)
    loc.replace_mol(2, 1, [5], [a])  # site 2 (vacant) gets a B atom as atom id 5
    m = loc.mol(loc.l_to_mol_id(2))
    assert m.species_index == B and m.component == [5] and loc.atom(5).n_jumps == 4
    assert loc.cand_size(loc.candidate_list().index(0, Va)) == 1
    assert loc.cand_size(loc.candidate_list().index(0, B)) == 3
    for cand in range(3):
        for i in range(loc.cand_size(cand)):
            assert loc.mol(loc.mol_id(cand, i)).loc == i
    _, occ2, tracked = _reservoir_setup(track_unique_atoms=True)
    tracked.initialize(occ2)
    with pytest.raises(RuntimeError, match="tracking unique atoms"):
        tracked.replace_mol(2, 1, [5], [a])


def test_reference_binding_names_and_dict_forms():
    """Methods and fields under the names of the reference's binding
    (python/src/monte_events.cpp) and the dict forms of OccCandidate_json_io.cc:40-209."""
    convert = ev.Conversions(ev.Prim.fcc(4.0, ["A", "B", "C"]), np.eye(3, dtype=int) * 2)
    assert convert.species_name_to_index("B") == 1 and convert.species_index_to_name(2) == "C"
    assert convert.occ_to_species_index(0, 1) == 1 and convert.species_to_occ_index(0, 2) == 2
    assert convert.species_index_to_occupant(0).name == "A" and convert.species_index_to_atoms_size(0) == 1
    assert np.array_equal(convert.unit_transformation_matrix_to_super(), np.eye(3))
    assert convert.unitcell_index_converter().total_unitcells() == 8
    assert convert.bijk_to_unitl(bijk(0, 1, 1, 0)) == 0 and convert.unitl_to_bijk(0) == bijk(0, 0, 0, 0)

    cand = ev.OccCandidate(0, 2)
    assert cand.asymmetric_unit_index == 0 and cand.is_valid(convert) and not ev.OccCandidate(1, 0).is_valid(convert)
    assert cand.to_dict(convert) == {"asym": 0, "spec": "C"}
    assert ev.OccCandidate.from_dict({"asym": 0, "spec": "C"}, convert) == cand
    with pytest.raises(RuntimeError, match="not a valid option"):
        ev.OccCandidate.from_dict({"asym": 0, "spec": "Q"}, convert)
    swap = ev.OccSwap(ev.OccCandidate(0, 2), ev.OccCandidate(0, 1))
    assert swap.first == ev.OccCandidate(0, 2) and swap.is_valid(convert)
    assert ev.OccSwap.from_dict(swap.to_dict(convert), convert) == swap
    m = ev.MultiOccSwap({swap: 2})
    swap.sort()  # in place; the multi-swap holds its own copy
    assert swap.first == ev.OccCandidate(0, 1) and list(m.swaps) == [ev.OccSwap(ev.OccCandidate(0, 2),
                                                                                 ev.OccCandidate(0, 1))]
    swap.reverse()
    assert swap.second == ev.OccCandidate(0, 1)
    assert ev.MultiOccSwap.from_dict(m.to_dict(convert), convert) == m
    m2 = m.__copy__()
    m2.reverse()
    assert m2 == m.reversed() and m2 != m
    assert m.to_dict(convert) == [{"swap": [{"asym": 0, "spec": "C"}, {"asym": 0, "spec": "B"}], "count": 2}]

    cl = ev.OccCandidateList(convert)
    d = cl.to_dict(convert)
    assert len(d["candidate"]) == 3 and len(d["canonical_swaps"]) == 3 and len(d["grand_canonical_swaps"]) == 6
    cl2 = ev.OccCandidateList.from_dict(d, convert)
    assert list(cl2) == list(cl) and cl2.matching_index(0, 1) == cl.index(ev.OccCandidate(0, 1))
    assert list(ev.OccCandidateList.from_dict(d["candidate"], convert)) == list(cl)

    occ = np.array([0, 1, 2, 0, 1, 2, 0, 1], dtype=np.int32)
    loc = ev.OccLocation(convert, cl)
    loc.initialize(occ)
    ci = cl.index(ev.OccCandidate(0, 1))
    assert loc.cand_size_by_candidate_index(ci) == 3 == loc.cand_size(ev.OccCandidate(0, 1))
    mol = loc.mol(loc.mol_id_by_candidate_index(ci, 0))
    assert mol.species_index == 1 and loc.linear_site_index_to_mol_id(mol.linear_site_index) == mol.id
    assert (mol.asymmetric_unit_index, mol.mol_location_index, mol.component_id) == (0, 0, [])
    g = monte.RandomNumberGenerator()
    assert loc.choose_mol_by_candidate_index(ci, g).species_index == 1
    traj = ev.AtomTraj(ev.AtomLocation(3, 3, 0), ev.AtomLocation(5, 5, 0))
    assert getattr(traj, "from").linear_site_index == 3
    e = ev.OccEvent([3], [1], [ev.OccTransform(3, 3, 0, 0, 1)], [traj])
    e2 = e.__copy__()
    e2.occ_transform[0].linear_site_index = 4
    assert e.occ_transform[0].l == 3 and e2.occ_transform[0].l == 4


def test_conversions_with_a_custom_unit_cell():
    """An asymmetric unit on a 2x1x1 unit supercell of a one-site cubic prim (two
    sublattices of alternating planes), Conversions.cc:114-174."""
    prim = ev.Prim.cubic(1.0, ["A", "B"])
    species = [prim.occupants["A"], prim.occupants["B"]]
    T = np.diag([4, 2, 2])
    convert = ev.Conversions.make_with_custom_unitcell(prim, species, T, np.diag([2, 1, 1]), [0, 1])
    assert convert.unitl_size() == 2 and convert.asym_size() == 2
    for l in range(convert.l_size()):
        i = int(convert.l_to_ijk(l)[0])
        assert convert.l_to_unitl(l) == i % 2 and convert.l_to_asym(l) == i % 2
    assert convert.asym_to_unitl(1) == {1} and convert.asym_to_b(1) == {0}
    assert convert.occ_size(1) == 2 and convert.species_index(1, 1) == 1
    with pytest.raises(ValueError, match="tile"):
        ev.Conversions.make_with_custom_unitcell(prim, species, T, np.diag([3, 1, 1]), [0, 1, 0])
    lower = ev.Conversions.make_with_custom_asym(prim, T, [0])
    assert lower.asym_size() == 1
