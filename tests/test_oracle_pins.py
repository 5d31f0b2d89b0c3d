"""Pin the oracle to the reference's known answers (CPU only).

* mt19937_64: the 10000th output of a default-constructed engine is 9981545732273789042
  (C++ standard [rand.predef]); the engine behind the reference's RandomNumberGenerator
  (include/casm/monte/definitions.hh:17).
* Philox4x32-10 known-answer vectors (Random123 distribution).
* Ising algebra known answers of tests/unit/monte/Ising_basic_semigrand_canonical_test.cpp:
  25x25 all +1, J = 0.1: E_f = -125.0 (per unit cell -0.2), dE_f(site 0 -> -1) = 8J,
  no-op dE = 0, N x = 625, N dx = -1, E_sgc = N(-2J - mu) at mu = 2, dE_sgc = 8J + mu.
* The oracle's independent cluster enumeration agrees with the generated basis tables.
* Golden trajectories committed under tests/golden/ (made by tests/golden/make_golden.py).
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

from tests import oracle_lib

HERE = os.path.dirname(os.path.abspath(__file__))


def test_mt19937_64_known_answer(oracle):
    assert oracle.orc_mt19937_64_10000th() == 9981545732273789042


@pytest.mark.parametrize("ctr,key,expect", [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
])
def test_philox_known_answers(oracle, ctr, key, expect):
    out = (C.c_uint * 4)()
    oracle.orc_philox4x32_10((C.c_uint * 4)(*ctr), (C.c_uint * 2)(*key), out)
    assert tuple(out) == expect


@pytest.mark.parametrize("use_nlist", [0, 1])
def test_ising_known_answers(oracle, use_nlist):
    occ = (C.c_int * 625)(*([1] * 625))
    J = C.c_double(0.1)
    ef = oracle.orc_ising_formation(25, 25, J, use_nlist, occ)
    assert ef == pytest.approx(-125.0, abs=1e-12)
    assert ef / 625 == pytest.approx(-0.2, abs=1e-15)
    # dE_f for site 0 -> -1 and the no-op, at mu = 0
    assert oracle.orc_ising_delta(25, 25, J, use_nlist, occ, 0, -1, C.c_double(0.0)) == pytest.approx(0.8)
    assert oracle.orc_ising_delta(25, 25, J, use_nlist, occ, 0, 1, C.c_double(0.0)) == 0.0
    # semi-grand canonical at mu = 2: dE = 8J - mu * N dx = 0.8 + 2
    assert oracle.orc_ising_delta(25, 25, J, use_nlist, occ, 0, -1, C.c_double(2.0)) == pytest.approx(2.8)
    # E_sgc = E_f - mu * N x = -125 - 2 * 625
    assert ef - 2.0 * 625 == pytest.approx(-1375.0)


@pytest.mark.parametrize("n_species,kind", [(2, "fcc_binary"), (3, "fcc_ternary")])
def test_oracle_classes_match_generated_tables(oracle, n_species, kind):
    n = oracle.orc_ce_n_classes_for(n_species)
    sizes = (C.c_int * n)()
    mults = (C.c_long * n)()
    dec = (C.c_long * n)()
    oracle.orc_ce_class_info(n_species, sizes, mults, dec)
    with open(os.path.join(HERE, "..", "casmcode_monte_gb300", "csrc", "generated", f"{kind}.json")) as f:
        d = json.load(f)
    assert n == len(d["classes"])
    for i, c in enumerate(d["classes"]):
        code = 0
        for b in c["decoration"]:
            code = code * 4 + (b + 1)
        assert (sizes[i], mults[i], dec[i]) == (c["size"], c["multiplicity"], code)
    # FCC neighbourhood: 12 + 6 + 24 + 12 = 54 sites in the 1-4NN shells
    assert len(d["neighbour_offsets"]) == 54


def test_oracle_ce_energy_consistency(oracle):
    """dE from the clexulator-style local formula equals the change of the energy
    recomputed from correlations, for the binary and ternary bases."""
    for n_species, kind in ((2, "fcc_binary"), (3, "fcc_ternary")):
        with open(os.path.join(HERE, "..", "casmcode_monte_gb300", "csrc", "generated", f"{kind}.json")) as f:
            nc = len(json.load(f)["classes"])
        rng = np.random.default_rng(4)
        eci = rng.normal(0, 0.03, nc)
        L = (6, 5, 7)
        orc = oracle_lib.OracleCE(L, n_species, eci)
        occ = rng.integers(0, n_species, size=orc.n).astype(np.int32)
        mu = rng.uniform(-0.2, 0.2, n_species - 1)
        for _ in range(10):
            l = int(rng.integers(0, orc.n))
            new = int((occ[l] + 1 + rng.integers(0, n_species - 1)) % n_species)
            dE = orc.delta_e(occ, l, new, mu)
            e0 = orc.formation(occ)
            occ2 = occ.copy()
            occ2[l] = new
            e1 = orc.formation(occ2)
            dmu = sum(mu[i] * (int(new == i + 1) - int(occ[l] == i + 1)) for i in range(n_species - 1))
            assert dE == pytest.approx((e1 - e0) - dmu, abs=1e-11)


def test_golden_ising_trajectory(oracle):
    """The oracle reproduces the committed golden Ising run."""
    path = os.path.join(HERE, "golden", "ising_25x25_seed1.json")
    with open(path) as f:
        g = json.load(f)
    ref = oracle_lib.ising_run(g["rows"], g["cols"], g["J"], g["use_nlist"], g["T"], g["mu"], np.array(g["occ0"]),
                               oracle_lib.make_cc_params(max_count=g["n_passes"]), 1,
                               oracle_lib.engine_state(g["seed"]))
    assert ref["out"].n_pass == g["n_passes"]
    assert ref["out"].n_accept == g["n_accept"]
    assert ref["occ"].tolist() == g["occ_final"]
    assert [float.hex(x) for x in ref["potential_energy"]] == g["potential_energy_hex"]


def test_golden_ce_delta_e(oracle):
    path = os.path.join(HERE, "golden", "ce_delta_e.json")
    with open(path) as f:
        g = json.load(f)
    for case in g["cases"]:
        orc = oracle_lib.OracleCE(tuple(case["L"]), case["n_species"], np.array(case["eci"]))
        occ = np.array(case["occ"], dtype=np.int32)
        for l, new, mu, dE_hex in case["proposals"]:
            assert orc.delta_e(occ, l, new, np.array(mu)) == float.fromhex(dE_hex)
