"""Serial replay of the reference's semi-grand canonical dynamics for cluster expansions.

The GPU replay (mg_ce_replay_*) consumes each chain's std::mt19937_64 exactly as the
reference's loop does (OccEventProposal.hh:260-336 swap and site choice, metropolis.hh:26-35,
OccLocation.cc:216-283 list updates).  Against the oracle's restatement of that loop, started
from the same engine state, the final occupations, per-pass accepted counts, the occupant
lists in list order and the final engine state must be identical; the per-pass potential
energies agree to rounding (the oracle tracks a running FP64 sum, the GPU reports exact
integer correlation sums).
"""
import numpy as np
import pytest

import casmcode_monte_gb300 as monte
from casmcode_monte_gb300 import clex
from tests.oracle_lib import OracleCE

pytestmark = pytest.mark.gpu


def _engine(seed):
    e = monte.RandomNumberEngine()
    e.seed(seed)
    return e.dump()


@pytest.mark.parametrize("kind,L,T,mu", [("fcc_binary", (8, 8, 8), [700.0, 1600.0], [[0.0], [0.04]]),
                                         ("fcc_ternary", (8, 8, 8), [900.0, 1800.0], [[0.02, -0.01], [0.0, 0.05]]),
                                         ("fcc_binary", (12, 8, 10), [500.0, 2000.0], [[-0.02], [0.1]])])
def test_replay_matches_reference_dynamics(gpu_lib, kind, L, T, mu):
    ns = 2 if kind == "fcc_binary" else 3
    model = clex.ClexModel(kind, clex.make_eci(kind, 7))
    rng = np.random.default_rng(3)
    N = L[0] * L[1] * L[2]
    occ = np.stack([clex.random_occupation(ns, N, rng) for _ in range(2)])
    mu = np.asarray(mu, dtype=float)
    states = [_engine(101), _engine(202)]
    n_passes = 100
    rb = clex.ReplayBatch(model, L, occ, T, mu, states)
    corr0 = np.stack([OracleCE(L, ns, model.eci).int_corr(occ[c], model.n_classes) for c in range(2)])
    out = rb.run(60)
    out = np.concatenate([out, rb.run(n_passes - 60)])  # two calls continue the same stream
    got = rb.occupation()
    acc, rej = rb.counts()
    orc = OracleCE(L, ns, model.eci)
    for c in range(2):
        ref = orc.sgc_run(occ[c], T[c], mu[c], states[c], n_passes)
        assert np.array_equal(got[c], ref["occ"].astype(np.int8)), c
        assert np.array_equal(out[:, c, 0], ref["n_accept"]), c
        assert int(acc[c]) == int(ref["n_accept"].sum()) and int(acc[c] + rej[c]) == n_passes * N
        assert np.array_equal(out[:, c, model.n_classes], N - ref["n_accept"])
        lists = rb.candidates(c)
        for s in range(ns):
            assert np.array_equal(lists[s], ref["lists"][s]), (c, s)
        assert rb.engine_state(c) == ref["engine"], c
        # energies from the exact integer correlation sums against the oracle's running sum
        d = out[:, c:c + 1, :].copy()
        d[:, :, model.n_classes:] = 0
        s = clex.accumulate(model, corr0[c:c + 1], d, mu[c:c + 1], N)
        np.testing.assert_allclose(s.potential_energy[:, 0], ref["potential_energy"], rtol=0, atol=1e-12)
        np.testing.assert_allclose(s.param_composition[:, 0, :], ref["param_composition"], rtol=0, atol=0)
        assert np.array_equal(s.int_corr[-1, 0], orc.int_corr(ref["occ"], model.n_classes))
    rb.close()


def test_replay_rejects_bad_input(gpu_lib):
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 1))
    occ = np.zeros((1, 512), dtype=np.int8)
    occ[0, 3] = 2
    with pytest.raises(RuntimeError, match="occupant index out of range"):
        clex.ReplayBatch(model, (8, 8, 8), occ, [1000.0], [[0.0]], [_engine(1)])
    with pytest.raises(RuntimeError, match="malformed engine state"):
        clex.ReplayBatch(model, (8, 8, 8), np.zeros((1, 512), dtype=np.int8), [1000.0], [[0.0]], ["1 2 3"])
