"""Canonical (fixed-composition) sweeps of FCC cluster expansions on the GPU.

The reference's canonical event (events.propose_canonical_event: a swap of two occupants of
different species, OccEventProposal.hh:108-237) accepted by metropolis_acceptance is made
parallel by exchanging the occupants of matched same-colour sites, passes alternating
between two colourings whose classes connect every site.  Checked here:

* trajectories equal the oracle's restatement of that sweep pass for pass (occupations,
  correlation sums after every pass, accepted swaps), binary and ternary, FP32 decisions
  with exact FP64 re-decision;
* composition is conserved and tracked correlations equal a full recompute;
* atoms move between the classes of a colouring (the alternation of colourings works);
* <E_f> and the heat capacity at fixed composition agree with a run of the reference's own
  canonical dynamics (random swaps of two different occupants, std::mt19937_64) within twice
  the combined 95 % autocorrelation-corrected error bars (BasicStatistics.cc:24-188).
"""
import numpy as np
import pytest

from casmcode_monte_gb300 import clex
from casmcode_monte_gb300.sampling import BasicStatisticsCalculator
from tests.oracle_lib import OracleCE

pytestmark = pytest.mark.gpu

KB = 8.6173303e-05


def _setup(kind, L, n_chains, seed):
    ns = 2 if kind == "fcc_binary" else 3
    model = clex.ClexModel(kind, clex.make_eci(kind, seed))
    rng = np.random.default_rng(seed)
    N = L[0] * L[1] * L[2]
    occ = np.stack([clex.random_occupation(ns, N, rng) for _ in range(n_chains)])
    T = np.linspace(600.0, 1800.0, n_chains)
    seeds = np.arange(31, 31 + n_chains, dtype=np.uint64) * np.uint64(7919)
    return model, occ, T, seeds, ns


@pytest.mark.parametrize("kind,L,n_chains", [("fcc_binary", (8, 8, 8), 2), ("fcc_binary", (16, 8, 12), 2),
                                             ("fcc_ternary", (12, 12, 12), 2), ("fcc_ternary", (9, 9, 9), 1),
                                             ("fcc_binary", (16, 16, 16), 3)])
def test_canonical_sweep_equals_oracle(gpu_lib, kind, L, n_chains):
    model, occ, T, seeds, ns = _setup(kind, L, n_chains, seed=L[0] + n_chains)
    b = clex.CanonicalBatch(model, L, occ, T, seeds)
    col_a, col_b = b.colors(0), b.colors(1)
    for col, order in ((col_a, b.class_order(0)), (col_b, b.class_order(1))):
        assert np.array_equal(np.sort(order), np.arange(order.size))  # a permutation of the sites
        assert (np.diff(col[order]) >= 0).all()                        # grouped colour by colour
    corr0 = b.corr()
    nc = model.n_classes
    outs = [b.run(3), b.run(4)]  # pass 0..2, then 3..6: both colourings, two launches
    out = np.concatenate(outs, axis=0)
    got = b.occupation()
    orc = OracleCE(L, ns, model.eci)
    for c in range(n_chains):
        occ_ref, corr_ref, nacc_ref = orc.canonical_sweep(occ[c], T[c], int(seeds[c]), c, col_a, b.n_colors[0],
                                                          col_b, b.n_colors[1], 0, 7, nc, b.class_order(0),
                                                          b.class_order(1))
        assert np.array_equal(got[c], occ_ref.astype(np.int8)), c
        d = out[:, c, :nc].copy()
        d[:, 0] = 0
        assert np.array_equal(corr0[c][None, :] + np.cumsum(d, axis=0), corr_ref), c
        assert np.array_equal(out[:, c, 0], nacc_ref), c
        assert nacc_ref.sum() > 0


def test_canonical_conserves_composition_and_tracks_correlations(gpu_lib):
    model, occ, T, seeds, ns = _setup("fcc_ternary", (16, 16, 16), 4, seed=5)
    b = clex.CanonicalBatch(model, (16, 16, 16), occ, T, seeds, precision="fp32")
    corr0 = b.corr()
    out = b.run(60)
    d = out[:, :, :model.n_classes].copy()
    d[:, :, 0] = 0
    assert np.array_equal(corr0 + d.sum(axis=0), b.corr())
    final = b.occupation()
    for c in range(4):
        assert np.array_equal(np.bincount(final[c], minlength=3), np.bincount(occ[c], minlength=3))
    assert (out[:, :, 0] > 0).all()


def test_canonical_moves_atoms_between_classes(gpu_lib):
    """All B atoms start in one class of colouring A: swaps within A's classes alone could
    never take them out, the passes on colouring B must."""
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 2))
    L = (16, 16, 16)
    N = 16 ** 3
    probe = clex.CanonicalBatch(model, L, np.zeros((1, N), dtype=np.int8), [1000.0], [1])
    col_a = probe.colors(0)
    occ = (col_a == 0).astype(np.int8)[None, :]
    b = clex.CanonicalBatch(model, L, occ, [3000.0], [77])
    b.run(40, want_output=False)
    final = b.occupation()[0]
    assert final.sum() == occ.sum()
    assert (final[col_a == 0] == 1).sum() < 0.5 * occ.sum()


def test_canonical_rejects_supercell_larger_than_shared_memory(gpu_lib):
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 1))
    with pytest.raises(RuntimeError, match="shared"):
        clex.CanonicalBatch(model, (64, 64, 64), np.zeros((1, 64 ** 3), dtype=np.int8), [1000.0], [1])


def _stat(series):
    st = BasicStatisticsCalculator(confidence=0.95)(np.ascontiguousarray(series, dtype=np.float64))
    return st.mean, st.calculated_precision


@pytest.mark.parametrize("kind,T,n_passes", [("fcc_binary", 900.0, 8000), ("fcc_ternary", 1200.0, 4000)])
def test_canonical_statistics_match_reference_dynamics(gpu_lib, kind, T, n_passes):
    L = (8, 8, 8)
    N = 512
    ns = 2 if kind == "fcc_binary" else 3
    model = clex.ClexModel(kind, clex.make_eci(kind, 3))
    occ0 = clex.random_occupation(ns, N, np.random.default_rng(23))
    discard = n_passes // 5

    b = clex.CanonicalBatch(model, L, occ0[None, :], [T], [123456789])
    corr = b.corr()
    e_gpu = []
    done = 0
    while done < n_passes:
        m = min(2000, n_passes - done)
        out = b.run(m)
        d = out[:, :, :model.n_classes].copy()
        d[:, :, 0] = 0
        ic = corr[None, :, :] + np.cumsum(d, axis=0)
        corr = ic[-1]
        e_gpu.append(model.formation_per_supercell(ic)[:, 0] / N)
        done += m
    e_gpu = np.concatenate(e_gpu)[discard:]

    orc = OracleCE(L, ns, model.eci)
    e_ref, _ = orc.canonical_samples(occ0, T, 424242, n_passes)
    e_ref = e_ref[discard:]

    for name, (g, r) in {"E": (e_gpu, e_ref),
                         "C": (N * (e_gpu - e_gpu.mean()) ** 2 / (KB * T) ** 2,
                               N * (e_ref - e_ref.mean()) ** 2 / (KB * T) ** 2)}.items():
        (mg, pg), (mr, pr) = _stat(g), _stat(r)
        bound = 2.0 * np.hypot(pg, pr)
        assert np.isfinite(bound) and abs(mg - mr) <= bound, (name, mg, mr, pg, pr)
