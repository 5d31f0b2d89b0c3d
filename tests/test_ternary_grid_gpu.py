"""Grid sweep of the ternary word layout (ce_sweep_tgrid_kernel) against the cluster word
layout and the oracle.

The grid sweep keeps each chain's padded word window in global memory, shares every colour's
word list between G CTAs (one cooperative launch, all CTAs resident) and separates the colours
with a grid barrier per chain.  The words, neighbours, Philox blocks and decisions are those of
the cluster kernel, so occupations and every per-pass output slot must be identical, in FP64 and
FP32 decision mode, and equal the oracle's coloured sweep; the single 96^3 chain of the
precision workload is checked against the oracle for two passes."""
import numpy as np
import pytest

from casmcode_monte_gb300 import clex
from tests import oracle_lib
from tests.oracle_lib import OracleCE

pytestmark = pytest.mark.gpu


def _setup(L, n_chains, seed):
    model = clex.ClexModel("fcc_ternary", clex.make_eci("fcc_ternary", seed))
    rng = np.random.default_rng(seed + 70)
    N = L[0] * L[1] * L[2]
    occ = np.stack([clex.random_occupation(3, N, rng) for _ in range(n_chains)])
    T = np.linspace(500.0, 1800.0, n_chains)
    mu = rng.uniform(-0.2, 0.2, size=(n_chains, 2))
    seeds = (np.arange(n_chains, dtype=np.uint64) + np.uint64(11)) * np.uint64(2654435761)
    return model, occ, T, mu, seeds


@pytest.mark.parametrize("L,n_chains,G", [((16, 16, 16), 2, 0), ((16, 16, 8), 3, 20), ((32, 16, 16), 1, 0),
                                          ((32, 32, 32), 4, 3), ((32, 32, 32), 2, 37)])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_grid_equals_cluster_word_layout(gpu_lib, L, n_chains, G, precision):
    """G = 0: set_layout("grid") with the resident CTAs shared between the chains; G <= 16:
    created on the cluster layout with G CTAs, then switched; G > 16 (more than a cluster
    holds): created on the grid sweep directly."""
    model, occ, T, mu, seeds = _setup(L, n_chains, seed=L[0] + n_chains)
    w = clex.ChainBatch(model, L, occ, T, mu, seeds, precision=precision)
    assert w.layout == "word"
    g = clex.ChainBatch(model, L, occ, T, mu, seeds, precision=precision, ctas_per_chain=G)
    if G <= 16:
        g.set_layout("grid")
    assert g.layout == "grid" and (G == 0 or g.ctas_per_chain == G)
    for n in (3, 4):
        assert np.array_equal(g.run(n), w.run(n)), n
        assert np.array_equal(g.occupation(), w.occupation()), n
    assert np.array_equal(g.corr(), w.corr())
    g.close()
    w.close()


def test_grid_matches_oracle(gpu_lib):
    L = (16, 16, 16)
    model, occ, T, mu, seeds = _setup(L, 2, seed=5)
    g = clex.ChainBatch(model, L, occ, T, mu, seeds)
    g.set_layout("grid")
    corr0 = g.corr()
    n_passes = 4
    s = clex.accumulate(model, corr0, g.run(n_passes), mu, g.n_sites)
    got = g.occupation()
    orc = OracleCE(L, 3, model.eci)
    for c in range(2):
        occ_ref, corr_ref, nacc_ref = orc.colored_sweep(occ[c], T[c], mu[c], int(seeds[c]), c, g.colors(),
                                                        g.n_colors, 0, n_passes, model.n_classes)
        assert np.array_equal(got[c], occ_ref.astype(np.int8))
        assert np.array_equal(s.int_corr[:, c, :], corr_ref)
        assert np.array_equal(s.n_accept[:, c], nacc_ref)
    g.close()


def test_grid_precision_chain_96_matches_oracle(gpu_lib):
    """The precision workload's chain: ternary 96^3 at 600 K, FP64 decisions, two passes on
    every resident CTA, against the oracle's coloured sweep (run in a spawn process while the
    GPU works), then the tracked correlations against a recompute after three more passes."""
    L = (96, 96, 96)
    model = clex.ClexModel("fcc_ternary", clex.make_eci("fcc_ternary", 4))
    rng = np.random.default_rng(4)
    occ = clex.random_occupation(3, 96**3, rng)[None, :]
    T, mu, seeds = np.array([600.0]), np.zeros((1, 2)), np.array([4 * 7919 + 1], dtype=np.uint64)
    g = clex.ChainBatch(model, L, occ, T, mu, seeds)
    g.set_layout("grid")
    assert g.layout == "grid" and g.ctas_per_chain > 16
    n_passes = 2
    colors = g.colors()
    with oracle_lib.oracle_pool(1) as pool:
        pending = oracle_lib.colored_sweeps(pool, [(L, 3, model.eci, occ[0], 600.0, mu[0], int(seeds[0]), 0, colors,
                                                    g.n_colors, 0, n_passes, model.n_classes)])
        corr0 = g.corr()
        s = clex.accumulate(model, corr0, g.run(n_passes), mu, g.n_sites)
        got = g.occupation()
        occ_ref, corr_ref, nacc_ref = pending.get(timeout=1800)[0]
    assert np.array_equal(got[0], occ_ref.astype(np.int8))
    assert np.array_equal(s.int_corr[:, 0, :], corr_ref)
    assert np.array_equal(s.n_accept[:, 0], nacc_ref)
    d = g.run(3)
    s2 = clex.accumulate(model, corr_ref[-1][None, :], d, mu, g.n_sites)
    assert np.array_equal(s2.int_corr[-1], g.corr())
    g.close()


def test_grid_layout_refusals(gpu_lib):
    Lb = (16, 16, 16)
    bm = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 1))
    rng = np.random.default_rng(1)
    b = clex.ChainBatch(bm, Lb, clex.random_occupation(2, 16**3, rng)[None, :], [900.0], [[0.0]], [3])
    with pytest.raises(RuntimeError, match="ternary basis"):
        b.set_layout("grid")
    b.close()
    # 40 chains x 4 CTAs are more CTAs than one cooperative launch can hold on GB300
    model, occ, T, mu, seeds = _setup(Lb, 40, seed=9)
    g = clex.ChainBatch(model, Lb, occ, T, mu, seeds, ctas_per_chain=4)
    with pytest.raises(RuntimeError, match="resident"):
        g.set_layout("grid")
    assert g.layout == "word"
    g.run(1)
    g.close()


def test_large_ternary_chain_chooses_grid(gpu_lib):
    """A ternary 128^3 chain: its word window does not fit in the shared memory of a 16-CTA
    cluster, so the batch chooses the grid sweep by itself; a batch held on a 16-CTA cluster
    (the byte layout) gives the same outputs and occupations."""
    L = (128, 128, 128)
    model, occ, T, mu, seeds = _setup(L, 1, seed=12)
    g = clex.ChainBatch(model, L, occ, T, mu, seeds)
    assert g.layout == "grid" and g.ctas_per_chain > 16
    w = clex.ChainBatch(model, L, occ, T, mu, seeds, ctas_per_chain=16)
    assert w.layout in ("word", "byte")
    assert np.array_equal(g.run(2), w.run(2))
    assert np.array_equal(g.occupation(), w.occupation())
    g.close()
    w.close()


def test_many_large_ternary_chains_stay_on_one_cta_each(gpu_lib):
    """152 chains of 48^3 (1728 words per CTA and colour on one CTA each) would get one CTA each
    from the grid sweep too: the batch keeps the one-CTA word layout."""
    L = (48, 48, 48)
    model, occ, T, mu, seeds = _setup(L, 152, seed=3)
    b = clex.ChainBatch(model, L, occ, T, mu, seeds)
    assert b.layout == "word" and b.ctas_per_chain == 1
    b.close()
