"""Word layout of the ternary Chebyshev basis (ce_sweep_tquad_kernel) against the byte
layout and the oracle.

Both layouts propose the same sites with the same per-site Philox blocks and take the same
FP32 decisions (the word layout's energy sums come from byte-parallel monomial counts, exact
integers equal to the per-site feature sums), so occupations and every per-pass output slot
(accepted proposals, correlation changes, FP64 re-decisions, FP32 flips) must be identical for
every CTA split, in FP64 and FP32 decision mode, and equal the oracle's coloured sweep."""
import numpy as np
import pytest

from casmcode_monte_gb300 import clex
from tests.oracle_lib import OracleCE

pytestmark = pytest.mark.gpu


def _setup(L, n_chains, seed):
    model = clex.ClexModel("fcc_ternary", clex.make_eci("fcc_ternary", seed))
    rng = np.random.default_rng(seed + 50)
    N = L[0] * L[1] * L[2]
    occ = np.stack([clex.random_occupation(3, N, rng) for _ in range(n_chains)])
    T = np.linspace(400.0, 2000.0, n_chains)
    mu = rng.uniform(-0.2, 0.2, size=(n_chains, 2))
    seeds = (np.arange(n_chains, dtype=np.uint64) + np.uint64(3)) * np.uint64(2654435761)
    return model, occ, T, mu, seeds


SHAPES = [((16, 16, 16), 1), ((16, 16, 16), 4), ((16, 16, 8), 3), ((32, 16, 16), 8), ((16, 32, 16), 7),
          ((32, 32, 32), 12)]


@pytest.mark.parametrize("L,S", SHAPES)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_ternary_word_equals_byte_layout(gpu_lib, L, S, precision):
    model, occ, T, mu, seeds = _setup(L, 3, seed=L[0] + S)
    w = clex.ChainBatch(model, L, occ, T, mu, seeds, precision=precision, ctas_per_chain=S)
    assert w.layout == "word" and w.ctas_per_chain == S
    b = clex.ChainBatch(model, L, occ, T, mu, seeds, precision=precision, ctas_per_chain=S)
    b.set_layout("byte")
    assert b.layout == "byte"
    for n in (4, 3):
        assert np.array_equal(w.run(n), b.run(n)), n
        assert np.array_equal(w.occupation(), b.occupation()), n
    assert np.array_equal(w.corr(), b.corr())
    w.close()
    b.close()


@pytest.mark.parametrize("L,S", [((16, 16, 16), 2), ((16, 16, 8), 3)])
def test_ternary_word_layout_matches_oracle(gpu_lib, L, S):
    model, occ, T, mu, seeds = _setup(L, 2, seed=31)
    w = clex.ChainBatch(model, L, occ, T, mu, seeds, ctas_per_chain=S)
    assert w.layout == "word"
    corr0 = w.corr()
    n_passes = 4
    s = clex.accumulate(model, corr0, w.run(n_passes), mu, w.n_sites)
    got = w.occupation()
    orc = OracleCE(L, 3, model.eci)
    for c in range(2):
        occ_ref, corr_ref, nacc_ref = orc.colored_sweep(occ[c], T[c], mu[c], int(seeds[c]), c, w.colors(),
                                                        w.n_colors, 0, n_passes, model.n_classes)
        assert np.array_equal(got[c], occ_ref.astype(np.int8))
        assert np.array_equal(s.int_corr[:, c, :], corr_ref)
        assert np.array_equal(s.n_accept[:, c], nacc_ref)
    w.close()


def test_ternary_word_full_size_tracks_correlations(gpu_lib):
    """8 chains of 64^3 (the batched ternary shape of the serving jobs' largest class): word
    and byte layouts agree over 5 passes, and the tracked correlations equal a recompute."""
    L = (64, 64, 64)
    model, occ, T, mu, seeds = _setup(L, 8, seed=2)
    w = clex.ChainBatch(model, L, occ, T, mu, seeds)
    assert w.layout == "word"
    b = clex.ChainBatch(model, L, occ, T, mu, seeds, ctas_per_chain=w.ctas_per_chain)
    b.set_layout("byte")
    corr0 = w.corr()
    ow, ob = w.run(5), b.run(5)
    assert np.array_equal(ow, ob)
    assert np.array_equal(w.occupation(), b.occupation())
    s = clex.accumulate(model, corr0, ow, mu, w.n_sites)
    assert np.array_equal(w.corr(), s.int_corr[-1])
    w.close()
    b.close()


def test_sweep_probe_reports_layout_and_rate(gpu_lib):
    """The sweep probe of the workloads module (used for the ternary ncu captures) runs a
    small batch on the layout asked for and reports a positive rate."""
    from casmcode_monte_gb300 import workloads

    for layout in ("auto", "byte", "grid"):
        r = workloads.run_sweep("fcc_ternary", L=16, n_chains=2, n_passes=2, layout=layout)
        assert r["layout"] == ("word" if layout == "auto" else layout)
        assert r["site_attempts_per_s"] > 0 and len(r["ms"]) == 3
