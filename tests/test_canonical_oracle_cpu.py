"""The oracle's canonical restatements (test infrastructure): the coloured canonical sweep
conserves composition and its per-pass correlation sums equal a recompute of the final
state; the reference-dynamics canonical run keeps composition and ends at the energy its
tracked series reports."""
import numpy as np

from casmcode_monte_gb300 import clex
from tests.oracle_lib import OracleCE


def test_oracle_canonical_sweep_conserves_composition():
    L = (8, 8, 8)
    model = clex.ClexModel("fcc_ternary", clex.make_eci("fcc_ternary", 4))
    occ = clex.random_occupation(3, 512, np.random.default_rng(3))
    col, nc, _ = clex.color_supercell("fcc_ternary", L)
    orc = OracleCE(L, 3, model.eci)
    occ2, corr, nacc = orc.canonical_sweep(occ, 900.0, 11, 0, col, nc, col, nc, 0, 5, model.n_classes)
    assert np.array_equal(np.bincount(occ2, minlength=3), np.bincount(occ, minlength=3))
    assert np.array_equal(corr[-1], orc.int_corr(occ2, model.n_classes))
    assert nacc.sum() > 0 and not np.array_equal(occ2, occ)


def test_oracle_canonical_samples_track_energy():
    L = (8, 8, 8)
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 4))
    occ = clex.random_occupation(2, 512, np.random.default_rng(5))
    orc = OracleCE(L, 2, model.eci)
    e, nacc = orc.canonical_samples(occ, 1200.0, 99, 20)
    assert e.shape == (20,) and np.isfinite(e).all() and nacc > 0
    assert abs(e[0] - orc.formation(occ) / 512) < 0.5
