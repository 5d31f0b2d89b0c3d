"""FP32 energy changes with FP64 energies: the decision rule pinned to the oracle, and the
precision study (ternary FCC, FP32 decisions against FP64 decisions) at a reduced size.

In FP32 decision mode the kernel decides from the FP32 energy change and ``ex2.approx``; a
decision inside the proven ambiguity band is also taken in FP64 and a disagreement counted
(``n_flipped``), the FP32 decision standing.  Outside the band the two decisions are equal by
construction, so until the first counted flip an FP32-mode trajectory must be the oracle's
FP64 coloured sweep exactly; after a flip the trajectories part, and only the statistics
must agree.
"""
import numpy as np
import pytest

from casmcode_monte_gb300 import clex, workloads
from tests.oracle_lib import OracleCE

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,L,S", [("fcc_binary", (16, 16, 16), 2), ("fcc_binary", (32, 32, 32), 4),
                                      ("fcc_ternary", (12, 12, 12), 1), ("fcc_ternary", (16, 16, 16), 2)])
def test_fp32_decisions_follow_fp64_oracle_until_a_flip(gpu_lib, kind, L, S):
    ns = 2 if kind == "fcc_binary" else 3
    model = clex.ClexModel(kind, clex.make_eci(kind, 11))
    rng = np.random.default_rng(5)
    N = L[0] * L[1] * L[2]
    n_chains = 3
    occ = np.stack([clex.random_occupation(ns, N, rng) for _ in range(n_chains)])
    T = np.array([400.0, 900.0, 1800.0])
    mu = rng.uniform(-0.1, 0.1, size=(n_chains, ns - 1))
    seeds = np.array([11, 12, 13], dtype=np.uint64)
    b = clex.ChainBatch(model, L, occ, T, mu, seeds, precision="fp32", ctas_per_chain=S)
    corr0 = b.corr()
    n_passes = 6
    s = clex.accumulate(model, corr0, b.run(n_passes), mu, b.n_sites)
    got = b.occupation()
    orc = OracleCE(L, ns, model.eci)
    for c in range(n_chains):
        occ_ref, corr_ref, nacc_ref = orc.colored_sweep(occ[c], T[c], mu[c], int(seeds[c]), c, b.colors(),
                                                        b.n_colors, 0, n_passes, model.n_classes)
        flips = s.n_flipped[:, c]
        # passes up to (not including) the first pass that counted a flip equal the oracle
        clean = int(np.argmax(flips > 0)) if flips.any() else n_passes
        assert np.array_equal(s.int_corr[:clean, c, :], corr_ref[:clean])
        assert np.array_equal(s.n_accept[:clean, c], nacc_ref[:clean])
        if clean == n_passes:
            assert np.array_equal(got[c], occ_ref.astype(np.int8))
        # FP64 re-decisions happen (the band is not empty) but flips are rare
        assert int(flips.sum()) <= int(s.n_exact[:, c].sum())


def test_precision_study_reduced_size(gpu_lib):
    """The precision configuration (ternary FCC, 600 K, FP64 recompute every 50 passes) at
    32^3 and 2000 passes: FP32-decision <E>, <x_B>, <x_C> and the heat capacity lie within
    twice the combined 95 % error bars of the FP64-decision run from the same start; the
    tracked integer correlations equal every full recompute; the flipped decisions are
    counted and rare."""
    r = workloads.run_precision(L=32, n_passes=2000, T=600.0, recompute_every=50, discard=400)
    for prec in ("fp64", "fp32"):
        assert r[prec]["recompute_mismatches"] == 0, prec
        assert r[prec]["fp64_redecisions"] > 0, prec
    assert r["fp64"]["fp32_flipped_decisions"] == 0
    n_decisions = 32**3 * 2000
    assert 0 <= r["fp32"]["fp32_flipped_decisions"] <= 1e-6 * n_decisions
    for k in ("E_per_site", "x_B", "x_C", "Cv"):
        d = r["fp32_minus_fp64"][k]
        assert np.isfinite(d["combined_error_bar"])
        assert abs(d["diff"]) <= 2.0 * d["combined_error_bar"] + 1e-12, (k, d)
