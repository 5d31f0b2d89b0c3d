"""Rejection-free (N-fold way) dynamics on the GPU: an event selector for the loop of
methods/nfold.hh, single-site flips chosen with probability proportional to their
Metropolis rates, residence times -ln(u) / R.

* the integer correlation sums the kernel tracks equal a full recompute, and the total rate
  it keeps in its tree of sums equals the oracle's sum of min(1, exp(-beta dE)) over the
  final state's sites (FP32 rates: within 1e-4 relative);
* time-weighted averages of the potential energy agree with the reference's Metropolis
  dynamics (oracle) within twice the combined 95 % error bars (BasicStatistics.cc:24-188);
* bases and sizes it does not take are refused.
"""
import numpy as np
import pytest

from casmcode_monte_gb300 import clex
from casmcode_monte_gb300.sampling import BasicStatisticsCalculator
from tests.oracle_lib import OracleCE

pytestmark = pytest.mark.gpu

KB = 8.6173303e-05


@pytest.mark.parametrize("L,small", [((8, 8, 12), True), ((24, 24, 24), False)])
def test_nfold_tracks_correlations_and_total_rate(gpu_lib, L, small):
    N = L[0] * L[1] * L[2]
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 2))
    rng = np.random.default_rng(4)
    occ = np.stack([clex.random_occupation(2, N, rng) for _ in range(2)])
    T = np.array([900.0, 1600.0])
    mu = np.array([[0.0], [0.03]])
    b = clex.NfoldBatch(model, L, occ, T, mu, [11, 12])
    assert (b.chains_per_sm, b.threads) == ((4, 128) if small else (1, 512))
    assert np.array_equal(b.corr(), b.corr(recompute=True))
    out = b.run(6 if small else 1)
    assert (out[:, :, 0] > 0).all()
    assert np.array_equal(b.corr(), b.corr(recompute=True))
    final = b.occupation()
    orc = OracleCE(L, 2, model.eci)
    for c in range(2):
        o = final[c].astype(np.int32)
        dE = np.array([orc.delta_e(o, l, 1 - int(o[l]), mu[c]) for l in range(N)])
        R = np.minimum(1.0, np.exp(-dE / (KB * T[c]))).sum()
        assert abs(out[-1, c, 1] - R) <= 1e-4 * R, (c, out[-1, c, 1], R)
        assert not np.array_equal(final[c], occ[c])


@pytest.mark.parametrize("T,mu", [(1500.0, 0.02), (900.0, -0.01)])
def test_nfold_time_averages_match_metropolis(gpu_lib, T, mu):
    L = (8, 8, 8)
    N = 512
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 3))
    occ0 = clex.random_occupation(2, N, np.random.default_rng(17))
    n_passes = 3000
    b = clex.NfoldBatch(model, L, occ0[None, :], [T], [[mu]], [2024])
    out = np.concatenate([b.run(1000) for _ in range(n_passes // 1000)], axis=0)[:, 0, :]
    t = out[:, 0]
    cbar = out[:, 2:] / t[:, None]  # time-averaged correlation sums of each pass
    e_pass = (model.formation_per_supercell(cbar) - mu * cbar[:, 1]) / N
    e_pass, t = e_pass[n_passes // 5:], t[n_passes // 5:]
    st = BasicStatisticsCalculator(confidence=0.95)(np.ascontiguousarray(e_pass))
    mean_gpu = float(np.sum(e_pass * t) / np.sum(t))

    e_ref, _, _ = OracleCE(L, 2, model.eci).sgc_samples(occ0, T, np.array([mu]), 99, n_passes)
    e_ref = e_ref[n_passes // 5:]
    sr = BasicStatisticsCalculator(confidence=0.95)(np.ascontiguousarray(e_ref))
    bound = 2.0 * np.hypot(st.calculated_precision, sr.calculated_precision)
    assert np.isfinite(bound) and abs(mean_gpu - sr.mean) <= bound, (mean_gpu, sr.mean, bound)


def test_nfold_refuses_ternary_and_large_supercells(gpu_lib):
    tern = clex.ClexModel("fcc_ternary", clex.make_eci("fcc_ternary", 1))
    with pytest.raises(RuntimeError, match="binary"):
        clex.NfoldBatch(tern, (8, 8, 8), np.zeros((1, 512), dtype=np.int8), [1000.0], [[0.0, 0.0]], [1])
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 1))
    with pytest.raises(RuntimeError, match="32768"):
        clex.NfoldBatch(model, (40, 40, 40), np.zeros((1, 40 ** 3), dtype=np.int8), [1000.0], [[0.0]], [1])
