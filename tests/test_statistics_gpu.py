"""Coloured-sweep statistics against the reference's own dynamics.

The coloured sweep visits sites in a different order from the reference's random-site
loop, so trajectories differ but the equilibrium ensemble is the same.  For binary and
ternary FCC cluster expansions (8^3 supercell) the GPU's per-pass potential energy and
composition series are compared with a run of the reference's semi-grand canonical
dynamics in the oracle (OccLocation proposals, metropolis_acceptance, std::mt19937_64):
<E>, <x>, the heat capacity C = N Var(e) / (kB T)^2 and the susceptibility
chi = N Var(x) / (kB T) agree within twice the combined 95 % error bars, each error bar
the reference's autocorrelation-corrected precision of the mean
(BasicStatistics.cc:24-188) of the series (for C and chi, of the per-pass squared
deviations from the mean).
"""
import numpy as np
import pytest

from casmcode_monte_gb300 import clex
from casmcode_monte_gb300.sampling import BasicStatisticsCalculator
from tests.oracle_lib import OracleCE

pytestmark = pytest.mark.gpu

KB = 8.6173303e-05
L = (8, 8, 8)
N = 512


def _stat(series):
    st = BasicStatisticsCalculator(confidence=0.95)(np.ascontiguousarray(series, dtype=np.float64))
    return st.mean, st.calculated_precision


def _quantities(e, x, T):
    out = {"E": _stat(e)}
    for i in range(x.shape[1]):
        out[f"x{i}"] = _stat(x[:, i])
    out["C"] = _stat(N * (e - e.mean()) ** 2 / (KB * T) ** 2)
    for i in range(x.shape[1]):
        out[f"chi{i}"] = _stat(N * (x[:, i] - x[:, i].mean()) ** 2 / (KB * T))
    return out


@pytest.mark.parametrize("kind,T,mu,n_passes", [("fcc_binary", 900.0, [0.02], 12000),
                                                ("fcc_binary", 1500.0, [-0.05], 8000),
                                                ("fcc_ternary", 1200.0, [0.02, -0.01], 5000)])
def test_coloured_statistics_match_reference_dynamics(gpu_lib, kind, T, mu, n_passes):
    ns = 2 if kind == "fcc_binary" else 3
    model = clex.ClexModel(kind, clex.make_eci(kind, 3))
    rng = np.random.default_rng(17)
    occ0 = clex.random_occupation(ns, N, rng)
    mu = np.asarray(mu, dtype=float)
    discard = n_passes // 5

    b = clex.ChainBatch(model, L, occ0[None, :], [T], mu[None, :], [987654321])
    corr = b.corr()
    e_gpu, x_gpu = [], []
    done = 0
    while done < n_passes:
        m = min(2000, n_passes - done)
        s = clex.accumulate(model, corr, b.run(m), mu[None, :], N)
        corr = s.int_corr[-1]
        e_gpu.append(s.potential_energy[:, 0])
        x_gpu.append(s.param_composition[:, 0, :])
        done += m
    e_gpu = np.concatenate(e_gpu)[discard:]
    x_gpu = np.concatenate(x_gpu)[discard:]

    orc = OracleCE(L, ns, model.eci)
    e_ref, x_ref, _ = orc.sgc_samples(occ0, T, mu, 424242, n_passes)
    e_ref, x_ref = e_ref[discard:], x_ref[discard:]

    qg, qr = _quantities(e_gpu, x_gpu, T), _quantities(e_ref, x_ref, T)
    for k in qg:
        (mg, pg), (mr, pr) = qg[k], qr[k]
        bound = 2.0 * np.hypot(pg, pr)
        assert np.isfinite(bound) and abs(mg - mr) <= bound, (k, mg, mr, pg, pr)


def test_bench_config_statistics_match_reference_dynamics(gpu_lib):
    """The benchmark's own chains (binary FCC 64^3, its ECIs, occupations and temperatures:
    543 K for chain 1, 1514 K for chain 5; mu = 0) swept on the GPU against the reference's
    semi-grand canonical dynamics in the oracle from the same starts: <E>, <x>, C and chi
    within twice the combined 95 % error bars.  Both dynamics equilibrate within a few passes
    at these temperatures; the first 30 passes are discarded."""
    import bench
    from tests import oracle_lib

    eci, occ, T, mu, seeds = bench.make_inputs(0)
    n = 64**3
    model = clex.ClexModel("fcc_binary", eci)
    chains = [1, 5]
    n_ref, n_gpu, discard = 160, 1000, 30
    with oracle_lib.oracle_pool(len(chains)) as pool:
        pending = oracle_lib.sgc_samples_async(pool, [((64, 64, 64), 2, eci, occ[c], float(T[c]), mu[c], 777 + c,
                                                       n_ref) for c in chains])
        b = clex.ChainBatch(model, (64, 64, 64), occ[chains], T[chains], mu[chains], seeds[chains], chain_ids=chains)
        corr = b.corr()
        s = clex.accumulate(model, corr, b.run(n_gpu), mu[chains], n)
        b.close()
        refs = pending.get(timeout=3600)
    for k, c in enumerate(chains):
        e_gpu, x_gpu = s.potential_energy[discard:, k], s.param_composition[discard:, k, :]
        e_ref, x_ref = refs[k][0][discard:], refs[k][1][discard:]
        Tc = float(T[c])

        def quantities(e, x):
            return {"E": _stat(e), "x": _stat(x[:, 0]),
                    "C": _stat(n * (e - e.mean()) ** 2 / (KB * Tc) ** 2),
                    "chi": _stat(n * (x[:, 0] - x[:, 0].mean()) ** 2 / (KB * Tc))}

        qg, qr = quantities(e_gpu, x_gpu), quantities(e_ref, x_ref)
        for q in qg:
            (mg, pg), (mr, pr) = qg[q], qr[q]
            bound = 2.0 * np.hypot(pg, pr)
            assert np.isfinite(bound) and abs(mg - mr) <= bound, (c, q, mg, mr, pg, pr)
