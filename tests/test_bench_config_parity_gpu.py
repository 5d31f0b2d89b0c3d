"""The benchmark's own configuration against the oracle, bit for bit.

The headline workload is binary FCC 64^3 (262,144 sites), the benchmark's ECIs, occupations,
temperatures and Philox seeds (``bench.make_inputs``), swept by the warp-specialised
word-layout kernel with the generated colouring (4i + 5j + 14k) mod 16.  On GB300 eight
chains run on 12-CTA clusters (row slabs of 341 or 342 rows); long runs rotate the chains over
seven 16-CTA clusters and one 12-CTA cluster.  Each of these launch geometries must give the
oracle's restated coloured sweep exactly: occupations, integer correlation sums after every
pass and accepted counts, in FP64 decision mode.  The oracle runs in a spawn process pool
while the GPU works.
"""
import numpy as np
import pytest

import bench
from casmcode_monte_gb300 import clex
from tests import oracle_lib

pytestmark = pytest.mark.gpu

L3 = (64, 64, 64)


def _bench_inputs():
    eci, occ, T, mu, seeds = bench.make_inputs(0)
    return clex.ClexModel("fcc_binary", eci), eci, occ, T, mu, seeds


def _check(b, model, mu, ids, corr0, out, pending):
    s = clex.accumulate(model, corr0, out, mu[ids], b.n_sites)
    got = b.occupation()
    results = pending.get(timeout=1800)
    for k, (occ_ref, corr_ref, nacc_ref) in enumerate(results):
        assert np.array_equal(got[k], occ_ref.astype(np.int8)), f"chain {ids[k]}: occupation"
        assert np.array_equal(s.int_corr[:, k, :], corr_ref), f"chain {ids[k]}: correlations"
        assert np.array_equal(s.n_accept[:, k], nacc_ref), f"chain {ids[k]}: accepted counts"


@pytest.mark.parametrize("ctas", [12, 16])
def test_fcc64_bench_chains_match_oracle(gpu_lib, ctas):
    """Chains 0 (300 K) and 7 (2000 K) of the benchmark, 3 passes, at 12 CTAs per chain (the
    unrotated choice for eight chains) and 16 (the fast clusters of a rotated run)."""
    model, eci, occ, T, mu, seeds = _bench_inputs()
    ids = [0, 7]
    b = clex.ChainBatch(model, L3, occ[ids], T[ids], mu[ids], seeds[ids], chain_ids=ids, ctas_per_chain=ctas)
    assert b.layout == "word_specialised" and b.ctas_per_chain == ctas and b.n_colors == 16
    n_passes = 3
    colors = b.colors()
    with oracle_lib.oracle_pool(len(ids)) as pool:
        pending = oracle_lib.colored_sweeps(pool, [
            (L3, 2, eci, occ[c], float(T[c]), mu[c], int(seeds[c]), c, colors, b.n_colors, 0, n_passes,
             model.n_classes) for c in ids])
        corr0 = b.corr()
        out = b.run(n_passes)
        _check(b, model, mu, ids, corr0, out, pending)
    b.close()


def test_fcc64_rotated_bench_run_matches_oracle(gpu_lib):
    """All eight chains of the benchmark through one rotated run of 16 passes (forced: too
    short to pay, but every chain visits the 12-CTA slot between sweeps on 16-CTA clusters)."""
    import torch

    model, eci, occ, T, mu, seeds = _bench_inputs()
    b = clex.ChainBatch(model, L3, occ, T, mu, seeds)
    if b.rotation()["ctas_fast"] == 0:
        pytest.skip("this GPU has no rotation plan for 8 chains of 64^3")
    if torch.cuda.get_device_properties(0).multi_processor_count == 152:
        assert b.ctas_per_chain == 12 and b.rotation()["ctas_fast"] == 16
    b.set_rotation("always")
    n_passes = 16
    colors = b.colors()
    ids = list(range(8))
    with oracle_lib.oracle_pool(8) as pool:
        pending = oracle_lib.colored_sweeps(pool, [
            (L3, 2, eci, occ[c], float(T[c]), mu[c], int(seeds[c]), c, colors, b.n_colors, 0, n_passes,
             model.n_classes) for c in ids])
        corr0 = b.corr()
        out = b.run(n_passes)
        assert b.last_launches() > 8, b.last_launches()
        _check(b, model, mu, ids, corr0, out, pending)
    b.close()
