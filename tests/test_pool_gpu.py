"""Chain pool (persistent kernel, one CTA per chain, mixed supercell shapes)."""
import numpy as np
import pytest

from casmcode_monte_gb300 import clex
from tests.oracle_lib import OracleCE

pytestmark = pytest.mark.gpu


def _chains(model, shapes, seed=1):
    rng = np.random.default_rng(seed)
    out = []
    for c, L in enumerate(shapes):
        n = L[0] * L[1] * L[2]
        occ = rng.integers(0, model.n_species, size=n).astype(np.int8)
        T = float(rng.uniform(300.0, 2000.0))
        mu = rng.uniform(-0.3, 0.3, size=model.n_species - 1)
        out.append((L, occ, T, mu, int(rng.integers(1, 2**63)), 1000 + c))
    return out


@pytest.mark.parametrize("kind", ["fcc_binary", "fcc_ternary"])
def test_pool_matches_oracle_mixed_shapes(gpu_lib, kind):
    model = clex.ClexModel(kind, clex.make_eci(kind, 5))
    shapes = [(8, 8, 8), (12, 12, 12), (16, 8, 12), (6, 9, 7), (8, 8, 8)]
    chains = _chains(model, shapes)
    pool = clex.ChainPool(model, arena_bytes=1 << 20, max_chains=8)
    slots = [pool.add(L, occ, T, mu, seed, cid) for (L, occ, T, mu, seed, cid) in chains]
    corr0 = [pool.corr(s) for s in slots]
    n_passes = 5
    out = pool.run(slots, n_passes)
    for i, ((L, occ, T, mu, seed, cid), s) in enumerate(zip(chains, slots)):
        col, nc = pool.colors(s)
        orc = OracleCE(L, model.n_species, model.eci)
        occ_ref, corr_ref, nacc_ref = orc.colored_sweep(occ, T, mu, seed, cid, col, nc, 0, n_passes,
                                                        model.n_classes)
        assert np.array_equal(pool.occupation(s), occ_ref.astype(np.int8)), (i, L)
        d = out[i, :, : model.n_classes].copy()
        d[:, 0] = 0
        ic = corr0[i][None, :] + np.cumsum(d, axis=0)
        assert np.array_equal(ic, corr_ref), (i, L)
        assert np.array_equal(out[i, :, 0], nacc_ref)
        assert np.array_equal(pool.corr(s), corr_ref[-1])


def test_pool_results_independent_of_batching(gpu_lib):
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 2))
    shapes = [(8, 8, 8), (12, 8, 8), (16, 16, 16), (10, 10, 10)]
    chains = _chains(model, shapes, seed=3)
    a = clex.ChainPool(model, 1 << 20, 8)
    b = clex.ChainPool(model, 1 << 20, 8)
    sa = [a.add(*c[:1], c[1], c[2], c[3], c[4], c[5]) for c in chains]
    sb = [b.add(*c[:1], c[1], c[2], c[3], c[4], c[5]) for c in chains]
    a.run(sa, 6)  # all together, 6 passes
    b.run(sb[:2], 2)  # uneven batching: subsets and splits
    b.run(sb, 3)
    b.run(sb[2:], 3)
    b.run(sb[:2], 1)
    for x, y in zip(sa, sb):
        assert np.array_equal(a.occupation(x), b.occupation(y))


def test_pool_admission_by_footprint(gpu_lib):
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 2))
    pool = clex.ChainPool(model, arena_bytes=3 * 4096, max_chains=8)
    occ = np.zeros(16 * 16 * 16, dtype=np.int8)
    s0 = pool.add((16, 16, 16), occ, 1000.0, [0.0], 1, 0)
    s1 = pool.add((16, 16, 16), occ, 1000.0, [0.0], 2, 1)
    s2 = pool.add((16, 16, 16), occ, 1000.0, [0.0], 3, 2)
    with pytest.raises(clex.PoolFull):
        pool.add((16, 16, 16), occ, 1000.0, [0.0], 4, 3)
    pool.remove(s1)
    s3 = pool.add((16, 16, 16), occ, 1000.0, [0.0], 4, 3)
    assert s3 == s1
    assert pool.info()["arena_free_bytes"] == 0
    pool.run([s0, s2, s3], 2)


@pytest.mark.parametrize("kind,L", [("fcc_binary", (64, 64, 64)), ("fcc_binary", (72, 72, 72)),
                                    ("fcc_ternary", (64, 64, 60)), ("fcc_binary", (48, 48, 48)),
                                    ("fcc_binary", (32, 32, 32))])
def test_pool_large_chains_match_batch(gpu_lib, kind, L):
    """Chains too large for one CTA run in the pool's cluster classes; same trajectory as the
    (oracle-validated) batch path."""
    model = clex.ClexModel(kind, clex.make_eci(kind, 8))
    chains = _chains(model, [L, (16, 16, 16)], seed=9)
    pool = clex.ChainPool(model, arena_bytes=2 * L[0] * L[1] * L[2] + (1 << 16), max_chains=4)
    slots = [pool.add(c[0], c[1], c[2], c[3], c[4], c[5]) for c in chains]
    out = pool.run(slots, 3)
    out2 = pool.run(slots, 2)
    for i, c in enumerate(chains):
        b = clex.ChainBatch(model, c[0], c[1][None, :], [c[2]], c[3][None, :], [c[4]], chain_ids=[c[5]])
        ref = b.run(3)
        ref2 = b.run(2)
        assert np.array_equal(out[i], ref[:, 0, :])
        assert np.array_equal(out2[i], ref2[:, 0, :])
        assert np.array_equal(pool.occupation(slots[i]), b.occupation()[0])
        b.close()


def test_pool_device_series_and_check_match_host(gpu_lib):
    from casmcode_monte_gb300 import sampling

    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 3))
    chains = _chains(model, [(12, 12, 12), (64, 64, 64), (8, 8, 8)], seed=11)
    pool = clex.ChainPool(model, arena_bytes=(1 << 19), max_chains=4)
    pool.enable_series(400)
    slots = [pool.add(c[0], c[1], c[2], c[3], c[4], c[5]) for c in chains]
    corr0 = [pool.corr(s) for s in slots]
    outs = [pool.run(slots, 150), pool.run(slots, 150)]
    for i, (c, s) in enumerate(zip(chains, slots)):
        n = int(np.prod(c[0]))
        o = np.concatenate([x[i] for x in outs])[:, None, :]
        smp = clex.accumulate(model, corr0[i][None, :], o, np.asarray(c[3])[None, :], n)
        ser = pool.series(s)
        assert ser.size == 300
        assert np.array_equal(ser, smp.potential_energy[:, 0])
    for prec in (1e-4, 1e-3, 5e-3):
        res = pool.check(slots, prec)
        for i, s in enumerate(slots):
            ser = pool.series(s)
            eq = sampling.default_equilibration_check(ser, None, sampling.RequestedPrecision(abs=prec))
            assert bool(res[i, 0]) == eq.is_equilibrated
            assert int(res[i, 1]) == eq.N_samples_for_equilibration
            if eq.is_equilibrated and eq.N_samples_for_equilibration < ser.size:
                st = sampling.BasicStatisticsCalculator()(ser[eq.N_samples_for_equilibration:])
                assert res[i, 3] == st.mean and res[i, 4] == st.calculated_precision
                assert bool(res[i, 5]) == (st.calculated_precision < prec)


def test_pool_ternary_word_layout_matches_oracle(gpu_lib):
    """Ternary chains whose L0 is a multiple of four take the pool's ternary word-layout
    kernels (one CTA, and a cluster for the largest), the others the byte layout; every
    trajectory equals the oracle's coloured sweep."""
    model = clex.ClexModel("fcc_ternary", clex.make_eci("fcc_ternary", 8))
    shapes = [(16, 16, 16), (32, 16, 16), (24, 12, 12), (48, 48, 48), (12, 12, 12)]
    chains = _chains(model, shapes, seed=7)
    pool = clex.ChainPool(model, arena_bytes=1 << 21, max_chains=8)
    slots = [pool.add(L, occ, T, mu, seed, cid) for (L, occ, T, mu, seed, cid) in chains]
    corr0 = [pool.corr(s) for s in slots]
    n_passes = 4
    out = pool.run(slots, n_passes)
    for i, ((L, occ, T, mu, seed, cid), s) in enumerate(zip(chains, slots)):
        col, nc = pool.colors(s)
        orc = OracleCE(L, 3, model.eci)
        occ_ref, corr_ref, nacc_ref = orc.colored_sweep(occ, T, mu, seed, cid, col, nc, 0, n_passes,
                                                        model.n_classes)
        assert np.array_equal(pool.occupation(s), occ_ref.astype(np.int8)), (i, L)
        d = out[i, :, : model.n_classes].copy()
        d[:, 0] = 0
        assert np.array_equal(corr0[i][None, :] + np.cumsum(d, axis=0), corr_ref), (i, L)
        assert np.array_equal(out[i, :, 0], nacc_ref), (i, L)


@pytest.mark.parametrize("kind", ["fcc_binary", "fcc_ternary"])
def test_pool_add_many_equals_single_adds(gpu_lib, kind):
    """Bulk admission gives the slots, trajectories, outputs and device series of one add per
    chain, with a freed slot and a non-multiple-of-16 arena gap in the way."""
    model = clex.ClexModel(kind, clex.make_eci(kind, 6))
    shapes = [(8, 8, 8), (5, 7, 9), (16, 8, 12), (12, 12, 12), (8, 8, 8), (16, 16, 16)]
    chains = _chains(model, shapes, seed=11)
    filler = np.zeros(6 * 9 * 7, dtype=np.int8)
    pools, slots, outs = [], [], []
    for bulk in (False, True):
        pool = clex.ChainPool(model, arena_bytes=1 << 20, max_chains=12)
        pool.enable_series(8)
        f = [pool.add((6, 9, 7), filler, 900.0, np.zeros(model.n_species - 1), 9, 90 + k) for k in range(3)]
        pool.remove(f[1])
        if bulk:
            s = pool.add_many([c[0] for c in chains], [c[1] for c in chains], [c[2] for c in chains],
                              np.stack([c[3] for c in chains]), [c[4] for c in chains], [c[5] for c in chains])
        else:
            s = [pool.add(*c) for c in chains]
        pools.append(pool)
        slots.append(s)
        outs.append(pool.run(s, 4))
        assert pool.last_launches() >= 2  # at least one sweep kernel and the series kernel
    assert slots[0] == slots[1] and slots[0][0] == 1
    assert np.array_equal(outs[0], outs[1])
    for x in slots[0]:
        assert np.array_equal(pools[0].occupation(x), pools[1].occupation(x))
        assert np.array_equal(pools[0].series(x), pools[1].series(x))
    assert pools[0].info() == pools[1].info()
    for p in pools:
        p.close()


def test_pool_add_many_all_or_none(gpu_lib):
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 2))
    pool = clex.ChainPool(model, arena_bytes=3 * 4096, max_chains=8)
    occ = np.zeros(16 * 16 * 16, dtype=np.int8)
    before = pool.info()
    # the fourth chain does not fit: nothing is admitted
    with pytest.raises(clex.PoolFull):
        pool.add_many([(16, 16, 16)] * 4, [occ] * 4, [1000.0] * 4, np.zeros((4, 1)), [1, 2, 3, 4], [0, 1, 2, 3])
    assert pool.info() == before
    # an occupant code out of range in the last chain: nothing is admitted
    bad = occ.copy()
    bad[7] = 2
    with pytest.raises(RuntimeError, match="occupant index out of range"):
        pool.add_many([(16, 16, 16)] * 2, [occ, bad], [1000.0] * 2, np.zeros((2, 1)), [1, 2], [0, 1])
    assert pool.info() == before
    s = pool.add_many([(16, 16, 16)] * 3, [occ] * 3, [1000.0] * 3, np.zeros((3, 1)), [1, 2, 3], [0, 1, 2])
    assert s == [0, 1, 2] and pool.info()["arena_free_bytes"] == 0
    assert pool.add_many([], [], [], np.zeros((0, 1)), [], []) == []
    pool.run(s, 2)
    pool.close()
