"""Rotation over two cluster sizes: 8 chains of FCC 64^3, seven on 16-CTA clusters beside one
on a 12-CTA cluster, the chains taking turns on the 12-CTA cluster within each run.

A trajectory is a pure function of (seed, chain, initial state and pass index), so a rotated
run must give the same occupations and per-pass outputs as the unrotated one (all chains on
12-CTA clusters, whose sweeps the oracle tests pin), whatever the sub-segment pass counts.
Successive runs re-measure the time ratio and so split their passes differently.
"""
import numpy as np
import pytest

from casmcode_monte_gb300 import clex

pytestmark = pytest.mark.gpu


def _inputs(n_chains=8, L=64, seed=31):
    rng = np.random.default_rng(seed)
    occ = np.stack([clex.random_occupation(2, L**3, rng) for _ in range(n_chains)])
    T = np.linspace(300.0, 2000.0, n_chains)
    mu = rng.uniform(-0.1, 0.1, size=(n_chains, 1))
    seeds = np.arange(101, 101 + n_chains, dtype=np.uint64)
    return occ, T, mu, seeds


def test_rotated_runs_equal_unrotated():
    torch = pytest.importorskip("torch")
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 5))
    occ, T, mu, seeds = _inputs()
    rot = clex.ChainBatch(model, (64, 64, 64), occ, T, mu, seeds)
    rot.set_rotation("always")  # rotate every run that has a plan, also where it does not pay
    plain = clex.ChainBatch(model, (64, 64, 64), occ, T, mu, seeds)
    plain.set_rotation(False)
    assert plain.rotation()["ctas_fast"] == 0
    info = rot.rotation()
    if torch.cuda.get_device_properties(0).multi_processor_count == 152:
        # GB300: seven 16-CTA clusters fit at once, eight 12-CTA ones
        assert rot.ctas_per_chain == 12 and info["ctas_fast"] == 16, info
    if info["ctas_fast"] == 0:
        pytest.skip("this GPU has no rotation plan for 8 chains of 64^3")
    for n in (40, 5, 37, 64):  # 5 < 2 x 8 chains: unrotated
        a = rot.run(n)
        assert rot.last_launches() == (1 if n < 16 else rot.last_launches()) and (n < 16 or rot.last_launches() > 8)
        b = plain.run(n)
        assert plain.last_launches() == 1
        assert np.array_equal(a, b), n
        assert np.array_equal(rot.occupation(), plain.occupation()), n
    assert 0.6 <= rot.rotation()["ratio"] <= 1.0
    assert rot.rotation()["ctas_fast"] == 16 or torch.cuda.get_device_properties(0).multi_processor_count != 152
    assert np.array_equal(rot.corr(), plain.corr())
    rot.close()
    plain.close()


def test_short_runs_stay_unrotated():
    """A run too short for the rotated schedule to beat one unrotated launch (20 passes of 8
    chains: the extra launches cost more than the faster clusters gain) runs unrotated; a long
    one (200 passes) rotates.  Both give the unrotated trajectory."""
    torch = pytest.importorskip("torch")
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 5))
    occ, T, mu, seeds = _inputs(seed=34)
    auto = clex.ChainBatch(model, (64, 64, 64), occ, T, mu, seeds)
    if auto.rotation()["ctas_fast"] == 0:
        pytest.skip("this GPU has no rotation plan for 8 chains of 64^3")
    plain = clex.ChainBatch(model, (64, 64, 64), occ, T, mu, seeds)
    plain.set_rotation(False)
    assert np.array_equal(auto.run(20), plain.run(20))
    assert auto.last_launches() == 1
    assert np.array_equal(auto.run(200), plain.run(200))
    if torch.cuda.get_device_properties(0).multi_processor_count == 152:
        assert auto.last_launches() > 8
    assert np.array_equal(auto.run(20), plain.run(20))
    assert auto.last_launches() == 1
    assert np.array_equal(auto.occupation(), plain.occupation())
    auto.close()
    plain.close()


def test_rotation_off_and_on_again():
    pytest.importorskip("torch")
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 5))
    occ, T, mu, seeds = _inputs(seed=32)
    b = clex.ChainBatch(model, (64, 64, 64), occ, T, mu, seeds)
    fast = b.rotation()["ctas_fast"]
    b.set_rotation(False)
    assert b.rotation() == {"ctas_fast": 0, "ratio": 0.0}
    b.set_rotation(True)
    assert b.rotation()["ctas_fast"] == fast
    # an explicit CTA count never rotates
    c = clex.ChainBatch(model, (64, 64, 64), occ, T, mu, seeds, ctas_per_chain=12)
    assert c.rotation()["ctas_fast"] == 0
    b.close()
    c.close()


def test_autotune_with_rotation_keeps_results():
    """The autotuner also times the rotated occupancy choice; whatever it keeps, the batch
    continues exactly as an untuned, unrotated one."""
    torch = pytest.importorskip("torch")
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 6))
    occ, T, mu, seeds = _inputs(seed=33)
    tuned = clex.ChainBatch(model, (64, 64, 64), occ, T, mu, seeds)
    plain = clex.ChainBatch(model, (64, 64, 64), occ, T, mu, seeds)
    plain.set_rotation(False)
    assert np.array_equal(tuned.run(3), plain.run(3))
    choice = tuned.autotune(probe_passes=3)
    assert choice["ms_per_pass"] > 0.0 and tuned.ctas_per_chain == choice["ctas_per_chain"]
    rot = tuned.rotation()
    if rot["ctas_fast"] > 0:
        assert choice["layout"] == "word_specialised"
    assert np.array_equal(tuned.occupation(), plain.occupation())
    assert np.array_equal(tuned.run(40), plain.run(40))
    assert np.array_equal(tuned.occupation(), plain.occupation())
    tuned.close()
    plain.close()
