"""Word layouts (four sites per 32-bit word, generic and pipelined) of the binary sweep
against the byte layout and the oracle.

The layouts implement the same coloured sweep (same colouring, same Philox counters,
same FP32/FP64 decision arithmetic), so occupations and every per-pass output slot must
be identical, in FP64 and in FP32 decision mode, for every CTA split.
"""
import numpy as np
import pytest

from casmcode_monte_gb300 import clex
from tests.oracle_lib import OracleCE

pytestmark = pytest.mark.gpu


def _setup(L, n_chains, seed):
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", seed))
    rng = np.random.default_rng(seed + 100)
    N = L[0] * L[1] * L[2]
    occ = np.stack([clex.random_occupation(2, N, rng) for _ in range(n_chains)])
    T = np.linspace(300.0, 2000.0, n_chains)
    mu = rng.uniform(-0.3, 0.3, size=(n_chains, 1))
    seeds = (np.arange(n_chains, dtype=np.uint64) + np.uint64(7)) * np.uint64(2654435761)
    return model, occ, T, mu, seeds


def test_layout_selection(gpu_lib):
    model, occ, T, mu, seeds = _setup((16, 16, 16), 1, 1)
    assert clex.ChainBatch(model, (16, 16, 16), occ, T, mu, seeds).layout == "word_specialised"
    m20, occ20, T20, mu20, s20 = _setup((20, 12, 10), 1, 1)
    b20 = clex.ChainBatch(m20, (20, 12, 10), occ20, T20, mu20, s20)
    assert b20.layout == "word"
    with pytest.raises(RuntimeError):
        b20.set_layout("word_pipelined")
    model8, occ8, T8, mu8, seeds8 = _setup((8, 8, 8), 1, 1)
    b8 = clex.ChainBatch(model8, (8, 8, 8), occ8, T8, mu8, seeds8)
    assert b8.layout == "byte"
    with pytest.raises(RuntimeError):
        b8.set_layout("word")
    tern = clex.ClexModel("fcc_ternary", clex.make_eci("fcc_ternary", 1))
    occt = clex.random_occupation(3, 16**3, np.random.default_rng(1))[None, :]
    bt = clex.ChainBatch(tern, (16, 16, 16), occt, [900.0], np.zeros((1, 2)), [5])
    assert bt.layout == "word"  # the ternary basis has a word layout (no pipelined form)
    with pytest.raises(RuntimeError):
        bt.set_layout("word_pipelined")


WORD_SHAPES = [((16, 16, 16), 1), ((16, 16, 16), 2), ((16, 16, 8), 3), ((32, 16, 16), 8), ((20, 12, 10), 5),
               ((16, 32, 16), 7), ((24, 24, 24), 12)]


@pytest.mark.parametrize("L,S", WORD_SHAPES)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_word_equals_byte_layout(gpu_lib, L, S, precision):
    n_chains = 3
    model, occ, T, mu, seeds = _setup(L, n_chains, seed=L[0] + S)
    auto = clex.ChainBatch(model, L, occ, T, mu, seeds, precision=precision, ctas_per_chain=S)
    assert auto.layout in ("word", "word_pipelined", "word_specialised")
    layouts = ["byte", "word"]
    if auto.layout in ("word_pipelined", "word_specialised"):
        layouts.append("word_pipelined")
    if auto.layout == "word_specialised":
        layouts.append("word_specialised")
    batches = []
    for lay in layouts:
        b = clex.ChainBatch(model, L, occ, T, mu, seeds, precision=precision, ctas_per_chain=S)
        b.set_layout(lay)
        assert b.layout == lay and b.ctas_per_chain == S
        batches.append(b)
    for n in (5, 3):
        outs = [b.run(n) for b in batches]
        occs = [b.occupation() for b in batches]
        for o, oc in zip(outs[1:], occs[1:]):
            assert np.array_equal(o, outs[0])
            assert np.array_equal(oc, occs[0])
    for b in batches[1:]:
        assert np.array_equal(b.corr(), batches[0].corr())


@pytest.mark.parametrize("L,S", [((16, 16, 16), 4), ((20, 12, 10), 1), ((16, 16, 8), 3), ((16, 32, 16), 7)])
def test_word_layout_matches_oracle(gpu_lib, L, S):
    """Row slabs that split planes between CTAs (16 x 8 rows over 3 CTAs, 32 x 16 over 7)
    and ones that do not give the oracle's trajectory."""
    n_chains = 2
    model, occ, T, mu, seeds = _setup(L, n_chains, seed=21)
    b = clex.ChainBatch(model, L, occ, T, mu, seeds, ctas_per_chain=S)
    assert b.layout in ("word", "word_pipelined", "word_specialised")
    corr0 = b.corr()
    n_passes = 4
    out = b.run(n_passes)
    s = clex.accumulate(model, corr0, out, mu, b.n_sites)
    occ_gpu = b.occupation()
    orc = OracleCE(L, 2, model.eci)
    for c in range(n_chains):
        occ_ref, corr_ref, nacc_ref = orc.colored_sweep(occ[c], T[c], mu[c], int(seeds[c]), c, b.colors(),
                                                        b.n_colors, 0, n_passes, model.n_classes)
        assert np.array_equal(occ_gpu[c], occ_ref.astype(np.int8))
        assert np.array_equal(s.int_corr[:, c, :], corr_ref)
        assert np.array_equal(s.n_accept[:, c], nacc_ref)


def test_word_layout_full_size(gpu_lib):
    """64^3, 8 temperatures (the benchmark's shape and CTA choice): both layouts agree
    over 10 passes in FP32 decision mode, and tracked correlations equal a recompute."""
    L = (64, 64, 64)
    model, occ, T, _, seeds = _setup(L, 8, seed=3)
    mu = np.zeros((8, 1))
    bw = clex.ChainBatch(model, L, occ, T, mu, seeds, precision="fp32")
    assert bw.layout == "word_specialised"
    bb = clex.ChainBatch(model, L, occ, T, mu, seeds, precision="fp32", ctas_per_chain=bw.ctas_per_chain)
    bb.set_layout("byte")
    bg = clex.ChainBatch(model, L, occ, T, mu, seeds, precision="fp32", ctas_per_chain=bw.ctas_per_chain)
    bg.set_layout("word")
    bp = clex.ChainBatch(model, L, occ, T, mu, seeds, precision="fp32", ctas_per_chain=bw.ctas_per_chain)
    bp.set_layout("word_pipelined")
    corr0 = bw.corr()
    ow, ob, og, op = bw.run(10), bb.run(10), bg.run(10), bp.run(10)
    assert np.array_equal(ow, ob) and np.array_equal(og, ob) and np.array_equal(op, ob)
    assert np.array_equal(bw.occupation(), bb.occupation())
    assert np.array_equal(bg.occupation(), bb.occupation())
    assert np.array_equal(bp.occupation(), bb.occupation())
    s = clex.accumulate(model, corr0, ow, mu, bw.n_sites)
    assert np.array_equal(bw.corr(), s.int_corr[-1])


def test_autotune_keeps_results(gpu_lib):
    """The autotuner times layouts and CTA counts on the batch's own chains but restores
    them: a tuned batch continues exactly as an untuned one."""
    L = (32, 32, 32)
    model, occ, T, mu, seeds = _setup(L, 4, seed=9)
    tuned = clex.ChainBatch(model, L, occ, T, mu, seeds)
    plain = clex.ChainBatch(model, L, occ, T, mu, seeds)
    o1, o2 = tuned.run(3), plain.run(3)
    choice = tuned.autotune(probe_passes=2)
    assert choice["layout"] in ("byte", "word", "word_pipelined", "word_specialised")
    assert tuned.layout == choice["layout"] and tuned.ctas_per_chain == choice["ctas_per_chain"]
    assert np.array_equal(tuned.occupation(), plain.occupation())
    assert np.array_equal(tuned.run(4), plain.run(4))
    assert np.array_equal(tuned.occupation(), plain.occupation())
