"""Edge cases of the GPU path: the largest supercell the sweep kernels hold in shared
memory, one too large (a clean error, the context stays usable), zero passes, and invalid
arguments (each a RuntimeError with the library's message)."""
import numpy as np
import pytest

from casmcode_monte_gb300 import clex

pytestmark = pytest.mark.gpu


def _model():
    return clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 2))


def test_largest_supercell_tracks_exact_correlations(gpu_lib):
    model = _model()
    L = (128, 128, 128)
    n = L[0] * L[1] * L[2]
    rng = np.random.default_rng(1)
    occ = np.stack([clex.random_occupation(2, n, rng) for _ in range(2)])
    b = clex.ChainBatch(model, L, occ, [800.0, 1600.0], np.zeros((2, 1)), [3, 4])
    corr0 = b.corr()
    out = b.run(3)
    s = clex.accumulate(model, corr0, out, np.zeros((2, 1)), n)
    assert np.array_equal(b.corr(), s.int_corr[-1])
    assert np.array_equal(b.occupation().sum(axis=1, dtype=np.int64), s.int_corr[-1][:, 1])
    assert np.all(out[:, :, 0] > 0)


def test_too_large_supercell_is_refused_cleanly(gpu_lib):
    model = _model()
    L = (256, 256, 256)
    occ = np.zeros((1, L[0] * L[1] * L[2]), dtype=np.int8)
    with pytest.raises(RuntimeError, match="does not fit in shared memory"):
        clex.ChainBatch(model, L, occ, [1000.0], np.zeros((1, 1)), [1])
    # the context is still usable
    small = clex.ChainBatch(model, (8, 8, 8), np.zeros((1, 512), dtype=np.int8), [1000.0], np.zeros((1, 1)), [1])
    assert small.run(2).shape == (2, 1, model.n_classes + 2)


def test_zero_passes_and_invalid_arguments(gpu_lib):
    model = _model()
    occ = clex.random_occupation(2, 512, np.random.default_rng(2))[None, :]
    b = clex.ChainBatch(model, (8, 8, 8), occ, [1000.0], np.zeros((1, 1)), [5])
    out = b.run(0)
    assert out.shape == (0, 1, model.n_classes + 2)
    assert np.array_equal(b.occupation(), occ)
    with pytest.raises(RuntimeError, match="invalid argument"):
        b.run(-1)
    with pytest.raises(RuntimeError, match="temperature must be > 0"):
        clex.ChainBatch(model, (8, 8, 8), occ, [0.0], np.zeros((1, 1)), [5])
    bad = occ.copy()
    bad[0, 7] = 2
    with pytest.raises(RuntimeError, match="occupant index out of range"):
        clex.ChainBatch(model, (8, 8, 8), bad, [1000.0], np.zeros((1, 1)), [5])
    with pytest.raises(RuntimeError, match=">= 4"):
        clex.ChainBatch(model, (3, 8, 8), occ[:, :192], [1000.0], np.zeros((1, 1)), [5])


@pytest.mark.parametrize("bad_value", [2, -1, 127])
def test_batch_occupant_check_on_device(gpu_lib, bad_value):
    """The creation check runs on the device after the copy: a bad code in the last chain's
    last site (and a negative one) is refused, and a batch created afterwards works."""
    model = _model()
    rng = np.random.default_rng(8)
    occ = np.stack([clex.random_occupation(2, 16**3, rng) for _ in range(3)])
    bad = occ.copy()
    bad[2, -1] = bad_value
    with pytest.raises(RuntimeError, match="occupant index out of range"):
        clex.ChainBatch(model, (16, 16, 16), bad, [900.0] * 3, np.zeros((3, 1)), [1, 2, 3])
    b = clex.ChainBatch(model, (16, 16, 16), occ, [900.0] * 3, np.zeros((3, 1)), [1, 2, 3])
    b.run(2)
    b.close()


def test_batch_block_cache_reuse(gpu_lib):
    """Closed batches leave their device block in the library's cache: a batch of the same shape
    created next takes it (device free memory unchanged), starts from its own inputs whatever the
    block held, and gives the trajectory of a batch on fresh memory; release_cached_memory frees
    the cached blocks."""
    import torch

    model = _model()
    rng = np.random.default_rng(9)
    L = (64, 64, 64)
    occ = np.stack([clex.random_occupation(2, 64**3, rng) for _ in range(8)])
    T, mu, seeds = np.linspace(400, 1600, 8), np.zeros((8, 1)), np.arange(1, 9, dtype=np.uint64)
    clex.release_cached_memory()
    torch.cuda.synchronize()
    a = clex.ChainBatch(model, L, occ, T, mu, seeds)
    ref = a.run(6)
    ref_occ = a.occupation()
    a.close()
    other = np.stack([clex.random_occupation(2, 64**3, rng) for _ in range(8)])
    for _ in range(3):
        x = clex.ChainBatch(model, L, other, T, mu, seeds)  # fills the block with other data
        x.run(3)
        x.close()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    b = clex.ChainBatch(model, L, occ, T, mu, seeds)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert np.array_equal(b.run(6), ref)
    assert np.array_equal(b.occupation(), ref_occ)
    b.close()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    clex.release_cached_memory()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] >= free1 + (2 << 20)  # the 8 x 64^3 block (2.2 MB)


def test_batch_corr_follows_occupation_changes(gpu_lib):
    """The initial correlation sums are computed when the batch is created; corr() must still
    follow every change of the occupations: after set_occupation (no pass run) and after runs
    it equals the sums of a fresh batch created on the same occupations."""
    model = _model()
    rng = np.random.default_rng(12)
    L = (16, 16, 16)
    occ = np.stack([clex.random_occupation(2, 16**3, rng) for _ in range(2)])
    other = np.stack([clex.random_occupation(2, 16**3, rng) for _ in range(2)])
    T, mu, seeds = [700.0, 1300.0], np.zeros((2, 1)), [5, 6]

    def fresh(o):
        f = clex.ChainBatch(model, L, o, T, mu, seeds)
        c = f.corr()
        f.close()
        return c

    b = clex.ChainBatch(model, L, occ, T, mu, seeds)
    assert np.array_equal(b.corr(), fresh(occ))
    b.set_occupation(other)
    assert np.array_equal(b.corr(), fresh(other))
    b.run(3)
    assert np.array_equal(b.corr(), fresh(b.occupation()))
    b.close()
