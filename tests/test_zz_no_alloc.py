"""The allocation-free sweep entry point (mg_ce_sweep_noalloc) against the batch API.

Callers that cannot allocate device memory (their framework owns the pool, or
allocation is forbidden while a run is in progress) hand the library their own device
buffers and get the same coloured sweep, with the library's scratch in a fixed device
array.  This test allocates the caller's buffers with torch (the caller may allocate;
the entry point must not), calls the entry point twice in a row through the C-ABI, and
requires the occupations and per-pass outputs to equal those of mg_ce_batch_run on the
same inputs exactly (the sweeps are deterministic integer trajectories), in FP64 and
FP32 decision mode and at the 262,144-site limit.  Device free memory must not change
across the second call, and occupant codes out of range must be refused before any
sweep runs.
"""
import ctypes as C

import numpy as np
import pytest

from casmcode_monte_gb300 import _lib, clex

pytestmark = pytest.mark.gpu


def _call(Lb, model, L, n_chains, T, mu, seeds, d_occ, pass0, n_passes, d_out, precision, stream):
    return Lb.mg_ce_sweep_noalloc(model._h, L[0], L[1], L[2], n_chains, _lib.ptr(T, C.c_double),
                                  _lib.ptr(mu, C.c_double), _lib.ptr(seeds, C.c_uint64),
                                  C.c_void_p(d_occ.data_ptr()), pass0, n_passes,
                                  C.c_void_p(d_out.data_ptr()), precision, C.c_void_p(stream.cuda_stream))


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("kind,L,n_chains", [("fcc_binary", (16, 16, 16), 3), ("fcc_ternary", (12, 8, 10), 2),
                                             ("fcc_binary", (64, 64, 64), 2)])
def test_noalloc_sweep_matches_batch_two_calls(kind, L, n_chains, precision):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    Lb = _lib.lib()
    model = clex.ClexModel(kind, clex.make_eci(kind, 21))
    rng = np.random.default_rng(4)
    N = L[0] * L[1] * L[2]
    occ0 = np.stack([clex.random_occupation(model.n_species, N, rng) for _ in range(n_chains)])
    T = np.ascontiguousarray(np.linspace(500.0, 1500.0, n_chains))
    mu = np.ascontiguousarray(rng.uniform(-0.2, 0.2, size=(n_chains, model.n_species - 1)))
    seeds = np.ascontiguousarray(np.arange(7, 7 + n_chains, dtype=np.uint64))
    nslot = model.n_classes + 2

    ref = clex.ChainBatch(model, L, occ0, T, mu, seeds, precision="fp64" if precision == 0 else "fp32")
    d_occ = torch.from_numpy(occ0.copy()).cuda()
    stream = torch.cuda.current_stream()
    pass0 = 0
    for call, n_passes in enumerate((3, 4)):
        d_out = torch.full((n_passes, n_chains, nslot), -7, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = _call(Lb, model, L, n_chains, T, mu, seeds, d_occ, pass0, n_passes, d_out, precision, stream)
        _lib.check(rc)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        if call == 1:
            # the first call on a device may load the module (and with it the scratch array)
            assert free_after == free_before, (free_before, free_after)
        want = ref.run(n_passes)
        assert np.array_equal(d_out.cpu().numpy(), want)
        assert np.array_equal(d_occ.cpu().numpy(), ref.occupation())
        pass0 += n_passes
    ref.close()


def test_noalloc_rejects_oversized_inputs():
    torch = pytest.importorskip("torch")
    Lb = _lib.lib()
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 1))
    T = np.array([1000.0])
    mu = np.zeros((1, 1))
    seeds = np.array([1], dtype=np.uint64)
    dummy = torch.zeros(8, dtype=torch.int64, device="cuda")
    # 96^3 sites exceed the 262144-site scratch limit
    rc = Lb.mg_ce_sweep_noalloc(model._h, 96, 96, 96, 1, _lib.ptr(T, C.c_double), _lib.ptr(mu, C.c_double),
                                _lib.ptr(seeds, C.c_uint64), C.c_void_p(dummy.data_ptr()), 0, 1,
                                C.c_void_p(dummy.data_ptr()), 0, None)
    assert rc != 0
    assert b"262144" in Lb.mg_last_error()


@pytest.mark.parametrize("bad", [2, -1, 100])
def test_noalloc_refuses_bad_occupant_codes(bad):
    """A code outside [0, n_species) is found by the device check before any sweep: the call
    fails with a clear message and leaves occupations and outputs untouched."""
    torch = pytest.importorskip("torch")
    Lb = _lib.lib()
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 2))
    L = (16, 16, 16)
    rng = np.random.default_rng(9)
    occ0 = np.stack([clex.random_occupation(2, 16**3, rng) for _ in range(2)])
    occ0[1, 1234] = bad
    T = np.array([800.0, 1200.0])
    mu = np.zeros((2, 1))
    seeds = np.array([3, 4], dtype=np.uint64)
    d_occ = torch.from_numpy(occ0.copy()).cuda()
    d_out = torch.full((2, 2, model.n_classes + 2), -7, dtype=torch.int64, device="cuda")
    rc = _call(Lb, model, L, 2, T, mu, seeds, d_occ, 0, 2, d_out, 0, torch.cuda.current_stream())
    assert rc != 0
    assert b"occupant index out of range" in Lb.mg_last_error()
    torch.cuda.synchronize()
    assert np.array_equal(d_occ.cpu().numpy(), occ0)
    assert bool((d_out == -7).all())
