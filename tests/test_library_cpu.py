"""The C-ABI library on the CPU: it loads, exports every symbol of include/montegpu.h,
and its host entry points (mt19937_64 engine, statistics numerics) agree exactly with the
oracle.  No device computation is attempted here."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import casmcode_monte_gb300 as monte
from casmcode_monte_gb300 import _lib
from tests import oracle_lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    with open(os.path.join(ROOT, "include", "montegpu.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"\b(mg_[a-z0-9_]+)\s*\(", src)))


def test_header_and_binding_agree():
    assert set(_declared()) == set(_lib.SIGNATURES)


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (mg_[a-z0-9_]+)", out))
    for name in _declared():
        assert name in exported, name
        assert getattr(L, name) is not None
    assert L.mg_version() >= 100


def test_engine_matches_std_mt19937_64(oracle):
    e = monte.RandomNumberEngine()
    e.seed(2024)
    st = e.dump()
    assert st == oracle_lib.engine_state(2024)
    g = monte.RandomNumberGenerator(e)
    ints = [g.random_int(624) for _ in range(2000)]
    reals = [g.random_real(1.0) for _ in range(2000)]
    out_i = (C.c_long * 2000)()
    out_r = (C.c_double * 2000)()
    buf = C.create_string_buffer(16384)
    oracle.orc_rng_draws(st.encode(), 0, C.c_long(624), C.c_double(0.0), 2000, out_i, out_r, buf, 16384)
    assert ints == list(out_i)
    oracle.orc_rng_draws(buf.value, 1, C.c_long(0), C.c_double(1.0), 2000, out_i, out_r, buf, 16384)
    assert reals == list(out_r)
    assert e.dump() == buf.value.decode()


def test_engine_dump_load_roundtrip():
    """test_RandomNumberGeneratory.py:12-35 (the reference's own RNG tests)."""
    rng = monte.RandomNumberGenerator()
    for _ in range(10000):
        r = rng.random_int(9)
        assert 0 <= r <= 9
    e = monte.RandomNumberEngine()
    state = e.dump()
    rng = monte.RandomNumberGenerator(e)
    x = [rng.random_int(9) for _ in range(10)]
    e.load(state)
    y = [rng.random_int(9) for _ in range(10)]
    assert x == y
    e.load(state)
    x = [rng.random_real(9) for _ in range(10)]
    e.load(state)
    y = [rng.random_real(9) for _ in range(10)]
    assert x == y


def test_engine_int_draws_match(oracle):
    e = monte.RandomNumberEngine()
    e.seed_seq([1, 2, 3])
    st = e.dump()
    g = monte.RandomNumberGenerator(e)
    for mx in (1, 624, 262143, 2**40 + 7):
        got = [g.random_int(mx) for _ in range(500)]
        out_i = (C.c_long * 500)()
        out_r = (C.c_double * 500)()
        buf = C.create_string_buffer(16384)
        oracle.orc_rng_draws(st.encode(), 0, C.c_long(mx), C.c_double(0.0), 500, out_i, out_r, buf, 16384)
        assert got == list(out_i)
        st = buf.value.decode()
        assert e.dump() == st


def test_bad_engine_state_is_an_error():
    e = monte.RandomNumberEngine()
    with pytest.raises(RuntimeError, match="malformed"):
        e.load("not a state")


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_statistics_match_oracle(oracle, seed):
    rng = np.random.default_rng(seed)
    x = np.cumsum(rng.normal(size=800)) * 0.01 + 3.0
    w = rng.uniform(0.5, 2.0, size=800)
    from casmcode_monte_gb300 import sampling

    for conf in (0.9, 0.95):
        s = sampling.BasicStatisticsCalculator(confidence=conf)(x)
        m, p = C.c_double(), C.c_double()
        oracle.orc_basic_statistics(oracle_lib.p(x, C.c_double), 800, None, 0, C.c_double(conf), 1, 10000,
                                    C.byref(m), C.byref(p))
        assert (s.mean, s.calculated_precision) == (m.value, p.value)
    for method in (1, 2):
        s = sampling.BasicStatisticsCalculator(method=method, n_resamples=3000)(x, w)
        m, p = C.c_double(), C.c_double()
        oracle.orc_basic_statistics(oracle_lib.p(x, C.c_double), 800, oracle_lib.p(w, C.c_double), 800,
                                    C.c_double(0.95), method, 3000, C.byref(m), C.byref(p))
        assert (s.mean, s.calculated_precision) == (m.value, p.value)
    for prec in (0.001, 0.01, 0.1):
        r = sampling.default_equilibration_check(x, None, sampling.RequestedPrecision(abs=prec))
        ie, ne = C.c_int(), C.c_long()
        oracle.orc_equilibration_check(oracle_lib.p(x, C.c_double), 800, C.c_double(prec), C.byref(ie), C.byref(ne))
        assert (r.is_equilibrated, r.N_samples_for_equilibration) == (bool(ie.value), ne.value)
    assert _lib.lib().mg_approx_erf_inv(0.95) == oracle.orc_approx_erf_inv(C.c_double(0.95))
    oracle.orc_autocorrelation_factor.argtypes = [C.POINTER(C.c_double), C.c_long, C.c_double]
    assert sampling.autocorrelation_factor(x) == oracle.orc_autocorrelation_factor(oracle_lib.p(x, C.c_double), 800, 1.0)


def test_statistics_edge_cases():
    from casmcode_monte_gb300 import sampling

    flat = np.full(50, 2.5)
    r = sampling.default_equilibration_check(flat, None, sampling.RequestedPrecision(abs=1e-6))
    assert r.is_equilibrated and r.N_samples_for_equilibration == 0
    s = sampling.BasicStatisticsCalculator()(flat)
    assert s.mean == 2.5 and s.calculated_precision == 0.0
    with pytest.raises(RuntimeError, match="observations.size"):
        sampling.BasicStatisticsCalculator()(np.zeros(0))
    with pytest.raises(RuntimeError, match="observations.size"):
        sampling.default_equilibration_check(np.zeros(0), None, sampling.RequestedPrecision(abs=1.0))
    # no precision requested: equilibrated immediately
    r = sampling.default_equilibration_check(np.arange(5.0), None, sampling.RequestedPrecision())
    assert r.is_equilibrated and r.N_samples_for_equilibration == 0


@pytest.mark.parametrize("kind,L,layout", [("fcc_binary", (64, 64, 64), "word_pipelined"),
                                           ("fcc_binary", (16, 16, 8), "word_pipelined"),
                                           ("fcc_binary", (16, 8, 16), "word_pipelined"),
                                           ("fcc_binary", (20, 12, 10), "word"),
                                           ("fcc_binary", (8, 8, 8), "byte"), ("fcc_ternary", (16, 16, 16), "word"),
                                           ("fcc_ternary", (12, 12, 12), "byte"),
                                           ("fcc_binary", (13, 11, 7), "byte")])
def test_colouring_is_proper_host(kind, L, layout):
    """The sweep's colouring (host entry point, no device): no neighbour offset of the
    basis set joins two sites of one colour; the word layouts apply exactly where the
    four sites i0 + t*L0/4 of every row share a colour; the pipelined one uses a
    generated colouring whose late neighbours are those of the previous colour."""
    from casmcode_monte_gb300 import clex
    import casmcode_monte_gb300.clex.orbits as O
    from casmcode_monte_gb300.clex import codegen

    col, n, lay = clex.color_supercell(kind, L)
    assert lay == layout
    w = lay != "byte"
    assert col.min() == 0 and col.max() == n - 1
    col3 = col.reshape(L[2], L[1], L[0])
    for (di, dj, dk) in O.make_basis_set(kind).neighbour_offsets():
        shifted = np.roll(col3, shift=(-dk, -dj, -di), axis=(0, 1, 2))
        assert not np.any(shifted == col3)
    if w:
        Q = L[0] // 4
        assert np.array_equal(col3[:, :, :Q], col3[:, :, Q:2 * Q])
        assert np.array_equal(col3[:, :, :Q], col3[:, :, 3 * Q:])
    if lay == "word_pipelined":
        offs = O.make_basis_set(kind).neighbour_offsets()
        a, b, c = int(col3[0, 0, 1]), int(col3[0, 1, 0]), int(col3[1, 0, 0])
        assert (a, b, c, n) in codegen.PIPELINE_COLOURINGS
        late = codegen.late_offsets(offs, (a, b, c, n))
        assert len(late) == 2
        for (di, dj, dk) in offs:
            shifted = np.roll(col3, shift=(-dk, -dj, -di), axis=(0, 1, 2))
            is_late = (di, dj, dk) in [tuple(o) for o in late]
            assert np.all((shifted == (col3 - 1) % n) == is_late)
