"""ctypes access to the CPU oracle (oracle/build/liboracle.so) -- test infrastructure only."""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PATH = os.path.join(ROOT, "oracle", "build", "liboracle.so")

_lib = None


class OrcCCParams(C.Structure):
    _fields_ = [
        ("has_min_count", C.c_int), ("has_min_sample", C.c_int), ("has_max_count", C.c_int),
        ("has_max_sample", C.c_int), ("min_count", C.c_long), ("min_sample", C.c_long),
        ("max_count", C.c_long), ("max_sample", C.c_long), ("log_spacing", C.c_int),
        ("check_begin", C.c_long), ("check_period", C.c_long), ("check_base", C.c_double),
        ("check_shift", C.c_double), ("check_period_max", C.c_long), ("confidence", C.c_double),
        ("n_req", C.c_int), ("req_sampler", C.c_int * 4), ("req_component", C.c_int * 4),
        ("req_abs_flag", C.c_int * 4), ("req_abs", C.c_double * 4), ("req_rel_flag", C.c_int * 4),
        ("req_rel", C.c_double * 4),
    ]


class OrcRunOut(C.Structure):
    _fields_ = [
        ("n_pass", C.c_long), ("n_accept", C.c_longlong), ("n_reject", C.c_longlong), ("n_samples", C.c_long),
        ("is_complete", C.c_int), ("all_equilibrated", C.c_int), ("all_converged", C.c_int),
        ("n_checks", C.c_long), ("N_samples_for_all_to_equilibrate", C.c_long),
        ("N_samples_for_statistics", C.c_long), ("mean", C.c_double * 4),
        ("calculated_precision", C.c_double * 4), ("is_converged", C.c_int * 4),
    ]


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(PATH):
            subprocess.run(["make", "-C", os.path.join(ROOT, "oracle")], check=True, capture_output=True)
        L = C.CDLL(PATH)
        dp, lp, ip = C.POINTER(C.c_double), C.POINTER(C.c_long), C.POINTER(C.c_int)
        L.orc_mt19937_64_10000th.restype = C.c_ulonglong
        L.orc_rng_draws.argtypes = [C.c_char_p, C.c_int, C.c_long, C.c_double, C.c_long, lp, dp, C.c_char_p, C.c_long]
        L.orc_engine_seed.argtypes = [C.c_ulonglong, C.c_char_p, C.c_long]
        L.orc_ce_sgc_samples.restype = C.c_longlong
        L.orc_ce_sgc_samples.argtypes = [C.c_void_p, ip, C.c_double, dp, C.c_int, C.c_ulonglong, C.c_long, dp, dp]
        L.orc_ce_sgc_run.restype = C.c_longlong
        L.orc_ce_sgc_run.argtypes = [C.c_void_p, ip, C.c_double, dp, C.c_int, C.c_char_p, C.c_long, dp, dp,
                                     C.POINTER(C.c_longlong), ip, ip, C.c_char_p, C.c_long]
        L.orc_sgc_proposals.argtypes = [C.c_long, C.c_int, ip, C.c_ulonglong, C.c_long, C.c_int, lp, ip]
        L.orc_ising_run.argtypes = [C.c_long, C.c_long, C.c_double, C.c_int, C.c_double, C.c_double, ip,
                                    C.POINTER(OrcCCParams), C.c_int, C.c_char_p, dp, C.c_long,
                                    C.POINTER(OrcRunOut), C.c_char_p, C.c_long]
        L.orc_ising_delta.argtypes = [C.c_long, C.c_long, C.c_double, C.c_int, ip, C.c_long, C.c_int, C.c_double]
        L.orc_ising_formation.argtypes = [C.c_long, C.c_long, C.c_double, C.c_int, ip]
        L.orc_equilibration_check.argtypes = [dp, C.c_long, C.c_double, ip, lp]
        L.orc_basic_statistics.argtypes = [dp, C.c_long, dp, C.c_long, C.c_double, C.c_long, C.c_long, dp, dp]
        L.orc_autocorrelation_factor.argtypes = [dp, C.c_long, C.c_double]
        L.orc_approx_erf_inv.argtypes = [C.c_double]
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint), C.POINTER(C.c_uint), C.POINTER(C.c_uint)]
        L.orc_ce_n_classes_for.argtypes = [C.c_int]
        L.orc_ce_class_info.argtypes = [C.c_int, ip, lp, lp]
        L.orc_ising_delta.restype = C.c_double
        L.orc_ising_formation.restype = C.c_double
        L.orc_autocorrelation_factor.restype = C.c_double
        L.orc_approx_erf_inv.restype = C.c_double
        L.orc_ce_create.restype = C.c_void_p
        L.orc_ce_create.argtypes = [C.c_long, C.c_long, C.c_long, C.c_int, C.POINTER(C.c_double), C.c_int]
        L.orc_ce_destroy.argtypes = [C.c_void_p]
        L.orc_ce_delta_e.restype = C.c_double
        L.orc_ce_delta_e.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_long, C.c_int, C.POINTER(C.c_double), C.c_int]
        L.orc_ce_formation.restype = C.c_double
        L.orc_ce_formation.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
        L.orc_ce_int_corr.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_longlong)]
        L.orc_ce_colored_sweep.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_double, C.POINTER(C.c_double), C.c_int,
                                           C.c_ulonglong, C.c_uint, C.POINTER(C.c_int), C.c_int, C.c_long, C.c_long,
                                           C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
        L.orc_ce_canonical_sweep.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_double, C.c_ulonglong, C.c_uint,
                                             C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int), C.c_int,
                                             C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_long, C.c_long,
                                             C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
        L.orc_ce_canonical_samples.restype = C.c_longlong
        L.orc_ce_canonical_samples.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_double, C.c_ulonglong, C.c_long,
                                               C.POINTER(C.c_double)]
        L.orc_ce_nfold_run.restype = C.c_longlong
        L.orc_ce_nfold_run.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_double, C.POINTER(C.c_double), C.c_int,
                                       C.c_ulonglong, C.c_longlong, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_ce_random_site_run.restype = C.c_longlong
        L.orc_ce_random_site_run.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_double, C.POINTER(C.c_double), C.c_int,
                                             C.c_ulonglong, C.c_longlong, C.POINTER(C.c_double)]
        _lib = L
    return _lib


def p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def engine_state(seed: int) -> str:
    L = load()
    buf = C.create_string_buffer(16384)
    assert L.orc_engine_seed(seed, buf, len(buf)) == 0
    return buf.value.decode()


def make_cc_params(min_sample=None, max_sample=None, min_count=None, max_count=None, check_begin=100,
                   check_period=100, log_spacing=False, reqs=(), confidence=0.95):
    """reqs: list of (sampler index (0 formation, 1 param_composition, 2 potential), abs)."""
    P = OrcCCParams()
    P.has_min_sample = int(min_sample is not None)
    P.min_sample = min_sample or 0
    P.has_max_sample = int(max_sample is not None)
    P.max_sample = max_sample or 0
    P.has_min_count = int(min_count is not None)
    P.min_count = min_count or 0
    P.has_max_count = int(max_count is not None)
    P.max_count = max_count or 0
    P.log_spacing = int(log_spacing)
    P.check_begin, P.check_period = check_begin, check_period
    P.check_base, P.check_shift, P.check_period_max = 10.0, 2.0, 10000
    P.confidence = confidence
    P.n_req = len(reqs)
    for i, (s, a) in enumerate(reqs):
        P.req_sampler[i] = s
        P.req_component[i] = 0
        P.req_abs_flag[i] = 1
        P.req_abs[i] = a
    return P


def ising_run(rows, cols, J, use_nlist, T, mu, occ, params, sample_period, seed_state, max_samples=200000):
    L = load()
    occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int32).copy())
    samples = np.zeros((3, max_samples), dtype=np.float64)
    out = OrcRunOut()
    st = C.create_string_buffer(16384)
    rc = L.orc_ising_run(rows, cols, J, int(use_nlist), T,
                         mu, p(occ, C.c_int), C.byref(params), sample_period,
                         seed_state.encode(), p(samples, C.c_double), max_samples, C.byref(out), st,
                         len(st))
    assert rc == 0, rc
    n = out.n_samples
    return {"occ": occ, "formation_energy": samples[0, :n].copy(), "param_composition": samples[1, :n].copy(),
            "potential_energy": samples[2, :n].copy(), "out": out, "engine": st.value.decode()}


class OracleCE:
    """Oracle cluster-expansion supercell."""

    def __init__(self, L, n_species, eci):
        self.L = L
        self.n = L[0] * L[1] * L[2]
        self.n_species = n_species
        self.eci = np.ascontiguousarray(np.asarray(eci, dtype=np.float64))
        lib = load()
        self.h = lib.orc_ce_create(L[0], L[1], L[2], n_species, p(self.eci, C.c_double), self.eci.size)
        assert self.h, "oracle CE construction failed (class count mismatch?)"

    def __del__(self):
        if getattr(self, "h", None):
            load().orc_ce_destroy(self.h)
            self.h = None

    def delta_e(self, occ, l, new, mu):
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int32))
        mu = np.ascontiguousarray(np.asarray(mu, dtype=np.float64))
        return load().orc_ce_delta_e(self.h, p(occ, C.c_int), l, new, p(mu, C.c_double), mu.size)

    def formation(self, occ):
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int32))
        return load().orc_ce_formation(self.h, p(occ, C.c_int))

    def int_corr(self, occ, n_classes):
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int32))
        out = np.zeros(n_classes, dtype=np.int64)
        load().orc_ce_int_corr(self.h, p(occ, C.c_int), p(out, C.c_longlong))
        return out

    def colored_sweep(self, occ, T, mu, seed, chain, colors, n_colors, pass0, n_passes, n_classes):
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int32).copy())
        mu = np.ascontiguousarray(np.asarray(mu, dtype=np.float64))
        colors = np.ascontiguousarray(np.asarray(colors, dtype=np.int32))
        corr = np.zeros((n_passes, n_classes), dtype=np.int64)
        nacc = np.zeros(n_passes, dtype=np.int64)
        load().orc_ce_colored_sweep(self.h, p(occ, C.c_int), T, p(mu, C.c_double), mu.size, C.c_ulonglong(seed),
                                    C.c_uint(chain), p(colors, C.c_int), n_colors, pass0, n_passes,
                                    p(corr, C.c_longlong), p(nacc, C.c_longlong))
        return occ, corr, nacc

    def canonical_sweep(self, occ, T, seed, chain, colors_a, n_a, colors_b, n_b, pass0, n_passes, n_classes,
                        order_a=None, order_b=None):
        """Coloured canonical sweep (matched same-colour pairs, colourings alternating by
        pass; classes in the given list orders, else ascending): final occupation,
        correlations after each pass, accepted swaps per pass."""
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int32).copy())
        ca = np.ascontiguousarray(np.asarray(colors_a, dtype=np.int32))
        cb = np.ascontiguousarray(np.asarray(colors_b, dtype=np.int32))
        oa = None if order_a is None else np.ascontiguousarray(np.asarray(order_a, dtype=np.int32))
        ob = None if order_b is None else np.ascontiguousarray(np.asarray(order_b, dtype=np.int32))
        corr = np.zeros((n_passes, n_classes), dtype=np.int64)
        nacc = np.zeros(n_passes, dtype=np.int64)
        load().orc_ce_canonical_sweep(self.h, p(occ, C.c_int), T, C.c_ulonglong(seed), C.c_uint(chain),
                                      p(ca, C.c_int), n_a, p(cb, C.c_int), n_b,
                                      p(oa, C.c_int) if oa is not None else None,
                                      p(ob, C.c_int) if ob is not None else None, pass0, n_passes,
                                      p(corr, C.c_longlong), p(nacc, C.c_longlong))
        return occ, corr, nacc

    def canonical_samples(self, occ, T, seed, n_passes):
        """Reference-dynamics canonical run (random swaps of two different occupants): formation
        energy per site after each pass [n_passes], accepted count."""
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int32).copy())
        e = np.zeros(n_passes, dtype=np.float64)
        nacc = load().orc_ce_canonical_samples(self.h, p(occ, C.c_int), T, C.c_ulonglong(seed), n_passes,
                                               p(e, C.c_double))
        assert nacc >= 0
        return e, nacc

    def sgc_samples(self, occ, T, mu, seed, n_passes):
        """Reference-dynamics SGC run: per-pass potential energy per site [n_passes] and
        composition [n_passes, n_species-1], accepted count."""
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int32).copy())
        mu = np.ascontiguousarray(np.asarray(mu, dtype=np.float64))
        e = np.zeros(n_passes, dtype=np.float64)
        x = np.zeros((n_passes, self.n_species - 1), dtype=np.float64)
        nacc = load().orc_ce_sgc_samples(self.h, p(occ, C.c_int), T, p(mu, C.c_double), mu.size, C.c_ulonglong(seed),
                                         n_passes, p(e, C.c_double), p(x, C.c_double))
        assert nacc >= 0
        return e, x, nacc

    def sgc_run(self, occ, T, mu, engine_state: str, n_passes):
        """The reference's semi-grand canonical dynamics from an engine state: dict with the final
        occupation, per-pass accepted counts, potential energy and composition per site, the
        final occupant lists per species and the final engine state."""
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int32).copy())
        mu = np.ascontiguousarray(np.asarray(mu, dtype=np.float64))
        e = np.zeros(n_passes, dtype=np.float64)
        x = np.zeros((n_passes, self.n_species - 1), dtype=np.float64)
        nacc = np.zeros(n_passes, dtype=np.int64)
        sizes = np.zeros(self.n_species, dtype=np.int32)
        lists = np.zeros(self.n, dtype=np.int32)
        st = C.create_string_buffer(16384)
        r = load().orc_ce_sgc_run(self.h, p(occ, C.c_int), T, p(mu, C.c_double), mu.size, engine_state.encode(),
                                  n_passes, p(e, C.c_double), p(x, C.c_double), p(nacc, C.c_longlong),
                                  p(sizes, C.c_int), p(lists, C.c_int), st, len(st))
        assert r >= 0, r
        out, off = [], 0
        for s in sizes:
            out.append(lists[off:off + s].copy())
            off += s
        return {"occ": occ, "n_accept": nacc, "potential_energy": e, "param_composition": x, "lists": out,
                "engine": st.value.decode()}

    def nfold_run(self, occ, T, mu, seed, n_events):
        """The N-fold way on the CPU (binary): final occupation, wall seconds, simulated time."""
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int32).copy())
        mu = np.ascontiguousarray(np.asarray(mu, dtype=np.float64))
        secs, t = C.c_double(), C.c_double()
        n = load().orc_ce_nfold_run(self.h, p(occ, C.c_int), T, p(mu, C.c_double), mu.size, C.c_ulonglong(seed),
                                    C.c_longlong(n_events), C.byref(secs), C.byref(t))
        assert n == n_events
        return occ, secs.value, t.value

    def random_site_run(self, occ, T, mu, seed, n_steps):
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int32).copy())
        mu = np.ascontiguousarray(np.asarray(mu, dtype=np.float64))
        secs = C.c_double()
        nacc = load().orc_ce_random_site_run(self.h, p(occ, C.c_int), T, p(mu, C.c_double), mu.size,
                                             C.c_ulonglong(seed), C.c_longlong(n_steps), C.byref(secs))
        return occ, nacc, secs.value


def sgc_proposals(occ, n_species, seed, n_steps, apply=True):
    """The oracle's semi-grand canonical proposal sequence: (sites, new occupants)."""
    occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int32))
    l_out = np.zeros(n_steps, dtype=np.int64)
    o_out = np.zeros(n_steps, dtype=np.int32)
    rc = load().orc_sgc_proposals(occ.size, n_species, p(occ, C.c_int), C.c_ulonglong(seed), n_steps, int(apply),
                                  p(l_out, C.c_long), p(o_out, C.c_int))
    assert rc == 0, rc
    return l_out, o_out


def _colored_sweep_job(args):
    """Process-pool job: the oracle's coloured sweep of one chain (see OracleCE.colored_sweep)."""
    L, n_species, eci, occ, T, mu, seed, chain, colors, n_colors, pass0, n_passes, n_classes = args
    orc = OracleCE(L, n_species, eci)
    return orc.colored_sweep(occ, T, mu, seed, chain, colors, n_colors, pass0, n_passes, n_classes)


def _sgc_samples_job(args):
    """Process-pool job: the oracle's reference-dynamics semi-grand canonical run."""
    L, n_species, eci, occ, T, mu, seed, n_passes = args
    return OracleCE(L, n_species, eci).sgc_samples(occ, T, mu, seed, n_passes)


def oracle_pool(n_workers: int):
    """A process pool for oracle jobs, started with ``spawn`` (safe after CUDA is initialised)."""
    import multiprocessing as mp
    import os

    return mp.get_context("spawn").Pool(max(1, min(n_workers, os.cpu_count() or 1)))


def colored_sweeps(pool, jobs):
    """Run coloured-sweep jobs (argument tuples of _colored_sweep_job) asynchronously."""
    return pool.map_async(_colored_sweep_job, jobs, chunksize=1)


def sgc_samples_async(pool, jobs):
    return pool.map_async(_sgc_samples_job, jobs, chunksize=1)
