"""Serving engine: continuous batching gives each job the result it gets alone."""
import numpy as np
import pytest

from casmcode_monte_gb300 import clex, serving

pytestmark = pytest.mark.gpu


def _models():
    return {k: clex.ClexModel(k, clex.make_eci(k, 2)) for k in ("fcc_binary", "fcc_ternary")}


def _stream(models, n=14, seed=5):
    return serving.poisson_jobs(n, rate=1e4, models=models, seed=seed, L_range=(8, 70), budget=(100, 450),
                                abs_precision=2e-3)


def test_results_same_alone_and_in_the_mix(gpu_lib):
    models = _models()
    mix = serving.ServingEngine(models, arena_bytes=64 << 20, max_chains=64, max_passes=500, keep_occupation=True)
    st = mix.run(_stream(models), realtime=False)
    assert len(st.jobs) == 14
    by_id = {j.id: j for j in st.jobs}
    for job in _stream(models):
        alone = serving.ServingEngine(models, arena_bytes=64 << 20, max_chains=4, max_passes=500,
                                      keep_occupation=True)
        a = alone.run([job], realtime=False).jobs[0]
        m = by_id[job.id]
        assert (a.n_pass, a.converged, a.equilibrated, a.n_equilibration) == \
               (m.n_pass, m.converged, m.equilibrated, m.n_equilibration)
        assert a.mean == m.mean and a.precision == m.precision
        assert np.array_equal(a.final_occ, m.final_occ)
        assert a.n_pass <= job.pass_budget
        assert a.converged or a.n_pass == job.pass_budget


def test_admission_waits_for_memory(gpu_lib):
    models = _models()
    jobs = serving.poisson_jobs(6, rate=1e4, models={"fcc_binary": models["fcc_binary"]}, seed=3, L_range=(16, 16),
                                budget=(200, 200), abs_precision=1e-9)
    # arena for two 16^3 chains only: the rest wait and are admitted as others finish
    eng = serving.ServingEngine({"fcc_binary": models["fcc_binary"]}, arena_bytes=2 * 4096, max_chains=8,
                                max_passes=300)
    st = eng.run(jobs, realtime=False)
    assert len(st.jobs) == 6
    starts = sorted(j.start for j in st.jobs)
    assert starts[2] > starts[1]  # the third job waited for a free arena block
    assert all(j.n_pass == 200 and not j.converged for j in st.jobs)
