"""Sampling and completion-check semantics (CPU), following the reference's own tests
python/tests/sampling/test_CompletionCheck.py:5-124 and the C++ CompletionCheck rules."""
import numpy as np
import pytest

import casmcode_monte_gb300 as monte
import casmcode_monte_gb300.sampling as sampling


def test_CompletionCheck_1(tmp_path):
    completion_check_params = sampling.CompletionCheckParams()
    completion_check_params.cutoff_params.max_count = 12
    completion_check = sampling.CompletionCheck(completion_check_params)
    samplers = sampling.SamplerMap()
    samplers["e"] = sampling.Sampler(shape=[])
    samplers["x"] = sampling.Sampler(shape=[3])
    sample_weight = sampling.Sampler(shape=[])
    method_log = monte.MethodLog(str(tmp_path / "log.txt"))
    n_steps = 0
    while not completion_check.count_check(samplers=samplers, sample_weight=sample_weight, count=n_steps,
                                           method_log=method_log):
        n_steps += 1
        if n_steps % 10 == 0:
            samplers["e"].append([0])
            samplers["x"].append([0, 0, 0])
    assert n_steps == 12


def test_CompletionCheck_2(tmp_path):
    completion_check_params = sampling.CompletionCheckParams()
    completion_check_params.cutoff_params.min_sample = 100
    e_key = sampling.SamplerComponent(sampler_name="e", component_name="", component_index=0)
    completion_check_params.requested_precision[e_key] = sampling.RequestedPrecision(abs=0.001)
    v_key = sampling.SamplerComponent(sampler_name="v", component_name="", component_index=0)
    completion_check_params.requested_precision[v_key] = sampling.RequestedPrecision(abs=0.01)
    completion_check = sampling.CompletionCheck(completion_check_params)
    samplers = sampling.SamplerMap()
    samplers["e"] = sampling.Sampler(shape=[], component_names=[""])
    samplers["v"] = sampling.Sampler(shape=[], component_names=[""])
    sample_weight = sampling.Sampler(shape=[])
    method_log = monte.MethodLog(str(tmp_path / "log.txt"))
    rng = monte.RandomNumberGenerator()
    n_steps = 0
    while not completion_check.count_check(samplers=samplers, sample_weight=sample_weight, count=n_steps,
                                           method_log=method_log):
        n_steps += 1
        e = 1.0 + rng.random_real(0.1) - 0.05
        v = 20.0 + rng.random_real(1.0) - 0.5
        if n_steps % 10 == 0:
            samplers["e"].append([e])
            samplers["v"].append([v])
    results = completion_check.results()
    assert sampling.get_n_samples(samplers) >= 100
    assert results.is_complete
    assert results.equilibration_check_results.all_equilibrated
    assert len(results.equilibration_check_results.individual_results) == 2
    assert results.convergence_check_results.all_converged
    assert len(results.convergence_check_results.individual_results) == 2
    cr = results.convergence_check_results.individual_results
    assert cr[e_key].stats.calculated_precision < 0.001
    assert cr[v_key].stats.calculated_precision < 0.01


def test_check_schedule_linear_and_log():
    p = sampling.CompletionCheckParams()
    assert [p.sample_check_linear(n) for n in range(3)] == [100, 200, 300]
    p.log_spacing = True
    p.check_begin = 0
    p.check_base = 10.0
    p.check_shift = 2.0
    p.check_period_max = 10000
    nbl = p.find_n_begin_linear()
    # 10^2, 10^3, 10^4 then linear steps of 10000
    assert [p.sample_check_log(n, nbl) for n in range(5)] == [100, 1000, 10000, 20000, 30000]


def test_sampler_growth_and_components():
    s = sampling.Sampler(shape=[2, 2], capacity_increment=3)
    assert s.component_names() == ["0,0", "1,0", "0,1", "1,1"]
    for i in range(7):
        s.append(np.arange(4) + 10 * i)
    assert s.n_samples() == 7 and s.sample_capacity() == 9
    assert np.array_equal(s.component(2), np.arange(7) * 10 + 2)
    assert s.values().shape == (7, 4)
    s.clear()
    assert s.n_samples() == 0


def test_requested_precision_constructor():
    sf = sampling.StateSamplingFunctionMap()
    sf["corr"] = sampling.StateSamplingFunction("corr", "", [3], lambda: [0, 0, 0])
    p = sampling.CompletionCheckParams()
    sampling.converge(sf, p).set_precision("corr", abs=0.1, component_index=[0, 2])
    assert sorted((k.sampler_name, k.component_index) for k in p.requested_precision) == [("corr", 0), ("corr", 2)]
    with pytest.raises(Exception):
        sampling.converge(sf, p).set_precision("nope", abs=0.1)


def test_repeat_calls_catch_up_matches_literal_calls():
    """The per-pass emulation of the reference's per-step calls advances the check
    schedule exactly as literal repeated calls do."""
    def make():
        p = sampling.CompletionCheckParams()
        p.cutoff_params.min_sample = 250
        p.check_begin = 10
        p.check_period = 10
        key = sampling.SamplerComponent("e", 0, "0")
        p.requested_precision[key] = sampling.RequestedPrecision(abs=1e-9)
        return p

    rng = np.random.default_rng(0)
    series = rng.normal(size=400)
    for steps_per_pass in (1, 3, 7, 50):
        a = sampling.CompletionCheck(make())
        b = sampling.CompletionCheck(make())
        sa = {"e": sampling.Sampler([])}
        sb = {"e": sampling.Sampler([])}
        w = sampling.Sampler([])
        for t in range(300):
            sa["e"].append([series[t]])
            sb["e"].append([series[t]])
            ra = a.count_check(sa, w, t + 1, None)
            for _ in range(steps_per_pass - 1):
                ra = a.count_check(sa, w, t + 1, None) or ra
            rb = b.count_check(sb, w, t + 1, None)
            b._repeat_calls(steps_per_pass - 1)
            assert ra == rb
            assert a._n_checks == b._n_checks


def test_sampling_binding_names_and_dict_forms():
    """Methods under the reference binding's names (python/src/monte_sampling.cpp) and the
    dict forms of Sampler_json_io.cc:39-95, CutoffCheck_json_io.cc:9-48 and
    CompletionCheck_json_io.hh:295-420."""
    import casmcode_monte_gb300.sampling as sp
    js = sp.jsonSampler()
    js.append({"a": 1})
    js.set_values([{"a": 2}, {"b": 3}])
    assert js.n_samples() == 2 == len(js) and js.values() == [{"a": 2}, {"b": 3}] and js.sample(1) == {"b": 3}
    assert js.values[-1] == {"b": 3} and js.to_list() == list(js)
    js.set_sample_capacity(10)
    assert js.sample_capacity() == 10
    js.clear()
    assert js.n_samples() == 0

    rp = sp.RequestedPrecision(abs=0.1, rel=0.2)
    assert rp.to_dict() == {"abs_precision": 0.1, "rel_precision": 0.2}
    old = sp.RequestedPrecision.from_dict({"precision": 0.5})
    assert old.abs_convergence_is_required and old.abs_precision == 0.5 and not old.rel_convergence_is_required

    st = sp.BasicStatistics(mean=-2.0, calculated_precision=0.5)
    assert st.relative_precision() == 0.25
    calc = sp.BasicStatisticsCalculator(0.9, 1, 500)
    assert sp.BasicStatisticsCalculator.from_dict(calc.to_dict()).to_dict() == calc.to_dict()
    assert calc.weighted_observations_method == 1
    x = np.random.default_rng(1).normal(size=400)
    assert calc.calculate(x, np.zeros(0)).mean == calc(x).mean

    cut = sp.CutoffCheckParams(min_sample=10, max_count=100, max_clocktime=5.0)
    assert cut.to_dict() == {"count": {"max": 100}, "sample": {"min": 10}, "clocktime": {"max": 5.0}}
    assert sp.CutoffCheckParams.from_dict(cut.to_dict()) == cut

    f = sp.StateSamplingFunction("comp", "composition", [2], lambda: np.zeros(2), ["x0", "x1"])
    g = sp.StateSamplingFunction("energy", "energy", [], lambda: np.zeros(1))
    fmap = sp.StateSamplingFunctionMap({"comp": f, "energy": g})
    d = {"cutoff": {"sample": {"max": 1000}}, "spacing": "log", "period_max": 500,
         "convergence": [{"quantity": "energy", "abs_precision": 0.001},
                         {"quantity": "comp", "component_name": ["x1"], "rel_precision": 0.01}],
         "confidence": 0.9}
    p = sp.CompletionCheckParams.from_dict(d, fmap)
    assert p.log_spacing and (p.check_begin, p.check_base, p.check_shift, p.check_period_max) == (0, 10.0, 2.0, 500)
    assert p.cutoff_params.max_sample == 1000 and p.calc_statistics_f.confidence == 0.9
    keys = sorted(p.requested_precision)
    assert [(k.sampler_name, k.component_index) for k in keys] == [("comp", 1), ("energy", 0)]
    assert p.requested_precision[keys[0]].rel_precision == 0.01
    p2 = sp.CompletionCheckParams.from_dict(p.to_dict(), fmap)
    assert p2.to_dict() == p.to_dict()
    with pytest.raises(RuntimeError, match="not a sampling option"):
        sp.CompletionCheckParams.from_dict({"convergence": [{"quantity": "nope", "abs_precision": 1.0}]}, fmap)
    with pytest.raises(RuntimeError, match="out of range"):
        sp.CompletionCheckParams.from_dict({"convergence": [{"quantity": "comp", "component_index": [2],
                                                             "abs_precision": 1.0}]}, fmap)

    s = sp.SamplingParams()
    s.extend_sampler_names(["a", "b", "a"])
    s.append_to_sampler_names("c")
    s.remove_from_sampler_names("a")
    s.remove_from_sampler_names("zz")
    s.append_to_json_sampler_names("config")
    assert s.sampler_names == ["b", "a", "c"] and s.json_sampler_names == ["config"]
