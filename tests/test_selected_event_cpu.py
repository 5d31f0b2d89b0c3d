"""Selected-event parameters, hop correlations and histograms (host-side API).

The first four tests restate python/tests/sampling/test_SelectedEventFunctionParams.py;
the rest check the binning rules of src/casm/monte/sampling/SelectedEventFunctions.cc on
cases worked out by hand from that code.
"""
import math

import numpy as np
import pytest

from casmcode_monte_gb300 import sampling


def test_SelectedEventFunctionParams():
    params = sampling.SelectedEventFunctionParams()
    params.collect("event_type")
    assert params.function_names == ["event_type"]
    params.do_not_collect("event_type")
    assert len(params.function_names) == 0


def test_SelectedEventFunctionParams_get_parameters():
    params = sampling.SelectedEventFunctionParams()
    params.collect(name="dE_activated", initial_begin=0.01, bin_width=1.0, max_size=10, spacing="linear")
    data = params.get_parameters("dE_activated")
    assert data == {"initial_begin": 0.01, "bin_width": 1.0, "max_size": 10, "spacing": "linear"}
    params.do_not_collect("dE_activated")
    assert params.get_parameters("dE_activated") == {}
    with pytest.raises(RuntimeError):
        params.collect("x", spacing="cubic")


def test_collect_hop_correlations():
    params = sampling.SelectedEventFunctionParams()
    assert params.correlations_data_params is None
    params.collect_hop_correlations(jumps_per_position_sample=10)
    assert isinstance(params.correlations_data_params, sampling.CorrelationsDataParams)
    assert params.correlations_data_params.jumps_per_position_sample == 10
    data = params.correlations_data_params.to_dict()
    assert data == {"jumps_per_position_sample": 10, "max_n_position_samples": 100,
                    "output_incomplete_samples": False, "stop_run_when_complete": False}
    assert isinstance(sampling.CorrelationsDataParams.from_dict(data), sampling.CorrelationsDataParams)
    assert sampling.CorrelationsDataParams.from_dict({}).max_n_position_samples == 100
    params.do_not_collect_hop_correlations()
    assert params.correlations_data_params is None
    params.collect_hop_correlations(**data)
    assert params.correlations_data_params.jumps_per_position_sample == 10


def test_SelectedEventFunctionParams_to_and_from_dict():
    params = sampling.SelectedEventFunctionParams()
    params.collect("event_type")
    params.collect(name="dE_activated", initial_begin=0.01, bin_width=1.0, max_size=10, spacing="linear")
    params.evaluate("count_events", order=3)
    params.collect_hop_correlations(jumps_per_position_sample=10)
    data = params.to_dict()
    assert data["quantities"] == ["event_type", "dE_activated", "count_events"]
    assert data["spacing"] == {"dE_activated": "linear"}
    assert "tol" not in data
    params_in = sampling.SelectedEventFunctionParams.from_dict(data)
    assert params_in.function_names == params.function_names
    assert params_in.get_parameters("dE_activated") == params.get_parameters("dE_activated")
    assert params_in.correlations_data_params.jumps_per_position_sample == 10
    with pytest.raises(RuntimeError):
        sampling.SelectedEventFunctionParams.from_dict({"quantities": ["a"], "spacing": {"a": "cubic"}})


def test_histogram1d_grows_both_ways():
    h = sampling.Histogram1D(initial_begin=0.0, bin_width=1.0)
    h.insert(2.5)
    assert h.begin() == 2.0 and h.count() == [1.0]
    h.insert(0.2)
    assert h.begin() == 0.0 and h.count() == [1.0, 0.0, 1.0]
    assert h.bin_coords() == [0.0, 1.0, 2.0]
    assert h.sum() == 2.0 and h.density() == [0.5, 0.0, 0.5]
    d = h.to_dict()
    assert d["begin"] == 0.0 and d["count"] == [1.0, 0.0, 1.0] and d["out_of_range_count"] == 0.0
    with pytest.raises(RuntimeError):
        h.insert_log_value(1.0)
    with pytest.raises(RuntimeError):
        sampling.Histogram1D().insert(math.inf)


def test_histogram1d_max_size():
    h = sampling.Histogram1D(initial_begin=0.0, bin_width=1.0, max_size=2)
    h.insert(0.5)
    h.insert(3.5)
    assert h.max_size_exceeded() and h.count() == [1.0, 0.0] and h.out_of_range_count() == 1.0
    h.insert(-1.5)
    assert h.count() == [1.0, 0.0] and h.out_of_range_count() == 2.0 and h.sum() == 3.0


def test_histogram1d_log_spacing():
    h = sampling.Histogram1D(initial_begin=-2.0, bin_width=0.5, is_log=True)
    h.insert(100.0)  # log10 = 2 lands on the upper edge of the first bin: bin 1
    assert h.begin() == 1.5 and h.count() == [0.0, 1.0]
    h.insert_log_value(1.6, 2.0)
    assert h.count() == [2.0, 1.0]
    with pytest.raises(RuntimeError):
        h.merge(sampling.Histogram1D(initial_begin=-2.0, bin_width=0.5, is_log=False))
    with pytest.raises(RuntimeError):
        sampling.combine([])


def test_partitioned_histogram_alignment():
    p = sampling.PartitionedHistogram1D(["A", "B"], initial_begin=0.0, bin_width=1.0)
    p.insert(0, 0.5)
    p.insert(1, 3.5)
    combined = p.combined_histogram()
    assert combined.begin() == 0.0 and combined.count() == [1.0, 0.0, 0.0, 1.0]
    a, b = p.histograms()
    assert a.count() == [1.0, 0.0, 0.0, 0.0] and b.count() == [0.0, 0.0, 0.0, 1.0]
    d = p.to_dict()
    assert d["partition_names"] == ["A", "B"]
    assert [x["partition_fraction"] for x in d["partitions"]] == [0.5, 0.5]
    assert d["partitions"][1]["partial_density"] == [0.0, 0.0, 0.0, 0.5]
    with pytest.raises(RuntimeError):
        p.insert(2, 1.0)
    with pytest.raises(RuntimeError):
        p.insert(0, math.nan)
    single = sampling.PartitionedHistogram1D(["only"])
    single.insert(0, 1.0)  # the upper edge of the first bin falls in the second
    assert single.to_dict()["count"] == [0.0, 1.0]


def test_discrete_vector_histograms():
    h = sampling.DiscreteVectorIntHistogram(["a", "b"], [2], max_size=2)
    for v in ([1, 0], [0, 1], [1, 0], [2, 2]):
        h.insert(np.array(v))
    assert [v.tolist() for v in h.values()] == [[0, 1], [1, 0]]
    assert h.count() == [1.0, 2.0] and h.out_of_range_count() == 1.0 and h.max_size_exceeded()
    assert h.sum() == 4.0 and h.fraction() == [0.25, 0.5]
    assert h.to_dict()["values"] == [[0, 1], [1, 0]]
    f = sampling.DiscreteVectorFloatHistogram(["x"], [1], tol=1e-3)
    f.insert([0.5])
    f.insert([0.5004])
    f.insert([0.6])
    f.insert([0.1], weight=2.0)
    assert [v.tolist() for v in f.values()] == [[0.1], [0.5], [0.6]]
    assert f.count() == [2.0, 2.0, 1.0]
    s = sampling.DiscreteVectorIntHistogram([], [], value_labels=[(np.array([3]), "three")])
    s.insert([3])
    s.insert([4])
    d = s.to_dict()
    assert d["values"] == [3, 4] and d["labels"] == ["three", 4] and "component_names" not in d


def test_correlations_data():
    c = sampling.CorrelationsData()
    c.initialize(n_atoms=2, jumps_per_position_sample=2, max_n_position_samples=3, output_incomplete_samples=False)
    c.insert(0, 1, [9.0, 9.0, 9.0], 1, 0, 0.1)  # not a multiple of 2: ignored
    c.insert(0, 2, [1.0, 2.0, 3.0], 5, 1, 0.5)
    assert c.n_position_samples == [1, 0] and c.n_complete_samples == 0
    c.insert(1, 2, [4.0, 5.0, 6.0], 7, 2, 1.5)
    assert c.n_position_samples == [1, 1] and c.n_complete_samples == 1
    assert getattr(c, "pass")[0].tolist() == [1, 2]
    assert c.indices_after_pass(2) == [0] and c.indices_after_pass(3) == []
    assert c.indices_after_time(1) == [0]
    d = c.to_dict()
    assert d["step"] == [[5, 7]] and d["atom_positions_cart"] == [[[1.0, 4.0], [2.0, 5.0], [3.0, 6.0]]]


def test_selected_event_data_collector():
    state = {"event": 0, "dE": 0.25, "n_generic": 0}
    funcs = sampling.SelectedEventFunctions()

    def bump():
        state["n_generic"] += 1

    funcs.insert(sampling.GenericSelectedEventFunction("count", "counter", False, bump))
    funcs.insert(sampling.VectorIntHistogramFunction("event_type", "type", [], False,
                                                     lambda: np.array([state["event"]])))
    funcs.insert(sampling.PartitionedHistogramFunction("dE_activated", "barrier", False, lambda: state["dE"],
                                                       ["hop", "swap"], lambda: state["event"]))
    params = sampling.SelectedEventFunctionParams()
    params.evaluate("count").collect("event_type").collect("dE_activated", bin_width=0.5)
    data = sampling.SelectedEventData()
    collector = sampling.SelectedEventDataCollector(funcs, params, data)
    for event, dE in ((0, 0.25), (1, 1.75), (1, 0.6)):
        state["event"], state["dE"] = event, dE
        collector.collect()
    assert state["n_generic"] == 3
    assert data.discrete_vector_int_histograms["event_type"].count() == [1.0, 2.0]
    hist = data.continuous_1d_histograms["dE_activated"]
    assert hist.combined_histogram().count() == [1.0, 1.0, 0.0, 1.0]
    assert set(data.to_dict()["histograms"]) == {"event_type", "dE_activated"}
    params.collect("missing")
    with pytest.raises(RuntimeError):
        sampling.SelectedEventDataCollector(funcs, params, data)
