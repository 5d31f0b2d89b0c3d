"""ValueMap and its typed maps (python/tests/test_ValueMap.py:8-113, python/src/monte.cpp:
106-109,385-470): each map converts what it stores (bool, float, 1-d and 2-d float64
arrays) and hands back the stored object, so elements can be changed in place; to_dict and
from_dict sort values by type; plain dicts assigned to the attributes are converted."""
import copy

import numpy as np
import pytest

import casmcode_monte_gb300 as mc


@pytest.mark.parametrize("name,value", [("BooleanValueMap", True), ("ScalarValueMap", 2.5),
                                        ("VectorValueMap", np.array([1.0, 3.0])),
                                        ("MatrixValueMap", np.eye(2))])
def test_typed_maps_at_the_bound_path(name, value):
    m = getattr(mc._monte, name)()
    assert len(m) == 0 and getattr(mc, name) is type(m)
    m["v"] = value
    assert len(m) == 1 and np.array_equal(m["v"], value)


def test_typed_maps_convert_values():
    assert mc.ScalarValueMap({"a": 2})["a"] == 2.0 and isinstance(mc.ScalarValueMap({"a": 2})["a"], float)
    assert mc.BooleanValueMap({"b": 1})["b"] is True
    v = mc.VectorValueMap({"x": [1, 2, 3]})["x"]
    assert v.dtype == np.float64 and v.shape == (3,)
    assert mc.VectorValueMap({"x": np.ones((3, 1))})["x"].shape == (3,)
    with pytest.raises(ValueError):
        mc.VectorValueMap({"x": np.ones((2, 2))})
    with pytest.raises(ValueError):
        mc.MatrixValueMap({"m": [1.0, 2.0]})


def test_value_map_members_change_in_place():
    values = mc.ValueMap()
    values.boolean_values["on"] = True
    values.scalar_values["T"] = 300.0
    values.vector_values["mu"] = np.array([0.1, 0.2])
    values.vector_values["mu"][1] = -0.5
    values.matrix_values["M"] = np.zeros((2, 2))
    values.matrix_values["M"][1, 0] = 7.0
    assert values.boolean_values["on"] is True and values.scalar_values["T"] == 300.0
    assert np.array_equal(values.vector_values["mu"], [0.1, -0.5])
    assert np.array_equal(values.matrix_values["M"], [[0.0, 0.0], [7.0, 0.0]])
    # assigning a plain dict converts it
    values.scalar_values = {"T": 400}
    assert isinstance(values.scalar_values, mc.ScalarValueMap) and values.scalar_values["T"] == 400.0
    # copies are deep
    c = copy.copy(values)
    c.vector_values["mu"][0] = 9.0
    assert values.vector_values["mu"][0] == 0.1


def test_value_map_dict_round_trip():
    values = mc.ValueMap()
    values.boolean_values["b"] = False
    values.scalar_values["s"] = 1.5
    values.vector_values["v"] = np.array([1.0, 2.0])
    values.matrix_values["m"] = np.array([[1.0, 2.0], [3.0, 4.0]])
    d = values.to_dict()
    assert set(d) == {"b", "s", "v", "m"} and d["b"] is False
    back = mc.ValueMap.from_dict(d)
    assert back.boolean_values == {"b": False} and back.scalar_values == {"s": 1.5}
    assert np.array_equal(back.vector_values["v"], [1.0, 2.0])
    assert np.array_equal(back.matrix_values["m"], [[1.0, 2.0], [3.0, 4.0]])
    assert not values.is_mismatched(back)
    assert mc.ValueMap(d).scalar_values["s"] == 1.5
