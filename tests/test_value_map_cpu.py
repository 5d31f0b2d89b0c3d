"""The core module's host types under the reference binding's names.

* ValueMap and its typed maps (python/tests/test_ValueMap.py:8-113, python/src/monte.cpp:
  106-109,385-470): each map converts what it stores (bool, float, 1-d and 2-d float64
  arrays) and hands back the stored object, so elements can be changed in place; to_dict
  and from_dict sort values by type; plain dicts assigned to the attributes are converted.
* MethodLog's sections, verbosity, indentation and paragraphs; the generator's engine();
  the semi-grand canonical potential's change for an OccEvent."""
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


def test_method_log_sections_and_text(tmp_path):
    """MethodLog's verbosity-gated sections, indentation and paragraph formatting
    (python/src/monte.cpp:150-384)."""
    path = tmp_path / "log.txt"
    log = mc.MethodLog(str(path))
    log.set_standard()
    log.begin_section_print_if_verbose()
    log.print("hidden\n")
    log.end_section()
    log.begin_section_print_if_standard()
    log.increase_indent()
    log.section("Run")
    log.set_paragraph_width(20)
    log.paragraph("one two three four five six seven")
    log.verbatim("a\nb", indent_first_line=False)
    log.decrease_indent()
    log.end_section()
    log.set_quiet()
    log.begin_section_print_if_standard()
    log.print("also hidden\n")
    log.end_section()
    log.begin_section_print_always()
    log.print("shown\n")
    log.end_section()
    text = path.read_text()
    assert "hidden" not in text and text.endswith("shown\n")
    lines = text.splitlines()
    assert lines[0] == "  -- Run -- " and all(len(x) <= 20 for x in lines[1:-3]) and lines[1].startswith("  one")
    assert lines[-3:] == ["a", "  b", "shown"]
    assert log.indent_str() == "" and log.paragraph_width() == 20 and log.paragraph_justification() == "left"


def test_generator_engine_and_event_delta():
    e = mc.RandomNumberEngine()
    g = mc.RandomNumberGenerator(e)
    assert g.engine() is e
    import casmcode_monte_gb300.events as ev
    import casmcode_monte_gb300.ising_cpp as ising
    import casmcode_monte_gb300.ising_cpp.semigrand_canonical as sgc
    state = ising.IsingState(ising.IsingConfiguration(shape=(5, 5)),
                             mc.ValueMap.from_dict({"temperature": 1000.0, "exchange_potential": [0.1]}))
    fe = ising.IsingFormationEnergy(J=0.1, lattice_type=1, state=state)
    pot = sgc.SemiGrandCanonicalPotential(ising.IsingSystem(fe, ising.IsingParamComposition(state=state)))
    pot.set_state(state, sgc.SemiGrandCanonicalConditions.from_values(state.conditions))
    e1 = ev.OccEvent([3], [-1])
    assert pot.occ_event_delta_per_supercell(e1) == pot.occ_delta_per_supercell([3], [-1])
    c = copy.copy(pot)
    assert c is not pot and c.formation_energy_calculator is pot.formation_energy_calculator
