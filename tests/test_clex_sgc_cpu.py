"""Host-side classes of the cluster-expansion semi-grand canonical calculator."""
import numpy as np
import pytest

import casmcode_monte_gb300 as monte
import casmcode_monte_gb300.clex as clex
import casmcode_monte_gb300.clex.semigrand_canonical as sgc


def test_configuration_roundtrip_and_errors():
    occ = np.arange(2 * 3 * 4) % 2
    cfg = sgc.ClexConfiguration((2, 3, 4), occ)
    assert cfg.n_sites == cfg.n_unitcells == 24 and cfg.occ(5) == 1
    assert sgc.ClexConfiguration.from_dict(cfg.to_dict()).to_dict() == cfg.to_dict()
    with pytest.raises(RuntimeError, match="size mismatch"):
        cfg.set_occupation(np.zeros(5))
    with pytest.raises(RuntimeError):
        sgc.ClexConfiguration((2, 3))


def test_conditions_and_composition():
    c = sgc.SemiGrandCanonicalConditions.from_dict({"temperature": 800.0, "exchange_potential": [0.1, -0.2]})
    assert c.temperature == 800.0 and np.array_equal(c.exchange_potential, [0.1, -0.2])
    assert sgc.SemiGrandCanonicalConditions.from_values(c.to_values()).to_dict() == c.to_dict()
    with pytest.raises(RuntimeError, match="temperature"):
        sgc.SemiGrandCanonicalConditions.from_values(monte.ValueMap.from_dict({"exchange_potential": [0.0]}))
    model = clex.ClexModel("fcc_ternary", clex.make_eci("fcc_ternary", 1))
    state = sgc.ClexState(sgc.ClexConfiguration((2, 2, 2), [0, 1, 2, 1, 0, 0, 2, 1]),
                          monte.ValueMap.from_dict({"temperature": 800.0, "exchange_potential": [0.0, 0.0]}))
    x = sgc.ClexParamComposition(model, state)
    assert x.n_independent_compositions() == 2
    assert np.array_equal(x.per_supercell(), [3.0, 2.0])
    assert np.array_equal(x.occ_delta_per_supercell([0, 2], [2, 1]), [1.0, 0.0])


def test_canonical_conditions_and_calculator_construction():
    import casmcode_monte_gb300.clex.canonical as can

    c = can.CanonicalConditions.from_values(monte.ValueMap.from_dict({"temperature": 900.0, "other": 1.0}))
    assert c.temperature == 900.0 and c.to_dict() == {"temperature": 900.0}
    assert can.CanonicalConditions.from_dict({"temperature": 5.0}).temperature == 5.0
    with pytest.raises(RuntimeError, match="temperature"):
        can.CanonicalConditions.from_values(monte.ValueMap())
    with pytest.raises(RuntimeError):
        can.CanonicalCalculator(None)
