"""The GPU path reproduces the committed golden fixtures (tests/golden/)."""
import json
import os

import numpy as np
import pytest

import casmcode_monte_gb300 as monte
import casmcode_monte_gb300.ising_cpp as ising
import casmcode_monte_gb300.ising_cpp.semigrand_canonical as sgc
import casmcode_monte_gb300.sampling as sampling
from casmcode_monte_gb300 import clex

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_golden_ising_trajectory_on_gpu(gpu_lib, tmp_path):
    with open(os.path.join(HERE, "golden", "ising_25x25_seed1.json")) as f:
        g = json.load(f)
    calc = sgc.SemiGrandCanonicalCalculator(ising.IsingSystem(ising.IsingFormationEnergy(J=g["J"]),
                                                              ising.IsingParamComposition()))
    state = ising.IsingState(ising.IsingConfiguration((g["rows"], g["cols"])),
                             monte.ValueMap.from_dict({"temperature": g["T"], "exchange_potential": [g["mu"]]}))
    state.configuration.set_occupation(g["occ0"])
    p = sampling.CompletionCheckParams()
    p.cutoff_params.max_count = g["n_passes"]
    e = monte.RandomNumberEngine()
    e.seed(g["seed"])
    calc.run(state, calc.default_sampling_functions(), {}, p, sgc.SemiGrandCanonicalEventGenerator(),
             method_log=monte.MethodLog(str(tmp_path / "s.json"), None), random_engine=e,
             write_status_f=lambda c, l: None)
    assert state.configuration.occupation().tolist() == g["occ_final"]
    assert calc.data.n_accept == g["n_accept"]
    pe = calc.data.samplers["potential_energy"].component(0)
    assert [float.hex(float(x)) for x in pe] == g["potential_energy_hex"]


def test_golden_ce_delta_e_on_gpu(gpu_lib):
    with open(os.path.join(HERE, "golden", "ce_delta_e.json")) as f:
        g = json.load(f)
    for case in g["cases"]:
        model = clex.ClexModel(case["kind"], case["eci"])
        occ = np.array(case["occ"], dtype=np.int8)
        for l, new, mu, dE_hex in case["proposals"]:
            b = clex.ChainBatch(model, case["L"], occ[None, :], [1000.0], np.array(mu)[None, :], [1])
            got = b.delta_e([0], [l], [new])[0]
            ref = float.fromhex(dE_hex)
            assert abs(got - ref) <= 1e-12 * max(abs(ref), 1e-3)
            b.close()
