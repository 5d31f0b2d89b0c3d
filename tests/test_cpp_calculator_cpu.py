"""The C++ generic Metropolis loop and completion check (include/montegpu_methods.hpp) on the host.

SemiGrandCanonicalCalculator::run with an event generator other than the built-in one runs the
reference's methods::basic_occupation_metropolis (basic_occupation_metropolis.hh:354-425) with
the reference's CompletionCheck (CompletionCheck.hh:175-376).  On the reference's convergence
scenario (25x25 Ising, J = 0.1, T = 2000 K, potential energy to 0.001, at most 4000 passes,
engine seeded 7) it must stop at the oracle's pass with the oracle's accepted count, final
occupation, every potential-energy sample, completion results and engine state.  No device
computation: the statistics are the library's host numerics.
"""
import json
import os
import subprocess

import numpy as np

from casmcode_monte_gb300 import _lib
from tests import oracle_lib
from tests.test_cpp_calculator_gpu import ROOT, _build


def test_cpp_generic_loop_matches_oracle(tmp_path):
    with open(os.path.join(ROOT, "tests", "golden", "ising_25x25_seed1.json")) as f:
        occ0 = json.load(f)["occ0"]
    exe = _build(tmp_path)
    r = subprocess.run([str(exe), "host"], input=" ".join(str(v) for v in occ0), capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr
    got = json.loads(r.stdout)["converge_host"]
    ref = oracle_lib.ising_run(25, 25, 0.1, True, 2000.0, 0.0, np.asarray(occ0, dtype=np.int32),
                               oracle_lib.make_cc_params(max_count=4000, reqs=[(2, 0.001)]), 1,
                               oracle_lib.engine_state(7))
    out = ref["out"]
    assert got["n_pass"] == out.n_pass and got["n_accept"] == out.n_accept and got["n_reject"] == out.n_reject
    assert got["n_samples"] == out.n_samples
    assert got["occ"] == ref["occ"].tolist()
    assert [float.hex(v) for v in got["potential_energy"]] == [float.hex(float(v)) for v in ref["potential_energy"]]
    assert got["all_equilibrated"] == out.all_equilibrated and got["all_converged"] == out.all_converged
    assert got["is_complete"] == out.is_complete == 1
    assert got["engine"] == ref["engine"]
