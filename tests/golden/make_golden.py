"""Generate the golden fixtures in tests/golden/ from the CPU oracle.

Run from the repository root:  python tests/golden/make_golden.py

* ising_25x25_seed1.json: the reference's Ising scenario (25x25, J = 0.1, T = 2000 K,
  mu = 0) for 1000 passes from a uniform +-1 occupation (numpy seed 1) with the
  mt19937_64 engine seeded by seed(1): final occupation, acceptance count and every
  potential-energy sample (as float.hex strings, bit-exact).
* ce_delta_e.json: FCC binary and ternary cluster-expansion dE for seeded proposals on
  small supercells (ECI from casmcode_monte_gb300.clex.make_eci), as float.hex.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tests import oracle_lib  # noqa: E402


def ising():
    rng = np.random.default_rng(1)
    occ = rng.choice(np.array([-1, 1], dtype=np.int32), size=625)
    ref = oracle_lib.ising_run(25, 25, 0.1, True, 2000.0, 0.0, occ, oracle_lib.make_cc_params(max_count=1000), 1,
                               oracle_lib.engine_state(1))
    return {
        "rows": 25, "cols": 25, "J": 0.1, "use_nlist": True, "T": 2000.0, "mu": 0.0, "seed": 1, "n_passes": 1000,
        "occ0": occ.tolist(), "occ_final": ref["occ"].tolist(), "n_accept": int(ref["out"].n_accept),
        "potential_energy_hex": [float.hex(float(x)) for x in ref["potential_energy"]],
    }


def ce():
    from casmcode_monte_gb300.clex import make_eci

    cases = []
    for kind, ns, L in (("fcc_binary", 2, (8, 8, 8)), ("fcc_ternary", 3, (8, 6, 10))):
        eci = make_eci(kind, 3)
        orc = oracle_lib.OracleCE(L, ns, eci)
        rng = np.random.default_rng(11)
        occ = rng.integers(0, ns, size=orc.n).astype(np.int32)
        props = []
        for _ in range(40):
            l = int(rng.integers(0, orc.n))
            new = int((occ[l] + 1 + rng.integers(0, ns - 1)) % ns)
            mu = rng.uniform(-0.3, 0.3, ns - 1).tolist()
            props.append([l, new, mu, float.hex(orc.delta_e(occ, l, new, np.array(mu)))])
        cases.append({"kind": kind, "n_species": ns, "L": list(L), "eci": eci.tolist(), "occ": occ.tolist(),
                      "proposals": props})
    return {"cases": cases}


if __name__ == "__main__":
    with open(os.path.join(HERE, "ising_25x25_seed1.json"), "w") as f:
        json.dump(ising(), f)
    with open(os.path.join(HERE, "ce_delta_e.json"), "w") as f:
        json.dump(ce(), f)
    print("written")
