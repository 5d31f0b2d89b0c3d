"""The header-only C++ Ising model (include/montegpu_ising.hpp) compiles with g++ and links the
library.  Its host arithmetic gives the reference's known answers
(tests/unit/monte/Ising_basic_semigrand_canonical_test.cpp:113-267: 25x25 all +1, J = 0.1:
E_f = -125.0, -0.2 per unit cell, dE_f = 0.8 for a flip, N x = 625, N dx = -1, E_sgc = -1375.0
at mu = 2.0) with and without neighbour lists, and on a random configuration its energies
equal the Python ising_cpp model's bit for bit.  The proposal draws are libstdc++'s
uniform_int_distribution<long>(0, N - 1) on std::mt19937_64.  The GPU pass loop
(run_metropolis_passes) is compiled and linked here, not run: no device computation."""
import os
import subprocess

import numpy as np

import casmcode_monte_gb300 as monte
import casmcode_monte_gb300.ising_cpp as ising
from casmcode_monte_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r'''
#include <cstdio>
#include "montegpu_ising.hpp"
using namespace montegpu::ising_cpp;
using namespace montegpu::ising_cpp::semigrand_canonical;
int main() {
  for (int nl = 1; nl >= 0; --nl) {
    ValueMap cond;
    cond.scalar_values["temperature"] = 2000.0;
    cond.vector_values["exchange_potential"] = {2.0};
    IsingState state(IsingConfiguration({25, 25}, 1), cond);
    auto system = std::make_shared<IsingSystem>(IsingFormationEnergy(0.1, 1, nl == 1), IsingParamComposition());
    SemiGrandCanonicalPotential pot(system);
    pot.set_state(&state, std::make_shared<SemiGrandCanonicalConditions>(
                              SemiGrandCanonicalConditions::from_values(state.conditions)));
    std::printf("kat %.17g %.17g %.17g %.17g %.17g %.17g\n", system->formation_energy_calculator.per_supercell(),
                system->formation_energy_calculator.per_unitcell(),
                system->formation_energy_calculator.occ_delta_per_supercell({0}, {-1}),
                system->param_composition_calculator.per_supercell()[0],
                system->param_composition_calculator.occ_delta_per_supercell({0}, {-1})[0], pot.per_supercell());
  }
  // random configuration, both paths, multi-site delta
  std::mt19937_64 g(11);
  IsingState state(IsingConfiguration({7, 9}, 1), ValueMap());
  std::vector<int> occ(63);
  for (auto& v : occ) v = std::uniform_int_distribution<long>(0, 1)(g) ? 1 : -1;
  state.configuration.set_occupation(occ);
  IsingFormationEnergy a(0.37, 1, true, &state), b(0.37, 1, false, &state);
  std::printf("occ");
  for (int v : occ) std::printf(" %d", v);
  std::printf("\nrand %.17g %.17g %.17g %.17g\n", a.per_supercell(), b.per_supercell(),
              a.occ_delta_per_supercell({5, 6, 12}, {-occ[5], -occ[6], -occ[12]}),
              b.occ_delta_per_supercell({5, 6, 12}, {-occ[5], -occ[6], -occ[12]}));
  // proposals
  auto eng = std::make_shared<std::mt19937_64>(2024);
  std::mt19937_64 ref(2024);
  RandomNumberGenerator<> rng(eng);
  SemiGrandCanonicalEventGenerator<> gen;
  gen.set_state(&state);
  for (int k = 0; k < 500; ++k) {
    const OccEvent& e = gen.propose(rng);
    const long l = std::uniform_int_distribution<long>(0, 62)(ref);
    if (e.linear_site_index[0] != l || e.new_occ[0] != -state.configuration.occ(l)) { std::printf("draw mismatch\n"); return 1; }
    gen.apply(e);
  }
  try {
    SemiGrandCanonicalConditions::from_values(ValueMap());
    return 1;
  } catch (const std::runtime_error& err) {
    std::printf("caught: %s\n", err.what());
  }
  if (false) {  // linked, not run: the GPU loop
    std::mt19937_64 e2(1);
    SemiGrandCanonicalPotential p2(std::make_shared<IsingSystem>(IsingFormationEnergy(), IsingParamComposition()));
    run_metropolis_passes(state, p2, 1, e2);
  }
  return 0;
}
'''


def test_cpp_ising_model(tmp_path):
    src = tmp_path / "ising.cpp"
    src.write_text(SRC)
    exe = tmp_path / "ising"
    libdir = os.path.dirname(_lib.LIB_PATH)
    _lib.lib()
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        "-L", libdir, "-lmontegpu", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.splitlines()
    for line in lines[:2]:
        assert [float(x) for x in line.split()[1:]] == [-125.0, -0.2, 0.8, 625.0, -1.0, -1375.0]
    occ = np.array([int(x) for x in lines[2].split()[1:]], dtype=np.int32)
    e_nl, e_rows, d_nl, d_rows = (float(x) for x in lines[3].split()[1:])
    assert e_nl == e_rows and d_nl == d_rows
    state = ising.IsingState(ising.IsingConfiguration(shape=(7, 9)), monte.ValueMap())
    state.configuration.set_occupation(occ)
    for use_nlist in (True, False):
        fe = ising.IsingFormationEnergy(J=0.37, lattice_type=1, use_nlist=use_nlist)
        fe.set_state(state)
        assert fe.per_supercell() == e_nl
        assert fe.occ_delta_per_supercell([5, 6, 12], [-occ[5], -occ[6], -occ[12]]) == d_nl
    assert lines[4].startswith("caught: Error in SemiGrandCanonicalConditions")
