"""The C++ Ising surface on the GPU: run_metropolis_passes (include/montegpu_ising.hpp) gives the
trajectory of the host loop of basic_occupation_metropolis written with the same header's
potential, event generator and the reference's acceptance (methods/metropolis.hh:26-35: no
draw when dE < 0, else random_real(1.0) < exp(-beta dE)): the same occupation, counts and
engine state after 40 passes of a 24x20 lattice, with and without neighbour lists."""
import os
import subprocess

import pytest

from casmcode_monte_gb300 import _lib

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r'''
#include <cmath>
#include <cstdio>
#include "montegpu_ising.hpp"
using namespace montegpu::ising_cpp;
using namespace montegpu::ising_cpp::semigrand_canonical;
int main() {
  for (int nl = 1; nl >= 0; --nl) {
    ValueMap cond;
    cond.scalar_values["temperature"] = 1700.0;
    cond.vector_values["exchange_potential"] = {0.05};
    IsingConfiguration config({24, 20}, 1);
    std::mt19937_64 g(5);
    std::vector<int> occ(480);
    for (auto& v : occ) v = std::uniform_int_distribution<long>(0, 1)(g) ? 1 : -1;
    config.set_occupation(occ);
    IsingState host(config, cond), dev(config, cond);
    auto cnd = std::make_shared<SemiGrandCanonicalConditions>(SemiGrandCanonicalConditions::from_values(cond));
    SemiGrandCanonicalPotential ph(std::make_shared<IsingSystem>(IsingFormationEnergy(0.1, 1, nl == 1), IsingParamComposition()));
    SemiGrandCanonicalPotential pd(std::make_shared<IsingSystem>(IsingFormationEnergy(0.1, 1, nl == 1), IsingParamComposition()));
    ph.set_state(&host, cnd);
    pd.set_state(&dev, cnd);
    auto eh = std::make_shared<std::mt19937_64>(99);
    std::mt19937_64 ed(99);
    RandomNumberGenerator<> rng(eh);
    SemiGrandCanonicalEventGenerator<> gen;
    gen.set_state(&host);
    unsigned long long acc = 0, rej = 0;
    for (long step = 0; step < 40L * 480; ++step) {
      const OccEvent& e = gen.propose(rng);
      const double dE = ph.occ_delta_per_supercell(e);
      const bool accept = dE < 0.0 || rng.random_real(1.0) < std::exp(-dE * cnd->beta);
      if (accept) { gen.apply(e); ++acc; } else { ++rej; }
    }
    MetropolisCounts c = run_metropolis_passes(dev, pd, 40, ed, nl == 1);
    const bool same = host.configuration.occupation() == dev.configuration.occupation() && *eh == ed &&
                      c.n_accept == acc && c.n_reject == rej;
    std::printf("nlist %d accept %llu same %d\n", nl, acc, same ? 1 : 0);
    if (!same) return 1;
  }
  return 0;
}
'''


def test_cpp_gpu_passes_equal_the_host_loop(gpu_lib, tmp_path):
    src = tmp_path / "ising_gpu.cpp"
    src.write_text(SRC)
    exe = tmp_path / "ising_gpu"
    libdir = os.path.dirname(_lib.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        "-L", libdir, "-lmontegpu", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("same 1") == 2
