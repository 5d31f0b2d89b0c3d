"""The C++ calculator surface (include/montegpu_ising.hpp, include/montegpu_methods.hpp) on the GPU.

SemiGrandCanonicalCalculator<IsingSystem, SemiGrandCanonicalEventGenerator<>>::run
(basic_semigrand_canonical.hh:416-470) hands its passes to the GPU serial replay; a C++ program
built against libmontegpu.so reproduces the golden 25x25 trajectory (tests/golden/
ising_25x25_seed1.json: 1000 passes, engine seeded 1) bit for bit: final occupation, accepted
count and every potential-energy sample.  The same calculator with an event generator of another
type (same proposals) runs the reference's generic loop (methods::basic_occupation_metropolis)
on the host; with a convergence request both runs must stop at the same pass with the same
samples, completion-check results and engine state.
"""
import json
import os
import subprocess

import pytest

from casmcode_monte_gb300 import _lib

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r'''
#include <cstdio>
#include <iostream>
#include "montegpu_ising.hpp"
using namespace montegpu;
using namespace montegpu::ising_cpp;
using namespace montegpu::ising_cpp::semigrand_canonical;

// the built-in proposal under another type: the calculator runs the generic host loop
struct HostFlip : SemiGrandCanonicalEventGenerator<std::mt19937_64> {};

template <typename Gen>
void scenario(const char* name, std::vector<int> const& occ0, int rows, int cols, double T, double mu,
              monte::CompletionCheckParams<monte::BasicStatistics> const& p, unsigned long long seed, bool first) {
  ValueMap cond;
  cond.scalar_values["temperature"] = T;
  cond.vector_values["exchange_potential"] = {mu};
  IsingConfiguration config({rows, cols}, 1);
  config.set_occupation(occ0);
  IsingState state(config, cond);
  auto system = std::make_shared<IsingSystem>(IsingFormationEnergy(0.1, 1, true), IsingParamComposition());
  auto calc = std::make_shared<SemiGrandCanonicalCalculator<IsingSystem, Gen>>(system);
  monte::StateSamplingFunctionMap fs;
  for (auto const& f : {make_parametric_composition_f(calc), make_formation_energy_f(calc),
                        make_potential_energy_f(calc)})
    fs.emplace(f.name, f);
  auto engine = std::make_shared<std::mt19937_64>(seed);
  auto data = calc->run(state, fs, {}, p, Gen(), 1, std::nullopt, engine);
  auto const& r = data->completion_check.results();
  std::printf("%s\"%s\": {\"n_pass\": %ld, \"n_accept\": %llu, \"n_reject\": %llu, \"n_samples\": %ld, "
              "\"all_equilibrated\": %d, \"all_converged\": %d, \"is_complete\": %d, \"gpu_ms\": %.6f, \"occ\": [",
              first ? "" : ", ", name, (long)data->n_pass, data->n_accept, data->n_reject,
              (long)monte::get_n_samples(data->samplers), (int)r.equilibration_check_results.all_equilibrated,
              (int)r.convergence_check_results.all_converged, (int)r.is_complete, calc->last_kernel_ms);
  auto const& o = state.configuration.occupation();
  for (size_t k = 0; k < o.size(); ++k) std::printf("%s%d", k ? ", " : "", o[k]);
  std::printf("], \"potential_energy\": [");
  auto e = data->samplers.at("potential_energy")->component(0);
  for (size_t k = 0; k < e.size(); ++k) std::printf("%s%.17g", k ? ", " : "", e[k]);
  std::printf("], \"param_composition\": [");
  auto x = data->samplers.at("param_composition")->component(0);
  for (size_t k = 0; k < x.size(); ++k) std::printf("%s%.17g", k ? ", " : "", x[k]);
  std::ostringstream es;
  es << *engine;
  std::printf("], \"engine\": \"%s\"}", es.str().c_str());
}

int main(int argc, char** argv) {
  const bool host_only = argc > 1 && std::string(argv[1]) == "host";
  std::vector<int> occ0(625);
  for (auto& v : occ0) std::cin >> v;
  std::printf("{");
  // convergence of the potential energy to 0.001 (the reference's Python scenario,
  // test_ising_semigrand_canonical_cpp.py), host loop
  monte::CompletionCheckParams<monte::BasicStatistics> q;
  q.cutoff_params.max_count = 4000;
  q.requested_precision.emplace(monte::SamplerComponent("potential_energy", 0, "0"),
                                monte::RequestedPrecision::abs(0.001));
  scenario<HostFlip>("converge_host", occ0, 25, 25, 2000.0, 0.0, q, 7, true);
  if (!host_only) {
    // the golden scenario (1000 passes) and the convergence scenario on the GPU
    monte::CompletionCheckParams<monte::BasicStatistics> p;
    p.cutoff_params.max_count = 1000;
    scenario<SemiGrandCanonicalEventGenerator<std::mt19937_64>>("golden", occ0, 25, 25, 2000.0, 0.0, p, 1, false);
    scenario<SemiGrandCanonicalEventGenerator<std::mt19937_64>>("converge_gpu", occ0, 25, 25, 2000.0, 0.0, q, 7,
                                                                false);
  }
  std::printf("}\n");
  return 0;
}
'''


def _build(tmp_path):
    src = tmp_path / "calc.cpp"
    src.write_text(SRC)
    exe = tmp_path / "calc"
    libdir = os.path.dirname(_lib.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                        str(src), "-o", str(exe), "-L", libdir, "-lmontegpu", f"-Wl,-rpath,{libdir}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_calculator_run_reproduces_golden_and_host_loop(gpu_lib, tmp_path):
    with open(os.path.join(ROOT, "tests", "golden", "ising_25x25_seed1.json")) as f:
        g = json.load(f)
    exe = _build(tmp_path)
    r = subprocess.run([str(exe)], input=" ".join(str(v) for v in g["occ0"]), capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr
    out = json.loads(r.stdout)
    gold = out["golden"]
    assert gold["n_pass"] == g["n_passes"] and gold["n_samples"] == g["n_passes"]
    assert gold["occ"] == g["occ_final"]
    assert gold["n_accept"] == g["n_accept"]
    assert gold["n_accept"] + gold["n_reject"] == 625 * g["n_passes"]
    assert [float.hex(v) for v in gold["potential_energy"]] == g["potential_energy_hex"]
    assert gold["gpu_ms"] > 0.0
    a, b = out["converge_gpu"], out["converge_host"]
    assert a["gpu_ms"] > 0.0 and b["gpu_ms"] == 0.0
    for k in ("n_pass", "n_accept", "n_reject", "n_samples", "all_equilibrated", "all_converged", "is_complete", "occ",
              "potential_energy", "param_composition", "engine"):
        assert a[k] == b[k], k
    assert a["is_complete"] == 1 and a["all_converged"] == 1 and a["n_pass"] < 4000
