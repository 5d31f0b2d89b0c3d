"""The C++ facade (include/montegpu.hpp) compiles with g++, links the library, and its
host entry points behave as the C-ABI does: exceptions carry the "Error in ..." message,
the engine reproduces std::mt19937_64 with libstdc++'s distributions, the colouring and
the statistics agree with the Python layer.  No device computation."""
import os
import subprocess

import numpy as np
from casmcode_monte_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r'''
#include <cstdio>
#include <random>
#include "montegpu.hpp"
int main() {
  montegpu::RandomNumberEngine e(false);
  e.seed(2024);
  std::mt19937_64 ref(2024);
  for (int i = 0; i < 1000; ++i) {
    const long a = (long)e.random_int(624);
    const long b = std::uniform_int_distribution<long>(0, 624)(ref);
    if (a != b) { std::printf("int mismatch\n"); return 1; }
    const double x = e.random_real(1.0);
    const double y = std::uniform_real_distribution<double>(0.0, 1.0)(ref);
    if (x != y) { std::printf("real mismatch\n"); return 1; }
  }
  auto c = montegpu::color_supercell(0, 64, 64, 64);
  std::printf("colours %d layout %d\n", c.n_colors, c.layout);
  try {
    montegpu::color_supercell(0, 2, 64, 64);
    std::printf("no exception\n");
    return 1;
  } catch (const std::runtime_error& err) {
    std::printf("caught: %s\n", err.what());
  }
  std::vector<double> obs(1000);
  std::mt19937_64 g(7);
  for (auto& v : obs) v = std::uniform_real_distribution<double>(0.0, 1.0)(g);
  auto st = montegpu::basic_statistics(obs);
  std::printf("mean %.17g precision %.17g\n", st.first, st.second);
  // the chain pool: without a device its creation throws the library's message; with one,
  // add_many checks its argument sizes on the host before any device work
  try {
    montegpu::CeModel m(0, std::vector<double>(10, 0.01));
    montegpu::CePool pool(m, 1 << 20, 4);
    try {
      pool.add_many({8, 8, 8}, {1000.0, 900.0}, {0.0}, {1}, {0}, std::vector<int8_t>(512, 0));
      std::printf("pool: no exception\n");
      return 1;
    } catch (const std::runtime_error& err) {
      std::printf("pool: %s\n", err.what());
    }
  } catch (const std::runtime_error& err) {
    std::printf("pool: %s\n", err.what());
  }
  return 0;
}
'''


def test_cpp_facade(tmp_path):
    src = tmp_path / "facade.cpp"
    src.write_text(SRC)
    exe = tmp_path / "facade"
    libdir = os.path.dirname(_lib.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        "-L", libdir, "-lmontegpu", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.splitlines()
    assert lines[0] == "colours 16 layout 2"
    assert lines[1].startswith("caught: Error in mg_ce_color_supercell")
    mean, prec = (float(x) for x in lines[2].split()[1::2])
    assert lines[3].startswith("pool: Error in CePool::add_many: argument sizes do not match") or \
        lines[3].startswith("pool: CUDA error") or lines[3].startswith("pool: Error in mg_ce_pool_create"), lines[3]
    import casmcode_monte_gb300 as monte
    from casmcode_monte_gb300.sampling import BasicStatisticsCalculator

    e = monte.RandomNumberEngine()
    e.seed(7)
    rng = monte.RandomNumberGenerator(e)
    obs = np.array([rng.random_real(1.0) for _ in range(1000)])
    st = BasicStatisticsCalculator(confidence=0.95)(obs)
    assert mean == st.mean and prec == st.calculated_precision
