"""The C++ facade's chain pool (montegpu::CePool in include/montegpu.hpp) on the GPU: a C++
program admits three chains of mixed shapes with one add_many call, sweeps them 4 passes and
prints the per-pass outputs and final occupations; the Python pool (clex.ChainPool, checked
against the oracle elsewhere) on the same inputs gives the same numbers exactly."""
import json
import os
import subprocess

import numpy as np
import pytest

from casmcode_monte_gb300 import _lib, clex

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r'''
#include <cstdio>
#include <iostream>
#include "montegpu.hpp"
int main() {
  int n_eci = 0;
  std::cin >> n_eci;
  std::vector<double> eci(n_eci);
  for (auto& v : eci) std::cin >> v;
  int n = 0;
  std::cin >> n;
  std::vector<int32_t> dims(3 * n);
  std::vector<double> T(n), mu(n);
  std::vector<uint64_t> seeds(n);
  std::vector<uint32_t> ids(n);
  long long total = 0;
  for (int i = 0; i < n; ++i) {
    std::cin >> dims[3 * i] >> dims[3 * i + 1] >> dims[3 * i + 2] >> T[i] >> mu[i] >> seeds[i] >> ids[i];
    total += (long long)dims[3 * i] * dims[3 * i + 1] * dims[3 * i + 2];
  }
  std::vector<int8_t> occ(total);
  for (auto& v : occ) { int x; std::cin >> x; v = (int8_t)x; }
  montegpu::CeModel m(0, eci);
  montegpu::CePool pool(m, total + (1 << 16), 8);
  auto slots = pool.add_many(dims, T, mu, seeds, ids, occ);
  auto out = pool.run(slots, 4);
  std::printf("{\"launches\": %d, \"out\": [", pool.last_launches());
  for (size_t k = 0; k < out.size(); ++k) std::printf("%s%lld", k ? ", " : "", out[k]);
  std::printf("], \"occ\": [");
  bool first = true;
  for (int s : slots)
    for (int8_t v : pool.occupation(s)) { std::printf("%s%d", first ? "" : ", ", (int)v); first = false; }
  std::printf("]}\n");
  montegpu::release_cached_memory();
  return 0;
}
'''


def test_cpp_pool_matches_python_pool(gpu_lib, tmp_path):
    model = clex.ClexModel("fcc_binary", clex.make_eci("fcc_binary", 4))
    rng = np.random.default_rng(21)
    shapes = [(8, 8, 8), (16, 16, 16), (12, 8, 10)]
    occs = [clex.random_occupation(2, int(np.prod(L)), rng) for L in shapes]
    T = [700.0, 1100.0, 1700.0]
    mu = [0.0, 0.05, -0.03]
    seeds = [11, 12, 13]
    ids = [0, 1, 2]
    src = tmp_path / "pool.cpp"
    src.write_text(SRC)
    exe = tmp_path / "pool"
    libdir = os.path.dirname(_lib.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        "-L", libdir, "-lmontegpu", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = [str(len(model.eci)), " ".join(repr(float(v)) for v in model.eci), str(len(shapes))]
    for L, t, m, s, i in zip(shapes, T, mu, seeds, ids):
        lines.append(f"{L[0]} {L[1]} {L[2]} {t!r} {m!r} {s} {i}")
    lines.append(" ".join(str(int(v)) for o in occs for v in o))
    r = subprocess.run([str(exe)], input="\n".join(lines), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr
    got = json.loads(r.stdout)
    pool = clex.ChainPool(model, arena_bytes=sum(o.size for o in occs) + (1 << 16), max_chains=8)
    slots = pool.add_many(shapes, occs, T, np.array(mu)[:, None], seeds, ids)
    ref = pool.run(slots, 4)
    assert got["out"] == ref.reshape(-1).tolist()
    assert got["occ"] == np.concatenate([pool.occupation(s) for s in slots]).astype(int).tolist()
    assert got["launches"] >= 1
    pool.close()
