"""The ternary word layout's monomial counts (generated counts_quad, tq_coef, tq_const in
csrc/generated/fcc_ternary.cuh) reproduce the per-site local features exactly.

The generated header is compiled for the host (its device qualifiers defined away) together
with the per-site features(): on random ternary lattices, for every word of four sites
(i0 + tQ, t = 0..3) and every feature k, F[k] of site t must equal
tq_const(k) + sum_j tq_coef(k, j) * (byte t of M[j]).  The Python expansion
(codegen.ternary_count_groups) is checked the same way against the feature terms."""
import os
import subprocess

import numpy as np

from casmcode_monte_gb300.clex import codegen
from casmcode_monte_gb300.clex import orbits as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GEN = os.path.join(ROOT, "casmcode_monte_gb300", "csrc", "generated")

SRC = r'''
#include <cstdio>
#include <cstdlib>
#include <random>
#define __host__
#define __device__
#define __forceinline__ inline
#include "fcc_ternary.cuh"
using namespace mg::fcc_ternary;
static int L0 = 16, L1 = 12, L2 = 10;
static int occ[16 * 12 * 10];
static int wrap(int a, int n) { return ((a % n) + n) % n; }
struct Site {  // code psi_0 = o - 1 of a neighbour
  int i, j, k;
  int operator()(int di, int dj, int dk) const {
    return occ[wrap(i + di, L0) + L0 * (wrap(j + dj, L1) + L1 * wrap(k + dk, L2))] - 1;
  }
};
struct Word {  // four sites i + tQ: occupant bytes
  int i, j, k;
  uint32_t operator()(int di, int dj, int dk) const {
    uint32_t w = 0;
    for (int t = 0; t < 4; ++t)
      w |= (uint32_t)occ[wrap(i + t * (L0 / 4) + di, L0) + L0 * (wrap(j + dj, L1) + L1 * wrap(k + dk, L2))] << (8 * t);
    return w;
  }
};
int main() {
  std::mt19937 g(7);
  long bad = 0, checked = 0;
  for (int rep = 0; rep < 3; ++rep) {
    for (int& o : occ) o = (int)(g() % 3);
    for (int k = 0; k < L2; ++k)
      for (int j = 0; j < L1; ++j)
        for (int i = 0; i < L0 / 4; ++i) {
          uint32_t M[NCOUNT];
          counts_quad(Word{i, j, k}, M);
          for (int t = 0; t < 4; ++t) {
            int F[NFEAT];
            features(Site{i + t * (L0 / 4), j, k}, F);
            for (int f = 0; f < NFEAT; ++f) {
              long v = tq_const(f);
              for (int q = 0; q < NCOUNT; ++q) v += (long)tq_coef(f, q) * (long)((M[q] >> (8 * t)) & 0xFFu);
              bad += v != F[f];
              ++checked;
            }
          }
        }
  }
  std::printf("checked %ld bad %ld\n", checked, bad);
  return bad != 0;
}
'''


def test_generated_counts_reproduce_features(tmp_path):
    src = tmp_path / "tq.cpp"
    src.write_text(SRC)
    exe = tmp_path / "tq"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", GEN, str(src), "-o", str(exe)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0" in r.stdout and "checked 0 " not in r.stdout


def test_count_expansion_matches_feature_terms():
    bs = O.make_basis_set("fcc_ternary")
    groups, coef, const = codegen.ternary_count_groups(bs)
    rng = np.random.default_rng(3)
    psi = {0: lambda o: o - 1, 1: lambda o: 1 if o != 1 else -2}
    for _ in range(20):
        occ = {o: int(rng.integers(0, 3)) for o in bs.neighbour_offsets()}
        ind = {(o, "u"): int(v != 1) for o, v in occ.items()}
        ind.update({(o, "s"): int(v == 2) for o, v in occ.items()})
        counts = [sum(int(np.prod([ind[x] for x in m])) for m in g) for g in groups]
        for k, f in enumerate(bs.features):
            direct = sum(int(np.prod([psi[b](occ[o]) for o, b in t])) for t in f.terms)
            assert direct == const[k] + sum(c * n for c, n in zip(coef[k], counts)), k
