"""FCC cluster-expansion Hamiltonians and GPU coloured-sweep chain batches.

The reference plugs a cluster expansion into its semi-grand canonical potential
(include/casm/monte/ising_cpp/basic_semigrand_canonical.hh:104-199: a system provides
``formation_energy_f_type`` and ``param_composition_f_type``); the evaluator itself lives
in the external libcasm-clexulator.  This package provides, for the FCC lattice:

* ``ClexModel``: basis set ("fcc_binary" occupation basis or "fcc_ternary" Chebyshev
  basis; see ``clex.orbits``) + one ECI per symmetrised cluster function;
* ``make_eci``: seeded ECIs N(0, sigma) / max(size, 1)^2;
* ``ChainBatch``: many chains (same supercell) resident on the GPU, advanced by
  graph-coloured Metropolis passes (Philox4x32-10 random numbers keyed per chain);
* ``SemiGrandCanonicalRun``: per-pass samples (formation/potential energy per unit cell,
  parametric composition) derived exactly from the integer correlation sums.
"""
from __future__ import annotations

import ctypes as C
import json
import os
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from .. import _lib

KB = 8.6173303e-05  # eV/K (libcasm-global)
_GEN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "csrc", "generated")
BASIS_KINDS = {"fcc_binary": 0, "fcc_ternary": 1}


def basis_description(kind: str) -> dict:
    """Classes, features and site basis of a generated basis set (JSON written by codegen)."""
    if kind not in BASIS_KINDS:
        raise ValueError(f"Error: unknown basis set '{kind}' (expected one of {sorted(BASIS_KINDS)})")
    with open(os.path.join(_GEN, f"{kind}.json")) as f:
        return json.load(f)


def make_eci(kind: str, seed: int, sigma: float = 0.03) -> np.ndarray:
    """ECI per class: N(0, sigma) scaled by 1 / max(cluster size, 1)^2 (numpy PCG64 stream)."""
    d = basis_description(kind)
    rng = np.random.default_rng(seed)
    v = rng.normal(0.0, sigma, size=len(d["classes"]))
    sizes = np.array([max(c["size"], 1) for c in d["classes"]], dtype=float)
    return v / sizes**2


class ClexModel:
    """A cluster-expansion formation energy on the FCC lattice (handle to mg_ce_model)."""

    def __init__(self, kind: str, eci: Sequence[float]):
        self.kind = kind
        self.desc = basis_description(kind)
        self.eci = np.ascontiguousarray(np.asarray(eci, dtype=np.float64))
        h = C.c_void_p()
        _lib.check(_lib.lib().mg_ce_model_create(BASIS_KINDS[kind], _lib.ptr(self.eci, C.c_double),
                                                 self.eci.size, C.byref(h)))
        self._h = h
        self.n_classes = len(self.desc["classes"])
        self.n_species = self.desc["basis"]["n_species"]
        self.multiplicity = np.array([c["multiplicity"] for c in self.desc["classes"]], dtype=np.int64)
        self.scale = np.array([c["scale"] for c in self.desc["classes"]], dtype=np.float64)
        # E_f per supercell = sum_f w_f * IntCorr_f
        self.class_weight = (self.eci / self.multiplicity) * self.scale

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.mg_ce_model_destroy(h)
            self._h = None

    def formation_per_supercell(self, int_corr: np.ndarray) -> np.ndarray:
        """E_f from integer correlation sums [..., n_classes] (sum over classes in order)."""
        ic = np.asarray(int_corr, dtype=np.float64)
        e = np.zeros(ic.shape[:-1])
        for f in range(self.n_classes):
            e = e + self.class_weight[f] * ic[..., f]
        return e

    def n_x(self, int_corr: np.ndarray, n_sites: int) -> np.ndarray:
        """N * parametric composition from the point correlation sums.

        binary (occupation basis): n_B = sum psi = IntCorr[point];
        ternary (Chebyshev): sum s = n_C - n_A, sum t = N - 3 n_B.
        """
        ic = np.asarray(int_corr, dtype=np.int64)
        if self.n_species == 2:
            return ic[..., 1:2].astype(np.float64)
        ss, st = ic[..., 1], ic[..., 2]
        nB = (n_sites - st) // 3
        nC = (n_sites - nB + ss) // 2
        return np.stack([nB, nC], axis=-1).astype(np.float64)


LAYOUTS = {0: "byte", 1: "word", 2: "word_pipelined", 3: "word_specialised", 4: "grid"}


def color_supercell(kind: str, shape) -> tuple[np.ndarray, int, str]:
    """The sweep's colouring of a supercell (host only): (colour per site, number of
    colours, the layout a batch of this shape uses: "byte", "word" or "word_pipelined")."""
    L0, L1, L2 = (int(x) for x in shape)
    col = np.zeros(L0 * L1 * L2, dtype=np.int32)
    word = C.c_int()
    n = _lib.lib().mg_ce_color_supercell(BASIS_KINDS[kind], L0, L1, L2, _lib.ptr(col, C.c_int32), C.byref(word))
    if n <= 0:
        _lib.check(-n if n else 1)
    return col, n, LAYOUTS[word.value]


def release_cached_memory() -> None:
    """Free the device blocks that closed batches left in the library's cache (later
    batches of a shape seen before reuse them instead of allocating)."""
    _lib.check(_lib.lib().mg_release_cached_memory())


class ChainBatch:
    """Chains of one L0 x L1 x L2 supercell resident on the GPU (handle to mg_ce_batch).

    occ: [n_chains, N] occupant indices (l = i + L0*(j + L1*k)); temperature [n_chains];
    mu [n_chains, n_species-1]; seeds [n_chains] (Philox keys).
    """

    def __init__(self, model: ClexModel, shape: Sequence[int], occ, temperature, mu, seeds,
                 chain_ids=None, precision: str = "fp64", ctas_per_chain: int = 0):
        self.model = model
        self.shape = tuple(int(x) for x in shape)
        L0, L1, L2 = self.shape
        self.n_sites = L0 * L1 * L2
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int8).reshape(-1, self.n_sites))
        self.n_chains = occ.shape[0]
        T = np.ascontiguousarray(np.asarray(temperature, dtype=np.float64).reshape(self.n_chains))
        mu = np.ascontiguousarray(np.asarray(mu, dtype=np.float64).reshape(self.n_chains, model.n_species - 1))
        seeds = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64).reshape(self.n_chains))
        ids = None
        if chain_ids is not None:
            ids = np.ascontiguousarray(np.asarray(chain_ids, dtype=np.uint32).reshape(self.n_chains))
        if precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        self.temperature, self.mu, self.seeds = T, mu, seeds
        self.precision = precision
        h = C.c_void_p()
        _lib.check(_lib.lib().mg_ce_batch_create(
            model._h, L0, L1, L2, self.n_chains, _lib.ptr(T, C.c_double), _lib.ptr(mu, C.c_double),
            _lib.ptr(seeds, C.c_uint64), _lib.ptr(ids, C.c_uint32) if ids is not None else None,
            _lib.ptr(occ, C.c_int8), 0 if precision == "fp64" else 1, int(ctas_per_chain), C.byref(h)))
        self._h = h
        self._read_info()
        self.pass_count = 0

    def _read_info(self) -> None:
        S, nc, nt, sm, lay = C.c_int(), C.c_int(), C.c_int(), C.c_size_t(), C.c_int()
        _lib.check(_lib.lib().mg_ce_batch_info(self._h, C.byref(S), C.byref(nc), C.byref(nt), C.byref(sm)))
        _lib.check(_lib.lib().mg_ce_batch_layout(self._h, C.byref(lay)))
        self.ctas_per_chain, self.n_colors, self.threads, self.smem_bytes = S.value, nc.value, nt.value, sm.value
        self.layout = LAYOUTS[lay.value]

    def autotune(self, probe_passes: int = 3) -> dict:
        """Time every applicable layout and CTA count on these chains (state restored after
        each trial) and keep the fastest; returns the choice and its ms per pass."""
        lay, S, ms = C.c_int(), C.c_int(), C.c_float()
        _lib.check(_lib.lib().mg_ce_batch_autotune(self._h, int(probe_passes), C.byref(lay), C.byref(S), C.byref(ms)))
        self._read_info()
        return {"layout": LAYOUTS[lay.value], "ctas_per_chain": S.value, "ms_per_pass": float(ms.value)}

    def set_layout(self, layout: str) -> None:
        """Sweep with one site per byte ("byte"), four sites per word ("word", L0 a multiple
        of 4 and a colouring that gives sites i and i + L0/4 one colour; byte-parallel
        features for the binary basis, byte-parallel monomial counts for the ternary one),
        and, binary basis only, four sites per word with the features split around the phase
        barrier ("word_pipelined") or the same with warp-specialised CTAs
        ("word_specialised"); ternary basis only, the word layout swept by CTAs on every SM
        ("grid": each chain's lattice in global memory, a grid barrier between colours);
        trajectories are identical."""
        codes = {v: k for k, v in LAYOUTS.items()}
        if layout not in codes:
            raise ValueError(f"layout must be one of {sorted(codes)}")
        _lib.check(_lib.lib().mg_ce_batch_set_layout(self._h, codes[layout]))
        self._read_info()

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.mg_ce_batch_destroy(h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def n_slots(self) -> int:
        return self.model.n_classes + 2

    def run(self, n_passes: int, want_output: bool = True, out: Optional[np.ndarray] = None) -> Optional[np.ndarray]:
        """Advance every chain by n_passes; returns [n_passes, n_chains, n_classes+2] int64
        (written into ``out`` when given, e.g. a pinned host buffer)."""
        if int(n_passes) < 0:
            raise RuntimeError("Error in mg_ce_batch_run: invalid argument")
        if out is not None:
            if out.dtype != np.int64 or not out.flags.c_contiguous or out.size < n_passes * self.n_chains * self.n_slots:
                raise ValueError("out must be a C-contiguous int64 array of n_passes * n_chains * (n_classes+2)")
        elif want_output:
            out = np.zeros((n_passes, self.n_chains, self.n_slots), dtype=np.int64)
        _lib.check(_lib.lib().mg_ce_batch_run(self._h, int(n_passes),
                                              _lib.ptr(out, C.c_longlong) if out is not None else None))
        self.pass_count += n_passes
        return out

    def last_kernel_ms(self) -> float:
        ms = C.c_float()
        _lib.check(_lib.lib().mg_ce_batch_last_kernel_ms(self._h, C.byref(ms)))
        return float(ms.value)

    def last_launches(self) -> int:
        """Sweep kernels launched by the last run (1 unless it rotated)."""
        n = C.c_int()
        _lib.check(_lib.lib().mg_ce_batch_last_launches(self._h, C.byref(n)))
        return int(n.value)

    def rotation_timeline(self) -> np.ndarray:
        """After a rotated run: [n_chains, 6] ms from the run's start to each chain's first
        fast sweep start/end, slow-slot sweep start/end and second fast sweep start/end."""
        ms = np.zeros((self.n_chains, 6), dtype=np.float32)
        _lib.check(_lib.lib().mg_ce_batch_rotation_timeline(self._h, _lib.ptr(ms, C.c_float)))
        return ms

    def rotation(self) -> dict:
        """Rotation over two cluster sizes: {"ctas_fast": 0} when the batch does not rotate,
        else the fast clusters' CTA count and the measured time ratio per pass."""
        S, r = C.c_int(), C.c_double()
        _lib.check(_lib.lib().mg_ce_batch_rotation(self._h, C.byref(S), C.byref(r)))
        return {"ctas_fast": S.value, "ratio": float(r.value)}

    def set_rotation(self, allowed) -> None:
        """Allow (re-plan) or forbid rotation over two cluster sizes; trajectories are the
        same either way.  ``allowed="always"`` rotates every run long enough to have a plan
        (at least 2 n_chains passes), also where one unrotated launch would be faster."""
        mode = 2 if allowed == "always" else (1 if allowed else 0)
        _lib.check(_lib.lib().mg_ce_batch_set_rotation(self._h, mode))

    def occupation(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        """The chains' occupations [n_chains, N] (into ``out`` when given, e.g. a pinned buffer)."""
        if out is None:
            out = np.zeros((self.n_chains, self.n_sites), dtype=np.int8)
        elif out.dtype != np.int8 or not out.flags.c_contiguous or out.size != self.n_chains * self.n_sites:
            raise ValueError("out must be a C-contiguous int8 array of n_chains * N")
        _lib.check(_lib.lib().mg_ce_batch_get_occ(self._h, _lib.ptr(out, C.c_int8)))
        return out

    def set_occupation(self, occ) -> None:
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int8).reshape(self.n_chains, self.n_sites))
        _lib.check(_lib.lib().mg_ce_batch_set_occ(self._h, _lib.ptr(occ, C.c_int8)))

    def corr(self) -> np.ndarray:
        """Integer correlation sums [n_chains, n_classes] recomputed from the occupation."""
        out = np.zeros((self.n_chains, self.model.n_classes), dtype=np.int64)
        _lib.check(_lib.lib().mg_ce_batch_corr(self._h, _lib.ptr(out, C.c_longlong)))
        return out

    def colors(self) -> np.ndarray:
        out = np.zeros(self.n_sites, dtype=np.int32)
        _lib.check(_lib.lib().mg_ce_batch_colors(self._h, _lib.ptr(out, C.c_int32)))
        return out

    def delta_e(self, chain, sites, new_occ) -> np.ndarray:
        """FP64 dE_sgc for proposals (chain, site, new occupant) on the current state."""
        chain = np.ascontiguousarray(np.asarray(chain, dtype=np.int32).reshape(-1))
        sites = np.ascontiguousarray(np.asarray(sites, dtype=np.int64).reshape(-1))
        new_occ = np.ascontiguousarray(np.asarray(new_occ, dtype=np.int8).reshape(-1))
        out = np.zeros(sites.size, dtype=np.float64)
        _lib.check(_lib.lib().mg_ce_batch_delta_e(self._h, _lib.ptr(chain, C.c_int32), _lib.ptr(sites, C.c_longlong),
                                                  _lib.ptr(new_occ, C.c_int8), sites.size, _lib.ptr(out, C.c_double)))
        return out


class CanonicalBatch:
    """Chains of one L0 x L1 x L2 supercell swept at fixed composition on the GPU (handle to
    mg_ce_canon): the canonical swap of the reference (events.propose_canonical_event with
    Metropolis acceptance) made parallel by exchanging the occupants of matched same-colour
    sites, passes alternating between two colourings whose classes connect every site.

    occ: [n_chains, N] occupant indices; temperature [n_chains]; seeds [n_chains] (Philox
    keys).  One CTA per chain: the supercell must fit in shared memory (up to 56^3).
    """

    def __init__(self, model: ClexModel, shape: Sequence[int], occ, temperature, seeds, chain_ids=None,
                 precision: str = "fp64"):
        self.model = model
        self.shape = tuple(int(x) for x in shape)
        L0, L1, L2 = self.shape
        self.n_sites = L0 * L1 * L2
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int8).reshape(-1, self.n_sites))
        self.n_chains = occ.shape[0]
        T = np.ascontiguousarray(np.asarray(temperature, dtype=np.float64).reshape(self.n_chains))
        seeds = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64).reshape(self.n_chains))
        ids = None
        if chain_ids is not None:
            ids = np.ascontiguousarray(np.asarray(chain_ids, dtype=np.uint32).reshape(self.n_chains))
        if precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        self.temperature, self.seeds, self.precision = T, seeds, precision
        h = C.c_void_p()
        _lib.check(_lib.lib().mg_ce_canon_create(
            model._h, L0, L1, L2, self.n_chains, _lib.ptr(T, C.c_double), _lib.ptr(seeds, C.c_uint64),
            _lib.ptr(ids, C.c_uint32) if ids is not None else None, _lib.ptr(occ, C.c_int8),
            0 if precision == "fp64" else 1, C.byref(h)))
        self._h = h
        na, nb, nt, sm = C.c_int(), C.c_int(), C.c_int(), C.c_size_t()
        _lib.check(_lib.lib().mg_ce_canon_info(self._h, C.byref(na), C.byref(nb), C.byref(nt), C.byref(sm)))
        self.n_colors = (na.value, nb.value)
        self.threads, self.smem_bytes = nt.value, sm.value
        self.pass_count = 0

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.mg_ce_canon_destroy(h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def n_slots(self) -> int:
        return self.model.n_classes + 2

    def run(self, n_passes: int, want_output: bool = True) -> Optional[np.ndarray]:
        """Advance every chain by n_passes; returns [n_passes, n_chains, n_classes+2] int64
        (slot 0 accepted swaps, then the batch's layout)."""
        if int(n_passes) < 0:
            raise RuntimeError("Error in mg_ce_canon_run: invalid argument")
        out = None
        if want_output:
            out = np.zeros((n_passes, self.n_chains, self.n_slots), dtype=np.int64)
        _lib.check(_lib.lib().mg_ce_canon_run(self._h, int(n_passes),
                                              _lib.ptr(out, C.c_longlong) if out is not None else None))
        self.pass_count += n_passes
        return out

    def last_kernel_ms(self) -> float:
        ms = C.c_float()
        _lib.check(_lib.lib().mg_ce_canon_last_kernel_ms(self._h, C.byref(ms)))
        return float(ms.value)

    def occupation(self) -> np.ndarray:
        occ = np.zeros((self.n_chains, self.n_sites), dtype=np.int8)
        _lib.check(_lib.lib().mg_ce_canon_get_occ(self._h, _lib.ptr(occ, C.c_int8)))
        return occ

    def corr(self) -> np.ndarray:
        out = np.zeros((self.n_chains, self.model.n_classes), dtype=np.int64)
        _lib.check(_lib.lib().mg_ce_canon_corr(self._h, _lib.ptr(out, C.c_longlong)))
        return out

    def colors(self, which: int) -> np.ndarray:
        """Colouring `which` (0: passes with even index, 1: odd), [N] int32."""
        col = np.zeros(self.n_sites, dtype=np.int32)
        _lib.check(_lib.lib().mg_ce_canon_colors(self._h, int(which), _lib.ptr(col, C.c_int32)))
        return col

    def class_order(self, which: int) -> np.ndarray:
        """The sites of colouring `which`'s per-colour lists, colour by colour ([N] int32): a
        phase's matching pairs positions k and (d - k) mod n of its colour's list."""
        order = np.zeros(self.n_sites, dtype=np.int32)
        _lib.check(_lib.lib().mg_ce_canon_class_order(self._h, int(which), _lib.ptr(order, C.c_int32)))
        return order


class NfoldBatch:
    """Chains of one binary L0 x L1 x L2 supercell run by rejection-free (N-fold way)
    semi-grand canonical dynamics on the GPU (handle to mg_ce_nfold): an event selector for
    the loop of methods.nfold, every event a single-site flip chosen with probability
    proportional to its Metropolis rate, residence times -ln(u) / R.  At most 32768 sites.

    ``run(n)`` returns [n, n_chains, n_classes + 2] float64: per pass (N events) its time,
    the total rate at its end, and the time-weighted integer correlation sums.
    """

    def __init__(self, model: ClexModel, shape: Sequence[int], occ, temperature, mu, seeds, chain_ids=None):
        self.model = model
        self.shape = tuple(int(x) for x in shape)
        L0, L1, L2 = self.shape
        self.n_sites = L0 * L1 * L2
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int8).reshape(-1, self.n_sites))
        self.n_chains = occ.shape[0]
        T = np.ascontiguousarray(np.asarray(temperature, dtype=np.float64).reshape(self.n_chains))
        mu = np.ascontiguousarray(np.asarray(mu, dtype=np.float64).reshape(self.n_chains, model.n_species - 1))
        seeds = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64).reshape(self.n_chains))
        ids = None
        if chain_ids is not None:
            ids = np.ascontiguousarray(np.asarray(chain_ids, dtype=np.uint32).reshape(self.n_chains))
        self.temperature, self.mu, self.seeds = T, mu, seeds
        h = C.c_void_p()
        _lib.check(_lib.lib().mg_ce_nfold_create(
            model._h, L0, L1, L2, self.n_chains, _lib.ptr(T, C.c_double), _lib.ptr(mu, C.c_double),
            _lib.ptr(seeds, C.c_uint64), _lib.ptr(ids, C.c_uint32) if ids is not None else None,
            _lib.ptr(occ, C.c_int8), C.byref(h)))
        self._h = h
        nt, cps, sm = C.c_int(), C.c_int(), C.c_size_t()
        _lib.check(_lib.lib().mg_ce_nfold_info(self._h, C.byref(nt), C.byref(cps), C.byref(sm)))
        self.threads, self.chains_per_sm, self.smem_bytes = nt.value, cps.value, sm.value

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.mg_ce_nfold_destroy(h)
            self._h = None

    def __del__(self):
        self.close()

    def run(self, n_passes: int) -> np.ndarray:
        if int(n_passes) < 0:
            raise RuntimeError("Error in mg_ce_nfold_run: invalid argument")
        out = np.zeros((n_passes, self.n_chains, self.model.n_classes + 2), dtype=np.float64)
        _lib.check(_lib.lib().mg_ce_nfold_run(self._h, int(n_passes), _lib.ptr(out, C.c_double)))
        return out

    def last_kernel_ms(self) -> float:
        ms = C.c_float()
        _lib.check(_lib.lib().mg_ce_nfold_last_kernel_ms(self._h, C.byref(ms)))
        return float(ms.value)

    def occupation(self) -> np.ndarray:
        occ = np.zeros((self.n_chains, self.n_sites), dtype=np.int8)
        _lib.check(_lib.lib().mg_ce_nfold_get_occ(self._h, _lib.ptr(occ, C.c_int8)))
        return occ

    def corr(self, recompute: bool = False) -> np.ndarray:
        out = np.zeros((self.n_chains, self.model.n_classes), dtype=np.int64)
        _lib.check(_lib.lib().mg_ce_nfold_corr(self._h, 1 if recompute else 0, _lib.ptr(out, C.c_longlong)))
        return out


class ReplayBatch:
    """Chains of one supercell replaying the reference's semi-grand canonical dynamics on the
    GPU (handle to mg_ce_replay): per step a swap type chosen by random_real over the occupant
    counts, a site by random_int over the chosen species' occupant list, Metropolis acceptance
    with random_real(1.0), occupant lists kept as OccLocation keeps them; each chain consumes
    its std::mt19937_64 exactly as the reference's RandomNumberGenerator would.

    occ: [n_chains, N] occupant indices; temperature [n_chains]; mu [n_chains, n_species-1];
    engine_states: per chain, the engine's text form (``RandomNumberEngine.dump()``).
    """

    def __init__(self, model: ClexModel, shape: Sequence[int], occ, temperature, mu, engine_states):
        self.model = model
        self.shape = tuple(int(x) for x in shape)
        L0, L1, L2 = self.shape
        self.n_sites = L0 * L1 * L2
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int8).reshape(-1, self.n_sites))
        self.n_chains = occ.shape[0]
        T = np.ascontiguousarray(np.asarray(temperature, dtype=np.float64).reshape(self.n_chains))
        mu = np.ascontiguousarray(np.asarray(mu, dtype=np.float64).reshape(self.n_chains, model.n_species - 1))
        if len(engine_states) != self.n_chains:
            raise ValueError("one engine state per chain")
        states = (C.c_char_p * self.n_chains)(*[s.encode() if isinstance(s, str) else s for s in engine_states])
        h = C.c_void_p()
        _lib.check(_lib.lib().mg_ce_replay_create(model._h, L0, L1, L2, self.n_chains, _lib.ptr(T, C.c_double),
                                                  _lib.ptr(mu, C.c_double), _lib.ptr(occ, C.c_int8), states,
                                                  C.byref(h)))
        self._h = h
        self.temperature, self.mu = T, mu

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.mg_ce_replay_destroy(h)
            self._h = None

    def __del__(self):
        self.close()

    def run(self, n_passes: int, want_output: bool = True) -> Optional[np.ndarray]:
        """n_passes passes of N steps; returns [n_passes, n_chains, n_classes+2] int64: accepted
        steps, the change of each integer correlation sum (classes 1..), rejected steps, 0."""
        if int(n_passes) < 0:
            raise RuntimeError("Error in mg_ce_replay_run: invalid argument")
        out = np.zeros((n_passes, self.n_chains, self.model.n_classes + 2), dtype=np.int64) if want_output else None
        _lib.check(_lib.lib().mg_ce_replay_run(self._h, int(n_passes),
                                               _lib.ptr(out, C.c_longlong) if out is not None else None))
        return out

    def occupation(self) -> np.ndarray:
        occ = np.zeros((self.n_chains, self.n_sites), dtype=np.int8)
        _lib.check(_lib.lib().mg_ce_replay_get_occ(self._h, _lib.ptr(occ, C.c_int8)))
        return occ

    def engine_state(self, chain: int) -> str:
        buf = C.create_string_buffer(16384)
        _lib.check(_lib.lib().mg_ce_replay_engine_state(self._h, int(chain), buf, len(buf)))
        return buf.value.decode()

    def candidates(self, chain: int) -> list:
        """The chain's occupant lists (one per species, list order), as OccLocation holds them."""
        sizes = np.zeros(self.model.n_species, dtype=np.int32)
        sites = np.zeros(self.n_sites, dtype=np.int32)
        _lib.check(_lib.lib().mg_ce_replay_candidates(self._h, int(chain), _lib.ptr(sizes, C.c_int32),
                                                      _lib.ptr(sites, C.c_int32)))
        out, off = [], 0
        for n in sizes:
            out.append(sites[off:off + n].copy())
            off += int(n)
        return out

    def counts(self) -> tuple[np.ndarray, np.ndarray]:
        """Accepted and rejected steps per chain since creation."""
        a = np.zeros(self.n_chains, dtype=np.uint64)
        r = np.zeros(self.n_chains, dtype=np.uint64)
        _lib.check(_lib.lib().mg_ce_replay_counts(self._h, _lib.ptr(a, C.c_ulonglong), _lib.ptr(r, C.c_ulonglong)))
        return a, r

    def last_kernel_ms(self) -> float:
        ms = C.c_float()
        _lib.check(_lib.lib().mg_ce_replay_last_kernel_ms(self._h, C.byref(ms)))
        return float(ms.value)


class PoolFull(RuntimeError):
    """Admission refused: no free chain slot or not enough arena memory."""


class ChainPool:
    """Chains of any supercell shape in one HBM arena (handle to mg_ce_pool).

    ``add`` admits a chain if its occupation fits in the arena (raises ``PoolFull``
    otherwise); ``run(slots, n_passes)`` sweeps the given chains in one launch of the
    persistent pool kernel; each chain keeps its own pass counter.
    """

    def __init__(self, model: ClexModel, arena_bytes: int, max_chains: int, precision: str = "fp64"):
        if precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        self.model = model
        h = C.c_void_p()
        _lib.check(_lib.lib().mg_ce_pool_create(model._h, int(arena_bytes), int(max_chains),
                                                0 if precision == "fp64" else 1, C.byref(h)))
        self._h = h
        self.shapes: dict = {}

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.mg_ce_pool_destroy(h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def n_slots(self) -> int:
        return self.model.n_classes + 2

    def add(self, shape, occ, temperature: float, mu, seed: int, chain_id: int) -> int:
        L0, L1, L2 = (int(x) for x in shape)
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int8).reshape(-1))
        mu = np.ascontiguousarray(np.asarray(mu, dtype=np.float64).reshape(self.model.n_species - 1))
        slot = C.c_int()
        rc = _lib.lib().mg_ce_pool_add(self._h, L0, L1, L2, float(temperature), _lib.ptr(mu, C.c_double),
                                       C.c_uint64(int(seed)), C.c_uint32(int(chain_id)), _lib.ptr(occ, C.c_int8),
                                       C.byref(slot))
        if rc == 5:
            raise PoolFull(_lib.lib().mg_last_error().decode())
        _lib.check(rc)
        self.shapes[slot.value] = (L0, L1, L2)
        return slot.value

    def add_many(self, shapes, occs, temperatures, mu, seeds, chain_ids) -> list:
        """Admit n chains in one call (all or none): ``shapes`` n triples, ``occs`` n
        occupations, ``temperatures``/``seeds``/``chain_ids`` length n, ``mu`` [n, n_species-1].
        Returns the slots, the ones n calls of ``add`` would give."""
        n = len(shapes)
        dims = np.ascontiguousarray(np.asarray(shapes, dtype=np.int32).reshape(n, 3))
        occ = np.ascontiguousarray(np.concatenate([np.asarray(o, dtype=np.int8).reshape(-1) for o in occs])
                                   if n else np.zeros(0, dtype=np.int8))
        if occ.size != int(np.prod(dims.astype(np.int64), axis=1).sum()):
            raise ValueError("occupation sizes do not match the shapes")
        T = np.ascontiguousarray(np.asarray(temperatures, dtype=np.float64).reshape(n))
        mu = np.ascontiguousarray(np.asarray(mu, dtype=np.float64).reshape(n, self.model.n_species - 1))
        sd = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64).reshape(n))
        ids = np.ascontiguousarray(np.asarray(chain_ids, dtype=np.uint32).reshape(n))
        slots = np.zeros(n, dtype=np.int32)
        rc = _lib.lib().mg_ce_pool_add_many(self._h, n, _lib.ptr(dims, C.c_int32), _lib.ptr(T, C.c_double),
                                            _lib.ptr(mu, C.c_double), _lib.ptr(sd, C.c_uint64),
                                            _lib.ptr(ids, C.c_uint32), _lib.ptr(occ, C.c_int8),
                                            _lib.ptr(slots, C.c_int32))
        if rc == 5:
            raise PoolFull(_lib.lib().mg_last_error().decode())
        _lib.check(rc)
        out = [int(s) for s in slots]
        for s, d in zip(out, dims):
            self.shapes[s] = tuple(int(x) for x in d)
        return out

    def prepare(self, shape) -> None:
        """Build and cache the geometry (colouring, site lists) of a supercell shape."""
        L0, L1, L2 = (int(x) for x in shape)
        _lib.check(_lib.lib().mg_ce_pool_prepare(self._h, L0, L1, L2))

    def remove(self, slot: int) -> None:
        _lib.check(_lib.lib().mg_ce_pool_remove(self._h, int(slot)))
        self.shapes.pop(slot, None)

    def info(self) -> dict:
        fb, ab, nu, mc = C.c_longlong(), C.c_longlong(), C.c_int(), C.c_int()
        _lib.check(_lib.lib().mg_ce_pool_info(self._h, C.byref(fb), C.byref(ab), C.byref(nu), C.byref(mc)))
        return {"arena_free_bytes": fb.value, "arena_bytes": ab.value, "n_used": nu.value, "max_chains": mc.value}

    def run(self, slots, n_passes: int, want_output: bool = True,
            out: Optional[np.ndarray] = None) -> Optional[np.ndarray]:
        """Sweep the chains in ``slots``; returns [len(slots), n_passes, n_classes+2] int64
        (written into ``out`` when given, e.g. a pinned host buffer)."""
        if int(n_passes) < 0:
            raise RuntimeError("Error in mg_ce_pool_run: invalid argument")
        sl = np.ascontiguousarray(np.asarray(slots, dtype=np.int32).reshape(-1))
        if out is not None:
            if out.dtype != np.int64 or not out.flags.c_contiguous or out.size < sl.size * n_passes * self.n_slots:
                raise ValueError("out must be a C-contiguous int64 array of len(slots) * n_passes * (n_classes+2)")
        elif want_output:
            out = np.zeros((sl.size, n_passes, self.n_slots), dtype=np.int64)
        _lib.check(_lib.lib().mg_ce_pool_run(self._h, _lib.ptr(sl, C.c_int32), sl.size, int(n_passes),
                                             _lib.ptr(out, C.c_longlong) if out is not None else None))
        return out

    def last_kernel_ms(self) -> float:
        ms = C.c_float()
        _lib.check(_lib.lib().mg_ce_pool_last_kernel_ms(self._h, C.byref(ms)))
        return float(ms.value)

    def last_launches(self) -> int:
        """Kernels the last run launched (one per CTA class and layout with chains, plus the
        series kernel when series are on)."""
        n = C.c_int()
        _lib.check(_lib.lib().mg_ce_pool_last_launches(self._h, C.byref(n)))
        return int(n.value)

    def occupation(self, slot: int) -> np.ndarray:
        n = int(np.prod(self.shapes[slot]))
        occ = np.zeros(n, dtype=np.int8)
        _lib.check(_lib.lib().mg_ce_pool_get_occ(self._h, int(slot), _lib.ptr(occ, C.c_int8)))
        return occ

    def colors(self, slot: int) -> tuple[np.ndarray, int]:
        n = int(np.prod(self.shapes[slot]))
        col = np.zeros(n, dtype=np.int32)
        nc = _lib.lib().mg_ce_pool_colors(self._h, int(slot), _lib.ptr(col, C.c_int32))
        if nc <= 0:
            _lib.check(nc if nc else 1)
        return col, nc

    def corr(self, slot: int) -> np.ndarray:
        out = np.zeros(self.model.n_classes, dtype=np.int64)
        _lib.check(_lib.lib().mg_ce_pool_corr(self._h, int(slot), _lib.ptr(out, C.c_longlong)))
        return out

    def enable_series(self, max_samples: int) -> None:
        """Keep a device-resident potential-energy-per-site sample per pass (before adds)."""
        _lib.check(_lib.lib().mg_ce_pool_enable_series(self._h, int(max_samples)))
        self.max_samples = int(max_samples)

    def series(self, slot: int) -> np.ndarray:
        buf = np.zeros(self.max_samples, dtype=np.float64)
        n = C.c_int()
        _lib.check(_lib.lib().mg_ce_pool_series(self._h, int(slot), _lib.ptr(buf, C.c_double), buf.size,
                                                C.byref(n)))
        return buf[: min(n.value, buf.size)].copy()

    def check(self, slots, abs_precision: float, confidence: float = 0.95) -> np.ndarray:
        """Device equilibration + convergence check of each slot's series.

        Returns [n, 6]: equilibrated, N_equilibration, N_statistics, mean, precision, converged.
        """
        sl = np.ascontiguousarray(np.asarray(slots, dtype=np.int32).reshape(-1))
        out = np.zeros((sl.size, 6), dtype=np.float64)
        _lib.check(_lib.lib().mg_ce_pool_check(self._h, _lib.ptr(sl, C.c_int32), sl.size, float(abs_precision),
                                               float(confidence), _lib.ptr(out, C.c_double)))
        return out


@dataclass
class SweepSamples:
    """Per-pass observables of a batch run (arrays [n_passes, n_chains])."""

    int_corr: np.ndarray          # [n_passes, n_chains, n_classes] after each pass
    formation_energy: np.ndarray  # per unit cell
    potential_energy: np.ndarray  # per unit cell
    param_composition: np.ndarray  # [n_passes, n_chains, n_species-1]
    n_accept: np.ndarray
    n_exact: np.ndarray
    n_flipped: np.ndarray


def accumulate(model: ClexModel, corr0: np.ndarray, out: np.ndarray, mu: np.ndarray, n_sites: int) -> SweepSamples:
    """Cumulative integer correlations and the observables for each pass.

    corr0: [n_chains, n_classes] before the passes; out: ChainBatch.run output.
    """
    nc = model.n_classes
    d = out[:, :, :nc].copy()
    d[:, :, 0] = 0
    ic = corr0[None, :, :] + np.cumsum(d, axis=0)
    ef = model.formation_per_supercell(ic)
    nx = model.n_x(ic, n_sites)
    pe = ef.copy()
    for i in range(model.n_species - 1):
        pe = pe - mu[None, :, i] * nx[..., i]
    return SweepSamples(ic, ef / n_sites, pe / n_sites, nx / n_sites, out[:, :, 0], out[:, :, nc], out[:, :, nc + 1])


def random_occupation(n_species: int, n_sites: int, rng: np.random.Generator,
                      composition: Optional[Sequence[float]] = None) -> np.ndarray:
    """Occupation with exact species counts (rounded composition) placed by a seeded shuffle."""
    if composition is None:
        composition = [1.0 / n_species] * n_species
    counts = [int(round(c * n_sites)) for c in composition]
    counts[-1] = n_sites - sum(counts[:-1])
    occ = np.concatenate([np.full(c, s, dtype=np.int8) for s, c in enumerate(counts)])
    rng.shuffle(occ)
    return occ


__all__ = ["ClexModel", "ChainBatch", "CanonicalBatch", "NfoldBatch", "ChainPool", "PoolFull", "SweepSamples", "accumulate", "basis_description", "make_eci",
           "random_occupation", "KB"]
