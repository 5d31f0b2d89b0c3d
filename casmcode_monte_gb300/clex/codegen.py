"""Generate CUDA feature functions and a JSON description for an FCC basis set.

CASM generates one C++ "Clexulator" per basis set (``ZrO_Clexulator.cc`` in the
reference's test data is such a file).  Here the same idea targets the GPU sweep: the
cluster geometry is compiled into straight-line integer code so that every neighbour load
uses a constant offset and every product is an integer multiply-add.

Generated for each basis set ``<name>``:

* ``csrc/generated/<name>.cuh``: ``features(ld, F)`` (the local sums F[k] of
  ``orbits.local_features``) and ``anchored(ld, C)`` (per-site contributions to the
  integer correlation sums of every class), both templated on a loader ``ld(di,dj,dk)``
  that returns the occupant code stored for the neighbour at primitive offset
  (di,dj,dk).  Binary stores ``occ`` (0/1), ternary stores ``s = occ-1`` (-1/0/1).
* ``csrc/generated/<name>.json``: classes (size, multiplicity, decoration multiset,
  squared pair distances, scale C_f), features (class, basis index at the site, bound
  on |F|) and the site basis, read by the host code at run time.

Run ``python -m casmcode_monte_gb300.clex.codegen`` to regenerate (the outputs are
committed).
"""
from __future__ import annotations

import json
import os

from . import orbits as O

HERE = os.path.dirname(os.path.abspath(__file__))
GEN_DIR = os.path.join(os.path.dirname(HERE), "csrc", "generated")


def _psi_expr(basis: O.SiteBasis, b: int, var: str) -> str:
    """C expression of integer psi_b from the stored code ``var``."""
    if basis.name == "occupation":
        assert b == 0
        return var  # stored value is occ in {0,1}
    if basis.name == "chebyshev":
        return var if b == 0 else f"t_{var}"
    raise ValueError(basis.name)


def _sum_expr(terms: list, n_acc: int = 4) -> str:
    """Sum of terms as n_acc interleaved partial sums, so that the products form
    independent multiply-add chains (instruction-level parallelism)."""
    if len(terms) <= n_acc:
        return " + ".join(terms)
    groups = [terms[i::n_acc] for i in range(n_acc)]
    parts = ["(" + " + ".join(g) + ")" for g in groups]
    return "(" + parts[0] + " + " + parts[1] + ") + (" + parts[2] + " + " + parts[3] + ")"


def _var(off) -> str:
    return "v_" + "_".join(("m" + str(-x)) if x < 0 else str(x) for x in off)


def _quad_features(bs, offs) -> list:
    """Byte-parallel features for an occupation basis: every loaded word holds the 0/1
    occupants of four sites (one per byte) and every F[k] the four sites' local sums.

    A product of 0/1 values is a bitwise AND; sums stay below 256 per byte (the largest
    feature of the FCC binary set counts 72 clusters), so byte lanes never carry into each
    other.  Pair products that share a site a are factored as mask(a) & (sum of the
    partners), mask(a) = a * 0xFF (0x00 or 0xFF per byte)."""
    out = ["// Byte-parallel features: ld(di,dj,dk) returns a word of four sites' occupants (one",
           "// per byte); F[k] receives the four sites' local sums, one per byte.",
           "template <class Loader>",
           "__device__ __forceinline__ void features_quad(const Loader& ld, uint32_t (&F)[NFEAT]) {"]
    for o in offs:
        out.append(f"  const uint32_t {_var(o)} = ld({o[0]}, {o[1]}, {o[2]});")
    masks = set()
    body = []
    for k, f in enumerate(bs.features):
        terms = [tuple(_var(o) for o, _ in t) for t in f.terms]
        if all(len(t) == 0 for t in terms):
            body.append(f"  F[{k}] = {len(terms)}u * 0x01010101u;")
            continue
        parts = []
        singles = [t[0] for t in terms if len(t) == 1]
        parts += singles
        pairs = [t for t in terms if len(t) == 2]
        while pairs:
            count: dict = {}
            for a, b in pairs:
                count[a] = count.get(a, 0) + 1
                count[b] = count.get(b, 0) + 1
            v = max(sorted(count), key=lambda x: count[x])
            if count[v] < 3:
                parts += [f"({a} & {b})" for a, b in pairs]
                break
            partners = [b if a == v else a for a, b in pairs if v in (a, b)]
            pairs = [t for t in pairs if v not in t]
            masks.add(v)
            parts.append(f"(m_{v} & ({' + '.join(partners)}))")
        for t in terms:
            if len(t) >= 3:
                parts.append("(" + " & ".join(t) + ")")
        body.append(f"  F[{k}] = " + _sum_expr(parts) + ";")
    for v in sorted(masks):
        out.append(f"  const uint32_t m_{v} = {v} * 0xFFu;")
    out += body
    out.append("}")
    return out


# Linear colourings (a i + b j + c k) mod m of the word-layout pipelines: a = 4 keeps the
# four sites i0 + tQ of a row in one colour whenever L0 is a multiple of 16; (b, c) are
# chosen so that a site has the fewest neighbours in the colour proposed just before its
# own.  Valid when a L0, b L1, c L2 are multiples of m (L0, L1 multiples of 16 and L2 of 8
# for the first; L0, L2 of 16 and L1 of 8 for the second).
PIPELINE_COLOURINGS = [(4, 5, 14, 16), (4, 6, 15, 16)]


def late_offsets(offs, colouring) -> list:
    """Neighbour offsets whose colour is one less (mod m) than the site's own."""
    a, b, c, m = colouring
    assert all((a * o[0] + b * o[1] + c * o[2]) % m for o in offs), "colouring is not proper"
    return [o for o in offs if (a * o[0] + b * o[1] + c * o[2]) % m == m - 1]


def _factor_pairs(pairs, prefer=None) -> tuple[list, set]:
    """Sum of (x & y) pair products as masked partner sums: mask(v) & (sum of v's
    partners), for the variable v in most remaining pairs (or only variables in
    ``prefer``); returns the expression parts and the masks used."""
    parts, masks = [], set()
    pairs = list(pairs)
    while pairs:
        count: dict = {}
        for a, b in pairs:
            for v in (a, b):
                if prefer is None or v in prefer:
                    count[v] = count.get(v, 0) + 1
        if not count:
            parts += [f"({a} & {b})" for a, b in pairs]
            break
        v = max(sorted(count), key=lambda x: count[x])
        if count[v] < 2 and prefer is None:
            parts += [f"({a} & {b})" for a, b in pairs]
            break
        partners = [b if a == v else a for a, b in pairs if v in (a, b)]
        pairs = [t for t in pairs if v not in t]
        if len(partners) == 1:
            parts.append(f"({v} & {partners[0]})")
        else:
            masks.add(v)
            parts.append(f"(m_{v} & ({' + '.join(partners)}))")
    return parts, masks


def _and(vs) -> str:
    return vs[0] if len(vs) == 1 else "(" + " & ".join(vs) + ")"


def _quad_pipelines(bs, offs) -> list:
    """Split byte-parallel features for the word-layout pipelines (see PIPELINE_COLOURINGS).

    For colouring p, early() runs while the previous colour's phase may still be writing:
    it loads every neighbour except the late ones (colour one less than the site's) and
    sums the cluster terms free of late neighbours into E[k].  A term with late part L
    and stable part R contributes AND(L) * AND(R); the terms of feature k that share L
    are summed early into one kept word K = sum AND(R), so that late() only loads the late
    neighbours and adds mask(AND(L)) & K (mask = 0xFF per set byte)."""
    out = ["// ---- word-layout pipelines (early / late split of features_quad)",
           f"constexpr int NPIPE = {len(PIPELINE_COLOURINGS)};",
           "__host__ __device__ constexpr int pipe_colouring(int p, int q) {",
           "  constexpr int t[NPIPE * 4] = {" + ", ".join(str(x) for col in PIPELINE_COLOURINGS for x in col) + "};",
           "  return t[p * 4 + q];  // a, b, c, m",
           "}",
           "template <int P>",
           "struct Pipe;"]
    for p, col in enumerate(PIPELINE_COLOURINGS):
        late_offs = late_offsets(offs, col)
        late = set(_var(o) for o in late_offs)
        stable = [o for o in offs if _var(o) not in late]
        early_lines, masks = [], set()
        kept = []    # (name, expression) computed early
        late_lines = []
        groups_all: list = []  # distinct late parts L (tuples of late variables)
        terms_tab = []         # (group, feature, kept index or -1, count)
        for k, f in enumerate(bs.features):
            terms = [tuple(_var(o) for o, _ in t) for t in f.terms]
            if all(len(t) == 0 for t in terms):
                early_lines.append(f"    s.E[{k}] = {len(terms)}u * 0x01010101u;")
                late_lines.append(f"    F[{k}] = s.E[{k}];")
                continue
            early_t = [t for t in terms if not (set(t) & late)]
            parts = [t[0] for t in early_t if len(t) == 1]
            pp, mm = _factor_pairs([t for t in early_t if len(t) == 2])
            parts += pp
            masks |= mm
            parts += [_and(t) for t in early_t if len(t) >= 3]
            early_lines.append(f"    s.E[{k}] = " + (_sum_expr(parts) if parts else "0u") + ";")
            groups: dict = {}
            for t in terms:
                Lp = tuple(v for v in t if v in late)
                if Lp:
                    groups.setdefault(Lp, []).append(tuple(v for v in t if v not in late))
            lparts = []
            for Lp, Rs in sorted(groups.items()):
                if Lp not in groups_all:
                    groups_all.append(Lp)
                gi = groups_all.index(Lp)
                if all(len(R) == 0 for R in Rs):
                    lparts += [_and(list(Lp))] * len(Rs)
                    terms_tab.append((gi, k, -1, len(Rs)))
                elif len(Rs) == 1:
                    # one term: AND(L) & AND(R), AND(R) kept
                    kept.append((f"K{len(kept)}", _and(list(Rs[0]))))
                    lparts.append(f"({_and(list(Lp))} & s.K[{len(kept) - 1}])")
                    terms_tab.append((gi, k, len(kept) - 1, 1))
                else:
                    kexpr = " + ".join(_and(list(R)) if R else "0x01010101u" for R in Rs)
                    kept.append((f"K{len(kept)}", kexpr))
                    lparts.append(f"((({_and(list(Lp))}) * 0xFFu) & s.K[{len(kept) - 1}])")
                    terms_tab.append((gi, k, len(kept) - 1, 1))
            late_lines.append(f"    F[{k}] = s.E[{k}]" + ("".join(" + " + x for x in lparts)) + ";")
        out.append(f"// colouring ({col[0]} i + {col[1]} j + {col[2]} k) mod {col[3]}: late neighbours "
                   + ", ".join(str(tuple(o)) for o in late_offs))
        out.append("template <>")
        out.append(f"struct Pipe<{p}> {{")
        out.append(f"  static constexpr int NKEEP = {max(1, len(kept))};")
        out.append("  // late groups g (AND of late neighbours); F[k] gains sum over terms (g, k, keep, n) of")
        out.append("  // n * group_g * (keep < 0 ? 1 : K[keep]) per byte")
        out.append(f"  static constexpr int NGROUP = {len(groups_all)};")
        out.append(f"  static constexpr int NTERM = {len(terms_tab)};")
        for name, col_i in (("term_group", 0), ("term_feature", 1), ("term_keep", 2), ("term_count", 3)):
            out.append(f"  __host__ __device__ static constexpr int {name}(int i) {{")
            out.append("    constexpr int t[NTERM] = {" + ", ".join(str(t[col_i]) for t in terms_tab) + "};")
            out.append("    return t[i];")
            out.append("  }")
        out.append("  struct State {")
        out.append("    uint32_t E[NFEAT];")
        out.append("    uint32_t K[NKEEP];")
        out.append("    uint32_t own;")
        out.append("  };")
        out.append("  template <class Loader>")
        out.append("  __device__ static __forceinline__ void early(const Loader& ld, State& s) {")
        for o in stable:
            out.append(f"    const uint32_t {_var(o)} = ld({o[0]}, {o[1]}, {o[2]});")
        out.append("    s.own = ld(0, 0, 0);")
        for v in sorted(masks):
            out.append(f"    const uint32_t m_{v} = {v} * 0xFFu;")
        out += early_lines
        for i, (_, kexpr) in enumerate(kept):
            out.append(f"    s.K[{i}] = {kexpr};")
        out.append("  }")
        out.append("  template <class Loader>")
        out.append("  __device__ static __forceinline__ void late(const Loader& ld, const State& s, uint32_t (&F)[NFEAT],")
        out.append("                                              uint32_t (&Lw)[NGROUP]) {")
        for o in late_offs:
            out.append(f"    const uint32_t {_var(o)} = ld({o[0]}, {o[1]}, {o[2]});")
        out += late_lines
        for gi, Lp in enumerate(groups_all):
            out.append(f"    Lw[{gi}] = {_and(list(Lp))};")
        out.append("  }")
        out.append("};")
    return out


# Site functions of the ternary Chebyshev basis over the indicators u = [o != 1] and
# s = [o == 2] of the occupant o in {0, 1, 2}: psi_0 = o - 1 = 2 s - u, psi_1 = 3 u - 2;
# coefficients of (1, u, s).
_CHEB_IND = {0: (0, -1, 2), 1: (-2, 3, 0)}


def ternary_count_groups(bs):
    """Monomial counts of the ternary word layout.

    Every product of the other sites' psi values in a feature term expands over the
    indicators (u, s) of those sites into monomials (products of one indicator per site, at
    most three sites).  Monomials with the same coefficient in every feature form one
    group; a group's count is the number of its monomials equal to 1, at most the group
    size (below 256, so four sites' counts share a word byte by byte).  Returns
    (groups, coef, const): groups[j] lists the monomials (tuples of (offset, 'u'|'s')),
    coef[k][j] the coefficient of count j in feature k, const[k] the constant term, so that
    F[k] = const[k] + sum_j coef[k][j] count[j]."""
    import itertools as it
    nf = bs.n_features
    mono: dict = {}
    for k, f in enumerate(bs.features):
        for term in f.terms:
            choices = []
            for off, b in term:
                a, be, g = _CHEB_IND[b]
                opts = []
                if a:
                    opts.append(((), a))
                if be:
                    opts.append((((off, "u"),), be))
                if g:
                    opts.append((((off, "s"),), g))
                choices.append(opts)
            for combo in it.product(*choices):
                m = tuple(sorted(sum((c[0] for c in combo), ())))
                c = 1
                for x in combo:
                    c *= x[1]
                mono.setdefault(m, [0] * nf)[k] += c
    const = mono.pop((), [0] * nf)
    by_vec: dict = {}
    for m in sorted(mono):
        v = tuple(mono[m])
        if any(v):
            by_vec.setdefault(v, []).append(m)
    groups = sorted(by_vec.values(), key=lambda ms: ms[0])
    assert all(len(g) < 256 for g in groups)
    coef = [[mono[g[0]][k] for g in groups] for k in range(nf)]
    return groups, coef, const


def _ternary_counts(bs, offs) -> list:
    """Byte-parallel monomial counts for the ternary word layout: ld(di,dj,dk) returns a
    word of four sites' occupants (bytes 0, 1, 2); M[j] receives the four sites' counts of
    group j (ternary_count_groups), one per byte.  Indicators per neighbour word:
    u = (c ^ 0x01010101) & 0x01010101, s = (c >> 1) & 0x01010101; products are ANDs.

    The neighbours are visited in order of distance, and every monomial is added when its
    last neighbour (in that order) arrives, so that a neighbour's indicators are live only
    until its last monomial (at most about 15 neighbours at a time instead of all 54);
    monomials completed by the same neighbour indicator x in one group are summed as
    mask(x) & (sum of the rest), mask(x) = x * 0xFF (0x00 or 0xFF per byte)."""
    groups, coef, const = ternary_count_groups(bs)
    nj = len(groups)
    out = [f"constexpr int NCOUNT = {nj};",
           "// F[k] = tq_const(k) + sum_j tq_coef(k, j) M[j] (M: monomial counts of counts_quad)",
           "__host__ __device__ constexpr int tq_coef(int k, int j) {",
           "  constexpr int t[NFEAT][NCOUNT] = {" + ", ".join(
               "{" + ", ".join(str(x) for x in row) + "}" for row in coef) + "};",
           "  return t[k][j];",
           "}",
           "__host__ __device__ constexpr int tq_const(int k) {",
           "  constexpr int t[NFEAT] = {" + ", ".join(str(x) for x in const) + "};",
           "  return t[k];",
           "}",
           "// Byte-parallel monomial counts of four sites (one per byte) from words of occupants.",
           "template <class Loader>",
           "__device__ __forceinline__ void counts_quad(const Loader& ld, uint32_t (&M)[NCOUNT]) {"]
    used = sorted({o for g in groups for m in g for o, _ in m}, key=lambda o: (sum(x * x for x in o), o))
    pos = {o: i for i, o in enumerate(used)}
    # monomials completed at each neighbour: by group, keyed by the arriving indicator
    due: dict = {}
    for j, g in enumerate(groups):
        for m in g:
            last = max(m, key=lambda f: pos[f[0]])
            rest = tuple(f for f in m if f != last)
            due.setdefault(pos[last[0]], {}).setdefault((j, last[1]), []).append(rest)
    started = [False] * nj
    for i, o in enumerate(used):
        v = _var(o)
        out.append(f"  const uint32_t c_{v} = ld({o[0]}, {o[1]}, {o[2]});")
        out.append(f"  const uint32_t u_{v} = (c_{v} ^ 0x01010101u) & 0x01010101u;")
        out.append(f"  const uint32_t s_{v} = (c_{v} >> 1) & 0x01010101u;")
        masked = set()
        for (j, ind), rests in sorted(due.get(i, {}).items()):
            x = f"{ind}_{v}"
            parts = []
            singles = [r for r in rests if len(r) == 0]
            if singles:
                parts.append(x if len(singles) == 1 else f"{len(singles)}u * {x}")
            others = [_and([f"{ind2}_{_var(o2)}" for o2, ind2 in r]) for r in rests if len(r) > 0]
            if len(others) == 1:
                parts.append(f"({x} & {others[0]})")
            elif others:
                if x not in masked:
                    out.append(f"  const uint32_t m_{x} = {x} * 0xFFu;")
                    masked.add(x)
                parts.append(f"(m_{x} & ({' + '.join(others)}))")
            expr = " + ".join(parts)
            if started[j]:
                out.append(f"  M[{j}] += {expr};")
            else:
                out.append(f"  M[{j}] = {expr};")
                started[j] = True
    assert all(started)
    out.append("}")
    return out


def generate(kind: str) -> tuple[str, dict]:
    bs = O.make_basis_set(kind)
    basis = bs.basis
    offs = bs.neighbour_offsets()
    need_t = basis.name == "chebyshev"
    lines = []
    ns = kind
    lines.append("// Generated by casmcode_monte_gb300/clex/codegen.py -- do not edit.")
    lines.append(f"// Basis set '{kind}': {len(bs.classes)} classes, {bs.n_features} local features,")
    lines.append(f"// {len(offs)} neighbour offsets (FCC 1-4NN pairs, 3 smallest triplets, NN tetrahedron).")
    lines.append("#pragma once")
    lines.append("#include <cstdint>")
    lines.append(f"namespace mg {{ namespace {ns} {{")
    lines.append(f"constexpr int NSPECIES = {basis.n_species};")
    lines.append(f"constexpr int NFUNC = {basis.n_functions};")
    lines.append(f"constexpr int NCLASS = {len(bs.classes)};")
    lines.append(f"constexpr int NFEAT = {bs.n_features};")
    lines.append(f"constexpr int NOFF = {len(offs)};")
    lines.append(f"constexpr int HALO = {max(max(abs(c) for c in o) for o in offs)};")
    # feature -> class, basis index tables
    lines.append("__host__ __device__ constexpr int feat_class(int k) {")
    lines.append("  constexpr int t[NFEAT] = {" + ", ".join(str(f.class_index) for f in bs.features) + "};")
    lines.append("  return t[k];")
    lines.append("}")
    lines.append("__host__ __device__ constexpr int feat_b(int k) {")
    lines.append("  constexpr int t[NFEAT] = {" + ", ".join(str(f.b_site) for f in bs.features) + "};")
    lines.append("  return t[k];")
    lines.append("}")
    # psi tables
    for b in range(basis.n_functions):
        lines.append(f"__host__ __device__ constexpr int psi{b}(int o) {{")
        lines.append("  constexpr int t[NSPECIES] = {" + ", ".join(str(x) for x in basis.psi[b]) + "};")
        lines.append("  return t[o];")
        lines.append("}")
    # psi(b, o) for a runtime occupant index, written arithmetically (no table lookups)
    if basis.name == "occupation":
        lines.append("__host__ __device__ __forceinline__ constexpr int psi(int b, int o) { return o; }")
    else:
        lines.append("__host__ __device__ __forceinline__ constexpr int psi(int b, int o) {")
        lines.append("  return b == 0 ? o - 1 : (o == 1 ? -2 : 1);")
        lines.append("}")
    # stored code from occupant index
    if basis.name == "occupation":
        lines.append("__host__ __device__ constexpr int8_t code_of_occ(int o) { return (int8_t)o; }")
        lines.append("__host__ __device__ constexpr int occ_of_code(int c) { return c; }")
    else:
        lines.append("__host__ __device__ constexpr int8_t code_of_occ(int o) { return (int8_t)(o - 1); }")
        lines.append("__host__ __device__ constexpr int occ_of_code(int c) { return c + 1; }")

    def emit_loads(offsets, indent="  "):
        out = []
        for o in offsets:
            v = _var(o)
            out.append(f"{indent}const int {v} = ld({o[0]}, {o[1]}, {o[2]});")
            if need_t:
                out.append(f"{indent}const int t_{v} = 3 * {v} * {v} - 2;")
        return out

    # features
    lines.append("// F[k] = sum over decorated clusters (class feat_class(k), basis feat_b(k) at the")
    lines.append("// changing site) of the product of the other sites' integer psi values.")
    lines.append("template <class Loader>")
    lines.append("__device__ __forceinline__ void features(const Loader& ld, int (&F)[NFEAT]) {")
    lines += emit_loads(offs)
    for k, f in enumerate(bs.features):
        terms = []
        for t in f.terms:
            if len(t) == 0:
                terms.append("1")
            else:
                terms.append(" * ".join(_psi_expr(basis, b, _var(o)) for o, b in t))
        lines.append(f"  F[{k}] = " + _sum_expr(terms) + ";")
    lines.append("}")

    if basis.name == "occupation":
        lines += _quad_features(bs, offs)
        lines += _quad_pipelines(bs, offs)
    else:
        lines += _ternary_counts(bs, offs)

    # anchored correlations
    anc_offs = sorted({o for cls in bs.anchored for t in cls for o, _ in t})
    lines.append("// C[f] += sum over decorated clusters of class f anchored at this site (its")
    lines.append("// lexicographically smallest member) of the product of integer psi values.")
    lines.append("template <class Loader>")
    lines.append("__device__ __forceinline__ void anchored(const Loader& ld, long long (&C)[NCLASS]) {")
    lines += emit_loads(anc_offs)
    for ci, cls in enumerate(bs.anchored):
        terms = []
        for t in cls:
            if len(t) == 0:
                terms.append("1")
            else:
                terms.append(" * ".join(_psi_expr(basis, b, _var(o)) for o, b in t))
        lines.append(f"  C[{ci}] += (long long)(" + _sum_expr(terms) + ");")
    lines.append("}")
    lines.append("}}  // namespace")
    src = "\n".join(lines) + "\n"

    desc = {
        "name": kind,
        "basis": {"name": basis.name, "n_species": basis.n_species, "psi": basis.psi,
                  "scale": basis.scale},
        "classes": [
            {
                "orbit": c.orbit_index,
                "size": c.size,
                "d2": list(c.d2),
                "multiplicity": c.multiplicity,
                "decoration": list(c.decoration_multiset()),
                "scale": bs.class_scale(i),
            }
            for i, c in enumerate(bs.classes)
        ],
        "features": [
            {"class": f.class_index, "b": f.b_site, "n_terms": len(f.terms),
             "max_abs": bs.max_abs_feature(k)}
            for k, f in enumerate(bs.features)
        ],
        "neighbour_offsets": [list(o) for o in offs],
        "halo": max(max(abs(c) for c in o) for o in offs),
    }
    return src, desc


def class_tables(descs: dict) -> str:
    """Host tables (multiplicity, scale, |F| bounds, neighbour offsets) as C++ source."""
    out = ["// Generated by casmcode_monte_gb300/clex/codegen.py -- do not edit."]
    for kind, cname in (("fcc_binary", "FccBinary"), ("fcc_ternary", "FccTernary")):
        d = descs[kind]
        rows = ", ".join("{%dL, %r}" % (c["multiplicity"], c["scale"]) for c in d["classes"])
        out.append(f"const mg::ClassInfo k{cname}Classes[] = {{{rows}}};")
        fm = ", ".join(str(f["max_abs"]) + "L" for f in d["features"])
        out.append(f"const long k{cname}FeatMax[] = {{{fm}}};")
        offs = ", ".join(f"{o[0]}, {o[1]}, {o[2]}" for o in d["neighbour_offsets"])
        out.append(f"const int k{cname}Offsets[] = {{{offs}}};")
        out.append(f"const int k{cname}NOffsets = {len(d['neighbour_offsets'])};")
    return "\n".join(out) + "\n"


def main():
    os.makedirs(GEN_DIR, exist_ok=True)
    descs = {}
    for kind in ("fcc_binary", "fcc_ternary"):
        src, desc = generate(kind)
        descs[kind] = desc
        with open(os.path.join(GEN_DIR, f"{kind}.cuh"), "w") as f:
            f.write(src)
        with open(os.path.join(GEN_DIR, f"{kind}.json"), "w") as f:
            json.dump(desc, f, indent=1)
        print(kind, len(src), "bytes")
    with open(os.path.join(GEN_DIR, "fcc_class_tables.inc"), "w") as f:
        f.write(class_tables(descs))


if __name__ == "__main__":
    main()
