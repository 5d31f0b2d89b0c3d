"""The committed generated sources equal a fresh generation from the cluster enumeration."""
import json
import os

from casmcode_monte_gb300.clex import codegen

GEN = codegen.GEN_DIR


def test_generated_sources_up_to_date():
    descs = {}
    for kind in ("fcc_binary", "fcc_ternary"):
        src, desc = codegen.generate(kind)
        descs[kind] = desc
        with open(os.path.join(GEN, f"{kind}.cuh")) as f:
            assert f.read() == src, f"{kind}.cuh is stale: run python -m casmcode_monte_gb300.clex.codegen"
        with open(os.path.join(GEN, f"{kind}.json")) as f:
            assert json.load(f) == json.loads(json.dumps(desc))
    with open(os.path.join(GEN, "fcc_class_tables.inc")) as f:
        assert f.read() == codegen.class_tables(descs)


def test_binary_cluster_counts():
    with open(os.path.join(GEN, "fcc_binary.json")) as f:
        d = json.load(f)
    # empty, point, 4 pairs, 3 triplets, 1 quadruplet
    assert [c["size"] for c in d["classes"]] == [0, 1, 2, 2, 2, 2, 3, 3, 3, 4]
    assert [c["multiplicity"] for c in d["classes"]] == [1, 1, 6, 3, 12, 6, 8, 12, 24, 2]
    assert [c["d2"] for c in d["classes"][2:6]] == [[8], [16], [24], [32]]
    assert [c["d2"] for c in d["classes"][6:9]] == [[8, 8, 8], [8, 8, 16], [8, 8, 24]]
    assert [f["n_terms"] for f in d["features"]] == [1, 12, 6, 24, 12, 24, 36, 72, 8]
