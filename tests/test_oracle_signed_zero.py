"""Box bounds of exactly +0.0 / -0.0 (tests/golden/signed_zero.npz, made by
the reference's own LBVH::Build): the sign of a zero bound is decided by the
order of the reference's min / max (std::min / std::max keep their first
argument on a tie).

  * Folding the reference's own ordered ids with that rule reproduces every
    reachable node of the reference bit for bit: the rule is pinned.
  * The oracle applies the same rule in its stable (cmpMorton) id order and
    equals that fold bit for bit; the GPU build must equal the oracle bit for
    bit (tests/test_gpu_lbvh.py).
  * Against the reference, the only bit differences are signs of zero bounds
    in leaves whose triangles the reference lists in another order (its
    in-place partition is unstable) and in their ancestors."""
import numpy as np

from bitcmp import assert_nodes_match_reference, fold_boxes, same_bits
from conftest import load_golden


def test_fixture_has_signed_zero_ties():
    g = load_golden("signed_zero")
    b = np.concatenate([g["nodes"]["min"], g["nodes"]["max"]]).ravel()
    z = b[b == 0.0]
    assert (np.signbit(z)).sum() > 100 and (~np.signbit(z)).sum() > 100


def test_reference_boxes_are_the_ordered_fold_of_its_ids():
    g = load_golden("signed_zero")
    mn, mx = fold_boxes(g["tris"], g["ids"], g["node_index"], g["nodes"])
    assert same_bits(mn, g["nodes"]["min"]) and same_bits(mx, g["nodes"]["max"])


def test_oracle_boxes_are_the_ordered_fold_of_its_stable_ids(oracle_mod):
    g = load_golden("signed_zero")
    nodes, ids, _, _ = oracle_mod.lbvh_build(g["tris"], int(g["depth"]))
    idx = g["node_index"]
    mn, mx = fold_boxes(g["tris"], ids, idx, nodes[idx])
    assert same_bits(mn, nodes[idx]["min"]) and same_bits(mx, nodes[idx]["max"])
    assert_nodes_match_reference(nodes, ids, g["nodes"], g["ids"], idx, "oracle")
