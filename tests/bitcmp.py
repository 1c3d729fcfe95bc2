"""Bit-level comparison of test arrays.

Parity in these tests means equal bits: -0.0 and +0.0 differ, and so would
two NaN payloads.  numpy's == (and np.array_equal on float or structured
arrays) compares values, under which -0.0 == +0.0, so every float or
structured comparison goes through same_bits."""
import numpy as np


def raw(a) -> np.ndarray:
    """The bytes of an array (any dtype, structured included) as uint8."""
    a = np.ascontiguousarray(a)
    return a.reshape(-1).view(np.uint8)


def same_bits(a, b) -> bool:
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and a.dtype.itemsize == b.dtype.itemsize and np.array_equal(raw(a), raw(b))


def first_diff(a, b) -> int:
    """Index of the first element whose bytes differ (-1: none)."""
    a = np.ascontiguousarray(a).reshape(len(a), -1)
    b = np.ascontiguousarray(b).reshape(len(b), -1)
    ra = a.view(np.uint8).reshape(len(a), -1)
    rb = b.view(np.uint8).reshape(len(b), -1)
    bad = np.nonzero((ra != rb).any(axis=1))[0]
    return int(bad[0]) if len(bad) else -1


def smin(a, b):
    """std::min as the reference's minBox evaluates it: the first argument on a tie."""
    return b if b < a else a


def smax(a, b):
    """std::max as maxBox evaluates it: the first argument on a tie."""
    return b if a < b else a


def fold_boxes(tris, ids, node_index, nodes):
    """Node boxes by the reference's rule (LBVH.cpp:199-206, 312-313,
    505-509): a triangle's bound is min(V0, min(V1, V2)), a leaf folds its
    triangles' bounds in the order `ids` lists them, an internal node is
    min(left, right) -- every min / max keeping its first argument on a tie,
    which decides the sign of a zero bound.  Returns (min, max), one row per
    entry of node_index."""
    t = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    recs = {}
    for h, nd in zip(node_index.tolist(), nodes):
        if nd["prim_count"] & 4:
            pos, cnt = int(nd["prim_pos"]), int(nd["prim_count"]) >> 3
            mn = mx = None
            for j in range(pos, pos + cnt):
                v = t[ids[j]]
                lo = [smin(v[0][k], smin(v[1][k], v[2][k])) for k in range(3)]
                hi = [smax(v[0][k], smax(v[1][k], v[2][k])) for k in range(3)]
                if mn is None:
                    mn, mx = lo, hi
                else:
                    mn = [smin(mn[k], lo[k]) for k in range(3)]
                    mx = [smax(mx[k], hi[k]) for k in range(3)]
            recs[h] = (mn, mx)
    for h in sorted(node_index.tolist(), reverse=True):
        if h not in recs:
            (lmn, lmx), (rmn, rmx) = recs[2 * h], recs[2 * h + 1]
            recs[h] = ([smin(lmn[k], rmn[k]) for k in range(3)], [smax(lmx[k], rmx[k]) for k in range(3)])
    mn = np.array([recs[h][0] for h in node_index.tolist()], np.float32)
    mx = np.array([recs[h][1] for h in node_index.tolist()], np.float32)
    return mn, mx


def assert_nodes_match_reference(nodes, ids, ref_nodes, ref_ids, node_index, what=""):
    """Reachable nodes against the reference's: count, leaf bit, axis and
    PrimPos equal; boxes equal bit for bit except the sign of a zero bound
    in a leaf whose triangles the reference lists in another order (its
    in-place partition is unstable, LBVH.cpp:238-258, while ids here are in
    stable cmpMorton order) and in that leaf's ancestors."""
    a = nodes[node_index]
    b = ref_nodes
    assert np.array_equal(a["prim_count"], b["prim_count"]), what
    assert np.array_equal(a["prim_pos"], b["prim_pos"]), what
    for f in ("min", "max"):
        assert np.array_equal(a[f], b[f]), f"{what}: {f} values"
    ra = np.ascontiguousarray(a).view(np.uint32).reshape(-1, 8)[:, :6]
    rb = np.ascontiguousarray(b).view(np.uint32).reshape(-1, 8)[:, :6]
    diff = ra != rb
    if not diff.any():
        return
    both = np.concatenate([a["min"], a["max"]], axis=1)
    assert np.all(both[diff] == 0.0), f"{what}: a box bound differs in more than the sign of zero"
    bad = set(np.asarray(node_index)[diff.any(axis=1)].tolist())
    for h in sorted(bad, reverse=True):
        k = int(np.searchsorted(node_index, h))
        nd = b[k]
        if nd["prim_count"] & 4:
            pos, cnt = int(nd["prim_pos"]), int(nd["prim_count"]) >> 3
            assert not np.array_equal(ids[pos:pos + cnt], ref_ids[pos:pos + cnt]), \
                f"{what}: leaf {h} lists its triangles in the reference's order and still differs"
        else:
            assert (2 * h in bad) or (2 * h + 1 in bad), f"{what}: internal node {h} differs, its children do not"
