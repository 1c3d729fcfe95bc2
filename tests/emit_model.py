"""Host model of the GPU node emission (k_emit_tiles / k_emit_prefix /
k_emit_leaves / k_emit_refit in csrc/rt_build.cu), written with the same
record-mask scans so the algorithm can be checked on the CPU against the
oracle's restatement of LBVH::build_recursive (LBVH.cpp:190-314)."""
import numpy as np


def hb(x: int) -> int:
    return x.bit_length() - 1


def keep_above(m: int, b: int) -> int:
    return m if b < 0 else m & ~((2 << b) - 1)


def rec_fwd(a: int, b: int) -> int:
    return (b | keep_above(a, hb(b))) if b else a


def rec_bwd(a: int, b: int) -> int:
    return (a | keep_above(b, hb(a))) if a else b


def emit(keys: np.ndarray, depth: int, tile: int = 7):
    """Returns {heap index: (prim_count field, prim_pos)} for every node the
    GPU writes, using tiles of `tile` boundaries to exercise the tile prefix."""
    keys = [int(k) for k in keys]
    n = len(keys)
    delta = [(-1 if keys[i] == keys[i + 1] else hb(keys[i] ^ keys[i + 1])) for i in range(n - 1)]
    r = [(1 << d) if d >= 0 else 0 for d in delta] + [0]  # boundary n-1 does not exist
    # tile aggregates, then tile-exclusive prefix / suffix, then in-tile scans
    T = (n + tile - 1) // tile
    aggf, aggb = [0] * T, [0] * T
    for t in range(T):
        for i in range(t * tile, min(n, (t + 1) * tile)):
            aggf[t] = rec_fwd(aggf[t], r[i])
        for i in reversed(range(t * tile, min(n, (t + 1) * tile))):
            aggb[t] = rec_bwd(r[i], aggb[t])
    pre, suf = [0] * T, [0] * T
    run = 0
    for t in range(T):
        pre[t] = run
        run = rec_fwd(run, aggf[t])
    run = 0
    for t in reversed(range(T)):
        suf[t] = run
        run = rec_bwd(aggb[t], run)
    L, R = [0] * (n + 1), [0] * (n + 1)
    for t in range(T):
        lo, hi = t * tile, min(n, (t + 1) * tile)
        run = pre[t]
        for k in range(lo, hi):
            L[k] = run
            run = rec_fwd(run, r[k])
        run = suf[t]
        for k in reversed(range(lo, hi)):
            run = rec_bwd(r[k], run)
            R[k] = run
    leaf_depth = depth - 1
    heads, tails = {}, {}
    for k in range(n):
        anc = L[k] | R[k]
        m, dep = anc, bin(anc).count("1")
        while dep > leaf_depth:
            m &= m - 1
            dep -= 1
        h = 1
        while m:
            b = hb(m)
            h = (h << 1) | ((keys[k] >> b) & 1)
            m ^= 1 << b
        dprev = delta[k - 1] if k >= 1 else -1
        dcur = delta[k] if k < n - 1 else -1
        head = k == 0 or (dprev >= 0 and bin(keep_above(anc, dprev)).count("1") < leaf_depth)
        tail = k == n - 1 or (dcur >= 0 and bin(keep_above(anc, dcur)).count("1") < leaf_depth)
        if head:
            heads[h] = k
        if tail:
            tails[h] = k
    assert heads.keys() == tails.keys()
    out = {}
    arrived = {}
    for h in heads:
        pos, end = heads[h], tails[h]
        count = end - pos + 1
        dh = hb(h)
        if dh == 0:
            axis = 0 if (count <= 1 or depth <= 1) else 1
        elif count == 1 or dh == depth - 1:
            a, b = (keys[pos - 1], keys[pos]) if (h & 1) else (keys[end], keys[end + 1])
            axis = (31 - hb(a ^ b)) % 3
        else:
            axis = 1
        out[h] = ((count << 3) | 4 | axis, pos)
        cur = h
        while cur > 1:
            p = cur >> 1
            if p not in arrived:
                arrived[p] = True
                break
            sib = cur ^ 1
            lpos = out[sib][1] if (cur & 1) else out[cur][1]
            rpos = out[cur][1] if (cur & 1) else out[sib][1]
            cnt = (out[cur][0] >> 3) + (out[sib][0] >> 3)
            d = hb(keys[rpos - 1] ^ keys[rpos])
            out[p] = ((cnt << 3) | ((30 - d) % 3), lpos)
            cur = p
    return out


SEP_BIT = 31


def emit_batch(keys: np.ndarray, offsets, depth: int, tile: int = 7):
    """Host model of the batched emission (kb_emit_tiles / kb_emit_leaves /
    kb_emit_refit): the scenes' sorted codes are concatenated, the boundary
    between two scenes carries a separator record (bit 31, above every code
    bit) so that no scan crosses it, and each scene's nodes and positions are
    local to it.  Returns one {heap index: (prim_count field, prim_pos)} per
    scene."""
    keys = [int(k) for k in keys]
    offsets = [int(o) for o in offsets]
    n = len(keys)
    starts = set(offsets[:-1])
    delta = []
    for i in range(n - 1):
        if i + 1 in starts:
            delta.append(SEP_BIT)
        else:
            delta.append(-1 if keys[i] == keys[i + 1] else hb(keys[i] ^ keys[i + 1]))
    r = [(1 << d) if d >= 0 else 0 for d in delta] + [0]
    T = (n + tile - 1) // tile
    aggf, aggb = [0] * T, [0] * T
    for t in range(T):
        for i in range(t * tile, min(n, (t + 1) * tile)):
            aggf[t] = rec_fwd(aggf[t], r[i])
        for i in reversed(range(t * tile, min(n, (t + 1) * tile))):
            aggb[t] = rec_bwd(r[i], aggb[t])
    pre, suf = [0] * T, [0] * T
    run = 0
    for t in range(T):
        pre[t] = run
        run = rec_fwd(run, aggf[t])
    run = 0
    for t in reversed(range(T)):
        suf[t] = run
        run = rec_bwd(aggb[t], run)
    L, R = [0] * (n + 1), [0] * (n + 1)
    for t in range(T):
        lo, hi = t * tile, min(n, (t + 1) * tile)
        run = pre[t]
        for k in range(lo, hi):
            L[k] = run
            run = rec_fwd(run, r[k])
        run = suf[t]
        for k in reversed(range(lo, hi)):
            run = rec_bwd(r[k], run)
            R[k] = run
    leaf_depth = depth - 1
    S = len(offsets) - 1
    heads = [dict() for _ in range(S)]
    tails = [dict() for _ in range(S)]
    sc = 0
    for k in range(n):
        while k >= offsets[sc + 1]:
            sc += 1
        first, last = offsets[sc], offsets[sc + 1] - 1
        anc = (L[k] | R[k]) & 0x3FFFFFFF
        m, dep = anc, bin(anc).count("1")
        while dep > leaf_depth:
            m &= m - 1
            dep -= 1
        h = 1
        while m:
            b = hb(m)
            h = (h << 1) | ((keys[k] >> b) & 1)
            m ^= 1 << b
        dprev = delta[k - 1] if k >= 1 else -1
        dcur = delta[k] if k < n - 1 else -1
        head = k == first or (dprev >= 0 and bin(keep_above(anc, dprev)).count("1") < leaf_depth)
        tail = k == last or (dcur >= 0 and bin(keep_above(anc, dcur)).count("1") < leaf_depth)
        if head:
            heads[sc][h] = k - first
        if tail:
            tails[sc][h] = k - first
    outs = []
    for s in range(S):
        assert heads[s].keys() == tails[s].keys()
        ks = keys[offsets[s]:offsets[s + 1]]
        out, arrived = {}, {}
        for h in heads[s]:
            pos, end = heads[s][h], tails[s][h]
            count = end - pos + 1
            dh = hb(h)
            if dh == 0:
                axis = 0 if (count <= 1 or depth <= 1) else 1
            elif count == 1 or dh == depth - 1:
                a, b = (ks[pos - 1], ks[pos]) if (h & 1) else (ks[end], ks[end + 1])
                axis = (31 - hb(a ^ b)) % 3
            else:
                axis = 1
            out[h] = ((count << 3) | 4 | axis, pos)
            cur = h
            while cur > 1:
                p = cur >> 1
                if p not in arrived:
                    arrived[p] = True
                    break
                sib = cur ^ 1
                lpos = out[sib][1] if (cur & 1) else out[cur][1]
                rpos = out[cur][1] if (cur & 1) else out[sib][1]
                cnt = (out[cur][0] >> 3) + (out[sib][0] >> 3)
                d = hb(ks[rpos - 1] ^ ks[rpos])
                out[p] = ((cnt << 3) | ((30 - d) % 3), lpos)
                cur = p
        outs.append(out)
    return outs
