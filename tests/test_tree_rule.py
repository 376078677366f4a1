"""The construction rule of the GPU build's bottom-up pass, restated in Python
and checked against the oracle's tree (the reference's recursive LBVH_build,
bvh.h:121-221): every gap between sorted codes gets a split level (the
common-prefix length of its two codes; inside a run of equal codes, 32 + the
depth of its node in the run's midpoint subtree), and a finished subtree
covering [lo, hi] hangs below whichever of its outer gaps lo - 1 and hi has the
higher level. The arrivals are simulated in random order inside chunks of
positions (a node finishes on its second arrival), each chunk hands at most one
subtree across its left border, and the hand-offs climb in random order: the
links, parents and root must equal the oracle's whatever the order and chunk
size."""
import numpy as np
import pytest

import gr.scenes as sc

NO = 0xFFFFFFFF


def _levels(code):
    n = len(code)
    lv = np.zeros(max(n - 1, 0), np.int64)
    for g in range(n - 1):
        if code[g] != code[g + 1]:
            lv[g] = 32 - int(code[g] ^ code[g + 1]).bit_length()
            continue
        c, s, e = code[g], g, g + 1
        while s > 0 and code[s - 1] == c:
            s -= 1
        while e + 1 < n and code[e + 1] == c:
            e += 1
        a, b, depth = s, e, 0
        G = a + ((b - a + 1) >> 1) - 1
        while G != g:
            if g < G:
                b = G
            else:
                a = G + 1
            G = a + ((b - a + 1) >> 1) - 1
            depth += 1
        lv[g] = 32 + depth
    return lv


def _build(code, chunk, rng):
    """Links {gap: [left, right]}, parent of every subtree id, and the root."""
    n = len(code)
    lv = _levels(code)
    links, parent, far, count = {}, {}, {}, {}
    root = None

    def slot_of(s):  # s = (id, lo, hi, level before lo, level after hi)
        return 0 if s[4] > s[3] else 1

    def attach(s, G, slot):
        links.setdefault(G, [None, None])[slot] = s[0]
        parent[s[0]] = G
        far[(G, slot)] = (s[1], s[3]) if slot == 0 else (s[2], s[4])
        count[G] = count.get(G, 0) + 1
        return count[G] == 2

    def widen(s, G, slot):
        end, lvl = far[(G, slot ^ 1)]
        return (G, s[1], end, s[3], lvl) if slot == 0 else (G, end, s[2], lvl, s[4])

    left_over = []
    for c in rng.permutation((n + chunk - 1) // chunk):
        base = c * chunk
        for p in rng.permutation(range(base, min(base + chunk, n))):
            s = (~int(p), int(p), int(p), int(lv[p - 1]) if p > 0 else -1, int(lv[p]) if p + 1 < n else -1)
            while True:
                if s[3] < 0 and s[4] < 0:
                    root = s[0]
                    break
                slot = slot_of(s)
                if slot == 1 and s[1] == base:  # parent across the chunk's left border
                    left_over.append(s)
                    break
                G = s[2] if slot == 0 else s[1] - 1
                if not attach(s, G, slot):
                    break
                s = widen(s, G, slot)
    for i in rng.permutation(len(left_over)):
        s = left_over[i]
        while True:
            if s[3] < 0 and s[4] < 0:
                root = s[0]
                break
            slot = slot_of(s)
            G = s[2] if slot == 0 else s[1] - 1
            if not attach(s, G, slot):
                break
            s = widen(s, G, slot)
    return links, parent, root


def _soup(n, kind, seed):
    v = sc.triangle_soup(n, seed_salt=300 + seed)
    if kind == 1:  # a long run of one centroid
        v[n // 4:n // 2] = v[n // 4]
    elif kind == 2:  # many short runs
        v[1::3] = v[0::3][:len(v[1::3])]
    elif kind == 3:  # all at one point
        v[:] = v[0]
    return v


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
@pytest.mark.parametrize("chunk", [1, 7, 32, 256])
def test_bottom_up_rule_gives_the_oracle_tree(oracle, kind, chunk):
    rng = np.random.default_rng(1000 * kind + chunk)
    for trial, n in enumerate((2, 3, 5, 33, 257, 1500)):
        ob = oracle.lbvh(_soup(n, kind, trial))
        code = [int(x) for x in ob["sorted_code"]]
        links, parent, root = _build(code, chunk, rng)
        q3 = ob["nodes"].reshape(-1, 16)[:n - 1, 12:15].view(np.int32)
        assert root == ob["root"], (n, kind, chunk)
        for G in range(n - 1):
            assert links[G] == [int(q3[G, 0]), int(q3[G, 1])], (n, kind, chunk, G)
            want_parent = int(np.uint32(q3[G, 2]))
            assert parent.get(G, NO) == want_parent, (n, kind, chunk, G)
