"""The per-matrix plan's item list, built on the host (spmm_bcsr_plan_items,
the same routine spmm_bcsr_plan_create runs): checked against a Python
restatement of its rules, and for the properties the kernel relies on. Each
(row, tile) block range is covered exactly once by its parts; items come
heaviest first; the parts of a split row sit together, part 0 first, so every
wait for a part 0 points to an earlier item. No GPU needed."""
import math

import numpy as np
import pytest

import matrixmultiplicationcuda_gb300 as m

MIN_PART, FACTOR, MAX_PARTS = 8, 3, 64


def restated(rp, ntiles, slots):
    """The plan's rules in plain Python: average load per slot (at least 8
    blocks); rows longer than 3x it cut into min(64, ceil(len / avg)) parts at
    len * q / k; every item keyed by its blocks (a part: its row's longest
    part); a stable sort, heaviest first."""
    MB = len(rp) - 1
    total = sum(int(rp[r + 1] - rp[r]) * ntiles for r in range(MB))
    avg = max(MIN_PART, -(-total // slots))
    items, groups = [], []
    for r in range(MB):
        a, ln = int(rp[r]), int(rp[r + 1] - rp[r])
        k = min(MAX_PARTS, -(-ln // avg)) if ln > FACTOR * avg else 1
        for t in range(ntiles):
            if k == 1:
                items.append(((r, t, a, a + ln), -1, ln))
                continue
            g = len(groups)
            groups.append(k)
            for q in range(k):
                items.append(((r, t, a + ln * q // k, a + ln * (q + 1) // k), 128 * g + q, -(-ln // k)))
    items.sort(key=lambda x: -x[2])   # stable
    return (np.array([i[0] for i in items], np.int32).reshape(-1, 4), np.array([i[1] for i in items], np.int32),
            np.array(groups, np.int32))


def lognormal_rows(MB, mean, cv, seed):
    rng = np.random.default_rng(seed)
    s2 = math.log(1 + cv * cv)
    lens = np.floor(rng.lognormal(math.log(mean) - s2 / 2, math.sqrt(s2), MB)).astype(np.int64)
    return np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)


CASES = [
    ("uniform rows", np.arange(0, 257 * 20, 20, dtype=np.int32), 2, 304),
    ("random 2 %", m.gen_structure(16384, 16384, 64, m.PATTERN_RANDOM, 0.02, 0, seed=20240)[0], 2, 304),
    ("log-normal", m.gen_structure(8192, 8192, 64, m.PATTERN_LOGNORMAL, 0.05, 1.5, seed=77)[0], 2, 304),
    ("log-normal, one tile", lognormal_rows(1000, 30, 2.0, 5), 1, 152),
    ("one huge row (parts capped at 64)", np.array([0, 5, 5000, 5003, 5010], np.int32), 1, 304),
    ("empty rows", np.array([0, 0, 0, 40, 40, 41], np.int32), 3, 16),
    ("no blocks at all", np.zeros(9, np.int32), 2, 304),
    ("one slot", np.array([0, 10, 30, 31], np.int32), 4, 1),
]


@pytest.mark.parametrize("name,rp,ntiles,slots", CASES, ids=[c[0] for c in CASES])
def test_plan_items_match_restatement(name, rp, ntiles, slots):
    items, pair, parts = m.plan_items(rp, ntiles, slots)
    ri, rpair, rparts = restated(rp, ntiles, slots)
    assert np.array_equal(items, ri)
    assert np.array_equal(pair, rpair)
    assert np.array_equal(parts, rparts)


@pytest.mark.parametrize("name,rp,ntiles,slots", CASES, ids=[c[0] for c in CASES])
def test_plan_items_properties(name, rp, ntiles, slots):
    items, pair, parts = m.plan_items(rp, ntiles, slots)
    MB = len(rp) - 1
    # every (row, tile) covered by contiguous, non-overlapping parts
    cover = {}
    for (r, t, a, b), code in zip(items, pair):
        assert 0 <= r < MB and 0 <= t < ntiles and rp[r] <= a <= b <= rp[r + 1]
        cover.setdefault((r, t), []).append((a, b))
    assert set(cover) == {(r, t) for r in range(MB) for t in range(ntiles)}
    for (r, t), spans in cover.items():
        spans.sort()
        assert spans[0][0] == rp[r] and spans[-1][1] == rp[r + 1]
        assert all(spans[i][1] == spans[i + 1][0] for i in range(len(spans) - 1))
    # heaviest first
    keys = []
    for i, ((r, t, a, b), code) in enumerate(zip(items, pair)):
        if code < 0:
            keys.append(b - a)
        else:
            g = code >> 7
            keys.append(-(-(int(rp[r + 1] - rp[r])) // int(parts[g])))
    assert all(keys[i] >= keys[i + 1] for i in range(len(keys) - 1))
    # split rows: parts 0..k-1 of a group, together and in order, so each
    # part's part 0 comes earlier in the list
    where = {}
    for i, code in enumerate(pair):
        if code >= 0:
            where.setdefault(code >> 7, []).append((i, code & 127))
    assert sorted(where) == list(range(len(parts)))
    for g, lst in where.items():
        idx = [i for i, _ in lst]
        assert [q for _, q in lst] == list(range(parts[g]))
        assert idx == list(range(idx[0], idx[0] + parts[g]))
        assert 2 <= parts[g] <= MAX_PARTS


def test_plan_items_rejects():
    with pytest.raises(m.SpmmError) as e:
        m.plan_items(np.array([0, 5, 3], np.int32), 1, 304)
    assert e.value.status == m.Status.INVALID_ARG
    with pytest.raises(m.SpmmError):
        m.plan_items(np.array([0, 5], np.int32), 0, 304)


def restated_stack(rp, ci, st):
    """Stacking in plain Python: per group of `st` block rows, the sorted union
    of their columns, and per union column the member rows' block indices."""
    srp, sci, smap = [0], [], []
    for g in range((len(rp) - 1) // st):
        cols = {}
        for t in range(st):
            r = g * st + t
            for b in range(rp[r], rp[r + 1]):
                cols.setdefault(int(ci[b]), [-1] * st)[t] = b
        for c in sorted(cols):
            sci.append(c)
            smap.append(cols[c])
        srp.append(len(sci))
    return np.array(srp, np.int32), np.array(sci, np.int32), np.array(smap, np.int32).reshape(-1, st)


STACK_CASES = [
    ("band 16", 4096, 16, m.PATTERN_BAND, 0.2, 8),
    ("band 32", 4096, 32, m.PATTERN_BAND, 0.2, 8),
    ("blockdiag 16", 4096, 16, m.PATTERN_BLOCKDIAG, 0.2, 256),
    ("random 16", 4096, 16, m.PATTERN_RANDOM, 0.05, 0),
    ("log-normal 32", 4096, 32, m.PATTERN_LOGNORMAL, 0.05, 1.5),
]


@pytest.mark.parametrize("name,M,bR,pattern,density,param", STACK_CASES, ids=[c[0] for c in STACK_CASES])
def test_stack_structure(name, M, bR, pattern, density, param):
    rp, ci = m.gen_structure(M, M, bR, pattern, density, param, seed=21)
    st = 64 // bR
    srp, sci, smap = m.stack_structure(rp, ci, st)
    rrp, rci, rmap = restated_stack(rp, ci, st)
    assert np.array_equal(srp, rrp) and np.array_equal(sci, rci) and np.array_equal(smap, rmap)
    # every block lands once, in its member row's slot of its own column
    seen = np.zeros(len(ci), np.int64)
    for g in range(len(srp) - 1):
        cols = sci[srp[g]:srp[g + 1]]
        assert np.all(np.diff(cols) > 0)
        for j in range(srp[g], srp[g + 1]):
            for t, b in enumerate(smap[j]):
                if b >= 0:
                    seen[b] += 1
                    assert rp[g * st + t] <= b < rp[g * st + t + 1] and ci[b] == sci[j]
    assert np.all(seen == 1)
    if pattern in (m.PATTERN_BAND, m.PATTERN_BLOCKDIAG):
        assert len(sci) * 100 <= len(ci) * 60      # the plan would stack these
    if pattern == m.PATTERN_RANDOM:
        assert len(sci) * 100 > len(ci) * 60       # and not this one


def test_stack_structure_rejects():
    with pytest.raises(m.SpmmError):
        m.stack_structure(np.array([0, 2, 2, 2, 2], np.int32), np.array([3, 3], np.int32), 4)   # repeated column
    with pytest.raises(m.SpmmError):
        m.stack_structure(np.array([0, 1, 2, 3], np.int32), np.array([0, 1, 2], np.int32), 2)   # 3 rows, stacks of 2


@pytest.mark.parametrize("bR", [16, 32])
def test_stacked_blocks_give_the_same_product(bR):
    """The 64-row blocks a stacked run multiplies: stacked block j holds member
    t's bR rows at rows t * bR .. (t + 1) * bR - 1 (source block map[j, t], or
    zeros for -1), the layout the pipeline assembles in its stage. Their 64-row
    product is the original one (FP64 oracle; zero blocks add exact zeros and
    each row keeps its column order)."""
    from oracle import oracle
    M = K = 1024
    rp, ci = m.gen_structure(M, K, bR, m.PATTERN_BAND, 0.2, 4, seed=31)
    st = 64 // bR
    srp, sci, smap = m.stack_structure(rp, ci, st)
    rng = np.random.default_rng(32)
    vals = rng.standard_normal(len(ci) * bR * 16)
    blocks = vals.reshape(-1, bR, 16)
    stacked = np.zeros((len(sci), 64, 16))
    for j in range(len(sci)):
        for t in range(st):
            if smap[j, t] >= 0:
                stacked[j, t * bR:(t + 1) * bR] = blocks[smap[j, t]]
    B = rng.standard_normal((K, 48))
    ref = oracle.bcsr_matmul_f64(rp, ci, vals, bR, 16, B)
    got = oracle.bcsr_matmul_f64(srp, sci, stacked.reshape(-1), 64, 16, B)
    assert np.array_equal(got, ref)
