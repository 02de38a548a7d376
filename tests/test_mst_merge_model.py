"""The round logic of the GPU MST (evoc-rs_gb300/csrc/mst.cu), restated in
numpy with brute-force queries, against the oracle's Boruvka MST
(oracle/evoc_labels_oracle.cpp, src/clustering/mst.rs:82-166).

The GPU does not add a round's picks one by one through a disjoint set as
the reference does. It computes the same result in parallel:
  * the picks form a functional graph on components (component -> component
    of its pick's other end); taken in ascending component id, the picks a
    disjoint set would skip are exactly the pick of each cycle's largest
    component, found by pointer doubling (2^K >= m steps lands every
    component on its cycle and gathers the cycle's maximum);
  * the merged components follow by pointer jumping to that component, and
    each takes its smallest point index as its id;
  * kept picks are appended in ascending component id.
This test checks that argument on the CPU, before any kernel: the model's
edge lists equal the oracle's on inputs with many equal values."""
import numpy as np
import pytest

import oracle as O


def _sqd(a, b):
    s = np.float32(0.0)
    for t in (a - b).astype(np.float32):
        s = np.float32(s + np.float32(t * t))
    return s


def gpu_round_model(x, min_samples):
    n = len(x)
    D = np.array([[_sqd(x[i], x[j]) for j in range(n)] for i in range(n)], np.float32)
    k = min(min_samples, n - 1)
    core = np.zeros(n, np.float32)
    if k > 0:
        for i in range(n):
            core[i] = np.sort(np.delete(D[i], i))[k - 1]
    comp = np.arange(n)
    A = list(range(n))
    out = []
    while len(A) > 1 and len(out) < n - 1:
        # queries: (value, other point) minimum per point; picks per component
        ckey, bj = {}, {}
        for i in range(n):
            best = None
            for j in range(n):
                if comp[j] == comp[i]:
                    continue
                mr = max(D[i, j], core[i], core[j])
                if best is None or (mr, j) < best:
                    best = (mr, j)
            if best is not None:
                bj[i] = best[1]
                key = (best[0], i)
                if comp[i] not in ckey or key < ckey[comp[i]]:
                    ckey[comp[i]] = key
        m = len(A)
        K = max(1, int(np.ceil(np.log2(m))))
        succ, has, picks = {}, {}, {}
        for c in A:
            if c not in ckey:
                succ[c], has[c] = c, False
                continue
            w, i = ckey[c]
            j = bj[i]
            succ[c], has[c], picks[c] = comp[j], True, (i, j, w)
        # pointer doubling: land on the cycle, gather its maximum
        jmp = dict(succ)
        mx = {c: max(c, succ[c]) for c in A}
        for _ in range(K):
            jmp, mx = {c: jmp[jmp[c]] for c in A}, {c: max(mx[c], mx[jmp[c]]) for c in A}
        on_cycle = {jmp[c] for c in A}
        root = {c: c in on_cycle and mx[c] == c for c in A}
        # pointer jumping to the skipped component; ids are smallest members
        par = {c: c if root[c] else succ[c] for c in A}
        for _ in range(K + 1):
            par = {c: par[par[c]] for c in A}
        nid = {}
        for c in A:
            nid[par[c]] = min(nid.get(par[c], n), c)
        lab = {c: nid[par[c]] for c in A}
        kept = [picks[c] for c in A if has[c] and not root[c]]
        out += kept
        comp = np.array([lab[c] for c in comp])
        A = [c for c in A if lab[c] == c]
        if not kept:
            break
    return (np.array([e[0] for e in out], np.int64), np.array([e[1] for e in out], np.int64),
            np.array([np.sqrt(np.float32(e[2])) for e in out], np.float32))


def _cases():
    rng = np.random.default_rng(1)
    g = np.stack(np.meshgrid(np.arange(9), np.arange(7)), -1).reshape(-1, 2)
    grid = np.concatenate([g, g[::5]]).astype(np.float32)
    yield "grid", grid[rng.permutation(len(grid))]
    yield "blobs", (rng.normal(size=(120, 3)) + 3 * rng.integers(0, 4, (120, 1))).astype(np.float32)
    yield "equal", np.ones((20, 2), np.float32)
    line = np.zeros((40, 2), np.float32)
    line[:, 0] = np.arange(40) % 10  # repeated positions on a line
    yield "line", line


@pytest.mark.parametrize("min_samples", [0, 1, 3, 5])
def test_gpu_round_logic_matches_oracle(min_samples):
    for name, x in _cases():
        u, v, w = O.build_mst(x, min_samples)
        mu, mv, mw = gpu_round_model(x, min_samples)
        assert np.array_equal(u, mu) and np.array_equal(v, mv), name
        assert np.array_equal(w.view(np.uint32), mw.view(np.uint32)), name
