"""The clustering oracle (oracle/evoc_labels_oracle.cpp) on the CPU.

The assertions are the reference's own unit and integration tests of its
clustering stage, replayed on the restatement:
  src/clustering/mst.rs:169-284, src/clustering/linkage.rs:90-224,
  src/clustering/condensed_tree.rs:473-604, src/clustering/persistence.rs:465-701,
  tests/integration_tests.rs:18-545 (the make_blobs data there comes from
  rand's SmallRng, so blobs of the same shape are drawn here with numpy).
The Boruvka MST is also checked against a brute-force Prim MST over the
same mutual-reachability distances (the sorted MST weights are unique), and
the adjusted Rand index against its definition.
"""
import numpy as np
import pytest

import oracle as O


def make_blobs(n_per_cluster, n_clusters, dim, separation, spread, seed):
    """Blobs laid out like tests/commons/mod.rs:11-40: centre c * separation
    on the first axis, Gaussian spread in every dimension."""
    rng = np.random.default_rng(seed)
    data, labels = [], []
    for c in range(n_clusters):
        p = spread * rng.standard_normal((n_per_cluster, dim))
        p[:, 0] += c * separation
        data.append(p)
        labels += [c] * n_per_cluster
    return np.concatenate(data).astype(np.float32), np.array(labels)


def count_clusters(labels):  # tests/commons/mod.rs:44-51
    pos = labels[labels >= 0]
    return int(pos.max()) + 1 if pos.size else 0


def cluster_accuracy(pred, gt):  # tests/commons/mod.rs:58-86
    correct = 0
    for c in np.unique(pred[pred >= 0]):
        correct += np.bincount(gt[pred == c]).max()
    return correct / len(pred)


# ---------------------------------------------------------------------------
# MST (mst.rs:169-284)
# ---------------------------------------------------------------------------
def test_mst_small_cases():
    assert len(O.build_mst(np.zeros((0, 2), np.float32), 1)[0]) == 0
    assert len(O.build_mst(np.array([[1, 2]], np.float32), 1)[0]) == 0
    u, v, w = O.build_mst(np.array([[0, 0], [3, 4]], np.float32), 1)
    assert len(u) == 1 and abs(w[0] - 5.0) < 1e-6
    u, v, w = O.build_mst(np.array([[0, 0], [1, 0], [0.5, 0.866]], np.float32), 1)
    assert len(u) == 2 and 1.9 < w.sum() < 2.1


def test_mst_two_clusters_one_long_edge():
    d = np.array([[0, 0], [0.1, 0], [0, 0.1], [10, 10], [10.1, 10], [10, 10.1]], np.float32)
    u, v, w = O.build_mst(d, 1)
    assert len(u) == 5 and np.count_nonzero(w > 5.0) == 1


def test_mst_min_samples_inflates():
    d = np.array([[0, 0], [1, 0], [2, 0], [3, 0]], np.float32)
    assert O.build_mst(d, 2)[2].sum() >= O.build_mst(d, 1)[2].sum()
    d = np.array([[0, 0], [0.01, 0], [10, 0]], np.float32)
    w = O.build_mst(d, 2)[2]
    assert len(w) == 2 and (w > 1.0).all()


def test_mst_spans_and_collinear():
    d = np.array([[0], [1], [3], [6], [10]], np.float32)
    u, v, _ = O.build_mst(d, 1)
    assert len(u) == 4 and set(u) | set(v) == set(range(5))
    w = O.build_mst(np.arange(5, dtype=np.float32)[:, None], 1)[2]
    assert abs(w.sum() - 4.0) < 1e-6
    w = O.build_mst(np.array([[0] * 8, [1] * 8, [2] * 8], np.float32), 1)[2]
    assert len(w) == 2 and (w > 0).all() and np.isfinite(w).all()


def test_mst_identical_points():  # integration_tests.rs:534-545
    w = O.build_mst(np.tile(np.array([[1, 2, 3]], np.float32), (10, 1)), 2)[2]
    assert np.isfinite(w).all() and (w >= 0).all()


def _prim_mr(d, min_samples):
    """Brute-force Prim over mutual reachability, the distances summed
    serially over dimensions in f32 like the oracle."""
    n, dim = d.shape
    sq = np.zeros((n, n), np.float32)
    for k in range(dim):
        t = (d[:, None, k] - d[None, :, k]).astype(np.float32)
        sq = sq + t * t
    k = min(min_samples, n - 1)
    core = np.sort(sq + np.diag(np.full(n, np.inf, np.float32)), axis=1)[:, k - 1] if k else \
        np.zeros(n, np.float32)
    mr = np.maximum(np.maximum(sq, core[:, None]), core[None, :])
    in_tree = np.zeros(n, bool)
    best = np.full(n, np.inf, np.float32)
    best[0] = 0
    out = []
    for _ in range(n):
        i = int(np.argmin(np.where(in_tree, np.inf, best)))
        if i != 0 or in_tree.any():
            out.append(best[i])
        in_tree[i] = True
        best = np.where(in_tree, best, np.minimum(best, mr[i]))
    return np.sort(np.sqrt(np.array(out, np.float32)))


@pytest.mark.parametrize("dim,ms,seed", [(2, 1, 0), (4, 5, 1), (8, 5, 2), (3, 10, 3)])
def test_boruvka_equals_prim(dim, ms, seed):
    rng = np.random.default_rng(seed)
    d = np.concatenate([rng.normal(c, 0.4, (150, dim)) for c in (0.0, 3.0, 7.0)]).astype(np.float32)
    w = np.sort(O.build_mst(d, ms)[2])
    ref = _prim_mr(d, ms)
    assert len(w) == len(d) - 1
    assert np.array_equal(w, ref), np.abs(w - ref).max()


# ---------------------------------------------------------------------------
# Linkage (linkage.rs:90-224)
# ---------------------------------------------------------------------------
def test_linkage_basic_and_sizes():
    lr, dist = O.linkage([0, 1], [1, 2], [1.0, 2.0], 3)
    assert list(dist) == [1.0, 2.0] and list(lr[:, 2]) == [2, 3]
    lr, dist = O.linkage([1, 0], [2, 1], [5.0, 1.0], 3)
    assert list(dist) == [1.0, 5.0]
    lr, dist = O.linkage([0, 1, 2], [1, 2, 3], [1.0, 2.0, 3.0], 4)
    assert list(lr[:, 2]) == [2, 3, 4]
    lr, dist = O.linkage([0, 2, 1], [1, 3, 2], [1.0, 1.5, 5.0], 4)  # two simultaneous merges
    assert list(lr[:, 2]) == [2, 2, 4]
    assert lr[0, 0] > lr[0, 1]  # larger label first (linkage.rs:67-69)


def test_linkage_monotonic():  # integration_tests.rs:80-104
    d, _ = make_blobs(20, 3, 4, 30.0, 0.5, 7)
    u, v, w = O.build_mst(d, 5)
    _, dist = O.linkage(u, v, w, len(d))
    assert (np.diff(dist) >= 0).all()


# ---------------------------------------------------------------------------
# Condensed tree and labels (condensed_tree.rs:473-604)
# ---------------------------------------------------------------------------
TWO = np.array([[0, 0], [0.1, 0], [0, 0.1], [10, 10], [10.1, 10], [10, 10.1]], np.float32)


def test_condensed_two_clusters():
    lab, st, k = O.leaf_labels(TWO, 1, 2)
    assert k == 2
    assert lab[0] == lab[1] == lab[2] and lab[3] == lab[4] == lab[5] and lab[0] != lab[3]
    assert (lab >= 0).all()
    assert ((st >= 0) & (st <= 1)).all()
    assert O.leaf_labels(TWO, 1, len(TWO))[2] <= 1


def test_labels_with_noise():
    d = np.array([[0, 0], [0.05, 0], [5, 5], [10, 0], [0, 10]], np.float32)
    lab, _, _ = O.leaf_labels(d, 1, 2)
    if lab[0] >= 0 and lab[1] >= 0:
        assert lab[0] == lab[1]


def test_labels_match_ground_truth():  # integration_tests.rs:142-166
    d, gt = make_blobs(40, 2, 4, 100.0, 0.3, 42)
    lab, st, _ = O.leaf_labels(d, 5, 5)
    assert np.count_nonzero(lab < 0) <= 2
    assert cluster_accuracy(lab, gt) > 0.95
    assert ((st[lab >= 0] >= 0) & (st[lab >= 0] <= 1)).all()


# ---------------------------------------------------------------------------
# Persistence layers (persistence.rs:465-701)
# ---------------------------------------------------------------------------
def test_find_peaks():
    assert list(O.find_peaks([0.0, 1.0, 0.0, 2.0, 0.0])) == [1, 3]
    p = O.find_peaks([0.0, 1.0, 1.0, 0.0])
    assert len(p) == 1 and p[0] in (1, 2)
    assert len(O.find_peaks([1.0, 2.0, 3.0, 4.0, 5.0])) == 0
    assert len(O.find_peaks([])) == 0 and len(O.find_peaks([1.0, 2.0])) == 0


TWO10 = np.array([[0, 0], [0.1, 0], [0, 0.1], [0.1, 0.1], [0.05, 0.05],
                  [10, 10], [10.1, 10], [10, 10.1], [10.1, 10.1], [10.05, 10.05]], np.float32)
THREE15 = np.concatenate([TWO10, np.array([[20, 0], [20.1, 0], [20, 0.1], [20.1, 0.1],
                                           [20.05, 0.05]], np.float32)])


def test_barcodes_and_persistence():
    bc, sizes, pers = O.barcodes(TWO10, 1, 2)
    assert len(bc) > 0 and int(bc[0, 1]) == len(TWO10)  # root dies at n
    assert len(sizes) == len(pers) > 0 and (pers >= 0).all()


def test_cluster_layers_two_and_three():
    labels, strengths, pers = O.build_cluster_layers(TWO10, 1, 2, 0.2, 10)
    assert len(labels) == len(strengths) == len(pers) >= 1
    b = labels[0]
    assert count_clusters(b) >= 2
    assert b[0] == b[1] == b[4] and b[5] == b[6] == b[9] and b[0] != b[5]
    for lab, st in zip(labels, strengths):
        assert ((st[lab >= 0] >= 0) & (st[lab >= 0] <= 1)).all()
    labels, _, _ = O.build_cluster_layers(THREE15, 1, 2, 0.2, 10)
    assert count_clusters(labels[0]) >= 3
    counts = [count_clusters(l) for l in labels]
    assert counts == sorted(counts, reverse=True)
    assert len(O.build_cluster_layers(THREE15, 1, 2, 0.2, 2)[0]) <= 2
    assert O.build_cluster_layers(np.zeros((0, 2), np.float32), 1, 2, 0.2, 10) == ([], [], [])


def test_cluster_layers_blobs():  # integration_tests.rs:192-251, 505-517
    d, gt = make_blobs(50, 2, 4, 50.0, 0.5, 42)
    labels, _, _ = O.build_cluster_layers(d, 5, 5, 0.2, 10)
    assert count_clusters(labels[0]) >= 2 and cluster_accuracy(labels[0], gt) > 0.9
    d, gt = make_blobs(50, 3, 4, 50.0, 0.5, 42)
    labels, _, _ = O.build_cluster_layers(d, 5, 5, 0.2, 10)
    assert count_clusters(labels[0]) >= 3 and cluster_accuracy(labels[0], gt) > 0.9
    d, _ = make_blobs(30, 1, 4, 0.0, 0.5, 42)
    assert count_clusters(O.build_cluster_layers(d, 5, 5, 0.2, 10)[0][0]) <= 1


def test_search_for_n_clusters():  # integration_tests.rs:253-335
    d, gt = make_blobs(30, 2, 4, 50.0, 0.5, 42)
    lab, _, k = O.search_for_n_clusters(d, 3, 2)
    assert count_clusters(lab) == 2 and cluster_accuracy(lab, gt) > 0.95
    d, _ = make_blobs(25, 5, 4, 50.0, 0.5, 42)
    lab, _, _ = O.search_for_n_clusters(d, 3, 5)
    assert 3 <= count_clusters(lab) <= 7


# ---------------------------------------------------------------------------
# Adjusted Rand index
# ---------------------------------------------------------------------------
def _ari_pairs(a, b):
    """Pair-counting definition, O(n^2): for small checks."""
    n = len(a)
    same_a = a[:, None] == a[None, :]
    same_b = b[:, None] == b[None, :]
    iu = np.triu_indices(n, 1)
    sa, sb = same_a[iu], same_b[iu]
    n11 = np.count_nonzero(sa & sb)
    pa, pb, tot = np.count_nonzero(sa), np.count_nonzero(sb), len(sa)
    exp = pa * pb / tot
    mx = (pa + pb) / 2
    return 1.0 if mx == exp else (n11 - exp) / (mx - exp)


def test_adjusted_rand_index():
    rng = np.random.default_rng(3)
    a = rng.integers(-1, 5, 300)
    assert O.adjusted_rand_index(a, a) == 1.0
    perm = np.array([3, 0, 4, 2, 1, 5])
    assert O.adjusted_rand_index(a, perm[a + 1]) == pytest.approx(1.0)
    b = rng.integers(-1, 5, 300)
    assert O.adjusted_rand_index(a, b) == pytest.approx(_ari_pairs(a, b), abs=1e-12)
    c = a.copy()
    c[:30] = rng.integers(0, 5, 30)
    assert O.adjusted_rand_index(a, c) == pytest.approx(_ari_pairs(a, c), abs=1e-12)
    skl = pytest.importorskip("sklearn.metrics")
    assert O.adjusted_rand_index(a, c) == pytest.approx(skl.adjusted_rand_score(a, c), abs=1e-12)


# ---------------------------------------------------------------------------
# The tie rules of the oracle's Boruvka MST, against an independent
# restatement with brute-force queries: a query takes the smallest point
# index among equal mutual-reachability values, a component's pick is its
# (value, point index) minimum, and each round adds the picks in ascending
# order of the component's smallest point index through a disjoint set.
# ---------------------------------------------------------------------------
def _sqd(a, b):
    s = np.float32(0.0)
    for t in (a - b).astype(np.float32):
        s = np.float32(s + np.float32(t * t))
    return s


def _mst_by_rules(x, min_samples):
    n = len(x)
    D = np.array([[_sqd(x[i], x[j]) for j in range(n)] for i in range(n)], np.float32)
    k = min(min_samples, n - 1)
    core = np.zeros(n, np.float32)
    if k > 0:
        for i in range(n):
            core[i] = np.sort(np.delete(D[i], i))[k - 1]
    parent = list(range(n))

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a
    out = []
    while len(out) < n - 1:
        comp = [min(j for j in range(n) if find(j) == find(i)) for i in range(n)]
        picks = {}
        for i in range(n):
            best = None
            for j in range(n):
                if comp[j] == comp[i]:
                    continue
                mr = max(D[i, j], core[i], core[j])
                if best is None or (mr, j) < best:
                    best = (mr, j)
            if best is not None and (comp[i] not in picks or (best[0], i) < picks[comp[i]][:2]):
                picks[comp[i]] = (best[0], i, best[1])
        if not picks:
            break
        merged = False
        for c in sorted(picks):
            w, i, j = picks[c]
            ri, rj = find(i), find(j)
            if ri != rj:
                parent[ri] = rj
                out.append((i, j, np.sqrt(np.float32(w))))
                merged = True
        if not merged:
            break
    return (np.array([e[0] for e in out], np.int64), np.array([e[1] for e in out], np.int64),
            np.array([e[2] for e in out], np.float32))


@pytest.mark.parametrize("min_samples", [0, 1, 3, 5])
def test_mst_tie_rules_match_restatement(min_samples):
    """Integer grid points with duplicates (many equal values) and a small
    blob set: the oracle's edge list equals the rule-by-rule restatement."""
    rng = np.random.default_rng(1)
    g = np.stack(np.meshgrid(np.arange(8), np.arange(6)), -1).reshape(-1, 2)
    grid = np.concatenate([g, g[::5]]).astype(np.float32)
    grid = grid[rng.permutation(len(grid))]
    blobs = (rng.normal(size=(60, 3)) + 3 * rng.integers(0, 3, (60, 1))).astype(np.float32)
    for x in (grid, blobs, np.ones((12, 2), np.float32)):
        u, v, w = O.build_mst(x, min_samples)
        ru, rv, rw = _mst_by_rules(x, min_samples)
        assert np.array_equal(u, ru) and np.array_equal(v, rv)
        assert np.array_equal(w.view(np.uint32), rw.view(np.uint32))
