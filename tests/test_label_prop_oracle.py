"""CPU pins of the label-propagation partition oracle, restated from the
reference's own unit tests (src/graph/label_prop.rs:571-739)."""
import numpy as np

import oracle as O


def test_iteration_skips_labelled_nodes():  # label_prop.rs:575-582
    assert list(O.lp_iteration([0, 1, 2, 3], [1, 0, 1], [1, 1, 1], [0, 1, 2])) == [0, 1, 2]


def test_iteration_propagates_strong_label():  # :584-592
    assert O.lp_iteration([0, 2, 2, 2], [1, 2], [2.0, 0.3], [-1, 5, 7])[0] == 5


def test_iteration_stays_unlabelled_below_threshold():  # :594-600
    assert O.lp_iteration([0, 1, 1], [1], [0.5], [-1, 3])[0] == -1


def test_iteration_ignores_unlabelled_neighbours():  # :602-609
    assert O.lp_iteration([0, 1, 1], [1], [5.0], [-1, -1])[0] == -1


def test_iteration_threshold_is_inclusive_and_last_tie_wins():
    # a total of exactly 1.0 ties the threshold and is accepted; of two equal
    # totals the label that appears last wins (label_prop.rs:69-83)
    assert O.lp_iteration([0, 1, 1], [1], [1.0], [-1, 4])[0] == 4
    assert O.lp_iteration([0, 2, 2, 2], [1, 2], [2.0, 2.0], [-1, 3, 9])[0] == 9
    # ties are ordered by first appearance, not by the last vote: label 3
    # appears first (1.5 + 0.5), label 9 second (2.0), so 9 wins
    assert O.lp_iteration([0, 3, 3, 3, 3], [1, 2, 3], [1.5, 2.0, 0.5], [-1, 3, 9, 3])[0] == 9


def test_outliers_finds_labelled_neighbour():  # :611-620
    lab = O.lp_outliers([0, 1, 3, 4], [1, 0, 2, 1], [-1, -1, 42], 99)
    assert lab[0] >= 0 and lab[1] == 42


def test_outliers_random_fallback_for_isolated():  # :622-630
    lab = O.lp_outliers([0, 0, 0], [], [-1, 5], 99)
    assert 0 <= lab[0] <= 5


def test_remap():  # :632-651
    lab, k = O.lp_remap([10, 10, 20, 20, 10])
    assert k == 2 and list(lab) == [0, 0, 1, 1, 0]
    lab, k = O.lp_remap([5, -1, 5, -1])
    assert k == 3 and lab[0] == 0 and lab[2] == 0 and {lab[1], lab[3]} == {1, 2}


def test_loop_returns_valid_partition():  # :653-680
    n = 5
    ip, ix = [0], []
    for i in range(n):
        ix += sorted({(i + 1) % n, (i - 1) % n})
        ip.append(len(ix))
    part, k = O.lp_partition(ip, ix, [1.0] * len(ix), 3, 10, 42)
    assert len(part) == n and k > 0 and np.all(part < k)


# ---- the rest of label_propagation_init (label_prop.rs:243-564) -------------

def test_unit_range_normalisation():  # label_prop.rs:682-696
    m = O.lp_unit_range([[0.0, 10.0], [4.0, 20.0], [8.0, 30.0]])
    assert np.all(m >= -1 - 1e-7) and np.all(m <= 1 + 1e-7)
    assert m[0, 0] == -1.0 and m[2, 0] == 1.0 and m[0, 1] == -1.0 and m[2, 1] == 1.0


def _graph(small_knn):
    idx, dist, _ = small_knn
    return O.fuzzy_set(idx, dist, float(idx.shape[1]), True)


def test_coarse_graph_against_scipy(small_knn):
    """clip(R^T G P) with R the column-L2-normalised partition indicator
    (label_prop.rs:455-462), against a float64 scipy evaluation."""
    sp = __import__("pytest").importorskip("scipy.sparse")
    ip, ix, w = _graph(small_knn)
    n = len(ip) - 1
    part, k = O.lp_partition(ip, ix, w, 256, 20, 42)
    cip, cix, cw = O.lp_coarse_graph(ip, ix, w, part, k)
    g = sp.csr_matrix((w.astype(np.float64), ix, ip), shape=(n, n))
    p = sp.csr_matrix((np.ones(n), part, np.arange(n + 1)), shape=(n, k))
    sizes = np.bincount(part, minlength=k).astype(np.float64)
    r = p.multiply(1.0 / np.sqrt(sizes)[None, :]).tocsr()
    want = (r.T @ g @ p).tocsr()
    want.data = np.clip(want.data, 0.0, 1.0)
    want.sort_indices()
    np.testing.assert_array_equal(cip, want.indptr)
    np.testing.assert_array_equal(cix, want.indices)
    np.testing.assert_allclose(cw, want.data, rtol=2e-5, atol=1e-7)


def test_init_small_graph_random_base():  # label_prop.rs:700-739
    n = 10
    ip, ix = [0], []
    for i in range(n):
        ix += [j for j in range(n) if j != i]
        ip.append(len(ix))
    out = O.lp_init(ip, ix, [0.5] * len(ix), 4, None, 42)
    assert out.shape == (n, 4) and np.all(np.isfinite(out))
    np.testing.assert_allclose(np.linalg.norm(out, axis=1), 1.0, rtol=1e-6)  # base case: unit rows


def test_init_recursive_with_data(small_knn):
    """The full recursion on a 2,000-point graph with its data (PCA base case):
    finite, centred columns, reproducible, seed-dependent."""
    import workloads as W
    x, _ = W.blobs_sphere_np(2_000, 64, 8, 0.1, seed=5)  # the points behind small_knn
    ip, ix, w = _graph(small_knn)
    a = O.lp_init(ip, ix, w, 4, x, 42)
    b = O.lp_init(ip, ix, w, 4, x, 42)
    c = O.lp_init(ip, ix, w, 4, x, 7)
    assert a.shape == (2_000, 4) and np.all(np.isfinite(a))
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c)
    assert np.all(np.abs(a.mean(0)) < 1e-4 * np.abs(a).max() + 1e-6)
    assert 0 < np.abs(a).max() < 10
