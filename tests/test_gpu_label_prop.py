"""GPU label-propagation partition (src/graph/label_prop.rs:202-230) against
the oracle: partitions and part counts must be identical (the vote sums are
the same f32 additions in the same order, and both draw from Philox)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _check(ctx, g, parts, n_iter, seed):
    ip, ix, w = g.export()
    got, k = ctx.label_prop_partition(g, parts, n_iter, seed)
    want, wk = O.lp_partition(ip, ix, w, parts, n_iter, seed)
    assert k == wk
    np.testing.assert_array_equal(got, want)
    assert got.max() < k
    return got, k


def test_ring(ctx):  # label_prop.rs:653-680 through the GPU
    n = 5
    adj = [[((i + 1) % n, 1.0), ((i - 1) % n, 1.0)] for i in range(n)]
    g = ctx.graph_from_adjacency([sorted(r) for r in adj])
    _check(ctx, g, 3, 10, 42)


@pytest.mark.parametrize("seed", [1, 42])
def test_fuzzy_graphs(ctx, small_knn, blobs_knn, seed):
    import evoc_gb300 as E
    for idx, dist, _ in (small_knn, blobs_knn):
        g = ctx.fuzzy_set(idx, dist, float(idx.shape[1]), True)
        _check(ctx, g, E.default_n_parts(g.n), 20, seed)
        _check(ctx, g, 37, 3, seed)  # few seeds, few rounds: the mop-up does most


def test_isolated_nodes_and_no_seeds(ctx):
    # nodes 3..5 have no edges: the fallback draws; with no seeds every node
    # stays unlabelled and gets its own part
    adj = [[(1, 1.0)], [(0, 1.0), (2, 0.4)], [(1, 0.4)], [], [], []]
    g = ctx.graph_from_adjacency(adj)
    _check(ctx, g, 2, 5, 7)
    part, k = _check(ctx, g, 0, 5, 7)
    assert k == 6 and sorted(part) == list(range(6))


def test_hub_rows_use_the_hashed_table(ctx):
    """A hub joined to every other node (degree 399, above the linear-search
    limit of 64) among ring-linked leaves: identical to the oracle."""
    n = 400
    rng = np.random.default_rng(11)
    hub_w = rng.uniform(0.3, 1.0, n - 1).astype(np.float32)
    adj = [[(j, float(hub_w[j - 1])) for j in range(1, n)]]
    for i in range(1, n):
        nb = {0: float(hub_w[i - 1]), 1 + (i % (n - 1)): 1.0, 1 + ((i - 2) % (n - 1)): 1.0}
        nb.pop(i, None)
        adj.append(sorted(nb.items()))
    g = ctx.graph_from_adjacency(adj)
    for parts, rounds, seed in ((40, 3, 5), (150, 20, 9), (400, 1, 2)):
        _check(ctx, g, parts, rounds, seed)
