"""GPU parity of the fuzzy simplicial set, through the C ABI.

Bar: bit-exact sigma, rho, CSR structure, neighbour order and weights against
the oracle (which is itself pinned by the golden fixtures and by the pins of
src/graph/fuzzy_graph.rs:306-454).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same_graph(g, ref):
    ip, ix, w = g.export()
    rip, rix, rw = ref
    assert np.array_equal(ip, rip), "indptr differs"
    assert np.array_equal(ix, rix), "neighbour order differs"
    assert np.array_equal(w.view(np.uint32), rw.view(np.uint32)), "weights differ"


@pytest.mark.parametrize("lc", [1.0, 0.0, 1.5, 2.3])
def test_smooth_knn_golden(ctx, golden, lc):
    z = golden["smooth_knn"]
    s, r = ctx.smooth_knn_dist(z["dists"], 6, lc)
    assert np.array_equal(s, z[f"lc{lc}_sigma"]) and np.array_equal(r, z[f"lc{lc}_rho"])
    s, r = ctx.smooth_knn_dist(z["dists"], 4, 1.0)
    assert np.array_equal(s, z["k4_sigma"]) and np.array_equal(r, z["k4_rho"])


def test_smooth_knn_pins(ctx):  # fuzzy_graph.rs:306-332
    s, r = ctx.smooth_knn_dist(np.array([[1.0, 2.0], [1.5, 3.0], [0.5, 1.5]]), 2, 1.0, 64)
    np.testing.assert_allclose(r, [1.0, 1.5, 0.5], atol=1e-4)
    assert (s > 0).all()
    s, r = ctx.smooth_knn_dist(np.array([[0.0, 1.0, 2.0], [0.0, 1.0, 2.0]]), 2, 0.0, 64)
    assert (r == 0).all()


def test_fuzzy_union_pins(ctx):  # fuzzy_graph.rs:372-415 through the whole path
    # rows 0 -> 1 (d small) and 1 -> 0: both directions, union of equal weights
    g = ctx.fuzzy_set(np.array([[1], [0]]), np.array([[0.5], [0.5]]), 1.0, True)
    ip, ix, w = g.export()
    assert ip.tolist() == [0, 1, 2] and ix.tolist() == [1, 0]
    np.testing.assert_allclose(w, 1.0)


def test_fuzzy_golden(ctx, golden):
    f = golden["fuzzy_set"]
    g = ctx.fuzzy_set(f["knn_idx"], f["knn_dist"], 5.0, True)
    _same_graph(g, (f["indptr"], f["indices"], f["weights"]))
    g = ctx.fuzzy_set(f["knn_idx"], f["knn_dist"], 5.0, False)
    _same_graph(g, (f["directed_indptr"], f["directed_indices"], f["directed_weights"]))


def test_fuzzy_blobs_vs_oracle(ctx, oracle, blobs_knn):
    """10,000 x 384, k = 15 (the CPU configuration's shape)."""
    idx, dist, _ = blobs_knn
    s_gpu, r_gpu = ctx.smooth_knn_dist(dist, 15)
    ref, s_ref, r_ref = oracle.fuzzy_set(idx, dist, 15.0, True, return_sigma_rho=True)
    assert np.array_equal(s_gpu, s_ref) and np.array_equal(r_gpu, r_ref)
    _same_graph(ctx.fuzzy_set(idx, dist, 15.0, True), ref)
    _same_graph(ctx.fuzzy_set(idx, dist, 15.0, False), oracle.fuzzy_set(idx, dist, 15.0, False))


@pytest.mark.parametrize("eff_k", [7.5, 30.0, -3.0])
def test_fuzzy_effective_k(ctx, oracle, small_knn, eff_k):
    """k = trunc(effective_n_neighbours), or row 0's length when it does not
    convert (fuzzy_graph.rs:284-286)."""
    idx, dist, _ = small_knn
    _same_graph(ctx.fuzzy_set(idx, dist, eff_k, True), oracle.fuzzy_set(idx, dist, eff_k, True))


def test_fuzzy_ragged_duplicates_self_loops(ctx, oracle):
    rng = np.random.default_rng(11)
    n, k = 3000, 24
    idx = rng.integers(0, n, size=(n, k)).astype(np.uint32)
    idx[:, 0] = np.arange(n)                      # self loops
    idx[::7, 5] = idx[::7, 4]                     # duplicates (last wins)
    lens = rng.integers(1, k + 1, size=n)
    for i in range(n):
        idx[i, lens[i]:] = 0xFFFFFFFF             # ragged rows
    dist = np.sort(rng.uniform(0.0, 2.0, size=(n, k)).astype(np.float32), axis=1)
    for sym in (True, False):
        _same_graph(ctx.fuzzy_set(idx, dist, float(k), sym), oracle.fuzzy_set(idx, dist, float(k), sym))


@pytest.mark.parametrize("k", [1, 33, 100])
def test_fuzzy_row_widths(ctx, oracle, k):
    rng = np.random.default_rng(k)
    n = 1500
    idx = np.stack([rng.permutation(n)[:k] for _ in range(n)]).astype(np.uint32)
    dist = np.sort(rng.uniform(0.01, 1.0, size=(n, k)).astype(np.float32), axis=1)
    _same_graph(ctx.fuzzy_set(idx, dist, float(k), True), oracle.fuzzy_set(idx, dist, float(k), True))


def test_fuzzy_errors(ctx):
    import evoc_gb300 as E
    idx = np.array([[1], [5]], np.uint32)          # 5 >= n
    with pytest.raises(E.EvocError) as ei:
        ctx.fuzzy_set(idx, np.ones((2, 1), np.float32), 1.0, True)
    assert ei.value.code == E.EVOC_ERR_INVALID_INPUT
    with pytest.raises(E.EvocError) as ei:
        ctx.fuzzy_set(np.array([[1], [0]]), np.array([[np.nan], [1.0]]), 1.0, True)
    assert ei.value.code == E.EVOC_ERR_INVALID_INPUT
    with pytest.raises(E.EvocError) as ei:  # empty row with local_connectivity 1
        ctx.fuzzy_set(np.array([[0xFFFFFFFF], [0]], np.uint32), np.ones((2, 1)), 1.0, True)
    assert ei.value.code == E.EVOC_ERR_INVALID_INPUT
    with pytest.raises(E.EvocError) as ei:
        ctx.fuzzy_set(np.zeros((0, 3), np.uint32), np.zeros((0, 3), np.float32), 3.0, True)
    assert ei.value.code == E.EVOC_ERR_INVALID_ARGUMENT
    # the context stays usable after errors
    g = ctx.fuzzy_set(np.array([[1], [0]]), np.array([[0.5], [0.5]]), 1.0, True)
    assert g.nnz == 2


def test_fuzzy_large_properties(ctx):
    """200,000 rows, k = 15: size-independent properties and run-to-run identity."""
    rng = np.random.default_rng(3)
    n, k = 200_000, 15
    base = np.arange(n)[:, None]
    idx = ((base + rng.integers(1, 2000, size=(n, k))) % n).astype(np.uint32)
    dist = np.sort(rng.uniform(0.0, 1.0, size=(n, k)).astype(np.float32), axis=1)
    g1 = ctx.fuzzy_set(idx, dist, float(k), True)
    ip, ix, w = g1.export()
    ip2, ix2, w2 = ctx.fuzzy_set(idx, dist, float(k), True).export()
    assert np.array_equal(ip, ip2) and np.array_equal(ix, ix2) and np.array_equal(w, w2)
    assert ((w > 0) & (w <= 1)).all()
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(ip))
    assert (rows != ix).all()
    key = rows * n + ix
    assert (np.diff(key) > 0).all()              # sorted, unique
    tkey = ix.astype(np.int64) * n + rows        # symmetric with identical bits
    order = np.argsort(tkey)
    assert np.array_equal(tkey[order], key)
    assert np.array_equal(w[order].view(np.uint32), w.view(np.uint32))


def _drop_self(raw_i, raw_d, k):
    """The reference's self removal (nearest_neighbour_gpu.rs:289-300): row i
    keeps its first k candidates that are not i; short rows are padded."""
    n = raw_i.shape[0]
    out_i = np.full((n, k), 0xFFFFFFFF, np.uint32)
    out_d = np.zeros((n, k), np.float32)
    for r in range(n):
        keep = [j for j in range(raw_i.shape[1]) if raw_i[r, j] != r][:k]
        out_i[r, :len(keep)] = raw_i[r, keep]
        out_d[r, :len(keep)] = raw_d[r, keep]
    return out_i, out_d


def test_fuzzy_set_from_raw_device_knn(ctx, small_knn):
    """A raw (k + 1)-wide device kNN result, the query itself at a random
    position in most rows, some rows without it, some padded at the end:
    removing self on the device gives the same graph as the host-side
    removal followed by evoc_fuzzy_set."""
    import torch
    idx, dist, _ = small_knn
    n, k = idx.shape
    rng = np.random.default_rng(3)
    raw_i = np.empty((n, k + 1), np.uint32)
    raw_d = np.empty((n, k + 1), np.float32)
    for r in range(n):
        row_i, row_d = list(idx[r].astype(np.uint32)), list(dist[r])
        if rng.random() < 0.9:
            p = int(rng.integers(0, k + 1))
            row_i.insert(p, r)
            row_d.insert(p, 0.0)
        else:
            row_i.append(int(rng.integers(0, n)))
            row_d.append(row_d[-1])
        raw_i[r], raw_d[r] = row_i, row_d
        if rng.random() < 0.05:  # a ragged candidate row
            raw_i[r, -3:] = 0xFFFFFFFF
    want_i, want_d = _drop_self(raw_i, raw_d, k)
    ref = ctx.fuzzy_set(want_i, want_d, float(k), True)
    di = torch.from_numpy(raw_i.view(np.int32)).cuda()
    dd = torch.from_numpy(raw_d).cuda()
    torch.cuda.synchronize()
    g = ctx.fuzzy_set_device_raw(di.data_ptr(), dd.data_ptr(), n, k + 1, k, float(k), True)
    for a, b in zip(g.export(), ref.export()):
        np.testing.assert_array_equal(a, b)
    import evoc_gb300 as E
    with pytest.raises(E.EvocError):
        ctx.fuzzy_set_device_raw(di.data_ptr(), dd.data_ptr(), n, k, k + 1, float(k), True)
