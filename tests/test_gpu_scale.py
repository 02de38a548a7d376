"""GPU parity at the sizes the benchmark reports, through the C ABI.

The 200,000-point configuration (512-d, 100 anisotropic clusters with
Zipf(1.1) sizes plus 10% uniform noise, k = 15, dim 8) is generated and its
exact cosine kNN graph built on the GPU (input preparation, untimed). Then:

* the fuzzy simplicial set (src/graph/fuzzy_graph.rs:275-295) must equal the
  oracle's bit for bit: sigma, rho, CSR structure, neighbour order, weights;
* the full 50-epoch embedding (src/graph/embedding.rs:48-298, default
  parameters, random init) must equal the oracle's bit for bit, and so must a
  one-epoch gradient from a perturbed state; the final cluster labels of the
  two embeddings must reach an adjusted Rand index of at least 0.98.

A second case puts hub nodes of degree 16,500 and 20,000 (the degree profile
of the 2M-point graph, whose largest degree is 16,487) next to ordinary rows;
every hub edge has weight 1 and fires in every epoch, so a hub's serial
gradient sum runs over about 20,000 terms per epoch.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _assert_bits(a, b, what):
    if not np.array_equal(_bits(a), _bits(b)):
        d = np.abs(a.astype(np.float64) - b)
        raise AssertionError(f"{what} differs: {np.count_nonzero(_bits(a) != _bits(b))} values, "
                             f"max abs diff {d.max():.3g}")


@pytest.fixture(scope="module")
def knn_200k():
    import torch
    import workloads as W
    x, _ = W.anisotropic_torch(200_000, 512, 100, seed=1)
    idx, dist = W.knn_torch(x, 15)
    out = idx.to(torch.int32).cpu().numpy().view(np.uint32), dist.cpu().numpy()
    del x, idx, dist
    torch.cuda.empty_cache()
    return out


@pytest.fixture(scope="module")
def graph_200k(ctx, oracle, knn_200k):
    idx, dist = knn_200k
    g = ctx.fuzzy_set(idx, dist, 15.0, True)
    ref, s_ref, r_ref = oracle.fuzzy_set(idx, dist, 15.0, True, return_sigma_rho=True)
    return g, ref, s_ref, r_ref


def test_fuzzy_set_200k_vs_oracle(ctx, knn_200k, graph_200k):
    idx, dist = knn_200k
    g, (rip, rix, rw), s_ref, r_ref = graph_200k
    s, r = ctx.smooth_knn_dist(dist, 15)
    _assert_bits(s, s_ref, "sigma")
    _assert_bits(r, r_ref, "rho")
    ip, ix, w = g.export()
    assert np.array_equal(ip, rip), "indptr differs"
    assert np.array_equal(ix, rix), "neighbour order differs"
    _assert_bits(w, rw, "weights")
    assert g.nnz > 200_000 * 15


def test_embedding_200k_vs_oracle(ctx, oracle, graph_200k):
    """The full default run: 50 epochs, dim 8, random init, seed 1; then the
    final labels (src/clustering/*.rs via the oracle's restatement) of both
    embeddings: adjusted Rand index >= 0.98 (they are identical)."""
    g, (ip, ix, w), _, _ = graph_200k
    gpu = ctx.embed(g, 8, seed=1)
    ref = oracle.evoc_embedding(ip, ix, w, 8, seed=1)
    _assert_bits(gpu, ref, "embedding")
    lg = oracle.best_labels(oracle.build_cluster_layers(gpu, 5, 5, 0.2, 10))
    lr = oracle.best_labels(oracle.build_cluster_layers(ref, 5, 5, 0.2, 10))
    assert oracle.adjusted_rand_index(lg, lr) >= 0.98
    assert np.array_equal(lg, lr)


def test_gradient_200k_vs_oracle(ctx, oracle, graph_200k):
    g, (ip, ix, w), _, _ = graph_200k
    init = np.random.default_rng(4).uniform(-3, 3, (g.n, 8)).astype(np.float32)
    plan = ctx.plan(g, 8, seed=1)
    out, grad = plan.debug_run(init, 17, 18, want_grad=True)
    rout, rgrad = oracle.evoc_embedding(ip, ix, w, 8, init=init, seed=1, start_epoch=17,
                                        end_epoch=18, want_grad=True)
    nz = np.abs(rgrad) > 0
    assert np.abs(grad[nz] - rgrad[nz]).max() <= 1e-5 * np.abs(rgrad[nz]).max()
    _assert_bits(grad, rgrad, "gradient")
    _assert_bits(out, rout, "embedding")


def _hub_graph(n, deg, hubs, seed):
    rng = np.random.default_rng(seed)
    rows = [list(rng.integers(0, n, size=deg)) for _ in range(n)]
    wts = [list(rng.uniform(0.05, 0.9, size=deg)) for _ in range(n)]
    for h, k in hubs.items():
        nb = rng.choice(np.setdiff1d(np.arange(n), [h]), size=k, replace=False)
        rows[h] += list(nb)
        wts[h] += [1.0] * k
        for j in nb:
            rows[j].append(h)
            wts[j].append(1.0)
    ip = np.zeros(n + 1, dtype=np.int64)
    ip[1:] = np.cumsum([len(r) for r in rows])
    return ip, np.concatenate(rows).astype(np.uint32), np.concatenate(wts).astype(np.float32)


@pytest.mark.parametrize("dim", [4, 8])
def test_degree_16k_hubs_vs_oracle(ctx, oracle, dim):
    n = 40_000
    ip, ix, w = _hub_graph(n, 5, {11: 16_500, 20_000: 20_000, 39_999: 3_000}, seed=8)
    assert np.diff(ip).max() >= 20_000
    g = ctx.graph_from_csr(ip, ix, w)
    _assert_bits(ctx.embed(g, dim, seed=5), oracle.evoc_embedding(ip, ix, w, dim, seed=5),
                 "embedding")
    init = np.random.default_rng(dim).uniform(-1, 1, (n, dim)).astype(np.float32)
    plan = ctx.plan(g, dim, seed=5)
    _, grad = plan.debug_run(init, 3, 4, want_grad=True)
    _, ref = oracle.evoc_embedding(ip, ix, w, dim, init=init, seed=5, start_epoch=3, end_epoch=4,
                                   want_grad=True)
    _assert_bits(grad, ref, "gradient")


def test_degree_16k_hubs_from_the_fuzzy_set(ctx, oracle):
    """Hubs in a canonical (fuzzy-union) graph: rows whose kNN lists all
    point at a few hub nodes."""
    rng = np.random.default_rng(21)
    n, k = 60_000, 8
    idx = rng.integers(0, n, size=(n, k)).astype(np.uint32)
    idx[: 18_000, 0] = 7          # node 7 is in 18,000 kNN lists
    idx[18_000: 35_000, 1] = 59_000  # node 59,000 in 17,000 (self loops are dropped)
    dist = np.sort(rng.uniform(0.0, 1.0, size=(n, k)).astype(np.float32), axis=1)
    g = ctx.fuzzy_set(idx, dist, float(k), True)
    ip, ix, w = g.export()
    rip, rix, rw = oracle.fuzzy_set(idx, dist, float(k), True)
    assert np.array_equal(ip, rip) and np.array_equal(ix, rix)
    _assert_bits(w, rw, "weights")
    assert np.diff(ip).max() >= 16_000
    _assert_bits(ctx.embed(g, 8, seed=3), oracle.evoc_embedding(ip, ix, w, 8, seed=3),
                 "embedding")
