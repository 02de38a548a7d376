"""label_propagation_init on the GPU (csrc/lp_init.cu) against the oracle's
restatement (oracle/evoc_oracle.cpp, label_prop.rs:403-564), through the C ABI.

The initial embedding must equal the oracle's bit for bit: the partition, the
coarse graphs' sparse algebra (its summation orders), the coarse data, the
base cases (PCA of the data, or random), the short coarse embeddings and the
expansion all follow the same arithmetic."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _same(a, b, what):
    if not np.array_equal(_bits(a), _bits(b)):
        d = np.abs(a.astype(np.float64) - b)
        raise AssertionError(f"{what}: {np.count_nonzero(_bits(a) != _bits(b))} of {a.size} values "
                             f"differ, max abs diff {d.max():.3g}")


@pytest.mark.parametrize("dim", [2, 4, 8])
def test_lp_init_with_data_vs_oracle(ctx, oracle, small_knn, dim):
    """2,000 x 64 blobs, k 15: one coarsening level, then the PCA base case."""
    import workloads as W
    idx, dist, _ = small_knn
    x, _ = W.blobs_sphere_np(2_000, 64, 8, 0.1, seed=5)
    g = ctx.fuzzy_set(idx, dist, 15.0, True)
    ip, ix, w = g.export()
    gpu = ctx.label_propagation_init(g, dim, x, seed=42)
    ref = oracle.lp_init(ip, ix, w, dim, x, seed=42)
    _same(gpu, ref, f"initial embedding dim {dim}")
    assert np.isfinite(gpu).all() and np.abs(gpu).max() > 0


def test_lp_init_without_data_vs_oracle(ctx, oracle, blobs_knn):
    """10,000 x 384 blobs, k 15, no data: the random base case, two levels."""
    idx, dist, _ = blobs_knn
    g = ctx.fuzzy_set(idx, dist, 15.0, True)
    ip, ix, w = g.export()
    gpu = ctx.label_propagation_init(g, 4, None, seed=7)
    _same(gpu, oracle.lp_init(ip, ix, w, 4, None, seed=7), "initial embedding")


def test_lp_init_blobs_10k_with_data_vs_oracle(ctx, oracle, blobs_knn):
    import workloads as W
    idx, dist, _ = blobs_knn
    x, _ = W.blobs_sphere_np(10_000, 384, 20, 0.15, seed=42)
    g = ctx.fuzzy_set(idx, dist, 15.0, True)
    ip, ix, w = g.export()
    gpu = ctx.label_propagation_init(g, 8, x, seed=42)
    _same(gpu, oracle.lp_init(ip, ix, w, 8, x, seed=42), "initial embedding")


def test_lp_init_general_graph_vs_oracle(ctx, oracle):
    """An asymmetric, unsorted-weight graph (not a fuzzy union): the expansion
    takes the graph's transpose."""
    rng = np.random.default_rng(3)
    n = 3_000
    rows = [np.unique(rng.integers(0, n, size=12)) for _ in range(n)]
    rows = [r[r != i] for i, r in enumerate(rows)]
    ip = np.zeros(n + 1, np.int64)
    ip[1:] = np.cumsum([len(r) for r in rows])
    ix = np.concatenate(rows).astype(np.uint32)
    w = rng.uniform(0.05, 1.0, size=len(ix)).astype(np.float32)
    g = ctx.graph_from_csr(ip, ix, w)
    gpu = ctx.label_propagation_init(g, 4, None, seed=11)
    _same(gpu, oracle.lp_init(ip, ix, w, 4, None, seed=11), "initial embedding")


def test_lp_init_then_embedding_is_the_reference_pipeline(ctx, oracle, small_knn):
    """evoc()'s order (lib.rs:271-310): the label-propagation init feeds the
    50-epoch embedding; the final embedding equals the oracle's."""
    import workloads as W
    idx, dist, _ = small_knn
    x, _ = W.blobs_sphere_np(2_000, 64, 8, 0.1, seed=5)
    g = ctx.fuzzy_set(idx, dist, 15.0, True)
    ip, ix, w = g.export()
    init = ctx.label_propagation_init(g, 4, x, seed=42)
    gpu = ctx.embed(g, 4, init=init, seed=42)
    ref = oracle.evoc_embedding(ip, ix, w, 4, init=oracle.lp_init(ip, ix, w, 4, x, seed=42),
                                seed=42)
    _same(gpu, ref, "embedding")
