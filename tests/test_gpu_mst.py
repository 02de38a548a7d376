"""build_mst on the GPU (csrc/mst.cu) against the oracle's restatement
(oracle/evoc_labels_oracle.cpp, src/clustering/mst.rs:82-166), through the C
ABI: the same edges in the same insertion order, weights bit for bit.

Equal mutual-reachability values are common (every edge shorter than both
core distances weighs the larger core distance), so the tie rules matter:
both sides take the smallest point index among equal values and add each
round's picks in ascending order of their component's smallest point index."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same_mst(gpu, ref, what):
    gu, gv, gw = gpu
    ru, rv, rw = ref
    assert len(gu) == len(ru), f"{what}: {len(gu)} edges against the oracle's {len(ru)}"
    bad = np.flatnonzero((gu != ru) | (gv != rv) | (gw.view(np.uint32) != rw.view(np.uint32)))
    if bad.size:
        i = bad[0]
        raise AssertionError(f"{what}: {bad.size} of {len(gu)} edges differ; first at {i}: "
                             f"gpu ({gu[i]}, {gv[i]}, {gw[i]!r}), "
                             f"oracle ({ru[i]}, {rv[i]}, {rw[i]!r})")


def _blobs(n, dim, k, seed, spread=0.3):
    rng = np.random.default_rng(seed)
    c = rng.normal(size=(k, dim)) * 4.0
    lab = rng.integers(0, k, n)
    return (c[lab] + spread * rng.normal(size=(n, dim))).astype(np.float32)


@pytest.mark.parametrize("dim", [1, 2, 3, 4, 5, 8, 12, 16])
def test_mst_blobs_vs_oracle(ctx, oracle, dim):
    x = _blobs(5_000, dim, 12, seed=dim)
    gpu = ctx.build_mst(x, 5)
    assert len(gpu[0]) == len(x) - 1
    _same_mst(gpu, oracle.build_mst(x, 5), f"dim {dim}")


@pytest.mark.parametrize("min_samples", [0, 1, 2, 10, 33, 64, 1000])
def test_mst_min_samples_vs_oracle(ctx, oracle, min_samples):
    """min_samples is clamped to n - 1 (mst.rs:104); 1000 > n - 1 here."""
    x = _blobs(3_000 if min_samples < 1000 else 60, 4, 8, seed=11)
    _same_mst(ctx.build_mst(x, min_samples), oracle.build_mst(x, min_samples),
              f"min_samples {min_samples}")


@pytest.mark.parametrize("min_samples", [1, 3, 5])
def test_mst_ties_vs_oracle(ctx, oracle, min_samples):
    """Integer grid points, every seventh one duplicated, in shuffled order:
    many equal distances (and zero distances), so the tie rules decide."""
    g = np.stack(np.meshgrid(np.arange(40), np.arange(30)), -1).reshape(-1, 2)
    x = np.concatenate([g, g[::7]]).astype(np.float32)
    x = x[np.random.default_rng(3).permutation(len(x))]
    _same_mst(ctx.build_mst(x, min_samples), oracle.build_mst(x, min_samples),
              f"grid, min_samples {min_samples}")


def test_mst_all_points_equal(ctx, oracle):
    x = np.ones((500, 4), np.float32)
    gpu = ctx.build_mst(x, 5)
    _same_mst(gpu, oracle.build_mst(x, 5), "identical points")
    assert (gpu[2] == 0).all()


def test_mst_reference_unit_cases(ctx):
    """The cases of mst.rs's own tests: empty, one point, two points at
    distance 5, a triangle, and a spanning tree with n - 1 edges."""
    assert len(ctx.build_mst(np.zeros((0, 2), np.float32), 1)[0]) == 0
    assert len(ctx.build_mst(np.array([[1.0, 2.0]], np.float32), 1)[0]) == 0
    u, v, w = ctx.build_mst(np.array([[0.0, 0.0], [3.0, 4.0]], np.float32), 1)
    assert len(u) == 1 and abs(float(w[0]) - 5.0) < 1e-6
    u, v, w = ctx.build_mst(np.array([[0.0, 0.0], [1.0, 0.0], [0.5, 0.866]], np.float32), 1)
    assert len(u) == 2
    x = _blobs(200, 3, 4, seed=1)
    u, v, w = ctx.build_mst(x, 3)
    parent = list(range(len(x)))

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a
    for a, b in zip(u, v):
        ra, rb = find(int(a)), find(int(b))
        assert ra != rb, "the edges form a cycle"
        parent[ra] = rb
    assert len({find(i) for i in range(len(x))}) == 1


def test_mst_of_gpu_embedding_and_labels(ctx, oracle, blobs_knn):
    """The 10k blobs embedded on the GPU (dim 4): the MST equals the oracle's,
    and the labels built on it by the clustering stage equal the labels the
    oracle builds from the embedding."""
    import evoc_gb300 as E
    idx, dist, _ = blobs_knn
    g = ctx.fuzzy_set(idx, dist, 15.0, True)
    emb = ctx.embed(g, 4, E.EvocEmbeddingParams(), seed=42)
    gpu = ctx.build_mst(emb, 5)
    _same_mst(gpu, oracle.build_mst(emb, 5), "embedding")
    lab_gpu = oracle.best_labels(oracle.build_cluster_layers_from_mst(*gpu, len(emb)))
    lab_ref = oracle.best_labels(oracle.build_cluster_layers(emb, 5, 5, 0.2, 10))
    assert np.array_equal(lab_gpu, lab_ref)


def test_mst_device_entry_matches_host_entry(ctx):
    torch = pytest.importorskip("torch")
    x = _blobs(20_000, 8, 30, seed=9)
    hu, hv, hw = ctx.build_mst(x, 5)
    dx = torch.from_numpy(x).cuda()
    du = torch.empty(len(x) - 1, dtype=torch.int64, device="cuda")
    dv = torch.empty_like(du)
    dw = torch.empty(len(x) - 1, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    m = ctx.build_mst_device(dx.data_ptr(), len(x), 8, 5, du.data_ptr(), dv.data_ptr(),
                             dw.data_ptr())
    assert m == len(x) - 1
    assert np.array_equal(du.cpu().numpy(), hu) and np.array_equal(dv.cpu().numpy(), hv)
    assert np.array_equal(dw.cpu().numpy().view(np.uint32), hw.view(np.uint32))
    again = ctx.build_mst(x, 5)
    assert all(np.array_equal(a, b) for a, b in zip(again, (hu, hv, hw)))


def test_mst_rejects_bad_input(ctx):
    import evoc_gb300 as E
    x = _blobs(100, 4, 3, seed=2)
    bad = x.copy()
    bad[17, 2] = np.nan
    with pytest.raises(E.EvocError) as e:
        ctx.build_mst(bad, 5)
    assert e.value.code == E.EVOC_ERR_INVALID_INPUT
    bad[17, 2] = np.inf
    with pytest.raises(E.EvocError):
        ctx.build_mst(bad, 5)
    with pytest.raises(E.EvocError) as e:
        ctx.build_mst(np.zeros((10, 17), np.float32), 5)
    assert e.value.code == E.EVOC_ERR_UNSUPPORTED
    with pytest.raises(E.EvocError) as e:
        ctx.build_mst(x, 65)
    assert e.value.code == E.EVOC_ERR_UNSUPPORTED
    # the context keeps working after the rejected calls
    assert len(ctx.build_mst(x, 5)[0]) == len(x) - 1
