"""CPU checks of the warm-start quality measures (evoc-rs_gb300/warm_start.py):
sampled trustworthiness@k (Venna & Kaski, 2001) and kNN label accuracy."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _blobs(n=1500, d=32, c=6, seed=0):
    import workloads as W
    x, lab = W.blobs_sphere_np(n, d, c, 0.1, seed)
    return torch.from_numpy(x), torch.from_numpy(lab.astype(np.int64))


def test_identity_embedding_is_perfect():
    import warm_start as WS
    x, lab = _blobs()
    q = WS.quality(x, x.clone(), lab, k=15, n_queries=400)
    assert q["trustworthiness"] == pytest.approx(1.0, abs=1e-9)
    assert q["knn_label_acc"] == 1.0


def test_random_embedding_is_about_one_half():
    import warm_start as WS
    x, lab = _blobs()
    emb = torch.from_numpy(np.random.default_rng(1).standard_normal((x.shape[0], 4)).astype(np.float32))
    q = WS.quality(x, emb, lab, k=15, n_queries=400)
    assert 0.4 < q["trustworthiness"] < 0.6
    assert q["knn_label_acc"] < 0.5


def test_trustworthiness_matches_the_definition():
    """Against a direct evaluation of T(k) = 1 - 2/(n k (2n - 3k - 1))
    sum_i sum_{j in U_k(i)} (r(i, j) - k) with every point as a query."""
    import warm_start as WS
    x, lab = _blobs(n=300, d=16, c=4, seed=3)
    emb = x[:, :3] + 0.05 * torch.from_numpy(
        np.random.default_rng(2).standard_normal((300, 3)).astype(np.float32))
    k, n = 10, 300
    xs, es = x.numpy().astype(np.float64), emb.numpy().astype(np.float64)
    sim = xs @ xs.T
    np.fill_diagonal(sim, -np.inf)
    d2 = ((es[:, None, :] - es[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d2, np.inf)
    pen = 0.0
    for i in range(n):
        order = np.argsort(-sim[i], kind="stable")
        rank = np.empty(n, np.int64)
        rank[order] = np.arange(1, n + 1)
        for j in np.argsort(d2[i], kind="stable")[:k]:
            pen += max(rank[j] - k, 0)
    want = 1.0 - 2.0 / (n * k * (2 * n - 3 * k - 1)) * pen
    got = WS.quality(x, emb, lab, k=k, n_queries=n)["trustworthiness"]
    assert got == pytest.approx(want, abs=2e-5)
