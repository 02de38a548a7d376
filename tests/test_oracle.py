"""CPU tests: the oracle against the reference's own pins and the golden fixtures.

The pins are the assertions of evoc-rs's unit and integration tests
(src/graph/fuzzy_graph.rs:306-454, src/graph/embedding.rs:317-464,
tests/integration_tests.rs:373-439, :476-501, :546-616). The golden fixtures
come from the independent pure-Python restatement in tests/golden/.
"""
import math

import numpy as np
import pytest

RANDOM123_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,expect", RANDOM123_KAT)
def test_philox_known_answers(oracle, ctr, key, expect):
    assert tuple(int(x) for x in oracle.philox(ctr, key)) == expect


def _ulps(got, x):
    ref = np.exp(x.astype(np.float64))
    sp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    return np.abs(got.astype(np.float64) - ref) / sp


def test_expf_error_bound(oracle):
    rng = np.random.default_rng(0)
    x = np.concatenate([np.linspace(-104, 88.7, 100001), -rng.exponential(3.0, 50000),
                        np.linspace(-103.9, -87.0, 20001)]).astype(np.float32)
    u = _ulps(oracle.expf_array(x), x)
    assert np.nanmax(u[np.isfinite(u)]) <= 1.5
    assert oracle.expf(0.0) == 1.0 and oracle.expf(-0.0) == 1.0
    assert oracle.expf(-200.0) == 0.0 and math.isinf(oracle.expf(100.0))
    assert math.isnan(oracle.expf(float("nan")))


def test_own_exp_vs_libm_exp_sigma(oracle, small_knn):
    """Deviation 1 (own exp instead of libm expf) moves sigma by < 1e-5 relative."""
    _, dist, _ = small_knn
    s1, r1 = oracle.smooth_knn_dist(dist, 15)
    s2, r2 = oracle.smooth_knn_dist(dist, 15, libm_exp=True)
    assert np.array_equal(r1, r2)
    rel = np.abs(s1 - s2) / np.abs(s2)
    assert rel.max() < 1e-5, rel.max()


# ---- fuzzy_graph.rs pins -------------------------------------------------------------
def test_smooth_knn_dist_basic(oracle):  # fuzzy_graph.rs:306-322
    sig, rho = oracle.smooth_knn_dist(np.array([[1.0, 2.0], [1.5, 3.0], [0.5, 1.5]]), 2, 1.0, 64)
    np.testing.assert_allclose(rho, [1.0, 1.5, 0.5], atol=1e-4)
    assert (sig > 0).all() and len(sig) == 3


def test_smooth_knn_dist_zero_local_connectivity(oracle):  # :324-332
    sig, rho = oracle.smooth_knn_dist(np.array([[0.0, 1.0, 2.0], [0.0, 1.0, 2.0]]), 2, 0.0, 64)
    assert (rho == 0).all() and len(sig) == 2


def test_knn_to_coo_basic(oracle):  # :334-351
    ip, ix, w = oracle.knn_to_coo(np.array([[1, 2], [0, 2], [0, 1]]),
                                  np.array([[1.0, 2.0], [1.0, 1.5], [2.0, 1.5]]),
                                  [1.0, 1.0, 1.0], [0.0, 0.0, 0.0])
    assert len(ip) == 4 and len(ix) == 6 and len(w) == 6
    assert ((w >= 0) & (w <= 1)).all()


def test_knn_to_coo_self_loop_excluded(oracle):  # :353-370
    ip, ix, w = oracle.knn_to_coo(np.array([[0, 1], [1, 0]]), np.array([[0.0, 1.0], [0.0, 1.0]]),
                                  [1.0, 1.0], [0.0, 0.0])
    assert len(w) == 2
    rows = np.repeat(np.arange(2), np.diff(ip))
    assert (rows != ix).all()


def test_symmetrise_fuzzy_union(oracle):  # :372-394
    ip, ix, w = oracle.symmetrise([0, 1, 2], [1, 0], [0.8, 0.6])
    assert len(ip) == 3 and len(ix) == 2
    np.testing.assert_allclose(w, 0.8 + 0.6 - 0.8 * 0.6, atol=1e-6)


def test_symmetrise_one_direction(oracle):  # :396-415
    ip, ix, w = oracle.symmetrise([0, 1, 1], [1], [0.7])
    assert len(ix) == 2
    np.testing.assert_allclose(w, 0.7, atol=1e-6)


def test_coo_to_adjacency_list(oracle):  # :417-437 (COO rows 0,0,1,2 -> CSR)
    ip, ix, w = oracle.symmetrise([0, 2, 3, 4], [1, 2, 2, 0], [0.5, 0.3, 0.8, 0.9])
    rows = [list(zip(ix[ip[i]:ip[i + 1]].tolist(), w[ip[i]:ip[i + 1]].tolist())) for i in range(3)]
    assert len(rows) == 3
    assert all(len(r) >= 1 for r in rows)


# ---- golden fixtures -------------------------------------------------------------
@pytest.mark.parametrize("lc", [1.0, 0.0, 1.5, 2.3])
def test_smooth_knn_golden(oracle, golden, lc):
    z = golden["smooth_knn"]
    s, r = oracle.smooth_knn_dist(z["dists"], 6, lc)
    assert np.array_equal(s, z[f"lc{lc}_sigma"]) and np.array_equal(r, z[f"lc{lc}_rho"])


def test_smooth_knn_golden_k_target(oracle, golden):
    z = golden["smooth_knn"]
    s, r = oracle.smooth_knn_dist(z["dists"], 4, 1.0)
    assert np.array_equal(s, z["k4_sigma"]) and np.array_equal(r, z["k4_rho"])


def test_fuzzy_set_golden(oracle, golden):
    f = golden["fuzzy_set"]
    (ip, ix, w), s, r = oracle.fuzzy_set(f["knn_idx"], f["knn_dist"], 5, True, True)
    assert np.array_equal(ip, f["indptr"]) and np.array_equal(ix, f["indices"])
    assert np.array_equal(w, f["weights"]) and np.array_equal(s, f["sigma"])
    ip, ix, w = oracle.fuzzy_set(f["knn_idx"], f["knn_dist"], 5, False)
    assert np.array_equal(ip, f["directed_indptr"]) and np.array_equal(ix, f["directed_indices"])
    assert np.array_equal(w, f["directed_weights"])


def test_embedding_golden(oracle, golden):
    e = golden["embedding"]
    o = oracle.evoc_embedding(e["g08_indptr"], e["g08_indices"], e["g08_weights"], 4,
                              n_epochs=30, seed=123)
    assert np.array_equal(o, e["g08_out"])
    o = oracle.evoc_embedding(e["tri_indptr"], e["tri_indices"], e["tri_weights"], 8,
                              n_epochs=50, seed=42)
    assert np.array_equal(o, e["tri_out"])
    o = oracle.evoc_embedding(e["cl_indptr"], e["cl_indices"], e["cl_weights"], 2, n_epochs=40,
                              seed=7, init=e["cl_init"], negative_sample_rate=2.0)
    assert np.array_equal(o, e["cl_out"])


# ---- embedding.rs pins -----------------------------------------------------------
TRI = ([0, 2, 4, 6], [1, 2, 0, 2, 0, 1], [1.0] * 6)


def test_embedding_empty_graph(oracle):  # embedding.rs:317-323
    out = oracle.evoc_embedding([0], [], [], 2)
    assert out.shape == (0, 2)


def test_embedding_single_node(oracle):  # :325-332
    out = oracle.evoc_embedding([0, 0], [], [], 2)
    assert out.shape == (1, 2)


@pytest.mark.parametrize("dim", [2, 4, 8, 16])
def test_embedding_output_shape(oracle, dim):  # :334-346
    assert oracle.evoc_embedding(*TRI, dim).shape == (3, dim)


def test_embedding_deterministic_and_seeds_differ(oracle):  # :348-376
    a = oracle.evoc_embedding(*TRI, 4, seed=123)
    b = oracle.evoc_embedding(*TRI, 4, seed=123)
    assert a.tobytes() == b.tobytes()
    c = oracle.evoc_embedding(*TRI, 4, seed=1)
    d = oracle.evoc_embedding(*TRI, 4, seed=2)
    assert not np.array_equal(c, d)


def test_embedding_initial_respected(oracle):  # :378-390
    init = np.array([[1.0, 2.0], [3.0, 4.0]], np.float32)
    out = oracle.evoc_embedding([0, 0, 0], [], [], 2, n_epochs=0, init=init)
    assert np.array_equal(out, init)


def test_embedding_attractive_edges_contract(oracle):  # :392-419
    init = np.array([[0.0, 0.0], [10.0, 0.0]], np.float32)
    out = oracle.evoc_embedding([0, 1, 2], [1, 0], [1.0, 1.0], 2, n_epochs=100,
                                negative_sample_rate=0.0, init=init)
    assert ((out[0] - out[1]) ** 2).sum() < 100.0


def test_embedding_no_nans_and_disconnected(oracle):  # :421-464
    assert np.isfinite(oracle.evoc_embedding(*TRI, 8)).all()
    out = oracle.evoc_embedding([0, 1, 2, 3, 4], [1, 0, 3, 2], [1.0] * 4, 4)
    assert out.shape == (4, 4) and np.isfinite(out).all()


# ---- integration-test analogues ---------------------------------------------------
def test_fuzzy_graph_cluster_separation(oracle):  # tests/integration_tests.rs:546-616
    rng = np.random.default_rng(42)
    data = np.concatenate([rng.normal(0, 0.5, (100, 4)), rng.normal(0, 0.5, (100, 4)) + [30, 0, 0, 0]])
    labels = np.repeat([0, 1], 100)
    d = np.sqrt(((data[:, None] - data[None]) ** 2).sum(-1))
    np.fill_diagonal(d, np.inf)
    idx = np.argsort(d, 1, kind="stable")[:, :8]
    dist = np.take_along_axis(d, idx, 1).astype(np.float32)
    ip, ix, w = oracle.fuzzy_set(idx, dist, 8.0, True)
    rows = np.repeat(np.arange(200), np.diff(ip))
    intra = w[labels[rows] == labels[ix]]
    inter = w[labels[rows] != labels[ix]]
    assert (intra.mean() if len(intra) else 0) > (inter.mean() if len(inter) else 0)


def test_embedding_reproducibility(oracle):  # tests/integration_tests.rs:476-501
    g = ([0, 2, 4, 7, 8], [1, 2, 0, 2, 0, 1, 3, 2], [1.0, 0.5, 1.0, 0.8, 0.5, 0.8, 0.9, 0.9])
    a = oracle.evoc_embedding(*g, 4, n_epochs=30, seed=123)
    b = oracle.evoc_embedding(*g, 4, n_epochs=30, seed=123)
    assert a.tobytes() == b.tobytes()


def test_fuzzy_set_properties(oracle, small_knn):
    idx, dist, _ = small_knn
    ip, ix, w = oracle.fuzzy_set(idx, dist, 15.0, True)
    n = len(ip) - 1
    rows = np.repeat(np.arange(n), np.diff(ip))
    assert (rows != ix).all()
    assert ((w > 0) & (w <= 1)).all()
    for i in range(0, n, 97):  # sorted, unique columns
        r = ix[ip[i]:ip[i + 1]]
        assert (np.diff(r.astype(np.int64)) > 0).all()
    a = {(int(r), int(c)): float(x) for r, c, x in zip(rows, ix, w)}
    assert all(a[(c, r)] == x for (r, c), x in a.items())  # symmetric, same bits
