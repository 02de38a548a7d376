"""GPU parity of evoc_embedding (src/graph/embedding.rs:48-298), through the C ABI.

Bar: bit-exact embeddings and one-epoch gradients against the oracle on the
same inputs (the shared arithmetic contract makes them bit-identical); the
1e-5 relative gradient tolerance of the specification is asserted as well.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _assert_bits(a, b, what="embedding"):
    if not np.array_equal(_bits(a), _bits(b)):
        d = np.abs(a.astype(np.float64) - b)
        raise AssertionError(f"{what} differs: {np.count_nonzero(_bits(a) != _bits(b))} values, "
                             f"max abs diff {d.max():.3g}")


def test_embedding_golden(ctx, golden):
    import evoc_gb300 as E
    e = golden["embedding"]
    g = ctx.graph_from_csr(e["g08_indptr"], e["g08_indices"], e["g08_weights"])
    _assert_bits(ctx.embed(g, 4, E.EvocEmbeddingParams(n_epochs=30), seed=123), e["g08_out"])
    g = ctx.graph_from_csr(e["tri_indptr"], e["tri_indices"], e["tri_weights"])
    _assert_bits(ctx.embed(g, 8, E.EvocEmbeddingParams(n_epochs=50), seed=42), e["tri_out"])
    g = ctx.graph_from_csr(e["cl_indptr"], e["cl_indices"], e["cl_weights"])
    p = E.EvocEmbeddingParams(n_epochs=40, negative_sample_rate=2.0)
    _assert_bits(ctx.embed(g, 2, p, init=e["cl_init"], seed=7), e["cl_out"])


def test_embedding_pins(ctx):  # embedding.rs:317-464
    import evoc_gb300 as E
    tri = ctx.graph_from_adjacency([[(1, 1.0), (2, 1.0)], [(0, 1.0), (2, 1.0)], [(0, 1.0), (1, 1.0)]])
    assert ctx.embed(ctx.graph_from_csr([0], [], []), 2).shape == (0, 2)
    assert ctx.embed(ctx.graph_from_csr([0, 0], [], []), 2).shape == (1, 2)
    for dim in (2, 4, 8, 16):
        assert ctx.embed(tri, dim).shape == (3, dim)
    a, b = ctx.embed(tri, 4, seed=123), ctx.embed(tri, 4, seed=123)
    assert a.tobytes() == b.tobytes()
    assert not np.array_equal(ctx.embed(tri, 4, seed=1), ctx.embed(tri, 4, seed=2))
    init = np.array([[1.0, 2.0], [3.0, 4.0]], np.float32)
    out = ctx.embed(ctx.graph_from_csr([0, 0, 0], [], []), 2, E.EvocEmbeddingParams(n_epochs=0), init=init)
    assert np.array_equal(out, init)
    pair = ctx.graph_from_adjacency([[(1, 1.0)], [(0, 1.0)]])
    out = ctx.embed(pair, 2, E.EvocEmbeddingParams(n_epochs=100, negative_sample_rate=0.0),
                    init=np.array([[0.0, 0.0], [10.0, 0.0]], np.float32))
    assert ((out[0] - out[1]) ** 2).sum() < 100.0
    assert np.isfinite(ctx.embed(tri, 8)).all()
    two = ctx.graph_from_adjacency([[(1, 1.0)], [(0, 1.0)], [(3, 1.0)], [(2, 1.0)]])
    assert np.isfinite(ctx.embed(two, 4)).all()


@pytest.fixture(scope="module")
def blobs_graph(ctx, oracle, blobs_knn):
    idx, dist, labels = blobs_knn
    g = ctx.fuzzy_set(idx, dist, 15.0, True)
    return g, g.export(), labels


def test_blobs_full_run_vs_oracle(ctx, oracle, blobs_graph):
    """10,000 points, k = 15, dim 4, default parameters, 50 epochs, random init."""
    g, (ip, ix, w), _ = blobs_graph
    gpu = ctx.embed(g, 4, seed=42)
    ref = oracle.evoc_embedding(ip, ix, w, 4, seed=42)
    _assert_bits(gpu, ref)


@pytest.mark.parametrize("dim,neg_rate,n_epochs", [(2, 1.0, 20), (8, 3.7, 15), (16, 0.0, 10),
                                                  (5, 1.0, 12), (12, 0.5, 8), (4, 1.0, 80)])
def test_blobs_dims_and_rates(ctx, oracle, blobs_graph, dim, neg_rate, n_epochs):
    import evoc_gb300 as E
    g, (ip, ix, w), _ = blobs_graph
    init = np.random.default_rng(dim).uniform(-1, 1, (g.n, dim)).astype(np.float32)
    p = E.EvocEmbeddingParams(n_epochs=n_epochs, negative_sample_rate=neg_rate, noise_level=0.3)
    gpu = ctx.embed(g, dim, p, init=init, seed=9)
    ref = oracle.evoc_embedding(ip, ix, w, dim, n_epochs=n_epochs, negative_sample_rate=neg_rate,
                                noise_level=0.3, init=init, seed=9)
    _assert_bits(gpu, ref)


def test_one_epoch_gradient(ctx, oracle, blobs_graph):
    """Gradient of epoch t from the same state (schedule advanced to t)."""
    g, (ip, ix, w), _ = blobs_graph
    rng = np.random.default_rng(1)
    init = rng.uniform(-2, 2, (g.n, 4)).astype(np.float32)
    plan = ctx.plan(g, 4, seed=42)
    for t in (1, 7, 30):
        out, grad = plan.debug_run(init, t, t + 1, want_grad=True)
        rout, rgrad = oracle.evoc_embedding(ip, ix, w, 4, init=init, seed=42, start_epoch=t,
                                            end_epoch=t + 1, want_grad=True)
        nz = np.abs(rgrad) > 0
        rel = np.abs(grad[nz] - rgrad[nz]) / np.abs(rgrad[nz])
        assert rel.max() <= 1e-5
        _assert_bits(grad, rgrad, "gradient")
        _assert_bits(out, rout)


def test_stats_vs_oracle(ctx, oracle, blobs_graph):
    g, (ip, ix, w), _ = blobs_graph
    plan = ctx.plan(g, 4, seed=42)
    st = plan.stats()
    _, rst = oracle.evoc_embedding(ip, ix, w, 4, seed=42, want_stats=True)
    assert np.array_equal(st, rst)
    assert st[0, 0] == 0 and st[1:, 0].min() > 0


def test_launch_shape_does_not_change_results(ctx, blobs_graph, monkeypatch):
    g, _, _ = blobs_graph
    outs = []
    for wpb in ("1", "2", "4"):
        monkeypatch.setenv("EVOC_WARPS_PER_BLOCK", wpb)
        outs.append(ctx.embed(g, 8, seed=5))
    monkeypatch.delenv("EVOC_WARPS_PER_BLOCK")
    for o in outs[1:]:
        _assert_bits(o, outs[0])


def test_slots_and_scan_paths_agree(ctx, oracle, blobs_graph, monkeypatch):
    """The per-epoch gradient-slot path and the bit-plane scanning fallback."""
    g, (ip, ix, w), _ = blobs_graph
    outs = {}
    for path in ("slots", "scan"):
        monkeypatch.setenv("EVOC_EPOCH_PATH", path)
        outs[path] = ctx.embed(g, 8, seed=21)
        plan = ctx.plan(g, 8, seed=21)
        rng = np.random.default_rng(2)
        init = rng.uniform(-1, 1, (g.n, 8)).astype(np.float32)
        outs[path + "_grad"] = plan.debug_run(init, 9, 10, want_grad=True)[1]
    monkeypatch.delenv("EVOC_EPOCH_PATH")
    _assert_bits(outs["slots"], outs["scan"])
    _assert_bits(outs["slots_grad"], outs["scan_grad"], "gradient")
    _assert_bits(outs["slots"], oracle.evoc_embedding(ip, ix, w, 8, seed=21))


def test_general_graph_path(ctx, oracle, blobs_graph):
    """A graph uploaded from the host takes the general set-up (transpose of
    the upper entries); on a symmetric graph it must equal the fuzzy output's."""
    g, (ip, ix, w), _ = blobs_graph
    g2 = ctx.graph_from_csr(ip, ix, w)
    _assert_bits(ctx.embed(g2, 4, seed=3), ctx.embed(g, 4, seed=3))


def test_asymmetric_graph_vs_oracle(ctx, oracle):
    """Directed graphs (symmetrise = false), duplicates and self loops:
    edges are the i < j entries of each row in adjacency order (embedding.rs:79-90)."""
    rng = np.random.default_rng(17)
    n, deg = 4000, 9
    ip = np.arange(0, n * deg + 1, deg, dtype=np.int64)
    ix = rng.integers(0, n, size=n * deg).astype(np.uint32)
    ix[::11] = np.repeat(np.arange(n), deg)[::11]        # some self loops
    ix[5::13] = ix[4::13][: len(ix[5::13])]              # duplicates
    w = rng.uniform(0.0, 1.0, size=n * deg).astype(np.float32)
    w[::17] = 0.0
    g = ctx.graph_from_csr(ip, ix, w)
    _assert_bits(ctx.embed(g, 8, seed=11), oracle.evoc_embedding(ip, ix, w, 8, seed=11))


@pytest.mark.parametrize("dim", [4, 8, 16])
def test_hub_nodes_vs_oracle(ctx, oracle, dim):
    """Hub nodes (degree in the thousands, weight 1: they fire every epoch)
    next to ordinary rows: a hub's serial gradient sum runs over hundreds of
    terms per epoch, longer than one window of the epoch kernel."""
    rng = np.random.default_rng(5)
    n, deg = 3000, 6
    hubs = {7: 2500, 1500: 900, 2999: 300}
    rows = [list(rng.integers(0, n, size=deg)) for _ in range(n)]
    wts = [list(rng.uniform(0.05, 0.9, size=deg)) for _ in range(n)]
    for h, k in hubs.items():
        nb = rng.choice(n, size=k, replace=False)
        rows[h] += list(nb)
        wts[h] += [1.0] * k
        for j in nb:  # symmetric: the partners list the hub too
            rows[j].append(h)
            wts[j].append(1.0)
    ip = np.zeros(n + 1, dtype=np.int64)
    ip[1:] = np.cumsum([len(r) for r in rows])
    ix = np.concatenate(rows).astype(np.uint32)
    w = np.concatenate(wts).astype(np.float32)
    g = ctx.graph_from_csr(ip, ix, w)
    _assert_bits(ctx.embed(g, dim, seed=13), oracle.evoc_embedding(ip, ix, w, dim, seed=13))
    init = rng.uniform(-1, 1, (n, dim)).astype(np.float32)
    plan = ctx.plan(g, dim, seed=13)
    _, grad = plan.debug_run(init, 4, 5, want_grad=True)
    _, ref = oracle.evoc_embedding(ip, ix, w, dim, init=init, seed=13, start_epoch=4,
                                   end_epoch=5, want_grad=True)
    _assert_bits(grad, ref, "gradient")


def test_errors_keep_context_usable(ctx):
    import evoc_gb300 as E
    with pytest.raises(E.EvocError) as ei:
        ctx.graph_from_csr([0, 1, 2], [1, 9], [1.0, 1.0])
    assert ei.value.code == E.EVOC_ERR_INVALID_INPUT
    g = ctx.graph_from_adjacency([[(1, 1.0)], [(0, 1.0)]])
    with pytest.raises(E.EvocError) as ei:
        ctx.embed(g, 17)
    assert ei.value.code == E.EVOC_ERR_UNSUPPORTED
    with pytest.raises(E.EvocError) as ei:
        ctx.embed(g, 2, E.EvocEmbeddingParams(negative_sample_rate=1e9))
    assert ei.value.code == E.EVOC_ERR_UNSUPPORTED
    assert ctx.embed(g, 2).shape == (2, 2)


def test_batched_equals_individual(ctx, oracle):
    import evoc_gb300 as E
    import workloads as W
    graphs, refs, seeds = [], [], []
    for q, n in enumerate([300, 1200, 2, 800, 1]):
        if n > 2:
            x, _ = W.blobs_sphere_np(n, 32, 4, 0.1, seed=100 + q)
            idx, dist = W.knn_np(x, 10)
            g = ctx.fuzzy_set(idx, dist, 10.0, True)
        elif n == 2:
            g = ctx.graph_from_adjacency([[(1, 0.5)], [(0, 0.5)]])
        else:
            g = ctx.graph_from_csr([0, 0], [], [])
        graphs.append(g)
        seeds.append(1000 + q)
    p = E.EvocEmbeddingParams(n_epochs=25)
    outs = ctx.embed_batched(graphs, 4, p, seeds=seeds)
    for g, o, s in zip(graphs, outs, seeds):
        _assert_bits(o, ctx.embed(g, 4, p, seed=s))
        ip, ix, w = g.export()
        _assert_bits(o, oracle.evoc_embedding(ip, ix, w, 4, n_epochs=25, seed=s))
    inits = [np.random.default_rng(q).uniform(-1, 1, (g.n, 4)).astype(np.float32)
             for q, g in enumerate(graphs)]
    outs = ctx.embed_batched(graphs, 4, p, inits=inits, seeds=seeds)
    for g, o, s, i0 in zip(graphs, outs, seeds, inits):
        _assert_bits(o, ctx.embed(g, 4, p, init=i0, seed=s))
    # the device-resident batched plan: problems' rows concatenated in order
    import torch
    plan = ctx.plan_batched(graphs, 4, p, seeds=seeds)
    d_out = torch.empty(plan.n, 4, dtype=torch.float32, device="cuda")
    plan.run_device(None, d_out.data_ptr())
    h = d_out.cpu().numpy()
    base = 0
    for g, s in zip(graphs, seeds):
        _assert_bits(h[base:base + g.n], ctx.embed(g, 4, p, seed=s))
        base += g.n


def test_gather_peak_measures_and_rejects_bad_sizes(ctx):
    import evoc_gb300 as E
    gbs = ctx.gather_peak(8 << 20)
    assert 50.0 < gbs < 100000.0
    with pytest.raises(E.EvocError) as ei:
        ctx.gather_peak(16)
    assert ei.value.code == E.EVOC_ERR_INVALID_ARGUMENT


def test_closing_a_context_frees_its_graphs_and_plans():
    """Graphs and plans must not outlive their context's stream: closing the
    context frees them first, and their later finalisers do nothing."""
    import evoc_gb300 as E
    c2 = E.Context(0)
    g = c2.graph_from_adjacency([[(1, 1.0)], [(0, 1.0)]])
    p = c2.plan(g, 4)
    c2.close()
    assert g.handle is None and p.handle is None
    g.free()
    p.free()
    del g, p


def test_blocks_equal_separate_problems(ctx):
    """Many problems as one block-diagonal graph: the batched fuzzy set's
    blocks equal the problems' own fuzzy sets (indices shifted), and the
    blocks' embeddings (host outputs and device plan) equal separate runs."""
    import torch
    import evoc_gb300 as E
    import workloads as W
    sizes, knn, graphs, seeds = [300, 1200, 40, 800], [], [], []
    for q, n in enumerate(sizes):
        x, _ = W.blobs_sphere_np(n, 32, 4, 0.1, seed=200 + q)
        idx, dist = W.knn_np(x, 10)
        idx[::7, 9] = 0xFFFFFFFF  # some ragged rows
        knn.append((idx, dist))
        graphs.append(ctx.fuzzy_set(idx, dist, 10.0, True))
        seeds.append(3000 + q)
    gb = ctx.fuzzy_set_batched(knn, 10.0, True)
    ip, ix, w = gb.export()
    base = 0
    for n, g in zip(sizes, graphs):
        rip, rix, rw = g.export()
        assert np.array_equal(ip[base:base + n + 1] - ip[base], rip)
        assert np.array_equal(ix[ip[base]:ip[base + n]] - base, rix)
        _assert_bits(w[ip[base]:ip[base + n]], rw, "weights")
        base += n
    p = E.EvocEmbeddingParams(n_epochs=20)
    outs = ctx.embed_blocks(gb, sizes, 4, p, seeds=seeds)
    for o, g, s in zip(outs, graphs, seeds):
        _assert_bits(o, ctx.embed(g, 4, p, seed=s))
    plan = ctx.plan_blocks(gb, sizes, 4, p, seeds=seeds)
    d_out = torch.empty(plan.n, 4, dtype=torch.float32, device="cuda")
    plan.run_device(None, d_out.data_ptr())
    _assert_bits(d_out.cpu().numpy(), np.concatenate(outs))


def test_blocks_reject_bad_input(ctx):
    import evoc_gb300 as E
    idx = np.array([[1], [0], [5]], np.uint32)  # 5 is outside a 3-row problem
    dist = np.ones((3, 1), np.float32)
    ok = np.array([[1], [0]], np.uint32), np.ones((2, 1), np.float32)
    with pytest.raises(E.EvocError) as ei:
        ctx.fuzzy_set_batched([ok, (idx, dist)], 1.0)
    assert ei.value.code == E.EVOC_ERR_INVALID_INPUT
    g = ctx.fuzzy_set_batched([ok, ok], 1.0)
    with pytest.raises(E.EvocError) as ei:
        ctx.plan_blocks(g, [2, 3], 4)
    assert ei.value.code == E.EVOC_ERR_INVALID_ARGUMENT
    cross = ctx.graph_from_adjacency([[(2, 1.0)], [(0, 1.0)], [(0, 1.0)], [(1, 1.0)]])
    with pytest.raises(E.EvocError) as ei:
        ctx.plan_blocks(cross, [2, 2], 4)
    assert ei.value.code == E.EVOC_ERR_INVALID_INPUT


def test_every_epoch_kernel_config_gives_the_same_embedding(ctx, blobs_knn):
    """All slots-kernel variants x warps per block x a blocks-per-SM cap give
    bit-identical embeddings (the autotuner may pick any of them), launched
    per epoch (variants 0-3) or as one cooperative launch for all epochs
    (4-7, run through the plan's normal run path)."""
    import torch
    idx, dist, _ = blobs_knn
    g = ctx.fuzzy_set(idx, dist, 15.0, True)
    plan = ctx.plan(g, 4, seed=3)
    ref = plan.debug_run(None, 0, plan.n_epochs)
    out_d = torch.empty(g.n, 4, dtype=torch.float32, device="cuda")
    for variant in range(8):
        for wpb in (1, 2, 4):
            for bps in (0, 2):
                plan.set_config(variant, wpb, bps)
                if variant < 4:
                    out = plan.debug_run(None, 0, plan.n_epochs)
                else:
                    plan.run_device(None, out_d.data_ptr())
                    out = out_d.cpu().numpy()
                assert np.array_equal(out.view(np.uint32), ref.view(np.uint32)), (variant, wpb, bps)
    with pytest.raises(Exception):
        plan.set_config(8, 2, 0)
    with pytest.raises(Exception):
        plan.set_config(0, 3, 0)
    plan.free()


def test_autotune_keeps_results_and_caches_the_shape(ctx, blobs_knn, oracle):
    idx, dist, _ = blobs_knn
    g = ctx.fuzzy_set(idx, dist, 15.0, True)
    ip, ix, w = g.export()
    plan = ctx.plan(g, 8, seed=5)
    cfg = plan.autotune()
    assert cfg["variant"] in range(8) and cfg["warps_per_block"] in (1, 2, 4)
    assert cfg["ms_per_launch"] > 0
    out = plan.debug_run(None, 0, plan.n_epochs)
    ref = oracle.evoc_embedding(ip, ix, w, 8, seed=5)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
    plan2 = ctx.plan(g, 8, seed=6)  # same shape: configured from the cache
    assert plan2.autotune() == cfg
    plan.free()
    plan2.free()
