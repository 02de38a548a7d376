"""GPU checks of the learned warm start, through the C ABI.

Bar: the network's forward pass and every parameter gradient agree with the
CPU oracle (`oracle/mlp_oracle.py`, which rounds to BF16 at the same places
as the kernels) within BF16 accumulation tolerance:
  * relative Frobenius error <= 1e-2 per tensor,
  * elementwise |gpu - oracle| <= 2e-2 * max |oracle| per tensor,
  * loss within 1e-3 relative.
Training is reproducible bit for bit, lowers the loss, recovers a rotated
copy of its own prediction exactly, and the trained initialisation beats the
random one at the same reduced epoch count.
"""
import numpy as np
import pytest

import mlp_oracle as M

pytestmark = pytest.mark.gpu

DIMS = [(768, 512, 8, 300), (40, 24, 5, 77), (64, 136, 16, 129)]


def _net(ctx, i, h, o, seed=1):
    return ctx.mlp(i, h, o, seed=seed)


def _data(i, o, n, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, i)).astype(np.float32)
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    t = rng.standard_normal((n, o)).astype(np.float32)
    return x, t


def _close(got, want, what):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    scale = np.abs(want).max()
    rel = np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-30)
    assert rel <= 1e-2, f"{what}: relative error {rel:.3g}"
    assert np.abs(got - want).max() <= 2e-2 * scale + 1e-30, f"{what}: max abs error"


def test_params_roundtrip_and_init(ctx):
    net = _net(ctx, 768, 512, 8)
    p = net.get_params()
    assert p.size == M.n_params(768, 512, 8) == net.n_params
    d = net.unpack(p)
    assert np.abs(d["w1"]).max() <= 1 / np.sqrt(768) and np.abs(d["w2"]).max() <= 1 / np.sqrt(512)
    q = np.random.default_rng(2).standard_normal(p.size).astype(np.float32) * 0.05
    net.set_params(q)
    np.testing.assert_array_equal(net.get_params(), q)
    # the same seed gives the same initialisation
    np.testing.assert_array_equal(_net(ctx, 768, 512, 8, seed=1).get_params(), p)


@pytest.mark.parametrize("i,h,o,n", DIMS)
def test_forward_matches_oracle(ctx, i, h, o, n):
    net = _net(ctx, i, h, o)
    x, _ = _data(i, o, n)
    y = net.predict(x)
    want = M.forward(M.unpack(net.get_params(), i, h, o), x)["y"]
    _close(y, want, "prediction")


@pytest.mark.parametrize("i,h,o,n", DIMS)
def test_gradients_match_oracle(ctx, i, h, o, n):
    net = _net(ctx, i, h, o)
    x, t = _data(i, o, n, seed=4)
    loss, grad = net.gradients(x, t)
    want_loss, want = M.loss_and_gradients(M.unpack(net.get_params(), i, h, o), x, t)
    assert loss == pytest.approx(want_loss, rel=1e-3)
    got = net.unpack(grad)
    for name in ("w1", "b1", "w2", "b2", "w3", "b3"):
        _close(got[name], want[name], name)


@pytest.mark.parametrize("path", ["persist", "tma", "cpasync"])
@pytest.mark.parametrize("stages", ["2", "4"])
@pytest.mark.parametrize("i,h,o,n", DIMS + [(128, 512, 8, 1000)])
def test_tcgen05_forward_matches_mma_sync(ctx, i, h, o, n, stages, path, monkeypatch):
    """The tcgen05 forward layers (the persistent warp-specialised kernel by
    default, the one-tile-per-CTA TMA kernel, or the cp.async-fed one; the
    second layer fused with the output layer) and the mma.sync kernels give
    the same prediction up to FP32 accumulation order, and both match the
    oracle, for either ring depth of the non-persistent kernels."""
    net = _net(ctx, i, h, o)
    x, _ = _data(i, o, n, seed=8)
    monkeypatch.setenv("EVOC_TC_STAGES", stages)
    if path != "persist":
        monkeypatch.setenv("EVOC_MLP_GEMM", path)
    y_tc = net.predict(x)
    monkeypatch.setenv("EVOC_MLP_GEMM", "mma")
    y_mma = net.predict(x)
    monkeypatch.delenv("EVOC_MLP_GEMM")
    want = M.forward(M.unpack(net.get_params(), i, h, o), x)["y"]
    _close(y_tc, want, "tcgen05 prediction")
    _close(y_mma, want, "mma.sync prediction")
    rel = np.linalg.norm(y_tc - y_mma) / np.linalg.norm(y_mma)
    assert rel <= 2e-3, rel


@pytest.mark.parametrize("i,h,o,n", DIMS + [(768, 512, 8, 8192)])
def test_tcgen05_gradients_match_mma_sync(ctx, i, h, o, n, monkeypatch):
    """The tcgen05 backward (default: GELU' epilogue on a W2^T operand,
    split-K weight gradients over transposed copies) and the mma.sync backward
    give the same gradients up to accumulation order; both match the oracle."""
    net = _net(ctx, i, h, o)
    x, t = _data(i, o, n, seed=12)
    l_tc, g_tc = net.gradients(x, t)
    monkeypatch.setenv("EVOC_MLP_GEMM", "mma")
    l_mma, g_mma = net.gradients(x, t)
    monkeypatch.delenv("EVOC_MLP_GEMM")
    want_loss, want = M.loss_and_gradients(M.unpack(net.get_params(), i, h, o), x, t)
    assert l_tc == pytest.approx(want_loss, rel=1e-3) and l_mma == pytest.approx(want_loss, rel=1e-3)
    a, b = net.unpack(g_tc), net.unpack(g_mma)
    for name in ("w1", "b1", "w2", "b2", "w3", "b3"):
        _close(a[name], want[name], "tcgen05 " + name)
        _close(b[name], want[name], "mma.sync " + name)


def test_tcgen05_prediction_over_chunks(ctx):
    """Rows beyond the 262,144-row prediction chunk and a ragged last tile."""
    net = _net(ctx, 64, 256, 8)
    x, _ = _data(64, 8, 262_144 + 1_001, seed=9)
    y = net.predict(x)
    for sl in (slice(0, 300), slice(262_000, 262_400), slice(-77, None)):
        want = M.forward(M.unpack(net.get_params(), 64, 256, 8), x[sl])["y"]
        _close(y[sl], want, f"rows {sl}")


def test_gradients_are_reproducible(ctx):
    net = _net(ctx, 768, 512, 8)
    x, t = _data(768, 8, 1000, seed=6)
    l1, g1 = net.gradients(x, t)
    l2, g2 = net.gradients(x, t)
    assert l1 == l2
    np.testing.assert_array_equal(g1, g2)


def test_predict_device_equals_host(ctx):
    import torch
    net = _net(ctx, 768, 512, 8)
    x, _ = _data(768, 8, 70_001, seed=7)  # a ragged last row tile
    want = net.predict(x)
    xd = torch.from_numpy(x).cuda()
    xb = torch.empty(xd.shape, dtype=torch.bfloat16, device="cuda")
    torch.cuda.synchronize()
    ctx.to_bf16_device(xd.data_ptr(), xd.numel(), xb.data_ptr())
    np.testing.assert_array_equal(xb.float().cpu().numpy(), M.bf16(x).astype(np.float32))
    out = torch.empty(x.shape[0], 8, dtype=torch.float32, device="cuda")
    net.predict_device(xb.data_ptr(), x.shape[0], out.data_ptr())
    np.testing.assert_array_equal(out.cpu().numpy(), want)


def _instances(ctx, m, n, i, o, seed):
    """Points and 'layouts' that are a fixed smooth function of the points,
    rotated and shifted differently per instance."""
    import torch
    rng = np.random.default_rng(seed)
    proj = rng.standard_normal((i, o)) / np.sqrt(i) * 4.0
    out = []
    for s in range(m):
        x, _ = _data(i, o, n, seed=seed + 10 + s)
        q, _ = np.linalg.qr(rng.standard_normal((o, o)))
        lay = (np.tanh(x @ proj) * 3.0) @ q + rng.standard_normal(o)
        xb = torch.empty(n, i, dtype=torch.bfloat16, device="cuda")
        xd = torch.from_numpy(x).cuda()
        torch.cuda.synchronize()
        ctx.to_bf16_device(xd.data_ptr(), xd.numel(), xb.data_ptr())
        out.append({"xb": xb, "layout": torch.from_numpy(lay.astype(np.float32)).cuda(),
                    "n": n, "x": x})
    torch.cuda.synchronize()
    return out


def _fit(net, inst, **kw):
    import evoc_gb300 as E
    p = E.MlpTrainParams(**kw)
    return net.fit_device([d["xb"].data_ptr() for d in inst], [d["layout"].data_ptr() for d in inst],
                          [d["n"] for d in inst], p)


def test_fit_recovers_rotated_prediction(ctx):
    """A layout that is a rotated, shifted copy of the network's own
    prediction aligns back onto it: the first step's loss is ~0."""
    import torch
    net = _net(ctx, 64, 64, 8, seed=3)
    x, _ = _data(64, 8, 5000, seed=11)
    pred = net.predict(x).astype(np.float64)
    q, _ = np.linalg.qr(np.random.default_rng(1).standard_normal((8, 8)))
    lay = ((pred - pred.mean(0)) @ q.T + 5.0).astype(np.float32)
    xb = torch.empty(5000, 64, dtype=torch.bfloat16, device="cuda")
    xd = torch.from_numpy(x).cuda()
    torch.cuda.synchronize()
    ctx.to_bf16_device(xd.data_ptr(), xd.numel(), xb.data_ptr())
    inst = [{"xb": xb, "layout": torch.from_numpy(lay).cuda(), "n": 5000}]
    torch.cuda.synchronize()
    hist = _fit(net, inst, steps=1, batch=1024, align_every=1, align_rows=5000, lr=0.0)
    assert hist[0] <= 1e-8 * float(np.mean(pred ** 2)) + 1e-10


def test_fit_lowers_loss_and_is_reproducible(ctx):
    inst = _instances(ctx, 3, 4096, 64, 4, seed=20)
    kw = dict(steps=400, batch=512, align_every=50, align_rows=2048, lr=3e-3, seed=5)
    a = _net(ctx, 64, 128, 4, seed=9)
    ha = _fit(a, inst, **kw)
    b = _net(ctx, 64, 128, 4, seed=9)
    hb = _fit(b, inst, **kw)
    np.testing.assert_array_equal(ha, hb)
    np.testing.assert_array_equal(a.get_params(), b.get_params())
    assert np.all(np.isfinite(ha))
    assert ha[-40:].mean() < 0.5 * ha[:40].mean()


def test_rejects_bad_shapes(ctx):
    import evoc_gb300 as E
    with pytest.raises(E.EvocError):
        ctx.mlp(30, 64, 8)     # in_dim not a multiple of 8
    with pytest.raises(E.EvocError):
        ctx.mlp(64, 60, 8)     # hidden not a multiple of 8
    with pytest.raises(E.EvocError):
        ctx.mlp(64, 64, 17)    # out_dim above 16
    net = _net(ctx, 64, 64, 8)
    with pytest.raises(E.EvocError):
        net.gradients(np.zeros((0, 64), np.float32), np.zeros((0, 8), np.float32))


def test_warm_start_beats_random_init_at_reduced_epochs(ctx):
    """The trained network's initialisation, run for 10 epochs, preserves
    neighbourhoods better than the random initialisation run for 10 epochs."""
    import evoc_gb300 as E
    import warm_start as WS
    gen = dict(n_parents=10, n_children=5)
    train = [WS.training_instance(ctx, 20_000, 768, 15, 8, seed=100 + s, init="random", **gen)
             for s in range(3)]
    net, hist, _ = WS.train(ctx, train, 512, 8,
                            E.MlpTrainParams(steps=600, batch=4096, align_every=100,
                                             align_rows=20_000, seed=1))
    assert hist[-50:].mean() < hist[:50].mean()
    ev = WS.make_instance(ctx, 20_000, 768, 15, seed=777, keep_points=True, **gen)
    g = WS.fuzzy_graph(ctx, ev)
    init = WS.predict(net, ev)
    warm = WS.embed_device(ctx, g, ev["n"], 8, 10, 777, init=init)
    rand = WS.embed_device(ctx, g, ev["n"], 8, 10, 777)
    qw = WS.quality(ev["x"], warm, ev["labels"], n_queries=1024)
    qr = WS.quality(ev["x"], rand, ev["labels"], n_queries=1024)
    print("warm", qw, "random", qr)
    assert qw["trustworthiness"] > qr["trustworthiness"]
    # final labels (the reference's clustering stage, restated in the oracle)
    # against those of the plain method (random init, 50 epochs)
    import oracle as O
    plain = WS.embed_device(ctx, g, ev["n"], 8, 50, 777)
    lab = lambda e: O.best_labels(O.build_cluster_layers(e.cpu().numpy(), 5, 5, 0.2, 10))
    lp = lab(plain)
    ari_w, ari_r = O.adjusted_rand_index(lab(warm), lp), O.adjusted_rand_index(lab(rand), lp)
    print("labels ARI vs the plain method: warm start", ari_w, "random init", ari_r)
    assert ari_w > ari_r


def test_bounded_wait_times_out_and_the_context_survives(ctx):
    """A wait that nothing satisfies gives up after its limit, the call
    returns the timeout status, and the same context keeps working."""
    import time
    import evoc_gb300 as E
    t = time.perf_counter()
    rc = ctx.lib.evoc_selftest_wait_timeout(ctx.handle, 50)
    dt = time.perf_counter() - t
    assert rc == E.EVOC_ERR_INTERNAL
    assert "timed out" in ctx.lib.evoc_last_error(ctx.handle).decode()
    assert 0.04 < dt < 5.0
    net = _net(ctx, 64, 64, 8)
    x, _ = _data(64, 8, 300, seed=13)
    _close(net.predict(x), M.forward(M.unpack(net.get_params(), 64, 64, 8), x)["y"], "after timeout")
