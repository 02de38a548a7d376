"""CPU checks of the warm-start oracle and of the library's host-side Procrustes.

The oracle's gradient formulas are pinned by central finite differences of
its own exact (unrounded) loss; its BF16 rounding by known values and by
torch's float32 -> bfloat16 conversion. evoc_procrustes runs on the host, so
it is checked here against numpy's SVD without a GPU.
"""
import numpy as np
import pytest

import mlp_oracle as M


def test_bf16_rounding_known_values():
    one = 1.0
    ulp = 2.0 ** -7
    x = np.array([one, one + ulp / 2, one + 1.5 * ulp, -one - ulp / 2, 3.0e38, 1e-40],
                 dtype=np.float32)
    got = M.bf16(x)
    # ties go to the even mantissa
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == 1.0 + 2 * ulp and got[3] == -1.0
    assert np.isfinite(got[4]) and got[5] > 0


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    x = np.random.default_rng(3).standard_normal(100_000).astype(np.float32) * 37.0
    want = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    np.testing.assert_array_equal(M.bf16(x).astype(np.float32), want)


def _tiny(seed=0, in_dim=8, hidden=8, out_dim=3, n=5):
    rng = np.random.default_rng(seed)
    p = M.unpack(rng.standard_normal(M.n_params(in_dim, hidden, out_dim)) * 0.5,
                 in_dim, hidden, out_dim)
    x = rng.standard_normal((n, in_dim))
    t = rng.standard_normal((n, out_dim))
    return p, x, t


def test_gradients_match_finite_differences():
    p, x, t = _tiny()
    _, g = M.loss_and_gradients(p, x, t, exact=True)
    flat = M.pack(p)
    gflat = M.pack(g)
    h = 1e-6
    for i in range(0, flat.size, 3):
        up, dn = flat.copy(), flat.copy()
        up[i] += h
        dn[i] -= h
        num = (M.loss_only(M.unpack(up, 8, 8, 3), x, t) -
               M.loss_only(M.unpack(dn, 8, 8, 3), x, t)) / (2 * h)
        assert abs(num - gflat[i]) <= 1e-6 * max(1.0, abs(num)), (i, num, gflat[i])


def test_gelu_derivative():
    x = np.linspace(-6, 6, 241)
    h = 1e-6
    num = (M.gelu(x + h) - M.gelu(x - h)) / (2 * h)
    np.testing.assert_allclose(M.gelu_grad(x), num, atol=1e-8)


def test_adam_matches_definition():
    p, m, v, g = np.array([1.0]), np.array([0.0]), np.array([0.0]), np.array([0.5])
    p1, m1, v1 = M.adam(p, m, v, g, 1, 0.1, 0.9, 0.999, 1e-8)
    # first step: m_hat = g, v_hat = g^2, so the step is lr * sign(g)
    assert m1[0] == pytest.approx(0.05) and v1[0] == pytest.approx(0.00025)
    assert p1[0] == pytest.approx(1.0 - 0.1, abs=1e-7)


def test_align_recovers_rotation_and_shift():
    rng = np.random.default_rng(5)
    pred = rng.standard_normal((500, 8))
    q, _ = np.linalg.qr(rng.standard_normal((8, 8)))
    layout = (pred - pred.mean(0)) @ q.T + 3.0  # a rotated, shifted copy
    np.testing.assert_allclose(M.align(layout, pred), pred, atol=1e-10)


@pytest.mark.parametrize("d", [1, 2, 8, 16])
def test_library_procrustes_matches_svd(d):
    import evoc_gb300 as E
    rng = np.random.default_rng(d)
    for _ in range(5):
        m = rng.standard_normal((d, d))
        r = E.procrustes(m)
        np.testing.assert_allclose(r @ r.T, np.eye(d), atol=1e-12)
        np.testing.assert_allclose(r, M.procrustes(m), atol=1e-9)


def test_library_procrustes_rank_deficient():
    import evoc_gb300 as E
    rng = np.random.default_rng(9)
    a = rng.standard_normal((8, 3))
    m = a @ rng.standard_normal((3, 8))  # rank 3
    r = E.procrustes(m)
    np.testing.assert_allclose(r @ r.T, np.eye(8), atol=1e-10)
    # still the maximiser of trace(R^T M): equals the sum of singular values
    assert np.trace(r.T @ m) == pytest.approx(np.linalg.svd(m, compute_uv=False).sum(), rel=1e-10)
    z = E.procrustes(np.zeros((4, 4)))
    np.testing.assert_allclose(z @ z.T, np.eye(4), atol=1e-12)


def test_library_procrustes_rejects_bad_size():
    import evoc_gb300 as E
    with pytest.raises(E.EvocError):
        E.procrustes(np.zeros((17, 17)))
