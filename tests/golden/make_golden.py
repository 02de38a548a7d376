"""Generate the golden fixtures in tests/golden/ from a pure-Python restatement.

This is a second, independent restatement of the evoc-rs 0.2.7 hot path,
written directly from the Rust source with numpy float32 scalar arithmetic
(one rounding per operation, like Rust without contraction):

    smooth_knn_dist        src/graph/fuzzy_graph.rs:33-98
    knn_to_coo             src/graph/fuzzy_graph.rs:114-159
    symmetrise_graph       src/graph/fuzzy_graph.rs:174-228 (dicts; rows sorted)
    evoc_embedding         src/graph/embedding.rs:48-298

It shares with the C++ oracle and the CUDA library only the documented
arithmetic contract (own exp, Philox4x32-10 negatives and initialisation,
serial squared distance). The fixtures pin the
C++ oracle bit for bit. Run from the repository root:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import math
from pathlib import Path

import numpy as np

F = np.float32
OUT = Path(__file__).resolve().parent
_libm = ctypes.CDLL("libm.so.6")
_libm.powf.argtypes = [ctypes.c_float, ctypes.c_float]
_libm.powf.restype = ctypes.c_float
_libm.sqrtf.argtypes = [ctypes.c_float]
_libm.sqrtf.restype = ctypes.c_float


def powf(a, b) -> np.float32:
    return F(_libm.powf(float(a), float(b)))


# ---- arithmetic contract --------------------------------------------------------
def expf(x) -> np.float32:
    x = F(x)
    if x != x:
        return x
    if x < F(-104.0):
        return F(0.0)
    if x > F(88.72):
        return F(np.inf)
    kf = np.rint(x * F(1.44269502))
    r = x - kf * F(0.693145751953125)
    r = r - kf * F(1.42860677e-06)
    p = F(1.98412701e-04)
    for c in (1.38888892e-03, 8.33333377e-03, 4.16666679e-02, 1.66666672e-01, 0.5, 1.0, 1.0):
        p = p * r + F(c)
    k = int(kf)

    def pow2(e):
        return np.array([(e + 127) << 23], dtype=np.uint32).view(np.float32)[0]

    if k >= -126:
        return p * pow2(k)
    return (p * pow2(k + 64)) * pow2(-64)


M32 = 0xFFFFFFFF


def philox(ctr, key):
    c0, c1, c2, c3 = ctr
    k0, k1 = key
    for _ in range(10):
        p0 = 0xD2511F53 * c0
        p1 = 0xCD9E8D57 * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ k0) & M32, p1 & M32, ((p0 >> 32) ^ c3 ^ k1) & M32, p0 & M32
        k0 = (k0 + 0x9E3779B9) & M32
        k1 = (k1 + 0xBB67AE85) & M32
    return c0, c1, c2, c3


def negative_draw(seed, j, epoch, eidx, n):
    o = philox((j, epoch, eidx & M32, (eidx >> 32) & 0x7FFFFFFF), (seed & M32, seed >> 32))
    return (o[0] * n) >> 32


def init_value(seed, idx):
    o = philox((idx & M32, idx >> 32, 0, 0x80000000 | 0x494E4954), (seed & M32, seed >> 32))
    bits = ((o[1] << 32) | o[0]) >> 11
    u = bits * (1.0 / 9007199254740992.0)
    return F(-0.25 + 0.5 * u)


def to_usize_or0(x) -> int:
    x = F(x)
    return int(x) if (x > F(-1.0) and x < F(18446744073709551616.0)) else 0


def max0(a):
    return a if a > F(0) else F(0)


# ---- fuzzy simplicial set ------------------------------------------------------------
def smooth_knn_dist(rows, k, lc, n_iter=64):
    target = math.log2(k) if k > 0 else -math.inf
    sig, rho_out = [], []
    lc = F(lc)
    for d in rows:
        d = [F(x) for x in d]
        if lc > F(0):
            lm1 = max0(lc - F(1))
            fl = F(math.floor(lm1))
            idx = min(int(fl), len(d) - 1)
            frac = lm1 - fl
            rho = d[idx] * (F(1) - frac) + d[idx + 1] * frac if (frac > F(0) and idx + 1 < len(d)) else d[idx]
        else:
            rho = F(0)
        lo, hi, mid = F(0), F(np.finfo(np.float32).max), F(1)
        for _ in range(n_iter):
            val = F(0)
            for x in d:
                val = val + expf(-(max0(x - rho) / mid))
            vd = float(val)
            if abs(vd - target) < 1e-5:
                break
            if vd > target:
                hi = mid
                mid = (lo + hi) / F(2)
            else:
                lo = mid
                mid = mid * F(2) if hi == F(np.finfo(np.float32).max) else (lo + hi) / F(2)
        sig.append(mid)
        rho_out.append(rho)
    return np.array(sig, np.float32), np.array(rho_out, np.float32)


def knn_to_coo(idx, dist, sig, rho):
    rows, cols, vals = [], [], []
    for i in range(len(idx)):
        for j, dd in zip(idx[i], dist[i]):
            if j == i:
                continue
            a = max0(F(dd) - rho[i])
            w = expf(-(a / sig[i])) if sig[i] > F(0) else (F(0) if a > F(0) else F(1))
            rows.append(i)
            cols.append(int(j))
            vals.append(w)
    return rows, cols, vals


def symmetrise(n, rows, cols, vals):
    fwd = [dict() for _ in range(n)]
    bwd = [dict() for _ in range(n)]
    for i, j, w in zip(rows, cols, vals):
        fwd[i][j] = w
        bwd[j][i] = w
    out = []
    for i in range(n):
        comb = {}
        for j in list(fwd[i].keys()) + list(bwd[i].keys()):
            a = fwd[i].get(j, F(0))
            b = bwd[i].get(j, F(0))
            s = a + b - a * b
            if s > F(0):
                comb[j] = s
        out.append(sorted(comb.items()))
    return out


# ---- node embedding ---------------------------------------------------------------
def evoc_embedding(adj, dim, n_epochs=50, noise=0.5, neg_rate=1.0, alpha=0.1, b1=0.5, b2=0.9,
                   eps=1e-7, init=None, seed=42):
    n = len(adj)
    if init is not None:
        e = [F(x) for x in np.asarray(init, np.float32).ravel()]
    else:
        e = [init_value(seed, q) for q in range(n * dim)]
    edges = [(i, j, F(w)) for i, row in enumerate(adj) for j, w in row if i < j]
    if not edges:
        return np.array(e, np.float32).reshape(n, dim)
    max_w = F(0)
    for _, _, w in edges:
        max_w = max(max_w, w)
    ps = []
    for _, _, w in edges:
        norm = w / max_w
        ps.append(F(1) / norm if norm > F(0) else F(1e8))
    ns = list(ps)
    negf = F(1.5) / F(neg_rate)
    pn = [p * negf for p in ps]
    nn = list(pn)
    inc = [[] for _ in range(n)]
    for ei, (i, j, _) in enumerate(edges):
        inc[i].append((ei, True, j))
        inc[j].append((ei, False, i))
    m = [F(0)] * (n * dim)
    v = [F(0)] * (n * dim)
    om1, om2 = F(1) - F(b1), F(1) - F(b2)
    denom = F(max(n_epochs - 1, 1))
    for ep in range(n_epochs):
        t = F(ep + 1)
        b1t, b2t = powf(F(b1), t), powf(F(b2), t)
        sb2 = F(_libm.sqrtf(float(F(1) - b2t)))
        ads, epsc = sb2 / (F(1) - b1t), sb2 * F(eps)
        gamma = F(0.5) + F(ep) / denom
        lr = F(alpha) * (F(1) - F(ep) / F(n_epochs))
        et = F(ep)
        grads = [None] * n
        for ni in range(n):
            g = [F(0)] * dim
            touched = False
            ei_ = e[ni * dim:(ni + 1) * dim]
            for eid, smaller, o in inc[ni]:
                if ns[eid] > et:
                    continue
                touched = True
                eo = e[o * dim:(o + 1) * dim]
                dsq = F(0)
                for d in range(dim):
                    df = ei_[d] - eo[d]
                    dsq = dsq + df * df
                if dsq >= F(1e-8):
                    dist = np.sqrt(dsq)
                    coeff = (-(F(2) * F(noise) * dist) - F(2)) / (F(2) * dsq - F(0.5) * dist + F(1))
                    for d in range(dim):
                        g[d] = g[d] + coeff * (ei_[d] - eo[d])
                if smaller:
                    nneg = to_usize_or0(np.floor((et - nn[eid]) / pn[eid]))
                    for jj in range(nneg):
                        kk = negative_draw(seed, jj, ep, eid, n)
                        if kk == ni:
                            continue
                        ek = e[kk * dim:(kk + 1) * dim]
                        dk = F(0)
                        for d in range(dim):
                            df = ei_[d] - ek[d]
                            dk = dk + df * df
                        if dk > F(0.01):
                            gc = gamma * F(4) / ((F(1) + F(0.25) * dk) * dk)
                            for d in range(dim):
                                c = gc * (ei_[d] - ek[d])
                                c = min(max(c, F(-4)), F(4))
                                g[d] = g[d] + c
            grads[ni] = g if touched else None
        lr_ad = lr * ads
        for ni in range(n):
            if grads[ni] is None:
                continue
            for d in range(dim):
                q = ni * dim + d
                gd = grads[ni][d]
                m[q] = m[q] + om1 * (gd - m[q])
                v[q] = v[q] + om2 * (gd * gd - v[q])
                e[q] = e[q] + lr_ad * m[q] / (np.sqrt(v[q]) + epsc)
        for eid in range(len(edges)):
            if ns[eid] <= et:
                ns[eid] = ns[eid] + ps[eid]
                cnt = to_usize_or0(np.floor((et - nn[eid]) / pn[eid]))
                nn[eid] = nn[eid] + F(cnt) * pn[eid]
    return np.array(e, np.float32).reshape(n, dim)


def adj_to_csr(adj):
    indptr = np.zeros(len(adj) + 1, np.int64)
    for i, r in enumerate(adj):
        indptr[i + 1] = indptr[i] + len(r)
    idx = np.array([j for r in adj for j, _ in r], np.uint32)
    w = np.array([w for r in adj for _, w in r], np.float32)
    return indptr, idx, w


def main() -> None:
    rng = np.random.default_rng(20261203)
    # smooth_knn_dist: the reference's pinned rows plus random rows
    rows = [[1.0, 2.0], [1.5, 3.0], [0.5, 1.5]]
    r = np.sort(rng.uniform(0.0, 1.5, size=(24, 6)).astype(np.float32), axis=1)
    r[3, :2] = 0.0  # zero distances
    r[5, :] = r[5, 0]  # all equal
    sk = {}
    for lc in (1.0, 0.0, 1.5, 2.3):
        s, rh = smooth_knn_dist(r, 6, lc)
        sk[f"lc{lc}_sigma"], sk[f"lc{lc}_rho"] = s, rh
    s, rh = smooth_knn_dist(r, 4, 1.0)  # k_target != row length
    sk["k4_sigma"], sk["k4_rho"] = s, rh
    s0, rh0 = smooth_knn_dist(rows, 2, 1.0)
    np.savez(OUT / "smooth_knn.npz", dists=r, pin_rows=np.array(rows, np.float32),
             pin_sigma=s0, pin_rho=rh0, **sk)

    # fuzzy set with duplicates and self loops
    n, k = 40, 5
    idx = rng.integers(0, n, size=(n, k)).astype(np.uint32)
    idx[:, 0] = np.arange(n)  # self loop first, like an unfiltered kNN
    idx[7, 3] = idx[7, 2]     # duplicate column: last wins
    dist = np.sort(rng.uniform(0.05, 1.0, size=(n, k)).astype(np.float32), axis=1)
    dist[:, 0] = 0.0
    sig, rho = smooth_knn_dist(dist, k, 1.0)
    rr, cc, vv = knn_to_coo(idx, dist, sig, rho)
    sym = symmetrise(n, rr, cc, vv)
    ip, ix, w = adj_to_csr(sym)
    dip = np.zeros(n + 1, np.int64)
    for i in rr:
        dip[i + 1] += 1
    dip = np.cumsum(dip)
    np.savez(OUT / "fuzzy_set.npz", knn_idx=idx, knn_dist=dist, sigma=sig, rho=rho,
             directed_indptr=dip, directed_indices=np.array(cc, np.uint32),
             directed_weights=np.array(vv, np.float32), indptr=ip, indices=ix, weights=w)

    # embeddings: the reference's reproducibility graph, a triangle, two clusters
    g08 = [[(1, 1.0), (2, 0.5)], [(0, 1.0), (2, 0.8)], [(0, 0.5), (1, 0.8), (3, 0.9)], [(2, 0.9)]]
    tri = [[(1, 1.0), (2, 1.0)], [(0, 1.0), (2, 1.0)], [(0, 1.0), (1, 1.0)]]
    emb = {}
    e08 = evoc_embedding(g08, 4, n_epochs=30, seed=123)
    emb["g08_indptr"], emb["g08_indices"], emb["g08_weights"] = adj_to_csr(g08)
    emb["g08_out"] = e08
    etri = evoc_embedding(tri, 8, n_epochs=50, seed=42)
    emb["tri_indptr"], emb["tri_indices"], emb["tri_weights"] = adj_to_csr(tri)
    emb["tri_out"] = etri
    # two clusters of 12 from the fuzzy set of a small kNN graph, with init
    pts = np.concatenate([rng.normal(0, 0.3, (12, 3)), rng.normal(5, 0.3, (12, 3))]).astype(np.float32)
    d2 = ((pts[:, None, :] - pts[None, :, :]) ** 2).sum(-1)
    kk = 5
    order = np.argsort(d2, axis=1, kind="stable")[:, 1:kk + 1]
    kd = np.sqrt(np.take_along_axis(d2, order, 1)).astype(np.float32)
    s2, r2 = smooth_knn_dist(kd, kk, 1.0)
    rr, cc, vv = knn_to_coo(order, kd, s2, r2)
    adj2 = symmetrise(24, rr, cc, vv)
    init2 = rng.uniform(-1, 1, (24, 2)).astype(np.float32)
    e2 = evoc_embedding(adj2, 2, n_epochs=40, seed=7, init=init2, neg_rate=2.0)
    emb["cl_indptr"], emb["cl_indices"], emb["cl_weights"] = adj_to_csr(adj2)
    emb["cl_init"], emb["cl_out"] = init2, e2
    np.savez(OUT / "embedding.npz", **emb)
    print("wrote", sorted(p.name for p in OUT.glob("*.npz")))


if __name__ == "__main__":
    main()
