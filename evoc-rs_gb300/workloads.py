"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is used. Points are f32, L2-normalised; the kNN graph uses
cosine distance 1 - <x, y> with the point itself removed, like
run_ann_search's query of k+1 neighbours (nearest_neighbour_cpu.rs:352-361).
Brute-force kNN stands in for ann-search-rs (not available here): exact in
the numpy functions, bf16-screened (approximate, recall measured) on the GPU.

    blobs_sphere      10,000 x 384, 20 isotropic Gaussians, sigma 0.15 per
                      coordinate, centres uniform on the sphere (k = 15, dim 4)
    anisotropic       200,000 x 512, 100 clusters with covariance eigenvalues
                      log-uniform in [0.01, 0.3] on random orthonormal bases,
                      Zipf(1.1) sizes, 10% uniform noise (k = 15, dim 8)
    hierarchical      2,000,000 x 768, 50 parents x 10 children at 0.2 rad,
                      Zipf(1.0) sizes, 5% noise (k = 30, dim 8)
    batch_problems    256 problems, n log-uniform in [2,000, 150,000], 384-d,
                      5-60 clusters each (k = 15, dim 4)

The numpy functions run anywhere (tests); the torch functions run on a GPU
(benchmark) and use tensor-core matmuls only to build the input graph.
"""
from __future__ import annotations

import numpy as np


# ---------------------------------------------------------------------------
# CPU (numpy) generators for tests
# ---------------------------------------------------------------------------
def _unit(x: np.ndarray) -> np.ndarray:
    return x / np.linalg.norm(x, axis=1, keepdims=True)


def blobs_sphere_np(n: int, d: int, n_clusters: int, sigma: float, seed: int):
    """Isotropic Gaussian clusters around centres uniform on the unit sphere."""
    rng = np.random.default_rng(seed)
    centres = _unit(rng.standard_normal((n_clusters, d)))
    labels = rng.integers(0, n_clusters, size=n)
    x = centres[labels] + sigma * rng.standard_normal((n, d))
    return _unit(x).astype(np.float32), labels


def knn_np(x: np.ndarray, k: int, chunk: int = 2048):
    """Exact cosine kNN (1 - <x, y>), self removed; ties broken by index."""
    n = x.shape[0]
    idx = np.zeros((n, k), dtype=np.uint32)
    dist = np.zeros((n, k), dtype=np.float32)
    xt = x.T.astype(np.float32)
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        sim = x[a:b] @ xt
        sim[np.arange(b - a), np.arange(a, b)] = -np.inf
        part = np.argpartition(-sim, k, axis=1)[:, :k]
        ps = np.take_along_axis(sim, part, 1)
        o = np.argsort(-ps, axis=1, kind="stable")
        part = np.take_along_axis(part, o, 1)
        ps = np.take_along_axis(ps, o, 1)
        idx[a:b] = part
        dist[a:b] = np.maximum(1.0 - ps, 0.0)
    return idx, dist


# ---------------------------------------------------------------------------
# GPU (torch) generators for the benchmark
# ---------------------------------------------------------------------------
def _torch():
    import torch
    return torch


def _zipf_sizes(n: int, n_clusters: int, s: float, rng: np.random.Generator) -> np.ndarray:
    w = 1.0 / np.arange(1, n_clusters + 1) ** s
    w = w / w.sum()
    sizes = np.floor(w * n).astype(np.int64)
    sizes[: n - sizes.sum()] += 1
    return rng.permutation(sizes)


def blobs_sphere_torch(n: int, d: int, n_clusters: int, sigma: float, seed: int, device="cuda"):
    torch = _torch()
    g = torch.Generator(device=device).manual_seed(seed)
    centres = torch.randn(n_clusters, d, generator=g, device=device)
    centres = centres / centres.norm(dim=1, keepdim=True)
    labels = torch.randint(0, n_clusters, (n,), generator=g, device=device)
    x = centres[labels] + sigma * torch.randn(n, d, generator=g, device=device)
    return x / x.norm(dim=1, keepdim=True), labels


def anisotropic_torch(n: int, d: int, n_clusters: int, seed: int, noise_frac: float = 0.10,
                      zipf: float = 1.1, device="cuda"):
    torch = _torch()
    rng = np.random.default_rng(seed)
    g = torch.Generator(device=device).manual_seed(seed)
    n_noise = int(round(noise_frac * n))
    sizes = _zipf_sizes(n - n_noise, n_clusters, zipf, rng)
    centres = torch.randn(n_clusters, d, generator=g, device=device)
    centres = centres / centres.norm(dim=1, keepdim=True)
    parts, labels = [], []
    for c in range(n_clusters):
        m = int(sizes[c])
        if m == 0:
            continue
        q, _ = torch.linalg.qr(torch.randn(d, d, generator=g, device=device))
        ev = torch.from_numpy(np.exp(rng.uniform(np.log(0.01), np.log(0.3), d))).float().to(device)
        z = torch.randn(m, d, generator=g, device=device) * ev.sqrt()
        parts.append(centres[c] + z @ q.T)
        labels.append(torch.full((m,), c, device=device))
    noise = torch.randn(n_noise, d, generator=g, device=device)
    parts.append(noise)
    labels.append(torch.full((n_noise,), -1, device=device))
    x = torch.cat(parts)
    lab = torch.cat(labels)
    perm = torch.randperm(n, generator=g, device=device)
    x = x[perm]
    x = x / x.norm(dim=1, keepdim=True)
    return x, lab[perm]


def hierarchical_torch(n: int, d: int, n_parents: int, n_children: int, seed: int,
                       angle: float = 0.2, spread: float = 0.015, noise_frac: float = 0.05,
                       zipf: float = 1.0, device="cuda"):
    """Children at angle `angle` from their parent; isotropic spread per
    coordinate. Returns (points, child label, parent label); noise is -1."""
    torch = _torch()
    rng = np.random.default_rng(seed)
    g = torch.Generator(device=device).manual_seed(seed)
    nc = n_parents * n_children
    n_noise = int(round(noise_frac * n))
    sizes = _zipf_sizes(n - n_noise, nc, zipf, rng)
    parents = torch.randn(n_parents, d, generator=g, device=device)
    parents = parents / parents.norm(dim=1, keepdim=True)
    # child = cos(a) p + sin(a) u with u a random unit vector orthogonal to p
    u = torch.randn(n_parents, n_children, d, generator=g, device=device)
    u = u - (u * parents[:, None, :]).sum(-1, keepdim=True) * parents[:, None, :]
    u = u / u.norm(dim=-1, keepdim=True)
    children = (np.cos(angle) * parents[:, None, :] + np.sin(angle) * u).reshape(nc, d)
    lab = torch.repeat_interleave(torch.arange(nc, device=device),
                                  torch.from_numpy(sizes).to(device))
    x = children[lab] + spread * torch.randn(lab.numel(), d, generator=g, device=device)
    noise = torch.randn(n_noise, d, generator=g, device=device)
    x = torch.cat([x, noise])
    lab = torch.cat([lab, torch.full((n_noise,), -1, device=device)])
    perm = torch.randperm(n, generator=g, device=device)
    x = x[perm]
    x = x / x.norm(dim=1, keepdim=True)
    lab = lab[perm]
    parent = torch.where(lab >= 0, lab // n_children, lab)
    return x, lab, parent


def knn_torch(x, k: int, groups=None, max_sim_elems: int = 1 << 31):
    """Cosine kNN on the GPU: a bf16 matmul screens 4 k candidates per
    query, which are re-ranked with f32 distances (ties by index). Returns
    (idx int64, dist float32), each n x k, the query itself removed.

    `groups` is a list of (query_idx, key_idx) index tensors: each group's
    queries are searched among its keys only (None: every point against every
    point). The 2M-point workload searches each parent cluster within itself
    and the noise points against all points; its parents are nearly orthogonal
    on the sphere. The bf16 screen can miss a true neighbour near the k-th
    distance, so the result is an approximate kNN, like the reference's own
    ANN search; tests/test_gpu_workloads.py measures its recall against
    exhaustive f32 search on a sample of queries at 200,000 points."""
    torch = _torch()
    n = x.shape[0]
    dev = x.device
    out_i = torch.full((n, k), -1, dtype=torch.int64, device=dev)
    out_d = torch.zeros(n, k, dtype=torch.float32, device=dev)
    if groups is None:
        a = torch.arange(n, device=dev)
        groups = [(a, a)]
    xb_all = x.to(torch.bfloat16)
    for q_idx, key_idx in groups:
        m = key_idx.numel()
        if q_idx.numel() == 0 or m == 0:
            continue
        kb = xb_all[key_idx]
        kk = min(4 * k, m)  # bf16 screen: a wide pool, so the f32 re-rank sees the true top k
        chunk = int(max(128, min(8192, max_sim_elems // max(m, 1), (1 << 30) // (kk * x.shape[1]))))
        for a in range(0, q_idx.numel(), chunk):
            qi = q_idx[a:a + chunk]
            sim = xb_all[qi] @ kb.T
            cand = torch.topk(sim, kk, dim=1).indices          # local key positions
            del sim
            gk = key_idx[cand]                                  # global key ids
            exact = (x[qi][:, None, :] * x[gk]).sum(-1)
            exact = torch.where(gk == qi[:, None], torch.full_like(exact, -4.0), exact)
            order = torch.argsort(gk, dim=1)                    # ties broken by index
            gk = torch.gather(gk, 1, order)
            exact = torch.gather(exact, 1, order)
            top = torch.sort(exact, dim=1, descending=True, stable=True)
            sel = top.indices[:, :k]
            out_i[qi] = torch.gather(gk, 1, sel)
            out_d[qi] = (1.0 - top.values[:, :k]).clamp_min(0.0)
    return out_i, out_d


def hierarchical_groups(parent):
    """(query, key) groups for knn_torch: one per parent cluster, plus the
    noise points (parent -1) against all points."""
    torch = _torch()
    dev = parent.device
    allidx = torch.arange(parent.numel(), device=dev)
    order = torch.argsort(parent, stable=True)
    ps = parent[order]
    uniq, counts = torch.unique_consecutive(ps, return_counts=True)
    groups = []
    start = 0
    for u, c in zip(uniq.tolist(), counts.tolist()):
        idx = order[start:start + c]
        start += c
        groups.append((idx, allidx) if u < 0 else (idx, idx))
    return groups
