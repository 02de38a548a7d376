"""The learned warm start end to end: training layouts from the plain method,
training the MLP on the GPU, and judging its initialisation.

Points come from the seeded hierarchical generator (`workloads.py`); each
instance's cosine kNN graph is built on the GPU, turned into a fuzzy
simplicial set and embedded by the plain method to give the layouts the
network learns from. The plain method is evoc()'s own pipeline: the
label-propagation initialisation with the points feeding its PCA base case
(lib.rs:281), then 50 epochs; random initialisation with 50 epochs is the
fallback form. A fresh instance is then embedded by the plain method and
warm (network prediction as the initial embedding, fewer epochs).

Quality is measured on the embedding against the input points:
  * trustworthiness@k (Venna & Kaski, 2001), estimated over a seeded sample
    of query points with exact ranks in the input space;
  * kNN label accuracy: how often the majority generator label among a
    query's k embedding neighbours equals its own (noise points excluded).

torch supplies device memory and the evaluation arithmetic; the network, the
fuzzy set and the embedding run in the library's kernels.
"""
from __future__ import annotations

import time

import numpy as np


def _torch():
    import torch
    return torch


def make_instance(ctx, n: int, d: int, k: int, seed: int, n_parents: int = 50,
                  n_children: int = 10, keep_points: bool = False) -> dict:
    """Points (BF16 copy on the device), labels and the device kNN graph."""
    torch = _torch()
    import workloads as W
    x, lab, parent = W.hierarchical_torch(n, d, n_parents, n_children, seed)
    groups = W.hierarchical_groups(parent)
    idx, dist = W.knn_torch(x, k, groups)
    idx32 = idx.to(torch.int32).contiguous()
    del idx, groups
    xb = torch.empty(n, d, dtype=torch.bfloat16, device=x.device)
    torch.cuda.synchronize()
    ctx.to_bf16_device(x.data_ptr(), n * d, xb.data_ptr())
    inst = {"n": n, "d": d, "k": k, "seed": seed, "xb": xb, "labels": lab, "idx": idx32,
            "dist": dist.contiguous()}
    if keep_points:
        inst["x"] = x
    else:
        del x
    return inst


def fuzzy_graph(ctx, inst: dict):
    return ctx.fuzzy_set_device(inst["idx"].data_ptr(), inst["dist"].data_ptr(), inst["n"],
                                inst["k"], float(inst["k"]), True)


def embed_device(ctx, graph, n: int, dim: int, n_epochs: int, seed: int, init=None,
                 initial_alpha: float = 0.1):
    """evoc_embedding on a device graph; init (n x dim f32 device tensor) or random."""
    torch = _torch()
    import evoc_gb300 as E
    params = E.EvocEmbeddingParams(n_epochs=n_epochs, initial_alpha=initial_alpha)
    plan = ctx.plan(graph, dim, params, seed=seed)
    out = torch.empty(n, dim, dtype=torch.float32, device="cuda")
    plan.run_device(None if init is None else init.data_ptr(), out.data_ptr())
    plan.free()
    return out


def lp_init(ctx, graph, inst: dict, dim: int, seed: int):
    """label_propagation_init (label_prop.rs:537-564) of the instance's graph,
    its f32 points feeding the PCA base case, as evoc() runs it (lib.rs:281)."""
    torch = _torch()
    out = torch.empty(inst["n"], dim, dtype=torch.float32, device="cuda")
    ctx.label_propagation_init_device(graph, dim, inst["x"].data_ptr(), inst["d"], seed,
                                      out.data_ptr())
    return out


def training_instance(ctx, n: int, d: int, k: int, dim: int, seed: int, n_epochs: int = 50,
                      init: str = "lp", **gen) -> dict:
    """Points and the plain method's layout of one training instance (device):
    init "lp" (label-propagation initialisation, evoc()'s own) or "random"."""
    inst = make_instance(ctx, n, d, k, seed, keep_points=(init == "lp"), **gen)
    g = fuzzy_graph(ctx, inst)
    start = lp_init(ctx, g, inst, dim, seed) if init == "lp" else None
    inst["layout"] = embed_device(ctx, g, n, dim, n_epochs, seed, init=start)
    g.free()
    for key in ("idx", "dist", "labels", "x"):
        inst.pop(key, None)
    return inst


def train(ctx, instances: list[dict], hidden: int, dim: int, params, seed: int = 0):
    """Create and fit the network on device-resident instances; returns
    (network, per-step loss, device seconds)."""
    torch = _torch()
    d = instances[0]["d"]
    net = ctx.mlp(d, hidden, dim, seed=seed)
    torch.cuda.synchronize()
    t = time.perf_counter()
    hist = net.fit_device([i["xb"].data_ptr() for i in instances],
                          [i["layout"].data_ptr() for i in instances],
                          [i["n"] for i in instances], params)
    torch.cuda.synchronize()
    return net, hist, time.perf_counter() - t


def predict(net, inst: dict):
    torch = _torch()
    out = torch.empty(inst["n"], net.out_dim, dtype=torch.float32, device="cuda")
    net.predict_device(inst["xb"].data_ptr(), inst["n"], out.data_ptr())
    return out


def quality(x, emb, labels, k: int = 15, n_queries: int = 2048, seed: int = 0,
            chunk: int = 256) -> dict:
    """Sampled trustworthiness@k and kNN label accuracy of emb (n x dim) for
    unit-norm points x (n x D); both torch tensors on the same device."""
    torch = _torch()
    n = x.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    q = torch.randperm(n, generator=g)[:min(n_queries, n)].to(x.device)
    penalty, correct, counted = 0.0, 0, 0
    emb = emb.float()
    for a in range(0, q.numel(), chunk):
        qi = q[a:a + chunk]
        rows = torch.arange(qi.numel(), device=x.device)
        sims = x[qi] @ x.T
        sims[rows, qi] = -float("inf")
        asc = torch.sort(-sims, dim=1).values            # ascending negated similarity
        d2 = torch.cdist(emb[qi], emb, compute_mode="donot_use_mm_for_euclid_dist")
        d2[rows, qi] = float("inf")
        nb = torch.topk(d2, k, dim=1, largest=False).indices
        s_nb = sims.gather(1, nb)
        rank = torch.searchsorted(asc, (-s_nb).contiguous(), right=False) + 1
        penalty += float((rank - k).clamp_min(0).sum().item())
        lq, ln = labels[qi], labels[nb]
        maj = torch.mode(ln, dim=1).values
        valid = lq >= 0
        correct += int(((maj == lq) & valid).sum().item())
        counted += int(valid.sum().item())
        del sims, asc, d2
    m = q.numel()
    trust = 1.0 - 2.0 / (m * k * (2.0 * n - 3.0 * k - 1.0)) * penalty
    return {"trustworthiness": round(trust, 5),
            "knn_label_acc": round(correct / max(counted, 1), 5), "queries": m}


def timed(fn, reps: int = 3):
    """Median wall time (synchronised) of fn() over reps runs, and its last result."""
    torch = _torch()
    ts, res = [], None
    for _ in range(reps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        res = fn()
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t)
    return float(np.median(ts)), res
