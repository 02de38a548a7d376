"""ctypes wrapper of the CPU oracle (oracle/evoc_oracle.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/, by __graft_entry__.smoke() as the
checker, and by bench.py's CPU baseline. The product never imports this.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
SRCS = [HERE / "evoc_oracle.cpp", HERE / "evoc_labels_oracle.cpp"]


class OracleParams(C.Structure):
    _fields_ = [("n_epochs", C.c_int32), ("noise_level", C.c_float),
                ("negative_sample_rate", C.c_float), ("initial_alpha", C.c_float),
                ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float)]


class OracleStats(C.Structure):
    _fields_ = [("fired_edges", C.c_int64), ("negatives", C.c_int64),
                ("active_nodes", C.c_int64)]


def build() -> Path:
    if not LIB.exists() or any(LIB.stat().st_mtime < s.stat().st_mtime for s in SRCS):
        subprocess.run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
                        "-ffp-contract=off", "-o", str(LIB), *map(str, SRCS)], check=True)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        vp, i32, i64, u32, u64, f32 = (C.c_void_p, C.c_int32, C.c_int64, C.c_uint32,
                                       C.c_uint64, C.c_float)
        sigs = {
            "oracle_set_threads": ([C.c_int], None),
            "oracle_max_threads": ([], C.c_int),
            "oracle_expf": ([f32], f32),
            "oracle_philox4x32_10": ([vp, vp, vp], None),
            "oracle_negative_draw": ([u64, u32, u32, u64, u32], u32),
            "oracle_init_value": ([u64, u64], f32),
            "oracle_smooth_knn_dist": ([vp, vp, i64, i32, u64, f32, i32, C.c_int, vp, vp], C.c_int),
            "oracle_knn_to_coo": ([vp, vp, i64, i32, vp, vp], vp),
            "oracle_symmetrise": ([vp], vp),
            "oracle_fuzzy_set": ([vp, vp, i64, i32, f32, C.c_int, vp, vp], vp),
            "oracle_graph_from_csr": ([vp, vp, vp, i64], vp),
            "oracle_graph_n": ([vp], i64),
            "oracle_graph_nnz": ([vp], i64),
            "oracle_graph_export": ([vp, vp, vp, vp], None),
            "oracle_graph_free": ([vp], None),
            "oracle_evoc_embedding": ([vp, vp, vp, i64, i32, C.POINTER(OracleParams), vp, u64,
                                       i32, i32, vp, vp, vp, vp], C.c_int),
            "oracle_lp_iteration": ([vp, vp, vp, i64, vp, vp], None),
            "oracle_lp_outliers": ([vp, vp, i64, vp, u64], None),
            "oracle_lp_remap": ([vp, i64], i64),
            "oracle_lp_partition": ([vp, vp, vp, i64, i64, i32, u64, vp], i64),
            "oracle_lp_unit_range": ([vp, i64, i64], None),
            "oracle_lp_coarse_graph": ([vp, vp, vp, i64, vp, i64], vp),
            "oracle_lp_init": ([vp, vp, vp, i64, i32, vp, i64, u64, vp], C.c_int),
            "oracle_build_mst": ([vp, i64, i64, i64, vp, vp, vp], i64),
            "oracle_linkage": ([vp, vp, vp, i64, i64, vp, vp], None),
            "oracle_leaf_labels": ([vp, i64, i64, i64, i64, vp, vp], i64),
            "oracle_cluster_layers": ([vp, i64, i64, i64, i64, C.c_double, i64], vp),
            "oracle_cluster_layers_mst": ([vp, vp, vp, i64, i64, i64, C.c_double, i64], vp),
            "oracle_layers_count": ([vp], i64),
            "oracle_layers_get": ([vp, i64, vp, vp, vp], None),
            "oracle_layers_free": ([vp], None),
            "oracle_find_peaks": ([vp, i64, vp], i64),
            "oracle_barcodes": ([vp, i64, i64, i64, i64, vp, vp, vp, vp], i64),
            "oracle_search_n_clusters": ([vp, i64, i64, i64, i64, vp, vp], i64),
        }
        for k, (a, r) in sigs.items():
            f = getattr(L, k)
            f.argtypes = a
            f.restype = r
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def max_threads() -> int:
    return lib().oracle_max_threads()


def expf(x: float) -> float:
    return lib().oracle_expf(float(x))


def expf_array(x: np.ndarray) -> np.ndarray:
    f = lib().oracle_expf
    return np.array([f(float(v)) for v in np.asarray(x, dtype=np.float32)], dtype=np.float32)


def philox(ctr, key) -> np.ndarray:
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib().oracle_philox4x32_10(_p(c), _p(k), _p(o))
    return o


def negative_draw(seed: int, j: int, epoch: int, eidx: int, n: int) -> int:
    return lib().oracle_negative_draw(seed, j, epoch, eidx, n)


def smooth_knn_dist(dists, k_target: int, local_connectivity: float = 1.0, n_iter: int = 64,
                    row_len=None, libm_exp: bool = False):
    d = np.ascontiguousarray(dists, dtype=np.float32)
    n, k = d.shape
    rl = None if row_len is None else np.ascontiguousarray(row_len, dtype=np.int32)
    sig = np.zeros(n, dtype=np.float32)
    rho = np.zeros(n, dtype=np.float32)
    rc = lib().oracle_smooth_knn_dist(_p(d), _p(rl), n, k, int(k_target), float(local_connectivity),
                                      int(n_iter), int(libm_exp), _p(sig), _p(rho))
    if rc != 0:
        raise ValueError("smooth_knn_dist: empty row with local_connectivity > 0")
    return sig, rho


def _export(g) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    L = lib()
    n = L.oracle_graph_n(g)
    nnz = L.oracle_graph_nnz(g)
    ip = np.zeros(n + 1, dtype=np.int64)
    ix = np.zeros(nnz, dtype=np.uint32)
    w = np.zeros(nnz, dtype=np.float32)
    L.oracle_graph_export(g, _p(ip), _p(ix), _p(w))
    L.oracle_graph_free(g)
    return ip, ix, w


def knn_to_coo(knn_idx, knn_dist, sigmas, rhos):
    idx = np.ascontiguousarray(knn_idx, dtype=np.uint32)
    dist = np.ascontiguousarray(knn_dist, dtype=np.float32)
    s = np.ascontiguousarray(sigmas, dtype=np.float32)
    r = np.ascontiguousarray(rhos, dtype=np.float32)
    g = lib().oracle_knn_to_coo(_p(idx), _p(dist), idx.shape[0], idx.shape[1], _p(s), _p(r))
    return _export(g)


def symmetrise(indptr, indices, weights):
    ip = np.ascontiguousarray(indptr, dtype=np.int64)
    ix = np.ascontiguousarray(indices, dtype=np.uint32)
    w = np.ascontiguousarray(weights, dtype=np.float32)
    L = lib()
    g = L.oracle_graph_from_csr(_p(ip), _p(ix), _p(w), len(ip) - 1)
    s = L.oracle_symmetrise(g)
    L.oracle_graph_free(g)
    return _export(s)


def fuzzy_set(knn_idx, knn_dist, effective_n_neighbours: float, symmetrise: bool = True,
              return_sigma_rho: bool = False):
    idx = np.ascontiguousarray(knn_idx, dtype=np.uint32)
    dist = np.ascontiguousarray(knn_dist, dtype=np.float32)
    n, k = idx.shape
    sig = np.zeros(n, dtype=np.float32)
    rho = np.zeros(n, dtype=np.float32)
    g = lib().oracle_fuzzy_set(_p(idx), _p(dist), n, k, float(effective_n_neighbours),
                               int(bool(symmetrise)), _p(sig), _p(rho))
    if not g:
        raise ValueError("build_fuzzy_simplicial_set panics on this input")
    out = _export(g)
    return (out, sig, rho) if return_sigma_rho else out


def evoc_embedding(indptr, indices, weights, dim: int, n_epochs: int = 50,
                   noise_level: float = 0.5, negative_sample_rate: float = 1.0,
                   initial_alpha: float = 0.1, beta1: float = 0.5, beta2: float = 0.9,
                   eps: float = 1e-7, init=None, seed: int = 42, start_epoch: int = 0,
                   end_epoch: int | None = None, want_grad: bool = False,
                   want_stats: bool = False, want_times: bool = False):
    ip = np.ascontiguousarray(indptr, dtype=np.int64)
    ix = np.ascontiguousarray(indices, dtype=np.uint32)
    w = np.ascontiguousarray(weights, dtype=np.float32)
    n = len(ip) - 1
    p = OracleParams(n_epochs, noise_level, negative_sample_rate, initial_alpha, beta1, beta2,
                     eps)
    ini = None if init is None else np.ascontiguousarray(init, dtype=np.float32)
    out = np.zeros((n, dim), dtype=np.float32)
    grad = np.zeros((n, dim), dtype=np.float32) if want_grad else None
    st = (OracleStats * max(n_epochs, 1))() if want_stats else None
    times = np.zeros(max(n_epochs, 1), dtype=np.float64) if want_times else None
    end = n_epochs if end_epoch is None else end_epoch
    rc = lib().oracle_evoc_embedding(_p(ip), _p(ix), _p(w), n, dim, C.byref(p), _p(ini),
                                     C.c_uint64(seed), start_epoch, end, _p(out), _p(grad),
                                     st if st is not None else None, _p(times))
    if rc != 0:
        raise ValueError("oracle_evoc_embedding: invalid arguments")
    res = [out]
    if want_grad:
        res.append(grad)
    if want_stats:
        s = np.array([(st[t].fired_edges, st[t].negatives, st[t].active_nodes)
                      for t in range(n_epochs)], dtype=np.int64).reshape(-1, 3)
        res.append(s)
    if want_times:
        res.append(times[:n_epochs])
    return res[0] if len(res) == 1 else tuple(res)


# ---- label propagation partition (label_prop.rs:45-230) ---------------------
def _csr(indptr, indices, weights=None):
    ip = np.ascontiguousarray(indptr, dtype=np.int64)
    ix = np.ascontiguousarray(indices, dtype=np.uint32)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float32)
    return ip, ix, w


def lp_iteration(indptr, indices, weights, labels) -> np.ndarray:
    ip, ix, w = _csr(indptr, indices, weights)
    lab = np.ascontiguousarray(labels, dtype=np.int64)
    out = np.empty_like(lab)
    lib().oracle_lp_iteration(_p(ip), _p(ix), _p(w), len(ip) - 1, _p(lab), _p(out))
    return out


def lp_outliers(indptr, indices, labels, seed: int) -> np.ndarray:
    ip, ix, _ = _csr(indptr, indices)
    lab = np.array(labels, dtype=np.int64)
    lib().oracle_lp_outliers(_p(ip), _p(ix), len(ip) - 1, _p(lab), seed)
    return lab


def lp_remap(labels) -> tuple[np.ndarray, int]:
    lab = np.array(labels, dtype=np.int64)
    k = lib().oracle_lp_remap(_p(lab), len(lab))
    return lab, int(k)


def lp_partition(indptr, indices, weights, approx_n_parts: int, n_iter: int = 20,
                 seed: int = 42) -> tuple[np.ndarray, int]:
    ip, ix, w = _csr(indptr, indices, weights)
    n = len(ip) - 1
    part = np.zeros(n, dtype=np.uint32)
    k = lib().oracle_lp_partition(_p(ip), _p(ix), _p(w), n, approx_n_parts, n_iter, seed,
                                  _p(part))
    return part, int(k)


def lp_unit_range(m) -> np.ndarray:
    """normalise_to_unit_range (label_prop.rs:243-280)."""
    a = np.array(m, dtype=np.float32, order="C")
    lib().oracle_lp_unit_range(_p(a), a.shape[0], a.shape[1])
    return a


def lp_coarse_graph(indptr, indices, weights, partition, n_parts: int):
    """clip(R^T G P) of one level (label_prop.rs:455-462) as CSR arrays."""
    ip, ix, w = _csr(indptr, indices, weights)
    part = np.ascontiguousarray(partition, dtype=np.uint32)
    g = lib().oracle_lp_coarse_graph(_p(ip), _p(ix), _p(w), len(ip) - 1, _p(part), n_parts)
    return _export(g)  # frees g


def lp_init(indptr, indices, weights, dim: int, data=None, seed: int = 42) -> np.ndarray:
    """label_propagation_init (label_prop.rs:537-564)."""
    ip, ix, w = _csr(indptr, indices, weights)
    n = len(ip) - 1
    dd = None if data is None else np.ascontiguousarray(data, dtype=np.float32)
    out = np.zeros((n, dim), dtype=np.float32)
    rc = lib().oracle_lp_init(_p(ip), _p(ix), _p(w), n, dim, _p(dd),
                              0 if dd is None else dd.shape[1], seed, _p(out))
    if rc != 0:
        raise ValueError("oracle_lp_init: invalid arguments")
    return out


# ---------------------------------------------------------------------------
# Clustering of the embedding (evoc_labels_oracle.cpp): the reference's own
# CPU stage after the embedding, restated to compare labels.
# ---------------------------------------------------------------------------
def _emb(embedding) -> np.ndarray:
    e = np.ascontiguousarray(embedding, dtype=np.float32)
    if e.ndim != 2:
        raise ValueError("embedding must be n x dim")
    return e


def build_mst(embedding, min_samples: int = 5):
    """Boruvka MST over mutual reachability (src/clustering/mst.rs:82-166):
    (u, v, weight) arrays of the n - 1 edges in insertion order."""
    e = _emb(embedding)
    n, d = e.shape
    m = max(n - 1, 0)
    u = np.zeros(m, np.int64)
    v = np.zeros(m, np.int64)
    w = np.zeros(m, np.float32)
    k = lib().oracle_build_mst(_p(e), n, d, int(min_samples), _p(u), _p(v), _p(w))
    return u[:k], v[:k], w[:k]


def linkage(u, v, w, n: int):
    """mst_to_linkage_tree (src/clustering/linkage.rs:39-85): rows (left,
    right, size) and distances."""
    u = np.ascontiguousarray(u, np.int64)
    v = np.ascontiguousarray(v, np.int64)
    w = np.ascontiguousarray(w, np.float32)
    m = len(u)
    lr = np.zeros((m, 3), np.int64)
    dist = np.zeros(m, np.float32)
    lib().oracle_linkage(_p(u), _p(v), _p(w), m, int(n), _p(lr), _p(dist))
    return lr, dist


def leaf_labels(embedding, min_samples: int = 5, min_cluster_size: int = 5):
    """Leaf clusters of the condensed tree at one min_cluster_size (the base
    layer of build_cluster_layers): (labels, strengths, n_leaves)."""
    e = _emb(embedding)
    n, d = e.shape
    lab = np.zeros(n, np.int64)
    st = np.zeros(n, np.float32)
    k = lib().oracle_leaf_labels(_p(e), n, d, int(min_samples), int(min_cluster_size), _p(lab),
                                 _p(st))
    return lab, st, int(k)


def build_cluster_layers(embedding, min_samples: int = 5, base_min_cluster_size: int = 5,
                         min_similarity_threshold: float = 0.2, max_layers: int = 10):
    """build_cluster_layers (src/clustering/persistence.rs:387-463): lists of
    per-layer labels, strengths and persistence scores, finest layer first."""
    e = _emb(embedding)
    n, d = e.shape
    L = lib()
    h = L.oracle_cluster_layers(_p(e), n, d, int(min_samples), int(base_min_cluster_size),
                                float(min_similarity_threshold), int(max_layers))
    return _layers(L, h, n)


def build_cluster_layers_from_mst(u, v, w, n: int, base_min_cluster_size: int = 5,
                                  min_similarity_threshold: float = 0.2, max_layers: int = 10):
    """build_cluster_layers from a given minimum spanning tree (the MST built
    by persistence.rs:402 replaced by (u, v, weight) in insertion order)."""
    u = np.ascontiguousarray(u, np.int64)
    v = np.ascontiguousarray(v, np.int64)
    w = np.ascontiguousarray(w, np.float32)
    L = lib()
    h = L.oracle_cluster_layers_mst(_p(u), _p(v), _p(w), len(u), int(n),
                                    int(base_min_cluster_size), float(min_similarity_threshold),
                                    int(max_layers))
    return _layers(L, h, n)


def _layers(L, h, n: int):
    labels, strengths, pers = [], [], []
    try:
        for i in range(L.oracle_layers_count(h)):
            lab = np.zeros(n, np.int64)
            st = np.zeros(n, np.float32)
            p = C.c_double(0.0)
            L.oracle_layers_get(h, i, _p(lab), _p(st), C.byref(p))
            labels.append(lab)
            strengths.append(st)
            pers.append(p.value)
    finally:
        L.oracle_layers_free(h)
    return labels, strengths, pers


def best_labels(layers) -> np.ndarray:
    """EvocResult::best_labels (src/lib.rs:124-137): the layer with the highest
    persistence score (Iterator::max_by: the last of equal maxima), or the
    only layer."""
    labels, _, pers = layers
    if len(labels) <= 1:
        return labels[0]
    best, bi = None, 0
    for i, p in enumerate(pers):  # max_by keeps the last of equal maxima
        if best is None or not (p < best):
            best, bi = p, i
    return labels[bi]


def find_peaks(x) -> np.ndarray:
    a = np.ascontiguousarray(x, np.float32)
    out = np.zeros(max(len(a), 1), np.int64)
    k = lib().oracle_find_peaks(_p(a), len(a), _p(out))
    return out[:k]


def barcodes(embedding, min_samples: int, min_cluster_size: int):
    """min_cluster_size_barcode + compute_total_persistence: (barcodes as
    rows of birth, death, parent, lambda_death; sizes; persistence)."""
    e = _emb(embedding)
    n, d = e.shape
    bc = np.zeros((max(n, 1), 4), np.float64)
    sizes = np.zeros(max(n, 1), np.float32)
    pers = np.zeros(max(n, 1), np.float32)
    ns = C.c_int64(0)
    k = lib().oracle_barcodes(_p(e), n, d, int(min_samples), int(min_cluster_size), _p(bc),
                              _p(sizes), _p(pers), C.byref(ns))
    return bc[:k], sizes[:ns.value], pers[:ns.value]


def search_for_n_clusters(embedding, min_samples: int, target_k: int):
    """search_for_n_clusters (src/lib.rs:377-452): (labels, strengths, k)."""
    e = _emb(embedding)
    n, d = e.shape
    lab = np.zeros(n, np.int64)
    st = np.zeros(n, np.float32)
    k = lib().oracle_search_n_clusters(_p(e), n, d, int(min_samples), int(target_k), _p(lab),
                                       _p(st))
    return lab, st, int(k)


def adjusted_rand_index(a, b) -> float:
    """Adjusted Rand index (Hubert and Arabie, 1985) of two labelings; every
    label value (noise -1 included) is its own class, as in the usual
    contingency-table formula."""
    a = np.asarray(a)
    b = np.asarray(b)
    if a.shape != b.shape:
        raise ValueError("labelings differ in length")
    n = a.size
    if n < 2:
        return 1.0
    _, ai = np.unique(a, return_inverse=True)
    _, bi = np.unique(b, return_inverse=True)
    cont = np.zeros((ai.max() + 1, bi.max() + 1), np.int64)
    np.add.at(cont, (ai, bi), 1)
    comb = lambda x: x * (x - 1) / 2.0
    s_ij = comb(cont.astype(np.float64)).sum()
    s_a = comb(cont.sum(1).astype(np.float64)).sum()
    s_b = comb(cont.sum(0).astype(np.float64)).sum()
    expected = s_a * s_b / comb(float(n))
    mx = 0.5 * (s_a + s_b)
    if mx == expected:
        return 1.0
    return float((s_ij - expected) / (mx - expected))
