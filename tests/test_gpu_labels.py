"""Final cluster labels of GPU embeddings against the oracle's, through the
reference's clustering stage (MST, linkage, condensed tree, persistence
layers: src/clustering/*.rs, restated in oracle/evoc_labels_oracle.cpp).

The fourth correctness check of the hot path: labels computed from the GPU
embedding must reach an adjusted Rand index of at least 0.98 against the
labels computed from the oracle's embedding of the same graph. The
embeddings are bit-identical, so the labels are expected to be identical.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _labels(O, emb):
    layers = O.build_cluster_layers(emb, 5, 5, 0.2, 10)  # EvocParams defaults, lib.rs:84-98
    return layers, O.best_labels(layers)


def test_labels_blobs_10k_vs_oracle(ctx, oracle, blobs_knn):
    """10,000 x 384 blobs, k 15, dim 4 (the CPU configuration), seed 42."""
    idx, dist, _ = blobs_knn
    g = ctx.fuzzy_set(idx, dist, 15.0, True)
    ip, ix, w = g.export()
    gpu = ctx.embed(g, 4, seed=42)
    ref = oracle.evoc_embedding(ip, ix, w, 4, seed=42)
    (gl, _, gp), gbest = _labels(oracle, gpu)
    (rl, _, rp), rbest = _labels(oracle, ref)
    ari = oracle.adjusted_rand_index(gbest, rbest)
    assert ari >= 0.98, ari
    assert len(gl) == len(rl) and all(np.array_equal(a, b) for a, b in zip(gl, rl))
    assert gp == rp


@pytest.mark.parametrize("dim", [2, 8])
def test_labels_other_dims_vs_oracle(ctx, oracle, small_knn, dim):
    idx, dist, _ = small_knn
    g = ctx.fuzzy_set(idx, dist, 15.0, True)
    ip, ix, w = g.export()
    _, gbest = _labels(oracle, ctx.embed(g, dim, seed=9))
    _, rbest = _labels(oracle, oracle.evoc_embedding(ip, ix, w, dim, seed=9))
    assert oracle.adjusted_rand_index(gbest, rbest) >= 0.98
