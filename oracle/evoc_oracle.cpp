// evoc_oracle.cpp — CPU restatement of the evoc-rs 0.2.7 hot path.
//
// TEST INFRASTRUCTURE ONLY. This file is the oracle that the CUDA library is
// checked against, and the timed CPU baseline of the benchmark. Nothing in the
// product links, loads or calls it.
//
// It restates, function by function (citations are paths inside evoc-rs):
//   smooth_knn_dist            src/graph/fuzzy_graph.rs:33-98
//   knn_to_coo                 src/graph/fuzzy_graph.rs:114-159
//   symmetrise_graph           src/graph/fuzzy_graph.rs:174-228
//   coo_to_adjacency_list      src/graph/fuzzy_graph.rs:242-256
//   build_fuzzy_simplicial_set src/graph/fuzzy_graph.rs:275-295
//   evoc_embedding             src/graph/embedding.rs:48-298
//   EvocEmbeddingParams        src/graph/mod.rs:22-67
//   label_prop_iteration       src/graph/label_prop.rs:45-92
//   label_outliers             src/graph/label_prop.rs:105-142
//   remap_labels               src/graph/label_prop.rs:155-180
//   label_prop_loop            src/graph/label_prop.rs:202-230
//   label_propagation_init     src/graph/label_prop.rs:243-564 with the CSR
//                              algebra of src/utils/sparse.rs:130-568
// with the same parallel decomposition as the reference's rayon code
// (parallel rows in smooth_knn_dist, serial knn_to_coo and hash inserts,
// parallel per-row union, parallel nodes / nodes / edges in the three epoch
// phases).
//
// Documented deviations (shared with the CUDA library, which makes the two
// bit-identical):
//   1. exp() is ora_expf below (Cody-Waite reduction + degree-7 Taylor
//      polynomial), not the platform libm expf. oracle_smooth_knn_dist can
//      also run with libm expf to measure the difference.
//   2. Per-row output order of symmetrise_graph is ascending column; the
//      reference emits FxHashMap iteration order (fuzzy_graph.rs:205), which
//      depends on rustc-hash 2.1.3 and std's hashbrown and is not reproducible
//      without a Rust toolchain.
//   3. Negative samples (embedding.rs:230-231) and the random initial
//      embedding (embedding.rs:69-76) come from Philox4x32-10 (Salmon et al.,
//      "Parallel random numbers: as easy as 1, 2, 3", SC 2011) instead of
//      rand 0.10's SmallRng: negatives of edge e at epoch t use counter
//      (j, t, e_lo, e_hi & 0x7fffffff) and key (seed_lo, seed_hi);
//      k = (u32 * n) >> 32. The label-propagation seed draws
//      (label_prop.rs:216-219) and outlier fallback draws (:138-140) use the
//      counters of lp_seed_draw / lp_outlier_draw below.
//   4. The squared distance (ann-search-rs 0.5.2 euclidean_simd, called at
//      embedding.rs:210,237) is the serial left fold sum_d (a_d - b_d)^2.
//   The per-node gradient is the reference's running sum (embedding.rs:
//   194-248) in incidence-list order; with deviation 2 that list order is the
//   canonical one.
// Floating-point expressions are evaluated exactly as written in the Rust
// source (no contraction: build with -ffp-contract=off).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// exp: Cody-Waite range reduction x = k ln2 + r, |r| <= ln2/2, then the
// degree-7 Taylor polynomial of e^r in Horner form, then scaling by 2^k.
// ln2 is split into ln2_hi (15 significant bits, so k*ln2_hi is exact for
// |k| < 512) and ln2_lo = ln2 - ln2_hi.
// ---------------------------------------------------------------------------
inline float pow2i(int k) {  // 2^k for -126 <= k <= 127
  uint32_t bits = (uint32_t)(k + 127) << 23;
  float f;
  std::memcpy(&f, &bits, 4);
  return f;
}

inline float ora_expf(float x) {
  if (x != x) return x;
  if (x < -104.0f) return 0.0f;
  if (x > 88.72f) return std::numeric_limits<float>::infinity();
  const float log2e = 1.44269502f;
  const float ln2_hi = 0.693145751953125f;
  const float ln2_lo = 1.42860677e-06f;
  float kf = std::nearbyintf(x * log2e);
  float r = x - kf * ln2_hi;
  r = r - kf * ln2_lo;
  float p = 1.98412701e-04f;   // 1/5040
  p = p * r + 1.38888892e-03f; // 1/720
  p = p * r + 8.33333377e-03f; // 1/120
  p = p * r + 4.16666679e-02f; // 1/24
  p = p * r + 1.66666672e-01f; // 1/6
  p = p * r + 0.5f;
  p = p * r + 1.0f;
  p = p * r + 1.0f;
  int k = (int)kf;
  if (k >= -126) return p * pow2i(k);
  return (p * pow2i(k + 64)) * pow2i(-64);
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Random123). Round: (hi0,lo0)=M0*c0, (hi1,lo1)=M1*c2,
// c' = (hi1^c1^k0, lo1, hi0^c3^k1, lo0); key += (W0, W1) between rounds.
// ---------------------------------------------------------------------------
inline void philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                          uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

inline uint32_t negative_draw(uint64_t seed, uint32_t j, uint32_t epoch,
                              uint64_t eidx, uint32_t n) {
  const uint32_t ctr[4] = {j, epoch, (uint32_t)eidx,
                           (uint32_t)(eidx >> 32) & 0x7fffffffu};
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  philox4x32_10(ctr, key, o);
  return (uint32_t)(((uint64_t)o[0] * (uint64_t)n) >> 32);
}

inline float init_value(uint64_t seed, uint64_t idx) {
  const uint32_t ctr[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), 0u,
                           0x80000000u | 0x494E4954u};
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  philox4x32_10(ctr, key, o);
  uint64_t bits = (((uint64_t)o[1] << 32) | o[0]) >> 11;
  double u = (double)bits * (1.0 / 9007199254740992.0);
  return (float)(-0.25 + 0.5 * u);
}

// num-traits ToPrimitive::to_usize for f32: Some(trunc) iff -1 < x < 2^64.
inline uint64_t to_usize_or0(float x) {
  if (x > -1.0f && x < 18446744073709551616.0f) return (uint64_t)x;
  return 0;
}

inline float max0(float a) { return (a > 0.0f) ? a : 0.0f; }

// Open-addressing map u32 -> f32 standing in for FxHashMap<usize, T>:
// insert overwrites (last wins), like HashMap::insert.
struct U32F32Map {
  std::vector<uint32_t> keys;
  std::vector<float> vals;
  uint32_t count = 0;
  static constexpr uint32_t EMPTY = 0xFFFFFFFFu;
  static inline uint32_t h(uint32_t k) { return k * 0x9E3779B1u; }
  void grow() {
    size_t cap = keys.empty() ? 8 : keys.size() * 2;
    std::vector<uint32_t> ok;
    std::vector<float> ov;
    ok.swap(keys);
    ov.swap(vals);
    keys.assign(cap, EMPTY);
    vals.assign(cap, 0.0f);
    count = 0;
    for (size_t i = 0; i < ok.size(); ++i)
      if (ok[i] != EMPTY) insert(ok[i], ov[i]);
  }
  void insert(uint32_t k, float v) {
    if ((count + 1) * 8 > keys.size() * 7) grow();
    size_t mask = keys.size() - 1;
    size_t s = (h(k) >> 7) & mask;
    while (true) {
      if (keys[s] == EMPTY) { keys[s] = k; vals[s] = v; ++count; return; }
      if (keys[s] == k) { vals[s] = v; return; }
      s = (s + 1) & mask;
    }
  }
  bool get(uint32_t k, float* v) const {
    if (keys.empty()) return false;
    size_t mask = keys.size() - 1;
    size_t s = (h(k) >> 7) & mask;
    while (true) {
      if (keys[s] == EMPTY) return false;
      if (keys[s] == k) { *v = vals[s]; return true; }
      s = (s + 1) & mask;
    }
  }
};

}  // namespace

// A graph in the reference's CoordinateList form; rows are non-decreasing,
// so it is also a CSR adjacency list (coo_to_adjacency_list keeps COO order).
struct OracleGraph {
  int64_t n = 0;
  std::vector<int64_t> indptr;
  std::vector<uint32_t> indices;
  std::vector<float> weights;
};

struct OracleEmbedParams {
  int32_t n_epochs;
  float noise_level;
  float negative_sample_rate;
  float initial_alpha;
  float beta1;
  float beta2;
  float eps;
};

struct OracleEpochStats {
  int64_t fired_edges;
  int64_t negatives;
  int64_t active_nodes;
};

extern "C" {

int oracle_abi_version(void) { return 1; }

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

float oracle_expf(float x) { return ora_expf(x); }

void oracle_philox4x32_10(const uint32_t* ctr, const uint32_t* key,
                          uint32_t* out) {
  philox4x32_10(ctr, key, out);
}

uint32_t oracle_negative_draw(uint64_t seed, uint32_t j, uint32_t epoch,
                              uint64_t eidx, uint32_t n) {
  return negative_draw(seed, j, epoch, eidx, n);
}

float oracle_init_value(uint64_t seed, uint64_t idx) {
  return init_value(seed, idx);
}

// smooth_knn_dist, fuzzy_graph.rs:33-98. Returns 0, or -1 when a row is empty
// while local_connectivity > 0 (the reference panics there: d.len() - 1 and
// d[idx] at :55/:61) or local_connectivity is not finite (.unwrap() at :54).
int oracle_smooth_knn_dist(const float* dists, const int32_t* row_len,
                           int64_t n, int32_t k, uint64_t k_target,
                           float local_connectivity, int32_t n_iter,
                           int use_libm_exp, float* sigmas, float* rhos) {
  const double target = std::log2((double)k_target);  // :42
  const double tolerance = 1e-5;                       // :43
  const float lc = local_connectivity;
  if (lc > 0.0f && !std::isfinite(lc)) return -1;
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(| : bad)
  for (int64_t i = 0; i < n; ++i) {
    const float* d = dists + i * (int64_t)k;
    const int64_t len = row_len ? row_len[i] : k;
    float rho;
    if (lc > 0.0f) {  // :49-62
      if (len <= 0) { bad = 1; sigmas[i] = 0; rhos[i] = 0; continue; }
      float lm1 = max0(lc - 1.0f);
      float fl = std::floor(lm1);
      uint64_t idx = (uint64_t)fl;
      if (idx > (uint64_t)(len - 1)) idx = (uint64_t)(len - 1);
      float frac = lm1 - fl;
      if (frac > 0.0f && (int64_t)idx + 1 < len)
        rho = d[idx] * (1.0f - frac) + d[idx + 1] * frac;
      else
        rho = d[idx];
    } else {
      rho = 0.0f;  // :63-65
    }
    float lo = 0.0f, hi = std::numeric_limits<float>::max(), mid = 1.0f;
    for (int32_t it = 0; it < n_iter; ++it) {  // :71-93
      float val = 0.0f;
      for (int64_t j = 0; j < len; ++j) {
        float adjusted = max0(d[j] - rho);
        float a = -(adjusted / mid);
        val += use_libm_exp ? std::exp(a) : ora_expf(a);
      }
      double vd = (double)val;
      if (std::fabs(vd - target) < tolerance) break;
      if (vd > target) {
        hi = mid;
        mid = (lo + hi) / 2.0f;
      } else {
        lo = mid;
        if (hi == std::numeric_limits<float>::max())
          mid = mid * 2.0f;
        else
          mid = (lo + hi) / 2.0f;
      }
    }
    sigmas[i] = mid;
    rhos[i] = rho;
  }
  return bad ? -1 : 0;
}

// knn_to_coo, fuzzy_graph.rs:114-159 (serial, like the reference). Entries
// whose index is EVOC_KNN_PAD (0xFFFFFFFF) end the row.
OracleGraph* oracle_knn_to_coo(const uint32_t* knn_idx, const float* knn_dist,
                               int64_t n, int32_t k, const float* sigmas,
                               const float* rhos) {
  OracleGraph* g = new OracleGraph();
  g->n = n;
  g->indptr.assign(n + 1, 0);
  g->indices.reserve((size_t)n * k);
  g->weights.reserve((size_t)n * k);
  for (int64_t i = 0; i < n; ++i) {
    const float sigma = sigmas[i], rho = rhos[i];
    for (int32_t j = 0; j < k; ++j) {
      uint32_t c = knn_idx[i * (int64_t)k + j];
      if (c == 0xFFFFFFFFu) break;
      if ((int64_t)c == i) continue;  // :135
      float adjusted = max0(knn_dist[i * (int64_t)k + j] - rho);
      float w;
      if (sigma > 0.0f)
        w = ora_expf(-(adjusted / sigma));
      else if (adjusted > 0.0f)
        w = 0.0f;
      else
        w = 1.0f;
      g->indices.push_back(c);
      g->weights.push_back(w);
    }
    g->indptr[i + 1] = (int64_t)g->indices.size();
  }
  return g;
}

// symmetrise_graph, fuzzy_graph.rs:174-228. Rows are emitted in ascending
// column order (deviation 2).
OracleGraph* oracle_symmetrise(const OracleGraph* in) {
  const int64_t n = in->n;
  std::vector<U32F32Map> forward(n), backward(n);
  for (int64_t i = 0; i < n; ++i)  // :183-191, serial
    for (int64_t p = in->indptr[i]; p < in->indptr[i + 1]; ++p) {
      uint32_t j = in->indices[p];
      float w = in->weights[p];
      forward[i].insert(j, w);
      backward[j].insert((uint32_t)i, w);
    }
  std::vector<std::vector<std::pair<uint32_t, float>>> rows(n);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {  // :193-207
    U32F32Map combined;
    auto visit = [&](uint32_t j) {
      float w_ij = 0.0f, w_ji = 0.0f;
      forward[i].get(j, &w_ij);
      backward[i].get(j, &w_ji);
      float w_sym = w_ij + w_ji - w_ij * w_ji;
      if (w_sym > 0.0f) combined.insert(j, w_sym);
    };
    for (size_t s = 0; s < forward[i].keys.size(); ++s)
      if (forward[i].keys[s] != U32F32Map::EMPTY) visit(forward[i].keys[s]);
    for (size_t s = 0; s < backward[i].keys.size(); ++s)
      if (backward[i].keys[s] != U32F32Map::EMPTY) visit(backward[i].keys[s]);
    auto& r = rows[i];
    r.reserve(combined.count);
    for (size_t s = 0; s < combined.keys.size(); ++s)
      if (combined.keys[s] != U32F32Map::EMPTY)
        r.emplace_back(combined.keys[s], combined.vals[s]);
    std::sort(r.begin(), r.end(),
              [](const std::pair<uint32_t, float>& a,
                 const std::pair<uint32_t, float>& b) {
                return a.first < b.first;
              });
  }
  OracleGraph* g = new OracleGraph();  // :209-227
  g->n = n;
  g->indptr.assign(n + 1, 0);
  for (int64_t i = 0; i < n; ++i)
    g->indptr[i + 1] = g->indptr[i] + (int64_t)rows[i].size();
  g->indices.resize(g->indptr[n]);
  g->weights.resize(g->indptr[n]);
  for (int64_t i = 0; i < n; ++i) {
    int64_t o = g->indptr[i];
    for (auto& e : rows[i]) {
      g->indices[o] = e.first;
      g->weights[o] = e.second;
      ++o;
    }
  }
  return g;
}

// build_fuzzy_simplicial_set, fuzzy_graph.rs:275-295. Returns NULL where the
// reference panics (n == 0 through knn_dists[0] at :286; empty rows).
OracleGraph* oracle_fuzzy_set(const uint32_t* knn_idx, const float* knn_dist,
                              int64_t n, int32_t k,
                              float effective_n_neighbours, int symmetrise,
                              float* sigmas_out, float* rhos_out) {
  if (n <= 0) return nullptr;
  std::vector<int32_t> row_len(n);
  for (int64_t i = 0; i < n; ++i) {
    int32_t l = 0;
    while (l < k && knn_idx[i * (int64_t)k + l] != 0xFFFFFFFFu) ++l;
    row_len[i] = l;
  }
  // :284-286; unwrap_or evaluates knn_dists[0].len() eagerly.
  float e = effective_n_neighbours;
  uint64_t kk = (e > -1.0f && e < 18446744073709551616.0f) ? (uint64_t)e
                                                            : (uint64_t)row_len[0];
  std::vector<float> sig(n), rho(n);
  if (oracle_smooth_knn_dist(knn_dist, row_len.data(), n, k, kk, 1.0f, 64, 0,
                             sig.data(), rho.data()) != 0)
    return nullptr;
  if (sigmas_out) std::memcpy(sigmas_out, sig.data(), n * sizeof(float));
  if (rhos_out) std::memcpy(rhos_out, rho.data(), n * sizeof(float));
  OracleGraph* coo = oracle_knn_to_coo(knn_idx, knn_dist, n, k, sig.data(),
                                       rho.data());
  if (!symmetrise) return coo;
  OracleGraph* s = oracle_symmetrise(coo);
  delete coo;
  return s;
}

OracleGraph* oracle_graph_from_csr(const int64_t* indptr,
                                   const uint32_t* indices,
                                   const float* weights, int64_t n) {
  OracleGraph* g = new OracleGraph();
  g->n = n;
  g->indptr.assign(indptr, indptr + n + 1);
  g->indices.assign(indices, indices + indptr[n]);
  g->weights.assign(weights, weights + indptr[n]);
  return g;
}

int64_t oracle_graph_n(const OracleGraph* g) { return g->n; }
int64_t oracle_graph_nnz(const OracleGraph* g) {
  return g->indptr.empty() ? 0 : g->indptr[g->n];
}
void oracle_graph_export(const OracleGraph* g, int64_t* indptr,
                         uint32_t* indices, float* weights) {
  std::memcpy(indptr, g->indptr.data(), (g->n + 1) * sizeof(int64_t));
  size_t nnz = (size_t)oracle_graph_nnz(g);
  if (nnz) {
    std::memcpy(indices, g->indices.data(), nnz * sizeof(uint32_t));
    std::memcpy(weights, g->weights.data(), nnz * sizeof(float));
  }
}
void oracle_graph_free(OracleGraph* g) { delete g; }

// evoc_embedding, embedding.rs:48-298, on a CSR adjacency list.
// Epochs [0, start_epoch) only advance the schedule (embedding.rs:274-286);
// epochs [start_epoch, end_epoch) run in full. grad_out (optional) receives
// the gradient of the last epoch run. stats (optional, n_epochs entries)
// receives per-epoch counts for the epochs run in full, epoch_seconds
// (optional, n_epochs entries) the wall time of each epoch run in full.
// Returns 0, or -1 for invalid arguments.
int oracle_evoc_embedding(const int64_t* indptr, const uint32_t* indices,
                          const float* weights, int64_t n, int32_t dim,
                          const OracleEmbedParams* params, const float* init,
                          uint64_t seed, int32_t start_epoch,
                          int32_t end_epoch, float* out, float* grad_out,
                          OracleEpochStats* stats, double* epoch_seconds) {
  if (n == 0) return 0;  // :61-64
  if (dim <= 0 || !params) return -1;
  const int64_t D = dim;
  std::vector<float> embd((size_t)(n * D));
  if (init) {  // :70-71
    std::memcpy(embd.data(), init, n * D * sizeof(float));
  } else {  // :72-75 (deviation 3)
    for (int64_t q = 0; q < n * D; ++q) embd[q] = init_value(seed, (uint64_t)q);
  }
  if (grad_out) std::memset(grad_out, 0, n * D * sizeof(float));

  // :78-90 extract undirected edges (i < j) in adjacency-list order
  struct Edge { uint32_t i, j; float w; };
  std::vector<Edge> edges;
  std::vector<int64_t> degree(n, 0);
  for (int64_t i = 0; i < n; ++i)
    for (int64_t p = indptr[i]; p < indptr[i + 1]; ++p) {
      uint32_t j = indices[p];
      if ((int64_t)i < (int64_t)j) {
        edges.push_back({(uint32_t)i, j, weights[p]});
        degree[i] += 1;
        degree[j] += 1;
      }
    }
  if (edges.empty()) {  // :92-96
    std::memcpy(out, embd.data(), n * D * sizeof(float));
    return 0;
  }
  const int64_t U = (int64_t)edges.size();

  // :99-118 epoch sampling schedules
  float max_weight = 0.0f;
  for (auto& e : edges) max_weight = std::fmax(max_weight, e.w);
  std::vector<float> eps_sample(U), next_sample(U), eps_neg(U), next_neg(U);
  const float neg_factor = 1.5f / params->negative_sample_rate;
  for (int64_t e = 0; e < U; ++e) {
    float norm = edges[e].w / max_weight;
    eps_sample[e] = (norm > 0.0f) ? 1.0f / norm : 1e8f;
    next_sample[e] = eps_sample[e];
    eps_neg[e] = eps_sample[e] * neg_factor;
    next_neg[e] = eps_neg[e];
  }

  // :121-135 per-node CSR of (edge_idx, is_smaller, other)
  std::vector<int64_t> offsets(n + 1, 0);
  for (int64_t i = 0; i < n; ++i) offsets[i + 1] = offsets[i] + degree[i];
  struct Inc { int64_t eidx; bool is_smaller; uint32_t other; };
  std::vector<Inc> csr_edges(2 * U);
  {
    std::vector<int64_t> cursor(offsets.begin(), offsets.end() - 1);
    for (int64_t e = 0; e < U; ++e) {
      csr_edges[cursor[edges[e].i]++] = {e, true, edges[e].j};
      csr_edges[cursor[edges[e].j]++] = {e, false, edges[e].i};
    }
  }

  // :138-175 Adam state and schedules
  const int32_t n_epochs = params->n_epochs;
  std::vector<float> m_buf(n * D, 0.0f), v_buf(n * D, 0.0f);
  const float one_m_b1 = 1.0f - params->beta1;
  const float one_m_b2 = 1.0f - params->beta2;
  std::vector<float> ad_scale(n_epochs), epsc(n_epochs), gamma(n_epochs);
  for (int32_t ep = 0; ep < n_epochs; ++ep) {
    float t = (float)(ep + 1);
    float b1t = std::pow(params->beta1, t);
    float b2t = std::pow(params->beta2, t);
    float sqrt_b2 = std::sqrt(1.0f - b2t);
    ad_scale[ep] = sqrt_b2 / (1.0f - b1t);
    epsc[ep] = sqrt_b2 * params->eps;
  }
  const float denom = (float)std::max(n_epochs - 1, 1);
  for (int32_t i = 0; i < n_epochs; ++i) gamma[i] = 0.5f + (float)i / denom;
  const float n_epochs_f = (float)n_epochs;
  const float noise = params->noise_level;

  std::vector<float> grads(n * D, 0.0f);
  std::vector<uint8_t> active(n, 0);

  auto schedule_update = [&](int32_t epoch) {  // :274-286
    const float epoch_t = (float)epoch;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < U; ++e) {
      if (next_sample[e] <= epoch_t) {
        next_sample[e] += eps_sample[e];
        uint64_t neg_count =
            to_usize_or0(std::floor((epoch_t - next_neg[e]) / eps_neg[e]));
        next_neg[e] += (float)neg_count * eps_neg[e];
      }
    }
  };

  const int32_t e0 = std::max(0, std::min(start_epoch, n_epochs));
  const int32_t e1 = std::max(e0, std::min(end_epoch, n_epochs));
  for (int32_t epoch = 0; epoch < e0; ++epoch) schedule_update(epoch);

  for (int32_t epoch = e0; epoch < e1; ++epoch) {
#ifdef _OPENMP
    const double t_start = omp_get_wtime();
#endif
    const float lr = params->initial_alpha * (1.0f - (float)epoch / n_epochs_f);
    const float epoch_t = (float)epoch;
    const float ads = ad_scale[epoch], epc = epsc[epoch], gam = gamma[epoch];
    int64_t fired_edges = 0, negs = 0, act = 0;

    // :188-253 gradient accumulation, parallel over nodes
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : fired_edges, negs, act)
    for (int64_t ni = 0; ni < n; ++ni) {
      float* g = &grads[ni * D];  // :194-196
      for (int64_t d = 0; d < D; ++d) g[d] = 0.0f;
      const float* ei = &embd[ni * D];
      bool touched = false;
      const int64_t start = offsets[ni], end = offsets[ni + 1];
      for (int64_t q = start; q < end; ++q) {
        const Inc& ce = csr_edges[q];
        if (next_sample[ce.eidx] > epoch_t) continue;  // :204
        touched = true;
        const float* eo = &embd[(int64_t)ce.other * D];
        float dsq = 0.0f;  // :210 (deviation 4)
        for (int64_t d = 0; d < D; ++d) {
          float df = ei[d] - eo[d];
          dsq = dsq + df * df;
        }
        if (dsq >= 1e-8f) {  // :213-221
          float dist = std::sqrt(dsq);
          float coeff = (-(2.0f * noise * dist) - 2.0f) /
                        (2.0f * dsq - 0.5f * dist + 1.0f);
          for (int64_t d = 0; d < D; ++d) g[d] += coeff * (ei[d] - eo[d]);
        }
        if (ce.is_smaller) {  // :224-247
          ++fired_edges;
          uint64_t n_neg = to_usize_or0(
              std::floor((epoch_t - next_neg[ce.eidx]) / eps_neg[ce.eidx]));
          negs += (int64_t)n_neg;
          for (uint64_t jj = 0; jj < n_neg; ++jj) {
            uint32_t kk = negative_draw(seed, (uint32_t)jj, (uint32_t)epoch,
                                        (uint64_t)ce.eidx, (uint32_t)n);
            if ((int64_t)kk == ni) continue;
            const float* ek = &embd[(int64_t)kk * D];
            float dsq_k = 0.0f;
            for (int64_t d = 0; d < D; ++d) {
              float df = ei[d] - ek[d];
              dsq_k = dsq_k + df * df;
            }
            if (dsq_k > 0.01f) {
              float gc = gam * 4.0f / ((1.0f + 0.25f * dsq_k) * dsq_k);
              for (int64_t d = 0; d < D; ++d) {
                float diff = ei[d] - ek[d];
                float c = gc * diff;
                c = std::fmax(c, -4.0f);
                c = std::fmin(c, 4.0f);
                g[d] += c;
              }
            }
          }
        }
      }
      active[ni] = touched ? 1 : 0;
      act += touched ? 1 : 0;
    }

    if (grad_out && epoch == e1 - 1)
      for (int64_t ni = 0; ni < n; ++ni)
        for (int64_t d = 0; d < D; ++d)
          grad_out[ni * D + d] = active[ni] ? grads[ni * D + d] : 0.0f;

    // :256-272 Adam moment update + embedding step, parallel over nodes
    const float lr_ad = lr * ads;
#pragma omp parallel for schedule(static)
    for (int64_t ni = 0; ni < n; ++ni) {
      if (!active[ni]) continue;
      for (int64_t d = 0; d < D; ++d) {
        int64_t q = ni * D + d;
        float gd = grads[q];
        m_buf[q] = m_buf[q] + one_m_b1 * (gd - m_buf[q]);
        v_buf[q] = v_buf[q] + one_m_b2 * (gd * gd - v_buf[q]);
        embd[q] += lr_ad * m_buf[q] / (std::sqrt(v_buf[q]) + epc);
      }
    }

    schedule_update(epoch);  // :274-286
    if (stats) stats[epoch] = {fired_edges, negs, act};
#ifdef _OPENMP
    if (epoch_seconds) epoch_seconds[epoch] = omp_get_wtime() - t_start;
#else
    if (epoch_seconds) epoch_seconds[epoch] = 0.0;
#endif
  }
  std::memcpy(out, embd.data(), n * D * sizeof(float));
  return 0;
}


// ---------------------------------------------------------------------------
// Label propagation partition (label_prop.rs:45-230). Labels are int64 as in
// the reference; -1 is "unlabelled". The seed draws (label_prop.rs:216-219)
// and the outlier fallback draws (:138-140) come from Philox4x32-10 instead of
// rand::SmallRng (the counters below; the CUDA library uses the same ones).
// ---------------------------------------------------------------------------
static uint32_t lp_seed_draw(uint64_t seed, uint32_t i, uint32_t n) {
  const uint32_t ctr[4] = {i, 0u, 0x4C50u, 0x53454544u};
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  philox4x32_10(ctr, key, o);
  return (uint32_t)(((uint64_t)o[0] * (uint64_t)n) >> 32);
}
static uint32_t lp_outlier_draw(uint64_t seed, uint64_t i, uint32_t range) {
  const uint32_t ctr[4] = {(uint32_t)i, (uint32_t)(i >> 32), 0x4C50u, 0x4F555431u};
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  philox4x32_10(ctr, key, o);
  return (uint32_t)(((uint64_t)o[0] * (uint64_t)range) >> 32);
}

// label_prop.rs:45-92: one conservative iteration, parallel over nodes.
void oracle_lp_iteration(const int64_t* indptr, const uint32_t* indices, const float* w,
                         int64_t n, const int64_t* in, int64_t* out) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    if (in[i] >= 0) {
      out[i] = in[i];
      continue;
    }
    std::vector<std::pair<int64_t, float>> votes;  // first-appearance order
    for (int64_t e = indptr[i]; e < indptr[i + 1]; ++e) {
      const int64_t l = in[indices[e]];
      bool hit = false;
      for (auto& v : votes)
        if (v.first == l) {
          v.second += w[e];
          hit = true;
          break;
        }
      if (!hit) votes.emplace_back(l, w[e]);
    }
    int64_t best = -1;
    float max_vote = 1.0f;  // threshold
    for (const auto& v : votes) {
      if (v.first < 0) continue;
      if (v.second > max_vote) {
        max_vote = v.second;
        best = v.first;
      } else if (v.second == max_vote) {
        best = v.first;  // last encountered wins
      }
    }
    out[i] = best;
  }
}

// label_prop.rs:105-142: sequential mop-up, a LIFO walk of at most 64 pops per
// unlabelled node, then a random existing label.
void oracle_lp_outliers(const int64_t* indptr, const uint32_t* indices, int64_t n,
                        int64_t* labels, uint64_t seed) {
  int64_t max_label = -1;
  for (int64_t i = 0; i < n; ++i) max_label = std::max(max_label, labels[i]);
  if (max_label < 0) return;
  std::vector<uint32_t> queue;
  for (int64_t i = 0; i < n; ++i) {
    if (labels[i] >= 0) continue;
    queue.assign(1, (uint32_t)i);
    bool found = false;
    for (int step = 0; step < 64 && !found; ++step) {
      if (queue.empty()) break;
      const uint32_t node = queue.back();
      queue.pop_back();
      for (int64_t e = indptr[node]; e < indptr[node + 1]; ++e) {
        const uint32_t j = indices[e];
        if (labels[j] >= 0) {
          labels[i] = labels[j];
          found = true;
          break;
        }
        queue.push_back(j);
      }
    }
    if (!found) labels[i] = (int64_t)lp_outlier_draw(seed, (uint64_t)i, (uint32_t)(max_label + 1));
  }
}

// label_prop.rs:155-180: labels >= 0 to 0..n_unique in sorted order; each -1
// gets the next new id in node order. Returns the number of labels.
int64_t oracle_lp_remap(int64_t* labels, int64_t n) {
  std::vector<int64_t> sorted;
  for (int64_t i = 0; i < n; ++i)
    if (labels[i] >= 0) sorted.push_back(labels[i]);
  std::sort(sorted.begin(), sorted.end());
  sorted.erase(std::unique(sorted.begin(), sorted.end()), sorted.end());
  int64_t next = (int64_t)sorted.size();
  for (int64_t i = 0; i < n; ++i) {
    if (labels[i] < 0)
      labels[i] = next++;
    else
      labels[i] = std::lower_bound(sorted.begin(), sorted.end(), labels[i]) - sorted.begin();
  }
  return next;
}

// label_prop.rs:202-230: seed, iterate, mop up, remap.
int64_t oracle_lp_partition(const int64_t* indptr, const uint32_t* indices, const float* w,
                            int64_t n, int64_t approx_n_parts, int32_t n_iter, uint64_t seed,
                            uint32_t* partition) {
  std::vector<int64_t> a((size_t)n, -1), b((size_t)n, -1);
  for (int64_t i = 0; i < approx_n_parts; ++i) a[lp_seed_draw(seed, (uint32_t)i, (uint32_t)n)] = i;
  for (int32_t it = 0; it < n_iter; ++it) {
    oracle_lp_iteration(indptr, indices, w, n, a.data(), b.data());
    a.swap(b);
  }
  oracle_lp_outliers(indptr, indices, n, a.data(), seed + 2000);
  const int64_t parts = oracle_lp_remap(a.data(), n);
  for (int64_t i = 0; i < n; ++i) partition[i] = (uint32_t)a[i];
  return parts;
}


// ---------------------------------------------------------------------------
// label_propagation_init (label_prop.rs:243-564) on the CSR algebra of
// src/utils/sparse.rs:130-568, with the reference's summation orders:
//   matmul        row-wise; per output row the products a_ik * b_kj are added
//                 in the order of A's row entries, then B's row entries (the
//                 first one set, later ones added), columns gathered sorted
//                 (sparse.rs:307-365, SpaAcc :9-60);
//   transpose     counting sort, rows in order (:256-296);
//   norms         serial sums in storage order (:404-470);
//   matmul_dense  per row, entries in order, row[k] += v * rhs[j][k] (:545-568).
// Deviations: random draws from Philox (deviation 3); the PCA base case takes
// its singular vectors from a Jacobi eigen-decomposition of X X^T, so their
// signs follow a fixed convention (largest-magnitude component positive)
// rather than faer's.
// ---------------------------------------------------------------------------
struct OCsr {
  int64_t nrows = 0, ncols = 0;
  std::vector<int64_t> indptr, indices;
  std::vector<float> data;
};

static OCsr ocsr_from_partition(const std::vector<int64_t>& part, int64_t n_parts) {  // :243-254
  OCsr m;
  m.nrows = (int64_t)part.size();
  m.ncols = n_parts;
  m.indptr.resize(m.nrows + 1);
  for (int64_t i = 0; i <= m.nrows; ++i) m.indptr[i] = i;
  m.indices = part;
  m.data.assign(m.nrows, 1.0f);
  return m;
}

static OCsr ocsr_transpose(const OCsr& a) {  // :256-296
  OCsr t;
  t.nrows = a.ncols;
  t.ncols = a.nrows;
  t.indptr.assign(t.nrows + 1, 0);
  for (int64_t c : a.indices) t.indptr[c + 1] += 1;
  for (int64_t i = 0; i < t.nrows; ++i) t.indptr[i + 1] += t.indptr[i];
  t.indices.resize(a.indices.size());
  t.data.resize(a.data.size());
  std::vector<int64_t> cur(t.indptr.begin(), t.indptr.end() - 1);
  for (int64_t r = 0; r < a.nrows; ++r)
    for (int64_t e = a.indptr[r]; e < a.indptr[r + 1]; ++e) {
      const int64_t p = cur[a.indices[e]]++;
      t.data[p] = a.data[e];
      t.indices[p] = r;
    }
  return t;
}

static OCsr ocsr_matmul(const OCsr& a, const OCsr& b) {  // :307-365
  OCsr c;
  c.nrows = a.nrows;
  c.ncols = b.ncols;
  std::vector<std::vector<std::pair<int64_t, float>>> rows((size_t)a.nrows);
#pragma omp parallel
  {
    std::vector<float> val((size_t)b.ncols, 0.0f);
    std::vector<char> flag((size_t)b.ncols, 0);
    std::vector<int64_t> touched;
#pragma omp for schedule(dynamic, 64)
    for (int64_t i = 0; i < a.nrows; ++i) {
      touched.clear();
      for (int64_t ae = a.indptr[i]; ae < a.indptr[i + 1]; ++ae) {
        const int64_t k = a.indices[ae];
        const float av = a.data[ae];
        for (int64_t be = b.indptr[k]; be < b.indptr[k + 1]; ++be) {
          const int64_t j = b.indices[be];
          const float prod = av * b.data[be];
          if (!flag[j]) {
            flag[j] = 1;
            touched.push_back(j);
            val[j] = prod;
          } else {
            val[j] = val[j] + prod;
          }
        }
      }
      std::sort(touched.begin(), touched.end());
      auto& row = rows[i];
      row.reserve(touched.size());
      for (int64_t j : touched) {
        row.emplace_back(j, val[j]);
        flag[j] = 0;
        val[j] = 0.0f;
      }
    }
  }
  c.indptr.assign(c.nrows + 1, 0);
  for (int64_t i = 0; i < c.nrows; ++i) c.indptr[i + 1] = c.indptr[i] + (int64_t)rows[i].size();
  c.indices.reserve(c.indptr[c.nrows]);
  c.data.reserve(c.indptr[c.nrows]);
  for (auto& row : rows)
    for (auto& e : row) {
      c.indices.push_back(e.first);
      c.data.push_back(e.second);
    }
  return c;
}

static OCsr ocsr_elementwise_mul(const OCsr& a, const OCsr& b) {  // :378-417
  OCsr c;
  c.nrows = a.nrows;
  c.ncols = a.ncols;
  c.indptr.assign(c.nrows + 1, 0);
  for (int64_t i = 0; i < a.nrows; ++i) {
    int64_t p = a.indptr[i], q = b.indptr[i];
    const int64_t ep = a.indptr[i + 1], eq = b.indptr[i + 1];
    while (p < ep && q < eq) {
      if (a.indices[p] == b.indices[q]) {
        c.indices.push_back(a.indices[p]);
        c.data.push_back(a.data[p] * b.data[q]);
        ++p;
        ++q;
      } else if (a.indices[p] < b.indices[q]) {
        ++p;
      } else {
        ++q;
      }
    }
    c.indptr[i + 1] = (int64_t)c.data.size();
  }
  return c;
}

static OCsr ocsr_normalise_cols_l2(const OCsr& a) {  // :427-458
  std::vector<float> sq((size_t)a.ncols, 0.0f);
  for (size_t e = 0; e < a.data.size(); ++e) sq[a.indices[e]] += a.data[e] * a.data[e];
  std::vector<float> inv((size_t)a.ncols);
  for (int64_t c = 0; c < a.ncols; ++c) {
    const float nrm = std::sqrt(sq[c]);
    inv[c] = nrm > 0.0f ? 1.0f / nrm : 1.0f;
  }
  OCsr r = a;
  for (size_t e = 0; e < r.data.size(); ++e) r.data[e] = a.data[e] * inv[a.indices[e]];
  return r;
}

static OCsr ocsr_normalise_rows_l1(const OCsr& a) {  // :468-492
  OCsr r = a;
  for (int64_t i = 0; i < a.nrows; ++i) {
    float nrm = 0.0f;
    for (int64_t e = a.indptr[i]; e < a.indptr[i + 1]; ++e) nrm += std::fabs(a.data[e]);
    if (nrm > 0.0f) {
      const float inv = 1.0f / nrm;
      for (int64_t e = a.indptr[i]; e < a.indptr[i + 1]; ++e) r.data[e] = r.data[e] * inv;
    }
  }
  return r;
}

static void ocsr_clip(OCsr& a, float lo, float hi) {  // :501-510
  for (float& d : a.data) {
    if (d < lo)
      d = lo;
    else if (d > hi)
      d = hi;
  }
}

static std::vector<float> ocsr_matmul_dense(const OCsr& a, const std::vector<float>& rhs,
                                            int64_t d) {  // :545-568
  std::vector<float> out((size_t)(a.nrows * d), 0.0f);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < a.nrows; ++i)
    for (int64_t e = a.indptr[i]; e < a.indptr[i + 1]; ++e) {
      const int64_t j = a.indices[e];
      const float v = a.data[e];
      for (int64_t k = 0; k < d; ++k) out[i * d + k] += v * rhs[j * d + k];
    }
  return out;
}

// label_prop.rs:243-280: per column, midpoint to 0 and half-range to 1.
static void lp_unit_range(std::vector<float>& m, int64_t n, int64_t d) {
  for (int64_t j = 0; j < d; ++j) {
    float lo = std::numeric_limits<float>::infinity(), hi = -std::numeric_limits<float>::infinity();
    for (int64_t i = 0; i < n; ++i) {
      const float v = m[i * d + j];
      if (v < lo) lo = v;
      if (v > hi) hi = v;
    }
    const float range = hi - lo;
    if (range > 0.0f) {
      const float mid = (hi + lo) / 2.0f, half = range / 2.0f;
      for (int64_t i = 0; i < n; ++i) m[i * d + j] = (m[i * d + j] - mid) / half;
    }
  }
}

// Symmetric Jacobi eigen-decomposition (cyclic sweeps) of a k x k matrix a
// (row-major, destroyed): eigenvalues in w, eigenvectors in the columns of v.
static void jacobi_eigen(std::vector<double>& a, int64_t k, std::vector<double>& w,
                         std::vector<double>& v) {
  v.assign((size_t)(k * k), 0.0);
  for (int64_t i = 0; i < k; ++i) v[i * k + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int64_t p = 0; p < k; ++p)
      for (int64_t q = p + 1; q < k; ++q) off += a[p * k + q] * a[p * k + q];
    if (off < 1e-30) break;
    for (int64_t p = 0; p < k; ++p)
      for (int64_t q = p + 1; q < k; ++q) {
        const double apq = a[p * k + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double theta = (a[q * k + q] - a[p * k + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int64_t r = 0; r < k; ++r) {  // A <- A J (columns p, q)
          const double ap = a[r * k + p], aq = a[r * k + q];
          a[r * k + p] = c * ap - sn * aq;
          a[r * k + q] = sn * ap + c * aq;
        }
        for (int64_t r = 0; r < k; ++r) {  // A <- J^T A (rows p, q)
          const double ap = a[p * k + r], aq = a[q * k + r];
          a[p * k + r] = c * ap - sn * aq;
          a[q * k + r] = sn * ap + c * aq;
        }
        for (int64_t r = 0; r < k; ++r) {
          const double vp = v[r * k + p], vq = v[r * k + q];
          v[r * k + p] = c * vp - sn * vq;
          v[r * k + q] = sn * vp + c * vq;
        }
      }
  }
  w.resize((size_t)k);
  for (int64_t i = 0; i < k; ++i) w[i] = a[i * k + i];
}

// label_prop.rs:288-330: the centred data's first components, u_j s_j, from
// the eigenvectors of X X^T (sigma_j^2 = eigenvalue), then the unit range.
static std::vector<float> lp_pca_init(const std::vector<float>& data, int64_t n, int64_t d,
                                      int64_t n_comp, int64_t* out_cols) {
  const int64_t k = std::min(std::min(n_comp, n), d);
  std::vector<double> mean((size_t)d, 0.0);
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = 0; j < d; ++j) mean[j] += (double)data[i * d + j];
  const double inv_n = 1.0 / (double)n;
  for (double& m : mean) m *= inv_n;
  std::vector<double> x((size_t)(n * d));
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = 0; j < d; ++j) x[i * d + j] = (double)data[i * d + j] - mean[j];
  std::vector<double> g((size_t)(n * n), 0.0);
  for (int64_t a = 0; a < n; ++a)
    for (int64_t b = 0; b < n; ++b) {
      double acc = 0.0;
      for (int64_t j = 0; j < d; ++j) acc += x[a * d + j] * x[b * d + j];
      g[a * n + b] = acc;
    }
  std::vector<double> w, v;
  jacobi_eigen(g, n, w, v);
  std::vector<int64_t> order((size_t)n);
  for (int64_t i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return w[a] > w[b]; });
  std::vector<float> out((size_t)(n * k));
  for (int64_t c = 0; c < k; ++c) {
    const int64_t e = order[c];
    const double sig = std::sqrt(std::max(w[e], 0.0));
    int64_t big = 0;  // sign convention: the largest-magnitude entry is positive
    for (int64_t i = 1; i < n; ++i)
      if (std::fabs(v[i * n + e]) > std::fabs(v[big * n + e])) big = i;
    const double sgn = v[big * n + e] < 0 ? -1.0 : 1.0;
    for (int64_t i = 0; i < n; ++i) out[i * k + c] = (float)(sgn * v[i * n + e] * sig);
  }
  lp_unit_range(out, n, k);
  *out_cols = k;
  return out;
}

// label_prop.rs:338-360: uniform in [-1, 1] per coordinate, rows L2-normalised
// (Philox draws: counter (q_lo, q_hi, "LP", "RINI"), key seed).
static std::vector<float> lp_random_init(int64_t n, int64_t dim, uint64_t seed) {
  std::vector<float> out((size_t)(n * dim));
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  for (int64_t q = 0; q < n * dim; ++q) {
    const uint32_t ctr[4] = {(uint32_t)q, (uint32_t)((uint64_t)q >> 32), 0x4C50u, 0x52494E49u};
    uint32_t o[4];
    philox4x32_10(ctr, key, o);
    const double u = (double)((((uint64_t)o[1] << 32) | o[0]) >> 11) * (1.0 / 9007199254740992.0);
    out[q] = (float)(u * 2.0 - 1.0);
  }
  for (int64_t i = 0; i < n; ++i) {
    double nrm = 0.0;
    for (int64_t j = 0; j < dim; ++j) nrm += (double)out[i * dim + j] * (double)out[i * dim + j];
    nrm = std::sqrt(nrm);
    if (nrm > 0.0)
      for (int64_t j = 0; j < dim; ++j) out[i * dim + j] = (float)((double)out[i * dim + j] / nrm);
  }
  return out;
}

static int64_t lp_partition_csr(const OCsr& g, int64_t parts, int32_t n_iter, uint64_t seed,
                                std::vector<int64_t>& part);

// label_prop.rs:403-535
static std::vector<float> lp_init_inner(const OCsr& g, int64_t dim, const std::vector<float>* data,
                                        int64_t d, int32_t n_emb_epochs, int64_t approx_parts,
                                        int32_t n_lp_iter, int64_t base_thr, double scaling,
                                        uint64_t seed) {
  const int64_t n = g.nrows;
  if (n < base_thr) {  // :440-445
    if (data && (int64_t)(data->size() / std::max<int64_t>(d, 1)) == n && dim <= d) {
      int64_t cols = 0;
      std::vector<float> pc = lp_pca_init(*data, n, d, dim, &cols);
      if (cols == dim) return pc;
      std::vector<float> full((size_t)(n * dim), 0.0f);  // fewer points than components
      for (int64_t i = 0; i < n; ++i)
        for (int64_t c = 0; c < cols; ++c) full[i * dim + c] = pc[i * cols + c];
      return full;
    }
    return lp_random_init(n, dim, seed);
  }
  std::vector<int64_t> part;  // :448
  const int64_t n_parts = lp_partition_csr(g, approx_parts, n_lp_iter, seed, part);
  const OCsr base = ocsr_from_partition(part, n_parts);  // :455-457
  const OCsr norm = ocsr_normalise_cols_l2(base);
  const OCsr reducer = ocsr_normalise_rows_l1(ocsr_transpose(norm));
  const OCsr nrt = ocsr_transpose(norm);  // :460-462
  OCsr reduced = ocsr_matmul(ocsr_matmul(nrt, g), base);
  ocsr_clip(reduced, 0.0f, 1.0f);
  std::vector<float> rdata;  // :464-469
  if (data) rdata = ocsr_matmul_dense(reducer, *data, d);
  const int32_t e = std::min(n_emb_epochs, 255);
  const std::vector<float> rinit =  // :472-483
      lp_init_inner(reduced, dim, data ? &rdata : nullptr, d, e, approx_parts / 4, n_lp_iter,
                    base_thr, scaling, seed + 3000);
  // :486-498 short embedding of the coarse graph
  std::vector<uint32_t> ridx(reduced.indices.begin(), reduced.indices.end());
  OracleEmbedParams ep{e, 0.5f, 1.0f, (float)(0.001 * (double)e), 0.5f, 0.9f, 1e-7f};
  std::vector<float> layout((size_t)(reduced.nrows * dim));
  oracle_evoc_embedding(reduced.indptr.data(), ridx.data(), reduced.data.data(), reduced.nrows,
                        (int32_t)dim, &ep, rinit.data(), seed + 4000, 0, e, layout.data(),
                        nullptr, nullptr, nullptr);
  // :500-510 expansion
  const OCsr sym = ocsr_elementwise_mul(g, ocsr_transpose(g));
  const OCsr expander = ocsr_normalise_rows_l1(ocsr_matmul(sym, norm));
  const OCsr nrm_l1 = ocsr_normalise_rows_l1(norm);
  const std::vector<float> expanded = ocsr_matmul_dense(expander, layout, dim);
  const std::vector<float> direct = ocsr_matmul_dense(nrm_l1, layout, dim);
  std::vector<float> res((size_t)(n * dim));
  for (int64_t q = 0; q < n * dim; ++q) res[q] = (expanded[q] + direct[q]) * 0.5f;  // :512-516
  const float inv_n = (float)(1.0 / (double)n);  // :518-528
  for (int64_t j = 0; j < dim; ++j) {
    float sum = 0.0f;
    for (int64_t i = 0; i < n; ++i) sum += res[i * dim + j];
    const float mean = sum * inv_n;
    for (int64_t i = 0; i < n; ++i) res[i * dim + j] = res[i * dim + j] - mean;
  }
  const float scale = (float)scaling;  // :530-534
  for (float& v : res) v = scale * v;
  return res;
}


static int64_t lp_partition_csr(const OCsr& g, int64_t parts, int32_t n_iter, uint64_t seed,
                                std::vector<int64_t>& part) {
  std::vector<uint32_t> idx(g.indices.begin(), g.indices.end());
  std::vector<uint32_t> p((size_t)g.nrows);
  const int64_t k = oracle_lp_partition(g.indptr.data(), idx.data(), g.data.data(), g.nrows,
                                        parts, n_iter, seed, p.data());
  part.assign(p.begin(), p.end());
  return k;
}

// label_prop.rs:243-280 on a row-major n x d f32 array (in place).
void oracle_lp_unit_range(float* m, int64_t n, int64_t d) {
  std::vector<float> v(m, m + n * d);
  lp_unit_range(v, n, d);
  std::memcpy(m, v.data(), v.size() * sizeof(float));
}

// The coarse graph of one level (label_prop.rs:455-462): clip(R^T G P) for the
// partition `part` (n entries, n_parts parts); returned as an OracleGraph.
OracleGraph* oracle_lp_coarse_graph(const int64_t* indptr, const uint32_t* indices,
                                    const float* w, int64_t n, const uint32_t* part,
                                    int64_t n_parts) {
  OCsr g;
  g.nrows = g.ncols = n;
  g.indptr.assign(indptr, indptr + n + 1);
  g.indices.assign(indices, indices + indptr[n]);
  g.data.assign(w, w + indptr[n]);
  std::vector<int64_t> pv(part, part + n);
  const OCsr base = ocsr_from_partition(pv, n_parts);
  const OCsr norm = ocsr_normalise_cols_l2(base);
  OCsr red = ocsr_matmul(ocsr_matmul(ocsr_transpose(norm), g), base);
  ocsr_clip(red, 0.0f, 1.0f);
  OracleGraph* out = new OracleGraph();
  out->n = red.nrows;
  out->indptr = red.indptr;
  out->indices.assign(red.indices.begin(), red.indices.end());
  out->weights = red.data;
  return out;
}

// label_propagation_init (label_prop.rs:537-564): data (n x d f32) may be NULL.
int oracle_lp_init(const int64_t* indptr, const uint32_t* indices, const float* w, int64_t n,
                   int32_t dim, const float* data, int64_t d, uint64_t seed, float* out) {
  if (n <= 0 || dim <= 0) return -1;
  OCsr g;
  g.nrows = g.ncols = n;
  g.indptr.assign(indptr, indptr + n + 1);
  g.indices.assign(indices, indices + indptr[n]);
  g.data.assign(w, w + indptr[n]);
  const int64_t parts =
      std::min<int64_t>(std::max<int64_t>((int64_t)(8.0 * std::sqrt((double)n)), 256), 16384);
  std::vector<float> dv;
  if (data) dv.assign(data, data + n * d);
  const std::vector<float> res = lp_init_inner(g, dim, data ? &dv : nullptr, d, 50,
                                               std::min(parts, n), 20, 64, 0.1, seed);
  std::memcpy(out, res.data(), res.size() * sizeof(float));
  return 0;
}

}  // extern "C"
