// lp_init.cu — label_propagation_init (src/graph/label_prop.rs:403-564,
// evoc-rs 0.2.7) on the GPU: the recursive coarsening initialisation that
// evoc() runs before the embedding.
//
// One level (label_prop_init_inner, label_prop.rs:403-535) of an n-node graph:
//   1. partition by label propagation (label_prop.cu);
//   2. per part P: node count c_P, inv_P = 1 / sqrt(c_P) (the L2 column
//      norm of the partition matrix, sparse.rs:427-458), the L1 row scale of
//      its transpose (serial sum of c_P copies of inv_P, sparse.rs:468-492);
//   3. coarse graph clip(N^T G B) (sparse.rs:307-365): the products
//      inv_P * w_ij of every entry are ordered (P, j, i) by two stable radix
//      sorts and summed serially per (P, j) (the sparse accumulator's order:
//      rows of P ascending), then re-ordered (P, Q = part(j), j) and summed
//      serially per (P, Q); clipped to [0, 1] (sparse.rs:501-510);
//   4. coarse data (sparse.rs:545-568): per part, its nodes in order,
//      acc += scale * x;
//   5. recursion on the coarse graph and data (base case: PCA of the data,
//      or a random unit-row init, below 64 nodes);
//   6. a short embedding of the coarse graph (the library's own plan path);
//   7. expansion: the graph's symmetric part G o G^T times N, L1 row
//      normalised, times the coarse layout (per (i, Q) serial sums after the
//      same sort), averaged with the direct term N_l1 x layout, centred by
//      serial column sums, scaled.
// Summation orders are the reference's (restated in the oracle), so the
// initial embedding equals the oracle's bit for bit. Random draws are Philox
// (the documented deviation); the PCA base case is a Jacobi eigen-solve of
// the small Gram matrix in double on the host, with a fixed sign convention.
#include "evoc_device.cuh"
#include "evoc_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace evoc {
namespace {

inline unsigned grid_of(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// ---------------------------------------------------------------------------
// Per-part constants.
// ---------------------------------------------------------------------------
__global__ void k_part_count(const uint32_t* __restrict__ part, int64_t n,
                             int32_t* __restrict__ cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(&cnt[part[i]], 1);
}

// inv = 1 / sqrt(c) (c is exact: c products 1 * 1 summed); rv = inv * (1 / s)
// with s the serial sum of c copies of inv; u = inv * (1 / inv).
__global__ void k_part_consts(const int32_t* __restrict__ cnt, int64_t np,
                              float* __restrict__ inv, float* __restrict__ rv,
                              float* __restrict__ u) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const int32_t c = cnt[p];
  const float nrm = fsqrt((float)c);
  const float iv = nrm > 0.0f ? fdiv(1.0f, nrm) : 1.0f;
  float s = 0.0f;
  for (int32_t k = 0; k < c; ++k) s = fadd(s, fabsf(iv));
  rv[p] = s > 0.0f ? fmul(iv, fdiv(1.0f, s)) : iv;
  const float a = fabsf(iv);
  u[p] = a > 0.0f ? fmul(iv, fdiv(1.0f, a)) : iv;
  inv[p] = iv;
}

// ---------------------------------------------------------------------------
// Sort-and-sum machinery. An entry list in a given order is sorted stably by
// (major, minor) with two radix passes (minor first), then equal (major,
// minor) runs are summed serially in list order (first value, then +).
// Keys are u32; values are uint2 (other key, float bits).
// ---------------------------------------------------------------------------
// Coarse-graph products in row-major order: key j, value (P, inv_P * w_ij).
__global__ void k_gen_products(const int64_t* __restrict__ indptr,
                               const uint32_t* __restrict__ indices,
                               const float* __restrict__ w, int64_t n,
                               const uint32_t* __restrict__ part,
                               const float* __restrict__ inv, uint32_t* __restrict__ keys,
                               uint2* __restrict__ vals) {
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const uint32_t P = part[i];
  const float iv = inv[P];
  for (int64_t e = indptr[i] + lane; e < indptr[i + 1]; e += 32) {
    keys[e] = indices[e];
    vals[e] = make_uint2(P, __float_as_uint(fmul(iv, w[e])));
  }
}

// vals[i] = (i, 0)
__global__ void k_iota_pairs(uint2* __restrict__ vals, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) vals[i] = make_uint2((uint32_t)i, 0u);
}

// Entries of G in row-major order as (key column j, value (row i, w bits)):
// the input of the stable transpose (sparse.rs:256-296).
__global__ void k_transpose_gen(const int64_t* __restrict__ indptr,
                                const uint32_t* __restrict__ indices,
                                const float* __restrict__ w, int64_t n,
                                uint32_t* __restrict__ keys, uint2* __restrict__ vals) {
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  for (int64_t e = indptr[i] + lane; e < indptr[i + 1]; e += 32) {
    keys[e] = indices[e];
    vals[e] = make_uint2((uint32_t)i, __float_as_uint(w[e]));
  }
}

__global__ void k_unpack_pairs(const uint2* __restrict__ vals, int64_t m,
                               uint32_t* __restrict__ idx, float* __restrict__ w) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m) return;
  idx[e] = vals[e].x;
  w[e] = __uint_as_float(vals[e].y);
}

// keys <- vals.x, vals <- (old key, vals.y)
__global__ void k_swap_keys(uint32_t* __restrict__ keys, uint2* __restrict__ vals, int64_t m) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m) return;
  const uint32_t k = keys[e];
  const uint2 v = vals[e];
  keys[e] = v.x;
  vals[e] = make_uint2(k, v.y);
}

// keys <- map[vals.x], vals unchanged
__global__ void k_map_keys(uint32_t* __restrict__ keys, const uint2* __restrict__ vals,
                           int64_t m, const uint32_t* __restrict__ map) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < m) keys[e] = map[vals[e].x];
}

// head[e] = 1 where (keys, vals.x) starts a new run
__global__ void k_run_heads(const uint32_t* __restrict__ keys, const uint2* __restrict__ vals,
                            int64_t m, int32_t* __restrict__ head) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m) return;
  head[e] = (e == 0 || keys[e] != keys[e - 1] || vals[e].x != vals[e - 1].x) ? 1 : 0;
}

// Serial sum of each run into slot rid[e]: (key, (vals.x, sum bits)).
__global__ void k_run_sums(const uint32_t* __restrict__ keys, const uint2* __restrict__ vals,
                           int64_t m, const int32_t* __restrict__ head,
                           const int64_t* __restrict__ rid, uint32_t* __restrict__ okeys,
                           uint2* __restrict__ ovals) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m || !head[e]) return;
  float s = __uint_as_float(vals[e].y);
  for (int64_t f = e + 1; f < m && !head[f]; ++f) s = fadd(s, __uint_as_float(vals[f].y));
  const int64_t r = rid[e];
  okeys[r] = keys[e];
  ovals[r] = make_uint2(vals[e].x, __float_as_uint(s));
}

// Sorts (keys, vals) by (keys major, vals.x minor), stably, then sums the
// equal-(key, minor) runs serially. Returns the run count; the runs replace
// the list's head (keys, vals).
int64_t sort_and_sum(uint32_t* keys, uint2* vals, int64_t m, int major_bits, int minor_bits,
                     cudaStream_t s) {
  if (m == 0) return 0;
  // minor first (keys <- vals.x), then major
  k_swap_keys<<<grid_of(m), 256, 0, s>>>(keys, vals, m);
  EVOC_CHECK_LAUNCH();
  radix_sort_pairs(keys, vals, m, minor_bits, s);
  k_swap_keys<<<grid_of(m), 256, 0, s>>>(keys, vals, m);
  EVOC_CHECK_LAUNCH();
  radix_sort_pairs(keys, vals, m, major_bits, s);
  DevBuf<int32_t> head(m, s);
  DevBuf<int64_t> rid(m + 1, s);
  k_run_heads<<<grid_of(m), 256, 0, s>>>(keys, vals, m, head.get());
  EVOC_CHECK_LAUNCH();
  exclusive_scan_i32_to_i64(head.get(), rid.get(), m, s);
  int64_t runs = 0;
  EVOC_CUDA(cudaMemcpyAsync(&runs, rid.get() + m, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaStreamSynchronize(s));
  DevBuf<uint32_t> ok(runs, s);
  DevBuf<uint2> ov(runs, s);
  k_run_sums<<<grid_of(m), 256, 0, s>>>(keys, vals, m, head.get(), rid.get(), ok.get(),
                                        ov.get());
  EVOC_CHECK_LAUNCH();
  EVOC_CUDA(cudaMemcpyAsync(keys, ok.get(), runs * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  EVOC_CUDA(cudaMemcpyAsync(vals, ov.get(), runs * sizeof(uint2), cudaMemcpyDeviceToDevice, s));
  EVOC_CUDA(cudaStreamSynchronize(s));
  return runs;
}

// Row counts of a (row, (col, value)) run list sorted by row.
__global__ void k_row_hist(const uint32_t* __restrict__ keys, int64_t m,
                           int32_t* __restrict__ cnt) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < m) atomicAdd(&cnt[keys[e]], 1);
}

// CSR columns and clipped values from the sorted runs.
__global__ void k_runs_to_csr(const uint2* __restrict__ vals, int64_t m, float lo, float hi,
                              uint32_t* __restrict__ idx, float* __restrict__ w) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m) return;
  float v = __uint_as_float(vals[e].y);
  if (v < lo)
    v = lo;
  else if (v > hi)
    v = hi;
  idx[e] = vals[e].x;
  w[e] = v;
}

// ---------------------------------------------------------------------------
// Data reduction: block per part, thread per feature column.
// ---------------------------------------------------------------------------
// Block (part, 128 feature columns); thread per column. The sum over the
// part's nodes stays serial in node order. Node ids come through shared
// memory 128 at a time, and each thread issues the loads of the next 16
// nodes before their adds, so a large part is not one long chain of
// dependent loads.
constexpr int RD_THREADS = 128;
__global__ void __launch_bounds__(RD_THREADS) k_reduce_data(
    const float* __restrict__ x, int64_t d, const int64_t* __restrict__ poff,
    const uint2* __restrict__ nodes, const float* __restrict__ rv, float* __restrict__ out) {
  constexpr int U = 16;
  __shared__ uint32_t ids[RD_THREADS];
  const int64_t P = blockIdx.x;
  const int64_t k = (int64_t)blockIdx.y * RD_THREADS + threadIdx.x;
  const bool on = k < d;
  const float v = rv[P];
  const int64_t a = poff[P], b = poff[P + 1];
  float acc = 0.0f;
  for (int64_t c = a; c < b; c += RD_THREADS) {
    const int cnt = (int)min((int64_t)RD_THREADS, b - c);
    __syncthreads();  // the previous chunk's ids are read
    if ((int)threadIdx.x < cnt) ids[threadIdx.x] = nodes[c + threadIdx.x].x;
    __syncthreads();
    if (on) {
      int q = 0;
      for (; q + U <= cnt; q += U) {
        float xv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) xv[u] = __ldg(x + (int64_t)ids[q + u] * d + k);
#pragma unroll
        for (int u = 0; u < U; ++u) acc = fadd(acc, fmul(v, xv[u]));
      }
      for (; q < cnt; ++q) acc = fadd(acc, fmul(v, __ldg(x + (int64_t)ids[q] * d + k)));
    }
  }
  if (on) out[P * d + k] = acc;
}

// ---------------------------------------------------------------------------
// Expansion.
// ---------------------------------------------------------------------------
// Products of the symmetric part G o G^T (rows merged with the transpose's,
// both sorted) times N: key Q = part(j), value (i, s_ij * inv_Q), in
// row-major order. With `same` the transpose is G itself (canonical graphs).
__global__ void k_sym_count(const int64_t* __restrict__ ap, const uint32_t* __restrict__ ai,
                            const int64_t* __restrict__ bp, const uint32_t* __restrict__ bi,
                            int64_t n, int32_t* __restrict__ cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t p = ap[i], q = bp[i];
  const int64_t ep = ap[i + 1], eq = bp[i + 1];
  int32_t c = 0;
  while (p < ep && q < eq) {
    if (ai[p] == bi[q]) {
      ++c;
      ++p;
      ++q;
    } else if (ai[p] < bi[q]) {
      ++p;
    } else {
      ++q;
    }
  }
  cnt[i] = c;
}

__global__ void k_sym_products(const int64_t* __restrict__ ap, const uint32_t* __restrict__ ai,
                               const float* __restrict__ aw, const int64_t* __restrict__ bp,
                               const uint32_t* __restrict__ bi, const float* __restrict__ bw,
                               int64_t n, const int64_t* __restrict__ off,
                               const uint32_t* __restrict__ part, const float* __restrict__ inv,
                               uint32_t* __restrict__ keys, uint2* __restrict__ vals) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t p = ap[i], q = bp[i], o = off[i];
  const int64_t ep = ap[i + 1], eq = bp[i + 1];
  while (p < ep && q < eq) {
    if (ai[p] == bi[q]) {
      const uint32_t j = ai[p];
      const float sv = fmul(aw[p], bw[q]);  // sparse.rs:378-417
      const uint32_t Q = part[j];
      keys[o] = Q;
      vals[o] = make_uint2((uint32_t)i, __float_as_uint(fmul(sv, inv[Q])));
      ++o;
      ++p;
      ++q;
    } else if (ai[p] < bi[q]) {
      ++p;
    } else {
      ++q;
    }
  }
}

// Row i of the expander (runs (i, Q, e) sorted by (i, Q)), L1-normalised, times
// the coarse layout, plus the direct term, halved: res[i][k].
__global__ void k_expand_rows(const int64_t* __restrict__ eptr, const uint2* __restrict__ ev,
                              int64_t n, int32_t dim, const float* __restrict__ layout,
                              const uint32_t* __restrict__ part, const float* __restrict__ u,
                              float* __restrict__ res) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t a = eptr[i], b = eptr[i + 1];
  float nrm = 0.0f;
  for (int64_t e = a; e < b; ++e) nrm = fadd(nrm, fabsf(__uint_as_float(ev[e].y)));
  const float sc = nrm > 0.0f ? fdiv(1.0f, nrm) : 1.0f;
  const bool scale = nrm > 0.0f;
  const uint32_t P = part[i];
  const float dv = u[P];
  for (int32_t k = 0; k < dim; ++k) {
    float acc = 0.0f;
    for (int64_t e = a; e < b; ++e) {
      const float v = scale ? fmul(__uint_as_float(ev[e].y), sc) : __uint_as_float(ev[e].y);
      acc = fadd(acc, fmul(v, layout[(int64_t)ev[e].x * dim + k]));
    }
    const float direct = fadd(0.0f, fmul(dv, layout[(int64_t)P * dim + k]));
    res[i * dim + k] = fmul(fadd(acc, direct), 0.5f);
  }
}

// Runs keyed by row i carry (Q, e) in vals; the row index of run e is keys[e].
// Column centring (serial column sums over all rows), then scaling.
// One block: the rows stream through shared memory in chunks of
// COLMEAN_FLOATS values (double buffered, all threads loading) while thread
// j < dim adds column j's values serially in row order, the next eight values
// read while the current eight are added.
constexpr int COLMEAN_THREADS = 1024;
constexpr int COLMEAN_FLOATS = 5120;  // per chunk: 5120 / dim rows
__global__ void __launch_bounds__(COLMEAN_THREADS) k_col_mean(const float* __restrict__ res,
                                                             int64_t n, int32_t dim, float inv_n,
                                                             float* __restrict__ mean) {
  __shared__ float buf[2][COLMEAN_FLOATS];
  const int j = threadIdx.x;
  const int64_t rows_per = COLMEAN_FLOATS / dim;
  const int64_t nch = (n + rows_per - 1) / rows_per;
  auto load = [&](int64_t c, int b) {
    const int64_t r0 = c * rows_per;
    const int64_t cnt = min(rows_per, n - r0) * dim;
    for (int64_t q = j; q < cnt; q += COLMEAN_THREADS) buf[b][q] = __ldg(res + r0 * dim + q);
  };
  float s = 0.0f;
  if (nch > 0) load(0, 0);
  __syncthreads();
  for (int64_t c = 0; c < nch; ++c) {
    const int b = (int)(c & 1);
    if (c + 1 < nch) load(c + 1, b ^ 1);  // the next chunk loads during this one's adds
    if (j < dim) {
      const float* col = buf[b] + j;
      const int rows = (int)min(rows_per, n - c * rows_per);
      int r = 0;
      if (rows >= 8) {
        float t[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) t[u] = col[u * dim];
        for (r = 8; r + 8 <= rows; r += 8) {
          float nx[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) nx[u] = col[(r + u) * dim];
#pragma unroll
          for (int u = 0; u < 8; ++u) s = fadd(s, t[u]);
#pragma unroll
          for (int u = 0; u < 8; ++u) t[u] = nx[u];
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) s = fadd(s, t[u]);  // rows r - 8 .. r - 1
      }
      for (; r < rows; ++r) s = fadd(s, col[r * dim]);
    }
    __syncthreads();
  }
  if (j < dim) mean[j] = fmul(s, inv_n);
}

__global__ void k_center_scale(float* __restrict__ res, int64_t n, int32_t dim,
                               const float* __restrict__ mean, float scale) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n * dim) return;
  const int32_t j = (int32_t)(q % dim);
  res[q] = fmul(scale, fsub(res[q], mean[j]));
}

// Random init of the base case (label_prop.rs:338-360): uniform in [-1, 1],
// rows L2-normalised in double. Philox counter (q_lo, q_hi, "LP", "RINI").
__global__ void k_lp_random_init(float* __restrict__ out, int64_t n, int32_t dim, uint64_t seed) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float r[32];
  double nrm = 0.0;
  for (int32_t j = 0; j < dim; ++j) {
    const uint64_t q = (uint64_t)i * dim + j;
    const uint4 o = philox4x32_10(make_uint4((uint32_t)q, (uint32_t)(q >> 32), 0x4C50u, 0x52494E49u),
                                  make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
    const double uu = (double)((((uint64_t)o.y << 32) | o.x) >> 11) * (1.0 / 9007199254740992.0);
    r[j] = (float)__dsub_rn(__dmul_rn(uu, 2.0), 1.0);
    nrm = __dadd_rn(nrm, __dmul_rn((double)r[j], (double)r[j]));
  }
  nrm = __dsqrt_rn(nrm);
  for (int32_t j = 0; j < dim; ++j)
    out[i * dim + j] = nrm > 0.0 ? (float)__ddiv_rn((double)r[j], nrm) : r[j];
}

// ---------------------------------------------------------------------------
// Host: the PCA base case (double, Jacobi eigen-solve of the Gram matrix).
// ---------------------------------------------------------------------------
void host_unit_range(std::vector<float>& m, int64_t n, int64_t d) {
  for (int64_t j = 0; j < d; ++j) {
    float lo = INFINITY, hi = -INFINITY;
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

void host_jacobi(std::vector<double>& a, int64_t k, std::vector<double>& w,
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
        const double t =
            (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int64_t r = 0; r < k; ++r) {
          const double ap = a[r * k + p], aq = a[r * k + q];
          a[r * k + p] = c * ap - sn * aq;
          a[r * k + q] = sn * ap + c * aq;
        }
        for (int64_t r = 0; r < k; ++r) {
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

// Principal components of n points in d dims (n small): the top k = min(dim,
// n, d) eigenvectors of the centred Gram matrix, scaled by sqrt(eigenvalue),
// each signed so its largest-magnitude entry is positive, then unit-range
// normalised per column; columns beyond k are zero.
std::vector<float> host_pca_init(const std::vector<float>& data, int64_t n, int64_t d,
                                 int64_t dim) {
  const int64_t k = std::min(std::min(dim, n), d);
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
  host_jacobi(g, n, w, v);
  std::vector<int64_t> order((size_t)n);
  for (int64_t i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return w[a] > w[b]; });
  std::vector<float> pc((size_t)(n * k));
  for (int64_t c = 0; c < k; ++c) {
    const int64_t e = order[c];
    const double sig = std::sqrt(std::max(w[e], 0.0));
    int64_t big = 0;
    for (int64_t i = 1; i < n; ++i)
      if (std::fabs(v[i * n + e]) > std::fabs(v[big * n + e])) big = i;
    const double sgn = v[big * n + e] < 0 ? -1.0 : 1.0;
    for (int64_t i = 0; i < n; ++i) pc[i * k + c] = (float)(sgn * v[i * n + e] * sig);
  }
  host_unit_range(pc, n, k);
  std::vector<float> out((size_t)(n * dim), 0.0f);
  for (int64_t i = 0; i < n; ++i)
    for (int64_t c = 0; c < k; ++c) out[i * dim + c] = pc[i * k + c];
  return out;
}

struct LpParams {
  int32_t n_lp_iter = 20;
  int64_t base_thr = 64;
  double scaling = 0.1;
};

// One level of label_prop_init_inner on graph g (device), data (device n x d
// or null): writes the n x dim initial embedding into d_out (device).
void lp_init_inner(evoc_ctx* ctx, const evoc_graph* g, int32_t dim, const float* d_data,
                   int64_t d, int32_t n_emb_epochs, int64_t approx_parts, uint64_t seed,
                   const LpParams& lp, float* d_out) {
  cudaStream_t s = ctx->stream;
  const int64_t n = g->n;
  if (n < lp.base_thr) {  // label_prop.rs:440-445
    if (d_data && dim <= d) {
      std::vector<float> x((size_t)(n * d));
      EVOC_CUDA(cudaMemcpyAsync(x.data(), d_data, x.size() * sizeof(float),
                                cudaMemcpyDeviceToHost, s));
      EVOC_CUDA(cudaStreamSynchronize(s));
      const std::vector<float> pc = host_pca_init(x, n, d, dim);
      EVOC_CUDA(cudaMemcpyAsync(d_out, pc.data(), pc.size() * sizeof(float),
                                cudaMemcpyHostToDevice, s));
      EVOC_CUDA(cudaStreamSynchronize(s));
    } else if (n > 0) {
      k_lp_random_init<<<grid_of(n), 128, 0, s>>>(d_out, n, dim, seed);
      EVOC_CHECK_LAUNCH();
    }
    return;
  }
  // stage trace (EVOC_TRACE=1): one block per level, innermost level first
  StageTrace tr(s);
  const std::string lvl = "lp n=" + std::to_string(n) + ": ";
  auto mark = [&](const char* what) {
    if (tr.on) tr.mark((lvl + what).c_str());
  };
  // 1. partition (label_prop.rs:448)
  DevBuf<uint32_t> part(n, s);
  const int64_t np = label_prop_partition(ctx, g, approx_parts, lp.n_lp_iter, seed, part.get());
  mark("partition");
  if (np <= 0) throw Error(EVOC_ERR_INTERNAL, "label propagation produced no parts");
  // 2. per-part constants and node lists
  DevBuf<int32_t> cnt(np, s);
  EVOC_CUDA(cudaMemsetAsync(cnt.get(), 0, np * sizeof(int32_t), s));
  k_part_count<<<grid_of(n), 256, 0, s>>>(part.get(), n, cnt.get());
  EVOC_CHECK_LAUNCH();
  DevBuf<float> inv(np, s), rv(np, s), u(np, s);
  k_part_consts<<<grid_of(np, 128), 128, 0, s>>>(cnt.get(), np, inv.get(), rv.get(), u.get());
  EVOC_CHECK_LAUNCH();
  const int pbits = bits_for((uint64_t)std::max<int64_t>(np - 1, 1));
  const int nbits = bits_for((uint64_t)std::max<int64_t>(n - 1, 1));
  // 3. coarse graph clip(N^T G B)
  evoc_graph coarse;
  coarse.ctx = ctx;
  coarse.n = np;
  coarse.canonical = false;
  coarse.indptr.alloc(np + 1, s);
  {
    const int64_t m = g->nnz;
    DevBuf<uint32_t> keys(std::max<int64_t>(m, 1), s);
    DevBuf<uint2> vals(std::max<int64_t>(m, 1), s);
    int64_t runs = 0;
    if (m > 0) {
      k_gen_products<<<grid_of(n * 32), 256, 0, s>>>(g->indptr.get(), g->indices.get(),
                                                     g->weights.get(), n, part.get(), inv.get(),
                                                     keys.get(), vals.get());
      EVOC_CHECK_LAUNCH();
      // keys j, vals (P, prod): order (P, j, i) -> runs (P, (j, A_Pj))
      k_swap_keys<<<grid_of(m), 256, 0, s>>>(keys.get(), vals.get(), m);  // keys P, vals (j, .)
      EVOC_CHECK_LAUNCH();
      runs = sort_and_sum(keys.get(), vals.get(), m, pbits, nbits, s);
      // (P, (j, a)) -> (P, Q = part(j), j order kept) -> runs (P, (Q, sum))
      DevBuf<uint32_t> q(runs, s);
      k_map_keys<<<grid_of(runs), 256, 0, s>>>(q.get(), vals.get(), runs, part.get());
      EVOC_CHECK_LAUNCH();
      // order (P, j) -> (P, Q, j): stable sort by Q, then by P
      {
        k_swap_keys<<<grid_of(runs), 256, 0, s>>>(keys.get(), vals.get(), runs);  // keys j, vals (P, a)
        EVOC_CHECK_LAUNCH();
        EVOC_CUDA(cudaMemcpyAsync(keys.get(), q.get(), runs * sizeof(uint32_t),
                                  cudaMemcpyDeviceToDevice, s));  // keys Q
        radix_sort_pairs(keys.get(), vals.get(), runs, pbits, s);
        k_swap_keys<<<grid_of(runs), 256, 0, s>>>(keys.get(), vals.get(), runs);  // keys P, vals (Q, a)
        EVOC_CHECK_LAUNCH();
        radix_sort_pairs(keys.get(), vals.get(), runs, pbits, s);
        DevBuf<int32_t> head(runs, s);
        DevBuf<int64_t> rid(runs + 1, s);
        k_run_heads<<<grid_of(runs), 256, 0, s>>>(keys.get(), vals.get(), runs, head.get());
        EVOC_CHECK_LAUNCH();
        exclusive_scan_i32_to_i64(head.get(), rid.get(), runs, s);
        int64_t r2 = 0;
        EVOC_CUDA(cudaMemcpyAsync(&r2, rid.get() + runs, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        EVOC_CUDA(cudaStreamSynchronize(s));
        DevBuf<uint32_t> ok(r2, s);
        DevBuf<uint2> ov(r2, s);
        k_run_sums<<<grid_of(runs), 256, 0, s>>>(keys.get(), vals.get(), runs, head.get(),
                                                 rid.get(), ok.get(), ov.get());
        EVOC_CHECK_LAUNCH();
        runs = r2;
        DevBuf<int32_t> rc(np, s);
        EVOC_CUDA(cudaMemsetAsync(rc.get(), 0, np * sizeof(int32_t), s));
        k_row_hist<<<grid_of(runs), 256, 0, s>>>(ok.get(), runs, rc.get());
        EVOC_CHECK_LAUNCH();
        exclusive_scan_i32_to_i64(rc.get(), coarse.indptr.get(), np, s);
        coarse.nnz = runs;
        coarse.indices.alloc(std::max<int64_t>(runs, 1), s);
        coarse.weights.alloc(std::max<int64_t>(runs, 1), s);
        k_runs_to_csr<<<grid_of(runs), 256, 0, s>>>(ov.get(), runs, 0.0f, 1.0f,
                                                    coarse.indices.get(), coarse.weights.get());
        EVOC_CHECK_LAUNCH();
        EVOC_CUDA(cudaStreamSynchronize(s));
      }
    } else {
      EVOC_CUDA(cudaMemsetAsync(coarse.indptr.get(), 0, (np + 1) * sizeof(int64_t), s));
      coarse.nnz = 0;
    }
  }
  mark("coarse graph");
  // 4. coarse data: per part, its nodes in order (stable sort of node ids by part)
  DevBuf<float> cdata;
  if (d_data) {
    DevBuf<uint32_t> pk(n, s);
    DevBuf<uint2> nodes(n, s);
    EVOC_CUDA(cudaMemcpyAsync(pk.get(), part.get(), n * sizeof(uint32_t),
                              cudaMemcpyDeviceToDevice, s));
    k_iota_pairs<<<grid_of(n), 256, 0, s>>>(nodes.get(), n);
    EVOC_CHECK_LAUNCH();
    radix_sort_pairs(pk.get(), nodes.get(), n, pbits, s);
    DevBuf<int64_t> poff(np + 1, s);
    exclusive_scan_i32_to_i64(cnt.get(), poff.get(), np, s);
    cdata.alloc(np * d, s);
    k_reduce_data<<<dim3((unsigned)np, (unsigned)((d + RD_THREADS - 1) / RD_THREADS)),
                    RD_THREADS, 0, s>>>(d_data, d, poff.get(), nodes.get(), rv.get(),
                                        cdata.get());
    EVOC_CHECK_LAUNCH();
  }
  mark("coarse data");
  // 5. recursion
  const int32_t e = std::min(n_emb_epochs, 255);
  DevBuf<float> cinit(np * dim, s), layout(np * dim, s);
  lp_init_inner(ctx, &coarse, dim, d_data ? cdata.get() : nullptr, d, e, approx_parts / 4,
                seed + 3000, lp, cinit.get());
  mark("coarser levels");
  // 6. short embedding of the coarse graph (label_prop.rs:486-498)
  {
    evoc_embed_params_t ep;
    evoc_embed_params_default(&ep);
    ep.n_epochs = e;
    ep.initial_alpha = (float)(0.001 * (double)e);
    std::vector<ProblemDesc> probs{ProblemDesc{&coarse, seed + 4000}};
    evoc_plan* pl = plan_create(ctx, probs, dim, ep);
    try {
      plan_run_device(pl, cinit.get(), layout.get());
    } catch (...) {
      plan_free(pl);
      throw;
    }
    EVOC_CUDA(cudaStreamSynchronize(s));
    plan_free(pl);
  }
  mark("coarse embedding");
  // 7. expansion (label_prop.rs:500-534)
  {
    // the transpose of g (rows of G^T, entries in row order)
    DevBuf<int64_t> tptr;
    DevBuf<uint32_t> tidx;
    DevBuf<float> tw;
    const int64_t *bp = g->indptr.get();
    const uint32_t* bi = g->indices.get();
    const float* bw = g->weights.get();
    if (!g->canonical && g->nnz > 0) {
      const int64_t m = g->nnz;
      DevBuf<uint32_t> tk(m, s);
      DevBuf<uint2> tv(m, s);
      k_transpose_gen<<<grid_of(n * 32), 256, 0, s>>>(g->indptr.get(), g->indices.get(),
                                                      g->weights.get(), n, tk.get(), tv.get());
      EVOC_CHECK_LAUNCH();
      radix_sort_pairs(tk.get(), tv.get(), m, nbits, s);
      DevBuf<int32_t> tc(n, s);
      EVOC_CUDA(cudaMemsetAsync(tc.get(), 0, n * sizeof(int32_t), s));
      k_row_hist<<<grid_of(m), 256, 0, s>>>(tk.get(), m, tc.get());
      EVOC_CHECK_LAUNCH();
      tptr.alloc(n + 1, s);
      exclusive_scan_i32_to_i64(tc.get(), tptr.get(), n, s);
      tidx.alloc(m, s);
      tw.alloc(m, s);
      k_unpack_pairs<<<grid_of(m), 256, 0, s>>>(tv.get(), m, tidx.get(), tw.get());
      EVOC_CHECK_LAUNCH();
      bp = tptr.get();
      bi = tidx.get();
      bw = tw.get();
    }
    mark("expansion: transpose");
    DevBuf<int32_t> sc(n, s);
    DevBuf<int64_t> soff(n + 1, s);
    k_sym_count<<<grid_of(n), 256, 0, s>>>(g->indptr.get(), g->indices.get(), bp, bi, n,
                                           sc.get());
    EVOC_CHECK_LAUNCH();
    exclusive_scan_i32_to_i64(sc.get(), soff.get(), n, s);
    int64_t ms = 0;
    EVOC_CUDA(cudaMemcpyAsync(&ms, soff.get() + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaStreamSynchronize(s));
    DevBuf<uint32_t> keys(std::max<int64_t>(ms, 1), s);
    DevBuf<uint2> vals(std::max<int64_t>(ms, 1), s);
    DevBuf<int64_t> eptr(n + 1, s);
    int64_t runs = 0;
    if (ms > 0) {
      k_sym_products<<<grid_of(n), 256, 0, s>>>(g->indptr.get(), g->indices.get(),
                                                g->weights.get(), bp, bi, bw, n, soff.get(),
                                                part.get(), inv.get(), keys.get(), vals.get());
      EVOC_CHECK_LAUNCH();
      // keys Q, vals (i, prod): order (i, Q, j) -> runs (i, (Q, e))
      k_swap_keys<<<grid_of(ms), 256, 0, s>>>(keys.get(), vals.get(), ms);  // keys i, vals (Q, .)
      EVOC_CHECK_LAUNCH();
      mark("expansion: symmetric products");
      runs = sort_and_sum(keys.get(), vals.get(), ms, nbits, pbits, s);
    }
    mark("expansion: sort and sum");
    DevBuf<int32_t> rc(n, s);
    EVOC_CUDA(cudaMemsetAsync(rc.get(), 0, n * sizeof(int32_t), s));
    if (runs > 0) {
      k_row_hist<<<grid_of(runs), 256, 0, s>>>(keys.get(), runs, rc.get());
      EVOC_CHECK_LAUNCH();
    }
    exclusive_scan_i32_to_i64(rc.get(), eptr.get(), n, s);
    k_expand_rows<<<grid_of(n, 128), 128, 0, s>>>(eptr.get(), vals.get(), n, dim, layout.get(),
                                                  part.get(), u.get(), d_out);
    EVOC_CHECK_LAUNCH();
    mark("expansion: rows");
    DevBuf<float> mean(dim, s);
    const float inv_n = (float)(1.0 / (double)n);
    k_col_mean<<<1, COLMEAN_THREADS, 0, s>>>(d_out, n, dim, inv_n, mean.get());
    EVOC_CHECK_LAUNCH();
    k_center_scale<<<grid_of(n * dim), 256, 0, s>>>(d_out, n, dim, mean.get(),
                                                    (float)lp.scaling);
    EVOC_CHECK_LAUNCH();
    EVOC_CUDA(cudaStreamSynchronize(s));
  }
  mark("expansion: centring");
}

}  // namespace

void label_propagation_init_device(evoc_ctx* ctx, const evoc_graph* g, int32_t dim,
                                   const float* d_data, int64_t d, uint64_t seed, float* d_out) {
  if (dim < 1 || dim > 16) throw Error(EVOC_ERR_UNSUPPORTED, "dim must be in 1..16");
  const int64_t n = g->n;
  if (n <= 0) throw Error(EVOC_ERR_INVALID_ARGUMENT, "empty graph");
  if (d_data && d <= 0) throw Error(EVOC_ERR_INVALID_ARGUMENT, "data dimension must be > 0");
  // label_prop.rs:555-560: approx parts = clamp(8 sqrt(n), 256, 16384), at most n
  const int64_t parts = std::min<int64_t>(
      std::min<int64_t>(std::max<int64_t>((int64_t)(8.0 * std::sqrt((double)n)), 256), 16384), n);
  LpParams lp;
  lp_init_inner(ctx, g, dim, d_data, d, 50, parts, seed, lp, d_out);
}

}  // namespace evoc
