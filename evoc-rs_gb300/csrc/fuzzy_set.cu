// fuzzy_set.cu — fuzzy simplicial set on the GPU.
//
// Replaces, in evoc-rs 0.2.7:
//   smooth_knn_dist            src/graph/fuzzy_graph.rs:33-98
//   knn_to_coo                 src/graph/fuzzy_graph.rs:114-159
//   symmetrise_graph           src/graph/fuzzy_graph.rs:174-228
//   coo_to_adjacency_list      src/graph/fuzzy_graph.rs:242-256
//   build_fuzzy_simplicial_set src/graph/fuzzy_graph.rs:275-295
//
// Pipeline (all on the context stream):
//   k_knn_rowlen     warp per row: row length (first EVOC_KNN_PAD) and index
//                    validation.
//   k_smooth_knn     lane per row (a pool of rows per warp, a finished lane
//                    takes the next): rho and the sigma bisection with the
//                    rows' distances staged in shared memory. The sum over the
//                    row is serial in row order, as in the reference
//                    (fuzzy_graph.rs:72-76), so sigma is bit-identical to a
//                    serial CPU evaluation.
//   k_knn_weights    elementwise membership weights (fuzzy_graph.rs:138-145).
//   k_forward_rows   thread per row: drop self loops, sort by column keeping
//                    the last of equal columns (HashMap::insert overwrites,
//                    fuzzy_graph.rs:189), count in-degrees.
//   radix sort       stable sort of the forward entries by column: each
//                    column bucket lists its source rows in ascending order,
//                    which is the backward map of fuzzy_graph.rs:190.
//   k_union          thread per row: merge the sorted forward and backward
//                    lists, w = w_ij + w_ji - w_ij * w_ji, keep w > 0
//                    (fuzzy_graph.rs:196-204); once to count, once to write.
#include "evoc_device.cuh"
#include "evoc_internal.h"

#include <algorithm>
#include <cmath>

namespace evoc {
namespace {

constexpr uint32_t PAD = EVOC_KNN_PAD;

// ---------------------------------------------------------------------------
// Row lengths and index validation (warp per row, coalesced).
// ---------------------------------------------------------------------------
__global__ void k_knn_rowlen(const uint32_t* __restrict__ idx, int64_t n,
                             int32_t k, int32_t* __restrict__ row_len,
                             int32_t* __restrict__ status) {
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const uint32_t* r = idx + row * (int64_t)k;
  int32_t len = k;
  for (int32_t base = 0; base < k; base += 32) {
    const int32_t j = base + lane;
    const uint32_t c = (j < k) ? r[j] : PAD;
    const uint32_t pads = __ballot_sync(0xffffffffu, j < k && c == PAD);
    if (pads) {
      const int32_t first = base + __ffs(pads) - 1;
      if (j < first && (int64_t)c >= n) set_status(status, ST_BAD_INDEX);
      len = first;
      break;
    }
    if (j < k && (int64_t)c >= n) set_status(status, ST_BAD_INDEX);
  }
  if (lane == 0) row_len[row] = len;
}

// ---------------------------------------------------------------------------
// smooth_knn_dist (fuzzy_graph.rs:33-98): rho and the sigma bisection, one
// row per lane at a time. The sum over the row stays serial in row order, so
// sigma is bit-identical to a serial CPU evaluation. Rows need different
// numbers of bisection steps (a handful up to n_iter), so instead of one row
// per lane for the whole launch, each warp owns a pool of rows staged in
// shared memory (odd row stride: lanes on different rows hit different banks)
// and a lane that finishes its row takes the pool's next one at the end of
// the step; the warp runs about the mean step count of its rows rather than
// their maximum. The membership weights are a separate elementwise pass.
// ---------------------------------------------------------------------------
constexpr int SK_WARPS = 4;

struct RowState {
  int32_t row;   // pool slot, or >= pool size when the lane is done
  int32_t len;
  int32_t it;
  float rho, lo, hi, mid;
};

__device__ __forceinline__ void sk_start_row(RowState& st, const float* __restrict__ d,
                                             int32_t len, float lc, int32_t* __restrict__ status,
                                             bool& ok) {
  st.len = len;
  st.it = 0;
  st.lo = 0.0f;
  st.hi = 3.40282347e+38f;
  st.mid = 1.0f;
  ok = true;
  for (int32_t j = 0; j < len; ++j)
    if (d[j] != d[j]) ok = false;
  if (!ok) set_status(status, ST_BAD_VALUE);
  float rho = 0.0f;
  if (lc > 0.0f) {  // fuzzy_graph.rs:49-62
    if (len <= 0) {
      set_status(status, ST_EMPTY_ROW);
      ok = false;
    } else {
      const float lm1 = max0(fsub(lc, 1.0f));
      const float fl = floorf(lm1);
      int64_t id = (int64_t)fl;
      if (id > len - 1) id = len - 1;
      const float frac = fsub(lm1, fl);
      if (frac > 0.0f && id + 1 < len)
        rho = fadd(fmul(d[id], fsub(1.0f, frac)), fmul(d[id + 1], frac));
      else
        rho = d[id];
    }
  }
  st.rho = rho;
}

__global__ void __launch_bounds__(32 * SK_WARPS) k_smooth_knn(
    const float* __restrict__ dist, const int32_t* __restrict__ row_len, int64_t n, int32_t k,
    int32_t kp, int32_t pool, double target, float lc, int32_t n_iter,
    float* __restrict__ sigma_out, float* __restrict__ rho_out, int32_t* __restrict__ status,
    unsigned long long* __restrict__ steps) {
  extern __shared__ float sm[];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float* sd = sm + (size_t)wid * pool * kp;
  const int64_t row0 = ((int64_t)blockIdx.x * SK_WARPS + wid) * pool;
  if (row0 >= n) return;  // whole warp
  const int rows = (int)min((int64_t)pool, n - row0);
  {
    const float* src = dist + row0 * (int64_t)k;
    const int64_t elems = (int64_t)rows * k;
    for (int64_t e = lane; e < elems; e += 32) {
      const int64_t r = e / k;
      sd[r * kp + (e - r * k)] = src[e];
    }
  }
  __syncwarp();
  const uint32_t lt = (1u << lane) - 1u;
  RowState st;
  bool ok = false;
  st.row = lane;
  int next = 32;  // the pool's next unstarted row (warp-uniform)
  uint32_t nsteps = 0;  // row sums evaluated by this lane
  if (st.row < rows) {
    sk_start_row(st, sd + st.row * kp, row_len ? row_len[row0 + st.row] : k, lc, status, ok);
  }
  for (;;) {
    const bool active = st.row < rows;
    if (__ballot_sync(FULL, active) == 0) break;
    bool done = false;
    if (active) {
      if (!ok) {
        st.mid = 0.0f;
        st.rho = 0.0f;
        done = true;
      } else if (st.it >= n_iter) {
        done = true;
      } else {  // one bisection step, fuzzy_graph.rs:71-93
        const float* d = sd + st.row * kp;
        ++nsteps;
        float val = 0.0f;
        for (int32_t j = 0; j < st.len; ++j) {
          const float adjusted = max0(fsub(d[j], st.rho));
          val = fadd(val, evoc_expf(-fdiv(adjusted, st.mid)));
        }
        const double vd = (double)val;
        if (fabs(vd - target) < 1e-5) {
          done = true;
        } else {
          if (vd > target) {
            st.hi = st.mid;
            st.mid = fdiv(fadd(st.lo, st.hi), 2.0f);
          } else {
            st.lo = st.mid;
            if (st.hi == 3.40282347e+38f)
              st.mid = fmul(st.mid, 2.0f);
            else
              st.mid = fdiv(fadd(st.lo, st.hi), 2.0f);
          }
          ++st.it;
        }
      }
      if (done) {
        sigma_out[row0 + st.row] = st.mid;
        rho_out[row0 + st.row] = st.rho;
      }
    }
    // lanes whose row is done take the pool's next rows, in lane order
    const uint32_t need = __ballot_sync(FULL, done);
    if (done) {
      st.row = next + __popc(need & lt);
      if (st.row < rows)
        sk_start_row(st, sd + st.row * kp, row_len ? row_len[row0 + st.row] : k, lc, status, ok);
    }
    next += __popc(need);
  }
  const unsigned tot = __reduce_add_sync(FULL, nsteps);
  if (lane == 0 && tot) atomicAdd(steps, (unsigned long long)tot);
}

// knn_to_coo's membership weights (fuzzy_graph.rs:138-145), elementwise:
// w = exp(-max(0, d - rho) / sigma), or 0 / 1 when sigma <= 0.
__global__ void k_knn_weights(const float* __restrict__ dist, const int32_t* __restrict__ row_len,
                              int64_t n, int32_t k, const float* __restrict__ sigma,
                              const float* __restrict__ rho, float* __restrict__ w) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * (int64_t)k) return;
  const int64_t i = e / k;
  const int32_t j = (int32_t)(e - i * k);
  const int32_t len = row_len ? row_len[i] : k;
  float out = 0.0f;
  if (j < len) {
    const float mid = sigma[i];
    const float adjusted = max0(fsub(dist[e], rho[i]));
    if (mid > 0.0f)
      out = evoc_expf(-fdiv(adjusted, mid));
    else
      out = (adjusted > 0.0f) ? 0.0f : 1.0f;
  }
  w[e] = out;
}

// ---------------------------------------------------------------------------
// Forward lists: drop self loops, stable insertion sort by column, keep the
// last entry of each column, count in-degrees. Rows stay padded to k.
// ---------------------------------------------------------------------------
__global__ void k_forward_rows(const uint32_t* __restrict__ idx,
                               const float* __restrict__ w,
                               const int32_t* __restrict__ row_len, int64_t n,
                               int32_t k, int32_t kp,
                               uint32_t* __restrict__ fcol,
                               float* __restrict__ fw,
                               int32_t* __restrict__ fcnt,
                               int32_t* __restrict__ indeg) {
  extern __shared__ uint32_t smu[];
  const int R = blockDim.x;
  uint32_t* sc = smu;
  float* sw = reinterpret_cast<float*>(smu + (size_t)R * kp);
  const int64_t row0 = (int64_t)blockIdx.x * R;
  const int64_t rows_here = min((int64_t)R, n - row0);
  const int64_t elems = rows_here * k;
  for (int64_t e = threadIdx.x; e < elems; e += R) {
    const int64_t r = e / k, j = e - r * k;
    sc[r * kp + j] = idx[row0 * (int64_t)k + e];
    sw[r * kp + j] = w[row0 * (int64_t)k + e];
  }
  __syncthreads();
  if (threadIdx.x < rows_here) {
    const int64_t i = row0 + threadIdx.x;
    uint32_t* c = sc + threadIdx.x * kp;
    float* ww = sw + threadIdx.x * kp;
    const int32_t len = row_len[i];
    int32_t m = 0;  // compact: drop self loops (fuzzy_graph.rs:135)
    for (int32_t j = 0; j < len; ++j)
      if ((int64_t)c[j] != i) {
        c[m] = c[j];
        ww[m] = ww[j];
        ++m;
      }
    for (int32_t j = 1; j < m; ++j) {  // stable insertion sort by column
      const uint32_t cj = c[j];
      const float wj = ww[j];
      int32_t q = j - 1;
      while (q >= 0 && c[q] > cj) {
        c[q + 1] = c[q];
        ww[q + 1] = ww[q];
        --q;
      }
      c[q + 1] = cj;
      ww[q + 1] = wj;
    }
    int32_t cnt = 0;  // keep the last of each run of equal columns
    for (int32_t j = 0; j < m; ++j)
      if (j + 1 == m || c[j + 1] != c[j]) {
        c[cnt] = c[j];
        ww[cnt] = ww[j];
        ++cnt;
      }
    fcnt[i] = cnt;
    for (int32_t j = 0; j < cnt; ++j) atomicAdd(&indeg[c[j]], 1);
    for (int32_t j = cnt; j < k; ++j) c[j] = PAD;
  }
  __syncthreads();
  for (int64_t e = threadIdx.x; e < elems; e += R) {
    const int64_t r = e / k, j = e - r * k;
    fcol[row0 * (int64_t)k + e] = sc[r * kp + j];
    fw[row0 * (int64_t)k + e] = sw[r * kp + j];
  }
}

// Compact the padded forward lists into (column key, (row, weight)) pairs in
// row-major order: the input of the stable transpose.
__global__ void k_forward_compact(const uint32_t* __restrict__ fcol,
                                  const float* __restrict__ fw,
                                  const int64_t* __restrict__ fptr, int64_t n,
                                  int32_t k, uint32_t* __restrict__ keys,
                                  uint2* __restrict__ vals) {
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const int64_t o = fptr[row];
  const int32_t cnt = (int32_t)(fptr[row + 1] - o);
  for (int32_t j = lane; j < cnt; j += 32) {
    keys[o + j] = fcol[row * (int64_t)k + j];
    vals[o + j] = make_uint2((uint32_t)row, __float_as_uint(fw[row * (int64_t)k + j]));
  }
}

// Fuzzy union of row i (fuzzy_graph.rs:193-205), warp per row: the forward
// list (sorted by column, at most k entries) merged with the backward list
// (sorted by source row). Each step loads the next 32 entries of both lists
// (coalesced); every entry finds its rank in the other chunk by a shuffle
// search, a column present in both is emitted once with both weights, and
// only columns up to the smaller of the two chunks' last entries are final.
// Emitted entries are placed by merged rank in shared memory, then the kept
// ones (w_sym > 0) are written in order. Output goes to the row's scratch
// region at i * k + bptr[i]; out_cnt[i] gets the kept count.
__global__ void __launch_bounds__(256) k_union(const uint32_t* __restrict__ fcol,
                                               const float* __restrict__ fw,
                                               const int32_t* __restrict__ fcnt,
                                               const int64_t* __restrict__ bptr,
                                               const uint2* __restrict__ bvals, int64_t n,
                                               int32_t k, int32_t* __restrict__ out_cnt,
                                               uint2* __restrict__ tmp) {
  __shared__ uint2 stage_all[8][64];
  uint2* stage = stage_all[threadIdx.x >> 5];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= n) return;
  const uint32_t* fa = fcol + i * (int64_t)k;
  const float* fwa = fw + i * (int64_t)k;
  const int32_t na = fcnt[i];
  const int64_t b0 = bptr[i], nb = bptr[i + 1] - b0;
  const uint2* bv = bvals + b0;
  uint2* out = tmp + i * (int64_t)k + b0;
  int32_t ia = 0;
  int64_t ib = 0;
  int32_t cnt = 0;
  while (ia < na || ib < nb) {
    const bool has_a = ia + lane < na, has_b = ib + lane < nb;
    const uint32_t a = has_a ? fa[ia + lane] : PAD;
    const float wa = has_a ? fwa[ia + lane] : 0.0f;
    const uint2 bb = has_b ? bv[ib + lane] : make_uint2(PAD, 0u);
    const uint32_t b = bb.x;
    const int ca = (int)min((int64_t)32, (int64_t)(na - ia));
    const int cb = (int)min((int64_t)32, nb - ib);
    // columns up to `bound` are final: every unread entry is larger
    uint32_t bound = 0xffffffffu;
    if (ia + 32 < na) bound = min(bound, __shfl_sync(FULL, a, 31));
    if (ib + 32 < nb) bound = min(bound, __shfl_sync(FULL, b, 31));
    // rank of a in the b chunk (# b < a) and of b in the a chunk (# a < b)
    int ra = 0, rb = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
      if (__shfl_sync(FULL, b, ra + step - 1) < a) ra += step;
      if (__shfl_sync(FULL, a, rb + step - 1) < b) rb += step;
    }
    if (ra < 32 && __shfl_sync(FULL, b, ra) < a) ++ra;  // lanes past the chunk hold PAD
    if (rb < 32 && __shfl_sync(FULL, a, rb) < b) ++rb;
    const uint32_t b_at = __shfl_sync(FULL, b, ra & 31);
    const uint32_t b_w = __shfl_sync(FULL, bb.y, ra & 31);
    const uint32_t a_at = __shfl_sync(FULL, a, rb & 31);
    const bool a_take = has_a && a <= bound;
    const bool a_match = a_take && ra < cb && b_at == a;
    const bool b_take = has_b && b <= bound;
    const bool b_match = b_take && rb < ca && a_at == b;
    const uint32_t ma = __ballot_sync(FULL, a_match), mb = __ballot_sync(FULL, b_match);
    // merged rank = # distinct columns before this one among the taken entries
    if (a_take) {
      const float w_ji = a_match ? __uint_as_float(b_w) : 0.0f;
      const float w_sym = fsub(fadd(wa, w_ji), fmul(wa, w_ji));
      stage[lane + ra - __popc(ma & lt)] = make_uint2(a, __float_as_uint(w_sym));
    }
    if (b_take && !b_match) {
      const float w_ji = __uint_as_float(bb.y);
      const float w_sym = fsub(fadd(0.0f, w_ji), fmul(0.0f, w_ji));
      stage[lane + rb - __popc(mb & lt)] = make_uint2(b, __float_as_uint(w_sym));
    }
    const int na_t = __popc(__ballot_sync(FULL, a_take));
    const int nb_t = __popc(__ballot_sync(FULL, b_take));
    const int m = na_t + nb_t - __popc(ma);  // distinct columns emitted
    __syncwarp();
    // kept entries (w_sym > 0) in merged order
    for (int base = 0; base < m; base += 32) {
      const int e = base + lane;
      const uint2 v = e < m ? stage[e] : make_uint2(0u, 0u);
      const bool keep = e < m && __uint_as_float(v.y) > 0.0f;
      const uint32_t kb = __ballot_sync(FULL, keep);
      if (keep) out[cnt + __popc(kb & lt)] = v;
      cnt += __popc(kb);
    }
    __syncwarp();
    ia += na_t;
    ib += nb_t;
  }
  if (lane == 0) out_cnt[i] = cnt;
}

// Warp per row: the row's kept pairs from its scratch region into the CSR.
__global__ void k_union_compact(const uint2* __restrict__ tmp,
                                const int64_t* __restrict__ bptr, int64_t n, int32_t k,
                                const int64_t* __restrict__ out_ptr,
                                uint32_t* __restrict__ out_idx, float* __restrict__ out_w) {
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const uint2* src = tmp + i * (int64_t)k + bptr[i];
  const int64_t dst = out_ptr[i], len = out_ptr[i + 1] - dst;
  for (int64_t j = lane; j < len; j += 32) {
    const uint2 v = src[j];
    out_idx[dst + j] = v.x;
    out_w[dst + j] = __uint_as_float(v.y);
  }
}

// symmetrise == false: the directed COO of knn_to_coo in kNN order.
template <bool WRITE>
__global__ void k_directed(const uint32_t* __restrict__ idx,
                           const float* __restrict__ w,
                           const int32_t* __restrict__ row_len, int64_t n,
                           int32_t k, int32_t* __restrict__ out_cnt,
                           const int64_t* __restrict__ out_ptr,
                           uint32_t* __restrict__ out_idx,
                           float* __restrict__ out_w) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t len = row_len[i];
  int64_t o = WRITE ? out_ptr[i] : 0;
  int32_t cnt = 0;
  for (int32_t j = 0; j < len; ++j) {
    const uint32_t c = idx[i * (int64_t)k + j];
    if ((int64_t)c == i) continue;
    if (WRITE) {
      out_idx[o] = c;
      out_w[o] = w[i * (int64_t)k + j];
      ++o;
    }
    ++cnt;
  }
  if (!WRITE) out_cnt[i] = cnt;
}

int rows_per_block(int32_t kp) {
  if ((size_t)128 * kp * 8 <= 48 * 1024) return 128;
  if ((size_t)64 * kp * 8 <= 96 * 1024) return 64;
  return 32;
}

void set_smem_limit(const void* fn, size_t bytes) {
  if (bytes > 48 * 1024)
    EVOC_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)bytes));
}

}  // namespace

void smooth_knn_device(evoc_ctx* ctx, const float* d_dist,
                       const int32_t* d_row_len, int64_t n, int32_t k,
                       uint64_t k_target, float local_connectivity,
                       int32_t n_iter, float* d_sigma, float* d_rho,
                       float* d_weights_out, const uint32_t* /*unused*/) {
  if (n == 0) return;
  const int32_t kp = k | 1;
  // rows per warp: 64 where they fit in 48 KB per block, else one per lane
  int pool = 64;
  while (pool > 32 && (size_t)SK_WARPS * pool * kp * sizeof(float) > 48 * 1024) pool /= 2;
  const size_t smem = (size_t)SK_WARPS * pool * kp * sizeof(float);
  if (smem > 200 * 1024)
    throw Error(EVOC_ERR_UNSUPPORTED, "k too large (k <= 399 supported)");
  set_smem_limit((const void*)k_smooth_knn, smem);
  const double target = std::log2((double)k_target);
  const int64_t per_block = (int64_t)SK_WARPS * pool;
  const int64_t blocks = (n + per_block - 1) / per_block;
  EVOC_CUDA(cudaMemsetAsync(ctx->sk_steps.get(), 0, sizeof(unsigned long long), ctx->stream));
  k_smooth_knn<<<(unsigned)blocks, 32 * SK_WARPS, smem, ctx->stream>>>(
      d_dist, d_row_len, n, k, kp, pool, target, local_connectivity, n_iter, d_sigma, d_rho,
      ctx->status.get(), ctx->sk_steps.get());
  EVOC_CHECK_LAUNCH();
  if (d_weights_out) {
    const int64_t elems = n * (int64_t)k;
    k_knn_weights<<<(unsigned)((elems + 255) / 256), 256, 0, ctx->stream>>>(
        d_dist, d_row_len, n, k, d_sigma, d_rho, d_weights_out);
    EVOC_CHECK_LAUNCH();
  }
}

void fuzzy_set_device(evoc_ctx* ctx, const uint32_t* d_idx,
                      const float* d_dist, int64_t n, int32_t k,
                      float effective_n_neighbours, bool symmetrise,
                      float* d_sigmas_out, float* d_rhos_out, evoc_graph* out) {
  cudaStream_t s = ctx->stream;
  if (n <= 0)
    throw Error(EVOC_ERR_INVALID_ARGUMENT,
                "empty kNN graph (build_fuzzy_simplicial_set reads row 0)");
  if (k <= 0) throw Error(EVOC_ERR_INVALID_ARGUMENT, "k must be positive");
  if (n >= (int64_t)PAD) throw Error(EVOC_ERR_UNSUPPORTED, "n must be < 2^32-1");

  StageTrace trace(s);
  DevBuf<int32_t> row_len(n, s);
  {
    const int64_t threads = n * 32;
    k_knn_rowlen<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
        d_idx, n, k, row_len.get(), ctx->status.get());
    EVOC_CHECK_LAUNCH();
  }
  check_status(ctx, "fuzzy set");
  trace.mark("row lengths");

  // k = effective_n_neighbors.to_usize().unwrap_or(knn_dists[0].len())
  // (fuzzy_graph.rs:284-286)
  uint64_t kk;
  const float e = effective_n_neighbours;
  if (e > -1.0f && e < 18446744073709551616.0f) {
    kk = (uint64_t)e;
  } else {
    int32_t len0 = 0;
    EVOC_CUDA(cudaMemcpyAsync(&len0, row_len.get(), sizeof(int32_t),
                              cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaStreamSynchronize(s));
    kk = (uint64_t)len0;
  }

  DevBuf<float> sig_local, rho_local;
  float* d_sig = d_sigmas_out;
  float* d_rho = d_rhos_out;
  if (!d_sig) { sig_local.alloc(n, s); d_sig = sig_local.get(); }
  if (!d_rho) { rho_local.alloc(n, s); d_rho = rho_local.get(); }
  DevBuf<float> wts(n * (int64_t)k, s);
  smooth_knn_device(ctx, d_dist, row_len.get(), n, k, kk, 1.0f, 64, d_sig,
                    d_rho, wts.get(), nullptr);
  check_status(ctx, "fuzzy set");
  trace.mark("smooth knn + weights");

  out->ctx = ctx;
  out->n = n;
  out->indptr.alloc(n + 1, s);
  const unsigned row_blocks = (unsigned)((n + 255) / 256);

  if (!symmetrise) {
    DevBuf<int32_t> cnt(n, s);
    k_directed<false><<<row_blocks, 256, 0, s>>>(d_idx, wts.get(), row_len.get(),
                                                  n, k, cnt.get(), nullptr,
                                                  nullptr, nullptr);
    EVOC_CHECK_LAUNCH();
    exclusive_scan_i32_to_i64(cnt.get(), out->indptr.get(), n, s);
    int64_t nnz = 0;
    EVOC_CUDA(cudaMemcpyAsync(&nnz, out->indptr.get() + n, sizeof(int64_t),
                              cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaStreamSynchronize(s));
    out->nnz = nnz;
    out->indices.alloc(nnz, s);
    out->weights.alloc(nnz, s);
    k_directed<true><<<row_blocks, 256, 0, s>>>(
        d_idx, wts.get(), row_len.get(), n, k, nullptr, out->indptr.get(),
        out->indices.get(), out->weights.get());
    EVOC_CHECK_LAUNCH();
    out->canonical = false;
    EVOC_CUDA(cudaStreamSynchronize(s));
    return;
  }

  // forward lists
  const int32_t kp = k | 1;
  int R = rows_per_block(kp);
  const size_t smem = (size_t)R * kp * 8;
  if (smem > 200 * 1024)
    throw Error(EVOC_ERR_UNSUPPORTED, "k too large (k <= 1599 supported)");
  set_smem_limit((const void*)k_forward_rows, smem);
  DevBuf<uint32_t> fcol(n * (int64_t)k, s);
  DevBuf<float> fw(n * (int64_t)k, s);
  DevBuf<int32_t> fcnt(n, s), indeg(n, s);
  EVOC_CUDA(cudaMemsetAsync(indeg.get(), 0, n * sizeof(int32_t), s));
  k_forward_rows<<<(unsigned)((n + R - 1) / R), R, smem, s>>>(
      d_idx, wts.get(), row_len.get(), n, k, kp, fcol.get(), fw.get(),
      fcnt.get(), indeg.get());
  EVOC_CHECK_LAUNCH();
  wts.release();
  trace.mark("forward rows");

  DevBuf<int64_t> fptr(n + 1, s), bptr(n + 1, s);
  exclusive_scan_i32_to_i64(fcnt.get(), fptr.get(), n, s);
  exclusive_scan_i32_to_i64(indeg.get(), bptr.get(), n, s);
  int64_t nf = 0;
  EVOC_CUDA(cudaMemcpyAsync(&nf, fptr.get() + n, sizeof(int64_t),
                            cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaStreamSynchronize(s));

  // stable transpose: sort forward entries by column
  DevBuf<uint32_t> keys(nf, s);
  DevBuf<uint2> vals(nf, s);
  if (nf > 0) {
    const int64_t threads = n * 32;
    k_forward_compact<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
        fcol.get(), fw.get(), fptr.get(), n, k, keys.get(), vals.get());
    EVOC_CHECK_LAUNCH();
    radix_sort_pairs(keys.get(), vals.get(), nf, bits_for((uint64_t)(n - 1)), s);
  }
  keys.release();
  fptr.release();
  trace.mark("transpose");

  DevBuf<int32_t> ucnt(n, s);
  int64_t nb_total = 0;
  EVOC_CUDA(cudaMemcpyAsync(&nb_total, bptr.get() + n, sizeof(int64_t),
                            cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaStreamSynchronize(s));
  DevBuf<uint2> utmp(n * (int64_t)k + nb_total, s);
  k_union<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(
      fcol.get(), fw.get(), fcnt.get(), bptr.get(), vals.get(), n, k, ucnt.get(), utmp.get());
  EVOC_CHECK_LAUNCH();
  exclusive_scan_i32_to_i64(ucnt.get(), out->indptr.get(), n, s);
  int64_t nnz = 0;
  EVOC_CUDA(cudaMemcpyAsync(&nnz, out->indptr.get() + n, sizeof(int64_t),
                            cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaStreamSynchronize(s));
  out->nnz = nnz;
  out->indices.alloc(nnz, s);
  out->weights.alloc(nnz, s);
  trace.mark("union merge");
  k_union_compact<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(
      utmp.get(), bptr.get(), n, k, out->indptr.get(), out->indices.get(),
      out->weights.get());
  EVOC_CHECK_LAUNCH();
  out->canonical = true;
  trace.mark("union compact");
  EVOC_CUDA(cudaStreamSynchronize(s));
}

}  // namespace evoc
