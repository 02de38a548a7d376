// embed.cu — the EVoC node-embedding optimiser on the GPU.
//
// Replaces evoc_embedding, src/graph/embedding.rs:48-298 (evoc-rs 0.2.7).
//
// Set-up (once per plan, embedding.rs:78-175):
//   k_row_counts   warp per row: upper (i < j) and lower entries per row.
//   k_edge_fill    warp per row: undirected edge list in adjacency order
//                  (eidx = rank among upper entries, embedding.rs:79-90) and
//                  the per-problem maximum weight (embedding.rs:99).
//   k_edge_ps      thread per edge: epochs_per_sample (embedding.rs:101-111).
//   radix sort     (general graphs only) edges by larger endpoint, stable, to
//                  list each node's "is_smaller = false" incidences in edge
//                  order (embedding.rs:130-135).
//   k_inc_fill     warp per node: the per-node incidence list of
//                  embedding.rs:121-135 (lower part in edge order, then the
//                  node's own upper entries).
//   k_schedule     thread per incidence entry: runs the epochs-per-sample
//                  recurrence of embedding.rs:274-286 for every epoch and
//                  stores, per epoch, one bit "fires" and P bits "negative
//                  count" (embedding.rs:225-228) for each entry. Both copies of
//                  an edge evaluate the same f32 recurrence, so they agree.
// Epoch loop (embedding.rs:178-292), one launch per epoch, captured in a CUDA
// graph:
//   k_epoch        G lanes per node (pull-based): the node's fire words are
//                  read G at a time and its fired entries compacted (prefix
//                  sum + __fns), so each lane takes a fired entry, gathers the
//                  partner row (float4) and the Philox negatives, and adds into
//                  partial sum (fired rank mod 32) in shared memory; the 32
//                  partials are combined by a pairwise tree (strides 16..1);
//                  the lane that owns a dimension applies Adam
//                  (embedding.rs:256-272) and writes the next embedding buffer
//                  (ping-pong). No float atomics; results do not depend on G.
#include "evoc_device.cuh"
#include "evoc_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <utility>

namespace evoc {

struct ProbInfo {
  uint32_t node_base;
  uint32_t n;
  uint64_t seed;
};

}  // namespace evoc

struct evoc_plan {
  evoc_ctx* ctx = nullptr;
  int64_t n = 0;          // nodes over all problems
  int32_t dim = 0;        // n_components
  int32_t dimp = 0;       // padded row width (4, 8 or 16)
  int32_t lanes = 0;      // warps (32-node tiles) per thread block of k_epoch
  evoc_embed_params_t params{};
  int32_t n_problems = 0;
  std::vector<int64_t> node_base;  // per problem, host
  std::vector<uint64_t> seeds;     // per problem, host
  bool has_edges = false;
  int64_t n_edges = 0;
  int64_t n_inc = 0;      // incidence entries (2 per edge)
  int32_t P = 0;          // negative-count bit planes
  int64_t W = 0;          // 32-bit words per plane
  uint64_t max_neg = 0;
  evoc::DevBuf<int64_t> inc_ptr;
  evoc::DevBuf<uint32_t> inc_other;
  evoc::DevBuf<int64_t> eidx_base;
  evoc::DevBuf<uint32_t> planes;
  evoc::DevBuf<uint32_t> prob_of_node;  // batched only
  evoc::DevBuf<evoc::ProbInfo> prob;    // batched only
  evoc::DevBuf<float> emb, m, v, grad;  // emb: both embedding buffers
  float* e0 = nullptr;                  // ping-pong halves of emb
  float* e1 = nullptr;
  std::vector<float> lr_ad, epsc, gamma;
  float one_m_b1 = 0, one_m_b2 = 0;
  std::vector<evoc_epoch_stats_t> stats;
  // per-epoch gradient slots (the fast path): for epoch t and tile T, slots
  // [tile_off[t * ntiles + T], tile_off[t * ntiles + T + 1]); a slot is
  // (source row, tile-local node | 32 for a negative sample)
  bool use_slots = false;
  int64_t ntiles = 0;
  int64_t n_slots = 0;
  evoc::DevBuf<int64_t> tile_off;
  evoc::DevBuf<uint32_t> tile_order;  // tiles by descending slot count (launch order)
  evoc::DevBuf<uint32_t> slots;
  evoc::DevBuf<unsigned long long> work_ctr;  // per epoch
  unsigned slot_grid = 0;                     // persistent grid of the slots kernel
  int32_t kvariant = 0;                       // slots-kernel variant (SLOT_VARIANTS)
  int32_t blocks_per_sm = 0;                  // persistent blocks per SM (0: as many as fit)
  bool all_epochs = false;                    // one cooperative launch for all epochs
  evoc::DevBuf<float4> ep_params;             // per epoch: gamma, lr * ad_scale, eps'
  evoc::DevBuf<unsigned> grid_bar;            // the all-epochs launch's barrier words
  bool stats_done = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
};

namespace evoc {
namespace {

constexpr int64_t NEG_LIMIT = 1 << 20;

__device__ __forceinline__ float ps_from_w(float w, float max_w) {
  const float norm = fdiv(w, max_w);
  return (norm > 0.0f) ? fdiv(1.0f, norm) : 1e8f;
}

__device__ __forceinline__ uint32_t prob_of(const uint32_t* pon, uint32_t v) {
  return pon ? pon[v] : 0u;
}

// ---------------------------------------------------------------------------
// Set-up kernels
// ---------------------------------------------------------------------------
__global__ void k_row_counts(const int64_t* __restrict__ indptr,
                             const uint32_t* __restrict__ indices, int64_t n,
                             int32_t* __restrict__ ucnt,
                             int32_t* __restrict__ lcnt_own) {
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= n) return;
  const int64_t a = indptr[r], b = indptr[r + 1];
  int32_t u = 0, l = 0;
  for (int64_t p = a + lane; p < b; p += 32) {
    const uint32_t c = indices[p];
    u += (int64_t)c > r;
    l += (int64_t)c < r;
  }
  u = __reduce_add_sync(0xffffffffu, (unsigned)u);
  l = __reduce_add_sync(0xffffffffu, (unsigned)l);
  if (lane == 0) {
    ucnt[r] = u;
    lcnt_own[r] = l;
  }
}

__global__ void k_edge_fill(const int64_t* __restrict__ indptr,
                            const uint32_t* __restrict__ indices,
                            const float* __restrict__ weights, int64_t n,
                            const int64_t* __restrict__ uptr,
                            const uint32_t* __restrict__ prob_of_node,
                            float* __restrict__ e_w, uint32_t* __restrict__ e_dst,
                            uint32_t* __restrict__ e_src,
                            int32_t* __restrict__ max_w_bits,
                            int32_t* __restrict__ lcnt /* general only */) {
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= n) return;
  const int64_t a = indptr[r], b = indptr[r + 1];
  int64_t e = uptr[r];
  int32_t mx = 0;
  const uint32_t lt = (1u << lane) - 1u;
  for (int64_t base = a; base < b; base += 32) {
    const int64_t p = base + lane;
    uint32_t c = 0;
    float w = 0.0f;
    bool up = false;
    if (p < b) {
      c = indices[p];
      w = weights[p];
      up = (int64_t)c > r;
    }
    const uint32_t bal = __ballot_sync(0xffffffffu, up);
    if (up) {
      const int64_t q = e + __popc(bal & lt);
      e_w[q] = w;
      e_dst[q] = c;
      e_src[q] = (uint32_t)r;
      if (w == w) mx = max(mx, __float_as_int(w));  // f32::max ignores NaN
      if (lcnt) atomicAdd(&lcnt[c], 1);
    }
    e += __popc(bal);
  }
  mx = __reduce_max_sync(0xffffffffu, mx);
  if (lane == 0 && mx > 0) atomicMax(&max_w_bits[prob_of(prob_of_node, (uint32_t)r)], mx);
}

__global__ void k_edge_ps(const float* __restrict__ e_w,
                          const uint32_t* __restrict__ e_src, int64_t U,
                          const uint32_t* __restrict__ prob_of_node,
                          const int32_t* __restrict__ max_w_bits,
                          float* __restrict__ e_ps) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= U) return;
  const float mw = __int_as_float(max_w_bits[prob_of(prob_of_node, e_src[e])]);
  e_ps[e] = ps_from_w(e_w[e], mw);
}

// Problem edge base: uptr at each problem's first node.
__global__ void k_prob_ebase(const int64_t* __restrict__ uptr,
                             const ProbInfo* __restrict__ prob, int32_t np,
                             int64_t* __restrict__ ebase) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < np) ebase[q] = prob ? uptr[prob[q].node_base] : 0;
}

__global__ void k_inc_fill(const int64_t* __restrict__ indptr,
                           const uint32_t* __restrict__ indices,
                           const float* __restrict__ weights, int64_t n,
                           const int64_t* __restrict__ uptr,
                           const int32_t* __restrict__ lcnt,
                           const int64_t* __restrict__ lptr,   // general
                           const uint2* __restrict__ lower,    // general
                           const float* __restrict__ e_ps,
                           const int64_t* __restrict__ inc_ptr,
                           const uint32_t* __restrict__ prob_of_node,
                           const int32_t* __restrict__ max_w_bits,
                           const int64_t* __restrict__ ebase,
                           uint32_t* __restrict__ inc_other,
                           float* __restrict__ inc_ps,
                           uint8_t* __restrict__ inc_up,
                           int64_t* __restrict__ eidx_base,
                           uint32_t* __restrict__ inc_eidx) {
  const int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (v >= n) return;
  const uint32_t pr = prob_of(prob_of_node, (uint32_t)v);
  const float mw = __int_as_float(max_w_bits[pr]);
  const int64_t p0 = inc_ptr[v];
  const int64_t nl = lcnt[v];
  const int64_t a = indptr[v], b = indptr[v + 1];
  const uint32_t lt = (1u << lane) - 1u;
  if (lower == nullptr) {
    // canonical symmetric graph: lower part = own entries with column < v
    int64_t o = p0;
    for (int64_t base = a; base < b; base += 32) {
      const int64_t p = base + lane;
      const bool lo = p < b && (int64_t)indices[p] < v;
      const uint32_t bal = __ballot_sync(0xffffffffu, lo);
      if (lo) {
        const int64_t q = o + __popc(bal & lt);
        const uint32_t c = indices[p];
        inc_other[q] = c;
        inc_ps[q] = ps_from_w(weights[p], mw);
        inc_up[q] = 0;
        inc_eidx[q] = 0xffffffffu;  // lower entries draw no negatives
      }
      o += __popc(bal);
    }
  } else {
    const int64_t l0 = lptr[v];
    for (int64_t j = lane; j < nl; j += 32) {
      const uint2 pe = lower[l0 + j];  // (eidx, smaller endpoint)
      inc_other[p0 + j] = pe.y;
      inc_ps[p0 + j] = e_ps[pe.x];
      inc_up[p0 + j] = 0;
      inc_eidx[p0 + j] = 0xffffffffu;  // lower entries draw no negatives
    }
  }
  int64_t o = p0 + nl;
  for (int64_t base = a; base < b; base += 32) {
    const int64_t p = base + lane;
    const bool up = p < b && (int64_t)indices[p] > v;
    const uint32_t bal = __ballot_sync(0xffffffffu, up);
    if (up) {
      const int64_t q = o + __popc(bal & lt);
      inc_other[q] = indices[p];
      inc_ps[q] = ps_from_w(weights[p], mw);
      inc_up[q] = 1;
      inc_eidx[q] = (uint32_t)(uptr[v] + (q - (p0 + nl)));
    }
    o += __popc(bal);
  }
  if (lane == 0) eidx_base[v] = (uptr[v] - ebase[pr]) - (p0 + nl);
}

// Epochs-per-sample recurrence of one incidence entry (embedding.rs:274-286)
// and the negative count of embedding.rs:225-228.
struct Sched {
  float ps, pn, ns, nn;
  bool up;
  __device__ __forceinline__ void init(float ps_, float neg_factor, bool up_) {
    ps = ps_;
    pn = fmul(ps_, neg_factor);
    ns = ps;
    nn = pn;
    up = up_;
  }
  // Returns fired; *nneg gets the negative count (upper entries only).
  // The count stays a float: for x = floor(q), to_usize(x).unwrap_or(0) as
  // f32 equals x when 0 < x < 2^64 and +0 otherwise (x is integer-valued).
  __device__ __forceinline__ bool step(float tf, uint64_t* nneg) {
    float cntf;
    const bool fire = stepf(tf, &cntf);
    *nneg = (uint64_t)cntf;
    return fire;
  }
  __device__ __forceinline__ bool stepf(float tf, float* cnt_out) {
    const bool fire = !(ns > tf);
    float cntf = 0.0f;
    if (ns <= tf) {
      ns = fadd(ns, ps);
      if (up) {
        const float x = floorf(fdiv(fsub(tf, nn), pn));
        cntf = (x > 0.0f && x < 18446744073709551616.0f) ? x : 0.0f;
        nn = fadd(nn, fmul(cntf, pn));
      }
    }
    *cnt_out = (fire && up) ? cntf : 0.0f;
    return fire;
  }
};

__global__ void k_schedule_scan(const float* __restrict__ inc_ps,
                                const uint8_t* __restrict__ inc_up,
                                int64_t n_inc, int32_t n_epochs,
                                float neg_factor,
                                unsigned long long* __restrict__ max_neg,
                                unsigned long long* __restrict__ st_fired,
                                unsigned long long* __restrict__ st_neg) {
  extern __shared__ unsigned long long sst[];  // [2 * n_epochs] or empty
  const bool stats = st_fired != nullptr;
  if (stats) {
    for (int t = threadIdx.x; t < 2 * n_epochs; t += blockDim.x) sst[t] = 0;
    __syncthreads();
  }
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = p < n_inc;
  Sched s;
  s.init(valid ? inc_ps[p] : 3.0e38f, neg_factor, valid && inc_up[p]);
  unsigned long long mx = 0;
  for (int32_t t = 0; t < n_epochs; ++t) {
    uint64_t nn = 0;
    const bool f = valid && s.step((float)t, &nn);
    if (nn > mx) mx = nn;
    if (stats) {
      const unsigned fu = __reduce_add_sync(0xffffffffu, (f && s.up) ? 1u : 0u);
      const unsigned long long ng = (unsigned long long)nn;
      unsigned long long ngs = ng;
      for (int o = 16; o > 0; o >>= 1) ngs += __shfl_xor_sync(0xffffffffu, ngs, o);
      if ((threadIdx.x & 31) == 0) {
        if (fu) atomicAdd(&sst[t], (unsigned long long)fu);
        if (ngs) atomicAdd(&sst[n_epochs + t], ngs);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = y > mx ? y : mx;
  }
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(max_neg, mx);
  if (stats) {
    __syncthreads();
    for (int t = threadIdx.x; t < n_epochs; t += blockDim.x) {
      if (sst[t]) atomicAdd(&st_fired[t], sst[t]);
      if (sst[n_epochs + t]) atomicAdd(&st_neg[t], sst[n_epochs + t]);
    }
  }
}

// Writes, per epoch t, the fire plane and P negative-count planes:
// planes[(t * (1 + P) + b) * W + word].
__global__ void k_schedule_write(const float* __restrict__ inc_ps,
                                 const uint8_t* __restrict__ inc_up,
                                 int64_t n_inc, int32_t n_epochs,
                                 float neg_factor, int32_t P, int64_t W,
                                 uint32_t* __restrict__ planes) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t word = p >> 5;
  if (word >= W) return;  // whole warps only
  const bool valid = p < n_inc;
  Sched s;
  s.init(valid ? inc_ps[p] : 3.0e38f, neg_factor, valid && inc_up[p]);
  const bool lane0 = (threadIdx.x & 31) == 0;
  for (int32_t t = 0; t < n_epochs; ++t) {
    uint64_t nn = 0;
    const bool f = valid && s.step((float)t, &nn);
    const uint32_t fw = __ballot_sync(0xffffffffu, f);
    uint32_t* base = planes + (size_t)t * (1 + P) * W + word;
    if (lane0) base[0] = fw;
    for (int32_t b = 0; b < P; ++b) {
      const uint32_t bw = __ballot_sync(0xffffffffu, (nn >> b) & 1ull);
      if (lane0) base[(size_t)(1 + b) * W] = bw;
    }
  }
}

// Active nodes per epoch: nodes with at least one fired incidence entry.
__global__ void k_active_count(const int64_t* __restrict__ inc_ptr, int64_t n,
                               const uint32_t* __restrict__ planes,
                               int32_t n_epochs, int32_t P, int64_t W,
                               unsigned long long* __restrict__ st_active) {
  const int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const bool valid = v < n;
  const int64_t p0 = valid ? inc_ptr[v] : 0, p1 = valid ? inc_ptr[v + 1] : 0;
  for (int32_t t = 0; t < n_epochs; ++t) {
    const uint32_t* fire = planes + (size_t)t * (1 + P) * W;
    bool any = false;
    for (int64_t p = p0 + lane; p < p1; p += 32) any |= (fire[p >> 5] >> (p & 31)) & 1u;
    any = __any_sync(0xffffffffu, any);
    if (lane == 0 && any) atomicAdd(&st_active[t], 1ull);
  }
}

// ---------------------------------------------------------------------------
// Random initialisation, padding and unpadding.
// ---------------------------------------------------------------------------
__global__ void k_init_random(float* __restrict__ e, int64_t n, int32_t dim,
                              int32_t dimp,
                              const uint32_t* __restrict__ prob_of_node,
                              const ProbInfo* __restrict__ prob, uint64_t seed) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n * dimp) return;
  const int64_t v = q / dimp;
  const int32_t d = (int32_t)(q - v * dimp);
  float val = 0.0f;
  if (d < dim) {
    uint64_t sd = seed;
    int64_t local = v;
    if (prob_of_node) {
      const ProbInfo pi = prob[prob_of_node[v]];
      sd = pi.seed;
      local = v - pi.node_base;
    }
    val = init_value(sd, (uint64_t)(local * dim + d));
  }
  e[q] = val;
}

__global__ void k_pad(const float* __restrict__ src, float* __restrict__ dst,
                      int64_t n, int32_t dim, int32_t dimp) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n * dimp) return;
  const int64_t v = q / dimp;
  const int32_t d = (int32_t)(q - v * dimp);
  dst[q] = (d < dim) ? src[v * dim + d] : 0.0f;
}

__global__ void k_unpad(const float* __restrict__ src, float* __restrict__ dst,
                        int64_t n, int32_t dim, int32_t dimp) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n * dim) return;
  const int64_t v = q / dim;
  const int32_t d = (int32_t)(q - v * dim);
  dst[q] = src[v * dimp + d];
}

// ---------------------------------------------------------------------------
// The fused epoch kernel.
// ---------------------------------------------------------------------------
struct EpochArgs {
  const int64_t* inc_ptr;
  const uint32_t* inc_other;
  const int64_t* eidx_base;
  const uint32_t* fire;  // fire plane of this epoch; neg planes follow
  int64_t W;
  int32_t P;
  const float* e_cur;
  float* e_next;
  float* m;
  float* v;
  float* grad_out;
  const uint32_t* prob_of_node;
  const ProbInfo* prob;
  const int64_t* tile_off;     // slot offsets of this epoch (slots path)
  const uint32_t* tile_order;  // slots path: tiles in launch order, heaviest first
  const uint32_t* slots;
  unsigned long long* work_ctr;  // slots path: next tile of this epoch (zeroed per launch)
  uint32_t n_total;
  uint32_t epoch;
  uint64_t seed;
  float noise, gamma, lr_ad, epsc, one_m_b1, one_m_b2;
};

// COH: the row may have been written earlier in the same launch (the
// persistent all-epochs kernel), so it is read through L2 (ld.global.cg)
// rather than the non-coherent read-only path.
template <int DIMP, bool COH = false>
__device__ __forceinline__ void load_row(const float* __restrict__ p, float (&r)[DIMP]) {
  const float4* p4 = reinterpret_cast<const float4*>(p);
#pragma unroll
  for (int i = 0; i < DIMP / 4; ++i) {
    const float4 x = COH ? __ldcg(p4 + i) : __ldg(p4 + i);
    r[4 * i + 0] = x.x;
    r[4 * i + 1] = x.y;
    r[4 * i + 2] = x.z;
    r[4 * i + 3] = x.w;
  }
}

// ---------------------------------------------------------------------------
// One epoch, one warp per tile of 32 consecutive nodes.
//
// Phase A (lane = node): incidence offsets and the tile's own rows are loaded
// coalesced into shared memory; running gradients start at +0.
// Phase B (lane = fired entry): the tile's fire words are read 32 at a time;
// fired entries (in incidence order, across node boundaries) are handed to
// lanes 32 at a time by a warp prefix sum + __fns. Each lane gathers its
// partner row and, for the smaller endpoint, its Philox negatives, and writes
// one contribution vector per slot (slot 0 = attraction, slot j+1 = negative
// j; skipped terms are +0) into a CAP-slot buffer. Then the slots of every
// node are added to its running gradient serially in slot order, one lane per
// (node, dim) segment: the reference's running sum (embedding.rs:194-248),
// term for term. An entry whose slots do not fit continues in the next chunk.
// Phase C (lane = node): Adam (embedding.rs:256-272) and the next embedding.
// ---------------------------------------------------------------------------
constexpr int TILE = 32;
constexpr int CAP = 64;

template <int DIMP>
struct alignas(16) TileSmem {
  float rows[TILE][DIMP];       // e_cur rows of the tile's nodes
  float S[TILE][DIMP + 1];      // running gradients
  float contrib[CAP][DIMP + 1]; // contribution slots of the current chunk
  int64_t pbeg[TILE + 1];       // incidence offsets of the tile
  uint8_t slot_node[CAP];       // tile-local node of each slot
};

template <int DIMP>
__global__ void __launch_bounds__(128) k_epoch(EpochArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  TileSmem<DIMP>& sm = reinterpret_cast<TileSmem<DIMP>*>(smem_raw)[threadIdx.x >> 5];
  const int64_t v0 = ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * TILE;
  if (v0 >= (int64_t)a.n_total) return;  // whole warp
  const int nt = (int)min((int64_t)TILE, (int64_t)a.n_total - v0);
  const bool has_node = lane < nt;

  // ---- phase A
  if (has_node) sm.pbeg[lane] = a.inc_ptr[v0 + lane];
  if (lane == 0) sm.pbeg[nt] = a.inc_ptr[v0 + nt];
  {
    const float4* src = reinterpret_cast<const float4*>(a.e_cur + (size_t)v0 * DIMP);
    float4* dst = reinterpret_cast<float4*>(&sm.rows[0][0]);
    for (int i = lane; i < nt * (DIMP / 4); i += 32) dst[i] = __ldg(src + i);
  }
  for (int i = lane; i < TILE * (DIMP + 1); i += 32) (&sm.S[0][0])[i] = 0.0f;
  __syncwarp();
  const int64_t P0 = sm.pbeg[0], P1 = sm.pbeg[nt];
  const float two_noise = fmul(2.0f, a.noise);
  const float gamma4 = fmul(a.gamma, 4.0f);
  uint32_t touched = 0;

  // ---- phase B
  if (P1 > P0) {
    const int64_t W0 = P0 >> 5, W1 = (P1 - 1) >> 5;
    for (int64_t wb = W0; wb <= W1; wb += 32) {
      const int64_t w = wb + lane;
      uint32_t word = 0;
      if (w <= W1) {
        word = __ldcs(a.fire + w);
        if (w == W0) word &= FULL << (P0 & 31);
        if (w == W1) {
          const int hi = (int)((P1 - 1) & 31);
          word &= (hi == 31) ? FULL : ((2u << hi) - 1u);
        }
      }
      const int cnt = __popc(word);
      int incl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
      }
      const int excl = incl - cnt;
      const int tot = __shfl_sync(FULL, incl, 31);
      int fi = 0;  // first fired entry (index in this round) of the next chunk
      int so = 0;  // slots of that entry consumed by earlier chunks
      while (fi < tot) {
        const int f = fi + lane;
        const bool valid = f < tot;
        int u = 0;  // lane whose word holds fired entry f
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
          const int e_ = __shfl_sync(FULL, excl, u + step);
          if (e_ <= f) u += step;
        }
        const uint32_t wu = __shfl_sync(FULL, word, u);
        const int eu = __shfl_sync(FULL, excl, u);
        int64_t p = 0;
        int node = 0;
        uint32_t o = 0, nneg = 0;
        if (valid) {
          p = ((wb + u) << 5) + (int64_t)__fns(wu, 0u, f - eu + 1);
          int lo = 0, hi = nt - 1;  // last node whose list starts at or before p
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (sm.pbeg[mid] <= p) lo = mid; else hi = mid - 1;
          }
          node = lo;
          o = __ldcs(a.inc_other + p);
          if ((int64_t)o > v0 + node)
            for (int32_t b = 0; b < a.P; ++b)
              nneg |= ((__ldcs(a.fire + (size_t)(1 + b) * a.W + (p >> 5)) >> (p & 31)) & 1u) << b;
        }
        const int k_first = (lane == 0) ? so : 0;
        const int cc = valid ? (int)(1 + nneg) - k_first : 0;
        int cincl = cc;
#pragma unroll
        for (int s2 = 1; s2 < 32; s2 <<= 1) {
          const int y = __shfl_up_sync(FULL, cincl, s2);
          if (lane >= s2) cincl += y;
        }
        const int cexcl = cincl - cc;
        const int nslots = max(0, min(cincl, CAP) - cexcl);
        if (nslots > 0) {
          const uint32_t vg = (uint32_t)(v0 + node);
          float ev[DIMP];
#pragma unroll
          for (int d = 0; d < DIMP; ++d) ev[d] = sm.rows[node][d];
          uint32_t nb = 0, np = a.n_total;
          uint64_t seed = a.seed;
          uint64_t eidx = 0;
          if (k_first + nslots > 1) {  // negatives in this chunk
            if (a.prob_of_node) {
              const ProbInfo pi = a.prob[a.prob_of_node[vg]];
              nb = pi.node_base;
              np = pi.n;
              seed = pi.seed;
            }
            eidx = (uint64_t)(p + a.eidx_base[vg]);
          }
          for (int t = 0; t < nslots; ++t) {
            const int k = k_first + t;
            float* dst = sm.contrib[cexcl + t];
            sm.slot_node[cexcl + t] = (uint8_t)node;
            float row[DIMP];
            bool skip = false;
            uint32_t src;
            if (k == 0) {
              src = o;
            } else {
              src = nb + negative_draw(seed, (uint32_t)(k - 1), a.epoch, eidx, np);
              skip = (src == vg);
            }
            if (skip) {
#pragma unroll
              for (int d = 0; d < DIMP; ++d) dst[d] = 0.0f;
              continue;
            }
            load_row<DIMP>(a.e_cur + (size_t)src * DIMP, row);
            float diff[DIMP];
            float dsq = 0.0f;
#pragma unroll
            for (int d = 0; d < DIMP; ++d) {
              diff[d] = fsub(ev[d], row[d]);
              dsq = fadd(dsq, fmul(diff[d], diff[d]));
            }
            if (k == 0) {  // attraction, embedding.rs:213-221
              if (dsq >= 1e-8f) {
                const float dist = fsqrt(dsq);
                const float coeff = fdiv(fsub(-fmul(two_noise, dist), 2.0f),
                                         fadd(fsub(fmul(2.0f, dsq), fmul(0.5f, dist)), 1.0f));
#pragma unroll
                for (int d = 0; d < DIMP; ++d) dst[d] = fmul(coeff, diff[d]);
              } else {
#pragma unroll
                for (int d = 0; d < DIMP; ++d) dst[d] = 0.0f;
              }
            } else {  // repulsion, embedding.rs:237-245
              if (dsq > 0.01f) {
                const float gc = fdiv(gamma4, fmul(fadd(1.0f, fmul(0.25f, dsq)), dsq));
#pragma unroll
                for (int d = 0; d < DIMP; ++d) {
                  float c = fmul(gc, diff[d]);
                  c = fmaxf(c, -4.0f);
                  dst[d] = fminf(c, 4.0f);
                }
              } else {
#pragma unroll
                for (int d = 0; d < DIMP; ++d) dst[d] = 0.0f;
              }
            }
          }
        }
        touched |= __reduce_or_sync(FULL, valid ? (1u << node) : 0u);
        const int ndone = __popc(__ballot_sync(FULL, valid && cincl <= CAP));
        const int used = min(__shfl_sync(FULL, cincl, 31), CAP);
        const int cex_nd = __shfl_sync(FULL, cexcl, ndone & 31);
        const int kf_nd = __shfl_sync(FULL, k_first, ndone & 31);
        __syncwarp();
        // serial accumulation of slots [0, used), one lane per (node, dim)
        {
          const int sa = lane, sb = lane + 32;
          const bool st_a = sa < used && (sa == 0 || sm.slot_node[sa] != sm.slot_node[sa - 1]);
          const bool st_b = sb < used && sm.slot_node[sb] != sm.slot_node[sb - 1];
          const uint32_t ma = __ballot_sync(FULL, st_a), mb = __ballot_sync(FULL, st_b);
          const int na = __popc(ma), nseg = na + __popc(mb);
          for (int tsk = lane; tsk < nseg * DIMP; tsk += 32) {
            const int seg = tsk / DIMP, d = tsk - seg * DIMP;
            const int start = (seg < na) ? (int)__fns(ma, 0u, seg + 1)
                                         : 32 + (int)__fns(mb, 0u, seg - na + 1);
            int end = used;
            if (seg + 1 < nseg)
              end = (seg + 1 < na) ? (int)__fns(ma, 0u, seg + 2)
                                   : 32 + (int)__fns(mb, 0u, seg + 1 - na + 1);
            const int nd = sm.slot_node[start];
            float acc = sm.S[nd][d];
            for (int s2 = start; s2 < end; ++s2) acc = fadd(acc, sm.contrib[s2][d]);
            sm.S[nd][d] = acc;
          }
        }
        __syncwarp();
        int next_so = 0;
        if (ndone < 32 && fi + ndone < tot) next_so = kf_nd + max(0, CAP - cex_nd);
        fi += ndone;
        so = next_so;
      }
    }
  }

  // ---- phase C
  if (has_node) {
    const size_t q = (size_t)(v0 + lane) * DIMP;
    const bool act = (touched >> lane) & 1u;
    float e[DIMP], g[DIMP];
#pragma unroll
    for (int d = 0; d < DIMP; ++d) {
      e[d] = sm.rows[lane][d];
      g[d] = act ? sm.S[lane][d] : 0.0f;
    }
    if (act) {
      const float4* m4 = reinterpret_cast<const float4*>(a.m + q);
      const float4* v4 = reinterpret_cast<const float4*>(a.v + q);
      float mm[DIMP], vv[DIMP];
#pragma unroll
      for (int i = 0; i < DIMP / 4; ++i) {
        const float4 x = __ldcs(m4 + i), y = __ldcs(v4 + i);
        mm[4 * i] = x.x; mm[4 * i + 1] = x.y; mm[4 * i + 2] = x.z; mm[4 * i + 3] = x.w;
        vv[4 * i] = y.x; vv[4 * i + 1] = y.y; vv[4 * i + 2] = y.z; vv[4 * i + 3] = y.w;
      }
#pragma unroll
      for (int d = 0; d < DIMP; ++d) {  // embedding.rs:266-271
        mm[d] = fadd(mm[d], fmul(a.one_m_b1, fsub(g[d], mm[d])));
        vv[d] = fadd(vv[d], fmul(a.one_m_b2, fsub(fmul(g[d], g[d]), vv[d])));
        e[d] = fadd(e[d], fdiv(fmul(a.lr_ad, mm[d]), fadd(fsqrt(vv[d]), a.epsc)));
      }
      float4* mo = reinterpret_cast<float4*>(a.m + q);
      float4* vo = reinterpret_cast<float4*>(a.v + q);
#pragma unroll
      for (int i = 0; i < DIMP / 4; ++i) {
        __stcs(mo + i, make_float4(mm[4 * i], mm[4 * i + 1], mm[4 * i + 2], mm[4 * i + 3]));
        __stcs(vo + i, make_float4(vv[4 * i], vv[4 * i + 1], vv[4 * i + 2], vv[4 * i + 3]));
      }
    }
    float4* eo = reinterpret_cast<float4*>(a.e_next + q);
#pragma unroll
    for (int i = 0; i < DIMP / 4; ++i)
      eo[i] = make_float4(e[4 * i], e[4 * i + 1], e[4 * i + 2], e[4 * i + 3]);
    if (a.grad_out) {
      float4* go = reinterpret_cast<float4*>(a.grad_out + q);
#pragma unroll
      for (int i = 0; i < DIMP / 4; ++i)
        go[i] = make_float4(g[4 * i], g[4 * i + 1], g[4 * i + 2], g[4 * i + 3]);
    }
  }
}

// ---------------------------------------------------------------------------
// Fast path: per-epoch gradient slots.
//
// The epochs-per-sample schedule and the negative draws do not depend on the
// embedding, so the set-up lists, for every epoch and every 32-node tile, the
// terms of the reference's gradient sums in their order: one slot (source
// row, tile-local node | 32 for a negative) per fired incidence entry and per
// negative sample it draws. The epoch kernel streams its tile's slots instead
// of scanning fire bits.
// ---------------------------------------------------------------------------
// Per-edge schedule (n_epochs <= 64): thread per undirected edge runs the
// recurrence once (embedding.rs:274-286) and stores the epochs in which the
// edge fires as a bit mask, and its negative count per epoch as two bit
// planes (bit 0 and bit 1 of the count; counts above 3 are caught through
// max_neg, and the per-entry path is used then). Both incidence copies of the
// edge take their fire pattern from here.
__global__ void k_edge_sched(const float* __restrict__ e_ps, int64_t U, int32_t ne,
                             float neg_factor, unsigned long long* __restrict__ fire_mask,
                             unsigned long long* __restrict__ neg_lo,
                             unsigned long long* __restrict__ neg_hi,
                             unsigned long long* __restrict__ max_neg) {
  const unsigned FULL = 0xffffffffu;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = e < U;
  const float ps = valid ? e_ps[e] : 3.0e38f;
  const float pn = fmul(ps, neg_factor);
  float ns = ps, nn = pn, mx = 0.0f;
  uint32_t fm[2] = {0u, 0u}, n0[2] = {0u, 0u}, n1[2] = {0u, 0u};  // epochs 0-31, 32-63
  // the same recurrence as Sched::stepf, with the count kept in float and its
  // two low bits taken by comparisons (count 3 stands for 3 or more)
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int32_t t_end = min(ne, 32 * (h + 1));
    float tf = (float)(32 * h);
    uint32_t bit = 1u;
    for (int32_t t = 32 * h; t < t_end; ++t, tf = fadd(tf, 1.0f), bit <<= 1) {
      if (!(ns > tf)) fm[h] |= bit;  // fires (also for a NaN schedule, which never updates)
      if (ns <= tf) {
        ns = fadd(ns, ps);
        const float x = floorf(fdiv(fsub(tf, nn), pn));
        const float c = (x > 0.0f && x < 18446744073709551616.0f) ? x : 0.0f;
        nn = fadd(nn, fmul(c, pn));
        if (c == 1.0f || c >= 3.0f) n0[h] |= bit;
        if (c >= 2.0f) n1[h] |= bit;
        mx = fmaxf(mx, c);
      }
    }
  }
  if (valid) {
    fire_mask[e] = ((unsigned long long)fm[1] << 32) | fm[0];
    neg_lo[e] = ((unsigned long long)n0[1] << 32) | n0[0];
    neg_hi[e] = ((unsigned long long)n1[1] << 32) | n1[0];
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(FULL, mx, o));
  if ((threadIdx.x & 31) == 0 && mx > 0.0f)
    atomicMax(max_neg, mx >= 1.8446744e19f ? ~0ull : (unsigned long long)mx);
}

// 32 x 32 bit transpose across a warp: lane l passes row word x (bit c =
// element (l, c)); lane c receives column c (bit l = element (l, c)), which
// is __ballot_sync of bit c. Five butterfly stages swap off-diagonal blocks.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x, int lane) {
#pragma unroll
  for (int j = 16; j >= 1; j >>= 1) {
    const uint32_t m = j == 16 ? 0x0000FFFFu
                     : j == 8  ? 0x00FF00FFu
                     : j == 4  ? 0x0F0F0F0Fu
                     : j == 2  ? 0x33333333u
                               : 0x55555555u;
    const uint32_t y = __shfl_xor_sync(0xffffffffu, x, j);
    x = (lane & j) ? ((x & ~m) | ((y >> j) & m)) : ((x & m) | ((y << j) & ~m));
  }
  return x;
}

// Fire and negative-count bit planes in incidence order (n_epochs <= 64).
// F[t * W + w] bit l = entry 32 w + l fires in epoch t; N0 / N1 hold bits 0 /
// 1 of its negative count (upper entries only). Block of 8 warps per 32 words:
// each warp takes the masks of 4 words and transposes them (lane t receives
// epoch t and t + 32); the words are staged in shared memory and every plane
// row leaves as one 128-byte line. Upper entries read their edge's masks
// (consecutive edges); a lower entry's fire mask is the same recurrence run
// on its own epochs-per-sample, which equals its upper twin's (both copies of
// an edge carry the same value).
constexpr int PLANE_BLOCK_WORDS = 32;
__global__ void __launch_bounds__(256) k_inc_planes(
    const uint32_t* __restrict__ inc_eidx, const uint8_t* __restrict__ inc_up,
    const float* __restrict__ inc_ps, int64_t n_inc,
    int64_t W, int32_t ne, const unsigned long long* __restrict__ edge_fire,
    const unsigned long long* __restrict__ edge_neg_lo,
    const unsigned long long* __restrict__ edge_neg_hi, uint32_t* __restrict__ fplane,
    uint32_t* __restrict__ nplane0, uint32_t* __restrict__ nplane1) {
  __shared__ uint32_t sbuf[3][64][PLANE_BLOCK_WORDS + 1];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t w0 = (int64_t)blockIdx.x * PLANE_BLOCK_WORDS;
  constexpr int J = PLANE_BLOCK_WORDS / 8;
  uint32_t e[J];
  bool up[J], ok[J];
  float ps[J];
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const int64_t p = ((w0 + wid * J + j) << 5) + lane;
    ok[j] = p < n_inc;
    up[j] = ok[j] && inc_up[p];
    e[j] = up[j] ? inc_eidx[p] : 0u;
    ps[j] = (ok[j] && !up[j]) ? inc_ps[p] : 3.0e38f;
  }
  unsigned long long fm[J], g0[J], g1[J];
#pragma unroll
  for (int j = 0; j < J; ++j) {
    fm[j] = up[j] ? edge_fire[e[j]] : 0ull;
    g0[j] = up[j] ? edge_neg_lo[e[j]] : 0ull;
    g1[j] = up[j] ? edge_neg_hi[e[j]] : 0ull;
  }
#pragma unroll
  for (int j = 0; j < J; ++j) {  // lower entries: fires only (embedding.rs:274-279)
    if (ok[j] && !up[j]) {
      float ns = ps[j];
      uint32_t m[2] = {0u, 0u};
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int32_t t_end = min(ne, 32 * (h + 1));
        for (int32_t t = 32 * h; t < t_end; ++t) {
          const float tf = (float)t;
          m[h] |= (!(ns > tf) ? 1u : 0u) << (t - 32 * h);
          if (ns <= tf) ns = fadd(ns, ps[j]);
        }
      }
      fm[j] = ((unsigned long long)m[1] << 32) | m[0];
    }
  }
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const int col = wid * J + j;
    sbuf[0][lane][col] = warp_transpose32((uint32_t)fm[j], lane);
    sbuf[0][lane + 32][col] = warp_transpose32((uint32_t)(fm[j] >> 32), lane);
    sbuf[1][lane][col] = warp_transpose32((uint32_t)g0[j], lane);
    sbuf[1][lane + 32][col] = warp_transpose32((uint32_t)(g0[j] >> 32), lane);
    sbuf[2][lane][col] = warp_transpose32((uint32_t)g1[j], lane);
    sbuf[2][lane + 32][col] = warp_transpose32((uint32_t)(g1[j] >> 32), lane);
  }
  __syncthreads();
  const int64_t w = w0 + lane;
  if (w >= W) return;
  for (int r = wid; r < 3 * ne; r += 8) {
    const int kind = r / ne, t = r - kind * ne;
    uint32_t* dst = kind == 0 ? fplane : kind == 1 ? nplane0 : nplane1;
    dst[(int64_t)t * W + w] = sbuf[kind][t][lane];
  }
}

// Words [wb, we) of a tile's entries [P0, P1) with the bits outside masked.
__device__ __forceinline__ uint32_t tile_word(const uint32_t* __restrict__ plane, int64_t w,
                                              int64_t wb, int64_t we, uint32_t lo_mask,
                                              uint32_t hi_mask) {
  if (w >= we) return 0u;
  uint32_t x = plane[w];
  if (w == wb) x &= lo_mask;
  if (w == we - 1) x &= hi_mask;
  return x;
}

// Count pass from the planes: warp per tile; slots per epoch = fired entries
// + their negatives (N0 + 2 N1), written to counts[t * ntiles + tile]. The
// loads of 8 epochs are issued together (the pass is latency-bound), and the
// per-epoch totals of fired entries and negatives (fired[t], negs[t]) are
// summed in shared memory by the block's 8 warps before one global atomic each.
constexpr int COUNT_EU = 8;
__global__ void __launch_bounds__(256) k_plane_count(
    const int64_t* __restrict__ inc_ptr, int64_t n, int64_t ntiles, int64_t W, int32_t ne,
    const uint32_t* __restrict__ fplane, const uint32_t* __restrict__ nplane0,
    const uint32_t* __restrict__ nplane1, int32_t* __restrict__ counts,
    unsigned long long* __restrict__ fired, unsigned long long* __restrict__ negs) {
  __shared__ unsigned long long sfired[64], snegs[64];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < 64; i += blockDim.x) sfired[i] = snegs[i] = 0ull;
  __syncthreads();
  const int64_t tile = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (tile < ntiles) {
    const int64_t v0 = tile * TILE;
    const int nt = (int)min((int64_t)TILE, n - v0);
    const int64_t P0 = inc_ptr[v0], P1 = inc_ptr[v0 + nt];
    const int64_t wb = P0 >> 5, we = P1 > P0 ? ((P1 - 1) >> 5) + 1 : wb;
    const uint32_t lo_mask = ~0u << (P0 & 31);
    const uint32_t hi_mask = ~0u >> (31 - (int)((P1 - 1) & 31));
    for (int32_t t0 = 0; t0 < ne; t0 += COUNT_EU) {
      int cf[COUNT_EU], cn[COUNT_EU];
#pragma unroll
      for (int u = 0; u < COUNT_EU; ++u) cf[u] = cn[u] = 0;
      for (int64_t w = wb + lane; w < we; w += 32) {
        uint32_t x[COUNT_EU], y0[COUNT_EU], y1[COUNT_EU];
#pragma unroll
        for (int u = 0; u < COUNT_EU; ++u) {
          const int64_t po = (int64_t)min(t0 + u, ne - 1) * W;
          x[u] = tile_word(fplane + po, w, wb, we, lo_mask, hi_mask);
          y0[u] = tile_word(nplane0 + po, w, wb, we, lo_mask, hi_mask);
          y1[u] = tile_word(nplane1 + po, w, wb, we, lo_mask, hi_mask);
        }
#pragma unroll
        for (int u = 0; u < COUNT_EU; ++u) {
          cf[u] += __popc(x[u]);
          cn[u] += __popc(y0[u]) + 2 * __popc(y1[u]);
        }
      }
#pragma unroll
      for (int u = 0; u < COUNT_EU; ++u) {
        const int32_t t = t0 + u;
        const int f = __reduce_add_sync(FULL, cf[u]), g = __reduce_add_sync(FULL, cn[u]);
        if (lane == 0 && t < ne) {
          counts[(int64_t)t * ntiles + tile] = f + g;
          if (f) atomicAdd_block(&sfired[t], (unsigned long long)f);
          if (g) atomicAdd_block(&snegs[t], (unsigned long long)g);
        }
      }
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < ne; t += blockDim.x) {
    if (sfired[t]) atomicAdd(&fired[t], sfired[t]);
    if (snegs[t]) atomicAdd(&negs[t], snegs[t]);
  }
}

// Position of the r-th (from 0) set bit of m; some lane index for r >= popc(m).
__device__ __forceinline__ int nth_set_bit(uint32_t m, int r) {
  int pos = 0;
#pragma unroll
  for (int w = 16; w >= 1; w >>= 1) {
    const int c = __popc(m & ((1u << w) - 1u));
    if (c <= r) {
      r -= c;
      m >>= w;
      pos += w;
    }
  }
  return pos;
}

// Fill pass from the planes, block per (tile, FILL_EPB epochs). The block
// stages the tile's partner ids and each entry's tile-local node in shared
// memory (FILL_SEG entries at a time, coalesced); warp w then writes the
// slots of epoch FILL_EPB * g + w. Per 32-word window of fire bits, lane l
// takes word l: its slot count (fired entries + their negatives) and its
// negative-draw count are prefix-summed over the lanes, and the lane walks its
// word's fired entries in order, storing each attraction slot at its place and
// queueing its negatives (slot position, edge, draw index) in shared memory.
// The queue is then drawn (Philox) 32 at a time by the whole warp. A window
// with more draws than the queue holds draws them inline instead (the same
// draws at the same places). Every (epoch, tile) segment holds the terms in
// the order of the reference's serial sum: entries in incidence order, each
// attraction followed by its negatives.
constexpr int FILL_EPB = 8;
constexpr int FILL_SEG = 4096;
constexpr int FILL_Q = 128;  // queued draws per warp and window
struct FillJob {
  int64_t q;        // slot index
  uint32_t eidx;    // edge id
  uint32_t jn;      // draw index j | tile-local node << 8
};
struct PlaneFillSmem {
  uint32_t part[FILL_SEG];           // partner of each staged entry
  uint8_t node[FILL_SEG];            // tile-local node of each staged entry
  int64_t pb[TILE + 1];              // incidence offsets of the tile's nodes
  int64_t eb[TILE];                  // edge-id bases of the tile's nodes
  FillJob job[FILL_EPB][FILL_Q];     // per-warp draw queues
};

// A gradient slot is one word: (source row << 6) | (1 << 5 for a negative
// sample) | tile-local node. Plans with 2^26 or more nodes take the scan path.
constexpr int SLOT_ROW_SHIFT = 6;
constexpr int64_t SLOT_MAX_ROWS = (int64_t)1 << 26;
__device__ __forceinline__ uint32_t make_slot(uint32_t row, uint32_t node_flags) {
  return (row << SLOT_ROW_SHIFT) | node_flags;
}

__device__ __forceinline__ uint32_t negative_slot(uint64_t seed, uint32_t j, int32_t t, uint32_t eidx,
                                               uint32_t node, int64_t v0, uint32_t n_total,
                                               const uint32_t* __restrict__ prob_of_node,
                                               const ProbInfo* __restrict__ prob) {
  uint32_t nb = 0, np = n_total;
  uint64_t sd = seed;
  if (prob_of_node) {
    const ProbInfo pi = prob[prob_of_node[v0 + node]];
    nb = pi.node_base;
    np = pi.n;
    sd = pi.seed;
  }
  return make_slot(nb + negative_draw(sd, j, (uint32_t)t, eidx, np), node | 32u);
}

__global__ void __launch_bounds__(32 * FILL_EPB) k_plane_fill(
    const int64_t* __restrict__ inc_ptr, const uint32_t* __restrict__ inc_other,
    const int64_t* __restrict__ eidx_base, int64_t n, int64_t ntiles, int64_t W, int32_t ne,
    const uint32_t* __restrict__ fplane, const uint32_t* __restrict__ nplane0,
    const uint32_t* __restrict__ nplane1, const int64_t* __restrict__ tile_off,
    const uint32_t* __restrict__ prob_of_node, const ProbInfo* __restrict__ prob,
    uint64_t seed, uint32_t* __restrict__ slots) {
  __shared__ PlaneFillSmem sm;
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int ngroups = (ne + FILL_EPB - 1) / FILL_EPB;
  const int64_t tile = blockIdx.x / ngroups;
  const int32_t t = (int32_t)(blockIdx.x % ngroups) * FILL_EPB + wid;
  const int64_t v0 = tile * TILE;
  const int nt = (int)min((int64_t)TILE, n - v0);
  if (threadIdx.x <= TILE) sm.pb[threadIdx.x] = inc_ptr[v0 + min((int)threadIdx.x, nt)];
  if (threadIdx.x < TILE) sm.eb[threadIdx.x] = (int)threadIdx.x < nt ? eidx_base[v0 + threadIdx.x] : 0;
  __syncthreads();
  const int64_t P0 = sm.pb[0], P1 = sm.pb[nt];
  if (P1 <= P0) return;  // the whole block: no entries
  const bool active = t < ne;
  int64_t cur = active ? tile_off[(int64_t)t * ntiles + tile] : 0;
  const int64_t po = (int64_t)t * W;
  FillJob* job = sm.job[wid];
  for (int64_t sb = P0; sb < P1; sb += FILL_SEG) {
    const int64_t se = min(sb + (int64_t)FILL_SEG, P1);
    __syncthreads();  // the previous segment's readers are done
    for (int64_t p = sb + threadIdx.x; p < se; p += blockDim.x) {
      sm.part[p - sb] = inc_other[p];
      int l = 0;  // last node l < nt with pb[l] <= p (empty rows are skipped)
#pragma unroll
      for (int step = 16; step >= 1; step >>= 1)
        if (l + step < nt && sm.pb[l + step] <= p) l += step;
      sm.node[p - sb] = (uint8_t)l;
    }
    __syncthreads();
    if (!active) continue;
    const int64_t wb = sb >> 5, we = ((se - 1) >> 5) + 1;
    const uint32_t lo_mask = ~0u << (sb & 31);
    const uint32_t hi_mask = ~0u >> (31 - (int)((se - 1) & 31));
    for (int64_t ws = wb; ws < we; ws += 32) {
      const int64_t w = ws + lane;
      uint32_t f = tile_word(fplane + po, w, wb, we, lo_mask, hi_mask);
      // negative bits are set only on fired entries: masking by f keeps the segment's
      const uint32_t g0 = f ? nplane0[po + w] & f : 0u, g1 = f ? nplane1[po + w] & f : 0u;
      const int nneg = __popc(g0) + 2 * __popc(g1);
      int sincl = __popc(f) + nneg, jincl = nneg;  // inclusive prefix sums over lanes
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, sincl, o), z = __shfl_up_sync(FULL, jincl, o);
        if (lane >= o) {
          sincl += y;
          jincl += z;
        }
      }
      const int stot = __shfl_sync(FULL, sincl, 31), jtot = __shfl_sync(FULL, jincl, 31);
      if (stot == 0) continue;
      const bool queued = jtot <= FILL_Q;
      int64_t q = cur + sincl - (__popc(f) + nneg);
      int jq = jincl - nneg;
      __syncwarp();  // the previous window's drain has read its jobs
      while (f) {
        const int b = __ffs(f) - 1;
        f &= f - 1;
        const int64_t p = (w << 5) + b;
        const int li = (int)(p - sb);
        const uint32_t node = sm.node[li];
        slots[q++] = make_slot(sm.part[li], node);
        const uint32_t nn = ((g0 >> b) & 1u) | (((g1 >> b) & 1u) << 1);
        if (nn) {
          const uint32_t eidx = (uint32_t)(p + sm.eb[node]);
          for (uint32_t j = 0; j < nn; ++j, ++q) {
            if (queued)
              job[jq++] = FillJob{q, eidx, j | (node << 8)};
            else
              slots[q] = negative_slot(seed, j, t, eidx, node, v0, (uint32_t)n, prob_of_node, prob);
          }
        }
      }
      cur += stot;
      if (queued && jtot > 0) {
        __syncwarp();  // the jobs are in shared memory
        for (int i = lane; i < jtot; i += 32) {
          const FillJob jb = job[i];
          const uint32_t node = jb.jn >> 8;
          slots[jb.q] = negative_slot(seed, jb.jn & 0xffu, t, jb.eidx, node, v0, (uint32_t)n,
                                      prob_of_node, prob);
        }
      }
    }
  }
}

// Count pass (general path): warp per tile; each lane runs the
// epochs-per-sample recurrence of one incidence entry over all epochs. Slots
// per epoch of the tile (fired entries + their negatives, saturating at 2^30)
// accumulate in shared memory (lane 0); per-epoch totals of fired entries
// and negatives go to fired[t] / negs[t], and the largest negative count per
// entry and epoch to *max_neg.
__global__ void k_sched_count(const int64_t* __restrict__ inc_ptr,
                              const float* __restrict__ inc_ps,
                              const uint8_t* __restrict__ inc_up, int64_t n,
                              int64_t ntiles, int32_t ne, float neg_factor,
                              int32_t* __restrict__ counts,
                              unsigned long long* __restrict__ max_neg,
                              unsigned long long* __restrict__ fired,
                              unsigned long long* __restrict__ negs) {
  extern __shared__ int32_t cnt_all[];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  int32_t* cnt = cnt_all + (size_t)wib * ne;
  const int64_t tile = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
  if (tile >= ntiles) return;
  for (int32_t t = lane; t < ne; t += 32) cnt[t] = 0;
  __syncwarp();
  const int64_t v0 = tile * TILE;
  const int nt = (int)min((int64_t)TILE, n - v0);
  const int64_t P0 = inc_ptr[v0], P1 = inc_ptr[v0 + nt];
  float mx = 0.0f;
  for (int64_t base = P0 & ~(int64_t)31; base < P1; base += 32) {
    const int64_t p = base + lane;
    const bool valid = p >= P0 && p < P1;
    Sched sc;
    sc.init(valid ? inc_ps[p] : 3.0e38f, neg_factor, valid && inc_up[p]);
    for (int32_t t = 0; t < ne; ++t) {
      float c = 0.0f;
      const bool f = valid && sc.stepf((float)t, &c);
      mx = fmaxf(mx, c);
      const uint32_t nn = c >= (float)NEG_LIMIT ? (uint32_t)NEG_LIMIT : (uint32_t)c;
      const uint32_t nf = __popc(__ballot_sync(FULL, f));
      if (nf == 0) continue;
      const uint32_t ng = __reduce_add_sync(FULL, f ? nn : 0u);
      if (lane == 0) {
        cnt[t] = (int32_t)min((int64_t)cnt[t] + nf + ng, (int64_t)1 << 30);
        atomicAdd(&fired[t], (unsigned long long)nf);
        if (ng) atomicAdd(&negs[t], (unsigned long long)ng);
      }
    }
  }
  __syncwarp();
  for (int32_t t = lane; t < ne; t += 32) counts[(int64_t)t * ntiles + tile] = cnt[t];
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(FULL, mx, o));
  if (lane == 0 && mx > 0.0f)
    atomicMax(max_neg, mx >= 1.8446744e19f ? ~0ull : (unsigned long long)mx);
}

// Fill pass (general path): the same recurrence; each fired entry writes its
// slots (attraction, then negatives j = 0.. drawn with Philox counter
// (j, epoch, edge)) at the per-epoch cursor of the tile (shared memory,
// lane 0), after the slots of the lower lanes.
__global__ void k_sched_fill(const int64_t* __restrict__ inc_ptr,
                             const uint32_t* __restrict__ inc_other,
                             const float* __restrict__ inc_ps,
                             const uint8_t* __restrict__ inc_up,
                             const int64_t* __restrict__ eidx_base, int64_t n,
                             int64_t ntiles, int32_t ne, float neg_factor,
                             const int64_t* __restrict__ tile_off,
                             const uint32_t* __restrict__ prob_of_node,
                             const ProbInfo* __restrict__ prob, uint64_t seed,
                             uint32_t* __restrict__ slots) {
  extern __shared__ int64_t cursors[];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  int64_t* cur = cursors + (size_t)wib * ne;
  const int64_t tile = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
  if (tile >= ntiles) return;
  const int64_t v0 = tile * TILE;
  const int nt = (int)min((int64_t)TILE, n - v0);
  const int64_t pbl = inc_ptr[v0 + min(lane, nt)];  // lanes >= nt hold the end
  const int64_t ebl = (lane < nt) ? eidx_base[v0 + lane] : 0;
  const int64_t P0 = __shfl_sync(FULL, pbl, 0);
  const int64_t P1 = inc_ptr[v0 + nt];  // nt may be 32: no lane holds the end
  if (lane == 0)
    for (int32_t t = 0; t < ne; ++t) cur[t] = tile_off[(int64_t)t * ntiles + tile];
  const uint32_t n_total = (uint32_t)n;
  for (int64_t base = P0 & ~(int64_t)31; base < P1; base += 32) {
    const int64_t p = base + lane;
    const bool valid = p >= P0 && p < P1;
    int node = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
      const int64_t st = __shfl_sync(FULL, pbl, node + step);
      if (node + step < nt && st <= p) node += step;
    }
    const int64_t eb = __shfl_sync(FULL, ebl, node);
    const uint32_t other = valid ? inc_other[p] : 0u;
    const uint32_t eidx = (uint32_t)(p + eb);
    uint32_t nb = 0, np = n_total;
    uint64_t sd = seed;
    if (prob_of_node && valid) {
      const ProbInfo pi = prob[prob_of_node[v0 + node]];
      nb = pi.node_base;
      np = pi.n;
      sd = pi.seed;
    }
    Sched sc;
    sc.init(valid ? inc_ps[p] : 3.0e38f, neg_factor, valid && inc_up[p]);
    for (int32_t t = 0; t < ne; ++t) {
      uint64_t nn = 0;
      const bool f = valid && sc.step((float)t, &nn);
      if (__ballot_sync(FULL, f) == 0) continue;
      const int64_t c = f ? 1 + (int64_t)nn : 0;
      int64_t incl = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
      }
      int64_t o0 = (lane == 0) ? cur[t] : 0;
      o0 = __shfl_sync(FULL, o0, 0);
      if (f) {
        int64_t q = o0 + incl - c;
        slots[q] = make_slot(other, (uint32_t)node);
        for (uint64_t j = 0; j < nn; ++j)
          slots[++q] = make_slot(nb + negative_draw(sd, (uint32_t)j, (uint32_t)t, eidx, np),
                                 (uint32_t)node | 32u);
      }
      const int64_t tot = __shfl_sync(FULL, incl, 31);
      if (lane == 0) cur[t] = o0 + tot;
    }
  }
}

// Per-epoch active nodes (a fired entry, i.e. an attraction slot) from the
// slots (on request).
__global__ void k_slot_stats(const int64_t* __restrict__ tile_off,
                             const uint32_t* __restrict__ slots, int64_t ntiles, int32_t ne,
                             unsigned long long* __restrict__ active) {
  const unsigned FULL = 0xffffffffu;
  const int64_t tile = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (tile >= ntiles) return;
  for (int32_t t = 0; t < ne; ++t) {
    const int64_t r0 = tile_off[(int64_t)t * ntiles + tile];
    const int64_t r1 = tile_off[(int64_t)t * ntiles + tile + 1];
    uint32_t mask = 0;
    for (int64_t r = r0 + lane; r < r1; r += 32) {
      const uint32_t y = slots[r];
      if (!(y & 32u)) mask |= 1u << (y & 31u);
    }
    mask = __reduce_or_sync(FULL, mask);
    if (lane == 0 && mask) atomicAdd(&active[t], (unsigned long long)__popc(mask));
  }
}

// One epoch, slots path: persistent warps; each takes the next 32-node tile
// in tile_order (heaviest first) from the epoch's work counter. The tile's
// slots of the epoch come in windows of SLOT_WIN. Phase 1: each lane computes
// slot contributions (attraction, embedding.rs:213-221, or repulsion,
// embedding.rs:237-245, from the slot's source row and the node's own row)
// into shared memory, SLOT_U slots at a time with all loads and gathers
// issued first; the first slot of each node run records its position.
// Phase 2: the slots are node-major in the order of the reference's serial
// sum (embedding.rs:194-253); each node present in the window is summed by
// SLOT_PARTS lanes, each adding its DIMP / SLOT_PARTS dims of the node's run,
// in slot order, onto the node's running gradient in shared memory.
// Then Adam (embedding.rs:256-272), lane per node.
template <int DIMP>
constexpr int slot_parts() { return DIMP >= 8 ? 2 : 1; }

template <int DIMP, int WIN>
struct alignas(16) SlotSmem {
  float rows[TILE][DIMP];      // e_cur rows of the tile's nodes
  float c[WIN][DIMP];          // contributions of the window's slots
  float S[TILE][DIMP];         // running gradients
  int32_t start[TILE];         // first window slot of each node's run (or none)
  int32_t end[TILE];           // one past its last
};

// Contribution of one slot; a signed zero where the reference adds nothing
// (adding +0 or -0 leaves the running sum unchanged: it starts at +0 and never
// becomes -0). One division serves both kinds; a negative sample equal to the
// node itself has dsq = 0 and contributes nothing, like the reference's skip.
// The "adds nothing" case zeroes the coefficient before the product, and an
// attraction's clamp bounds are infinite, so each dimension is one product,
// one max and one min.
template <int DIMP>
__device__ __forceinline__ void slot_contrib(float (&c)[DIMP], bool neg,
                                             const float (&ev)[DIMP],
                                             const float (&row)[DIMP], float two_noise,
                                             float gamma4) {
  float2 diff[DIMP / 2];
  float dsq = 0.0f;
#pragma unroll
  for (int h = 0; h < DIMP / 2; ++h) {
    diff[h] = fsub2(make_float2(ev[2 * h], ev[2 * h + 1]), make_float2(row[2 * h], row[2 * h + 1]));
    const float2 sq = fmul2(diff[h], diff[h]);
    dsq = fadd(fadd(dsq, sq.x), sq.y);  // serial, dims in order
  }
  const float dist = fsqrt(dsq);
  const float num = neg ? gamma4 : fsub(-fmul(two_noise, dist), 2.0f);
  const float den = neg ? fmul(fadd(1.0f, fmul(0.25f, dsq)), dsq)
                        : fadd(fsub(fmul(2.0f, dsq), fmul(0.5f, dist)), 1.0f);
  const bool on = neg ? (dsq > 0.01f) : (dsq >= 1e-8f);
  const float k = on ? fdiv(num, den) : 0.0f;
  const float lo = neg ? -4.0f : -__int_as_float(0x7f800000);
  const float hi = neg ? 4.0f : __int_as_float(0x7f800000);
#pragma unroll
  for (int h = 0; h < DIMP / 2; ++h) {
    const float2 x = fmul2(make_float2(k, k), diff[h]);
    c[2 * h] = fminf(fmaxf(x.x, lo), hi);
    c[2 * h + 1] = fminf(fmaxf(x.y, lo), hi);
  }
}

// Phase 1 for U slots per lane: window slots ib + 32 u + lane, u < U.
template <int DIMP, int WIN, int U, bool COH>
__device__ __forceinline__ void slot_group(const EpochArgs& a, SlotSmem<DIMP, WIN>& sm,
                                           const uint32_t* __restrict__ wslots, int ib, int wn,
                                           int lane, int& carry,
                                           float two_noise, float gamma4) {
  const unsigned FULL = 0xffffffffu;
  uint32_t sl[U];
  float row[U][DIMP];
#pragma unroll
  for (int u = 0; u < U; ++u) {  // past the end: the window's last slot again
    const int i = ib + 32 * u + lane;
    sl[u] = __ldcs(wslots + (i < wn ? i : wn - 1));
  }
#pragma unroll
  for (int u = 0; u < U; ++u)
    load_row<DIMP, COH>(a.e_cur + (size_t)(sl[u] >> SLOT_ROW_SHIFT) * DIMP, row[u]);
#pragma unroll
  for (int u = 0; u < U; ++u) {  // run starts (a repeated last slot starts nothing)
    const int i = ib + 32 * u + lane;
    const int node = (int)(sl[u] & 31u);
    int prev = __shfl_up_sync(FULL, node, 1);
    if (lane == 0) prev = carry;
    carry = __shfl_sync(FULL, node, 31);
    if (i < wn && node != prev) sm.start[node] = i;
  }
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int i = ib + 32 * u + lane;
    if (i < wn) {
      const int node = (int)(sl[u] & 31u);
      float ev[DIMP], c[DIMP];
#pragma unroll
      for (int d = 0; d < DIMP; ++d) ev[d] = sm.rows[node][d];
      slot_contrib<DIMP>(c, (sl[u] & 32u) != 0, ev, row[u], two_noise, gamma4);
      float4* cd = reinterpret_cast<float4*>(&sm.c[i][0]);
#pragma unroll
      for (int q = 0; q < DIMP / 4; ++q)
        cd[q] = make_float4(c[4 * q], c[4 * q + 1], c[4 * q + 2], c[4 * q + 3]);
    }
  }
}

template <int DIMP, int WIN, int SU, bool COH>
__device__ __forceinline__ void slot_tile(const EpochArgs& a, SlotSmem<DIMP, WIN>& sm, int64_t tile,
                                          int lane) {
  const unsigned FULL = 0xffffffffu;
  const int64_t v0 = tile * TILE;
  const int nt = (int)min((int64_t)TILE, (int64_t)a.n_total - v0);
  const int64_t s0 = a.tile_off[tile], s1 = a.tile_off[tile + 1];
  __syncwarp();  // the previous tile's readers of the shared rows and sums are done
  {
    const float4* src = reinterpret_cast<const float4*>(a.e_cur + (size_t)v0 * DIMP);
    float4* dst = reinterpret_cast<float4*>(&sm.rows[0][0]);
    for (int i = lane; i < nt * (DIMP / 4); i += 32) dst[i] = COH ? __ldcg(src + i) : __ldg(src + i);
    float4* sz = reinterpret_cast<float4*>(&sm.S[0][0]);
    for (int i = lane; i < TILE * (DIMP / 4); i += 32) sz[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  const float two_noise = fmul(2.0f, a.noise);
  const float gamma4 = fmul(a.gamma, 4.0f);
  uint32_t act_mask = 0;
  for (int64_t w0 = s0; w0 < s1; w0 += WIN) {
    const int wn = (int)min((int64_t)WIN, s1 - w0);
    const uint32_t* wslots = a.slots + w0;
    sm.start[lane] = WIN;  // none
    __syncwarp();
    int carry = -1;  // node of the previous slot of the window
    int ib = 0;
    for (; ib + 32 * SU <= wn; ib += 32 * SU)
      slot_group<DIMP, WIN, SU, COH>(a, sm, wslots, ib, wn, lane, carry, two_noise,
                                     gamma4);
    for (; ib < wn; ib += 32)
      slot_group<DIMP, WIN, 1, COH>(a, sm, wslots, ib, wn, lane, carry, two_noise,
                                    gamma4);
    __syncwarp();
    // run of node l: [start[l], first start of a later node or wn)
    const int st = sm.start[lane];
    int sfx = (st == WIN) ? wn : st;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_down_sync(FULL, sfx, o);
      if (lane + o < 32) sfx = min(sfx, y);
    }
    int en = __shfl_down_sync(FULL, sfx, 1);
    if (lane == 31) en = wn;
    sm.end[lane] = en;
    const uint32_t present = __ballot_sync(FULL, st != WIN);
    act_mask |= present;  // a node's first slot of the epoch is an attraction
    __syncwarp();
    constexpr int PARTS = slot_parts<DIMP>(), PD = DIMP / PARTS;  // dims per lane
    const int ntask = __popc(present) * PARTS;
    for (int tsk = lane; tsk < ntask; tsk += 32) {
      const int node = nth_set_bit(present, tsk / PARTS), d0 = (tsk % PARTS) * PD;
      const int s2b = sm.start[node], s2e = sm.end[node];
      float4* srow = reinterpret_cast<float4*>(&sm.S[node][d0]);
      float4 acc[PD / 4];
#pragma unroll
      for (int q = 0; q < PD / 4; ++q) acc[q] = srow[q];
      for (int s2 = s2b; s2 < s2e; ++s2) {
        const float4* cd = reinterpret_cast<const float4*>(&sm.c[s2][d0]);
#pragma unroll
        for (int q = 0; q < PD / 4; ++q) {
          const float4 x = cd[q];
          const float2 lo = fadd2(make_float2(acc[q].x, acc[q].y), make_float2(x.x, x.y));
          const float2 hi = fadd2(make_float2(acc[q].z, acc[q].w), make_float2(x.z, x.w));
          acc[q] = make_float4(lo.x, lo.y, hi.x, hi.y);
        }
      }
#pragma unroll
      for (int q = 0; q < PD / 4; ++q) srow[q] = acc[q];
    }
    __syncwarp();  // contributions, runs and sums are settled before the next window
  }
  __syncwarp();  // the shared rows are complete for Adam (also with no slots)

  if (lane < nt) {  // Adam, embedding.rs:256-272
    const size_t q = (size_t)(v0 + lane) * DIMP;
    const bool act = (act_mask >> lane) & 1u;
    float e[DIMP], g[DIMP];
#pragma unroll
    for (int d = 0; d < DIMP; ++d) {
      e[d] = sm.rows[lane][d];
      g[d] = act ? sm.S[lane][d] : 0.0f;
    }
    if (act) {
      const float4* m4 = reinterpret_cast<const float4*>(a.m + q);
      const float4* v4 = reinterpret_cast<const float4*>(a.v + q);
      float mm[DIMP], vv[DIMP];
#pragma unroll
      for (int i = 0; i < DIMP / 4; ++i) {
        const float4 x = COH ? __ldcg(m4 + i) : __ldcs(m4 + i);
        const float4 y = COH ? __ldcg(v4 + i) : __ldcs(v4 + i);
        mm[4 * i] = x.x; mm[4 * i + 1] = x.y; mm[4 * i + 2] = x.z; mm[4 * i + 3] = x.w;
        vv[4 * i] = y.x; vv[4 * i + 1] = y.y; vv[4 * i + 2] = y.z; vv[4 * i + 3] = y.w;
      }
#pragma unroll
#pragma unroll
      for (int d = 0; d < DIMP; ++d) {  // scalar: a packed multiply feeding a packed
        // add did not reproduce the unfused result
        mm[d] = fadd(mm[d], fmul(a.one_m_b1, fsub(g[d], mm[d])));
        vv[d] = fadd(vv[d], fmul(a.one_m_b2, fsub(fmul(g[d], g[d]), vv[d])));
        e[d] = fadd(e[d], fdiv(fmul(a.lr_ad, mm[d]), fadd(fsqrt(vv[d]), a.epsc)));
      }
      float4* mo = reinterpret_cast<float4*>(a.m + q);
      float4* vo = reinterpret_cast<float4*>(a.v + q);
#pragma unroll
      for (int i = 0; i < DIMP / 4; ++i) {
        __stcs(mo + i, make_float4(mm[4 * i], mm[4 * i + 1], mm[4 * i + 2], mm[4 * i + 3]));
        __stcs(vo + i, make_float4(vv[4 * i], vv[4 * i + 1], vv[4 * i + 2], vv[4 * i + 3]));
      }
    }
    float4* eo = reinterpret_cast<float4*>(a.e_next + q);
#pragma unroll
    for (int i = 0; i < DIMP / 4; ++i)  // evict-first: keep e_cur's rows in L2 for the gathers
      __stcs(eo + i, make_float4(e[4 * i], e[4 * i + 1], e[4 * i + 2], e[4 * i + 3]));
    if (a.grad_out) {
      float4* go = reinterpret_cast<float4*>(a.grad_out + q);
#pragma unroll
      for (int i = 0; i < DIMP / 4; ++i)
        go[i] = make_float4(g[4 * i], g[4 * i + 1], g[4 * i + 2], g[4 * i + 3]);
    }
  }
}

using EpochKernel = void (*)(EpochArgs);

// Register cap: 7 blocks of 128 threads per SM (72 registers) for DIMP <= 8
// measured fastest; the occupancy it buys outweighs per-warp parallelism.
template <int DIMP, int WIN, int SU>
__global__ void __launch_bounds__(128, DIMP <= 8 ? 7 : 4) k_epoch_slot(EpochArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  SlotSmem<DIMP, WIN>& sm = reinterpret_cast<SlotSmem<DIMP, WIN>*>(smem_raw)[threadIdx.x >> 5];
  const int64_t ntiles = ((int64_t)a.n_total + TILE - 1) / TILE;
  for (;;) {
    unsigned long long w = 0;
    if (lane == 0) w = atomicAdd(a.work_ctr, 1ull);
    w = __shfl_sync(0xffffffffu, w, 0);
    if ((int64_t)w >= ntiles) break;
    slot_tile<DIMP, WIN, SU, false>(a, sm, (int64_t)a.tile_order[w], lane);
  }
}

// ---------------------------------------------------------------------------
// All epochs in one persistent launch (cooperative: every block resident).
// Each epoch runs exactly as k_epoch_slot (tiles from the epoch's work
// counter, heaviest first), reading rows and moments through L2 because they
// were written earlier in the same launch; a grid-wide barrier separates the
// epochs. The barrier waits at most GRID_WAIT_NS; on expiry it records
// ST_WAIT_TIMEOUT, raises an abort word that every block checks, and the
// launch returns.
// ---------------------------------------------------------------------------
struct EpochAllArgs {
  const float4* ep;               // per epoch: gamma, lr * ad_scale, eps', 0
  const int64_t* tile_off;        // all epochs: [t * ntiles + tile]
  unsigned long long* work_ctr;   // per epoch, zeroed before the launch
  float* e0;                      // embedding at epoch t0 (ping-pong with e1)
  float* e1;
  unsigned* bar;                  // arrivals, generation, abort (zeroed)
  int32_t* status;
  int32_t t0, t1;                 // epochs [t0, t1)
  unsigned nblocks;
};
constexpr unsigned long long GRID_WAIT_NS = 2000000000ull;

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ bool grid_barrier(unsigned* bar, unsigned nblocks, int32_t* status) {
  __shared__ int ok_s;
  __syncthreads();  // the block's epoch is done
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned* vbar = bar;
    const unsigned gen = vbar[1];
    __threadfence();  // this block's writes before its arrival
    if (atomicAdd(bar, 1u) == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const uint64_t start = globaltimer_ns();
      while (vbar[1] == gen) {
        if (vbar[2]) {
          ok = 0;
          break;
        }
        if (globaltimer_ns() - start > GRID_WAIT_NS) {
          atomicOr(status, (int32_t)ST_WAIT_TIMEOUT);
          atomicExch(bar + 2, 1u);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    ok_s = ok && !vbar[2];
  }
  __syncthreads();
  return ok_s != 0;
}

template <int DIMP, int WIN, int SU>
__global__ void __launch_bounds__(128, DIMP <= 8 ? 7 : 4)
    k_epoch_slot_all(EpochArgs base, EpochAllArgs x) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  SlotSmem<DIMP, WIN>& sm = reinterpret_cast<SlotSmem<DIMP, WIN>*>(smem_raw)[threadIdx.x >> 5];
  const int64_t ntiles = ((int64_t)base.n_total + TILE - 1) / TILE;
  for (int32_t t = x.t0; t < x.t1; ++t) {
    EpochArgs a = base;
    const int k = t - x.t0;
    a.e_cur = (k & 1) ? x.e1 : x.e0;
    a.e_next = (k & 1) ? x.e0 : x.e1;
    a.tile_off = x.tile_off + (size_t)t * ntiles;
    a.work_ctr = x.work_ctr + t;
    const float4 ep = x.ep[t];
    a.gamma = ep.x;
    a.lr_ad = ep.y;
    a.epsc = ep.z;
    a.epoch = (uint32_t)t;
    for (;;) {
      unsigned long long w = 0;
      if (lane == 0) w = atomicAdd(a.work_ctr, 1ull);
      w = __shfl_sync(0xffffffffu, w, 0);
      if ((int64_t)w >= ntiles) break;
      slot_tile<DIMP, WIN, SU, true>(a, sm, (int64_t)a.tile_order[w], lane);
    }
    if (t + 1 < x.t1 && !grid_barrier(x.bar, x.nblocks, x.status)) return;
  }
}

EpochKernel pick_kernel(int dimp) {
  if (dimp == 4) return k_epoch<4>;
  if (dimp == 8) return k_epoch<8>;
  if (dimp == 16) return k_epoch<16>;
  return nullptr;
}

size_t tile_smem(int dimp) {
  if (dimp == 4) return sizeof(TileSmem<4>);
  if (dimp == 8) return sizeof(TileSmem<8>);
  return sizeof(TileSmem<16>);
}

// Variants of the slots kernel: (slot window, slots per lane per group). All
// give identical results; the autotuner picks one per plan shape.
struct SlotVariant {
  int win, u;
};
constexpr SlotVariant SLOT_VARIANTS[] = {{128, 2}, {64, 2}, {256, 2}, {128, 1}};
constexpr int N_SLOT_VARIANTS = 4;

template <int WIN, int SU>
EpochKernel pick_slot_wu(int dimp) {
  if (dimp == 4) return k_epoch_slot<4, WIN, SU>;
  if (dimp == 8) return k_epoch_slot<8, WIN, SU>;
  return k_epoch_slot<16, WIN, SU>;
}
EpochKernel pick_slot_kernel(int dimp, int kv) {
  switch (kv) {
    case 1: return pick_slot_wu<64, 2>(dimp);
    case 2: return pick_slot_wu<256, 2>(dimp);
    case 3: return pick_slot_wu<128, 1>(dimp);
    default: return pick_slot_wu<128, 2>(dimp);
  }
}
using EpochAllKernel = void (*)(EpochArgs, EpochAllArgs);
template <int WIN, int SU>
EpochAllKernel pick_all_wu(int dimp) {
  if (dimp == 4) return k_epoch_slot_all<4, WIN, SU>;
  if (dimp == 8) return k_epoch_slot_all<8, WIN, SU>;
  return k_epoch_slot_all<16, WIN, SU>;
}
EpochAllKernel pick_all_kernel(int dimp, int kv) {
  switch (kv) {
    case 1: return pick_all_wu<64, 2>(dimp);
    case 2: return pick_all_wu<256, 2>(dimp);
    case 3: return pick_all_wu<128, 1>(dimp);
    default: return pick_all_wu<128, 2>(dimp);
  }
}
template <int WIN>
size_t slot_smem_w(int dimp) {
  if (dimp == 4) return sizeof(SlotSmem<4, WIN>);
  if (dimp == 8) return sizeof(SlotSmem<8, WIN>);
  return sizeof(SlotSmem<16, WIN>);
}
size_t slot_smem(int dimp, int kv) {
  const int win = SLOT_VARIANTS[kv].win;
  return win == 64 ? slot_smem_w<64>(dimp) : win == 256 ? slot_smem_w<256>(dimp)
                                                        : slot_smem_w<128>(dimp);
}

// Warps (node tiles) per thread block of k_epoch; EVOC_WARPS_PER_BLOCK
// overrides (1, 2 or 4). Results do not depend on it.
int default_wpb() {
  int w = 2;
  if (const char* env = std::getenv("EVOC_WARPS_PER_BLOCK")) {
    const int e = std::atoi(env);
    if (e == 1 || e == 2 || e == 4) w = e;
  }
  return w;
}

void launch_epoch(evoc_plan* pl, int32_t t, const float* e_cur, float* e_next,
                  float* grad_out, cudaStream_t s) {
  EpochArgs a;
  a.inc_ptr = pl->inc_ptr.get();
  a.inc_other = pl->inc_other.get();
  a.eidx_base = pl->eidx_base.get();
  a.fire = pl->use_slots ? nullptr : pl->planes.get() + (size_t)t * (1 + pl->P) * pl->W;
  a.W = pl->W;
  a.P = pl->P;
  a.e_cur = e_cur;
  a.e_next = e_next;
  a.m = pl->m.get();
  a.v = pl->v.get();
  a.grad_out = grad_out;
  a.prob_of_node = pl->n_problems > 1 ? pl->prob_of_node.get() : nullptr;
  a.prob = pl->n_problems > 1 ? pl->prob.get() : nullptr;
  a.n_total = (uint32_t)pl->n;
  a.epoch = (uint32_t)t;
  a.seed = pl->seeds.empty() ? 0 : pl->seeds[0];
  a.noise = pl->params.noise_level;
  a.gamma = pl->gamma[t];
  a.lr_ad = pl->lr_ad[t];
  a.epsc = pl->epsc[t];
  a.one_m_b1 = pl->one_m_b1;
  a.one_m_b2 = pl->one_m_b2;
  a.tile_off = nullptr;
  a.tile_order = nullptr;
  a.slots = nullptr;
  a.work_ctr = nullptr;
  const int wpb = pl->lanes;
  const int64_t tiles = (pl->n + TILE - 1) / TILE;
  const unsigned grid = (unsigned)((tiles + wpb - 1) / wpb);
  if (pl->use_slots) {
    a.tile_off = pl->tile_off.get() + (size_t)t * pl->ntiles;
    a.tile_order = pl->tile_order.get();
    a.slots = pl->slots.get();
    a.work_ctr = pl->work_ctr.get() + t;  // zeroed before the epoch loop
    pick_slot_kernel(pl->dimp, pl->kvariant)<<<pl->slot_grid, 32 * wpb,
                                                wpb * slot_smem(pl->dimp, pl->kvariant), s>>>(a);
  } else {
    pick_kernel(pl->dimp)<<<grid, 32 * wpb, wpb * tile_smem(pl->dimp), s>>>(a);
  }
  EVOC_CHECK_LAUNCH();
}

// Epochs [t0, t1) in one cooperative launch (slots path): from e0, ending in
// e0 or e1 by the parity of t1 - t0. Work counters and barrier words are
// zeroed first.
void launch_all_epochs(evoc_plan* pl, int32_t t0, int32_t t1, cudaStream_t s) {
  EpochArgs a;
  std::memset(&a, 0, sizeof(a));
  a.m = pl->m.get();
  a.v = pl->v.get();
  a.prob_of_node = pl->n_problems > 1 ? pl->prob_of_node.get() : nullptr;
  a.prob = pl->n_problems > 1 ? pl->prob.get() : nullptr;
  a.n_total = (uint32_t)pl->n;
  a.seed = pl->seeds.empty() ? 0 : pl->seeds[0];
  a.noise = pl->params.noise_level;
  a.one_m_b1 = pl->one_m_b1;
  a.one_m_b2 = pl->one_m_b2;
  a.tile_order = pl->tile_order.get();
  a.slots = pl->slots.get();
  EpochAllArgs x;
  x.ep = pl->ep_params.get();
  x.tile_off = pl->tile_off.get();
  x.work_ctr = pl->work_ctr.get();
  x.e0 = pl->e0;
  x.e1 = pl->e1;
  x.bar = pl->grid_bar.get();
  x.status = pl->ctx->status.get();
  x.t0 = t0;
  x.t1 = t1;
  x.nblocks = pl->slot_grid;
  EVOC_CUDA(cudaMemsetAsync(pl->work_ctr.get(), 0, pl->work_ctr.bytes(), s));
  EVOC_CUDA(cudaMemsetAsync(pl->grid_bar.get(), 0, pl->grid_bar.bytes(), s));
  void* args[] = {&a, &x};
  const int wpb = pl->lanes;
  EVOC_CUDA(cudaLaunchCooperativeKernel((const void*)pick_all_kernel(pl->dimp, pl->kvariant),
                                        dim3(pl->slot_grid), dim3(32 * wpb), args,
                                        wpb * slot_smem(pl->dimp, pl->kvariant), s));
}

unsigned blocks_for(int64_t threads, int bs = 256) {
  return (unsigned)((threads + bs - 1) / bs);
}

}  // namespace

void concat_graph(const evoc_graph* g, int64_t node_off, int64_t entry_off,
                  int64_t* dptr, uint32_t* didx, cudaStream_t s);
void fill_eidx_src(uint2* out, const uint32_t* e_src, int64_t U, cudaStream_t s);
void add_counts(const int32_t* a, const int32_t* b, int32_t* out, int64_t n,
                cudaStream_t s);

// Launch order of the slots kernel: sort key per tile = ~(its slots over all
// epochs), so that an ascending sort puts the heaviest tiles (hub nodes)
// first and their long serial sums overlap the many light tiles.
__global__ void k_tile_weight(const int32_t* __restrict__ counts, int64_t ntiles, int32_t ne,
                              uint32_t* __restrict__ keys, uint2* __restrict__ vals) {
  const int64_t tile = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tile >= ntiles) return;
  uint64_t tot = 0;
  for (int32_t t = 0; t < ne; ++t) tot += (uint32_t)counts[(int64_t)t * ntiles + tile];
  keys[tile] = ~(uint32_t)min(tot, (uint64_t)0xffffffffu);
  vals[tile] = make_uint2((uint32_t)tile, 0u);
}

__global__ void k_tile_order(const uint2* __restrict__ vals, int64_t ntiles,
                             uint32_t* __restrict__ order) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ntiles) order[i] = vals[i].x;
}

// Slots path of the schedule set-up: per-edge schedule and incidence planes
// (n_epochs <= 64 and at most 3 negatives per edge and epoch) or the
// per-entry recurrence (otherwise), then count pass, offset scan, tile order
// and fill pass. Returns false (nothing built) when EVOC_EPOCH_PATH=scan,
// when the epoch count exceeds the shared-memory cursors, or when the slots
// would take more than half of the free device memory (unless
// EVOC_EPOCH_PATH=slots).
static bool build_slots(evoc_plan* pl, const float* inc_ps, const uint8_t* inc_up,
                        const uint32_t* inc_eidx, const float* e_ps, int64_t U,
                        float neg_factor) {
  cudaStream_t s = pl->ctx->stream;
  const int32_t ne = pl->params.n_epochs;
  const int64_t n = pl->n;
  pl->ntiles = (n + TILE - 1) / TILE;
  const char* env = std::getenv("EVOC_EPOCH_PATH");
  const bool force_scan = env && std::strcmp(env, "scan") == 0;
  const bool force_slots = env && std::strcmp(env, "slots") == 0;
  if (force_scan || (size_t)ne * sizeof(int64_t) > 200 * 1024) return false;
  if (n >= SLOT_MAX_ROWS) return false;  // a slot's row field holds 26 bits
  const int wpb = (int)std::max<size_t>(
      1, std::min<size_t>(4, (200 * 1024) / ((size_t)ne * sizeof(int64_t))));
  const unsigned grid = (unsigned)((pl->ntiles + wpb - 1) / wpb);
  const int64_t cells = (int64_t)ne * pl->ntiles;
  StageTrace trace(s);
  DevBuf<int32_t> counts(cells, s);
  DevBuf<unsigned long long> mx(1, s), tot(2 * ne, s);  // tot: fired[ne], negs[ne]
  EVOC_CUDA(cudaMemsetAsync(mx.get(), 0, sizeof(unsigned long long), s));
  EVOC_CUDA(cudaMemsetAsync(tot.get(), 0, tot.bytes(), s));
  unsigned long long maxneg = 0;
  // n_epochs <= 64: the recurrence runs once per edge into bit masks, turned
  // into incidence-order bit planes that the count and fill passes read.
  bool use_planes = ne <= 64;
  DevBuf<uint32_t> fpl, npl0, npl1;
  int64_t planes_w = 0;
  if (use_planes) {
    DevBuf<unsigned long long> efire(U, s), eneg_lo(U, s), eneg_hi(U, s);
    trace.mark("alloc masks");
    k_edge_sched<<<blocks_for(U), 256, 0, s>>>(e_ps, U, ne, neg_factor, efire.get(),
                                               eneg_lo.get(), eneg_hi.get(), mx.get());
    EVOC_CHECK_LAUNCH();
    EVOC_CUDA(cudaMemcpyAsync(&maxneg, mx.get(), sizeof(maxneg), cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaStreamSynchronize(s));
    trace.mark("edge schedule");
    use_planes = maxneg <= 3;  // the planes hold negative counts 0..3
    if (use_planes) {
      planes_w = (pl->n_inc + 31) / 32;
      const int64_t pw = planes_w * ne;
      fpl.alloc(pw, s);
      npl0.alloc(pw, s);
      npl1.alloc(pw, s);
      k_inc_planes<<<(unsigned)((planes_w + PLANE_BLOCK_WORDS - 1) / PLANE_BLOCK_WORDS), 256,
                     0, s>>>(inc_eidx, inc_up, inc_ps, pl->n_inc, planes_w, ne, efire.get(),
                             eneg_lo.get(), eneg_hi.get(), fpl.get(), npl0.get(), npl1.get());
      EVOC_CHECK_LAUNCH();
      trace.mark("incidence planes");
      k_plane_count<<<blocks_for(pl->ntiles * 32), 256, 0, s>>>(
          pl->inc_ptr.get(), n, pl->ntiles, planes_w, ne, fpl.get(), npl0.get(), npl1.get(),
          counts.get(), tot.get(), tot.get() + ne);
      EVOC_CHECK_LAUNCH();
    }
  }
  if (!use_planes) {
    const size_t csmem = (size_t)wpb * ne * sizeof(int32_t);
    if (csmem > 48 * 1024)
      EVOC_CUDA(cudaFuncSetAttribute((const void*)k_sched_count,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csmem));
    k_sched_count<<<grid, 32 * wpb, csmem, s>>>(pl->inc_ptr.get(), inc_ps, inc_up, n,
                                                pl->ntiles, ne, neg_factor, counts.get(),
                                                mx.get(), tot.get(), tot.get() + ne);
    EVOC_CHECK_LAUNCH();
  }
  trace.mark("count pass");
  DevBuf<int64_t> off(cells + 1, s);
  exclusive_scan_i32_to_i64(counts.get(), off.get(), cells, s);
  int64_t total = 0;
  std::vector<unsigned long long> htot(2 * ne);
  EVOC_CUDA(cudaMemcpyAsync(&total, off.get() + cells, sizeof(int64_t),
                            cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaMemcpyAsync(&maxneg, mx.get(), sizeof(maxneg), cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaMemcpyAsync(htot.data(), tot.get(), tot.bytes(), cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaStreamSynchronize(s));
  if (maxneg > (unsigned long long)NEG_LIMIT)
    throw Error(EVOC_ERR_UNSUPPORTED,
                "more than 2^20 negative samples per edge and epoch "
                "(negative_sample_rate too large)");
  size_t free_b = 0, total_b = 0;
  EVOC_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const double need = (double)sizeof(uint32_t) * (double)total;
  const double avail = (double)free_b + (double)pl->ctx->slot_cache.bytes();  // the cache is reusable
  if (!force_slots && need > 0.5 * avail) return false;
  pl->max_neg = maxneg;
  trace.mark("offset scan + sync");
  {
    DevBuf<uint32_t> keys(pl->ntiles, s);
    DevBuf<uint2> vals(pl->ntiles, s);
    k_tile_weight<<<blocks_for(pl->ntiles), 256, 0, s>>>(counts.get(), pl->ntiles, ne,
                                                          keys.get(), vals.get());
    EVOC_CHECK_LAUNCH();
    radix_sort_pairs(keys.get(), vals.get(), pl->ntiles, 32, s);
    pl->tile_order.alloc(pl->ntiles, s);
    k_tile_order<<<blocks_for(pl->ntiles), 256, 0, s>>>(vals.get(), pl->ntiles,
                                                         pl->tile_order.get());
    EVOC_CHECK_LAUNCH();
  }
  trace.mark("tile order");
  if (total > 0 && pl->ctx->slot_cache.count >= (size_t)total) {
    pl->slots = std::move(pl->ctx->slot_cache);
  } else {
    pl->ctx->slot_cache.release();
    pl->slots.alloc(total, s);
  }
  trace.mark("alloc slots");
  const uint32_t* pon = pl->n_problems > 1 ? pl->prob_of_node.get() : nullptr;
  const ProbInfo* pinfo = pl->n_problems > 1 ? pl->prob.get() : nullptr;
  const uint64_t seed0 = pl->seeds.empty() ? 0 : pl->seeds[0];
  if (use_planes) {
    const int64_t ngroups = (ne + FILL_EPB - 1) / FILL_EPB;
    k_plane_fill<<<(unsigned)(ngroups * pl->ntiles), 32 * FILL_EPB, 0, s>>>(
        pl->inc_ptr.get(), pl->inc_other.get(), pl->eidx_base.get(), n, pl->ntiles, planes_w,
        ne, fpl.get(), npl0.get(), npl1.get(), off.get(), pon, pinfo, seed0, pl->slots.get());
  } else {
    const size_t fsmem = (size_t)wpb * ne * sizeof(int64_t);
    if (fsmem > 48 * 1024)
      EVOC_CUDA(cudaFuncSetAttribute((const void*)k_sched_fill,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem));
    k_sched_fill<<<grid, 32 * wpb, fsmem, s>>>(
        pl->inc_ptr.get(), pl->inc_other.get(), inc_ps, inc_up, pl->eidx_base.get(), n,
        pl->ntiles, ne, neg_factor, off.get(), pon, pinfo, seed0, pl->slots.get());
  }
  EVOC_CHECK_LAUNCH();
  trace.mark("fill pass");
  // fired edges per epoch = fired incidence entries / 2 (both copies fire)
  for (int32_t t = 0; t < ne; ++t) {
    pl->stats[t].fired_edges = (int64_t)(htot[t] / 2);
    pl->stats[t].negatives = (int64_t)htot[ne + t];
  }
  pl->tile_off = std::move(off);
  pl->n_slots = total;
  pl->use_slots = true;
  pl->inc_other.release();
  return true;
}

evoc_ctx* plan_ctx(const evoc_plan* p) { return p->ctx; }
void plan_info(const evoc_plan* p, int64_t* n_edges, int64_t* n_inc,
               int32_t* planes, int32_t* wpb, int64_t* n_slots) {
  if (n_edges) *n_edges = p->n_edges;
  if (n_inc) *n_inc = p->n_inc;
  if (planes) *planes = p->P;
  if (wpb) *wpb = p->lanes;
  if (n_slots) *n_slots = p->use_slots ? p->n_slots : 0;
}
static void load_init(evoc_plan* pl, const float* d_init, cudaStream_t s);
void plan_apply_tuned(evoc_plan* pl);

// Epoch-kernel configuration of a plan: slots-kernel variant, warps per
// block and a cap on persistent blocks per SM (0: as many as fit). The
// persistent grid is recomputed and the captured epoch loop dropped (it is
// captured again with the new launch shape on the next run). Results do not
// depend on the configuration.
void plan_configure(evoc_plan* pl, int variant, int wpb, int bps) {
  if (variant < 0 || variant >= 2 * N_SLOT_VARIANTS)
    throw Error(EVOC_ERR_INVALID_ARGUMENT, "epoch kernel variant out of range");
  const int kv = variant % N_SLOT_VARIANTS;
  const bool all = variant >= N_SLOT_VARIANTS;
  if (wpb != 1 && wpb != 2 && wpb != 4)
    throw Error(EVOC_ERR_INVALID_ARGUMENT, "warps per block must be 1, 2 or 4");
  if (bps < 0) throw Error(EVOC_ERR_INVALID_ARGUMENT, "blocks per SM must be >= 0");
  pl->kvariant = kv;
  pl->lanes = wpb;
  pl->blocks_per_sm = bps;
  pl->all_epochs = all && pl->use_slots;
  if (pl->graph_exec) {
    cudaGraphExecDestroy(pl->graph_exec);
    pl->graph_exec = nullptr;
  }
  if (pl->graph) {
    cudaGraphDestroy(pl->graph);
    pl->graph = nullptr;
  }
  if (!pl->use_slots) return;
  const void* fn = all ? (const void*)pick_all_kernel(pl->dimp, kv)
                       : (const void*)pick_slot_kernel(pl->dimp, kv);
  const size_t smem = (size_t)wpb * slot_smem(pl->dimp, kv);
  if (smem > 48 * 1024)
    EVOC_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int nb = 0, dev = 0, sms = 0;
  EVOC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 32 * wpb, smem));
  if (bps) nb = std::min(nb, bps);
  EVOC_CUDA(cudaGetDevice(&dev));
  EVOC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t want = (int64_t)std::max(nb, 1) * sms;
  const int64_t need = (pl->ntiles + wpb - 1) / wpb;
  pl->slot_grid = (unsigned)std::max<int64_t>(1, std::min(want, need));
}

namespace {
// Autotuner cache: plan shape -> configuration and its time per launch. In
// memory for the process; with EVOC_TUNE_CACHE=<file> also read from and
// appended to that file (one "key variant wpb bps ms" line per shape).
struct TuneEntry {
  int kv, wpb, bps;
  float ms;
};
std::mutex g_tune_mu;
std::map<std::string, TuneEntry> g_tune;
bool g_tune_loaded = false;

void tune_load_locked() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const char* f = std::getenv("EVOC_TUNE_CACHE");
  if (!f || !*f) return;
  std::ifstream in(f);
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    std::string key;
    TuneEntry e{};
    if (ls >> key >> e.kv >> e.wpb >> e.bps >> e.ms && e.kv >= 0 && e.kv < 2 * N_SLOT_VARIANTS &&
        (e.wpb == 1 || e.wpb == 2 || e.wpb == 4) && e.bps >= 0)
      g_tune[key] = e;
  }
}

// The shape a configuration is tuned for: padded row width, nodes and slots
// per epoch (each on a half-octave grid), problem count (one or many), epoch
// count and the device's SM count.
std::string tune_key(const evoc_plan* pl, int sms) {
  const int32_t ne = std::max(pl->params.n_epochs, 1);
  const double spe = (double)pl->n_slots / ne;
  auto bucket = [](double x) { return x < 1.0 ? 0 : (int)std::lround(2.0 * std::log2(x)); };
  std::ostringstream k;
  k << "d" << pl->dimp << "_n" << bucket((double)pl->n) << "_s" << bucket(spe) << "_p"
    << (pl->n_problems > 1 ? "m" : "1") << "_e" << ne << "_sm" << sms;
  return k.str();
}
}  // namespace

// Configures a plan from the tuning cache when its shape was tuned before
// (in this process or in the EVOC_TUNE_CACHE file); otherwise leaves it as it is.
void plan_apply_tuned(evoc_plan* pl) {
  if (!pl->use_slots || !pl->has_edges || pl->params.n_epochs <= 1) return;
  int dev = 0, sms = 0;
  EVOC_CUDA(cudaGetDevice(&dev));
  EVOC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const std::string key = tune_key(pl, sms);
  TuneEntry e{};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_load_locked();
    auto it = g_tune.find(key);
    if (it == g_tune.end()) return;
    e = it->second;
  }
  plan_configure(pl, e.kv, e.wpb, e.bps);
}

// Times every configuration on a sample of this plan's epochs (the real
// slots kernel from a random state, CUDA events on the plan's stream) and
// keeps the fastest; a shape tuned before in this process (or found in the
// EVOC_TUNE_CACHE file) is configured without timing. Plans on the bit-plane
// path have nothing to tune.
void plan_autotune(evoc_plan* pl, int32_t* config, float* ms_out) {
  cudaStream_t s = pl->ctx->stream;
  const int32_t ne = pl->params.n_epochs;
  float best_ms = 0.0f;
  if (pl->use_slots && pl->has_edges && ne > 1) {
    int dev = 0, sms = 0;
    EVOC_CUDA(cudaGetDevice(&dev));
    EVOC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const std::string key = tune_key(pl, sms);
    TuneEntry hit{};
    bool found = false;
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      tune_load_locked();
      auto it = g_tune.find(key);
      if (it != g_tune.end()) {
        hit = it->second;
        found = true;
      }
    }
    if (found) {
      plan_configure(pl, hit.kv, hit.wpb, hit.bps);
      best_ms = hit.ms;
    } else {
      std::vector<int32_t> ts;  // sample epochs spread over the run (epoch 0 fires nothing)
      for (int q = 1; q <= 5; ++q) {
        const int32_t t = std::max(1, std::min(ne - 1, (int32_t)((int64_t)q * ne / 6)));
        if (ts.empty() || ts.back() != t) ts.push_back(t);
      }
      load_init(pl, nullptr, s);
      EVOC_CUDA(cudaMemsetAsync(pl->m.get(), 0, pl->m.bytes(), s));
      EVOC_CUDA(cudaMemsetAsync(pl->v.get(), 0, pl->v.bytes(), s));
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      EVOC_CUDA(cudaEventCreate(&e0));
      EVOC_CUDA(cudaEventCreate(&e1));
      TuneEntry best{0, pl->lanes, 0, 3.0e38f};
      try {
        const int wpbs[3] = {1, 2, 4};
        for (int kv = 0; kv < N_SLOT_VARIANTS; ++kv)
          for (int wpb : wpbs) {
            plan_configure(pl, kv, wpb, 0);
            float total = 0.0f;
            for (int rep = 0; rep < 2; ++rep) {  // the first pass warms up
              EVOC_CUDA(cudaMemsetAsync(pl->work_ctr.get(), 0, pl->work_ctr.bytes(), s));
              EVOC_CUDA(cudaEventRecord(e0, s));
              for (int32_t t : ts) launch_epoch(pl, t, pl->e0, pl->e1, nullptr, s);
              EVOC_CUDA(cudaEventRecord(e1, s));
              EVOC_CUDA(cudaEventSynchronize(e1));
              EVOC_CUDA(cudaEventElapsedTime(&total, e0, e1));
            }
            const float per = total / (float)ts.size();
            if (per < best.ms) best = TuneEntry{kv, wpb, 0, per};
          }
      } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
      }
      // the chosen variant launched per epoch (the captured loop) or as one
      // cooperative launch for all epochs: the faster over a whole run
      {
        float per_epoch_ms = 0.0f, all_ms = 0.0f;
        for (int mode = 0; mode < 2; ++mode) {
          plan_configure(pl, best.kv + (mode ? N_SLOT_VARIANTS : 0), best.wpb, best.bps);
          float el = 0.0f;
          for (int rep = 0; rep < 2; ++rep) {  // the first run captures / warms up
            load_init(pl, nullptr, s);
            EVOC_CUDA(cudaMemsetAsync(pl->m.get(), 0, pl->m.bytes(), s));
            EVOC_CUDA(cudaMemsetAsync(pl->v.get(), 0, pl->v.bytes(), s));
            EVOC_CUDA(cudaEventRecord(e0, s));
            if (mode) {
              launch_all_epochs(pl, 0, ne, s);
            } else {
              EVOC_CUDA(cudaMemsetAsync(pl->work_ctr.get(), 0, pl->work_ctr.bytes(), s));
              for (int32_t t = 0; t < ne; ++t)
                launch_epoch(pl, t, (t & 1) ? pl->e1 : pl->e0, (t & 1) ? pl->e0 : pl->e1,
                             nullptr, s);
            }
            EVOC_CUDA(cudaEventRecord(e1, s));
            EVOC_CUDA(cudaEventSynchronize(e1));
            EVOC_CUDA(cudaEventElapsedTime(&el, e0, e1));
          }
          (mode ? all_ms : per_epoch_ms) = el;
        }
        check_status(pl->ctx, "autotune (all-epochs launch)");
        if (all_ms < per_epoch_ms) best.kv += N_SLOT_VARIANTS;
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      plan_configure(pl, best.kv, best.wpb, best.bps);
      best_ms = best.ms;
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tune[key] = best;
      if (const char* f = std::getenv("EVOC_TUNE_CACHE"))
        if (*f) {
          std::ofstream o(f, std::ios::app);
          o << key << " " << best.kv << " " << best.wpb << " " << best.bps << " " << best.ms
            << "\n";
        }
    }
  }
  if (config) {
    config[0] = pl->kvariant + (pl->all_epochs ? N_SLOT_VARIANTS : 0);
    config[1] = pl->lanes;
    config[2] = pl->blocks_per_sm;
  }
  if (ms_out) *ms_out = best_ms;
}

int64_t plan_n(const evoc_plan* p) { return p->n; }
int32_t plan_n_epochs(const evoc_plan* p) { return p->params.n_epochs; }
bool plan_has_edges(const evoc_plan* p) { return p->has_edges; }

namespace {
// Thread per row of a block-diagonal graph: every column must lie in the
// row's own problem.
__global__ void k_check_blocks(const int64_t* __restrict__ indptr,
                               const uint32_t* __restrict__ indices, int64_t n,
                               const uint32_t* __restrict__ prob_of_node,
                               const ProbInfo* __restrict__ prob, int32_t* __restrict__ status) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const ProbInfo pi = prob[prob_of_node[r]];
  for (int64_t p = indptr[r]; p < indptr[r + 1]; ++p) {
    const uint32_t c = indices[p];
    if (c < pi.node_base || c - pi.node_base >= pi.n) {
      atomicOr(status, (int32_t)ST_CROSS_BLOCK);
      return;
    }
  }
}
}  // namespace

evoc_plan* plan_create(evoc_ctx* ctx, const std::vector<ProblemDesc>& probs,
                       int32_t dim, const evoc_embed_params_t& params) {
  cudaStream_t s = ctx->stream;
  if (probs.empty()) throw Error(EVOC_ERR_INVALID_ARGUMENT, "no problems");
  if (dim < 1 || dim > 16)
    throw Error(EVOC_ERR_UNSUPPORTED, "dim must be in 1..16");
  if (params.n_epochs < 0)
    throw Error(EVOC_ERR_INVALID_ARGUMENT, "n_epochs must be >= 0");
  std::unique_ptr<evoc_plan> pl(new evoc_plan());
  pl->ctx = ctx;
  pl->dim = dim;
  pl->dimp = dim <= 4 ? 4 : (dim <= 8 ? 8 : 16);
  pl->params = params;
  pl->n_problems = (int32_t)probs.size();
  int64_t n = 0, nnz = 0;
  bool canonical = true;
  // blocks: every problem is a row range of one block-diagonal graph
  const bool blocks = probs.size() > 1 && probs[0].begin >= 0;
  for (auto& p : probs) {
    if (!p.graph || p.graph->ctx != ctx)
      throw Error(EVOC_ERR_INVALID_ARGUMENT, "graph belongs to another context");
    if (blocks) {
      if (p.graph != probs[0].graph || p.begin != n || p.count < 0)
        throw Error(EVOC_ERR_INVALID_ARGUMENT, "blocks must tile one graph in order");
      pl->node_base.push_back(n);
      pl->seeds.push_back(p.seed);
      n += p.count;
      continue;
    }
    pl->node_base.push_back(n);
    pl->seeds.push_back(p.seed);
    n += p.graph->n;
    nnz += p.graph->nnz;
    canonical = canonical && p.graph->canonical;
  }
  if (blocks) {
    if (n != probs[0].graph->n)
      throw Error(EVOC_ERR_INVALID_ARGUMENT, "block sizes do not add up to the graph's n");
    nnz = probs[0].graph->nnz;
    canonical = probs[0].graph->canonical;
  }
  if (n >= (int64_t)0xFFFFFFFFu)
    throw Error(EVOC_ERR_UNSUPPORTED, "more than 2^32-2 nodes in total");
  pl->n = n;

  // per-epoch constants (embedding.rs:141-160, :179)
  const int32_t ne = params.n_epochs;
  pl->one_m_b1 = 1.0f - params.beta1;
  pl->one_m_b2 = 1.0f - params.beta2;
  const float denom = (float)std::max(ne - 1, 1);
  const float ne_f = (float)ne;
  for (int32_t ep = 0; ep < ne; ++ep) {
    const float t = (float)(ep + 1);
    const float b1t = std::pow(params.beta1, t);
    const float b2t = std::pow(params.beta2, t);
    const float sqrt_b2 = std::sqrt(1.0f - b2t);
    const float ad_scale = sqrt_b2 / (1.0f - b1t);
    pl->epsc.push_back(sqrt_b2 * params.eps);
    const float lr = params.initial_alpha * (1.0f - (float)ep / ne_f);
    pl->lr_ad.push_back(lr * ad_scale);
    pl->gamma.push_back(0.5f + (float)ep / denom);
  }
  pl->stats.assign(ne, evoc_epoch_stats_t{0, 0, 0});
  if (n == 0) return pl.release();

  // concatenated graph (batched) or the single graph's buffers
  const int64_t* indptr;
  const uint32_t* indices;
  const float* weights;
  DevBuf<int64_t> cat_ptr;
  DevBuf<uint32_t> cat_idx;
  DevBuf<float> cat_w;
  if (probs.size() == 1) {
    indptr = probs[0].graph->indptr.get();
    indices = probs[0].graph->indices.get();
    weights = probs[0].graph->weights.get();
  } else if (blocks) {
    indptr = probs[0].graph->indptr.get();
    indices = probs[0].graph->indices.get();
    weights = probs[0].graph->weights.get();
    std::vector<uint32_t> pon_host(n);
    std::vector<ProbInfo> info;
    for (size_t q = 0; q < probs.size(); ++q) {
      info.push_back(ProbInfo{(uint32_t)probs[q].begin, (uint32_t)probs[q].count, probs[q].seed});
      for (int64_t i = 0; i < probs[q].count; ++i) pon_host[probs[q].begin + i] = (uint32_t)q;
    }
    pl->prob_of_node.alloc(n, s);
    pl->prob.alloc(info.size(), s);
    EVOC_CUDA(cudaMemcpyAsync(pl->prob_of_node.get(), pon_host.data(), n * sizeof(uint32_t),
                              cudaMemcpyHostToDevice, s));
    EVOC_CUDA(cudaMemcpyAsync(pl->prob.get(), info.data(), info.size() * sizeof(ProbInfo),
                              cudaMemcpyHostToDevice, s));
    if (nnz > 0) {  // every edge must stay inside its problem
      k_check_blocks<<<blocks_for(n), 256, 0, s>>>(indptr, indices, n, pl->prob_of_node.get(),
                                                   pl->prob.get(), ctx->status.get());
      EVOC_CHECK_LAUNCH();
    }
    check_status(ctx, "block-diagonal graph");  // synchronises: host vectors go out of scope
  } else {
    cat_ptr.alloc(n + 1, s);
    cat_idx.alloc(nnz, s);
    cat_w.alloc(nnz, s);
    std::vector<uint32_t> pon_host;
    std::vector<ProbInfo> info;
    int64_t eoff = 0;
    for (size_t q = 0; q < probs.size(); ++q) {
      const evoc_graph* g = probs[q].graph;
      const int64_t nb = pl->node_base[q];
      info.push_back(ProbInfo{(uint32_t)nb, (uint32_t)g->n, probs[q].seed});
      if (g->n == 0) continue;
      concat_graph(g, nb, eoff, cat_ptr.get(), cat_idx.get(), s);
      if (g->nnz)
        EVOC_CUDA(cudaMemcpyAsync(cat_w.get() + eoff, g->weights.get(),
                                  g->nnz * sizeof(float),
                                  cudaMemcpyDeviceToDevice, s));
      eoff += g->nnz;
    }
    EVOC_CUDA(cudaMemcpyAsync(cat_ptr.get() + n, &nnz, sizeof(int64_t),
                              cudaMemcpyHostToDevice, s));
    pon_host.resize(n);
    for (size_t q = 0; q < probs.size(); ++q)
      for (int64_t i = 0; i < probs[q].graph->n; ++i)
        pon_host[pl->node_base[q] + i] = (uint32_t)q;
    pl->prob_of_node.alloc(n, s);
    pl->prob.alloc(info.size(), s);
    EVOC_CUDA(cudaMemcpyAsync(pl->prob_of_node.get(), pon_host.data(),
                              n * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    EVOC_CUDA(cudaMemcpyAsync(pl->prob.get(), info.data(),
                              info.size() * sizeof(ProbInfo),
                              cudaMemcpyHostToDevice, s));
    EVOC_CUDA(cudaStreamSynchronize(s));  // host vectors go out of scope
    indptr = cat_ptr.get();
    indices = cat_idx.get();
    weights = cat_w.get();
  }
  const uint32_t* pon = pl->n_problems > 1 ? pl->prob_of_node.get() : nullptr;

  StageTrace trace(s);
  trace.mark("graph concat");
  // upper / lower counts and the edge list
  DevBuf<int32_t> ucnt(n, s), lcnt(n, s);
  k_row_counts<<<blocks_for(n * 32), 256, 0, s>>>(indptr, indices, n, ucnt.get(),
                                                  lcnt.get());
  EVOC_CHECK_LAUNCH();
  DevBuf<int64_t> uptr(n + 1, s);
  exclusive_scan_i32_to_i64(ucnt.get(), uptr.get(), n, s);
  int64_t U = 0;
  EVOC_CUDA(cudaMemcpyAsync(&U, uptr.get() + n, sizeof(int64_t),
                            cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaStreamSynchronize(s));
  pl->n_edges = U;
  pl->emb.alloc(2 * n * pl->dimp, s);
  pl->e0 = pl->emb.get();
  pl->e1 = pl->emb.get() + n * pl->dimp;
  if (U == 0) {  // embedding.rs:92-96
    pl->has_edges = false;
    return pl.release();
  }
  if (U >= (int64_t)0xFFFFFFFFu)
    throw Error(EVOC_ERR_UNSUPPORTED, "more than 2^32-2 edges");
  pl->has_edges = true;

  trace.mark("row counts + scan");
  DevBuf<float> e_w(U, s), e_ps(U, s);
  DevBuf<uint32_t> e_dst(U, s), e_src(U, s);
  DevBuf<int32_t> max_w(pl->n_problems, s);
  EVOC_CUDA(cudaMemsetAsync(max_w.get(), 0, pl->n_problems * sizeof(int32_t), s));
  if (!canonical) EVOC_CUDA(cudaMemsetAsync(lcnt.get(), 0, n * sizeof(int32_t), s));
  k_edge_fill<<<blocks_for(n * 32), 256, 0, s>>>(
      indptr, indices, weights, n, uptr.get(), pon, e_w.get(), e_dst.get(),
      e_src.get(), max_w.get(), canonical ? nullptr : lcnt.get());
  EVOC_CHECK_LAUNCH();
  k_edge_ps<<<blocks_for(U), 256, 0, s>>>(e_w.get(), e_src.get(), U, pon,
                                          max_w.get(), e_ps.get());
  EVOC_CHECK_LAUNCH();
  e_w.release();

  DevBuf<int64_t> lptr;
  DevBuf<uint2> lower;
  if (!canonical) {
    DevBuf<uint32_t> keys(U, s);
    lower.alloc(U, s);
    EVOC_CUDA(cudaMemcpyAsync(keys.get(), e_dst.get(), U * sizeof(uint32_t),
                              cudaMemcpyDeviceToDevice, s));
    fill_eidx_src(lower.get(), e_src.get(), U, s);
    radix_sort_pairs(keys.get(), lower.get(), U, bits_for((uint64_t)(n - 1)), s);
    lptr.alloc(n + 1, s);
    exclusive_scan_i32_to_i64(lcnt.get(), lptr.get(), n, s);
  }
  e_dst.release();
  e_src.release();

  trace.mark("edges + transpose");
  // incidence lists
  DevBuf<int32_t> deg(n, s);
  add_counts(ucnt.get(), lcnt.get(), deg.get(), n, s);
  pl->inc_ptr.alloc(n + 1, s);
  exclusive_scan_i32_to_i64(deg.get(), pl->inc_ptr.get(), n, s);
  deg.release();
  int64_t n_inc = 0;
  EVOC_CUDA(cudaMemcpyAsync(&n_inc, pl->inc_ptr.get() + n, sizeof(int64_t),
                            cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaStreamSynchronize(s));
  if (n_inc != 2 * U)
    throw Error(EVOC_ERR_INTERNAL, "incidence count mismatch (graph not symmetric?)");
  pl->n_inc = n_inc;
  DevBuf<int64_t> ebase(pl->n_problems, s);
  k_prob_ebase<<<blocks_for(pl->n_problems), 256, 0, s>>>(
      uptr.get(), pl->n_problems > 1 ? pl->prob.get() : nullptr,
      pl->n_problems, ebase.get());
  EVOC_CHECK_LAUNCH();
  pl->inc_other.alloc(n_inc, s);
  pl->eidx_base.alloc(n, s);
  DevBuf<float> inc_ps(n_inc, s);
  DevBuf<uint8_t> inc_up(n_inc, s);
  DevBuf<uint32_t> inc_eidx(n_inc, s);
  k_inc_fill<<<blocks_for(n * 32), 256, 0, s>>>(
      indptr, indices, weights, n, uptr.get(), lcnt.get(), lptr.get(),
      lower.get(), e_ps.get(), pl->inc_ptr.get(), pon, max_w.get(), ebase.get(),
      pl->inc_other.get(), inc_ps.get(), inc_up.get(), pl->eidx_base.get(),
      inc_eidx.get());
  EVOC_CHECK_LAUNCH();
  lower.release();
  lptr.release();

  trace.mark("incidence lists");
  // schedule: per-epoch gradient slots (fast path) or bit planes (fallback)
  const float neg_factor = 1.5f / params.negative_sample_rate;  // embedding.rs:116
  pl->W = (n_inc + 31) / 32;
  if (ne > 0 && !build_slots(pl.get(), inc_ps.get(), inc_up.get(), inc_eidx.get(),
                               e_ps.get(), U, neg_factor)) {
    DevBuf<unsigned long long> mx(1, s), st(2 * ne, s);
    EVOC_CUDA(cudaMemsetAsync(mx.get(), 0, sizeof(unsigned long long), s));
    EVOC_CUDA(cudaMemsetAsync(st.get(), 0, st.bytes(), s));
    const bool want_stats = ne <= 4096;
    const size_t smem = want_stats ? 2 * ne * sizeof(unsigned long long) : 0;
    if (smem > 48 * 1024)
      EVOC_CUDA(cudaFuncSetAttribute((const void*)k_schedule_scan,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
    k_schedule_scan<<<blocks_for(n_inc), 256, smem, s>>>(
        inc_ps.get(), inc_up.get(), n_inc, ne, neg_factor, mx.get(),
        want_stats ? st.get() : nullptr, want_stats ? st.get() + ne : nullptr);
    EVOC_CHECK_LAUNCH();
    unsigned long long maxneg = 0;
    std::vector<unsigned long long> sth(2 * ne);
    EVOC_CUDA(cudaMemcpyAsync(&maxneg, mx.get(), sizeof(maxneg),
                              cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaMemcpyAsync(sth.data(), st.get(), 2 * ne * sizeof(unsigned long long),
                              cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaStreamSynchronize(s));
    if (maxneg > (unsigned long long)NEG_LIMIT)
      throw Error(EVOC_ERR_UNSUPPORTED,
                  "more than 2^20 negative samples per edge and epoch "
                  "(negative_sample_rate too large)");
    pl->max_neg = maxneg;
    pl->P = bits_for(maxneg);
    for (int32_t t = 0; t < ne; ++t) {
      pl->stats[t].fired_edges = (int64_t)sth[t];
      pl->stats[t].negatives = (int64_t)sth[ne + t];
    }
    pl->planes.alloc((size_t)ne * (1 + pl->P) * pl->W, s);
    k_schedule_write<<<blocks_for(pl->W * 32), 256, 0, s>>>(
        inc_ps.get(), inc_up.get(), n_inc, ne, neg_factor, pl->P, pl->W,
        pl->planes.get());
    EVOC_CHECK_LAUNCH();
  }

  trace.mark("schedule");
  pl->m.alloc(n * pl->dimp, s);
  pl->v.alloc(n * pl->dimp, s);
  pl->lanes = default_wpb();
  if (pl->use_slots) {
    pl->work_ctr.alloc(std::max<int32_t>(ne, 1), s);
    std::vector<float4> ep(std::max<int32_t>(ne, 1), make_float4(0.f, 0.f, 0.f, 0.f));
    for (int32_t t = 0; t < ne; ++t) ep[t] = make_float4(pl->gamma[t], pl->lr_ad[t], pl->epsc[t], 0.f);
    pl->ep_params.alloc(ep.size(), s);
    EVOC_CUDA(cudaMemcpyAsync(pl->ep_params.get(), ep.data(), ep.size() * sizeof(float4),
                              cudaMemcpyHostToDevice, s));
    pl->grid_bar.alloc(4, s);
    EVOC_CUDA(cudaStreamSynchronize(s));  // ep goes out of scope
    plan_configure(pl.get(), 0, pl->lanes, 0);
    plan_apply_tuned(pl.get());  // a configuration tuned for this shape, if any
  }
  trace.mark("moments");
  EVOC_CUDA(cudaStreamSynchronize(s));
  return pl.release();
}

void plan_stats(const evoc_plan* cpl, evoc_epoch_stats_t* out) {
  evoc_plan* pl = const_cast<evoc_plan*>(cpl);
  const int32_t ne = pl->params.n_epochs;
  if (pl->has_edges && !pl->stats_done && ne > 0) {  // active nodes, on request
    cudaStream_t s = pl->ctx->stream;
    DevBuf<unsigned long long> act(ne, s);
    EVOC_CUDA(cudaMemsetAsync(act.get(), 0, act.bytes(), s));
    if (pl->use_slots) {
      k_slot_stats<<<blocks_for(pl->ntiles * 32), 256, 0, s>>>(
          pl->tile_off.get(), pl->slots.get(), pl->ntiles, ne, act.get());
    } else {
      k_active_count<<<blocks_for(pl->n * 32), 256, 0, s>>>(
          pl->inc_ptr.get(), pl->n, pl->planes.get(), ne, pl->P, pl->W, act.get());
    }
    EVOC_CHECK_LAUNCH();
    std::vector<unsigned long long> ha(ne);
    EVOC_CUDA(cudaMemcpyAsync(ha.data(), act.get(), ne * sizeof(unsigned long long),
                              cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaStreamSynchronize(s));
    for (int32_t t = 0; t < ne; ++t) pl->stats[t].active_nodes = (int64_t)ha[t];
    pl->stats_done = true;
  }
  for (int32_t t = 0; t < ne; ++t) out[t] = pl->stats[t];
}

// Initial embedding into e0 (padded): from d_init (n*dim) or random.
static void load_init(evoc_plan* pl, const float* d_init, cudaStream_t s) {
  const int64_t tot = pl->n * pl->dimp;
  if (d_init) {
    k_pad<<<blocks_for(tot), 256, 0, s>>>(d_init, pl->e0, pl->n, pl->dim,
                                          pl->dimp);
  } else {
    k_init_random<<<blocks_for(tot), 256, 0, s>>>(
        pl->e0, pl->n, pl->dim, pl->dimp,
        pl->n_problems > 1 ? pl->prob_of_node.get() : nullptr,
        pl->n_problems > 1 ? pl->prob.get() : nullptr,
        pl->seeds.empty() ? 0 : pl->seeds[0]);
  }
  EVOC_CHECK_LAUNCH();
}

void plan_run_device(evoc_plan* pl, const float* d_init, float* d_out) {
  cudaStream_t s = pl->ctx->stream;
  const int64_t n = pl->n;
  if (n == 0) return;
  const int32_t ne = pl->params.n_epochs;
  load_init(pl, d_init, s);
  if (pl->has_edges && ne > 0) {
    EVOC_CUDA(cudaMemsetAsync(pl->m.get(), 0, pl->m.bytes(), s));
    EVOC_CUDA(cudaMemsetAsync(pl->v.get(), 0, pl->v.bytes(), s));
    if (pl->all_epochs) {  // one cooperative launch for all epochs
      launch_all_epochs(pl, 0, ne, s);
      EVOC_CHECK_LAUNCH();
    } else {
    if (pl->use_slots)  // tile counters of the slots kernel, one per epoch
      EVOC_CUDA(cudaMemsetAsync(pl->work_ctr.get(), 0, pl->work_ctr.bytes(), s));
    if (!pl->graph_exec) {
      EVOC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      try {
        for (int32_t t = 0; t < ne; ++t) {
          const float* cur = (t & 1) ? pl->e1 : pl->e0;
          float* nxt = (t & 1) ? pl->e0 : pl->e1;
          launch_epoch(pl, t, cur, nxt, nullptr, s);
        }
      } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(s, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      EVOC_CUDA(cudaStreamEndCapture(s, &pl->graph));
      EVOC_CUDA(cudaGraphInstantiate(&pl->graph_exec, pl->graph, 0));
    }
    EVOC_CUDA(cudaGraphLaunch(pl->graph_exec, s));
    }
  }
  const float* fin = (pl->has_edges && (ne & 1)) ? pl->e1 : pl->e0;
  k_unpad<<<blocks_for(n * pl->dim), 256, 0, s>>>(fin, d_out, n, pl->dim, pl->dimp);
  EVOC_CHECK_LAUNCH();
}

void plan_profile_epochs(evoc_plan* pl, const float* d_init, float* d_out,
                         float* epoch_ms) {
  cudaStream_t s = pl->ctx->stream;
  const int64_t n = pl->n;
  const int32_t ne = pl->params.n_epochs;
  for (int32_t t = 0; t < ne; ++t) epoch_ms[t] = 0.0f;
  if (n == 0) return;
  load_init(pl, d_init, s);
  const float* fin = pl->e0;
  if (pl->has_edges && ne > 0) {
    EVOC_CUDA(cudaMemsetAsync(pl->m.get(), 0, pl->m.bytes(), s));
    EVOC_CUDA(cudaMemsetAsync(pl->v.get(), 0, pl->v.bytes(), s));
    if (pl->use_slots)  // tile counters of the slots kernel, one per epoch
      EVOC_CUDA(cudaMemsetAsync(pl->work_ctr.get(), 0, pl->work_ctr.bytes(), s));
    std::vector<cudaEvent_t> ev(ne + 1, nullptr);
    try {
      for (auto& e : ev) EVOC_CUDA(cudaEventCreate(&e));
      EVOC_CUDA(cudaEventRecord(ev[0], s));
      for (int32_t t = 0; t < ne; ++t) {
        const float* cur = (t & 1) ? pl->e1 : pl->e0;
        float* nxt = (t & 1) ? pl->e0 : pl->e1;
        launch_epoch(pl, t, cur, nxt, nullptr, s);
        EVOC_CUDA(cudaEventRecord(ev[t + 1], s));
        fin = nxt;
      }
      EVOC_CUDA(cudaEventSynchronize(ev[ne]));
      for (int32_t t = 0; t < ne; ++t)
        EVOC_CUDA(cudaEventElapsedTime(&epoch_ms[t], ev[t], ev[t + 1]));
    } catch (...) {
      for (auto& e : ev)
        if (e) cudaEventDestroy(e);
      throw;
    }
    for (auto& e : ev) cudaEventDestroy(e);
  }
  k_unpad<<<blocks_for(n * pl->dim), 256, 0, s>>>(fin, d_out, n, pl->dim, pl->dimp);
  EVOC_CHECK_LAUNCH();
  EVOC_CUDA(cudaStreamSynchronize(s));
}

void plan_debug_run(evoc_plan* pl, const float* h_init, int32_t start_epoch,
                    int32_t end_epoch, float* h_out, float* h_grad) {
  cudaStream_t s = pl->ctx->stream;
  const int64_t n = pl->n;
  if (n == 0) return;
  const int32_t ne = pl->params.n_epochs;
  const int64_t nd = n * pl->dim;
  DevBuf<float> io(nd, s);
  if (h_init) {
    EVOC_CUDA(cudaMemcpyAsync(io.get(), h_init, nd * sizeof(float),
                              cudaMemcpyHostToDevice, s));
    load_init(pl, io.get(), s);
  } else {
    load_init(pl, nullptr, s);
  }
  const int32_t e0 = std::max(0, std::min(start_epoch, ne));
  const int32_t e1 = std::max(e0, std::min(end_epoch, ne));
  DevBuf<float> grad;
  if (h_grad) {
    grad.alloc(n * pl->dimp, s);
    EVOC_CUDA(cudaMemsetAsync(grad.get(), 0, grad.bytes(), s));
  }
  const float* fin = pl->e0;
  if (pl->has_edges && e1 > e0) {
    EVOC_CUDA(cudaMemsetAsync(pl->m.get(), 0, pl->m.bytes(), s));
    EVOC_CUDA(cudaMemsetAsync(pl->v.get(), 0, pl->v.bytes(), s));
    if (pl->use_slots)  // tile counters of the slots kernel, one per epoch
      EVOC_CUDA(cudaMemsetAsync(pl->work_ctr.get(), 0, pl->work_ctr.bytes(), s));
    for (int32_t t = e0; t < e1; ++t) {
      const int k = t - e0;
      const float* cur = (k & 1) ? pl->e1 : pl->e0;
      float* nxt = (k & 1) ? pl->e0 : pl->e1;
      launch_epoch(pl, t, cur, nxt, (t == e1 - 1) ? grad.get() : nullptr, s);
      fin = nxt;
    }
  }
  k_unpad<<<blocks_for(nd), 256, 0, s>>>(fin, io.get(), n, pl->dim, pl->dimp);
  EVOC_CHECK_LAUNCH();
  EVOC_CUDA(cudaMemcpyAsync(h_out, io.get(), nd * sizeof(float),
                            cudaMemcpyDeviceToHost, s));
  if (h_grad) {
    k_unpad<<<blocks_for(nd), 256, 0, s>>>(grad.get(), io.get(), n, pl->dim,
                                           pl->dimp);
    EVOC_CHECK_LAUNCH();
    EVOC_CUDA(cudaMemcpyAsync(h_grad, io.get(), nd * sizeof(float),
                              cudaMemcpyDeviceToHost, s));
  }
  EVOC_CUDA(cudaStreamSynchronize(s));
}

void plan_upload_init_and_run(evoc_plan* pl, const float* const* h_inits,
                              float* const* h_outs, int verbose) {
  cudaStream_t s = pl->ctx->stream;
  const int64_t n = pl->n;
  if (n == 0) return;
  const int64_t nd = n * pl->dim;
  DevBuf<float> io(nd, s);
  bool all_init = true, any_init = false;
  for (int32_t q = 0; q < pl->n_problems; ++q) {
    all_init = all_init && h_inits && h_inits[q];
    any_init = any_init || (h_inits && h_inits[q]);
  }
  if (any_init && !all_init)
    throw Error(EVOC_ERR_INVALID_ARGUMENT,
                "either every problem or none must have an initial embedding");
  if (all_init) {
    for (int32_t q = 0; q < pl->n_problems; ++q) {
      const int64_t nq = (q + 1 < pl->n_problems ? pl->node_base[q + 1] : n) -
                         pl->node_base[q];
      if (nq)
        EVOC_CUDA(cudaMemcpyAsync(io.get() + pl->node_base[q] * pl->dim,
                                  h_inits[q], nq * pl->dim * sizeof(float),
                                  cudaMemcpyHostToDevice, s));
    }
  }
  plan_run_device(pl, all_init ? io.get() : nullptr, io.get());
  for (int32_t q = 0; q < pl->n_problems; ++q) {
    const int64_t nq = (q + 1 < pl->n_problems ? pl->node_base[q + 1] : n) -
                       pl->node_base[q];
    if (nq)
      EVOC_CUDA(cudaMemcpyAsync(h_outs[q], io.get() + pl->node_base[q] * pl->dim,
                                nq * pl->dim * sizeof(float),
                                cudaMemcpyDeviceToHost, s));
  }
  EVOC_CUDA(cudaStreamSynchronize(s));
  if (verbose == 2) {  // embedding.rs:288-291
    const int32_t ne = pl->params.n_epochs;
    for (int32_t e = 0; e < ne; ++e)
      if ((e + 1) % 10 == 0 || e + 1 == ne)
        std::printf("   Embedding epoch %d/%d\n", e + 1, ne);
    std::fflush(stdout);
  }
}

void plan_free(evoc_plan* pl) {
  if (!pl) return;
  if (pl->ctx && pl->slots.count > pl->ctx->slot_cache.count)
    pl->ctx->slot_cache = std::move(pl->slots);
  if (pl->graph_exec) cudaGraphExecDestroy(pl->graph_exec);
  if (pl->graph) cudaGraphDestroy(pl->graph);
  delete pl;
}

// ---- small helpers used by plan_create --------------------------------------
namespace {
__global__ void k_concat(const int64_t* __restrict__ src_ptr,
                         const uint32_t* __restrict__ src_idx, int64_t n,
                         int64_t nnz, int64_t node_off, int64_t entry_off,
                         int64_t* __restrict__ dptr, uint32_t* __restrict__ didx) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) dptr[node_off + q] = entry_off + src_ptr[q];
  if (q < nnz) didx[entry_off + q] = (uint32_t)(src_idx[q] + node_off);
}
__global__ void k_fill_eidx_src(uint2* __restrict__ out,
                                const uint32_t* __restrict__ e_src, int64_t U) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < U) out[e] = make_uint2((uint32_t)e, e_src[e]);
}
__global__ void k_add_counts(const int32_t* __restrict__ a,
                             const int32_t* __restrict__ b,
                             int32_t* __restrict__ out, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] + b[i];
}
}  // namespace

void concat_graph(const evoc_graph* g, int64_t node_off, int64_t entry_off,
                  int64_t* dptr, uint32_t* didx, cudaStream_t s) {
  const int64_t m = std::max(g->n, g->nnz);
  k_concat<<<blocks_for(m), 256, 0, s>>>(g->indptr.get(), g->indices.get(),
                                         g->n, g->nnz, node_off, entry_off,
                                         dptr, didx);
  EVOC_CHECK_LAUNCH();
}

void fill_eidx_src(uint2* out, const uint32_t* e_src, int64_t U,
                   cudaStream_t s) {
  k_fill_eidx_src<<<blocks_for(U), 256, 0, s>>>(out, e_src, U);
  EVOC_CHECK_LAUNCH();
}

void add_counts(const int32_t* a, const int32_t* b, int32_t* out, int64_t n,
                cudaStream_t s) {
  k_add_counts<<<blocks_for(n), 256, 0, s>>>(a, b, out, n);
  EVOC_CHECK_LAUNCH();
}

}  // namespace evoc
