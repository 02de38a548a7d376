// mst.cu — build_mst (src/clustering/mst.rs:82-166, evoc-rs 0.2.7) on the
// GPU: Boruvka's minimum spanning tree over mutual reachability distance, the
// first step of the clustering stage that turns the embedding into labels.
//
// Spatial index. Points are sorted by a 64-bit Morton code of their
// coordinates (quantised on the bounding box); an implicit complete binary
// tree over leaves of 32 consecutive sorted points holds the bounding box of
// each node (heap order: node v has children 2v and 2v + 1, leaves are P..2P-1).
// It plays the part of the reference's KD-tree (kd_tree.rs:93-236): only
// pruning bounds come from it, never a result.
//
// Core distances (mst.rs:101-113): per point, the k-th smallest squared
// distance to another point, k = min(min_samples, n - 1); a warp walks the
// tree for 32 consecutive points at once (see the traversal kernels), nearer
// child first, and skips a node whose box lower bound exceeds every lane's
// current k-th distance (knn_recurse, kd_tree.rs:489-535).
//
// Boruvka rounds (mst.rs:115-160):
//   1. node components, bottom-up (update_node_components, kd_tree.rs:387-419);
//   2. per point, the nearest point of another component under squared mutual
//      reachability max(d^2, core_i, core_j) (nearest_other_component,
//      kd_tree.rs:275-378), with the same three pruning rules; among equal
//      values the smallest point index. A per-component bound starts each
//      query just above it and is lowered while the round runs: first the
//      smallest value over the component's leaving kNN edges (kept from the
//      core-distance pass), then the best value found so far by its points.
//      Each is the value of a real edge leaving the component, so no
//      component's pick changes;
//   3. per component (its id is its smallest point index), the pick with the
//      smallest value, then the smallest point index: one 64-bit atomicMin of
//      (value bits, point index);
//   4. merge. The reference adds the picks one at a time through a disjoint
//      set and skips those that would close a cycle. Taken in ascending
//      component id, the skipped picks are exactly, on each cycle of the pick
//      graph (component -> component of its pick's other end), the pick of the
//      largest component id: the rest of a functional graph's weak component
//      hangs off its cycle in trees. Pointer doubling (2^K >= m steps) lands
//      every component on its cycle and gathers the cycle's maximum; pointer
//      jumping to the skipped component gives the merged components; kept
//      edges are appended in ascending component id.
// Squared distances are serial left folds over the dimensions with IEEE
// round-to-nearest operations and weights are square roots of them, so the
// edge list equals the oracle's edge for edge, weights bit for bit.
#include "evoc_device.cuh"
#include "evoc_internal.h"

#include <cfloat>
#include <cstring>

namespace evoc {
namespace {

constexpr int MST_LEAF = 32;     // points per leaf
constexpr uint32_t NC_MIXED = 0xffffffffu;  // node holds points of several components
constexpr uint32_t NC_EMPTY = 0xfffffffeu;  // node holds no point
constexpr uint32_t NO_POINT = 0xffffffffu;
constexpr uint32_t FMAX_BITS = 0x7f7fffffu;  // FLT_MAX

inline unsigned grid_of(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// Order-preserving integer image of a float (for min / max atomics).
__device__ __forceinline__ uint32_t ord_of(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float of_ord(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Bounding box of dimension blockIdx.y; every coordinate must be finite.
__global__ void k_mst_bbox(const float* __restrict__ x, int64_t n, int dim,
                           uint32_t* __restrict__ omin, uint32_t* __restrict__ omax,
                           int32_t* __restrict__ status) {
  const int d = blockIdx.y;
  float lo = FLT_MAX, hi = -FLT_MAX;
  bool bad = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float v = x[i * dim + d];
    bad |= !isfinite(v);
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
  if (bad) set_status(status, ST_BAD_VALUE);
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&omin[d], ord_of(lo));
    atomicMax(&omax[d], ord_of(hi));
  }
}

// Morton code: each coordinate quantised to `bits` bits on the box, bits
// interleaved from the top (dimension 0 first). Low 32 bits as the sort key,
// (point, high 32 bits) as the value.
__global__ void k_mst_morton(const float* __restrict__ x, int64_t n, int dim, int bits,
                             const uint32_t* __restrict__ omin, const uint32_t* __restrict__ omax,
                             uint32_t* __restrict__ key, uint2* __restrict__ val) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t q[16];
  const float maxq = (float)((1u << bits) - 1u);
  for (int d = 0; d < dim; ++d) {
    const float lo = of_ord(omin[d]), hi = of_ord(omax[d]);
    const float span = hi - lo;
    const float t = span > 0.0f ? (x[i * dim + d] - lo) / span * maxq : 0.0f;
    q[d] = (uint32_t)fminf(fmaxf(t, 0.0f), maxq);
  }
  uint64_t code = 0;
  for (int b = bits - 1; b >= 0; --b)
    for (int d = 0; d < dim; ++d) code = (code << 1) | ((q[d] >> b) & 1u);
  key[i] = (uint32_t)code;
  val[i] = make_uint2((uint32_t)i, (uint32_t)(code >> 32));
}

__global__ void k_mst_hi_keys(const uint2* __restrict__ val, int64_t n, uint32_t* __restrict__ key) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) key[i] = val[i].y;
}

// Sorted copy of the points, padded with zeros to DIMP (a zero pad adds +0 to
// a squared distance, which leaves it unchanged).
template <int DIMP>
__global__ void k_mst_gather(const float* __restrict__ x, int64_t n, int dim,
                             const uint2* __restrict__ val, float* __restrict__ xs,
                             uint32_t* __restrict__ orig, uint32_t* __restrict__ pos_of) {
  const int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= n) return;
  const uint32_t p = val[pos].x;
  orig[pos] = p;
  pos_of[p] = (uint32_t)pos;
#pragma unroll
  for (int d = 0; d < DIMP; ++d) xs[pos * DIMP + d] = d < dim ? x[(int64_t)p * dim + d] : 0.0f;
}

template <int DIMP>
__device__ __forceinline__ void mst_load(const float* __restrict__ xs, int64_t pos,
                                         float (&p)[DIMP]) {
  const float4* s = reinterpret_cast<const float4*>(xs + pos * DIMP);
#pragma unroll
  for (int q = 0; q < DIMP / 4; ++q) {
    const float4 v = __ldg(s + q);
    p[4 * q] = v.x;
    p[4 * q + 1] = v.y;
    p[4 * q + 2] = v.z;
    p[4 * q + 3] = v.w;
  }
}

// sum_d (a_d - b_d)^2, serial over the dimensions (mst.rs's squared metric).
template <int DIMP>
__device__ __forceinline__ float mst_sqd(const float (&a)[DIMP], const float (&b)[DIMP]) {
  float s = 0.0f;
#pragma unroll
  for (int d = 0; d < DIMP; ++d) {
    const float t = fsub(a[d], b[d]);
    s = fadd(s, fmul(t, t));
  }
  return s;
}

// Squared distance from p to node v's box (aabb_sq, kd_tree.rs:247-265). It
// never exceeds the squared distance to a point inside the box: every step is
// a monotone rounded operation on a smaller operand.
template <int DIMP>
__device__ __forceinline__ float mst_box_lb(const float* __restrict__ lo,
                                            const float* __restrict__ hi, int64_t v,
                                            const float (&p)[DIMP]) {
  const float4* l4 = reinterpret_cast<const float4*>(lo + v * DIMP);
  const float4* h4 = reinterpret_cast<const float4*>(hi + v * DIMP);
  float r = 0.0f;
#pragma unroll
  for (int q = 0; q < DIMP / 4; ++q) {
    const float4 a = __ldg(l4 + q), b = __ldg(h4 + q);
    const float la[4] = {a.x, a.y, a.z, a.w}, hb[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float x = p[4 * q + e];
      const float diff = x < la[e] ? fsub(la[e], x) : (x > hb[e] ? fsub(x, hb[e]) : 0.0f);
      r = fadd(r, fmul(diff, diff));
    }
  }
  return r;
}

// Leaf boxes (empty leaves: +inf / -inf, so every bound to them is +inf).
template <int DIMP>
__global__ void k_mst_leaf_boxes(const float* __restrict__ xs, int64_t n, int64_t P, int64_t L,
                                 float* __restrict__ lo, float* __restrict__ hi) {
  const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= P) return;
  float a[DIMP], b[DIMP];
#pragma unroll
  for (int d = 0; d < DIMP; ++d) {
    a[d] = __int_as_float(0x7f800000);
    b[d] = -__int_as_float(0x7f800000);
  }
  if (l < L) {
    const int64_t e = min(n, (l + 1) * MST_LEAF);
    for (int64_t j = l * MST_LEAF; j < e; ++j) {
      float y[DIMP];
      mst_load<DIMP>(xs, j, y);
#pragma unroll
      for (int d = 0; d < DIMP; ++d) {
        a[d] = fminf(a[d], y[d]);
        b[d] = fmaxf(b[d], y[d]);
      }
    }
  }
  float4* lo4 = reinterpret_cast<float4*>(lo + (P + l) * DIMP);
  float4* hi4 = reinterpret_cast<float4*>(hi + (P + l) * DIMP);
#pragma unroll
  for (int q = 0; q < DIMP / 4; ++q) {
    lo4[q] = make_float4(a[4 * q], a[4 * q + 1], a[4 * q + 2], a[4 * q + 3]);
    hi4[q] = make_float4(b[4 * q], b[4 * q + 1], b[4 * q + 2], b[4 * q + 3]);
  }
}

// Internal boxes of one level: nodes [first, first + count).
template <int DIMP>
__global__ void k_mst_level_boxes(float* __restrict__ lo, float* __restrict__ hi, int64_t first,
                                  int64_t count) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const int64_t v = first + k;
  const float4* l4 = reinterpret_cast<const float4*>(lo);
  const float4* h4 = reinterpret_cast<const float4*>(hi);
  float4* lo4 = reinterpret_cast<float4*>(lo);
  float4* hi4 = reinterpret_cast<float4*>(hi);
  constexpr int Q = DIMP / 4;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const float4 a = l4[2 * v * Q + q], b = l4[(2 * v + 1) * Q + q];
    const float4 c = h4[2 * v * Q + q], e = h4[(2 * v + 1) * Q + q];
    lo4[v * Q + q] = make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), fminf(a.w, b.w));
    hi4[v * Q + q] = make_float4(fmaxf(c.x, e.x), fmaxf(c.y, e.y), fmaxf(c.z, e.z), fmaxf(c.w, e.w));
  }
}

// Warp-cooperative traversal. A warp serves 32 consecutive sorted points
// (spatially close in Morton order) and walks the union of their searches in
// lockstep: it enters a node when any lane's own pruning rule keeps it,
// descends first into the child most lanes find nearer and pushes the other
// (re-tested when popped); the stack is warp-uniform, entry i held by lane i
// (the tree is at most 28 levels deep). A leaf's points are staged once in
// shared memory and every lane that needs the leaf scans them.
constexpr int MST_WARPS = 4;  // warps per block

template <int DIMP>
struct MstLeafStage {
  float4 pt[MST_LEAF][DIMP / 4];
  uint32_t comp[MST_LEAF];
  float core[MST_LEAF];
  uint32_t orig[MST_LEAF];
};

template <int DIMP>
__device__ __forceinline__ void mst_stage_leaf(MstLeafStage<DIMP>& st,
                                               const float* __restrict__ xs, int64_t b0, int cnt,
                                               int lane) {
  if (lane < cnt) {
    const float4* src = reinterpret_cast<const float4*>(xs + (b0 + lane) * DIMP);
#pragma unroll
    for (int q = 0; q < DIMP / 4; ++q) st.pt[lane][q] = __ldg(src + q);
  }
}

template <int DIMP>
__device__ __forceinline__ void mst_staged(const MstLeafStage<DIMP>& st, int s2,
                                           float (&y)[DIMP]) {
#pragma unroll
  for (int q = 0; q < DIMP / 4; ++q) {
    const float4 t = st.pt[s2][q];
    y[4 * q] = t.x;
    y[4 * q + 1] = t.y;
    y[4 * q + 2] = t.z;
    y[4 * q + 3] = t.w;
  }
}

// Core distances: per sorted point, the k-th smallest squared distance to
// another point (the k smallest kept sorted in registers); a node is skipped
// when its box bound exceeds the current k-th distance (kd_tree.rs:499).
template <int DIMP, int KMAX>
__global__ void __launch_bounds__(32 * MST_WARPS) k_mst_core(
    const float* __restrict__ xs, int64_t n, int64_t P, int64_t L, const float* __restrict__ lo,
    const float* __restrict__ hi, int k, float* __restrict__ core, uint32_t* __restrict__ knn_j,
    float* __restrict__ knn_d, int32_t* __restrict__ status) {
  __shared__ MstLeafStage<DIMP> stage_s[MST_WARPS];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t q0 = ((int64_t)blockIdx.x * MST_WARPS + wid) * 32;
  if (q0 >= n) return;
  MstLeafStage<DIMP>& st = stage_s[wid];
  const int64_t pos = q0 + lane;
  const bool act = pos < n;
  float q[DIMP];
  mst_load<DIMP>(xs, act ? pos : q0, q);
  const float INF = __int_as_float(0x7f800000);
  float kd[KMAX];
  uint32_t kj[KMAX];
#pragma unroll
  for (int t = 0; t < KMAX; ++t) {
    kd[t] = INF;
    kj[t] = NO_POINT;
  }
  float kth = act ? INF : -1.0f;  // an idle lane needs no node
  const unsigned actm = __ballot_sync(FULL, act);
  uint32_t stk = 0;
  int sp = 0;
  int64_t v = 1;
  float lbv = 0.0f;
  for (;;) {
    if (__any_sync(FULL, lbv <= kth)) {
      if (v >= P) {
        const int64_t l = v - P;
        if (l < L) {
          const int64_t b0 = l * MST_LEAF;
          const int cnt = (int)min((int64_t)MST_LEAF, n - b0);
          __syncwarp();
          mst_stage_leaf<DIMP>(st, xs, b0, cnt, lane);
          __syncwarp();
          if (lbv <= kth) {
            for (int s2 = 0; s2 < cnt; ++s2) {
              if (b0 + s2 == pos) continue;
              float y[DIMP];
              mst_staged<DIMP>(st, s2, y);
              const float d = mst_sqd<DIMP>(q, y);
              if (d < kth) {
                const uint32_t j = (uint32_t)(b0 + s2);
#pragma unroll
                for (int t = KMAX - 1; t > 0; --t) {
                  if (kd[t - 1] > d) {
                    kd[t] = kd[t - 1];
                    kj[t] = kj[t - 1];
                  } else if (kd[t] > d) {
                    kd[t] = d;
                    kj[t] = j;
                  }
                }
                if (kd[0] > d) {
                  kd[0] = d;
                  kj[0] = j;
                }
                float kt = kd[0];
#pragma unroll
                for (int t = 1; t < KMAX; ++t)
                  if (t == k - 1) kt = kd[t];
                kth = kt;
              }
            }
          }
        }
      } else {
        const float l0 = mst_box_lb<DIMP>(lo, hi, 2 * v, q);
        const float l1 = mst_box_lb<DIMP>(lo, hi, 2 * v + 1, q);
        const bool n0 = __any_sync(FULL, l0 <= kth), n1 = __any_sync(FULL, l1 <= kth);
        if (n0 || n1) {
          const bool left = 2 * __popc(__ballot_sync(FULL, l0 <= l1) & actm) >= __popc(actm);
          const bool na = left ? n0 : n1, nb = left ? n1 : n0;
          const int64_t a = left ? 2 * v : 2 * v + 1;
          if (na && nb) {
            if (sp >= 32) {
              if (lane == 0) set_status(status, ST_INTERNAL);
              return;
            }
            if (lane == sp) stk = (uint32_t)(a ^ 1);
            ++sp;
          }
          const int64_t c = na ? a : (a ^ 1);
          lbv = (c == 2 * v) ? l0 : l1;
          v = c;
          continue;
        }
      }
    }
    if (sp == 0) break;
    --sp;
    v = __shfl_sync(FULL, stk, sp);
    lbv = mst_box_lb<DIMP>(lo, hi, v, q);
  }
  if (act) {
    core[pos] = kth;
#pragma unroll
    for (int t = 0; t < KMAX; ++t)
      if (t < k) {
        knn_j[pos * k + t] = kj[t];
        knn_d[pos * k + t] = kd[t];
      }
  }
}

// Upper bounds before a round's queries: per component, the smallest mutual
// reachability value over the kNN edges (from the core-distance pass) that
// leave it. Each is the value of a real edge leaving the component, so it is
// never below the component's pick and starting the queries just above it
// changes no pick.
__global__ void k_mst_knn_bound(int64_t n, int k, const uint32_t* __restrict__ knn_j,
                                const float* __restrict__ knn_d,
                                const uint32_t* __restrict__ comp, const float* __restrict__ core,
                                uint32_t* __restrict__ cbest) {
  const int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= n) return;
  const uint32_t qc = comp[pos];
  const float cq = core[pos];
  float best = __uint_as_float(FMAX_BITS);
  bool any = false;
  for (int t = 0; t < k; ++t) {
    const uint32_t j = knn_j[pos * k + t];
    if (j >= n || comp[j] == qc) continue;  // an unfilled entry (no finite distance)
    const float mr = fmaxf(fmaxf(knn_d[pos * k + t], cq), core[j]);
    if (mr < best) {
      best = mr;
      any = true;
    }
  }
  if (any) atomicMin(cbest + qc, __float_as_uint(best));
}

// Node components: a leaf's common component, NC_MIXED or NC_EMPTY.
__global__ void k_mst_leaf_comp(const uint32_t* __restrict__ comp, int64_t n, int64_t P, int64_t L,
                                uint32_t* __restrict__ nd) {
  const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= P) return;
  if (l >= L) {
    nd[P + l] = NC_EMPTY;
    return;
  }
  const int64_t b = l * MST_LEAF, e = min(n, b + MST_LEAF);
  const uint32_t c = comp[b];
  bool same = true;
  for (int64_t j = b + 1; j < e; ++j) same &= comp[j] == c;
  nd[P + l] = same ? c : NC_MIXED;
}

__global__ void k_mst_level_comp(uint32_t* __restrict__ nd, int64_t first, int64_t count) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const int64_t v = first + k;
  const uint32_t a = nd[2 * v], b = nd[2 * v + 1];
  nd[v] = a == NC_EMPTY ? b : (b == NC_EMPTY ? a : (a == b ? a : NC_MIXED));
}

__global__ void k_mst_round_reset(const uint32_t* __restrict__ A, int64_t m,
                                  uint32_t* __restrict__ cbest,
                                  unsigned long long* __restrict__ ckey) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const uint32_t c = A[k];
  cbest[c] = FMAX_BITS;
  ckey[c] = ~0ull;
}

// Nearest point of another component under squared mutual reachability
// (kd_tree.rs:318-378): a lane keeps a node when its box bound and its own
// core distance do not exceed the lane's best value and the node is not
// wholly of the lane's component. After each pop a lane lowers its bound to
// just above its component's best value so far this round; a pick it holds
// above that bound is dropped (it cannot be the component's pick).
template <int DIMP>
__global__ void __launch_bounds__(32 * MST_WARPS) k_mst_noc(
    const float* __restrict__ xs, int64_t n, int64_t P, int64_t L, const float* __restrict__ lo,
    const float* __restrict__ hi, const uint32_t* __restrict__ nd,
    const uint32_t* __restrict__ comp, const float* __restrict__ core,
    const uint32_t* __restrict__ orig, uint32_t* __restrict__ cbest,
    unsigned long long* __restrict__ ckey, uint32_t* __restrict__ bj_out,
    int32_t* __restrict__ status) {
  __shared__ MstLeafStage<DIMP> stage_s[MST_WARPS];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t q0 = ((int64_t)blockIdx.x * MST_WARPS + wid) * 32;
  if (q0 >= n) return;
  MstLeafStage<DIMP>& st = stage_s[wid];
  const int64_t pos = q0 + lane;
  const bool act = pos < n;
  if (act) bj_out[pos] = NO_POINT;
  const uint32_t root_c = nd[1];
  const uint32_t qc = act ? comp[pos] : NC_MIXED;
  const float cq = act ? core[pos] : 0.0f;
  float bd = __uint_as_float(FMAX_BITS);
  bool live = act && root_c != qc;  // root_c == qc: a single component
  if (live) {
    const uint32_t bb = __ldcg(cbest + qc);
    if (bb < FMAX_BITS) bd = __uint_as_float(bb + 1u);
    live = !(cq > bd);
  }
  if (!__any_sync(FULL, live)) return;
  const unsigned actm = __ballot_sync(FULL, act);
  float q[DIMP];
  mst_load<DIMP>(xs, act ? pos : q0, q);
  uint32_t bj = NO_POINT, bo = 0;
  uint32_t stk = 0;
  int sp = 0;
  int64_t v = 1;
  float lbv = 0.0f;
  for (;;) {
    const bool need = live && !(lbv > bd) && nd[v] != qc;
    if (__any_sync(FULL, need)) {
      if (v >= P) {
        const int64_t l = v - P;
        if (l < L) {
          const int64_t b0 = l * MST_LEAF;
          const int cnt = (int)min((int64_t)MST_LEAF, n - b0);
          __syncwarp();
          mst_stage_leaf<DIMP>(st, xs, b0, cnt, lane);
          if (lane < cnt) {
            st.comp[lane] = comp[b0 + lane];
            st.core[lane] = core[b0 + lane];
            st.orig[lane] = orig[b0 + lane];
          }
          __syncwarp();
          if (need) {
            for (int s2 = 0; s2 < cnt; ++s2) {
              if (st.comp[s2] == qc) continue;
              const float cj = st.core[s2];
              if (cj > bd) continue;
              float y[DIMP];
              mst_staged<DIMP>(st, s2, y);
              const float mr = fmaxf(fmaxf(mst_sqd<DIMP>(q, y), cq), cj);
              const uint32_t oj = st.orig[s2];
              if (mr < bd || (mr == bd && bj != NO_POINT && oj < bo)) {
                bd = mr;
                bj = (uint32_t)(b0 + s2);
                bo = oj;
              }
            }
          }
        }
      } else {
        const float l0 = mst_box_lb<DIMP>(lo, hi, 2 * v, q);
        const float l1 = mst_box_lb<DIMP>(lo, hi, 2 * v + 1, q);
        const bool ok = live && !(cq > bd);
        const bool n0 = __any_sync(FULL, ok && !(l0 > bd) && nd[2 * v] != qc);
        const bool n1 = __any_sync(FULL, ok && !(l1 > bd) && nd[2 * v + 1] != qc);
        if (n0 || n1) {
          const bool left = 2 * __popc(__ballot_sync(FULL, l0 <= l1) & actm) >= __popc(actm);
          const bool na = left ? n0 : n1, nb = left ? n1 : n0;
          const int64_t a = left ? 2 * v : 2 * v + 1;
          if (na && nb) {
            if (sp >= 32) {
              if (lane == 0) set_status(status, ST_INTERNAL);
              return;
            }
            if (lane == sp) stk = (uint32_t)(a ^ 1);
            ++sp;
          }
          const int64_t c = na ? a : (a ^ 1);
          lbv = (c == 2 * v) ? l0 : l1;
          v = c;
          continue;
        }
      }
    }
    if (sp == 0) break;
    --sp;
    v = __shfl_sync(FULL, stk, sp);
    lbv = mst_box_lb<DIMP>(lo, hi, v, q);
    if (live) {  // the component's best so far, found by other lanes and warps
      const uint32_t cb = __ldcg(cbest + qc);
      if (cb < FMAX_BITS) {
        const float nb = __uint_as_float(cb + 1u);
        if (nb < bd) {
          bd = nb;
          bj = NO_POINT;
        }
      }
      live = !(cq > bd);
    }
  }
  if (bj != NO_POINT) {
    bj_out[pos] = bj;
    const uint32_t db = __float_as_uint(bd);
    atomicMin(cbest + qc, db);
    atomicMin(ckey + qc, ((unsigned long long)db << 32) | orig[pos]);
  }
}

// Per active component k (id A[k]): its pick (point, other point, value bits)
// and the component of the other end.
__global__ void k_mst_picks(const uint32_t* __restrict__ A, int64_t m,
                            const unsigned long long* __restrict__ ckey,
                            const uint32_t* __restrict__ pos_of, const uint32_t* __restrict__ bj,
                            const uint32_t* __restrict__ orig, const uint32_t* __restrict__ comp,
                            uint32_t* __restrict__ succ, uint32_t* __restrict__ eu,
                            uint32_t* __restrict__ ev, uint32_t* __restrict__ ew,
                            int32_t* __restrict__ has) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const uint32_t c = A[k];
  const unsigned long long key = ckey[c];
  if (key == ~0ull) {
    succ[c] = c;
    has[k] = 0;
    return;
  }
  const uint32_t i = (uint32_t)key, pj = bj[pos_of[i]];
  succ[c] = comp[pj];
  eu[k] = i;
  ev[k] = orig[pj];
  ew[k] = (uint32_t)(key >> 32);
  has[k] = 1;
}

__global__ void k_mst_dbl_init(const uint32_t* __restrict__ A, int64_t m,
                               const uint32_t* __restrict__ succ, uint32_t* __restrict__ jmp,
                               uint32_t* __restrict__ mx, uint32_t* __restrict__ oncyc) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const uint32_t c = A[k], s = succ[c];
  jmp[c] = s;
  mx[c] = max(c, s);
  oncyc[c] = 0u;
}

// One doubling step: jmp becomes succ applied twice as often, and mx the
// maximum over the path c .. jmp (both inclusive).
__global__ void k_mst_dbl_step(const uint32_t* __restrict__ A, int64_t m,
                               const uint32_t* __restrict__ jin, const uint32_t* __restrict__ min_,
                               uint32_t* __restrict__ jout, uint32_t* __restrict__ mout) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const uint32_t c = A[k], j = jin[c];
  jout[c] = jin[j];
  mout[c] = max(min_[c], min_[j]);
}

__global__ void k_mst_mark(const uint32_t* __restrict__ A, int64_t m,
                           const uint32_t* __restrict__ jmp, uint32_t* __restrict__ oncyc) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  oncyc[jmp[A[k]]] = 1u;
}

// The skipped pick of each cycle: its largest component (also a component
// without a pick). par: the skipped component itself, else the pick's target.
__global__ void k_mst_skip(const uint32_t* __restrict__ A, int64_t m,
                           const uint32_t* __restrict__ succ, const uint32_t* __restrict__ mx,
                           const uint32_t* __restrict__ oncyc, const int32_t* __restrict__ has,
                           uint32_t* __restrict__ par, uint32_t* __restrict__ nid,
                           int32_t* __restrict__ keep) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const uint32_t c = A[k];
  const bool root = oncyc[c] != 0u && mx[c] == c;
  par[c] = root ? c : succ[c];
  nid[c] = 0xffffffffu;
  keep[k] = (has[k] && !root) ? 1 : 0;
}

__global__ void k_mst_jump(const uint32_t* __restrict__ A, int64_t m,
                           const uint32_t* __restrict__ pin, uint32_t* __restrict__ pout) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const uint32_t c = A[k];
  pout[c] = pin[pin[c]];
}

__global__ void k_mst_newid(const uint32_t* __restrict__ A, int64_t m,
                            const uint32_t* __restrict__ par, uint32_t* __restrict__ nid) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const uint32_t c = A[k];
  atomicMin(nid + par[c], c);
}

__global__ void k_mst_label(const uint32_t* __restrict__ A, int64_t m,
                            const uint32_t* __restrict__ par, const uint32_t* __restrict__ nid,
                            uint32_t* __restrict__ lab, int32_t* __restrict__ alive) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const uint32_t c = A[k], l = nid[par[c]];
  lab[c] = l;
  alive[k] = l == c ? 1 : 0;
}

// Kept picks appended at base in ascending component id; weights square-rooted.
__global__ void k_mst_emit(int64_t m, const int32_t* __restrict__ keep,
                           const int64_t* __restrict__ off, const uint32_t* __restrict__ eu,
                           const uint32_t* __restrict__ ev, const uint32_t* __restrict__ ew,
                           int64_t base, int64_t* __restrict__ u, int64_t* __restrict__ v,
                           float* __restrict__ w) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m || !keep[k]) return;
  const int64_t o = base + off[k];
  u[o] = eu[k];
  v[o] = ev[k];
  w[o] = fsqrt(__uint_as_float(ew[k]));
}

__global__ void k_mst_relabel(uint32_t* __restrict__ comp, int64_t n,
                              const uint32_t* __restrict__ lab) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) comp[i] = lab[comp[i]];
}

__global__ void k_mst_compact(const uint32_t* __restrict__ A, int64_t m,
                              const int32_t* __restrict__ alive, const int64_t* __restrict__ off,
                              uint32_t* __restrict__ A2) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < m && alive[k]) A2[off[k]] = A[k];
}

__global__ void k_mst_iota(uint32_t* __restrict__ a, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = (uint32_t)i;
}

int log2_ceil(int64_t m) {
  int k = 0;
  while (((int64_t)1 << k) < m) ++k;
  return k;
}

template <int DIMP>
void launch_core(int kmax_bucket, const float* xs, int64_t n, int64_t P, int64_t L,
                 const float* lo, const float* hi, int k, float* core, uint32_t* kj, float* kd,
                 int32_t* st, cudaStream_t s) {
  const unsigned g = grid_of((n + 31) / 32, MST_WARPS);
  switch (kmax_bucket) {
    case 8: k_mst_core<DIMP, 8><<<g, 32 * MST_WARPS, 0, s>>>(xs, n, P, L, lo, hi, k, core, kj, kd, st); break;
    case 16: k_mst_core<DIMP, 16><<<g, 32 * MST_WARPS, 0, s>>>(xs, n, P, L, lo, hi, k, core, kj, kd, st); break;
    case 32: k_mst_core<DIMP, 32><<<g, 32 * MST_WARPS, 0, s>>>(xs, n, P, L, lo, hi, k, core, kj, kd, st); break;
    default: k_mst_core<DIMP, 64><<<g, 32 * MST_WARPS, 0, s>>>(xs, n, P, L, lo, hi, k, core, kj, kd, st); break;
  }
  EVOC_CHECK_LAUNCH();
}

template <int DIMP>
int64_t mst_run(evoc_ctx* ctx, const float* d_data, int64_t n, int dim, int k, int64_t* d_u,
                int64_t* d_v, float* d_w) {
  cudaStream_t s = ctx->stream;
  int32_t* st = ctx->status.get();
  StageTrace tr(s);
  // bounding box and Morton order
  DevBuf<uint32_t> bmin(dim, s), bmax(dim, s);
  EVOC_CUDA(cudaMemsetAsync(bmin.get(), 0xff, bmin.bytes(), s));
  EVOC_CUDA(cudaMemsetAsync(bmax.get(), 0, bmax.bytes(), s));
  {
    const unsigned gx = (unsigned)std::min<int64_t>(grid_of(n), 4 * ctx->num_sms);
    k_mst_bbox<<<dim3(gx, dim), 256, 0, s>>>(d_data, n, dim, bmin.get(), bmax.get(), st);
    EVOC_CHECK_LAUNCH();
  }
  check_status(ctx, "build_mst");  // non-finite coordinates are rejected before any search
  const int bits = std::min(16, 64 / dim), total_bits = bits * dim;
  DevBuf<uint32_t> key(n, s);
  DevBuf<uint2> val(n, s);
  k_mst_morton<<<grid_of(n), 256, 0, s>>>(d_data, n, dim, bits, bmin.get(), bmax.get(), key.get(),
                                          val.get());
  EVOC_CHECK_LAUNCH();
  radix_sort_pairs(key.get(), val.get(), n, std::min(32, total_bits), s);
  if (total_bits > 32) {
    k_mst_hi_keys<<<grid_of(n), 256, 0, s>>>(val.get(), n, key.get());
    EVOC_CHECK_LAUNCH();
    radix_sort_pairs(key.get(), val.get(), n, total_bits - 32, s);
  }
  DevBuf<float> xs(n * DIMP, s);
  DevBuf<uint32_t> orig(n, s), pos_of(n, s);
  k_mst_gather<DIMP><<<grid_of(n), 256, 0, s>>>(d_data, n, dim, val.get(), xs.get(), orig.get(),
                                                pos_of.get());
  EVOC_CHECK_LAUNCH();
  key.release();
  val.release();
  tr.mark("morton order");
  // implicit tree
  const int64_t L = (n + MST_LEAF - 1) / MST_LEAF;
  int64_t P = 1;
  while (P < L) P <<= 1;
  DevBuf<float> lo(2 * P * DIMP, s), hi(2 * P * DIMP, s);
  k_mst_leaf_boxes<DIMP><<<grid_of(P), 256, 0, s>>>(xs.get(), n, P, L, lo.get(), hi.get());
  EVOC_CHECK_LAUNCH();
  for (int64_t first = P >> 1; first >= 1; first >>= 1) {
    k_mst_level_boxes<DIMP><<<grid_of(first), 256, 0, s>>>(lo.get(), hi.get(), first, first);
    EVOC_CHECK_LAUNCH();
  }
  tr.mark("tree boxes");
  // core distances
  DevBuf<float> core(n, s), knn_d(n * (int64_t)k, s);
  DevBuf<uint32_t> knn_j(n * (int64_t)k, s);
  if (k == 0) {
    EVOC_CUDA(cudaMemsetAsync(core.get(), 0, core.bytes(), s));
  } else {
    const int kb = k <= 8 ? 8 : k <= 16 ? 16 : k <= 32 ? 32 : 64;
    launch_core<DIMP>(kb, xs.get(), n, P, L, lo.get(), hi.get(), k, core.get(), knn_j.get(),
                      knn_d.get(), st, s);
  }
  tr.mark("core distances");
  // Boruvka rounds
  DevBuf<uint32_t> comp(n, s), nd(2 * P, s), cbest(n, s), bj(n, s), succ(n, s);
  DevBuf<unsigned long long> ckey(n, s);
  DevBuf<uint32_t> jA(n, s), jB(n, s), mA(n, s), mB(n, s), oncyc(n, s), nid(n, s), lab(n, s);
  DevBuf<uint32_t> A(n, s), A2(n, s), eu(n, s), ev(n, s), ew(n, s);
  DevBuf<int32_t> has(n, s), keep(n, s), alive(n, s);
  DevBuf<int64_t> off(n + 1, s), off2(n + 1, s);
  EVOC_CUDA(cudaMemcpyAsync(comp.get(), orig.get(), comp.bytes(), cudaMemcpyDeviceToDevice, s));
  k_mst_iota<<<grid_of(n), 256, 0, s>>>(A.get(), n);
  EVOC_CHECK_LAUNCH();
  int64_t m = n, len = 0;
  int64_t h_tot[2];
  while (m > 1 && len < n - 1) {
    const unsigned gm = grid_of(m), gn = grid_of(n);
    k_mst_leaf_comp<<<grid_of(P), 256, 0, s>>>(comp.get(), n, P, L, nd.get());
    EVOC_CHECK_LAUNCH();
    for (int64_t first = P >> 1; first >= 1; first >>= 1) {
      k_mst_level_comp<<<grid_of(first), 256, 0, s>>>(nd.get(), first, first);
      EVOC_CHECK_LAUNCH();
    }
    k_mst_round_reset<<<gm, 256, 0, s>>>(A.get(), m, cbest.get(), ckey.get());
    EVOC_CHECK_LAUNCH();
    if (k > 0) {
      k_mst_knn_bound<<<gn, 256, 0, s>>>(n, k, knn_j.get(), knn_d.get(), comp.get(), core.get(),
                                         cbest.get());
      EVOC_CHECK_LAUNCH();
    }
    k_mst_noc<DIMP><<<grid_of((n + 31) / 32, MST_WARPS), 32 * MST_WARPS, 0, s>>>(xs.get(), n, P, L, lo.get(), hi.get(),
                                                     nd.get(), comp.get(), core.get(), orig.get(),
                                                     cbest.get(), ckey.get(), bj.get(), st);
    EVOC_CHECK_LAUNCH();
    k_mst_picks<<<gm, 256, 0, s>>>(A.get(), m, ckey.get(), pos_of.get(), bj.get(), orig.get(),
                                   comp.get(), succ.get(), eu.get(), ev.get(), ew.get(), has.get());
    EVOC_CHECK_LAUNCH();
    // cycles of the pick graph: 2^K >= m doubling steps
    const int K = std::max(1, log2_ceil(m));
    k_mst_dbl_init<<<gm, 256, 0, s>>>(A.get(), m, succ.get(), jA.get(), mA.get(), oncyc.get());
    EVOC_CHECK_LAUNCH();
    uint32_t *jin = jA.get(), *jout = jB.get(), *min_ = mA.get(), *mout = mB.get();
    for (int t = 0; t < K; ++t) {  // after t steps: jmp = succ^(2^(t+1)), mx over that path
      k_mst_dbl_step<<<gm, 256, 0, s>>>(A.get(), m, jin, min_, jout, mout);
      EVOC_CHECK_LAUNCH();
      std::swap(jin, jout);
      std::swap(min_, mout);
    }
    k_mst_mark<<<gm, 256, 0, s>>>(A.get(), m, jin, oncyc.get());
    EVOC_CHECK_LAUNCH();
    // the skipped picks, then the merged components by pointer jumping
    uint32_t *pin = jout, *pout = mout;  // free ping-pong buffers
    k_mst_skip<<<gm, 256, 0, s>>>(A.get(), m, succ.get(), min_, oncyc.get(), has.get(), pin,
                                  nid.get(), keep.get());
    EVOC_CHECK_LAUNCH();
    for (int t = 0; t <= K; ++t) {
      k_mst_jump<<<gm, 256, 0, s>>>(A.get(), m, pin, pout);
      EVOC_CHECK_LAUNCH();
      std::swap(pin, pout);
    }
    k_mst_newid<<<gm, 256, 0, s>>>(A.get(), m, pin, nid.get());
    EVOC_CHECK_LAUNCH();
    k_mst_label<<<gm, 256, 0, s>>>(A.get(), m, pin, nid.get(), lab.get(), alive.get());
    EVOC_CHECK_LAUNCH();
    exclusive_scan_i32_to_i64(keep.get(), off.get(), m, s);
    exclusive_scan_i32_to_i64(alive.get(), off2.get(), m, s);
    k_mst_emit<<<gm, 256, 0, s>>>(m, keep.get(), off.get(), eu.get(), ev.get(), ew.get(), len,
                                  d_u, d_v, d_w);
    EVOC_CHECK_LAUNCH();
    k_mst_relabel<<<gn, 256, 0, s>>>(comp.get(), n, lab.get());
    EVOC_CHECK_LAUNCH();
    k_mst_compact<<<gm, 256, 0, s>>>(A.get(), m, alive.get(), off2.get(), A2.get());
    EVOC_CHECK_LAUNCH();
    EVOC_CUDA(cudaMemcpyAsync(&h_tot[0], off.get() + m, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaMemcpyAsync(&h_tot[1], off2.get() + m, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaStreamSynchronize(s));
    std::swap(A, A2);
    const int64_t kept = h_tot[0];
    len += kept;
    if (tr.on) {
      const std::string name = "round, " + std::to_string(m) + " components";
      tr.mark(name.c_str());
    }
    m = h_tot[1];
    if (kept == 0) break;  // no pick merged anything (mst.rs:143-160)
  }
  return len;
}

}  // namespace

int64_t build_mst_device(evoc_ctx* ctx, const float* d_data, int64_t n, int32_t dim,
                         int32_t min_samples, int64_t* d_u, int64_t* d_v, float* d_w) {
  if (n < 0) throw Error(EVOC_ERR_INVALID_ARGUMENT, "n must be >= 0");
  if (n > 0xfffffff0LL) throw Error(EVOC_ERR_UNSUPPORTED, "n must be below 2^32 - 16");
  if (dim < 1 || dim > 16) throw Error(EVOC_ERR_UNSUPPORTED, "dim must be in 1..16");
  if (min_samples < 0) throw Error(EVOC_ERR_INVALID_ARGUMENT, "min_samples must be >= 0");
  if (n <= 1) return 0;
  if (!d_data || !d_u || !d_v || !d_w)
    throw Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  const int k = (int)std::min<int64_t>(min_samples, n - 1);
  if (k > 64) throw Error(EVOC_ERR_UNSUPPORTED, "min_samples above 64 is not supported");
  if (dim <= 4) return mst_run<4>(ctx, d_data, n, dim, k, d_u, d_v, d_w);
  if (dim <= 8) return mst_run<8>(ctx, d_data, n, dim, k, d_u, d_v, d_w);
  return mst_run<16>(ctx, d_data, n, dim, k, d_u, d_v, d_w);
}

}  // namespace evoc
