// label_prop.cu — the partition step of the label-propagation initialisation
// (evoc-rs 0.2.7, src/graph/label_prop.rs:45-230) on the GPU.
//
//   seed      approx_n_parts random nodes get labels 0.. (a later draw of the
//             same node overwrites: label_prop.rs:216-219);
//   iterate   n_iter conservative rounds (label_prop.rs:45-92): an unlabelled
//             node sums its neighbours' weights per label in row order, and
//             adopts the label with the largest total if that total is at
//             least 1.0 (ties: the label that first appears last);
//   mop up    unlabelled nodes walk a LIFO stack of at most 64 pops for a
//             labelled node, else take a random existing label
//             (label_prop.rs:105-142); the reference's sequential order is
//             kept by resolving walks that meet earlier outliers afterwards;
//   remap     labels to 0..n_parts in sorted order, any -1 to new ids in
//             node order (label_prop.rs:155-180).
//
// The vote sums are the same f32 additions in the same order as the
// reference's loop, so labels match the CPU restatement exactly. Random draws
// come from Philox4x32-10 (counters below) instead of rand::SmallRng. Each
// node keeps its vote table in its own CSR row range of a scratch array
// (a row has at most as many distinct labels as entries), so no node can
// overflow it; rows longer than 64 also get a hash index (at most half full)
// in four entries per row of two more scratch arrays.
#include "evoc_internal.h"
#include "evoc_device.cuh"

#include <algorithm>

namespace evoc {
namespace {

__device__ __forceinline__ uint32_t lp_seed_draw(uint64_t seed, uint32_t i, uint32_t n) {
  const uint4 o = philox4x32_10(make_uint4(i, 0u, 0x4C50u, 0x53454544u),
                                make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
  return __umulhi(o.x, n);
}
__device__ __forceinline__ uint32_t lp_outlier_draw(uint64_t seed, uint64_t i, uint32_t range) {
  const uint4 o = philox4x32_10(make_uint4((uint32_t)i, (uint32_t)(i >> 32), 0x4C50u, 0x4F555431u),
                                make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
  return __umulhi(o.x, range);
}

__global__ void k_lp_fill(int32_t* __restrict__ labels, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) labels[i] = -1;
}

// Draw i labels node lp_seed_draw(i); the largest i drawn for a node is the
// last write of the reference's sequential loop.
__global__ void k_lp_seed(int32_t* __restrict__ labels, int64_t n, int64_t parts, uint64_t seed) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < parts) atomicMax(&labels[lp_seed_draw(seed, (uint32_t)i, (uint32_t)n)], (int32_t)i);
}

// One conservative iteration, thread per node.
// Rows up to this degree search their vote table linearly; longer rows (hubs)
// index it through a hash table, so a vote costs O(1) instead of O(distinct).
constexpr int64_t LP_LINEAR_DEG = 64;

__global__ void k_lp_iter(const int64_t* __restrict__ indptr, const uint32_t* __restrict__ indices,
                          const float* __restrict__ w, int64_t n, const int32_t* __restrict__ in,
                          int32_t* __restrict__ out, int32_t* __restrict__ vlab,
                          float* __restrict__ vsum, const int64_t* __restrict__ hoff,
                          int32_t* __restrict__ hkey, int32_t* __restrict__ hpos,
                          int32_t* __restrict__ changed) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t cur = in[i];
  if (cur >= 0) {
    out[i] = cur;
    return;
  }
  const int64_t b = indptr[i], e = indptr[i + 1], deg = e - b;
  int64_t cnt = 0;  // distinct labelled labels, in first-appearance order
  if (deg <= LP_LINEAR_DEG) {
    for (int64_t q = b; q < e; ++q) {
      const int32_t l = in[indices[q]];
      if (l < 0) continue;  // unlabelled votes never win
      int64_t k = 0;
      while (k < cnt && vlab[b + k] != l) ++k;
      if (k < cnt) {
        vsum[b + k] = __fadd_rn(vsum[b + k], w[q]);
      } else {
        vlab[b + cnt] = l;
        vsum[b + cnt] = w[q];
        ++cnt;
      }
    }
  } else {
    // long row: an open-addressing table (label -> position in vlab/vsum) in
    // the row's own range [hoff[i], hoff[i + 1]) of hkey/hpos, at most half full
    const int64_t cap = hoff[i + 1] - hoff[i];
    int32_t* key = hkey + hoff[i];
    int32_t* hp = hpos + hoff[i];
    for (int64_t h = 0; h < cap; ++h) key[h] = -1;
    const int64_t mask = cap - 1;
    for (int64_t q = b; q < e; ++q) {
      const int32_t l = in[indices[q]];
      if (l < 0) continue;
      int64_t h = (int64_t)(((uint32_t)l * 2654435761u) & (uint32_t)mask);
      while (key[h] != -1 && key[h] != l) h = (h + 1) & mask;
      if (key[h] == l) {
        const int64_t k = hp[h];
        vsum[b + k] = __fadd_rn(vsum[b + k], w[q]);
      } else {
        key[h] = l;
        hp[h] = (int32_t)cnt;
        vlab[b + cnt] = l;
        vsum[b + cnt] = w[q];
        ++cnt;
      }
    }
  }
  int32_t best = -1;
  float max_vote = 1.0f;  // threshold
  for (int64_t k = 0; k < cnt; ++k) {
    const float v = vsum[b + k];
    if (v > max_vote) {
      max_vote = v;
      best = vlab[b + k];
    } else if (v == max_vote) {
      best = vlab[b + k];  // last encountered wins
    }
  }
  out[i] = best;
  if (best >= 0) *changed = 1;
}

// Hash-table slots of each row: the power of two >= 2 deg for rows longer
// than LP_LINEAR_DEG, none for the others (they search their votes linearly).
__global__ void k_lp_hcap(const int64_t* __restrict__ indptr, int64_t n,
                          int64_t* __restrict__ cap_out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t deg = indptr[i + 1] - indptr[i];
  int64_t cap = 0;
  if (deg > LP_LINEAR_DEG) {
    cap = 1;
    while (cap < 2 * deg) cap <<= 1;
  }
  cap_out[i] = cap;
}

__global__ void k_lp_max(const int32_t* __restrict__ labels, int64_t n, int32_t* __restrict__ mx,
                         int32_t* __restrict__ unl) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t l = labels[i];
  unl[i] = l < 0 ? 1 : 0;
  if (l >= 0) atomicMax(mx, l);
}

__global__ void k_lp_list(const int32_t* __restrict__ unl, const int64_t* __restrict__ pos,
                          int64_t n, uint32_t* __restrict__ list) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && unl[i]) list[pos[i]] = (uint32_t)i;
}

// The mop-up (label_prop.rs:105-142) in parallel. In the reference's
// sequential order, outlier i's walk stops at the first node that is labelled
// by then: a node labelled before the mop-up, or an earlier outlier j < i
// (every processed outlier has a label). So each walk runs against the
// labels before the mop-up and yields a label, a pointer to an earlier
// outlier (-2 - its list index), or the fallback draw; k_lp_jump then
// resolves the pointers. A walk pops at most 64 nodes, so only the top 64
// stack entries can ever be popped: the stack is a 64-entry ring that drops
// its bottom entry when full.
__global__ void k_lp_walk(const int64_t* __restrict__ indptr, const uint32_t* __restrict__ indices,
                          const int32_t* __restrict__ labels, const int32_t* __restrict__ unl,
                          const int64_t* __restrict__ pos, const uint32_t* __restrict__ list,
                          int64_t count, int32_t max_label, uint64_t seed,
                          int32_t* __restrict__ res) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= count) return;
  const uint32_t i = list[u];
  uint32_t ring[64];
  int64_t top = 0, bottom = 0;  // entries [bottom, top), slot = index % 64
  ring[0] = i;
  top = 1;
  for (int step = 0; step < 64 && top > bottom; ++step) {
    --top;
    const uint32_t node = ring[top & 63];
    for (int64_t q = indptr[node]; q < indptr[node + 1]; ++q) {
      const uint32_t j = indices[q];
      const int32_t l = labels[j];
      if (l >= 0) {
        res[u] = l;
        return;
      }
      if (unl[j] && j < i) {  // an earlier outlier: labelled by then
        res[u] = (int32_t)(-2 - pos[j]);
        return;
      }
      ring[top & 63] = j;
      ++top;
      if (top - bottom > 64) ++bottom;
    }
  }
  res[u] = (int32_t)lp_outlier_draw(seed, i, (uint32_t)max_label + 1u);
}

// Pointer jumping over the walk results; pointers only go to earlier
// outliers, so the chains end.
__global__ void k_lp_jump(int32_t* __restrict__ res, int64_t count, int32_t* __restrict__ changed) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= count) return;
  const int32_t r = res[u];
  if (r >= 0) return;
  const int32_t rk = res[-2 - (int64_t)r];
  res[u] = rk;
  *changed = 1;
}

__global__ void k_lp_assign(const uint32_t* __restrict__ list, const int32_t* __restrict__ res,
                            int64_t count, int32_t* __restrict__ labels) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u < count) labels[list[u]] = res[u];
}

__global__ void k_lp_present(const int32_t* __restrict__ labels, int64_t n,
                             int32_t* __restrict__ present, int32_t* __restrict__ neg) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t l = labels[i];
  neg[i] = l < 0 ? 1 : 0;
  if (l >= 0) present[l] = 1;
}

__global__ void k_lp_remap(const int32_t* __restrict__ labels, int64_t n,
                           const int64_t* __restrict__ newid, int64_t n_unique,
                           const int64_t* __restrict__ negrank, uint32_t* __restrict__ part) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t l = labels[i];
  part[i] = (uint32_t)(l >= 0 ? newid[l] : n_unique + negrank[i]);
}

inline unsigned grid_for(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace

int64_t label_prop_partition(evoc_ctx* ctx, const evoc_graph* g, int64_t approx_n_parts,
                             int32_t n_iter, uint64_t seed, uint32_t* d_partition) {
  cudaStream_t s = ctx->stream;
  const int64_t n = g->n, nnz = g->nnz;
  if (n == 0) return 0;
  if (approx_n_parts < 0 || approx_n_parts >= (1LL << 31))
    throw Error(EVOC_ERR_INVALID_ARGUMENT, "approx_n_parts outside [0, 2^31)");
  if (n_iter < 0) throw Error(EVOC_ERR_INVALID_ARGUMENT, "n_iter < 0");
  DevBuf<int32_t> la(n, s), lb(n, s), vlab(std::max<int64_t>(nnz, 1), s), flag(1, s);
  DevBuf<float> vsum(std::max<int64_t>(nnz, 1), s);
  // hash tables only for the long rows, packed by a prefix sum of their sizes
  DevBuf<int64_t> hcap(n, s), hoff(n + 1, s);
  k_lp_hcap<<<grid_for(n), 256, 0, s>>>(g->indptr.get(), n, hcap.get());
  EVOC_CHECK_LAUNCH();
  exclusive_scan_i64(hcap.get(), hoff.get(), n, s);
  int64_t htot = 0;
  EVOC_CUDA(cudaMemcpyAsync(&htot, hoff.get() + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaStreamSynchronize(s));
  hcap.release();
  DevBuf<int32_t> hkey(std::max<int64_t>(htot, 1), s), hpos(std::max<int64_t>(htot, 1), s);
  k_lp_fill<<<grid_for(n), 256, 0, s>>>(la.get(), n);
  if (approx_n_parts > 0)
    k_lp_seed<<<grid_for(approx_n_parts), 256, 0, s>>>(la.get(), n, approx_n_parts, seed);
  EVOC_CHECK_LAUNCH();
  // n_iter rounds; a round that labels no node is a fixed point, so the rest
  // would leave the labels unchanged and are skipped.
  for (int32_t it = 0; it < n_iter; ++it) {
    EVOC_CUDA(cudaMemsetAsync(flag.get(), 0, sizeof(int32_t), s));
    k_lp_iter<<<grid_for(n, 128), 128, 0, s>>>(g->indptr.get(), g->indices.get(),
                                               g->weights.get(), n, la.get(), lb.get(),
                                               vlab.get(), vsum.get(), hoff.get(), hkey.get(),
                                               hpos.get(),
                                               flag.get());
    EVOC_CHECK_LAUNCH();
    std::swap(la, lb);
    int32_t h = 0;
    EVOC_CUDA(cudaMemcpyAsync(&h, flag.get(), sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaStreamSynchronize(s));
    if (!h) break;
  }
  // mop-up of the nodes still unlabelled, in node order
  DevBuf<int32_t> mx(1, s), unl(n, s);
  DevBuf<int64_t> pos(n + 1, s);
  EVOC_CUDA(cudaMemsetAsync(mx.get(), 0xff, sizeof(int32_t), s));  // -1
  k_lp_max<<<grid_for(n), 256, 0, s>>>(la.get(), n, mx.get(), unl.get());
  EVOC_CHECK_LAUNCH();
  exclusive_scan_i32_to_i64(unl.get(), pos.get(), n, s);
  int64_t count = 0;
  EVOC_CUDA(cudaMemcpyAsync(&count, pos.get() + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaStreamSynchronize(s));
  int32_t max_label = -1;
  EVOC_CUDA(cudaMemcpyAsync(&max_label, mx.get(), sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaStreamSynchronize(s));
  if (count > 0 && max_label >= 0) {
    DevBuf<uint32_t> list(count, s);
    DevBuf<int32_t> res(count, s);
    k_lp_list<<<grid_for(n), 256, 0, s>>>(unl.get(), pos.get(), n, list.get());
    k_lp_walk<<<grid_for(count, 128), 128, 0, s>>>(g->indptr.get(), g->indices.get(), la.get(),
                                                   unl.get(), pos.get(), list.get(), count,
                                                   max_label, seed + 2000, res.get());
    EVOC_CHECK_LAUNCH();
    for (int pass = 0; pass < 64; ++pass) {  // chains halve per pass
      EVOC_CUDA(cudaMemsetAsync(flag.get(), 0, sizeof(int32_t), s));
      k_lp_jump<<<grid_for(count), 256, 0, s>>>(res.get(), count, flag.get());
      EVOC_CHECK_LAUNCH();
      int32_t h = 0;
      EVOC_CUDA(cudaMemcpyAsync(&h, flag.get(), sizeof(int32_t), cudaMemcpyDeviceToHost, s));
      EVOC_CUDA(cudaStreamSynchronize(s));
      if (!h) break;
    }
    k_lp_assign<<<grid_for(count), 256, 0, s>>>(list.get(), res.get(), count, la.get());
    EVOC_CHECK_LAUNCH();
  }
  // remap: labels are below approx_n_parts, or -1 if nothing was labelled
  const int64_t np = std::max<int64_t>(approx_n_parts, 1);
  DevBuf<int32_t> present(np, s), neg(n, s);
  DevBuf<int64_t> newid(np + 1, s), negrank(n + 1, s);
  EVOC_CUDA(cudaMemsetAsync(present.get(), 0, np * sizeof(int32_t), s));
  k_lp_present<<<grid_for(n), 256, 0, s>>>(la.get(), n, present.get(), neg.get());
  EVOC_CHECK_LAUNCH();
  exclusive_scan_i32_to_i64(present.get(), newid.get(), np, s);
  exclusive_scan_i32_to_i64(neg.get(), negrank.get(), n, s);
  int64_t n_unique = 0, n_neg = 0;
  EVOC_CUDA(cudaMemcpyAsync(&n_unique, newid.get() + np, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaMemcpyAsync(&n_neg, negrank.get() + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaStreamSynchronize(s));
  k_lp_remap<<<grid_for(n), 256, 0, s>>>(la.get(), n, newid.get(), n_unique, negrank.get(),
                                         d_partition);
  EVOC_CHECK_LAUNCH();
  return n_unique + n_neg;
}

}  // namespace evoc
