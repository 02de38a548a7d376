// label_prop.cu — the partition step of the label-propagation initialisation
// (evoc-rs 0.2.7, src/graph/label_prop.rs:45-230) on the GPU.
//
//   seed      approx_n_parts random nodes get labels 0.. (a later draw of the
//             same node overwrites: label_prop.rs:216-219);
//   iterate   n_iter conservative rounds (label_prop.rs:45-92): an unlabelled
//             node sums its neighbours' weights per label in row order, and
//             adopts the label with the largest total if that total is at
//             least 1.0 (ties: the label that first appears last);
//   mop up    unlabelled nodes, in node order, walk a LIFO stack of at most
//             64 pops for a labelled node, else take a random existing label
//             (label_prop.rs:105-142);
//   remap     labels to 0..n_parts in sorted order, any -1 to new ids in
//             node order (label_prop.rs:155-180).
//
// The vote sums are the same f32 additions in the same order as the
// reference's loop, so labels match the CPU restatement exactly. Random draws
// come from Philox4x32-10 (counters below) instead of rand::SmallRng. Each
// node keeps its vote table in its own CSR row range of a scratch array
// (a row has at most as many distinct labels as entries), so no node can
// overflow it.
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
__global__ void k_lp_iter(const int64_t* __restrict__ indptr, const uint32_t* __restrict__ indices,
                          const float* __restrict__ w, int64_t n, const int32_t* __restrict__ in,
                          int32_t* __restrict__ out, int32_t* __restrict__ vlab,
                          float* __restrict__ vsum, int32_t* __restrict__ changed) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t cur = in[i];
  if (cur >= 0) {
    out[i] = cur;
    return;
  }
  const int64_t b = indptr[i], e = indptr[i + 1];
  int64_t cnt = 0;  // distinct labelled labels, in first-appearance order
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

// The sequential mop-up: one thread, unlabelled nodes in node order. Each
// walk pops at most 64 nodes and pushes at most max_degree per pop, so the
// stack (1 + 64 max_degree entries) cannot overflow.
__global__ void k_lp_outliers(const int64_t* __restrict__ indptr,
                              const uint32_t* __restrict__ indices, int32_t* __restrict__ labels,
                              const uint32_t* __restrict__ list, int64_t count,
                              const int32_t* __restrict__ mx, uint64_t seed,
                              uint32_t* __restrict__ stack) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const int32_t max_label = *mx;
  if (max_label < 0) return;
  for (int64_t u = 0; u < count; ++u) {
    const uint32_t i = list[u];
    int64_t top = 0;
    stack[top++] = i;
    bool found = false;
    for (int step = 0; step < 64 && !found && top > 0; ++step) {
      const uint32_t node = stack[--top];
      for (int64_t q = indptr[node]; q < indptr[node + 1]; ++q) {
        const uint32_t j = indices[q];
        if (labels[j] >= 0) {
          labels[i] = labels[j];
          found = true;
          break;
        }
        stack[top++] = j;
      }
    }
    if (!found) labels[i] = (int32_t)lp_outlier_draw(seed, i, (uint32_t)max_label + 1u);
  }
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

__global__ void k_lp_maxdeg(const int64_t* __restrict__ indptr, int64_t n,
                            unsigned long long* __restrict__ mx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicMax(mx, (unsigned long long)(indptr[i + 1] - indptr[i]));
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
                                               vlab.get(), vsum.get(), flag.get());
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
  if (count > 0) {
    DevBuf<unsigned long long> md(1, s);
    EVOC_CUDA(cudaMemsetAsync(md.get(), 0, sizeof(unsigned long long), s));
    k_lp_maxdeg<<<grid_for(n), 256, 0, s>>>(g->indptr.get(), n, md.get());
    unsigned long long maxdeg = 0;
    EVOC_CUDA(cudaMemcpyAsync(&maxdeg, md.get(), sizeof(maxdeg), cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaStreamSynchronize(s));
    DevBuf<uint32_t> list(count, s), stack(1 + 64 * (size_t)maxdeg, s);
    k_lp_list<<<grid_for(n), 256, 0, s>>>(unl.get(), pos.get(), n, list.get());
    k_lp_outliers<<<1, 32, 0, s>>>(g->indptr.get(), g->indices.get(), la.get(), list.get(), count,
                                   mx.get(), seed + 2000, stack.get());
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
