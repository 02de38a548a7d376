// capi.cu — the extern "C" boundary of the GB300 EVoC library.
//
// Each entry point validates its arguments on the host, runs the device work
// on the context's stream, reads the device status word (kernels never trap;
// they set bits that become error codes here) and returns a status code.
// C++ exceptions never cross the boundary.
#include "evoc_internal.h"

#include <cmath>
#include <cstring>
#include <memory>
#include <new>

namespace {

thread_local std::string g_thread_error = "";

void set_err(evoc_ctx* ctx, const std::string& m) {
  if (ctx)
    ctx->last_error = m;
  else
    g_thread_error = m;
}

__global__ void k_validate_indices(const uint32_t* __restrict__ idx,
                                   int64_t nnz, int64_t n,
                                   int32_t* __restrict__ status) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nnz && (int64_t)idx[q] >= n) atomicOr(status, (int32_t)evoc::ST_BAD_INDEX);
}

void use_device(evoc_ctx* ctx) { EVOC_CUDA(cudaSetDevice(ctx->device)); }

// Concatenated kNN lists of many problems: each entry of problem p (rows
// [row_start[p], row_start[p + 1])) gets the problem's first row added, so
// the lists form one block-diagonal kNN graph; padding stays padding, and an
// index outside the problem sets the status.
__global__ void k_knn_offset(uint32_t* __restrict__ idx, int64_t total, int32_t k,
                             const int64_t* __restrict__ row_start, int32_t m,
                             int32_t* __restrict__ status) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= total * (int64_t)k) return;
  const uint32_t v = idx[e];
  if (v == 0xFFFFFFFFu) return;
  const int64_t row = e / k;
  int lo = 0, hi = m - 1;  // last problem whose first row is <= row
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (row_start[mid] <= row) lo = mid; else hi = mid - 1;
  }
  const int64_t base = row_start[lo], np = row_start[lo + 1] - base;
  if ((int64_t)v >= np) {
    atomicOr(status, (int32_t)evoc::ST_BAD_INDEX);
    return;
  }
  idx[e] = (uint32_t)(v + base);
}

// Self removal of a raw kNN search result (n rows of kr candidates that may
// include the query itself): row i keeps its first k entries whose index is
// not i, in order, and pads the rest with EVOC_KNN_PAD -- the reference's
// filter(|j| j != i).take(k) (nearest_neighbour_gpu.rs:289-300), on the device.
__global__ void k_knn_drop_self(const uint32_t* __restrict__ idx_raw,
                                const float* __restrict__ dist_raw, int64_t n, int32_t kr,
                                int32_t k, uint32_t* __restrict__ idx, float* __restrict__ dist) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t* ri = idx_raw + i * kr;
  const float* rd = dist_raw + i * kr;
  uint32_t* oi = idx + i * k;
  float* od = dist + i * k;
  int c = 0;
  for (int j = 0; j < kr && c < k; ++j) {
    const uint32_t v = ri[j];
    if ((int64_t)v == i) continue;
    oi[c] = v;
    od[c] = rd[j];
    ++c;
  }
  for (; c < k; ++c) {
    oi[c] = EVOC_KNN_PAD;
    od[c] = 0.0f;
  }
}

std::vector<evoc::ProblemDesc> block_problems(const evoc_graph_t* g, int32_t m,
                                              const int64_t* n_per, const uint64_t* seeds) {
  if (!g || m <= 0 || !n_per || !seeds)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "bad argument");
  std::vector<evoc::ProblemDesc> probs;
  int64_t b = 0;
  for (int32_t q = 0; q < m; ++q) {
    if (n_per[q] < 0) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "negative block size");
    probs.push_back({g, seeds[q], b, n_per[q]});
    b += n_per[q];
  }
  if (b != g->n)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "block sizes do not add up to the graph's n");
  return probs;
}

}  // namespace

void evoc::set_thread_error(const std::string& message) { g_thread_error = message; }

#define EVOC_API_BEGIN try {
#define EVOC_API_END(ctx)                                        \
  }                                                              \
  catch (const evoc::Error& e) {                                 \
    set_err(ctx, e.what());                                      \
    return e.code;                                               \
  }                                                              \
  catch (const std::bad_alloc&) {                                \
    set_err(ctx, "host allocation failed");                      \
    return EVOC_ERR_OUT_OF_MEMORY;                               \
  }                                                              \
  catch (const std::exception& e) {                              \
    set_err(ctx, e.what());                                      \
    return EVOC_ERR_INTERNAL;                                    \
  }                                                              \
  return EVOC_OK;

extern "C" {

int evoc_abi_version(void) { return EVOC_ABI_VERSION; }

void evoc_embed_params_default(evoc_embed_params_t* p) {
  if (!p) return;
  p->n_epochs = 50;
  p->noise_level = 0.5f;
  p->negative_sample_rate = 1.0f;
  p->initial_alpha = 0.1f;
  p->beta1 = 0.5f;
  p->beta2 = 0.9f;
  p->eps = 1e-7f;
}

int evoc_ctx_create(int device, evoc_ctx_t** out) {
  evoc_ctx* ctx = nullptr;
  EVOC_API_BEGIN
  if (!out) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    (void)cudaGetLastError();
    throw evoc::Error(EVOC_ERR_NO_DEVICE, "no CUDA device available");
  }
  if (device < 0 || device >= count)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "device index out of range");
  cudaDeviceProp prop;
  EVOC_CUDA(cudaGetDeviceProperties(&prop, device));
  if (!(prop.major == 10 && prop.minor == 3))
    throw evoc::Error(EVOC_ERR_NO_DEVICE,
                      std::string("this library is built for sm_103a; device is ") +
                          prop.name + " (sm_" + std::to_string(prop.major) +
                          std::to_string(prop.minor) + ")");
  std::unique_ptr<evoc_ctx> c(new evoc_ctx());
  c->device = device;
  c->num_sms = prop.multiProcessorCount;
  EVOC_CUDA(cudaSetDevice(device));
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;  // keep freed blocks for reuse in this process
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  (void)cudaGetLastError();
  EVOC_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  c->status.alloc(1, c->stream);
  EVOC_CUDA(cudaMemsetAsync(c->status.get(), 0, sizeof(int32_t), c->stream));
  c->sk_steps.alloc(1, c->stream);
  EVOC_CUDA(cudaMemsetAsync(c->sk_steps.get(), 0, sizeof(unsigned long long), c->stream));
  EVOC_CUDA(cudaStreamSynchronize(c->stream));
  *out = c.release();
  EVOC_API_END(ctx)
}

void evoc_ctx_destroy(evoc_ctx_t* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  ctx->status.release();
  ctx->sk_steps.release();
  ctx->slot_cache.release();
  if (s) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
  delete ctx;
}

const char* evoc_last_error(const evoc_ctx_t* ctx) {
  return ctx ? ctx->last_error.c_str() : g_thread_error.c_str();
}

void* evoc_ctx_stream(const evoc_ctx_t* ctx) {
  return ctx ? (void*)ctx->stream : nullptr;
}

int evoc_ctx_smooth_knn_steps(evoc_ctx_t* ctx, int64_t* steps) {
  EVOC_API_BEGIN
  if (!ctx || !steps) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  use_device(ctx);
  unsigned long long v = 0;
  EVOC_CUDA(cudaMemcpyAsync(&v, ctx->sk_steps.get(), sizeof(v), cudaMemcpyDeviceToHost,
                            ctx->stream));
  EVOC_CUDA(cudaStreamSynchronize(ctx->stream));
  *steps = (int64_t)v;
  EVOC_API_END(ctx)
}

int evoc_smooth_knn_dist(evoc_ctx_t* ctx, const float* dists,
                         const int32_t* row_len, int64_t n, int32_t k,
                         uint64_t k_target, float local_connectivity,
                         int32_t n_iter, float* sigmas, float* rhos) {
  EVOC_API_BEGIN
  if (!ctx) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "ctx is NULL");
  if (n < 0 || k < 0 || n_iter < 0)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "negative size");
  if (n == 0) return EVOC_OK;
  if (!dists || !sigmas || !rhos || k == 0)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL array or k == 0");
  if (local_connectivity > 0.0f && !std::isfinite(local_connectivity))
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "local_connectivity is not finite");
  if (row_len)
    for (int64_t i = 0; i < n; ++i)
      if (row_len[i] < 0 || row_len[i] > k)
        throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "row_len outside [0, k]");
  use_device(ctx);
  cudaStream_t s = ctx->stream;
  evoc::DevBuf<float> d(n * (int64_t)k, s), sg(n, s), rh(n, s);
  evoc::DevBuf<int32_t> rl;
  EVOC_CUDA(cudaMemcpyAsync(d.get(), dists, d.bytes(), cudaMemcpyHostToDevice, s));
  if (row_len) {
    rl.alloc(n, s);
    EVOC_CUDA(cudaMemcpyAsync(rl.get(), row_len, rl.bytes(), cudaMemcpyHostToDevice, s));
  }
  evoc::smooth_knn_device(ctx, d.get(), rl.get(), n, k, k_target,
                          local_connectivity, n_iter, sg.get(), rh.get(),
                          nullptr, nullptr);
  EVOC_CUDA(cudaMemcpyAsync(sigmas, sg.get(), sg.bytes(), cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaMemcpyAsync(rhos, rh.get(), rh.bytes(), cudaMemcpyDeviceToHost, s));
  evoc::check_status(ctx, "smooth_knn_dist");
  EVOC_API_END(ctx)
}

int evoc_fuzzy_set_device(evoc_ctx_t* ctx, const uint32_t* d_knn_idx,
                          const float* d_knn_dist, int64_t n, int32_t k,
                          float effective_n_neighbours, int symmetrise,
                          float* d_sigmas, float* d_rhos,
                          evoc_graph_t** out_graph) {
  EVOC_API_BEGIN
  if (!ctx || !out_graph)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "ctx or out_graph is NULL");
  *out_graph = nullptr;
  if (n > 0 && (!d_knn_idx || !d_knn_dist))
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL kNN array");
  use_device(ctx);
  std::unique_ptr<evoc_graph> g(new evoc_graph());
  evoc::fuzzy_set_device(ctx, d_knn_idx, d_knn_dist, n, k,
                         effective_n_neighbours, symmetrise != 0, d_sigmas,
                         d_rhos, g.get());
  evoc::check_status(ctx, "fuzzy set");
  *out_graph = g.release();
  EVOC_API_END(ctx)
}

int evoc_fuzzy_set_device_raw(evoc_ctx_t* ctx, const uint32_t* d_knn_idx_raw,
                              const float* d_knn_dist_raw, int64_t n, int32_t k_raw,
                              int32_t k, float effective_n_neighbours, int symmetrise,
                              evoc_graph_t** out_graph) {
  EVOC_API_BEGIN
  if (!ctx || !out_graph)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "ctx or out_graph is NULL");
  *out_graph = nullptr;
  if (n < 0 || k < 1 || k_raw < k)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "need n >= 0 and 1 <= k <= k_raw");
  if (n > 0 && (!d_knn_idx_raw || !d_knn_dist_raw))
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL kNN array");
  use_device(ctx);
  cudaStream_t s = ctx->stream;
  evoc::DevBuf<uint32_t> idx((size_t)n * k, s);
  evoc::DevBuf<float> dist((size_t)n * k, s);
  if (n > 0) {
    k_knn_drop_self<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d_knn_idx_raw, d_knn_dist_raw, n,
                                                               k_raw, k, idx.get(), dist.get());
    EVOC_CHECK_LAUNCH();
  }
  std::unique_ptr<evoc_graph> g(new evoc_graph());
  evoc::fuzzy_set_device(ctx, idx.get(), dist.get(), n, k, effective_n_neighbours,
                         symmetrise != 0, nullptr, nullptr, g.get());
  evoc::check_status(ctx, "fuzzy set");
  *out_graph = g.release();
  EVOC_API_END(ctx)
}

int evoc_fuzzy_set(evoc_ctx_t* ctx, const uint32_t* knn_idx,
                   const float* knn_dist, int64_t n, int32_t k,
                   float effective_n_neighbours, int symmetrise,
                   evoc_graph_t** out_graph) {
  EVOC_API_BEGIN
  if (!ctx || !out_graph)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "ctx or out_graph is NULL");
  *out_graph = nullptr;
  if (n <= 0)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT,
                      "empty kNN graph (build_fuzzy_simplicial_set reads row 0)");
  if (k <= 0) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "k must be positive");
  if (!knn_idx || !knn_dist)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL kNN array");
  use_device(ctx);
  cudaStream_t s = ctx->stream;
  evoc::DevBuf<uint32_t> di(n * (int64_t)k, s);
  evoc::DevBuf<float> dd(n * (int64_t)k, s);
  EVOC_CUDA(cudaMemcpyAsync(di.get(), knn_idx, di.bytes(), cudaMemcpyHostToDevice, s));
  EVOC_CUDA(cudaMemcpyAsync(dd.get(), knn_dist, dd.bytes(), cudaMemcpyHostToDevice, s));
  std::unique_ptr<evoc_graph> g(new evoc_graph());
  evoc::fuzzy_set_device(ctx, di.get(), dd.get(), n, k, effective_n_neighbours,
                         symmetrise != 0, nullptr, nullptr, g.get());
  evoc::check_status(ctx, "fuzzy set");
  *out_graph = g.release();
  EVOC_API_END(ctx)
}

int evoc_fuzzy_set_batched(evoc_ctx_t* ctx, int32_t n_problems,
                           const uint32_t* const* knn_idx, const float* const* knn_dist,
                           const int64_t* n_per, int32_t k, float effective_n_neighbours,
                           int symmetrise, evoc_graph_t** out_graph) {
  EVOC_API_BEGIN
  if (!ctx || !out_graph || n_problems <= 0 || !knn_idx || !knn_dist || !n_per)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "bad argument");
  *out_graph = nullptr;
  if (k <= 0) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "k must be positive");
  std::vector<int64_t> start(n_problems + 1, 0);
  for (int32_t q = 0; q < n_problems; ++q) {
    if (n_per[q] <= 0)
      throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT,
                        "empty kNN graph (build_fuzzy_simplicial_set reads row 0)");
    if (!knn_idx[q] || !knn_dist[q])
      throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL kNN array");
    start[q + 1] = start[q] + n_per[q];
  }
  const int64_t n = start[n_problems];
  if (n >= (int64_t)0xFFFFFFFFu)
    throw evoc::Error(EVOC_ERR_UNSUPPORTED, "more than 2^32-2 points in total");
  use_device(ctx);
  cudaStream_t s = ctx->stream;
  evoc::DevBuf<uint32_t> di(n * (int64_t)k, s);
  evoc::DevBuf<float> dd(n * (int64_t)k, s);
  evoc::DevBuf<int64_t> dstart(n_problems + 1, s);
  for (int32_t q = 0; q < n_problems; ++q) {
    const size_t off = (size_t)start[q] * k, cnt = (size_t)n_per[q] * k;
    EVOC_CUDA(cudaMemcpyAsync(di.get() + off, knn_idx[q], cnt * sizeof(uint32_t),
                              cudaMemcpyHostToDevice, s));
    EVOC_CUDA(cudaMemcpyAsync(dd.get() + off, knn_dist[q], cnt * sizeof(float),
                              cudaMemcpyHostToDevice, s));
  }
  EVOC_CUDA(cudaMemcpyAsync(dstart.get(), start.data(), start.size() * sizeof(int64_t),
                            cudaMemcpyHostToDevice, s));
  k_knn_offset<<<(unsigned)((n * k + 255) / 256), 256, 0, s>>>(di.get(), n, k, dstart.get(),
                                                              n_problems, ctx->status.get());
  EVOC_CHECK_LAUNCH();
  evoc::check_status(ctx, "batched kNN");  // synchronises: `start` goes out of scope
  std::unique_ptr<evoc_graph> g(new evoc_graph());
  evoc::fuzzy_set_device(ctx, di.get(), dd.get(), n, k, effective_n_neighbours,
                         symmetrise != 0, nullptr, nullptr, g.get());
  evoc::check_status(ctx, "fuzzy set");
  *out_graph = g.release();
  EVOC_API_END(ctx)
}

int evoc_graph_from_csr(evoc_ctx_t* ctx, const int64_t* indptr,
                        const uint32_t* indices, const float* weights,
                        int64_t n, evoc_graph_t** out_graph) {
  EVOC_API_BEGIN
  if (!ctx || !out_graph || (n > 0 && !indptr) || n < 0)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "bad argument");
  *out_graph = nullptr;
  if (n >= (int64_t)0xFFFFFFFFu)
    throw evoc::Error(EVOC_ERR_UNSUPPORTED, "n must be < 2^32-1");
  int64_t nnz = 0;
  if (n > 0) {
    if (indptr[0] != 0)
      throw evoc::Error(EVOC_ERR_INVALID_INPUT, "indptr[0] must be 0");
    for (int64_t i = 0; i < n; ++i)
      if (indptr[i + 1] < indptr[i])
        throw evoc::Error(EVOC_ERR_INVALID_INPUT, "indptr must be non-decreasing");
    nnz = indptr[n];
    if (nnz > 0 && (!indices || !weights))
      throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL indices or weights");
  }
  use_device(ctx);
  cudaStream_t s = ctx->stream;
  std::unique_ptr<evoc_graph> g(new evoc_graph());
  g->ctx = ctx;
  g->n = n;
  g->nnz = nnz;
  g->canonical = false;
  g->indptr.alloc(n + 1, s);
  g->indices.alloc(nnz, s);
  g->weights.alloc(nnz, s);
  if (n > 0)
    EVOC_CUDA(cudaMemcpyAsync(g->indptr.get(), indptr, (n + 1) * sizeof(int64_t),
                              cudaMemcpyHostToDevice, s));
  else
    EVOC_CUDA(cudaMemsetAsync(g->indptr.get(), 0, sizeof(int64_t), s));
  if (nnz > 0) {
    EVOC_CUDA(cudaMemcpyAsync(g->indices.get(), indices, nnz * sizeof(uint32_t),
                              cudaMemcpyHostToDevice, s));
    EVOC_CUDA(cudaMemcpyAsync(g->weights.get(), weights, nnz * sizeof(float),
                              cudaMemcpyHostToDevice, s));
    k_validate_indices<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(
        g->indices.get(), nnz, n, ctx->status.get());
    EVOC_CHECK_LAUNCH();
  }
  evoc::check_status(ctx, "graph upload");
  *out_graph = g.release();
  EVOC_API_END(ctx)
}

int evoc_graph_info(const evoc_graph_t* g, int64_t* n, int64_t* nnz) {
  if (!g) return EVOC_ERR_INVALID_ARGUMENT;
  if (n) *n = g->n;
  if (nnz) *nnz = g->nnz;
  return EVOC_OK;
}

int evoc_graph_export(const evoc_graph_t* g, int64_t* indptr,
                      uint32_t* indices, float* weights) {
  evoc_ctx* ctx = g ? g->ctx : nullptr;
  EVOC_API_BEGIN
  if (!g || !indptr || (g->nnz > 0 && (!indices || !weights)))
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  use_device(ctx);
  cudaStream_t s = ctx->stream;
  EVOC_CUDA(cudaMemcpyAsync(indptr, g->indptr.get(), (g->n + 1) * sizeof(int64_t),
                            cudaMemcpyDeviceToHost, s));
  if (g->nnz > 0) {
    EVOC_CUDA(cudaMemcpyAsync(indices, g->indices.get(), g->nnz * sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaMemcpyAsync(weights, g->weights.get(), g->nnz * sizeof(float),
                              cudaMemcpyDeviceToHost, s));
  }
  EVOC_CUDA(cudaStreamSynchronize(s));
  EVOC_API_END(ctx)
}

void evoc_graph_free(evoc_graph_t* g) {
  if (!g) return;
  if (g->ctx) cudaSetDevice(g->ctx->device);
  delete g;
}

int evoc_plan_create(evoc_ctx_t* ctx, const evoc_graph_t* g, int32_t dim,
                     const evoc_embed_params_t* params, uint64_t seed,
                     evoc_plan_t** out_plan) {
  EVOC_API_BEGIN
  if (!ctx || !g || !params || !out_plan)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  *out_plan = nullptr;
  use_device(ctx);
  std::vector<evoc::ProblemDesc> probs{{g, seed}};
  *out_plan = evoc::plan_create(ctx, probs, dim, *params);
  EVOC_API_END(ctx)
}

int evoc_plan_create_batched(evoc_ctx_t* ctx, int32_t n_problems,
                             const evoc_graph_t* const* graphs, int32_t dim,
                             const evoc_embed_params_t* params, const uint64_t* seeds,
                             evoc_plan_t** out_plan) {
  EVOC_API_BEGIN
  if (!ctx || n_problems <= 0 || !graphs || !params || !seeds || !out_plan)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "bad argument");
  *out_plan = nullptr;
  use_device(ctx);
  std::vector<evoc::ProblemDesc> probs;
  for (int32_t q = 0; q < n_problems; ++q) {
    if (!graphs[q]) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL graph");
    probs.push_back({graphs[q], seeds[q]});
  }
  *out_plan = evoc::plan_create(ctx, probs, dim, *params);
  EVOC_API_END(ctx)
}

int evoc_plan_create_blocks(evoc_ctx_t* ctx, const evoc_graph_t* g, int32_t n_problems,
                            const int64_t* n_per, int32_t dim,
                            const evoc_embed_params_t* params, const uint64_t* seeds,
                            evoc_plan_t** out_plan) {
  EVOC_API_BEGIN
  if (!ctx || !params || !out_plan) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "bad argument");
  *out_plan = nullptr;
  std::vector<evoc::ProblemDesc> probs = block_problems(g, n_problems, n_per, seeds);
  use_device(ctx);
  if (n_problems == 1) probs[0].begin = probs[0].count = -1;  // the whole graph
  *out_plan = evoc::plan_create(ctx, probs, dim, *params);
  EVOC_API_END(ctx)
}

int evoc_embed_blocks(evoc_ctx_t* ctx, const evoc_graph_t* g, int32_t n_problems,
                      const int64_t* n_per, int32_t dim, const evoc_embed_params_t* params,
                      const float* const* inits, const uint64_t* seeds, float* const* outs) {
  EVOC_API_BEGIN
  if (!ctx || !params || !outs) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "bad argument");
  std::vector<evoc::ProblemDesc> probs = block_problems(g, n_problems, n_per, seeds);
  for (int32_t q = 0; q < n_problems; ++q)
    if (n_per[q] > 0 && !outs[q]) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL output");
  use_device(ctx);
  if (n_problems == 1) probs[0].begin = probs[0].count = -1;
  std::unique_ptr<evoc_plan, void (*)(evoc_plan*)> pl(
      evoc::plan_create(ctx, probs, dim, *params), evoc::plan_free);
  evoc::plan_upload_init_and_run(pl.get(), inits, outs, 0);
  EVOC_API_END(ctx)
}

int evoc_plan_run_device(evoc_plan_t* plan, const float* d_init, float* d_out) {
  evoc_ctx* ctx = plan ? evoc::plan_ctx(plan) : nullptr;
  EVOC_API_BEGIN
  if (!plan || !d_out) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  use_device(ctx);
  evoc::plan_run_device(plan, d_init, d_out);
  EVOC_CUDA(cudaStreamSynchronize(ctx->stream));
  EVOC_API_END(ctx)
}

int evoc_plan_enqueue_device(evoc_plan_t* plan, const float* d_init,
                             float* d_out) {
  evoc_ctx* ctx = plan ? evoc::plan_ctx(plan) : nullptr;
  EVOC_API_BEGIN
  if (!plan || !d_out) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  use_device(ctx);
  evoc::plan_run_device(plan, d_init, d_out);
  EVOC_API_END(ctx)
}

int evoc_plan_profile_epochs(evoc_plan_t* plan, const float* d_init,
                             float* d_out, float* epoch_ms) {
  evoc_ctx* ctx = plan ? evoc::plan_ctx(plan) : nullptr;
  EVOC_API_BEGIN
  if (!plan || !d_out || !epoch_ms)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  use_device(ctx);
  evoc::plan_profile_epochs(plan, d_init, d_out, epoch_ms);
  EVOC_API_END(ctx)
}

int evoc_gather_peak(evoc_ctx_t* ctx, int64_t bytes, double* gbs) {
  EVOC_API_BEGIN
  if (!ctx || !gbs) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  if (bytes < 32 || bytes > ((int64_t)1 << 36))
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "bytes out of range [32, 2^36]");
  use_device(ctx);
  *gbs = evoc::gather_peak(ctx, bytes);
  EVOC_API_END(ctx)
}

int evoc_plan_info(const evoc_plan_t* plan, int64_t* n_edges,
                   int64_t* n_incidence, int32_t* neg_planes,
                   int32_t* warps_per_block, int64_t* n_slots) {
  if (!plan) return EVOC_ERR_INVALID_ARGUMENT;
  evoc::plan_info(plan, n_edges, n_incidence, neg_planes, warps_per_block, n_slots);
  return EVOC_OK;
}

int evoc_plan_set_config(evoc_plan_t* plan, int32_t variant, int32_t warps_per_block,
                         int32_t blocks_per_sm) {
  evoc_ctx* ctx = plan ? evoc::plan_ctx(plan) : nullptr;
  EVOC_API_BEGIN
  if (!plan) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL plan");
  use_device(ctx);
  evoc::plan_configure(plan, variant, warps_per_block, blocks_per_sm);
  EVOC_API_END(ctx)
}

int evoc_plan_autotune(evoc_plan_t* plan, int32_t* config, float* ms_per_launch) {
  evoc_ctx* ctx = plan ? evoc::plan_ctx(plan) : nullptr;
  EVOC_API_BEGIN
  if (!plan) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL plan");
  use_device(ctx);
  evoc::plan_autotune(plan, config, ms_per_launch);
  EVOC_API_END(ctx)
}

int evoc_plan_stats(const evoc_plan_t* plan, evoc_epoch_stats_t* stats) {
  evoc_ctx* ctx = plan ? evoc::plan_ctx(plan) : nullptr;
  EVOC_API_BEGIN
  if (!plan || !stats) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  use_device(ctx);
  evoc::plan_stats(plan, stats);
  EVOC_API_END(ctx)
}

int evoc_plan_debug_run(evoc_plan_t* plan, const float* init,
                        int32_t start_epoch, int32_t end_epoch, float* out,
                        float* grad_out) {
  evoc_ctx* ctx = plan ? evoc::plan_ctx(plan) : nullptr;
  EVOC_API_BEGIN
  if (!plan || !out) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  use_device(ctx);
  evoc::plan_debug_run(plan, init, start_epoch, end_epoch, out, grad_out);
  EVOC_API_END(ctx)
}

void evoc_plan_free(evoc_plan_t* plan) {
  if (!plan) return;
  evoc_ctx* ctx = evoc::plan_ctx(plan);
  if (ctx) cudaSetDevice(ctx->device);
  evoc::plan_free(plan);
}

int evoc_embed(evoc_ctx_t* ctx, const evoc_graph_t* g, int32_t dim,
               const evoc_embed_params_t* params, const float* init,
               uint64_t seed, int32_t verbose, float* out) {
  EVOC_API_BEGIN
  if (!ctx || !g || !params)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  if (g->n > 0 && !out) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "out is NULL");
  if (g->n == 0) return EVOC_OK;  // embedding.rs:61-64
  use_device(ctx);
  std::vector<evoc::ProblemDesc> probs{{g, seed}};
  std::unique_ptr<evoc_plan, void (*)(evoc_plan*)> pl(
      evoc::plan_create(ctx, probs, dim, *params), evoc::plan_free);
  const float* inits[1] = {init};
  float* outs[1] = {out};
  evoc::plan_upload_init_and_run(pl.get(), inits, outs, verbose);
  EVOC_API_END(ctx)
}

int evoc_embed_batched(evoc_ctx_t* ctx, int32_t n_problems,
                       const evoc_graph_t* const* graphs, int32_t dim,
                       const evoc_embed_params_t* params,
                       const float* const* inits, const uint64_t* seeds,
                       float* const* outs) {
  EVOC_API_BEGIN
  if (!ctx || n_problems < 0 || (n_problems > 0 && (!graphs || !seeds || !outs)) ||
      !params)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "bad argument");
  if (n_problems == 0) return EVOC_OK;
  use_device(ctx);
  std::vector<evoc::ProblemDesc> probs;
  for (int32_t q = 0; q < n_problems; ++q) {
    if (!graphs[q]) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL graph");
    if (graphs[q]->n > 0 && !outs[q])
      throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL output");
    probs.push_back({graphs[q], seeds[q]});
  }
  std::unique_ptr<evoc_plan, void (*)(evoc_plan*)> pl(
      evoc::plan_create(ctx, probs, dim, *params), evoc::plan_free);
  evoc::plan_upload_init_and_run(pl.get(), inits, outs, 0);
  EVOC_API_END(ctx)
}

// ---- label propagation partition -------------------------------------------

int evoc_label_prop_partition(evoc_ctx_t* ctx, const evoc_graph_t* g, int64_t approx_n_parts,
                              int32_t n_iter, uint64_t seed, uint32_t* partition,
                              int64_t* n_parts) {
  EVOC_API_BEGIN
  if (!ctx || !g || !n_parts || (g->n > 0 && !partition))
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  use_device(ctx);
  evoc::DevBuf<uint32_t> d((size_t)g->n, ctx->stream);
  *n_parts = evoc::label_prop_partition(ctx, g, approx_n_parts, n_iter, seed, d.get());
  if (g->n > 0)
    EVOC_CUDA(cudaMemcpyAsync(partition, d.get(), d.bytes(), cudaMemcpyDeviceToHost, ctx->stream));
  EVOC_CUDA(cudaStreamSynchronize(ctx->stream));
  EVOC_API_END(ctx)
}

int evoc_label_propagation_init(evoc_ctx_t* ctx, const evoc_graph_t* g, int32_t dim,
                                const float* data, int64_t d, uint64_t seed, float* out) {
  EVOC_API_BEGIN
  if (!ctx || !g || !out) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  use_device(ctx);
  cudaStream_t s = ctx->stream;
  const int64_t n = g->n;
  evoc::DevBuf<float> dd, dout(n * (int64_t)std::max(dim, 1), s);
  if (data) {
    if (d <= 0) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "data dimension must be > 0");
    dd.alloc(n * d, s);
    EVOC_CUDA(cudaMemcpyAsync(dd.get(), data, dd.bytes(), cudaMemcpyHostToDevice, s));
  }
  evoc::label_propagation_init_device(ctx, g, dim, data ? dd.get() : nullptr, d, seed,
                                      dout.get());
  EVOC_CUDA(cudaMemcpyAsync(out, dout.get(), n * (int64_t)dim * sizeof(float),
                            cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaStreamSynchronize(s));
  evoc::check_status(ctx, "label_propagation_init");
  EVOC_API_END(ctx)
}

int evoc_label_propagation_init_device(evoc_ctx_t* ctx, const evoc_graph_t* g, int32_t dim,
                                       const float* d_data, int64_t d, uint64_t seed,
                                       float* d_out) {
  EVOC_API_BEGIN
  if (!ctx || !g || !d_out) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  use_device(ctx);
  evoc::label_propagation_init_device(ctx, g, dim, d_data, d, seed, d_out);
  EVOC_CUDA(cudaStreamSynchronize(ctx->stream));
  evoc::check_status(ctx, "label_propagation_init");
  EVOC_API_END(ctx)
}

// ---- clustering: minimum spanning tree -------------------------------------

int evoc_build_mst(evoc_ctx_t* ctx, const float* data, int64_t n, int32_t dim,
                   int32_t min_samples, int64_t* u, int64_t* v, float* w, int64_t* n_edges) {
  EVOC_API_BEGIN
  if (!ctx || !n_edges || (n > 1 && (!data || !u || !v || !w)))
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  use_device(ctx);
  cudaStream_t s = ctx->stream;
  *n_edges = 0;
  if (dim < 1 || dim > 16) throw evoc::Error(EVOC_ERR_UNSUPPORTED, "dim must be in 1..16");
  if (n < 0) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "n must be >= 0");
  const int64_t m = std::max<int64_t>(n - 1, 0);
  evoc::DevBuf<float> dd(n * (int64_t)dim, s), dw(m, s);
  evoc::DevBuf<int64_t> du(m, s), dv(m, s);
  if (n > 1)
    EVOC_CUDA(cudaMemcpyAsync(dd.get(), data, dd.bytes(), cudaMemcpyHostToDevice, s));
  const int64_t k = evoc::build_mst_device(ctx, dd.get(), n, dim, min_samples, du.get(), dv.get(),
                                           dw.get());
  EVOC_CUDA(cudaStreamSynchronize(s));
  evoc::check_status(ctx, "build_mst");
  if (k > 0) {
    EVOC_CUDA(cudaMemcpyAsync(u, du.get(), k * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaMemcpyAsync(v, dv.get(), k * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaMemcpyAsync(w, dw.get(), k * sizeof(float), cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaStreamSynchronize(s));
  }
  *n_edges = k;
  EVOC_API_END(ctx)
}

int evoc_build_mst_device(evoc_ctx_t* ctx, const float* d_data, int64_t n, int32_t dim,
                          int32_t min_samples, int64_t* d_u, int64_t* d_v, float* d_w,
                          int64_t* n_edges) {
  EVOC_API_BEGIN
  if (!ctx || !n_edges) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  use_device(ctx);
  *n_edges = 0;
  const int64_t k = evoc::build_mst_device(ctx, d_data, n, dim, min_samples, d_u, d_v, d_w);
  EVOC_CUDA(cudaStreamSynchronize(ctx->stream));
  evoc::check_status(ctx, "build_mst");
  *n_edges = k;
  EVOC_API_END(ctx)
}

// ---- learned warm start ----------------------------------------------------

void evoc_mlp_train_params_default(evoc_mlp_train_params_t* p) {
  if (!p) return;
  p->steps = 3000;
  p->batch = 8192;
  p->align_every = 250;
  p->align_rows = 65536;
  p->lr = 1e-3f;
  p->beta1 = 0.9f;
  p->beta2 = 0.999f;
  p->eps = 1e-8f;
  p->lr_end = 1e-4f;
  p->seed = 0;
}

int evoc_mlp_create(evoc_ctx_t* ctx, int32_t in_dim, int32_t hidden, int32_t out_dim,
                    uint64_t seed, evoc_mlp_t** out) {
  EVOC_API_BEGIN
  if (!ctx || !out) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = nullptr;
  use_device(ctx);
  *out = evoc::mlp_create(ctx, in_dim, hidden, out_dim, seed);
  EVOC_API_END(ctx)
}

void evoc_mlp_free(evoc_mlp_t* mlp) {
  if (!mlp) return;
  evoc_ctx* ctx = evoc::mlp_ctx(mlp);
  if (ctx) cudaSetDevice(ctx->device);
  evoc::mlp_free(mlp);
}

int64_t evoc_mlp_n_params(const evoc_mlp_t* mlp) { return mlp ? evoc::mlp_n_params(mlp) : 0; }

int evoc_mlp_get_params(const evoc_mlp_t* mlp, float* params) {
  evoc_ctx* ctx = mlp ? evoc::mlp_ctx(mlp) : nullptr;
  EVOC_API_BEGIN
  if (!mlp || !params) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  use_device(ctx);
  evoc::mlp_get_params(mlp, params);
  EVOC_API_END(ctx)
}

int evoc_mlp_set_params(evoc_mlp_t* mlp, const float* params) {
  evoc_ctx* ctx = mlp ? evoc::mlp_ctx(mlp) : nullptr;
  EVOC_API_BEGIN
  if (!mlp || !params) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL argument");
  use_device(ctx);
  evoc::mlp_set_params(mlp, params);
  EVOC_API_END(ctx)
}

int evoc_mlp_predict(evoc_mlp_t* mlp, const float* x, int64_t n, float* out) {
  evoc_ctx* ctx = mlp ? evoc::mlp_ctx(mlp) : nullptr;
  EVOC_API_BEGIN
  if (!mlp || n < 0 || (n > 0 && (!x || !out)))
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "bad argument");
  use_device(ctx);
  evoc::mlp_predict_host(mlp, x, n, out);
  EVOC_API_END(ctx)
}

int evoc_mlp_predict_device(evoc_mlp_t* mlp, const uint16_t* d_x_bf16, int64_t n,
                            float* d_out) {
  evoc_ctx* ctx = mlp ? evoc::mlp_ctx(mlp) : nullptr;
  EVOC_API_BEGIN
  if (!mlp || n < 0 || (n > 0 && (!d_x_bf16 || !d_out)))
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "bad argument");
  if (((uintptr_t)d_x_bf16 & 15) != 0)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "points must be 16-byte aligned");
  use_device(ctx);
  evoc::mlp_predict_device(mlp, d_x_bf16, n, d_out);
  EVOC_CUDA(cudaStreamSynchronize(ctx->stream));
  EVOC_API_END(ctx)
}

int evoc_mlp_gradients(evoc_mlp_t* mlp, const float* x, const float* target, int64_t n,
                       float* loss, float* grad) {
  evoc_ctx* ctx = mlp ? evoc::mlp_ctx(mlp) : nullptr;
  EVOC_API_BEGIN
  if (!mlp || !x || !target || !loss || !grad || n <= 0)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "bad argument");
  use_device(ctx);
  evoc::mlp_gradients_host(mlp, x, target, n, loss, grad);
  EVOC_API_END(ctx)
}

int evoc_mlp_fit_device(evoc_mlp_t* mlp, int32_t n_instances, const uint16_t* const* d_x_bf16,
                        const float* const* d_layouts, const int64_t* n_rows,
                        const evoc_mlp_train_params_t* params, float* loss_history) {
  evoc_ctx* ctx = mlp ? evoc::mlp_ctx(mlp) : nullptr;
  EVOC_API_BEGIN
  if (!mlp || n_instances <= 0 || !d_x_bf16 || !d_layouts || !n_rows || !params)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "bad argument");
  for (int32_t i = 0; i < n_instances; ++i)
    if (((uintptr_t)d_x_bf16[i] & 15) != 0 || ((uintptr_t)d_layouts[i] & 3) != 0)
      throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "misaligned instance buffer");
  use_device(ctx);
  evoc::mlp_fit_device(mlp, n_instances, d_x_bf16, d_layouts, n_rows, params, loss_history);
  EVOC_API_END(ctx)
}

int evoc_to_bf16_device(evoc_ctx_t* ctx, const float* d_in, int64_t count, uint16_t* d_out) {
  EVOC_API_BEGIN
  if (!ctx || count < 0 || (count > 0 && (!d_in || !d_out)))
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "bad argument");
  use_device(ctx);
  evoc::to_bf16_device(ctx, d_in, count, d_out);
  EVOC_CUDA(cudaStreamSynchronize(ctx->stream));
  EVOC_API_END(ctx)
}

int evoc_selftest_wait_timeout(evoc_ctx_t* ctx, int32_t limit_ms) {
  EVOC_API_BEGIN
  if (!ctx || limit_ms < 1 || limit_ms > 2000)
    throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "limit_ms outside [1, 2000]");
  use_device(ctx);
  evoc::wait_timeout_selftest(ctx, limit_ms);
  EVOC_API_END(ctx)
}

int evoc_procrustes(const double* m, int32_t d, double* r) {
  evoc_ctx* ctx = nullptr;
  EVOC_API_BEGIN
  if (!m || !r || d < 1 || d > 16) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "bad argument");
  evoc::procrustes(m, d, r);
  EVOC_API_END(ctx)
}

}  // extern "C"
