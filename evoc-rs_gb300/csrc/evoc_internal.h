// evoc_internal.h — shared declarations of the GB300 EVoC library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/evoc_gb300.h"

namespace evoc {

// ---------------------------------------------------------------------------
// Errors: internal code throws Error; the C ABI catches it and returns code.
// ---------------------------------------------------------------------------
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void throw_cuda(cudaError_t e, const char* what, const char* file,
                             int line);

#define EVOC_CUDA(call)                                           \
  do {                                                            \
    cudaError_t _e = (call);                                      \
    if (_e != cudaSuccess) ::evoc::throw_cuda(_e, #call, __FILE__, __LINE__); \
  } while (0)

#define EVOC_CHECK_LAUNCH() EVOC_CUDA(cudaGetLastError())

// Device-side status flags (one int32 word per condition). Kernels set a
// flag with atomicOr and never trap; the host reads the words after a call.
enum StatusBit : int32_t {
  ST_BAD_INDEX = 1,      // kNN / graph index >= n
  ST_BAD_VALUE = 2,      // NaN distance / weight where not allowed
  ST_EMPTY_ROW = 4,      // empty kNN row with local_connectivity > 0
  ST_TOO_MANY_NEG = 8,   // negative count per edge-epoch above the limit
  ST_INTERNAL = 16,      // self-check failed
  ST_CROSS_BLOCK = 32,   // an edge joins two problems of a block-diagonal graph
  ST_WAIT_TIMEOUT = 64,  // a bounded wait on an mbarrier gave up
};

// ---------------------------------------------------------------------------
// Stream-ordered device buffer.
// ---------------------------------------------------------------------------
template <typename T>
struct DevBuf {
  T* ptr = nullptr;
  size_t count = 0;
  cudaStream_t stream = nullptr;
  DevBuf() = default;
  DevBuf(size_t n, cudaStream_t s) { alloc(n, s); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept { *this = std::move(o); }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      ptr = o.ptr; count = o.count; stream = o.stream;
      o.ptr = nullptr; o.count = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t n, cudaStream_t s) {
    release();
    stream = s;
    count = n;
    if (n == 0) return;
    cudaError_t e = cudaMallocAsync((void**)&ptr, n * sizeof(T), s);
    if (e != cudaSuccess) {
      ptr = nullptr;
      count = 0;
      (void)cudaGetLastError();
      throw Error(EVOC_ERR_OUT_OF_MEMORY,
                  "device allocation of " + std::to_string(n * sizeof(T)) +
                      " bytes failed: " + cudaGetErrorString(e));
    }
  }
  void release() {
    if (ptr) cudaFreeAsync(ptr, stream);
    ptr = nullptr;
    count = 0;
  }
  size_t bytes() const { return count * sizeof(T); }
  T* get() const { return ptr; }
};

// Optional stage timing (EVOC_TRACE=1 prints to stderr):
// CUDA events between stages (device time) and the host clock.
struct StageTrace {
  bool on = false;
  cudaStream_t s = nullptr;
  std::vector<std::pair<std::string, cudaEvent_t>> ev;
  std::vector<double> host;
  explicit StageTrace(cudaStream_t st) : s(st) {
    const char* e = std::getenv("EVOC_TRACE");
    on = e && e[0] == '1';
    mark("start");
  }
  static double now_ms() {
    return std::chrono::duration<double, std::milli>(
               std::chrono::steady_clock::now().time_since_epoch()).count();
  }
  void mark(const char* name) {
    if (!on) return;
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) { on = false; return; }
    cudaEventRecord(e, s);
    ev.emplace_back(name, e);
    host.push_back(now_ms());
  }
  ~StageTrace() {
    if (!on) return;
    cudaEventSynchronize(ev.back().second);
    for (size_t i = 1; i < ev.size(); ++i) {
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, ev[i - 1].second, ev[i].second);
      std::fprintf(stderr, "[evoc trace] %-22s device %8.3f ms  host %8.3f ms\n",
                   ev[i].first.c_str(), ms, host[i] - host[i - 1]);
    }
    for (auto& x : ev) cudaEventDestroy(x.second);
  }
};

}  // namespace evoc

// ---------------------------------------------------------------------------
// Opaque handles of the C ABI.
// ---------------------------------------------------------------------------
struct evoc_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  evoc::DevBuf<int32_t> status;  // device status word
  // The largest gradient-slot buffer of a freed plan, handed to the next plan
  // that fits in it (stream order makes the reuse safe): repeated one-shot
  // embeddings skip a multi-gigabyte allocation each.
  evoc::DevBuf<uint32_t> slot_cache;
  // Row-sum evaluations (bisection steps over all rows) of the most recent
  // smooth_knn pass on this context: the work figure of its ALU bound.
  evoc::DevBuf<unsigned long long> sk_steps;
};

struct evoc_graph {
  evoc_ctx* ctx = nullptr;
  int64_t n = 0;
  int64_t nnz = 0;
  // true when rows are sorted by column, free of duplicates and self loops,
  // and symmetric with identical weights in both directions (the output of
  // the fuzzy union). The embedding set-up then skips its transpose.
  bool canonical = false;
  evoc::DevBuf<int64_t> indptr;
  evoc::DevBuf<uint32_t> indices;
  evoc::DevBuf<float> weights;
};

namespace evoc {

// ---- primitives.cu ---------------------------------------------------------
// out[0..n] = exclusive prefix sum of in[0..n-1]; out[n] = total.
void exclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, int64_t n,
                               cudaStream_t s);
void exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n,
                        cudaStream_t s);
// Stable LSD radix sort of (key, value) pairs by key, keys < 2^key_bits.
// Results are written back to keys/vals.
void radix_sort_pairs(uint32_t* keys, uint2* vals, int64_t n, int key_bits,
                      cudaStream_t s);
int bits_for(uint64_t max_value);
// Read the context's status word and reset it; throw on any set bit.
void check_status(evoc_ctx* ctx, const char* where);
// Message returned by evoc_last_error(NULL) on this thread.
void set_thread_error(const std::string& message);

// ---- fuzzy_set.cu ----------------------------------------------------------
void smooth_knn_device(evoc_ctx* ctx, const float* d_dist,
                       const int32_t* d_row_len, int64_t n, int32_t k,
                       uint64_t k_target, float local_connectivity,
                       int32_t n_iter, float* d_sigma, float* d_rho,
                       float* d_weights_out, const uint32_t* d_idx_for_len);
void fuzzy_set_device(evoc_ctx* ctx, const uint32_t* d_idx,
                      const float* d_dist, int64_t n, int32_t k,
                      float effective_n_neighbours, bool symmetrise,
                      float* d_sigmas_out, float* d_rhos_out, evoc_graph* out);

// ---- embed.cu --------------------------------------------------------------
// One problem of a plan: a whole graph, or (begin >= 0) the rows [begin,
// begin + count) of a block-diagonal graph shared by all the plan's problems.
struct ProblemDesc {
  const evoc_graph* graph;
  uint64_t seed;
  int64_t begin = -1;
  int64_t count = -1;
};

// ---- label_prop.cu ---------------------------------------------------------
// Partition of g by label propagation (label_prop.rs:202-230) into
// d_partition[n]; returns the number of parts.
int64_t label_prop_partition(evoc_ctx* ctx, const evoc_graph* g, int64_t approx_n_parts,
                             int32_t n_iter, uint64_t seed, uint32_t* d_partition);

// ---- lp_init.cu ------------------------------------------------------------
// label_propagation_init (label_prop.rs:537-564) of g: the n x dim initial
// embedding into d_out (device); d_data (device n x d) feeds the PCA base
// case, or is null (random base case).
void label_propagation_init_device(evoc_ctx* ctx, const evoc_graph* g, int32_t dim,
                                   const float* d_data, int64_t d, uint64_t seed, float* d_out);

// ---- mst.cu ----------------------------------------------------------------
// build_mst (mst.rs:82-166) of the n x dim device points d_data: writes the
// minimum spanning tree's edges (u, v, weight) in the reference's insertion
// order into d_u, d_v, d_w (n - 1 entries each); returns the edge count.
int64_t build_mst_device(evoc_ctx* ctx, const float* d_data, int64_t n, int32_t dim,
                         int32_t min_samples, int64_t* d_u, int64_t* d_v, float* d_w);

// ---- mlp.cu ----------------------------------------------------------------
}  // namespace evoc

struct evoc_mlp;  // defined in mlp.cu

namespace evoc {
evoc_mlp* mlp_create(evoc_ctx* ctx, int in, int hid, int out, uint64_t seed);
void mlp_free(evoc_mlp* net);
evoc_ctx* mlp_ctx(const evoc_mlp* net);
int64_t mlp_n_params(const evoc_mlp* net);
void mlp_dims(const evoc_mlp* net, int32_t* in, int32_t* hid, int32_t* out);
void mlp_get_params(const evoc_mlp* net, float* host);
void mlp_set_params(evoc_mlp* net, const float* host);
void mlp_predict_device(evoc_mlp* net, const uint16_t* x, int64_t n, float* y);
void mlp_predict_host(evoc_mlp* net, const float* x, int64_t n, float* y);
void mlp_gradients_host(evoc_mlp* net, const float* x, const float* target, int64_t n,
                        float* loss, float* grad);
void mlp_fit_device(evoc_mlp* net, int32_t m, const uint16_t* const* xs,
                    const float* const* layouts, const int64_t* ns,
                    const evoc_mlp_train_params_t* p, float* loss_history);
void to_bf16_device(evoc_ctx* ctx, const float* x, int64_t count, uint16_t* y);
void procrustes(const double* m, int d, double* r);
// Runs a kernel whose bounded wait cannot be satisfied; throws the
// ST_WAIT_TIMEOUT error after limit_ms.
void wait_timeout_selftest(evoc_ctx* ctx, int32_t limit_ms);
}  // namespace evoc

struct evoc_plan;  // defined in embed.cu

namespace evoc {
evoc_plan* plan_create(evoc_ctx* ctx, const std::vector<ProblemDesc>& probs,
                       int32_t dim, const evoc_embed_params_t& params);
void plan_run_device(evoc_plan* plan, const float* d_init, float* d_out);
void plan_profile_epochs(evoc_plan* plan, const float* d_init, float* d_out,
                         float* epoch_ms);
void plan_debug_run(evoc_plan* plan, const float* h_init, int32_t start_epoch,
                    int32_t end_epoch, float* h_out, float* h_grad);
void plan_stats(const evoc_plan* plan, evoc_epoch_stats_t* stats);
void plan_free(evoc_plan* plan);
void plan_configure(evoc_plan* plan, int variant, int warps_per_block, int blocks_per_sm);
void plan_autotune(evoc_plan* plan, int32_t* config, float* ms_per_launch);
evoc_ctx* plan_ctx(const evoc_plan* plan);
// Random 32-byte row gathers over an L2-resident buffer of `bytes`: GB/s
// (measurement hook for the roofline's L2 bound).
double gather_peak(evoc_ctx* ctx, int64_t bytes);
void plan_info(const evoc_plan* plan, int64_t* n_edges, int64_t* n_inc,
               int32_t* planes, int32_t* wpb, int64_t* n_slots);
int64_t plan_n(const evoc_plan* plan);
int32_t plan_n_epochs(const evoc_plan* plan);
bool plan_has_edges(const evoc_plan* plan);
void plan_upload_init_and_run(evoc_plan* plan, const float* const* h_inits,
                              float* const* h_outs, int verbose);
}  // namespace evoc
