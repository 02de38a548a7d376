// noalloc.cu — kNN graph -> weighted directed CSR without any allocation.
//
// For callers that must not allocate device memory while they run: services
// that reserve their whole device-memory budget up front and forbid later
// cudaMalloc calls, and host frameworks that own the device heap through
// their own pool and do not let an operator allocate behind their back.
// Those callers cannot use evoc_fuzzy_set_device, whose scratch buffers come
// from cudaMallocAsync.
//
// This entry point computes what evoc_fuzzy_set_device computes with
// symmetrise = 0 (smooth_knn_dist + knn_to_coo + coo_to_adjacency_list,
// src/graph/fuzzy_graph.rs:33-159, :242-256), bit for bit, into caller-owned
// output buffers. Its per-row scratch lives in one file-scope device array of
// fixed size (EVOC_NOALLOC_SCRATCH_BYTES). CUDA loads device code lazily by
// default, so the array (with this file's kernels) is placed on a GPU by the
// first call there, and stays until the process exits; callers that reserve
// their memory budget make a small first call at start-up, or run with
// CUDA_MODULE_LOADING=EAGER.
//
// Set-up: on its first call on a device (with that device current) the entry
// point looks up the array's device address with cudaGetSymbolAddress and
// keeps it for the life of the process; the host-side symbol itself is only a
// stand-in and is never passed to a kernel. Make that first call before any
// stream capture, and do not reset the device while the library is in use
// (the kept address would go stale).
//
// Sharing: every call on a device uses the same array and leaves the last
// call's contents in it. The status word is cleared at the start of each
// call; everything else is written before it is read. Calls whose GPU work
// overlaps (for example on two streams) race on the array.
#include "evoc_device.cuh"
#include "evoc_internal.h"

#include <cmath>
#include <mutex>

namespace {

constexpr size_t kScratchBytes = (size_t)EVOC_NOALLOC_SCRATCH_BYTES;
constexpr size_t kHeaderBytes = 256;  // status word, padded
constexpr size_t kBytesPerRow = 16;   // row_len, count, sigma, rho

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 256;
std::mutex g_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

void* scratch_for_current_device() {
  int dev = 0;
  EVOC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices)
    throw evoc::Error(EVOC_ERR_UNSUPPORTED, "device index too large");
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      (void)cudaGetLastError();
      throw evoc::Error(EVOC_ERR_CUDA,
                        std::string("cudaGetSymbolAddress of the scratch array failed: ") +
                            cudaGetErrorString(e));
    }
    g_scratch_ptr[dev] = p;
  }
  return g_scratch_ptr[dev];
}

struct Scratch {
  int32_t* status;
  int32_t* row_len;
  int32_t* count;
  float* sigma;
  float* rho;
};

Scratch carve(void* base, int64_t n) {
  unsigned char* b = static_cast<unsigned char*>(base);
  Scratch s;
  s.status = reinterpret_cast<int32_t*>(b);
  s.row_len = reinterpret_cast<int32_t*>(b + kHeaderBytes);
  s.count = s.row_len + n;
  s.sigma = reinterpret_cast<float*>(s.count + n);
  s.rho = s.sigma + n;
  return s;
}

// Row lengths (first EVOC_KNN_PAD), index validation, non-self entry counts.
__global__ void k_na_rows(const uint32_t* __restrict__ idx, int64_t n, int32_t k,
                          Scratch sc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t* r = idx + i * (int64_t)k;
  int32_t len = k, cnt = 0;
  for (int32_t j = 0; j < k; ++j) {
    const uint32_t c = r[j];
    if (c == EVOC_KNN_PAD) {
      len = j;
      break;
    }
    if ((int64_t)c >= n) evoc::set_status(sc.status, evoc::ST_BAD_INDEX);
    if ((int64_t)c != i) ++cnt;
  }
  sc.row_len[i] = len;
  sc.count[i] = cnt;
}

// rho and the sigma bisection of fuzzy_graph.rs:49-95 (local_connectivity 1,
// 64 iterations), serial over the row in row order.
__global__ void k_na_sigma(const float* __restrict__ dist, int64_t n, int32_t k,
                           double target, Scratch sc) {
  using namespace evoc;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* d = dist + i * (int64_t)k;
  const int32_t len = sc.row_len[i];
  for (int32_t j = 0; j < len; ++j)
    if (d[j] != d[j]) set_status(sc.status, ST_BAD_VALUE);
  if (len <= 0) {
    set_status(sc.status, ST_EMPTY_ROW);
    sc.sigma[i] = 0.0f;
    sc.rho[i] = 0.0f;
    return;
  }
  const float rho = d[0];  // local_connectivity = 1: index 0, no interpolation
  float lo = 0.0f, hi = 3.40282347e+38f, mid = 1.0f;
  for (int it = 0; it < 64; ++it) {
    float val = 0.0f;
    for (int32_t j = 0; j < len; ++j)
      val = fadd(val, evoc_expf(-fdiv(max0(fsub(d[j], rho)), mid)));
    const double vd = (double)val;
    if (fabs(vd - target) < 1e-5) break;
    if (vd > target) {
      hi = mid;
      mid = fdiv(fadd(lo, hi), 2.0f);
    } else {
      lo = mid;
      mid = (hi == 3.40282347e+38f) ? fmul(mid, 2.0f) : fdiv(fadd(lo, hi), 2.0f);
    }
  }
  sc.sigma[i] = mid;
  sc.rho[i] = rho;
}

// Exclusive scan of the counts into indptr (one block; n is bounded by the
// scratch size).
__global__ void k_na_scan(Scratch sc, int64_t n, int64_t* __restrict__ indptr) {
  __shared__ int64_t part[1024];
  const int64_t per = (n + blockDim.x - 1) / blockDim.x;
  const int64_t a = threadIdx.x * per, b = min(n, a + per);
  int64_t s = 0;
  for (int64_t i = a; i < b; ++i) s += sc.count[i];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t run = 0;
    for (unsigned t = 0; t < blockDim.x; ++t) {
      const int64_t c = part[t];
      part[t] = run;
      run += c;
    }
    indptr[n] = run;
  }
  __syncthreads();
  int64_t run = part[threadIdx.x];
  for (int64_t i = a; i < b; ++i) {
    indptr[i] = run;
    run += sc.count[i];
  }
}

// knn_to_coo weights (fuzzy_graph.rs:134-150) in kNN order, self loops skipped.
__global__ void k_na_write(const uint32_t* __restrict__ idx,
                           const float* __restrict__ dist, int64_t n, int32_t k,
                           Scratch sc, const int64_t* __restrict__ indptr,
                           uint32_t* __restrict__ out_idx, float* __restrict__ out_w) {
  using namespace evoc;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t len = sc.row_len[i];
  const float sigma = sc.sigma[i], rho = sc.rho[i];
  int64_t o = indptr[i];
  for (int32_t j = 0; j < len; ++j) {
    const uint32_t c = idx[i * (int64_t)k + j];
    if ((int64_t)c == i) continue;
    const float adjusted = max0(fsub(dist[i * (int64_t)k + j], rho));
    float w;
    if (sigma > 0.0f)
      w = evoc_expf(-fdiv(adjusted, sigma));
    else
      w = (adjusted > 0.0f) ? 0.0f : 1.0f;
    out_idx[o] = c;
    out_w[o] = w;
    ++o;
  }
}

}  // namespace

extern "C" int evoc_knn_to_csr_noalloc(const uint32_t* d_knn_idx, const float* d_knn_dist,
                                       int64_t n, int32_t k, float effective_n_neighbours,
                                       int64_t* d_indptr, uint32_t* d_indices,
                                       float* d_weights, int64_t capacity,
                                       int64_t* nnz_out, void* stream) {
  try {
    if (!d_knn_idx || !d_knn_dist || !d_indptr || !nnz_out || capacity < 0 ||
        (capacity > 0 && (!d_indices || !d_weights)))
      throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "NULL pointer or negative capacity");
    if (n <= 0)
      throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT,
                        "empty kNN graph (build_fuzzy_simplicial_set reads row 0)");
    if (k <= 0) throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT, "k must be positive");
    if ((size_t)n > (kScratchBytes - kHeaderBytes) / kBytesPerRow)
      throw evoc::Error(EVOC_ERR_UNSUPPORTED,
                        "n = " + std::to_string(n) + " rows exceeds the no-allocation limit of " +
                            std::to_string((kScratchBytes - kHeaderBytes) / kBytesPerRow) +
                            " rows (" + std::to_string(kScratchBytes >> 20) + " MiB scratch)");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const Scratch sc = carve(scratch_for_current_device(), n);
    EVOC_CUDA(cudaMemsetAsync(sc.status, 0, sizeof(int32_t), s));
    const unsigned blocks = (unsigned)((n + 255) / 256);
    k_na_rows<<<blocks, 256, 0, s>>>(d_knn_idx, n, k, sc);
    EVOC_CHECK_LAUNCH();
    // k = effective_n_neighbors.to_usize().unwrap_or(row 0's length)
    uint64_t kk;
    const float e = effective_n_neighbours;
    if (e > -1.0f && e < 18446744073709551616.0f) {
      kk = (uint64_t)e;
    } else {
      int32_t len0 = 0;
      EVOC_CUDA(cudaMemcpyAsync(&len0, sc.row_len, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
      EVOC_CUDA(cudaStreamSynchronize(s));
      kk = (uint64_t)len0;
    }
    k_na_sigma<<<blocks, 256, 0, s>>>(d_knn_dist, n, k, std::log2((double)kk), sc);
    EVOC_CHECK_LAUNCH();
    k_na_scan<<<1, 1024, 0, s>>>(sc, n, d_indptr);
    EVOC_CHECK_LAUNCH();
    int32_t st = 0;
    int64_t total = 0;
    EVOC_CUDA(cudaMemcpyAsync(&st, sc.status, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaMemcpyAsync(&total, d_indptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaStreamSynchronize(s));
    if (st & evoc::ST_BAD_INDEX)
      throw evoc::Error(EVOC_ERR_INVALID_INPUT, "knn_to_csr_noalloc: an index is >= n");
    if (st & evoc::ST_BAD_VALUE)
      throw evoc::Error(EVOC_ERR_INVALID_INPUT, "knn_to_csr_noalloc: a distance is NaN");
    if (st & evoc::ST_EMPTY_ROW)
      throw evoc::Error(EVOC_ERR_INVALID_INPUT,
                        "knn_to_csr_noalloc: empty kNN row with local_connectivity > 0");
    if (total > capacity)
      throw evoc::Error(EVOC_ERR_INVALID_ARGUMENT,
                        "output capacity " + std::to_string(capacity) + " < " +
                            std::to_string(total) + " entries");
    k_na_write<<<blocks, 256, 0, s>>>(d_knn_idx, d_knn_dist, n, k, sc, d_indptr, d_indices,
                                       d_weights);
    EVOC_CHECK_LAUNCH();
    EVOC_CUDA(cudaStreamSynchronize(s));
    *nnz_out = total;
    return EVOC_OK;
  } catch (const evoc::Error& e) {
    evoc::set_thread_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    evoc::set_thread_error(e.what());
    return EVOC_ERR_INTERNAL;
  }
}
