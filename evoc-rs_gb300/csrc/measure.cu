// Measurement hook: the random-gather bandwidth of L2 for rows of 32 bytes,
// the access pattern of the epoch kernel's source-row gathers (one dim-8 f32
// row = one 32-byte sector). The roofline of the epoch kernel takes the
// larger of its HBM time and its L2-gather time; this kernel supplies the
// measured L2 denominator.
#include "evoc_internal.h"

namespace evoc {
namespace {

// Each thread gathers `per_thread` rows picked by an integer hash of (thread,
// i) and folds them into one value, so no load can be elided. Rows are
// `row_words` floats (8 = 32 bytes).
__global__ void k_gather_probe(const float4* __restrict__ rows, uint32_t n_rows,
                               int per_thread, float* __restrict__ sink) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  float acc = 0.0f;
  uint32_t h = tid * 0x9E3779B9u + 0x7F4A7C15u;
  for (int i = 0; i < per_thread; ++i) {
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    const uint32_t r = (uint32_t)(((uint64_t)h * n_rows) >> 32);
    const float4 a = __ldg(rows + 2 * (size_t)r), b = __ldg(rows + 2 * (size_t)r + 1);
    acc += a.x + a.y + a.z + a.w + b.x + b.y + b.z + b.w;
  }
  sink[tid] = acc;
}

}  // namespace

double gather_peak(evoc_ctx* ctx, int64_t bytes) {
  cudaStream_t s = ctx->stream;
  const uint32_t n_rows = (uint32_t)std::max<int64_t>(1, bytes / 32);
  DevBuf<float> buf((size_t)n_rows * 8, s), sink;
  EVOC_CUDA(cudaMemsetAsync(buf.get(), 0, buf.bytes(), s));
  const int threads = 256, per_thread = 256;
  const int blocks = ctx->num_sms * 8;
  sink.alloc((size_t)blocks * threads, s);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  EVOC_CUDA(cudaEventCreate(&e0));
  EVOC_CUDA(cudaEventCreate(&e1));
  float best_ms = 0.0f;
  try {
    for (int rep = 0; rep < 8; ++rep) {  // the first three warm L2
      EVOC_CUDA(cudaEventRecord(e0, s));
      k_gather_probe<<<blocks, threads, 0, s>>>(reinterpret_cast<const float4*>(buf.get()),
                                                n_rows, per_thread, sink.get());
      EVOC_CHECK_LAUNCH();
      EVOC_CUDA(cudaEventRecord(e1, s));
      EVOC_CUDA(cudaEventSynchronize(e1));
      float ms = 0.0f;
      EVOC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (rep >= 3 && (best_ms == 0.0f || ms < best_ms)) best_ms = ms;
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double gathered = (double)blocks * threads * per_thread * 32.0;
  return gathered / ((double)best_ms * 1e-3) / 1e9;
}

}  // namespace evoc
