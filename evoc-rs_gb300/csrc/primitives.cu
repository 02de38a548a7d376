// primitives.cu — device-wide exclusive scan and stable LSD radix sort.
//
// Both are deterministic (no floating point, fixed traversal order) and are
// used to build CSR offsets and the stable column-major transposes of the
// fuzzy union and of the embedding's per-node incidence lists.
#include "evoc_internal.h"

#include <string>

namespace evoc {

[[noreturn]] void throw_cuda(cudaError_t e, const char* what, const char* file,
                             int line) {
  (void)cudaGetLastError();
  int code = (e == cudaErrorMemoryAllocation) ? EVOC_ERR_OUT_OF_MEMORY
                                              : EVOC_ERR_CUDA;
  throw Error(code, std::string(what) + " failed: " + cudaGetErrorString(e) +
                        " (" + file + ":" + std::to_string(line) + ")");
}

int bits_for(uint64_t max_value) {
  int b = 0;
  while (b < 64 && (max_value >> b) != 0) ++b;
  return b;
}

void check_status(evoc_ctx* ctx, const char* where) {
  int32_t st = 0;
  EVOC_CUDA(cudaMemcpyAsync(&st, ctx->status.get(), sizeof(int32_t),
                            cudaMemcpyDeviceToHost, ctx->stream));
  EVOC_CUDA(cudaStreamSynchronize(ctx->stream));
  if (st == 0) return;
  EVOC_CUDA(cudaMemsetAsync(ctx->status.get(), 0, sizeof(int32_t), ctx->stream));
  std::string w(where);
  if (st & ST_BAD_INDEX)
    throw Error(EVOC_ERR_INVALID_INPUT, w + ": an index is >= n");
  if (st & ST_BAD_VALUE)
    throw Error(EVOC_ERR_INVALID_INPUT, w + ": a distance or weight is NaN");
  if (st & ST_EMPTY_ROW)
    throw Error(EVOC_ERR_INVALID_INPUT,
                w + ": empty kNN row with local_connectivity > 0");
  if (st & ST_TOO_MANY_NEG)
    throw Error(EVOC_ERR_UNSUPPORTED,
                w + ": more than 2^20 negative samples per edge and epoch "
                    "(negative_sample_rate too large)");
  throw Error(EVOC_ERR_INTERNAL, w + ": device self-check failed");
}

// ---------------------------------------------------------------------------
// Scan: tiles of 2048 elements (256 threads x 8). Pass 1 reduces each tile,
// the tile sums are scanned recursively, pass 2 scans each tile with its
// carry-in.
// ---------------------------------------------------------------------------
namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename Tin>
__global__ void k_scan_reduce(const Tin* __restrict__ in, int64_t n,
                              int64_t* __restrict__ tile_sums) {
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  int64_t s = 0;
  for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
    int64_t g = base + i;
    if (g < n) s += (int64_t)in[g];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ int64_t warp_sums[SCAN_THREADS / 32];
  if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t t = 0;
    for (int w = 0; w < SCAN_THREADS / 32; ++w) t += warp_sums[w];
    tile_sums[blockIdx.x] = t;
  }
}

// Exclusive scan of one tile with carry-in; writes out[g] for g < n and,
// from the tile containing element n-1 (or tile 0 when n == 0), out[n].
template <typename Tin>
__global__ void k_scan_tile(const Tin* __restrict__ in, int64_t n,
                            const int64_t* __restrict__ carry,
                            int64_t* __restrict__ out) {
  __shared__ int64_t sm[SCAN_TILE];
  __shared__ int64_t warp_tot[SCAN_THREADS / 32];
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
    int64_t g = base + i;
    sm[i] = (g < n) ? (int64_t)in[g] : 0;
  }
  __syncthreads();
  int64_t local[SCAN_ITEMS];
  int64_t run = 0;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    local[j] = run;
    run += sm[threadIdx.x * SCAN_ITEMS + j];
  }
  // inclusive warp scan of per-thread totals
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t incl = run;
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  int64_t warp_off = 0;
  for (int w = 0; w < warp; ++w) warp_off += warp_tot[w];
  const int64_t thread_off = carry[blockIdx.x] + warp_off + incl - run;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) sm[threadIdx.x * SCAN_ITEMS + j] = thread_off + local[j];
  __syncthreads();
  for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
    int64_t g = base + i;
    if (g < n) out[g] = sm[i];
  }
  if (threadIdx.x == SCAN_THREADS - 1) {
    const int64_t tile_end = base + SCAN_TILE;
    if ((n > base && n <= tile_end) || (n == 0 && blockIdx.x == 0)) {
      int64_t tot = 0;
      for (int w = 0; w < SCAN_THREADS / 32; ++w) tot += warp_tot[w];
      out[n] = carry[blockIdx.x] + tot;
    }
  }
}

template <typename Tin>
void scan_impl(const Tin* in, int64_t* out, int64_t n, cudaStream_t s) {
  const int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles <= 1) {
    DevBuf<int64_t> zero(1, s);
    EVOC_CUDA(cudaMemsetAsync(zero.get(), 0, sizeof(int64_t), s));
    k_scan_tile<Tin><<<1, SCAN_THREADS, 0, s>>>(in, n, zero.get(), out);
    EVOC_CHECK_LAUNCH();
    return;
  }
  DevBuf<int64_t> sums(tiles, s), carry(tiles + 1, s);
  k_scan_reduce<Tin><<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, n, sums.get());
  EVOC_CHECK_LAUNCH();
  scan_impl<int64_t>(sums.get(), carry.get(), tiles, s);
  k_scan_tile<Tin><<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, n, carry.get(), out);
  EVOC_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// Radix sort: 8-bit digits, tiles of 4096 elements (256 threads x 16 rounds).
// Counts are laid out digit-major (count[d * tiles + t]) so that one exclusive
// scan gives every (digit, tile) its stable output offset. The scatter ranks
// elements in input order: round, then warp, then lane.
// ---------------------------------------------------------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;
constexpr int RS_WARPS = RS_THREADS / 32;

__global__ void k_radix_hist(const uint32_t* __restrict__ keys, int64_t n,
                             int shift, int64_t tiles,
                             int32_t* __restrict__ counts) {
  __shared__ int32_t hist[256];
  hist[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
  for (int r = 0; r < RS_ROUNDS; ++r) {
    int64_t g = base + r * RS_THREADS + threadIdx.x;
    if (g < n) atomicAdd(&hist[(keys[g] >> shift) & 255u], 1);
  }
  __syncthreads();
  counts[(int64_t)threadIdx.x * tiles + blockIdx.x] = hist[threadIdx.x];
}

__global__ void k_radix_scatter(const uint32_t* __restrict__ keys_in,
                                const uint2* __restrict__ vals_in, int64_t n,
                                int shift, int64_t tiles,
                                const int64_t* __restrict__ offsets,
                                uint32_t* __restrict__ keys_out,
                                uint2* __restrict__ vals_out) {
  __shared__ int64_t digit_base[256];
  __shared__ int32_t warp_cnt[RS_WARPS][256];
  __shared__ int64_t warp_off[RS_WARPS][256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int dd = threadIdx.x;  // the digit this thread keeps offsets for
  digit_base[dd] = offsets[(int64_t)dd * tiles + blockIdx.x];
  for (int w = 0; w < RS_WARPS; ++w) warp_cnt[w][dd] = 0;
  __syncthreads();
  const uint32_t lt_mask = (1u << lane) - 1u;
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
  for (int r = 0; r < RS_ROUNDS; ++r) {
    const int64_t g = base + r * RS_THREADS + threadIdx.x;
    const bool valid = g < n;
    uint32_t key = 0;
    uint2 val = make_uint2(0, 0);
    uint32_t d = 256;  // lanes past the end form their own peer group
    if (valid) {
      key = keys_in[g];
      val = vals_in[g];
      d = (key >> shift) & 255u;
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & lt_mask);
    if (valid && rank == 0) warp_cnt[warp][d] = __popc(peers);
    __syncthreads();
    // Output offset of digit dd for each warp of this round; advance the
    // digit's running base by the round's total. Counts are cleared for the
    // next round.
    int64_t run = digit_base[dd];
    for (int w = 0; w < RS_WARPS; ++w) {
      const int32_t c = warp_cnt[w][dd];
      warp_cnt[w][dd] = 0;
      warp_off[w][dd] = run;
      run += c;
    }
    digit_base[dd] = run;
    __syncthreads();
    if (valid) {
      const int64_t pos = warp_off[warp][d] + rank;
      keys_out[pos] = key;
      vals_out[pos] = val;
    }
    // warp_off is rewritten only after the next round's first barrier.
  }
}

}  // namespace

void exclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, int64_t n,
                               cudaStream_t s) {
  scan_impl<int32_t>(in, out, n, s);
}

void exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n,
                        cudaStream_t s) {
  scan_impl<int64_t>(in, out, n, s);
}

void radix_sort_pairs(uint32_t* keys, uint2* vals, int64_t n, int key_bits,
                      cudaStream_t s) {
  if (n <= 1 || key_bits <= 0) return;
  const int passes = (key_bits + 7) / 8;
  const int64_t tiles = (n + RS_TILE - 1) / RS_TILE;
  DevBuf<uint32_t> k2(n, s);
  DevBuf<uint2> v2(n, s);
  DevBuf<int32_t> counts(256 * tiles, s);
  DevBuf<int64_t> offsets(256 * tiles + 1, s);
  uint32_t* kin = keys;
  uint2* vin = vals;
  uint32_t* kout = k2.get();
  uint2* vout = v2.get();
  for (int p = 0; p < passes; ++p) {
    const int shift = 8 * p;
    k_radix_hist<<<(unsigned)tiles, RS_THREADS, 0, s>>>(kin, n, shift, tiles,
                                                       counts.get());
    EVOC_CHECK_LAUNCH();
    exclusive_scan_i32_to_i64(counts.get(), offsets.get(), 256 * tiles, s);
    k_radix_scatter<<<(unsigned)tiles, RS_THREADS, 0, s>>>(
        kin, vin, n, shift, tiles, offsets.get(), kout, vout);
    EVOC_CHECK_LAUNCH();
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  if (kin != keys) {
    EVOC_CUDA(cudaMemcpyAsync(keys, kin, n * sizeof(uint32_t),
                              cudaMemcpyDeviceToDevice, s));
    EVOC_CUDA(cudaMemcpyAsync(vals, vin, n * sizeof(uint2),
                              cudaMemcpyDeviceToDevice, s));
  }
}

}  // namespace evoc
