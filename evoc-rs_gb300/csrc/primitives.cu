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
    throw Error(EVOC_ERR_INVALID_INPUT, w + ": a distance or weight is NaN, or a coordinate "
                                            "is not finite");
  if (st & ST_EMPTY_ROW)
    throw Error(EVOC_ERR_INVALID_INPUT,
                w + ": empty kNN row with local_connectivity > 0");
  if (st & ST_CROSS_BLOCK)
    throw Error(EVOC_ERR_INVALID_INPUT, w + ": an edge joins two problems (graph not block-diagonal)");
  if (st & ST_WAIT_TIMEOUT)
    throw Error(EVOC_ERR_INTERNAL, w + ": a tensor-core wait timed out (results discarded)");
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

// Scatter of one 8-bit digit pass, tile per block. The tile is first sorted
// by digit in shared memory (stable: rounds in element order, lanes ranked by
// __match_any_sync, warps by per-digit prefix), then written out in digit
// order, so each digit's elements of the tile leave as one contiguous run.
struct RadixSmem {
  uint32_t keys[RS_TILE];
  uint2 vals[RS_TILE];
  int32_t warp_cnt[2][RS_WARPS][256];  // per round (alternating): counts, then offsets
  int32_t run[256];                 // elements of each digit placed so far
  int32_t tile_start[256];          // digit segment starts within the tile
  int64_t digit_base[256];          // the segments' global starts
};

__global__ void __launch_bounds__(RS_THREADS) k_radix_scatter(
    const uint32_t* __restrict__ keys_in, const uint2* __restrict__ vals_in, int64_t n,
    int shift, int64_t tiles, const int32_t* __restrict__ counts,
    const int64_t* __restrict__ offsets, uint32_t* __restrict__ keys_out,
    uint2* __restrict__ vals_out) {
  extern __shared__ __align__(16) unsigned char rs_raw[];
  RadixSmem& sm = *reinterpret_cast<RadixSmem*>(rs_raw);
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int dd = threadIdx.x;  // the digit this thread keeps bookkeeping for
  const int32_t c_dd = counts[(int64_t)dd * tiles + blockIdx.x];
  // exclusive prefix of the tile's digit counts (block scan over 256 digits)
  int32_t x = c_dd;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y = __shfl_up_sync(FULL, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm.run[warp] = x;  // warp totals (run is reset below)
  __syncthreads();
  int32_t before = 0;
  for (int w = 0; w < warp; ++w) before += sm.run[w];
  __syncthreads();
  sm.tile_start[dd] = before + x - c_dd;
  sm.digit_base[dd] = offsets[(int64_t)dd * tiles + blockIdx.x];
  sm.run[dd] = 0;
  for (int w = 0; w < RS_WARPS; ++w) sm.warp_cnt[0][w][dd] = sm.warp_cnt[1][w][dd] = 0;
  __syncthreads();
  const uint32_t lt_mask = (1u << lane) - 1u;
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
  const int tile_n = (int)min((int64_t)RS_TILE, n - base);
  for (int r = 0; r < RS_ROUNDS; ++r) {
    const int e = r * RS_THREADS + threadIdx.x;
    const bool valid = e < tile_n;
    uint32_t key = 0;
    uint2 val = make_uint2(0, 0);
    uint32_t d = 256;  // lanes past the end form their own peer group
    if (valid) {
      key = keys_in[base + e];
      val = vals_in[base + e];
      d = (key >> shift) & 255u;
    }
    const uint32_t peers = __match_any_sync(FULL, d);
    const int rank = __popc(peers & lt_mask);
    int32_t (*wc)[256] = sm.warp_cnt[r & 1];
    if (valid && rank == 0) wc[warp][d] = __popc(peers);
    __syncthreads();
    int32_t o = sm.run[dd];  // this round's warp offsets for digit dd
    for (int w = 0; w < RS_WARPS; ++w) {
      const int32_t c = wc[w][dd];
      wc[w][dd] = o;
      o += c;
      sm.warp_cnt[(r + 1) & 1][w][dd] = 0;  // last read before this round's first barrier
    }
    sm.run[dd] = o;
    __syncthreads();
    if (valid) {
      const int pos = sm.tile_start[d] + wc[warp][d] + rank;
      sm.keys[pos] = key;
      sm.vals[pos] = val;
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < tile_n; e += RS_THREADS) {
    const uint32_t key = sm.keys[e];
    const uint32_t d = (key >> shift) & 255u;
    const int64_t pos = sm.digit_base[d] + (e - sm.tile_start[d]);
    keys_out[pos] = key;
    vals_out[pos] = sm.vals[e];
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
  EVOC_CUDA(cudaFuncSetAttribute((const void*)k_radix_scatter,  // the staged tile > 48 KB
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(RadixSmem)));
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
    k_radix_scatter<<<(unsigned)tiles, RS_THREADS, sizeof(RadixSmem), s>>>(
        kin, vin, n, shift, tiles, counts.get(), offsets.get(), kout, vout);
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
