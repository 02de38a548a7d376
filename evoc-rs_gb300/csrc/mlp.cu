// mlp.cu — the learned warm start.
//
// A multilayer perceptron in_dim -> hidden -> hidden -> out_dim, with GELU after
// both hidden layers, predicts an initial embedding from the input points so
// that the embedding optimiser needs fewer epochs. It is trained on layouts
// that the plain optimiser itself produced, each aligned to the network's
// current prediction by an orthogonal Procrustes rotation (layouts are
// defined only up to isometry), with a mean-squared-error loss and Adam.
//
// Numerics: weights and activations feed the tensor cores as BF16 and are
// accumulated in FP32 (tcgen05.mma kind::f16 into tensor memory by default;
// an mma.sync m16n8k16 path stays as a cross-check); pre-activations, the loss, all
// gradients and the Adam state are FP32; an FP32 master copy of every
// parameter is what Adam updates, and its BF16 copy is refreshed each step.
// Every reduction has a fixed order, so results are reproducible run to run.
//
// Parameters are packed in one float array:
//   [W1 (hidden x in_dim), b1 (hidden), W2 (hidden x hidden), b2 (hidden),
//    W3 (out_dim x hidden), b3 (out_dim)]
// with every weight matrix row-major, output by input (a Linear layer's
// layout).
#include "evoc_internal.h"
#include "evoc_device.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>

using bf16 = __nv_bfloat16;

struct evoc_mlp {
  evoc_ctx* ctx = nullptr;
  int in = 0, hid = 0, out = 0;
  int64_t n_params = 0;
  int64_t o_w1 = 0, o_b1 = 0, o_w2 = 0, o_b2 = 0, o_w3 = 0, o_b3 = 0;
  evoc::DevBuf<float> master, adam_m, adam_v, grad;
  evoc::DevBuf<bf16> wb;   // BF16 copy of `master`, same packing
  evoc::DevBuf<bf16> w2t;  // BF16 W2 transposed ([in][out]), the K-major B operand of dH2 W2
  int64_t adam_steps = 0;
};

namespace evoc {
namespace {

// ---------------------------------------------------------------------------
// Tensor-core GEMM: C[M x N] = sum_k A(m, k) * B(n, k), BF16 in, FP32 out.
//
// Each operand is stored either K-major (row m holds A(m, 0..K) contiguously,
// leading dimension ld) or MN-major (row k holds A(0..M, k) contiguously).
// The forward layers are K-major x K-major; the input-gradient GEMM reads a
// weight matrix MN-major; the weight gradients read both operands MN-major
// (the batch is the reduction dimension). Tiles move global -> shared memory
// with 16-byte cp.async in their stored layout, and ldmatrix (.trans for
// MN-major tiles) builds the m16n8k16 fragments.
//
// 256 threads = 8 warps as 2 (M) x 4 (N), each warp owning a 64 x 32 piece of
// the 128 x 128 block tile; K advances 32 at a time through a 3-stage ring.
// ---------------------------------------------------------------------------
constexpr int GBM = 128, GBN = 128, GBK = 32, GSTAGES = 3, GTHREADS = 256;
constexpr int KPAD = GBK + 8;   // K-major tile row, in elements (80 bytes)
constexpr int MNPAD = GBM + 8;  // MN-major tile row, in elements (272 bytes)
constexpr int GTILE = (GBM * KPAD > GBK * MNPAD) ? GBM * KPAD : GBK * MNPAD;
constexpr int GEMM_SMEM = GSTAGES * 2 * GTILE * (int)sizeof(bf16);

enum GemmEpi : int {
  EPI_BIAS_GELU = 0,  // pre = acc + bias (f32, optional); outb = bf16(gelu(pre))
  EPI_GELU_GRAD = 1,  // outb = bf16(acc * gelu'(pre))
  EPI_PARTIAL = 2,    // outf[split][m][n] = acc
};

struct GemmArgs {
  const bf16* a;
  int64_t lda;
  const bf16* b;
  int64_t ldb;
  int M, N, K;
  int kchunk;          // rows of K per split (multiple of GBK)
  const float* bias;   // EPI_BIAS_GELU
  float* pre;          // EPI_BIAS_GELU: written if not null; EPI_GELU_GRAD: read
  bf16* outb;          // [M][N]
  float* outf;         // EPI_PARTIAL: [splits][M][N]
};

// GELU in its tanh form (Hendrycks & Gimpel, 2016):
//   gelu(x) = x/2 (1 + tanh(c (x + a x^3))),  c = sqrt(2/pi), a = 0.044715,
//   gelu'(x) = (1 + t)/2 + x/2 (1 - t^2) c (1 + 3 a x^2),  t = tanh(c (x + a x^3)),
// with the hardware tanh (tanh.approx.f32, relative error about 2^-11, below
// the BF16 rounding that follows every activation).
__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
constexpr float GELU_C = 0.7978845608028654f;
constexpr float GELU_A = 0.044715f;
__device__ __forceinline__ float gelu(float x) {
  const float t = tanh_approx(GELU_C * x * fmaf(GELU_A, x * x, 1.0f));
  const float hx = 0.5f * x;
  return fmaf(hx, t, hx);
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float x2 = x * x;
  const float t = tanh_approx(GELU_C * x * fmaf(GELU_A, x2, 1.0f));
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * GELU_C * fmaf(3.0f * GELU_A, x2, 1.0f);
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  const int n = valid ? 16 : 0;  // 0: fill the 16 bytes with zeros, read nothing
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const bf16* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const bf16* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}
__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Stage one operand tile (rows r0.. of the M or N dimension, K from kb) into
// shared memory. 512 chunks of 16 bytes per tile, two per thread. Chunks
// outside [0, rows) x [kb, kend) are zero-filled.
template <bool KMAJ>
__device__ __forceinline__ void load_tile(bf16* dst, const bf16* src, int64_t ld, int r0,
                                          int rows, int kb, int kend, int tid) {
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int c = tid + i * GTHREADS;
    if (KMAJ) {  // 128 rows x 4 chunks of 8 along K
      const int r = c >> 2, kc = (c & 3) << 3;
      const bool ok = (r0 + r < rows) && (kb + kc < kend);
      const bf16* g = ok ? src + (int64_t)(r0 + r) * ld + kb + kc : src;
      cp_async16(dst + r * KPAD + kc, g, ok);
    } else {  // 32 rows of K x 16 chunks of 8 along M (or N)
      const int kr = c >> 4, mc = (c & 15) << 3;
      const bool ok = (kb + kr < kend) && (r0 + mc < rows);
      const bf16* g = ok ? src + (int64_t)(kb + kr) * ld + r0 + mc : src;
      cp_async16(dst + kr * MNPAD + mc, g, ok);
    }
  }
}

template <bool A_KMAJ, bool B_KMAJ, int EPI>
__global__ void __launch_bounds__(GTHREADS) k_gemm(GemmArgs g) {
  extern __shared__ __align__(16) unsigned char gsm[];
  bf16* sA = reinterpret_cast<bf16*>(gsm);
  bf16* sB = sA + GSTAGES * GTILE;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 2, wn = warp & 3;
  const int m0 = blockIdx.y * GBM, n0 = blockIdx.x * GBN;
  const int kbeg = blockIdx.z * g.kchunk;
  const int kend = min(g.K, kbeg + g.kchunk);
  const int ntiles = kend > kbeg ? (kend - kbeg + GBK - 1) / GBK : 0;

  float acc[4][4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.0f;

#pragma unroll
  for (int s = 0; s < GSTAGES - 1; ++s) {
    if (s < ntiles) {
      load_tile<A_KMAJ>(sA + s * GTILE, g.a, g.lda, m0, g.M, kbeg + s * GBK, kend, tid);
      load_tile<B_KMAJ>(sB + s * GTILE, g.b, g.ldb, n0, g.N, kbeg + s * GBK, kend, tid);
    }
    cp_async_commit();
  }

  const int q = lane >> 3, r = lane & 7;
  for (int t = 0; t < ntiles; ++t) {
    cp_async_wait<GSTAGES - 2>();
    __syncthreads();
    {  // prefetch tile t + STAGES - 1 into the stage computed at t - 1
      const int tn = t + GSTAGES - 1;
      if (tn < ntiles) {
        const int st = tn % GSTAGES;
        load_tile<A_KMAJ>(sA + st * GTILE, g.a, g.lda, m0, g.M, kbeg + tn * GBK, kend, tid);
        load_tile<B_KMAJ>(sB + st * GTILE, g.b, g.ldb, n0, g.N, kbeg + tn * GBK, kend, tid);
      }
      cp_async_commit();
    }
    const bf16* tA = sA + (t % GSTAGES) * GTILE;
    const bf16* tB = sB + (t % GSTAGES) * GTILE;
#pragma unroll
    for (int kk = 0; kk < GBK; kk += 16) {
      uint32_t af[4][4], bfr[4][2];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int mr = wm * 64 + i * 16;
        if (A_KMAJ)
          ldsm_x4(af[i], tA + (mr + (lane & 15)) * KPAD + kk + ((lane >> 4) << 3));
        else
          ldsm_x4_t(af[i], tA + (kk + r + ((q >> 1) << 3)) * MNPAD + mr + ((q & 1) << 3));
      }
#pragma unroll
      for (int jj = 0; jj < 2; ++jj) {
        const int nc = wn * 32 + jj * 16;
        uint32_t tb[4];
        if (B_KMAJ)
          ldsm_x4(tb, tB + (nc + r + ((q >> 1) << 3)) * KPAD + kk + ((q & 1) << 3));
        else
          ldsm_x4_t(tb, tB + (kk + r + ((q & 1) << 3)) * MNPAD + nc + ((q >> 1) << 3));
        bfr[2 * jj][0] = tb[0];
        bfr[2 * jj][1] = tb[1];
        bfr[2 * jj + 1][0] = tb[2];
        bfr[2 * jj + 1][1] = tb[3];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j][0], bfr[j][1]);
    }
  }
  cp_async_wait<0>();

  // Epilogue: thread (g, c) of each 16 x 8 fragment holds rows g and g + 8,
  // columns 2c and 2c + 1.
  const int gq = lane >> 2, cq = lane & 3;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int col = n0 + wn * 32 + j * 8 + 2 * cq;
      if (col >= g.N) continue;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int row = m0 + wm * 64 + i * 16 + gq + 8 * h;
        if (row >= g.M) continue;
        const float v0 = acc[i][j][2 * h], v1 = acc[i][j][2 * h + 1];
        const int64_t o = (int64_t)row * g.N + col;
        if (EPI == EPI_BIAS_GELU) {
          const float p0 = v0 + g.bias[col], p1 = v1 + g.bias[col + 1];
          if (g.pre) *reinterpret_cast<float2*>(g.pre + o) = make_float2(p0, p1);
          *reinterpret_cast<__nv_bfloat162*>(g.outb + o) = __floats2bfloat162_rn(gelu(p0), gelu(p1));
        } else if (EPI == EPI_GELU_GRAD) {
          const float2 p = *reinterpret_cast<const float2*>(g.pre + o);
          *reinterpret_cast<__nv_bfloat162*>(g.outb + o) =
              __floats2bfloat162_rn(v0 * gelu_grad(p.x), v1 * gelu_grad(p.y));
        } else {
          *reinterpret_cast<float2*>(g.outf + (int64_t)blockIdx.z * g.M * g.N + o) =
              make_float2(v0, v1);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// GEMM layers on the 5th-generation tensor cores (tcgen05):
//   C = A B^T with A [M][K] and B [N][K] K-major BF16, then one of the TcEpi
//   epilogues (forward: bias + GELU, or with the output layer fused;
//   backward: times gelu'(pre), or FP32 split-K partials).
// One CTA computes a 128 x 256 tile whose FP32 accumulator lives in tensor
// memory (256 columns x 128 lanes).
//
// Mainloop (k_gemm_tc, the cp.async-fed variant; k_gemm_tma below moves the
// same tiles by TMA): K advances 64 elements (one 128-byte swizzle atom) per
// stage through a 2- or 4-stage shared-memory ring in the 128-byte swizzled
// K-major layout (row r, 16-byte chunk c at r * 128 + ((c ^ (r % 8)) * 16),
// 8-row groups 1024 bytes apart). One thread issues the four
// K = 16 MMAs of a stage (M = 128, N = 256, kind::f16 with BF16 inputs, FP32
// accumulation) and commits them to the stage's mbarrier; the ring slot is
// refilled once that barrier reports the MMAs done. Every wait is bounded
// (about two seconds of %globaltimer); on expiry the kernel records
// ST_WAIT_TIMEOUT, drains its own copies, frees its tensor memory and
// returns without writing.
//
// Epilogue: warp w reads tensor-memory lanes 32 (w % 4) .. +31 (its rows) and
// columns 128 (w / 4) .. +127 with tcgen05.ld, adds the bias, applies GELU
// and stores BF16 (and the FP32 pre-activation when asked). With HEAD (the
// second hidden layer at inference) the activations stay on chip: they feed
// a second tcgen05 MMA chain against the output layer's weights (see
// tc_epilogue), the CTA writes one partial output per row and column tile,
// and k_head_combine adds the tiles in order and the bias b3.
//
// Two stages of 48 KB let two CTAs share an SM (2 x 256 tensor-memory
// columns), so one CTA's epilogue overlaps the other's mainloop.
// ---------------------------------------------------------------------------
constexpr int TC_BM = 128, TC_BN = 256, TC_BK = 64, TC_THREADS = 256;
constexpr int TC_A_BYTES = TC_BM * TC_BK * 2;
constexpr int TC_B_BYTES = TC_BN * TC_BK * 2;
constexpr int TC_STAGE_BYTES = TC_A_BYTES + TC_B_BYTES;
constexpr uint32_t TC_TMEM_COLS = 256;

// Epilogues of the tcgen05 kernels.
enum TcEpi : int {
  TC_GELU = 0,  // outb = bf16(gelu(acc + bias)), pre = acc + bias (optional)
  TC_HEAD = 1,  // TC_GELU kept on chip, then the output layer (partials to ypart)
  TC_GRAD = 2,  // outb = bf16(acc * gelu'(pre))
  TC_F32 = 3,   // outf[split][m][n] = acc
};

struct HeadArgs {
  const bf16* w3;  // [out][N]
  int out;         // output width (<= 16)
  float* ypart;    // [column tiles][M][out]
};

// W3's columns of a tile for the head MMA: 16 rows (zero beyond out) x 256
// columns, K-major BF16 in four 128-byte swizzle atoms of 2 KB.
constexpr int TC_W3_BYTES = 16 * TC_BN * 2;

// Dynamic shared memory of the tcgen05 kernels: the ring (1024-byte aligned,
// 1 KB of slack), then with the head the W3 tile, then the tile's bias as f32.
inline int tc_smem_bytes(int stages, bool head) {
  return stages * TC_STAGE_BYTES + 1024 + (head ? TC_W3_BYTES : 0) + TC_BN * (int)sizeof(float);
}
constexpr unsigned long long TC_WAIT_NS = 2000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
// Wait for the completion of the phase with the given parity; false once
// limit_ns have passed since t0.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint64_t t0,
                                          uint64_t limit_ns = TC_WAIT_NS) {
  const uint32_t a = smem_u32(bar);
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}
// Non-blocking: has the phase with the given parity completed?
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) |
         ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t tc_idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}
__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(tmem_d), "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
        "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// One stage: A rows m0.. (128 x 64) and W rows n0.. (256 x 64) at K offset kb.
__device__ __forceinline__ void tc_load_stage(unsigned char* st, const GemmArgs& g, int m0, int n0,
                                              int kb, int tid) {
  unsigned char* sa = st;
  unsigned char* sb = st + TC_A_BYTES;
#pragma unroll
  for (int i = 0; i < (TC_BM * 8) / TC_THREADS; ++i) {
    const int c = tid + i * TC_THREADS, r = c >> 3, ch = c & 7;
    const int gm = m0 + r, gk = kb + ch * 8;
    const bool ok = gm < g.M && gk < g.K;
    const bf16* src = ok ? g.a + (int64_t)gm * g.lda + gk : g.a;
    cp_async16(sa + r * 128 + ((ch ^ (r & 7)) << 4), src, ok);
  }
#pragma unroll
  for (int i = 0; i < (TC_BN * 8) / TC_THREADS; ++i) {
    const int c = tid + i * TC_THREADS, r = c >> 3, ch = c & 7;
    const int gn = n0 + r, gk = kb + ch * 8;
    const bool ok = gn < g.N && gk < g.K;
    const bf16* src = ok ? g.b + (int64_t)gn * g.ldb + gk : g.b;
    cp_async16(sb + r * 128 + ((ch ^ (r & 7)) << 4), src, ok);
  }
}

// Per-CTA constants of the tcgen05 forward layers, staged before the
// mainloop: the bias of the tile's columns (zero beyond N) and, with the head,
// W3's columns of the tile as the B operand of the head MMA (16 rows, zero
// beyond out and beyond N; K-major, 128-byte swizzle).
template <bool HEAD>
__device__ __forceinline__ void tc_stage_constants(const GemmArgs& g, const HeadArgs& h,
                                                   unsigned char* w3b, float* bias_s, int n0,
                                                   int tid) {
  for (int j = tid; j < TC_BN; j += TC_THREADS)
    bias_s[j] = (g.bias && n0 + j < g.N) ? g.bias[n0 + j] : 0.0f;
  if (HEAD) {
    for (int i = tid; i < 16 * TC_BN; i += TC_THREADS) {
      const int o = i / TC_BN, j = i - o * TC_BN, n = n0 + j;
      const bf16 w = (o < h.out && n < g.N) ? h.w3[(int64_t)o * g.N + n] : __float2bfloat16_rn(0.0f);
      const int atom = j >> 6, ch = (j & 63) >> 3;
      *reinterpret_cast<bf16*>(w3b + atom * 2048 + o * 128 + ((ch ^ (o & 7)) << 4) + (j & 7) * 2) = w;
    }
  }
}

__device__ __forceinline__ void tc_ld16_nowait(uint32_t taddr, uint32_t* v) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
        "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}

// Epilogue of the tcgen05 forward layers (after the accumulator is complete);
// every thread of the CTA calls it. Returns false if the head MMA's bounded
// wait gave up.
//
// Without HEAD: bias + GELU, BF16 activations (and FP32 pre-activations) to
// global memory. With HEAD: the BF16 activations of the tile are written to
// the (now idle) ring as a K-major, 128-byte swizzled A operand
// (4 atoms of 128 rows x 64 columns), and one thread issues the output-layer
// MMA chain M = 128, N = 16, K = 256 against the staged W3 tile into tensor
// memory columns 0..15 (all accumulator reads are complete by then); the
// first four warps read the 16 results per row and store the out_dim partial
// outputs of this column tile.
template <int EPI>
__device__ __forceinline__ bool tc_epilogue(const GemmArgs& g, const HeadArgs& h, uint32_t tmem,
                                            unsigned char* ring, const unsigned char* w3b,
                                            const float* bias_s, uint64_t* hbar, uint64_t t0,
                                            int m0, int n0, int warp, int lane) {
  constexpr bool HEAD = EPI == TC_HEAD;
  const int lg = warp & 3, half = warp >> 2;
  const int r = lg * 32 + lane;  // row within the tile = tensor-memory lane
  const int row = m0 + r;
  const uint32_t tl = tmem + ((uint32_t)(lg * 32) << 16);
#pragma unroll 1
  for (int c = 0; c < TC_BN / 2; c += 32) {
    const int col0 = half * (TC_BN / 2) + c;
    uint32_t v[32];
    tc_ld16_nowait(tl + (uint32_t)col0, v);
    tc_ld16_nowait(tl + (uint32_t)col0 + 16u, v + 16);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      const int col = col0 + 16 * hh, n = n0 + col;
      if constexpr (EPI == TC_F32 || EPI == TC_GRAD) {
        if (row >= g.M || n >= g.N) continue;
        const int64_t o = (int64_t)row * g.N + n;
        const bool full = n + 16 <= g.N;
        if (EPI == TC_F32) {
          float* dst = g.outf + (int64_t)blockIdx.z * g.M * g.N + o;
          if (full) {
#pragma unroll
            for (int q = 0; q < 4; ++q)
              reinterpret_cast<float4*>(dst)[q] =
                  make_float4(__uint_as_float(v[16 * hh + 4 * q]), __uint_as_float(v[16 * hh + 4 * q + 1]),
                              __uint_as_float(v[16 * hh + 4 * q + 2]), __uint_as_float(v[16 * hh + 4 * q + 3]));
          } else {
#pragma unroll
            for (int j = 0; j < 16; ++j)
              if (n + j < g.N) dst[j] = __uint_as_float(v[16 * hh + j]);
          }
        } else {
          __align__(16) bf16 gb[16];
          if (full) {
            const float4* pr = reinterpret_cast<const float4*>(g.pre + o);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const float4 pq = pr[q];
              gb[4 * q] = __float2bfloat16_rn(__uint_as_float(v[16 * hh + 4 * q]) * gelu_grad(pq.x));
              gb[4 * q + 1] = __float2bfloat16_rn(__uint_as_float(v[16 * hh + 4 * q + 1]) * gelu_grad(pq.y));
              gb[4 * q + 2] = __float2bfloat16_rn(__uint_as_float(v[16 * hh + 4 * q + 2]) * gelu_grad(pq.z));
              gb[4 * q + 3] = __float2bfloat16_rn(__uint_as_float(v[16 * hh + 4 * q + 3]) * gelu_grad(pq.w));
            }
            uint4* dst = reinterpret_cast<uint4*>(g.outb + o);
            dst[0] = reinterpret_cast<const uint4*>(gb)[0];
            dst[1] = reinterpret_cast<const uint4*>(gb)[1];
          } else {
#pragma unroll
            for (int j = 0; j < 16; ++j)
              if (n + j < g.N)
                g.outb[o + j] =
                    __float2bfloat16_rn(__uint_as_float(v[16 * hh + j]) * gelu_grad(g.pre[o + j]));
          }
        }
      } else {
        float p[16];
        __align__(16) bf16 hb[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          p[j] = __uint_as_float(v[16 * hh + j]) + bias_s[col + j];
          hb[j] = __float2bfloat16_rn(gelu(p[j]));
        }
        if (HEAD) {
          // columns beyond N hold gelu(0) = 0
          const int atom = col >> 6, ch = (col & 63) >> 3;
          unsigned char* base = ring + atom * 16384 + r * 128;
          *reinterpret_cast<uint4*>(base + ((ch ^ (r & 7)) << 4)) =
              reinterpret_cast<const uint4*>(hb)[0];
          *reinterpret_cast<uint4*>(base + (((ch + 1) ^ (r & 7)) << 4)) =
              reinterpret_cast<const uint4*>(hb)[1];
        } else if (row < g.M && n < g.N) {
          const int64_t o = (int64_t)row * g.N + n;
          if (n + 16 <= g.N) {
            uint4* dst = reinterpret_cast<uint4*>(g.outb + o);
            dst[0] = reinterpret_cast<const uint4*>(hb)[0];
            dst[1] = reinterpret_cast<const uint4*>(hb)[1];
            if (g.pre) {
              float4* pd = reinterpret_cast<float4*>(g.pre + o);
#pragma unroll
              for (int q = 0; q < 4; ++q)
                pd[q] = make_float4(p[4 * q], p[4 * q + 1], p[4 * q + 2], p[4 * q + 3]);
            }
          } else {
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              if (n + j < g.N) {
                g.outb[o + j] = hb[j];
                if (g.pre) g.pre[o + j] = p[j];
              }
            }
          }
        }
      }
    }
  }
  if constexpr (!HEAD) return true;
  fence_async_smem();  // the activation tile -> visible to the tensor cores
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc_fence_after();
    const uint32_t a0 = smem_u32(ring), b0 = smem_u32(w3b);
    constexpr uint32_t idesc16 = tc_idesc(TC_BM, 16);
#pragma unroll
    for (int k = 0; k < TC_BN / 16; ++k) {
      const int atom = k >> 2, off = (k & 3) * 32;
      tc_mma(tmem, sw128_desc(a0 + atom * 16384 + off), sw128_desc(b0 + atom * 2048 + off),
             idesc16, k > 0 ? 1u : 0u);
    }
    tc_commit(hbar);
  }
  bool hok = mbar_wait(hbar, 0u, t0);
  hok = __syncthreads_and(hok ? 1 : 0) != 0;
  tc_fence_after();
  if (!hok) return false;
  if (half == 0) {
    uint32_t y[16];
    tc_ld16(tl, y);
    if (row < g.M) {
      float* dst = h.ypart + ((int64_t)blockIdx.x * g.M + row) * h.out;
#pragma unroll
      for (int o = 0; o < 16; ++o)
        if (o < h.out) dst[o] = __uint_as_float(y[o]);
    }
  }
  return true;
}

template <int STAGES, bool HEAD>
__global__ void __launch_bounds__(TC_THREADS, (STAGES <= 2 ? 2 : 1))
    k_gemm_tc(GemmArgs g, HeadArgs h, int32_t* __restrict__ status) {
  extern __shared__ unsigned char tc_raw[];
  __shared__ __align__(8) uint64_t mbar[STAGES];
  __shared__ __align__(8) uint64_t hbar;
  __shared__ uint32_t tmem_slot;
  const uint32_t raw = smem_u32(tc_raw);
  unsigned char* ring = tc_raw + (((raw + 1023u) & ~1023u) - raw);
  unsigned char* w3b = ring + STAGES * TC_STAGE_BYTES;  // HEAD: W3 tile
  float* bias_s = reinterpret_cast<float*>(w3b + (HEAD ? TC_W3_BYTES : 0));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * TC_BN;
  const int kt = (g.K + TC_BK - 1) / TC_BK;
  const uint64_t t0 = global_ns();

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) mbar_init(&mbar[s], 1);
    mbar_init(&hbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_stage_constants<HEAD>(g, h, w3b, bias_s, n0, tid);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

#pragma unroll
  for (int s = 0; s < STAGES - 1; ++s) {
    if (s < kt) tc_load_stage(ring + s * TC_STAGE_BYTES, g, m0, n0, s * TC_BK, tid);
    cp_async_commit();
  }
  constexpr uint32_t idesc = tc_idesc(TC_BM, TC_BN);
  bool ok = true;
  for (int t = 0; t < kt; ++t) {
    const int st = t % STAGES;
    cp_async_wait<STAGES - 2>();
    fence_async_smem();  // this thread's copies -> visible to the tensor cores
    // barrier + block-wide vote: every thread leaves the loop together
    if (!__syncthreads_and(ok ? 1 : 0)) {
      ok = false;
      break;
    }
    if (tid == 0) {
      tc_fence_after();
      const uint32_t a0 = smem_u32(ring + st * TC_STAGE_BYTES);
      const uint32_t b0 = a0 + TC_A_BYTES;
#pragma unroll
      for (int k = 0; k < TC_BK / 16; ++k)
        tc_mma(tmem, sw128_desc(a0 + k * 32), sw128_desc(b0 + k * 32), idesc,
               (t > 0 || k > 0) ? 1u : 0u);
      tc_commit(&mbar[st]);
    }
    const int tn = t + STAGES - 1;  // refill the slot read by tile t - 1
    if (tn < kt) {
      const int sn = tn % STAGES;
      if (t >= 1) ok = mbar_wait(&mbar[sn], (uint32_t)(((t - 1) / STAGES) & 1), t0);
      if (ok) tc_load_stage(ring + sn * TC_STAGE_BYTES, g, m0, n0, tn * TC_BK, tid);
    }
    cp_async_commit();
  }
  cp_async_wait<0>();
  if (ok) ok = mbar_wait(&mbar[(kt - 1) % STAGES], (uint32_t)(((kt - 1) / STAGES) & 1), t0);
  // every thread agrees on success before any tensor-memory read
  ok = __syncthreads_and(ok ? 1 : 0) != 0;
  tc_fence_after();
  if (!ok) {
    if (tid == 0) atomicOr(status, (int32_t)ST_WAIT_TIMEOUT);
  } else if (!tc_epilogue<HEAD ? TC_HEAD : TC_GELU>(g, h, tmem, ring, w3b, bias_s, &hbar, t0,
                                                  m0, n0, warp, lane)) {
    if (tid == 0) atomicOr(status, (int32_t)ST_WAIT_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TC_TMEM_COLS)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// The same forward layer with its operands moved by the Tensor Memory
// Accelerator: one thread (lane 0 of warp 0) runs the whole mainloop. For
// each stage it arms the stage's "full" mbarrier with the stage's byte count
// and issues two cp.async.bulk.tensor loads (A: 64 x 128 box at (k, m0);
// W: 64 x 256 box at (k, n0)), which land 128-byte swizzled, rows outside the
// matrices zero-filled; it waits for "full", issues the four MMAs and commits
// them to the stage's "empty" mbarrier, and refills a slot once "empty"
// reports its MMAs done. The other threads only wait for the final commit,
// then run the shared epilogue. No thread spends issue slots on address
// arithmetic or barriers during the mainloop.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, "
      "{%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

template <int STAGES, int EPI>
__global__ void __launch_bounds__(TC_THREADS, (STAGES <= 2 ? 2 : 1))
    k_gemm_tma(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
               GemmArgs g, HeadArgs h, int32_t* __restrict__ status) {
  constexpr bool HEAD = EPI == TC_HEAD;
  extern __shared__ unsigned char tc_raw[];
  __shared__ __align__(8) uint64_t full[STAGES];
  __shared__ __align__(8) uint64_t empty[STAGES];
  __shared__ __align__(8) uint64_t done;
  __shared__ __align__(8) uint64_t hbar;
  __shared__ uint32_t tmem_slot;
  __shared__ int aborted;
  const uint32_t raw = smem_u32(tc_raw);
  unsigned char* ring = tc_raw + (((raw + 1023u) & ~1023u) - raw);
  unsigned char* w3b = ring + STAGES * TC_STAGE_BYTES;  // HEAD: W3 tile
  float* bias_s = reinterpret_cast<float*>(w3b + (HEAD ? TC_W3_BYTES : 0));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * TC_BN;
  // this CTA's K range (split-K over blockIdx.z; kchunk is a multiple of TC_BK)
  const int kbeg = blockIdx.z * g.kchunk;
  const int kend = min(g.K, kbeg + g.kchunk);
  const int kt = kend > kbeg ? (kend - kbeg + TC_BK - 1) / TC_BK : 0;
  const uint64_t t0 = global_ns();

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    mbar_init(&hbar, 1);
    aborted = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_stage_constants<HEAD>(g, h, w3b, bias_s, n0, tid);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      auto issue = [&](int slot, int tile) {
        const uint32_t a_dst = smem_u32(ring + slot * TC_STAGE_BYTES);
        mbar_expect_tx(&full[slot], (uint32_t)TC_STAGE_BYTES);
        tma_load_2d(a_dst, &map_a, kbeg + tile * TC_BK, m0, &full[slot]);
        tma_load_2d(a_dst + TC_A_BYTES, &map_b, kbeg + tile * TC_BK, n0, &full[slot]);
      };
      constexpr uint32_t idesc = tc_idesc(TC_BM, TC_BN);
      int issued = 0, t = 0;
      bool okp = true;
      for (; issued < STAGES && issued < kt; ++issued) issue(issued, issued);
      for (; t < kt; ++t) {
        const int st = t % STAGES;
        if (!mbar_wait(&full[st], (uint32_t)((t / STAGES) & 1), t0)) {
          okp = false;
          break;
        }
        tc_fence_after();
        const uint32_t a0 = smem_u32(ring + st * TC_STAGE_BYTES);
        const uint32_t b0 = a0 + TC_A_BYTES;
#pragma unroll
        for (int k = 0; k < TC_BK / 16; ++k)
          tc_mma(tmem, sw128_desc(a0 + k * 32), sw128_desc(b0 + k * 32), idesc,
                 (t > 0 || k > 0) ? 1u : 0u);
        tc_commit(&empty[st]);
        // refill the slot of tile t - 1 once its MMAs are done (tile t's run meanwhile)
        if (t >= 1 && issued < kt) {
          const int sn = (t - 1) % STAGES;
          if (!mbar_wait(&empty[sn], (uint32_t)(((t - 1) / STAGES) & 1), t0)) {
            okp = false;
            ++t;  // tile t was consumed
            break;
          }
          issue(sn, issued);
          ++issued;
        }
      }
      if (okp) {
        tc_commit(&done);
      } else {
        aborted = 1;
        const uint64_t t1 = global_ns();  // drain the loads still in flight, bounded
        for (int u = t; u < issued; ++u)
          if (!mbar_wait(&full[u % STAGES], (uint32_t)((u / STAGES) & 1), t1)) break;
        mbar_arrive(&done);
      }
    }
    __syncwarp();
  }
  bool ok = mbar_wait(&done, 0u, t0);
  ok = __syncthreads_and(ok ? 1 : 0) != 0;
  ok = ok && !aborted;
  tc_fence_after();
  if (!ok) {
    if (tid == 0) atomicOr(status, (int32_t)ST_WAIT_TIMEOUT);
  } else if (!tc_epilogue<EPI>(g, h, tmem, ring, w3b, bias_s, &hbar, t0, m0, n0, warp, lane)) {
    if (tid == 0) atomicOr(status, (int32_t)ST_WAIT_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TC_TMEM_COLS)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// Persistent, warp-specialised forward layer (TMA + tcgen05), for N <= 2 x 256
// columns: one CTA per SM, a fixed column tile per CTA (CTA c takes column
// tile c % nc and row tiles c / nc, c / nc + G / nc, ...), so its bias slice
// and W3 slice are staged once.
//   warp 0 (lane 0): TMA producer, running ahead through the smem ring across
//                    tile boundaries (empty/full mbarriers);
//   warp 1 (lane 0): MMA issuer into one of two 256-column TMEM accumulators
//                    (tfull/tempty mbarriers), and, with HEAD, the output-layer
//                    MMA chain of the previous tile once its activations are
//                    staged (a2full -> hfull);
//   warps 4..11:     epilogue, warp w on TMEM lanes 32 (w % 4) and column half
//                    (w - 4) / 4; with HEAD the BF16 activations go to a
//                    dedicated 64 KB swizzled tile instead of global memory.
// The epilogue of tile i overlaps the mainloop of tile i + 1. Every wait is
// bounded (2 s each); a timeout sets ST_WAIT_TIMEOUT and an abort flag that
// every role checks before its next wait.
// ---------------------------------------------------------------------------
constexpr int PS_THREADS = 384;
constexpr int PS_A2_BYTES = TC_BM * TC_BN * 2;  // the staged activation tile (HEAD)

inline int ps_smem_bytes(int stages, bool head) {
  return stages * TC_STAGE_BYTES + 1024 + (head ? PS_A2_BYTES + TC_W3_BYTES : 0) +
         TC_BN * (int)sizeof(float);
}

template <int STAGES, bool HEAD>
__global__ void __launch_bounds__(PS_THREADS, 1)
    k_gemm_persist(const __grid_constant__ CUtensorMap map_a,
                   const __grid_constant__ CUtensorMap map_b, GemmArgs g, HeadArgs h,
                   int32_t* __restrict__ status) {
  extern __shared__ unsigned char tc_raw[];
  __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES];
  __shared__ __align__(8) uint64_t tfull[2], tempty[2], a2full, hfull;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int aborted;
  const uint32_t raw = smem_u32(tc_raw);
  unsigned char* ring = tc_raw + (((raw + 1023u) & ~1023u) - raw);
  unsigned char* a2s = ring + STAGES * TC_STAGE_BYTES;            // HEAD: [4 atoms][128][128 B]
  unsigned char* w3b = a2s + (HEAD ? PS_A2_BYTES : 0);            // HEAD: W3 slice
  float* bias_s = reinterpret_cast<float*>(w3b + (HEAD ? TC_W3_BYTES : 0));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nc = (g.N + TC_BN - 1) / TC_BN;          // column tiles (1 or 2)
  const int n0 = (int)(blockIdx.x % nc) * TC_BN;
  const int mt = (g.M + TC_BM - 1) / TC_BM;          // row tiles
  const int first = (int)(blockIdx.x / nc), step = (int)(gridDim.x / nc);
  const int kt = (g.K + TC_BK - 1) / TC_BK;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(2 * TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 8);  // one arrival per epilogue warp
    }
    mbar_init(&a2full, 8);
    mbar_init(&hfull, 1);
    aborted = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_stage_constants<HEAD>(g, h, w3b, bias_s, n0, tid);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  auto fail = [&]() {
    aborted = 1;
    atomicOr(status, (int32_t)ST_WAIT_TIMEOUT);
  };

  if (warp == 0) {
    if (lane == 0) {  // ---- TMA producer
      int64_t gk = 0;
      for (int mtile = first; mtile < mt && !aborted; mtile += step) {
        for (int kb = 0; kb < kt; ++kb, ++gk) {
          const int slot = (int)(gk % STAGES);
          if (gk >= STAGES &&
              !mbar_wait(&empty[slot], (uint32_t)(((gk / STAGES) - 1) & 1), global_ns())) {
            fail();
            break;
          }
          if (aborted) break;
          const uint32_t dst = smem_u32(ring + slot * TC_STAGE_BYTES);
          mbar_expect_tx(&full[slot], (uint32_t)TC_STAGE_BYTES);
          tma_load_2d(dst, &map_a, kb * TC_BK, mtile * TC_BM, &full[slot]);
          tma_load_2d(dst + TC_A_BYTES, &map_b, kb * TC_BK, n0, &full[slot]);
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {  // ---- MMA issuer
      constexpr uint32_t idesc = tc_idesc(TC_BM, TC_BN);
      constexpr uint32_t idesc16 = tc_idesc(TC_BM, 16);
      auto issue_head = [&](int it) {  // output layer of local tile it (a2full seen)
        tc_fence_after();
        const uint32_t a0 = smem_u32(a2s), b0 = smem_u32(w3b);
        const uint32_t acc = tmem + (uint32_t)((it & 1) * TC_BN);
#pragma unroll
        for (int k = 0; k < TC_BN / 16; ++k) {
          const int atom = k >> 2, off = (k & 3) * 32;
          tc_mma(acc, sw128_desc(a0 + atom * 16384 + off), sw128_desc(b0 + atom * 2048 + off),
                 idesc16, k > 0 ? 1u : 0u);
        }
        tc_commit(&hfull);
      };
      // The head of tile i is issued as soon as its activations are staged:
      // polled between the K steps of tile i + 1, or waited for at its end.
      int pending = -1;
      auto poll_head = [&]() {
        if (HEAD && pending >= 0 && mbar_test(&a2full, (uint32_t)(pending & 1))) {
          issue_head(pending);
          pending = -1;
        }
      };
      auto flush_head = [&]() {
        if (HEAD && pending >= 0) {
          if (!mbar_wait(&a2full, (uint32_t)(pending & 1), global_ns())) return false;
          issue_head(pending);
          pending = -1;
        }
        return true;
      };
      int64_t gk = 0;
      int it = 0;
      for (int mtile = first; mtile < mt && !aborted; mtile += step, ++it) {
        const int b = it & 1;
        if (it >= 2) {
          bool okt = false;  // wait for buffer b, polling the pending head meanwhile
          const uint64_t tw = global_ns();
          while (true) {
            poll_head();
            if (mbar_test(&tempty[b], (uint32_t)(((it >> 1) - 1) & 1))) {
              okt = true;
              break;
            }
            if (global_ns() - tw > TC_WAIT_NS) break;
          }
          if (!okt) {
            fail();
            break;
          }
        }
        tc_fence_after();
        const uint32_t acc = tmem + (uint32_t)(b * TC_BN);
        bool okk = true;
        for (int kb = 0; kb < kt; ++kb, ++gk) {
          const int slot = (int)(gk % STAGES);
          if (!mbar_wait(&full[slot], (uint32_t)((gk / STAGES) & 1), global_ns())) {
            okk = false;
            break;
          }
          tc_fence_after();
          const uint32_t a0 = smem_u32(ring + slot * TC_STAGE_BYTES);
          const uint32_t b0 = a0 + TC_A_BYTES;
#pragma unroll
          for (int k = 0; k < TC_BK / 16; ++k)
            tc_mma(acc, sw128_desc(a0 + k * 32), sw128_desc(b0 + k * 32), idesc,
                   (kb > 0 || k > 0) ? 1u : 0u);
          tc_commit(&empty[slot]);
          poll_head();
        }
        if (!okk) {
          fail();
          break;
        }
        tc_commit(&tfull[b]);
        if (HEAD) {
          if (!flush_head()) {  // the previous tile's head, if still pending
            fail();
            break;
          }
          pending = it;
        }
      }
      if (HEAD && !aborted && !flush_head()) fail();
    }
    __syncwarp();
  } else if (warp >= 4) {
    // ---- epilogue (part 2)
    const unsigned FULL = 0xffffffffu;
    const int ew = warp - 4, lg = warp & 3, half = ew >> 2;
    const int r = lg * 32 + lane;
    // a bounded wait whose outcome the whole warp shares
    auto wwait = [&](uint64_t* bar, uint32_t parity) {
      const bool okw = mbar_wait(bar, parity, global_ns());
      return __all_sync(FULL, okw ? 1 : 0) != 0;
    };
    int it = 0;
    for (int mtile = first; mtile < mt; mtile += step, ++it) {
      if (__any_sync(FULL, aborted)) break;
      const int b = it & 1;
      if (!wwait(&tfull[b], (uint32_t)((it >> 1) & 1))) {
        fail();
        break;
      }
      tc_fence_after();
      const int row = mtile * TC_BM + r;
      const uint32_t tl = tmem + (uint32_t)(b * TC_BN) + ((uint32_t)(lg * 32) << 16);
#pragma unroll 1
      for (int c = 0; c < TC_BN / 2; c += 32) {
        const int col0 = half * (TC_BN / 2) + c;
        uint32_t v[32];
        tc_ld16_nowait(tl + (uint32_t)col0, v);
        tc_ld16_nowait(tl + (uint32_t)col0 + 16u, v + 16);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          const int col = col0 + 16 * hh, n = n0 + col;
          float pv[16];
          __align__(16) bf16 hb[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            pv[j] = __uint_as_float(v[16 * hh + j]) + bias_s[col + j];
            hb[j] = __float2bfloat16_rn(gelu(pv[j]));
          }
          if (HEAD) {  // columns beyond N hold gelu(0) = 0
            const int atom = col >> 6, ch = (col & 63) >> 3;
            unsigned char* base = a2s + atom * 16384 + r * 128;
            *reinterpret_cast<uint4*>(base + ((ch ^ (r & 7)) << 4)) =
                reinterpret_cast<const uint4*>(hb)[0];
            *reinterpret_cast<uint4*>(base + (((ch + 1) ^ (r & 7)) << 4)) =
                reinterpret_cast<const uint4*>(hb)[1];
          } else if (row < g.M && n < g.N) {
            const int64_t o = (int64_t)row * g.N + n;
            if (n + 16 <= g.N) {
              uint4* dst = reinterpret_cast<uint4*>(g.outb + o);
              dst[0] = reinterpret_cast<const uint4*>(hb)[0];
              dst[1] = reinterpret_cast<const uint4*>(hb)[1];
              if (g.pre) {
                float4* pd = reinterpret_cast<float4*>(g.pre + o);
#pragma unroll
                for (int q = 0; q < 4; ++q)
                  pd[q] = make_float4(pv[4 * q], pv[4 * q + 1], pv[4 * q + 2], pv[4 * q + 3]);
              }
            } else {
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                if (n + j < g.N) {
                  g.outb[o + j] = hb[j];
                  if (g.pre) g.pre[o + j] = pv[j];
                }
              }
            }
          }
        }
      }
      if (HEAD) {
        fence_async_smem();  // the activation tile -> visible to the tensor cores
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&a2full);
        if (!wwait(&hfull, (uint32_t)(it & 1))) {
          fail();
          break;
        }
        tc_fence_after();
        if (half == 0) {
          uint32_t y[16];
          tc_ld16(tmem + (uint32_t)(b * TC_BN) + ((uint32_t)(lg * 32) << 16), y);
          if (row < g.M) {
            float* dst = h.ypart + ((int64_t)(blockIdx.x % nc) * g.M + row) * h.out;
#pragma unroll
            for (int o = 0; o < 16; ++o)
              if (o < h.out) dst[o] = __uint_as_float(y[o]);
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[b]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(2 * TC_TMEM_COLS)
                 : "memory");
  }
}

// Self-test of the timeout path: every thread waits on an mbarrier that
// nothing arrives on, gives up after limit_ns, and the block records
// ST_WAIT_TIMEOUT, as a tcgen05 kernel whose wait expired would.
__global__ void k_wait_probe(int32_t* __restrict__ status, uint64_t limit_ns) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  const bool ok = mbar_wait(&bar, 0u, global_ns(), limit_ns);
  if (!__syncthreads_and(ok ? 1 : 0) && threadIdx.x == 0)
    atomicOr(status, (int32_t)ST_WAIT_TIMEOUT);
}

// y[r][o] = sum over column tiles t (in order) of ypart[t][r][o], plus b3[o].
__global__ void k_head_combine(const float* __restrict__ ypart, int tiles, int64_t rows, int out,
                               const float* __restrict__ b3, float* __restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * out) return;
  const int o = (int)(i % out);
  float s = 0.0f;
  for (int t = 0; t < tiles; ++t) s += ypart[(int64_t)t * rows * out + i];
  y[i] = s + b3[o];
}

// ---------------------------------------------------------------------------
// Output layer (hidden -> out_dim, out_dim <= 16), one warp per row: the
// training step's head (loss and its gradients) and the output layer of the
// mma.sync cross-check path; tcgen05 inference fuses it into the second
// layer instead.
// Inference writes y. Training also forms the MSE gradient
//   dY = 2 (y - target) / (rows * out_dim),
// its back-projection dH2 = (dY W3) * gelu'(H2) in BF16, and per-block sums of
// (y - target)^2.
// ---------------------------------------------------------------------------
constexpr int MLP_MAX_OUT = 16;
constexpr int HEAD_THREADS = 256;

template <bool TRAIN>
__global__ void __launch_bounds__(HEAD_THREADS)
    k_head(const bf16* __restrict__ a2, const float* __restrict__ h2, int hid, int out,
           int64_t rows, const bf16* __restrict__ w3, const float* __restrict__ b3,
           float* __restrict__ y, const float* __restrict__ target, float grad_scale,
           float* __restrict__ dy, bf16* __restrict__ dh2, float* __restrict__ loss_part) {
  extern __shared__ float w3s[];  // [out][hid]
  __shared__ float wsum[HEAD_THREADS / 32];
  for (int i = threadIdx.x; i < out * hid; i += blockDim.x) w3s[i] = __bfloat162float(w3[i]);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nchunks = hid >> 3;
  float lsum = 0.0f;
  for (int64_t row = (int64_t)blockIdx.x * (HEAD_THREADS / 32) + warp; row < rows;
       row += (int64_t)gridDim.x * (HEAD_THREADS / 32)) {
    float acc[MLP_MAX_OUT];
#pragma unroll
    for (int o = 0; o < MLP_MAX_OUT; ++o) acc[o] = 0.0f;
    for (int c = lane; c < nchunks; c += 32) {
      const uint4 raw = *reinterpret_cast<const uint4*>(a2 + row * hid + c * 8);
      const bf16* av = reinterpret_cast<const bf16*>(&raw);
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const float x = __bfloat162float(av[e]);
#pragma unroll
        for (int o = 0; o < MLP_MAX_OUT; ++o)
          if (o < out) acc[o] += x * w3s[o * hid + c * 8 + e];
      }
    }
#pragma unroll
    for (int o = 0; o < MLP_MAX_OUT; ++o) {
      if (o >= out) break;
#pragma unroll
      for (int sh = 16; sh > 0; sh >>= 1) acc[o] += __shfl_xor_sync(0xffffffffu, acc[o], sh);
      acc[o] += b3[o];
    }
    if (!TRAIN) {
#pragma unroll
      for (int o = 0; o < MLP_MAX_OUT; ++o)
        if (o < out && lane == o) y[row * out + o] = acc[o];
      continue;
    }
    float gy[MLP_MAX_OUT];
    float rsum = 0.0f;
#pragma unroll
    for (int o = 0; o < MLP_MAX_OUT; ++o) {
      gy[o] = 0.0f;
      if (o < out) {
        const float d = acc[o] - target[row * out + o];
        rsum += d * d;
        gy[o] = d * grad_scale;
        if (lane == o) dy[row * out + o] = gy[o];
      }
    }
    lsum += rsum;  // identical on every lane; lane 0's copy is summed below
    for (int c = lane; c < nchunks; c += 32) {
      const float4 p0 = *reinterpret_cast<const float4*>(h2 + row * hid + c * 8);
      const float4 p1 = *reinterpret_cast<const float4*>(h2 + row * hid + c * 8 + 4);
      const float pv[8] = {p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w};
      __align__(16) bf16 res[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        float da = 0.0f;
#pragma unroll
        for (int o = 0; o < MLP_MAX_OUT; ++o)
          if (o < out) da += gy[o] * w3s[o * hid + c * 8 + e];
        res[e] = __float2bfloat16_rn(da * gelu_grad(pv[e]));
      }
      *reinterpret_cast<uint4*>(dh2 + row * hid + c * 8) = *reinterpret_cast<const uint4*>(res);
    }
  }
  if (TRAIN) {
    if (lane == 0) wsum[warp] = lsum;
    __syncthreads();
    if (threadIdx.x == 0) {
      float s = 0.0f;
      for (int w = 0; w < HEAD_THREADS / 32; ++w) s += wsum[w];
      loss_part[blockIdx.x] = s;
    }
  }
}

// Column sums over row splits (thread per column c < hid):
//   pw[z][o][c] = sum_{b in split z} dy[b][o] * a2[b][c]   (o < out; skipped if out == 0)
//   pb[z][c]    = sum_{b in split z} dh[b][c]
//   pb3[z][o]   = sum_{b in split z} dy[b][o]               (threads c < out of block 0)
__global__ void k_colreduce(const float* __restrict__ dy, int out, const bf16* __restrict__ a2,
                            const bf16* __restrict__ dh, int hid, int64_t rows,
                            int64_t rows_per_split, float* __restrict__ pw,
                            float* __restrict__ pb, float* __restrict__ pb3) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int z = blockIdx.y;
  const int64_t b0 = (int64_t)z * rows_per_split;
  const int64_t b1 = min(rows, b0 + rows_per_split);
  if (c >= hid) return;
  float acc[MLP_MAX_OUT];
#pragma unroll
  for (int o = 0; o < MLP_MAX_OUT; ++o) acc[o] = 0.0f;
  float accb = 0.0f, acc3 = 0.0f;
  const bool do3 = pb3 && blockIdx.x == 0 && c < out;
  for (int64_t b = b0; b < b1; ++b) {
    accb += __bfloat162float(dh[b * hid + c]);
    if (out > 0) {
      const float x = __bfloat162float(a2[b * hid + c]);
#pragma unroll
      for (int o = 0; o < MLP_MAX_OUT; ++o)
        if (o < out) acc[o] += dy[b * out + o] * x;
    }
    if (do3) acc3 += dy[b * out + c];
  }
  pb[(int64_t)z * hid + c] = accb;
#pragma unroll
  for (int o = 0; o < MLP_MAX_OUT; ++o)
    if (o < out) pw[((int64_t)z * out + o) * hid + c] = acc[o];
  if (do3) pb3[(int64_t)z * out + c] = acc3;
}

// grad[i] = sum_{z < splits} part[z * count + i], in split order.
__global__ void k_sum_splits(const float* __restrict__ part, int splits, int64_t count,
                             float* __restrict__ grad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  float s = 0.0f;
  for (int z = 0; z < splits; ++z) s += part[(int64_t)z * count + i];
  grad[i] = s;
}

// Adam with bias correction (Kingma & Ba, 2015): bc1 = 1 / (1 - beta1^t),
// bc2 = 1 / (1 - beta2^t).
__global__ void k_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, bf16* __restrict__ pb, int64_t count,
                       float lr, float beta1, float beta2, float eps, float bc1, float bc2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = beta1 * m[i] + (1.0f - beta1) * gi;
  const float vi = beta2 * v[i] + (1.0f - beta2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi * bc1) / (sqrtf(vi * bc2) + eps);
  p[i] = pi;
  pb[i] = __float2bfloat16_rn(pi);
}

__global__ void k_to_bf16(const float* __restrict__ x, int64_t count, bf16* __restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) y[i] = __float2bfloat16_rn(x[i]);
}

// dst[c][r] = src[r][c] for a rows x cols BF16 matrix (row strides lds, ldd),
// through 64 x 64 shared-memory tiles; coalesced on both sides.
__global__ void __launch_bounds__(256) k_transpose_bf16(const bf16* __restrict__ src, int64_t lds,
                                                        int rows, int cols, bf16* __restrict__ dst,
                                                        int64_t ldd) {
  __shared__ bf16 tile[64][66];
  const int r0 = blockIdx.y * 64, c0 = blockIdx.x * 64;
  const int tx = threadIdx.x & 63, ty = threadIdx.x >> 6;  // 64 x 4
  for (int i = ty; i < 64; i += 4) {
    const int r = r0 + i, c = c0 + tx;
    tile[i][tx] = (r < rows && c < cols) ? src[(int64_t)r * lds + c] : __float2bfloat16_rn(0.0f);
  }
  __syncthreads();
  for (int i = ty; i < 64; i += 4) {
    const int c = c0 + i, r = r0 + tx;
    if (c < cols && r < rows) dst[(int64_t)c * ldd + r] = tile[tx][i];
  }
}

// Row indices drawn uniformly with replacement from [0, n), keyed by (seed, draw).
__global__ void k_sample_rows(uint32_t* __restrict__ rows, int64_t count, uint32_t n,
                              uint64_t seed, uint32_t draw) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const uint4 o = philox4x32_10(make_uint4((uint32_t)i, draw, 0x4D4C5052u, 0x53414D50u),
                                make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
  rows[i] = __umulhi(o.x, n);
}

// dst[i][w] = src[rows[i]][w] for rows of `words` 32-bit words.
__global__ void k_gather_rows(const uint32_t* __restrict__ src, int64_t words,
                              const uint32_t* __restrict__ rows, int64_t count,
                              uint32_t* __restrict__ dst) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count * words) return;
  const int64_t i = t / words, w = t - i * words;
  dst[t] = src[(int64_t)rows[i] * words + w];
}

// out[r][j] = sum_i (x[r][i] - xmean[i]) * R[i][j] + ymean[j], d <= 16.
// aff = [R (d x d), xmean (d), ymean (d)].
__global__ void k_affine_rows(const float* __restrict__ x, int64_t rows, int d,
                              const float* __restrict__ aff, float* __restrict__ out) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  float xc[MLP_MAX_OUT];
#pragma unroll
  for (int i = 0; i < MLP_MAX_OUT; ++i) xc[i] = i < d ? x[r * d + i] - aff[d * d + i] : 0.0f;
  for (int j = 0; j < d; ++j) {
    float s = aff[d * d + d + j];
#pragma unroll
    for (int i = 0; i < MLP_MAX_OUT; ++i)
      if (i < d) s += xc[i] * aff[i * d + j];
    out[r * d + j] = s;
  }
}

__global__ void k_loss_total(const float* __restrict__ part, int nparts, float scale,
                             float* __restrict__ dst) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float s = 0.0f;
  for (int i = 0; i < nparts; ++i) s += part[i];
  *dst = s * scale;
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
inline unsigned blocks_for(int64_t n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

template <bool A_KMAJ, bool B_KMAJ, int EPI>
void launch_gemm(const GemmArgs& ga, int splits, cudaStream_t s) {
  EVOC_CUDA(cudaFuncSetAttribute(k_gemm<A_KMAJ, B_KMAJ, EPI>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, GEMM_SMEM));
  dim3 grid((unsigned)((ga.N + GBN - 1) / GBN), (unsigned)((ga.M + GBM - 1) / GBM),
            (unsigned)splits);
  k_gemm<A_KMAJ, B_KMAJ, EPI><<<grid, GTHREADS, GEMM_SMEM, s>>>(ga);
  EVOC_CHECK_LAUNCH();
}

// Forward-layer kernel: the persistent warp-specialised tcgen05 kernel
// (default, N <= 512); EVOC_MLP_GEMM=tma selects the one-tile-per-CTA TMA
// kernel, cpasync the cp.async-fed one, mma the mma.sync kernel (the
// cross-checks of the four paths).
enum class FwdPath { kPersist, kTma, kCpAsync, kMma };
FwdPath forward_path() {
  const char* e = std::getenv("EVOC_MLP_GEMM");
  if (e && std::strcmp(e, "mma") == 0) return FwdPath::kMma;
  if (e && std::strcmp(e, "cpasync") == 0) return FwdPath::kCpAsync;
  if (e && std::strcmp(e, "tma") == 0) return FwdPath::kTma;
  return FwdPath::kPersist;
}
bool use_tcgen05() { return forward_path() != FwdPath::kMma; }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    EVOC_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                               cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p)
      throw Error(EVOC_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// Tensor map of a K-major BF16 matrix [rows][k] (row stride ld elements):
// 64 x box_rows boxes, 128-byte swizzle, zero fill outside the matrix.
CUtensorMap tmap_kmajor(const bf16* base, int64_t rows, int64_t k, int64_t ld, int box_rows) {
  if ((reinterpret_cast<uintptr_t>(base) & 15) != 0 || (ld * 2) % 16 != 0)
    throw Error(EVOC_ERR_INVALID_ARGUMENT, "tensor-map operand not 16-byte aligned");
  CUtensorMap m;
  const cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = tmap_encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                                    const_cast<bf16*>(base), dims, strides, box, estr,
                                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    throw Error(EVOC_ERR_CUDA, "cuTensorMapEncodeTiled failed with code " + std::to_string((int)r));
  return m;
}

// Ring depth of the one-tile-per-CTA kernels (k_gemm_tc, k_gemm_tma): 2 stages
// (two CTAs per SM) unless EVOC_TC_STAGES=4 (one CTA per SM, deeper prefetch).
int tc_stages() {
  const char* e = std::getenv("EVOC_TC_STAGES");
  return (e && std::atoi(e) == 4) ? 4 : 2;
}

template <int S, int EPI>
void launch_tc(const GemmArgs& ga, const HeadArgs& ha, evoc_ctx* ctx, int splits = 1) {
  constexpr bool HEAD = EPI == TC_HEAD;
  const int smem = tc_smem_bytes(S, HEAD);
  dim3 grid((unsigned)((ga.N + TC_BN - 1) / TC_BN), (unsigned)((ga.M + TC_BM - 1) / TC_BM),
            (unsigned)splits);
  if constexpr (EPI == TC_GELU || EPI == TC_HEAD) {
    if (forward_path() == FwdPath::kCpAsync) {
      EVOC_CUDA(cudaFuncSetAttribute(k_gemm_tc<S, HEAD>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
      k_gemm_tc<S, HEAD><<<grid, TC_THREADS, smem, ctx->stream>>>(ga, ha, ctx->status.get());
      EVOC_CHECK_LAUNCH();
      return;
    }
  }
  const CUtensorMap ma = tmap_kmajor(ga.a, ga.M, ga.K, ga.lda, TC_BM);
  const CUtensorMap mb = tmap_kmajor(ga.b, ga.N, ga.K, ga.ldb, TC_BN);
  EVOC_CUDA(cudaFuncSetAttribute(k_gemm_tma<S, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem));
  k_gemm_tma<S, EPI><<<grid, TC_THREADS, smem, ctx->stream>>>(ma, mb, ga, ha, ctx->status.get());
  EVOC_CHECK_LAUNCH();
}

// Splits of K (multiples of TC_BK) so that tiles x splits covers about two
// CTAs per SM.
void choose_splits_tc(int M, int N, int K, int num_sms, int* splits, int* kchunk) {
  const int tiles = ((M + TC_BM - 1) / TC_BM) * ((N + TC_BN - 1) / TC_BN);
  const int ktiles = std::max(1, (K + TC_BK - 1) / TC_BK);
  int want = std::max(1, (2 * num_sms) / tiles);
  want = std::min(want, ktiles);
  const int per = (ktiles + want - 1) / want;
  *kchunk = per * TC_BK;
  *splits = std::max(1, (K + *kchunk - 1) / *kchunk);
}

// The persistent kernel: one CTA per SM (a multiple of the column tiles).
template <int S, bool HEAD>
void launch_persist(const GemmArgs& ga, const HeadArgs& ha, evoc_ctx* ctx) {
  const int nc = (ga.N + TC_BN - 1) / TC_BN;
  const int mt = (ga.M + TC_BM - 1) / TC_BM;
  const int grid = nc * std::max(1, std::min(mt, ctx->num_sms / nc));
  const int smem = ps_smem_bytes(S, HEAD);
  const CUtensorMap ma = tmap_kmajor(ga.a, ga.M, ga.K, ga.lda, TC_BM);
  const CUtensorMap mb = tmap_kmajor(ga.b, ga.N, ga.K, ga.ldb, TC_BN);
  EVOC_CUDA(cudaFuncSetAttribute(k_gemm_persist<S, HEAD>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  k_gemm_persist<S, HEAD><<<grid, PS_THREADS, smem, ctx->stream>>>(ma, mb, ga, ha,
                                                                   ctx->status.get());
  EVOC_CHECK_LAUNCH();
}

bool use_persist(const GemmArgs& ga) {
  return forward_path() == FwdPath::kPersist && ga.N <= 2 * TC_BN;
}

void launch_forward_gemm(const GemmArgs& ga, evoc_ctx* ctx) {
  if (!use_tcgen05()) {
    launch_gemm<true, true, EPI_BIAS_GELU>(ga, 1, ctx->stream);
    return;
  }
  if (use_persist(ga)) {
    launch_persist<4, false>(ga, HeadArgs{}, ctx);
    return;
  }
  const HeadArgs none{};
  if (tc_stages() == 4)
    launch_tc<4, TC_GELU>(ga, none, ctx);
  else
    launch_tc<2, TC_GELU>(ga, none, ctx);
}

// Second hidden layer fused with the output layer (inference on tcgen05).
void launch_forward_head(const GemmArgs& ga, const HeadArgs& ha, evoc_ctx* ctx) {
  if (use_persist(ga)) {
    launch_persist<3, true>(ga, ha, ctx);
    return;
  }
  if (tc_stages() == 4)
    launch_tc<4, TC_HEAD>(ga, ha, ctx);
  else
    launch_tc<2, TC_HEAD>(ga, ha, ctx);
}

int tc_col_tiles(int n) { return (n + TC_BN - 1) / TC_BN; }

void transpose_bf16(const bf16* src, int64_t lds, int rows, int cols, bf16* dst, int64_t ldd,
                    cudaStream_t s) {
  dim3 grid((unsigned)((cols + 63) / 64), (unsigned)((rows + 63) / 64));
  k_transpose_bf16<<<grid, 256, 0, s>>>(src, lds, rows, cols, dst, ldd);
  EVOC_CHECK_LAUNCH();
}

// Row stride (elements) of a transposed [cols][rows] copy: rows rounded up
// to 8, so every row starts 16-byte aligned (a TMA requirement).
int64_t transposed_ld(int64_t rows) { return (rows + 7) / 8 * 8; }

// Splits of the K dimension so that tiles x splits covers about two waves.
void choose_splits(int M, int N, int K, int num_sms, int* splits, int* kchunk) {
  const int tiles = ((M + GBM - 1) / GBM) * ((N + GBN - 1) / GBN);
  int want = std::max(1, (2 * num_sms + tiles - 1) / tiles);
  const int ktiles = std::max(1, (K + GBK - 1) / GBK);
  want = std::min(want, ktiles);
  const int per = (ktiles + want - 1) / want;
  *kchunk = per * GBK;
  *splits = std::max(1, (K + *kchunk - 1) / *kchunk);
}

// Scratch of one forward/backward pass over `rows` rows.
struct MlpScratch {
  DevBuf<bf16> x, a1, a2, dh1, dh2;
  DevBuf<bf16> xt, a1t, dh1t, dh2t;  // [features][batch] copies for the weight gradients
  DevBuf<float> h1, h2, target, dy, part, loss_part, loss, ypart;
  DevBuf<uint32_t> rows;
  int64_t cap = 0;
  int head_grid = 0;
};

int head_grid_for(const evoc_mlp* net, int64_t rows) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(
      (rows + HEAD_THREADS / 32 - 1) / (HEAD_THREADS / 32), 8LL * net->ctx->num_sms));
}

size_t head_smem(const evoc_mlp* net) { return (size_t)net->out * net->hid * sizeof(float); }

void set_head_smem(const evoc_mlp* net) {
  const int bytes = (int)head_smem(net);
  EVOC_CUDA(cudaFuncSetAttribute(k_head<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  EVOC_CUDA(cudaFuncSetAttribute(k_head<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
}

// Split-K partial buffer size of one training pass: the largest of the three
// weight-gradient reductions.
int64_t partial_floats(const evoc_mlp* net, int64_t rows, int* s1, int* kc1, int* s2, int* kc2,
                       int* s3, int64_t* rps3) {
  const int sms = net->ctx->num_sms;
  choose_splits(net->hid, net->in, (int)rows, sms, s1, kc1);
  choose_splits(net->hid, net->hid, (int)rows, sms, s2, kc2);
  const int colblocks = (net->hid + 127) / 128;
  int want3 = std::max(1, (2 * sms + colblocks - 1) / colblocks);
  *rps3 = std::max<int64_t>(1, (rows + want3 - 1) / want3);
  *s3 = (int)((rows + *rps3 - 1) / *rps3);
  int t1, tk1, t2, tk2;  // the tcgen05 weight-gradient splits
  choose_splits_tc(net->hid, net->in, (int)rows, sms, &t1, &tk1);
  choose_splits_tc(net->hid, net->hid, (int)rows, sms, &t2, &tk2);
  const int64_t p1 = (int64_t)std::max(*s1, t1) * net->hid * net->in;
  const int64_t p2 = (int64_t)std::max(*s2, t2) * net->hid * net->hid;
  const int64_t p3 = (int64_t)*s3 * ((int64_t)net->out * net->hid + 2 * net->hid + net->out);
  return std::max(p1, std::max(p2, p3));
}

void alloc_scratch(const evoc_mlp* net, MlpScratch& sc, int64_t rows, bool train) {
  cudaStream_t s = net->ctx->stream;
  sc.cap = rows;
  sc.x.alloc((size_t)rows * net->in, s);
  sc.a1.alloc((size_t)rows * net->hid, s);
  sc.a2.alloc((size_t)rows * net->hid, s);
  sc.head_grid = head_grid_for(net, rows);
  if (!train) {
    sc.ypart.alloc((size_t)tc_col_tiles(net->hid) * rows * net->out, s);
    return;
  }
  int s1, kc1, s2, kc2, s3;
  int64_t rps3;
  const int64_t pf = partial_floats(net, rows, &s1, &kc1, &s2, &kc2, &s3, &rps3);
  sc.h1.alloc((size_t)rows * net->hid, s);
  sc.h2.alloc((size_t)rows * net->hid, s);
  sc.dh1.alloc((size_t)rows * net->hid, s);
  sc.dh2.alloc((size_t)rows * net->hid, s);
  sc.target.alloc((size_t)rows * net->out, s);
  sc.dy.alloc((size_t)rows * net->out, s);
  sc.part.alloc((size_t)pf, s);
  sc.loss_part.alloc((size_t)sc.head_grid, s);
  if (use_tcgen05()) {
    const int64_t ldt = transposed_ld(rows);
    sc.xt.alloc((size_t)net->in * ldt, s);
    sc.a1t.alloc((size_t)net->hid * ldt, s);
    sc.dh1t.alloc((size_t)net->hid * ldt, s);
    sc.dh2t.alloc((size_t)net->hid * ldt, s);
  }
  sc.rows.alloc((size_t)rows, s);
}

// Forward over `rows` rows of BF16 input x (device); inference writes y.
void forward(const evoc_mlp* net, const bf16* x, int64_t rows, MlpScratch& sc, bool train,
             float* y) {
  cudaStream_t s = net->ctx->stream;
  const bf16* wb = net->wb.get();
  const float* mp = net->master.get();
  GemmArgs g1{};
  g1.a = x; g1.lda = net->in;
  g1.b = wb + net->o_w1; g1.ldb = net->in;
  g1.M = (int)rows; g1.N = net->hid; g1.K = net->in; g1.kchunk = ((net->in + GBK - 1) / GBK) * GBK;
  g1.bias = mp + net->o_b1;
  g1.pre = train ? sc.h1.get() : nullptr;
  g1.outb = sc.a1.get();
  launch_forward_gemm(g1, net->ctx);
  GemmArgs g2{};
  g2.a = sc.a1.get(); g2.lda = net->hid;
  g2.b = wb + net->o_w2; g2.ldb = net->hid;
  g2.M = (int)rows; g2.N = net->hid; g2.K = net->hid; g2.kchunk = ((net->hid + GBK - 1) / GBK) * GBK;
  g2.bias = mp + net->o_b2;
  g2.pre = train ? sc.h2.get() : nullptr;
  g2.outb = sc.a2.get();
  if (!train && use_tcgen05()) {
    const HeadArgs ha{wb + net->o_w3, net->out, sc.ypart.get()};
    launch_forward_head(g2, ha, net->ctx);
    k_head_combine<<<blocks_for(rows * net->out, 256), 256, 0, s>>>(
        sc.ypart.get(), tc_col_tiles(net->hid), rows, net->out, mp + net->o_b3, y);
    EVOC_CHECK_LAUNCH();
    return;
  }
  launch_forward_gemm(g2, net->ctx);
  if (!train) {
    k_head<false><<<head_grid_for(net, rows), HEAD_THREADS, head_smem(net), s>>>(
        sc.a2.get(), nullptr, net->hid, net->out, rows, wb + net->o_w3, mp + net->o_b3, y,
        nullptr, 0.0f, nullptr, nullptr, nullptr);
    EVOC_CHECK_LAUNCH();
  }
}

// Forward + backward over the batch in sc.x / sc.target (rows rows); leaves
// the packed gradient in net->grad and the mean-squared error in *loss_dst.
void forward_backward(evoc_mlp* net, int64_t rows, MlpScratch& sc, float* loss_dst) {
  cudaStream_t s = net->ctx->stream;
  const bf16* wb = net->wb.get();
  const float* mp = net->master.get();
  forward(net, sc.x.get(), rows, sc, true, nullptr);
  const int hg = head_grid_for(net, rows);
  const float scale = 1.0f / (float)((double)rows * net->out);
  k_head<true><<<hg, HEAD_THREADS, head_smem(net), s>>>(
      sc.a2.get(), sc.h2.get(), net->hid, net->out, rows, wb + net->o_w3, mp + net->o_b3,
      nullptr, sc.target.get(), 2.0f * scale, sc.dy.get(), sc.dh2.get(), sc.loss_part.get());
  EVOC_CHECK_LAUNCH();
  k_loss_total<<<1, 32, 0, s>>>(sc.loss_part.get(), hg, scale, loss_dst);
  EVOC_CHECK_LAUNCH();
  int s1, kc1, s2, kc2, s3;
  int64_t rps3;
  partial_floats(net, rows, &s1, &kc1, &s2, &kc2, &s3, &rps3);
  float* grad = net->grad.get();
  const int64_t cw1 = (int64_t)net->hid * net->in, cw2 = (int64_t)net->hid * net->hid;
  if (use_tcgen05()) {
    // dH1 = (dH2 W2) * gelu'(H1) with W2^T as the K-major B operand.
    const HeadArgs none{};
    GemmArgs gd{};
    gd.a = sc.dh2.get(); gd.lda = net->hid;
    gd.b = net->w2t.get(); gd.ldb = net->hid;
    gd.M = (int)rows; gd.N = net->hid; gd.K = net->hid;
    gd.kchunk = (net->hid + TC_BK - 1) / TC_BK * TC_BK;
    gd.pre = sc.h1.get();
    gd.outb = sc.dh1.get();
    launch_tc<2, TC_GRAD>(gd, none, net->ctx);
    // Weight gradients over the batch: K-major copies [features][batch].
    const int64_t ldt = transposed_ld(rows);
    transpose_bf16(sc.dh2.get(), net->hid, (int)rows, net->hid, sc.dh2t.get(), ldt, s);
    transpose_bf16(sc.a1.get(), net->hid, (int)rows, net->hid, sc.a1t.get(), ldt, s);
    transpose_bf16(sc.dh1.get(), net->hid, (int)rows, net->hid, sc.dh1t.get(), ldt, s);
    transpose_bf16(sc.x.get(), net->in, (int)rows, net->in, sc.xt.get(), ldt, s);
    int t2, tk2, t1, tk1;
    choose_splits_tc(net->hid, net->hid, (int)rows, net->ctx->num_sms, &t2, &tk2);
    choose_splits_tc(net->hid, net->in, (int)rows, net->ctx->num_sms, &t1, &tk1);
    GemmArgs gw2{};  // dW2 = dH2^T A1
    gw2.a = sc.dh2t.get(); gw2.lda = ldt;
    gw2.b = sc.a1t.get(); gw2.ldb = ldt;
    gw2.M = net->hid; gw2.N = net->hid; gw2.K = (int)rows; gw2.kchunk = tk2;
    gw2.outf = sc.part.get();
    launch_tc<2, TC_F32>(gw2, none, net->ctx, t2);
    k_sum_splits<<<blocks_for(cw2, 256), 256, 0, s>>>(sc.part.get(), t2, cw2, grad + net->o_w2);
    EVOC_CHECK_LAUNCH();
    GemmArgs gw1{};  // dW1 = dH1^T X
    gw1.a = sc.dh1t.get(); gw1.lda = ldt;
    gw1.b = sc.xt.get(); gw1.ldb = ldt;
    gw1.M = net->hid; gw1.N = net->in; gw1.K = (int)rows; gw1.kchunk = tk1;
    gw1.outf = sc.part.get();
    launch_tc<2, TC_F32>(gw1, none, net->ctx, t1);
    k_sum_splits<<<blocks_for(cw1, 256), 256, 0, s>>>(sc.part.get(), t1, cw1, grad + net->o_w1);
    EVOC_CHECK_LAUNCH();
  } else {
    // dH1 = (dH2 W2) * gelu'(H1): W2 is [out][in] = [K][N], read MN-major.
    GemmArgs gd{};
    gd.a = sc.dh2.get(); gd.lda = net->hid;
    gd.b = wb + net->o_w2; gd.ldb = net->hid;
    gd.M = (int)rows; gd.N = net->hid; gd.K = net->hid;
    gd.kchunk = ((net->hid + GBK - 1) / GBK) * GBK;
    gd.pre = sc.h1.get();
    gd.outb = sc.dh1.get();
    launch_gemm<true, false, EPI_GELU_GRAD>(gd, 1, s);
    // dW2 = dH2^T A1 (both [batch][hidden]: MN-major with the batch as K).
    GemmArgs gw2{};
    gw2.a = sc.dh2.get(); gw2.lda = net->hid;
    gw2.b = sc.a1.get(); gw2.ldb = net->hid;
    gw2.M = net->hid; gw2.N = net->hid; gw2.K = (int)rows; gw2.kchunk = kc2;
    gw2.outf = sc.part.get();
    launch_gemm<false, false, EPI_PARTIAL>(gw2, s2, s);
    k_sum_splits<<<blocks_for(cw2, 256), 256, 0, s>>>(sc.part.get(), s2, cw2, grad + net->o_w2);
    EVOC_CHECK_LAUNCH();
    // dW1 = dH1^T X.
    GemmArgs gw1{};
    gw1.a = sc.dh1.get(); gw1.lda = net->hid;
    gw1.b = sc.x.get(); gw1.ldb = net->in;
    gw1.M = net->hid; gw1.N = net->in; gw1.K = (int)rows; gw1.kchunk = kc1;
    gw1.outf = sc.part.get();
    launch_gemm<false, false, EPI_PARTIAL>(gw1, s1, s);
    k_sum_splits<<<blocks_for(cw1, 256), 256, 0, s>>>(sc.part.get(), s1, cw1, grad + net->o_w1);
    EVOC_CHECK_LAUNCH();
  }
  // dW3, db2, db3 in one column pass; then db1.
  float* pw3 = sc.part.get();
  float* pb2 = pw3 + (int64_t)s3 * net->out * net->hid;
  float* pb3 = pb2 + (int64_t)s3 * net->hid;
  float* pb1 = pb3 + (int64_t)s3 * net->out;
  dim3 cg((unsigned)((net->hid + 127) / 128), (unsigned)s3);
  k_colreduce<<<cg, 128, 0, s>>>(sc.dy.get(), net->out, sc.a2.get(), sc.dh2.get(), net->hid,
                                 rows, rps3, pw3, pb2, pb3);
  EVOC_CHECK_LAUNCH();
  k_colreduce<<<cg, 128, 0, s>>>(nullptr, 0, nullptr, sc.dh1.get(), net->hid, rows, rps3,
                                 nullptr, pb1, nullptr);
  EVOC_CHECK_LAUNCH();
  const int64_t cw3 = (int64_t)net->out * net->hid;
  k_sum_splits<<<blocks_for(cw3, 256), 256, 0, s>>>(pw3, s3, cw3, grad + net->o_w3);
  k_sum_splits<<<blocks_for(net->hid, 256), 256, 0, s>>>(pb2, s3, net->hid, grad + net->o_b2);
  k_sum_splits<<<1, 32, 0, s>>>(pb3, s3, net->out, grad + net->o_b3);
  k_sum_splits<<<blocks_for(net->hid, 256), 256, 0, s>>>(pb1, s3, net->hid, grad + net->o_b1);
  EVOC_CHECK_LAUNCH();
}

void refresh_w2t(evoc_mlp* net) {
  transpose_bf16(net->wb.get() + net->o_w2, net->hid, net->hid, net->hid, net->w2t.get(),
                 net->hid, net->ctx->stream);
}

void adam_step(evoc_mlp* net, float lr, float beta1, float beta2, float eps) {
  net->adam_steps += 1;
  const double t = (double)net->adam_steps;
  const float bc1 = (float)(1.0 / (1.0 - std::pow((double)beta1, t)));
  const float bc2 = (float)(1.0 / (1.0 - std::pow((double)beta2, t)));
  k_adam<<<blocks_for(net->n_params, 256), 256, 0, net->ctx->stream>>>(
      net->master.get(), net->adam_m.get(), net->adam_v.get(), net->grad.get(), net->wb.get(),
      net->n_params, lr, beta1, beta2, eps, bc1, bc2);
  EVOC_CHECK_LAUNCH();
  refresh_w2t(net);
}

void refresh_bf16(evoc_mlp* net) {
  k_to_bf16<<<blocks_for(net->n_params, 256), 256, 0, net->ctx->stream>>>(
      net->master.get(), net->n_params, net->wb.get());
  EVOC_CHECK_LAUNCH();
  refresh_w2t(net);
}

// splitmix64: the host-side generator of the initial weights.
uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

// ---------------------------------------------------------------------------
// Orthogonal Procrustes: the orthogonal R (d x d) maximising tr(R^T M), i.e.
// R = U V^T for M = U S V^T, by one-sided Jacobi rotations on the columns of
// M (Hestenes' method). For M = X^T Y with centred X, Y it minimises
// ||X R - Y||_F. Columns with a vanishing singular value get an orthonormal
// completion.
// ---------------------------------------------------------------------------
void procrustes(const double* m, int d, double* r) {
  std::vector<double> a(m, m + (size_t)d * d), v((size_t)d * d, 0.0), u((size_t)d * d, 0.0);
  for (int i = 0; i < d; ++i) v[(size_t)i * d + i] = 1.0;
  auto A = [&](int i, int j) -> double& { return a[(size_t)i * d + j]; };
  auto V = [&](int i, int j) -> double& { return v[(size_t)i * d + j]; };
  for (int sweep = 0; sweep < 100; ++sweep) {
    bool rotated = false;
    for (int p = 0; p < d - 1; ++p) {
      for (int q = p + 1; q < d; ++q) {
        double alpha = 0, beta = 0, gamma = 0;
        for (int i = 0; i < d; ++i) {
          alpha += A(i, p) * A(i, p);
          beta += A(i, q) * A(i, q);
          gamma += A(i, p) * A(i, q);
        }
        if (std::fabs(gamma) <= 1e-15 * std::sqrt(alpha * beta) || gamma == 0.0) continue;
        rotated = true;
        const double zeta = (beta - alpha) / (2.0 * gamma);
        const double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
        for (int i = 0; i < d; ++i) {
          const double ap = A(i, p), aq = A(i, q);
          A(i, p) = c * ap - s * aq;
          A(i, q) = s * ap + c * aq;
          const double vp = V(i, p), vq = V(i, q);
          V(i, p) = c * vp - s * vq;
          V(i, q) = s * vp + c * vq;
        }
      }
    }
    if (!rotated) break;
  }
  // U = A S^-1, columns in order of decreasing singular value get first pick
  // when a completion is needed.
  std::vector<double> sig(d);
  double smax = 0;
  for (int j = 0; j < d; ++j) {
    double s2 = 0;
    for (int i = 0; i < d; ++i) s2 += A(i, j) * A(i, j);
    sig[j] = std::sqrt(s2);
    smax = std::max(smax, sig[j]);
  }
  std::vector<int> order(d);
  for (int j = 0; j < d; ++j) order[j] = j;
  std::sort(order.begin(), order.end(), [&](int x, int y) { return sig[x] > sig[y]; });
  std::vector<bool> done(d, false);
  for (int j : order) {
    if (sig[j] > 1e-12 * smax && smax > 0) {
      for (int i = 0; i < d; ++i) u[(size_t)i * d + j] = A(i, j) / sig[j];
      done[j] = true;
    }
  }
  for (int j : order) {
    if (done[j]) continue;
    for (int e = 0; e < d && !done[j]; ++e) {  // Gram-Schmidt on unit vectors
      std::vector<double> w(d, 0.0);
      w[e] = 1.0;
      for (int k = 0; k < d; ++k) {
        if (!done[k]) continue;
        double dot = 0;
        for (int i = 0; i < d; ++i) dot += w[i] * u[(size_t)i * d + k];
        for (int i = 0; i < d; ++i) w[i] -= dot * u[(size_t)i * d + k];
      }
      double nrm = 0;
      for (int i = 0; i < d; ++i) nrm += w[i] * w[i];
      nrm = std::sqrt(nrm);
      if (nrm < 1e-6) continue;
      for (int i = 0; i < d; ++i) u[(size_t)i * d + j] = w[i] / nrm;
      done[j] = true;
    }
  }
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) {
      double s = 0;
      for (int k = 0; k < d; ++k) s += u[(size_t)i * d + k] * V(j, k);
      r[(size_t)i * d + j] = s;
    }
}

void wait_timeout_selftest(evoc_ctx* ctx, int32_t limit_ms) {
  k_wait_probe<<<1, 64, 0, ctx->stream>>>(ctx->status.get(), (uint64_t)limit_ms * 1000000ull);
  EVOC_CHECK_LAUNCH();
  check_status(ctx, "wait self-test");
}

evoc_mlp* mlp_create(evoc_ctx* ctx, int in, int hid, int out, uint64_t seed) {
  if (in <= 0 || hid <= 0 || out <= 0 || in % 8 != 0 || hid % 8 != 0)
    throw Error(EVOC_ERR_INVALID_ARGUMENT, "in_dim and hidden must be positive multiples of 8");
  if (out > MLP_MAX_OUT) throw Error(EVOC_ERR_UNSUPPORTED, "out_dim must be in 1..16");
  if (in > 65536 || hid > 8192)
    throw Error(EVOC_ERR_UNSUPPORTED, "in_dim above 65536 or hidden above 8192");
  if ((size_t)out * hid * sizeof(float) > 200 * 1024)
    throw Error(EVOC_ERR_UNSUPPORTED, "out_dim x hidden too large for the output layer");
  std::unique_ptr<evoc_mlp> net(new evoc_mlp());
  net->ctx = ctx;
  net->in = in;
  net->hid = hid;
  net->out = out;
  net->o_w1 = 0;
  net->o_b1 = net->o_w1 + (int64_t)hid * in;
  net->o_w2 = net->o_b1 + hid;
  net->o_b2 = net->o_w2 + (int64_t)hid * hid;
  net->o_w3 = net->o_b2 + hid;
  net->o_b3 = net->o_w3 + (int64_t)out * hid;
  net->n_params = net->o_b3 + out;
  cudaStream_t s = ctx->stream;
  const size_t np = (size_t)net->n_params;
  net->master.alloc(np, s);
  net->adam_m.alloc(np, s);
  net->adam_v.alloc(np, s);
  net->grad.alloc(np, s);
  net->wb.alloc(np, s);
  net->w2t.alloc((size_t)hid * hid, s);
  // Linear-layer initialisation: weights and biases uniform in
  // [-1/sqrt(fan_in), 1/sqrt(fan_in)).
  std::vector<float> h(np);
  uint64_t st = seed;
  auto fill = [&](int64_t off, int64_t count, int fan_in) {
    const double bound = 1.0 / std::sqrt((double)fan_in);
    for (int64_t i = 0; i < count; ++i) {
      const double u = (double)(splitmix64(st) >> 11) * (1.0 / 9007199254740992.0);
      h[(size_t)(off + i)] = (float)((2.0 * u - 1.0) * bound);
    }
  };
  fill(net->o_w1, (int64_t)hid * in, in);
  fill(net->o_b1, hid, in);
  fill(net->o_w2, (int64_t)hid * hid, hid);
  fill(net->o_b2, hid, hid);
  fill(net->o_w3, (int64_t)out * hid, hid);
  fill(net->o_b3, out, hid);
  EVOC_CUDA(cudaMemcpyAsync(net->master.get(), h.data(), np * sizeof(float),
                            cudaMemcpyHostToDevice, s));
  EVOC_CUDA(cudaMemsetAsync(net->adam_m.get(), 0, np * sizeof(float), s));
  EVOC_CUDA(cudaMemsetAsync(net->adam_v.get(), 0, np * sizeof(float), s));
  EVOC_CUDA(cudaMemsetAsync(net->grad.get(), 0, np * sizeof(float), s));
  refresh_bf16(net.get());
  set_head_smem(net.get());
  EVOC_CUDA(cudaStreamSynchronize(s));
  return net.release();
}

void mlp_free(evoc_mlp* net) {
  if (!net) return;
  cudaStream_t s = net->ctx ? net->ctx->stream : nullptr;
  net->master.release();
  net->adam_m.release();
  net->adam_v.release();
  net->grad.release();
  net->wb.release();
  net->w2t.release();
  if (s) cudaStreamSynchronize(s);
  delete net;
}

evoc_ctx* mlp_ctx(const evoc_mlp* net) { return net->ctx; }
int64_t mlp_n_params(const evoc_mlp* net) { return net->n_params; }
void mlp_dims(const evoc_mlp* net, int32_t* in, int32_t* hid, int32_t* out) {
  if (in) *in = net->in;
  if (hid) *hid = net->hid;
  if (out) *out = net->out;
}

void mlp_get_params(const evoc_mlp* net, float* host) {
  cudaStream_t s = net->ctx->stream;
  EVOC_CUDA(cudaMemcpyAsync(host, net->master.get(), net->master.bytes(), cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaStreamSynchronize(s));
}

void mlp_set_params(evoc_mlp* net, const float* host) {
  cudaStream_t s = net->ctx->stream;
  EVOC_CUDA(cudaMemcpyAsync(net->master.get(), host, net->master.bytes(), cudaMemcpyHostToDevice, s));
  EVOC_CUDA(cudaMemsetAsync(net->adam_m.get(), 0, net->adam_m.bytes(), s));
  EVOC_CUDA(cudaMemsetAsync(net->adam_v.get(), 0, net->adam_v.bytes(), s));
  net->adam_steps = 0;
  refresh_bf16(net);
  EVOC_CUDA(cudaStreamSynchronize(s));
}

void to_bf16_device(evoc_ctx* ctx, const float* x, int64_t count, uint16_t* y) {
  if (count == 0) return;
  k_to_bf16<<<blocks_for(count, 256), 256, 0, ctx->stream>>>(x, count, reinterpret_cast<bf16*>(y));
  EVOC_CHECK_LAUNCH();
}

constexpr int64_t PREDICT_CHUNK = 262144;

void mlp_predict_device(evoc_mlp* net, const uint16_t* x, int64_t n, float* y) {
  if (n == 0) return;
  MlpScratch sc;
  const int64_t chunk = std::min(n, PREDICT_CHUNK);
  alloc_scratch(net, sc, chunk, false);
  const bf16* xb = reinterpret_cast<const bf16*>(x);
  for (int64_t r0 = 0; r0 < n; r0 += chunk) {
    const int64_t rows = std::min(chunk, n - r0);
    forward(net, xb + r0 * net->in, rows, sc, false, y + r0 * net->out);
  }
  check_status(net->ctx, "evoc_mlp_predict_device");
}

void mlp_predict_host(evoc_mlp* net, const float* x, int64_t n, float* y) {
  if (n == 0) return;
  cudaStream_t s = net->ctx->stream;
  const int64_t chunk = std::min(n, PREDICT_CHUNK);
  MlpScratch sc;
  alloc_scratch(net, sc, chunk, false);
  DevBuf<float> xf((size_t)chunk * net->in, s), yd((size_t)chunk * net->out, s);
  for (int64_t r0 = 0; r0 < n; r0 += chunk) {
    const int64_t rows = std::min(chunk, n - r0);
    EVOC_CUDA(cudaMemcpyAsync(xf.get(), x + r0 * net->in, (size_t)rows * net->in * sizeof(float),
                              cudaMemcpyHostToDevice, s));
    to_bf16_device(net->ctx, xf.get(), rows * net->in, reinterpret_cast<uint16_t*>(sc.x.get()));
    forward(net, sc.x.get(), rows, sc, false, yd.get());
    EVOC_CUDA(cudaMemcpyAsync(y + r0 * net->out, yd.get(), (size_t)rows * net->out * sizeof(float),
                              cudaMemcpyDeviceToHost, s));
  }
  check_status(net->ctx, "evoc_mlp_predict");
}

void mlp_gradients_host(evoc_mlp* net, const float* x, const float* target, int64_t n,
                        float* loss, float* grad) {
  if (n <= 0) throw Error(EVOC_ERR_INVALID_ARGUMENT, "n must be positive");
  if (n > (1LL << 24)) throw Error(EVOC_ERR_UNSUPPORTED, "at most 2^24 rows per gradient call");
  cudaStream_t s = net->ctx->stream;
  MlpScratch sc;
  alloc_scratch(net, sc, n, true);
  DevBuf<float> xf((size_t)n * net->in, s), ld(1, s);
  EVOC_CUDA(cudaMemcpyAsync(xf.get(), x, xf.bytes(), cudaMemcpyHostToDevice, s));
  EVOC_CUDA(cudaMemcpyAsync(sc.target.get(), target, (size_t)n * net->out * sizeof(float),
                            cudaMemcpyHostToDevice, s));
  to_bf16_device(net->ctx, xf.get(), n * net->in, reinterpret_cast<uint16_t*>(sc.x.get()));
  forward_backward(net, n, sc, ld.get());
  EVOC_CUDA(cudaMemcpyAsync(grad, net->grad.get(), net->grad.bytes(), cudaMemcpyDeviceToHost, s));
  EVOC_CUDA(cudaMemcpyAsync(loss, ld.get(), sizeof(float), cudaMemcpyDeviceToHost, s));
  check_status(net->ctx, "evoc_mlp_gradients");
}

// Training on layouts of several instances (step size falling linearly from
// lr to lr_end): every `align_every` steps each
// instance's layout is re-aligned to the network's prediction on a fixed
// sample of its rows (means removed, Procrustes rotation, prediction mean
// added); each step then draws `batch` rows of one instance (round robin)
// and takes one Adam step on the MSE against the aligned layout.
void mlp_fit_device(evoc_mlp* net, int32_t m, const uint16_t* const* xs,
                    const float* const* layouts, const int64_t* ns,
                    const evoc_mlp_train_params_t* p, float* loss_history) {
  if (m <= 0 || !xs || !layouts || !ns || !p) throw Error(EVOC_ERR_INVALID_ARGUMENT, "bad argument");
  if (p->steps < 0 || p->batch <= 0 || p->batch > (1 << 22) || p->align_every <= 0 ||
      p->align_rows <= 0)
    throw Error(EVOC_ERR_INVALID_ARGUMENT, "bad training parameters");
  for (int32_t i = 0; i < m; ++i) {
    if (!xs[i] || !layouts[i] || ns[i] <= 0 || ns[i] >= 0xFFFFFFFFLL)
      throw Error(EVOC_ERR_INVALID_ARGUMENT, "bad instance " + std::to_string(i));
  }
  cudaStream_t s = net->ctx->stream;
  const int d = net->out;
  const int64_t batch = p->batch;
  MlpScratch sc;
  alloc_scratch(net, sc, batch, true);
  // aligned layouts and the fixed alignment sample of every instance
  std::vector<DevBuf<float>> aligned(m);
  std::vector<DevBuf<uint32_t>> sample(m);
  std::vector<int64_t> ns_sample(m);
  for (int32_t i = 0; i < m; ++i) {
    aligned[i].alloc((size_t)ns[i] * d, s);
    EVOC_CUDA(cudaMemcpyAsync(aligned[i].get(), layouts[i], (size_t)ns[i] * d * sizeof(float),
                              cudaMemcpyDeviceToDevice, s));
    ns_sample[i] = std::min<int64_t>(ns[i], p->align_rows);
    sample[i].alloc((size_t)ns_sample[i], s);
    k_sample_rows<<<blocks_for(ns_sample[i], 256), 256, 0, s>>>(
        sample[i].get(), ns_sample[i], (uint32_t)ns[i], p->seed ^ 0xA11A11A11ull, (uint32_t)i);
    EVOC_CHECK_LAUNCH();
  }
  const int64_t max_sample = *std::max_element(ns_sample.begin(), ns_sample.end());
  MlpScratch sp;  // prediction on an alignment sample
  alloc_scratch(net, sp, std::min<int64_t>(max_sample, PREDICT_CHUNK), false);
  DevBuf<bf16> xs_s((size_t)max_sample * net->in, s);
  DevBuf<float> pred((size_t)max_sample * d, s), tsamp((size_t)max_sample * d, s);
  DevBuf<float> aff((size_t)d * d + 2 * d, s);
  DevBuf<float> losses((size_t)std::max(1, p->steps), s);
  std::vector<float> hp((size_t)max_sample * d), ht((size_t)max_sample * d);
  std::vector<float> haff((size_t)d * d + 2 * d);

  auto realign = [&](int32_t i) {
    const int64_t k = ns_sample[i];
    k_gather_rows<<<blocks_for(k * net->in / 2, 256), 256, 0, s>>>(
        reinterpret_cast<const uint32_t*>(xs[i]), net->in / 2, sample[i].get(), k,
        reinterpret_cast<uint32_t*>(xs_s.get()));
    EVOC_CHECK_LAUNCH();
    k_gather_rows<<<blocks_for(k * d, 256), 256, 0, s>>>(
        reinterpret_cast<const uint32_t*>(layouts[i]), d, sample[i].get(), k,
        reinterpret_cast<uint32_t*>(tsamp.get()));
    EVOC_CHECK_LAUNCH();
    const int64_t chunk = std::min<int64_t>(k, PREDICT_CHUNK);
    for (int64_t r0 = 0; r0 < k; r0 += chunk) {
      const int64_t rows = std::min(chunk, k - r0);
      forward(net, xs_s.get() + r0 * net->in, rows, sp, false, pred.get() + r0 * d);
    }
    EVOC_CUDA(cudaMemcpyAsync(hp.data(), pred.get(), (size_t)k * d * sizeof(float),
                              cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaMemcpyAsync(ht.data(), tsamp.get(), (size_t)k * d * sizeof(float),
                              cudaMemcpyDeviceToHost, s));
    EVOC_CUDA(cudaStreamSynchronize(s));
    std::vector<double> tm(d, 0.0), pm(d, 0.0), mm((size_t)d * d, 0.0), rr((size_t)d * d);
    for (int64_t r = 0; r < k; ++r)
      for (int j = 0; j < d; ++j) {
        tm[j] += ht[(size_t)r * d + j];
        pm[j] += hp[(size_t)r * d + j];
      }
    for (int j = 0; j < d; ++j) {
      tm[j] /= (double)k;
      pm[j] /= (double)k;
    }
    for (int64_t r = 0; r < k; ++r)
      for (int a = 0; a < d; ++a) {
        const double ta = ht[(size_t)r * d + a] - tm[a];
        for (int b = 0; b < d; ++b) mm[(size_t)a * d + b] += ta * (hp[(size_t)r * d + b] - pm[b]);
      }
    procrustes(mm.data(), d, rr.data());
    for (int j = 0; j < d * d; ++j) haff[j] = (float)rr[j];
    for (int j = 0; j < d; ++j) {
      haff[(size_t)d * d + j] = (float)tm[j];
      haff[(size_t)d * d + d + j] = (float)pm[j];
    }
    check_status(net->ctx, "evoc_mlp_fit_device (alignment)");
    EVOC_CUDA(cudaMemcpyAsync(aff.get(), haff.data(), haff.size() * sizeof(float),
                              cudaMemcpyHostToDevice, s));
    k_affine_rows<<<blocks_for(ns[i], 256), 256, 0, s>>>(layouts[i], ns[i], d, aff.get(),
                                                         aligned[i].get());
    EVOC_CHECK_LAUNCH();
    EVOC_CUDA(cudaStreamSynchronize(s));  // haff is reused by the next call
  };

  for (int32_t step = 0; step < p->steps; ++step) {
    if (step % p->align_every == 0)
      for (int32_t i = 0; i < m; ++i) realign(i);
    const int32_t i = step % m;
    k_sample_rows<<<blocks_for(batch, 256), 256, 0, s>>>(sc.rows.get(), batch, (uint32_t)ns[i],
                                                         p->seed, (uint32_t)step);
    EVOC_CHECK_LAUNCH();
    k_gather_rows<<<blocks_for(batch * net->in / 2, 256), 256, 0, s>>>(
        reinterpret_cast<const uint32_t*>(xs[i]), net->in / 2, sc.rows.get(), batch,
        reinterpret_cast<uint32_t*>(sc.x.get()));
    EVOC_CHECK_LAUNCH();
    k_gather_rows<<<blocks_for(batch * d, 256), 256, 0, s>>>(
        reinterpret_cast<const uint32_t*>(aligned[i].get()), d, sc.rows.get(), batch,
        reinterpret_cast<uint32_t*>(sc.target.get()));
    EVOC_CHECK_LAUNCH();
    forward_backward(net, batch, sc, losses.get() + step);
    const double frac = p->steps > 1 ? (double)step / (double)(p->steps - 1) : 0.0;
    const float lr = (float)((double)p->lr + ((double)p->lr_end - (double)p->lr) * frac);
    adam_step(net, lr, p->beta1, p->beta2, p->eps);
  }
  if (loss_history && p->steps > 0)
    EVOC_CUDA(cudaMemcpyAsync(loss_history, losses.get(), (size_t)p->steps * sizeof(float),
                              cudaMemcpyDeviceToHost, s));
  check_status(net->ctx, "evoc_mlp_fit_device");
}

}  // namespace evoc
