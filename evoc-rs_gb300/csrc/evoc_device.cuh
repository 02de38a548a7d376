// evoc_device.cuh — device arithmetic shared by the EVoC kernels.
//
// Every floating-point expression that mirrors the reference's Rust arithmetic
// uses the explicitly rounded intrinsics (__fadd_rn, __fmul_rn, __fdiv_rn,
// __fsqrt_rn) so that nvcc cannot contract a multiply and an add into one FMA:
// Rust evaluates `a * b + c` with two roundings.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace evoc {

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

// Packed pairs: one sm_100-family f32x2 instruction performs two IEEE
// round-to-nearest operations (subnormals kept), the same results as two
// fadd / fsub / fmul.
__device__ __forceinline__ unsigned long long pack2(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 unpack2(unsigned long long r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
__device__ __forceinline__ float2 fadd2(float2 a, float2 b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
  return unpack2(r);
}
__device__ __forceinline__ float2 fsub2(float2 a, float2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
  return unpack2(r);
}
__device__ __forceinline__ float2 fmul2(float2 a, float2 b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
  return unpack2(r);
}

// max(a, 0) with NaN -> 0, the result of Rust's f32::max(a, 0.0).
__device__ __forceinline__ float max0(float a) { return (a > 0.0f) ? a : 0.0f; }

// 2^k for -126 <= k <= 127, built from the exponent field.
__device__ __forceinline__ float pow2i(int k) {
  return __uint_as_float((uint32_t)(k + 127) << 23);
}

// exp(x): Cody-Waite reduction x = k*ln2 + r (|r| <= ln2/2) with ln2 split
// into a 15-bit head (so k*ln2_hi is exact) and a tail, then the degree-7
// Taylor polynomial of e^r in Horner form, then scaling by 2^k (two steps
// below the normal range). Maximum error about 1 ulp against the true value.
__device__ __forceinline__ float evoc_expf(float x) {
  if (x != x) return x;
  if (x < -104.0f) return 0.0f;
  if (x > 88.72f) return __int_as_float(0x7f800000);
  const float log2e = 1.44269502f;
  const float ln2_hi = 0.693145751953125f;
  const float ln2_lo = 1.42860677e-06f;
  float kf = rintf(fmul(x, log2e));
  float r = fsub(x, fmul(kf, ln2_hi));
  r = fsub(r, fmul(kf, ln2_lo));
  float p = 1.98412701e-04f;           // 1/5040
  p = fadd(fmul(p, r), 1.38888892e-03f); // 1/720
  p = fadd(fmul(p, r), 8.33333377e-03f); // 1/120
  p = fadd(fmul(p, r), 4.16666679e-02f); // 1/24
  p = fadd(fmul(p, r), 1.66666672e-01f); // 1/6
  p = fadd(fmul(p, r), 0.5f);
  p = fadd(fmul(p, r), 1.0f);
  p = fadd(fmul(p, r), 1.0f);
  int k = (int)kf;
  if (k >= -126) return fmul(p, pow2i(k));
  return fmul(fmul(p, pow2i(k + 64)), pow2i(-64));
}

// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC 2011).
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c.x;
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

// Negative sample j of edge `eidx` at `epoch`, uniform in [0, n).
__device__ __forceinline__ uint32_t negative_draw(uint64_t seed, uint32_t j,
                                                  uint32_t epoch, uint64_t eidx,
                                                  uint32_t n) {
  uint4 o = philox4x32_10(
      make_uint4(j, epoch, (uint32_t)eidx, (uint32_t)(eidx >> 32) & 0x7fffffffu),
      make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
  return __umulhi(o.x, n);
}

// Initial coordinate `idx` (row-major n*dim) of the random initialisation:
// uniform in [-0.25, 0.25) from 53 random bits, rounded to f32.
__device__ __forceinline__ float init_value(uint64_t seed, uint64_t idx) {
  uint4 o = philox4x32_10(
      make_uint4((uint32_t)idx, (uint32_t)(idx >> 32), 0u, 0x80000000u | 0x494E4954u),
      make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
  uint64_t bits = ((((uint64_t)o.y) << 32) | o.x) >> 11;
  double u = (double)bits * (1.0 / 9007199254740992.0);
  return (float)__dadd_rn(-0.25, __dmul_rn(0.5, u));
}

// num-traits ToPrimitive::to_usize(f32) followed by unwrap_or(0).
__device__ __forceinline__ uint64_t to_usize_or0(float x) {
  return (x > -1.0f && x < 18446744073709551616.0f) ? (uint64_t)x : 0ull;
}

__device__ __forceinline__ void set_status(int32_t* status, int32_t bit) {
  atomicOr(status, bit);
}

}  // namespace evoc
