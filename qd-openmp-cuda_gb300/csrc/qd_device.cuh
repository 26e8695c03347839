// Device helpers shared by the kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <algorithm>

namespace qd {

__host__ __device__ inline double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ inline double2 ldg2(const double2 *p) { return __ldg(p); }

inline unsigned grid_for(int64_t n, int threads, int max_blocks = 152 * 16) {
  int64_t b = (n + threads - 1) / threads;
  if (b > max_blocks) b = max_blocks;
  if (b < 1) b = 1;
  return (unsigned)b;
}

// Division by a runtime divisor d with a precomputed magic number
// (round-up method): q = (t + ((x - t) >> 1)) >> (s - 1), t = umulhi(x, m),
// exact for every 32-bit x.  Replaces the long integer-division sequences in
// index arithmetic.
struct FastDiv {
  uint32_t d, m, s;
};
inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f{d, 0u, 0u};
  if (d <= 1) return f;
  uint32_t s = 0;
  while ((1ull << s) < d) s++;
  f.s = s;
  f.m = (uint32_t)(((((uint64_t)1 << 32) * (((uint64_t)1 << s) - d)) / d) + 1);
  return f;
}
__device__ inline uint32_t fdiv(const FastDiv &f, uint32_t x) {
  if (f.d <= 1) return x;
  const uint32_t t = __umulhi(x, f.m);
  return (t + ((x - t) >> 1)) >> (f.s - 1);
}

// FP64 <-> FP32 conversion with integer instructions.  On GB300 the F2F
// conversion instructions issue on the FP64 pipe (1/58 of the FP32 rate), so
// kernels that compute in FP32 on FP64 storage convert with bit operations:
//   d2f_rn: round to nearest even; |x| < 2^-126 -> signed zero; overflow -> inf;
//           NaN -> NaN.
//   f2d:    exact; FP32 subnormals -> signed zero.
__device__ inline float d2f_rn(double x) {
  const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
  const uint32_t sign = hi & 0x80000000u;
  const uint32_t ef = (hi >> 20) & 0x7ffu;
  if (ef == 0x7ffu) return __uint_as_float(sign | 0x7f800000u | ((hi & 0xfffffu) | lo ? 0x400000u : 0u));
  const int e = (int)ef - 896;   // rebias 1023 -> 127
  if (e <= 0) return __uint_as_float(sign);
  if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
  uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29);
  const uint32_t rem = lo & 0x1fffffffu;
  m += (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u;
  return __uint_as_float(sign | (((uint32_t)e << 23) + m));   // a mantissa carry rounds up the exponent
}

__device__ inline double f2d(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t sign = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  if (e == 0u) return __hiloint2double((int)sign, 0);
  if (e == 0xffu) return __hiloint2double((int)(sign | 0x7ff00000u | (m >> 3) | (m ? 0x80000u : 0u)), 0);
  return __hiloint2double((int)(sign | ((e + 896u) << 20) | (m >> 3)), (int)(m << 29));
}

// psi_j element access for either storage: c128 (FP64 form) or c64 (mixed
// form, one round-to-nearest on store)
__device__ inline double2 load_c(const double2 *p) { return *p; }
__device__ inline double2 load_c(const float2 *p) {
  const float2 v = *p;
  return make_double2(f2d(v.x), f2d(v.y));
}
__device__ inline void store_c(double2 *p, double2 v) { *p = v; }
__device__ inline void store_c(float2 *p, double2 v) { *p = make_float2(d2f_rn(v.x), d2f_rn(v.y)); }

// Deterministic block-wide sum (fixed shuffle tree then fixed smem tree);
// every thread gets the result.  red must hold 32 doubles; all threads call.
__device__ inline double block_sum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (warp == 0) {
    s = lane < nw ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) red[0] = s;
  }
  __syncthreads();
  s = red[0];
  __syncthreads();
  return s;
}

}  // namespace qd
