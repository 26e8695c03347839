// Coriolis coupling across Omega blocks, in place in HBM.
//
// Reference: for every ordered pair of blocks (Omega, Omega1) and every l, the
// kernel _evolution_with_coriolis_ (evolutionCUDAaux.cu:178-209) accumulates
//   psi_out^Omega_l(R, r) += U_{Omega Omega1}(R) psi^Omega1_l(R, r),
//   U(R) = sum_a exp(-i dt e_a/(2 m1 R^2)) V[Omega,a] V[Omega1,a],
// into a zeroed scratch (omegawavepacket.cu:555-564) that is then copied back
// (omegawavepacket.cu:479-489); (e, V) diagonalise the tridiagonal Omega matrix
// of each l (CoriolisMatrix.C:63-99).  That is the exact exponential of the
// matrix, dense in Omega.  Here one thread owns one (l, R, r) point of one
// problem, loads the whole Omega column, applies U = V diag(phase(R)) V^T as
// two real n x n products around the diagonal phase, and writes the column
// back in place: no scratch, no memset, no copy, one read and one write.
// This file holds the phase tables, the FP32 kernel of the mixed form and the
// dispatch of the FP64 kernel, whose body is in qd_coriolis64.cuh.
// The coupling energy (omegawavepacket.cu:503-553) is evaluated on the
// pre-update values in the same pass: sum over |Omega-Omega1| <= 1 of
// conj(psi^Omega) H_{Omega Omega1}/(2 m1 R^2) psi^Omega1, doubled off the
// diagonal and attributed to the lower Omega.
#include "qd_internal.h"
#include "qd_device.cuh"

#include <type_traits>

namespace qd {

int coriolis_tiles(const Grid &g) { return (int)((g.npt + CORIOLIS_THREADS - 1) / CORIOLIS_THREADS); }

__global__ void k_build_coriolis_phase(Grid g, const CoriolisGroup *__restrict__ groups, const double *__restrict__ e,
                                       double dt, double2 *__restrict__ ph) {
  const CoriolisGroup gr = groups[blockIdx.y];
  const int64_t n = (int64_t)gr.n * g.n1;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(q / g.n1), i = (int)(q % g.n1);
    const double R = g.left1 + i * g.dr1;
    const double I = 2 * g.m1 * R * R;
    double s, c;
    sincos(dt * e[gr.e0 + a] / I, &s, &c);
    ph[gr.ph0 + q] = make_double2(c, -s);
  }
}

void launch_build_coriolis_phase(cudaStream_t s, const Grid &g, const CoriolisGroup *groups, int n_groups, int,
                                 const double *e, double dt, double2 *ph) {
  if (n_groups == 0) return;
  k_build_coriolis_phase<<<dim3(4, n_groups), 256, 0, s>>>(g, groups, e, dt, ph);
}

// ------------------------------------------------------------ mixed form
// Same operator in FP32 arithmetic on the c64 pool, for up to 24 coupled
// Omega blocks.  The eigenvectors are held as FP32 pairs V = Vh + Vl (the
// pair carries V to ~2^-48), so the applied U stays unitary to FP64 level and
// the per-step rounding is random rather than a fixed bias; the phases
// exp(-i dt e_a/(2 m1 R^2)) and the rotational phases before/after are
// three-shear rotations of determinant exactly 1.  Each CTA walks a strided
// 1/tiles of the points of one group (one l), so the coupling and rotational
// energy partials are [group][omega][tiles] and [slab][tiles].
namespace {
__device__ inline void lift2c(float2 &v, float2 ts) {
  float x = v.x, y = v.y;
  x = fmaf(ts.x, y, x);
  y = fmaf(ts.y, x, y);
  x = fmaf(ts.x, y, x);
  x = fmaf(ts.x, y, x);
  y = fmaf(ts.y, x, y);
  x = fmaf(ts.x, y, x);
  v.x = x;
  v.y = y;
}
// Two (hi, lo) eigenvector pairs in one 16-byte shared-memory load.  The load
// is volatile so that it stays inside the point loop: V held in registers
// across the loop would leave room for only a few warps.
__device__ __forceinline__ float4 lds_pair2(const float *p) {
  float4 v;
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a));
  return v;
}
}  // namespace

template <int MAXN, bool EN>
__device__ __forceinline__ void coriolis_f32_body(const Grid &g, float2 *__restrict__ psi_j,
                                                              const BlockDesc *__restrict__ blocks,
                                                              const CoriolisGroup *__restrict__ groups,
                                                              const float *__restrict__ Vh, const float *__restrict__ Vl,
                                                              const float2 *__restrict__ phl, const double *__restrict__ Hp,
                                                              const float2 *__restrict__ rotR, const float2 *__restrict__ rotr,
                                                              int pro, int epi, const float *__restrict__ I1f,
                                                              const float *__restrict__ I2f, double *__restrict__ ce_part,
                                                              double *__restrict__ re_part, int tiles, int ce_n,
                                                              int gid, float *sV, float *Hd, float *Ho,
                                                              float (*red)[2 * CORIOLIS_F32_MAXN], int64_t *base) {
  const CoriolisGroup gr = groups[gid];
  const int n = gr.n, l = gr.l;
  // sV[(o MAXN + a) 2 + {0, 1}] = (Vh, Vl)[o][a], zero outside n x n: row
  // stride MAXN makes every offset below a compile-time constant, and the
  // zero padding lets the products run over whole pairs of a
  for (int q = threadIdx.x; q < MAXN * MAXN; q += blockDim.x) {
    const int o = q / MAXN, a = q % MAXN;
    const bool in = o < n && a < n;
    sV[2 * q] = in ? Vh[gr.v0 + o * n + a] : 0.0f;
    sV[2 * q + 1] = in ? Vl[gr.v0 + o * n + a] : 0.0f;
  }
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    Hd[q] = (float)Hp[gr.h0 + q * n + q];
    Ho[q] = q + 1 < n ? (float)Hp[gr.h0 + q * n + q + 1] : 0.0f;
  }
  for (int o = threadIdx.x; o < n; o += blockDim.x) {   // slab offset of each member block
    const BlockDesc bd = blocks[gr.block_lo + o];
    base[o] = (int64_t)(bd.slab0 + (l - bd.omega)) * g.npt;
  }
  __syncthreads();
  const float ll = (float)l * (float)(l + 1);
  constexpr int NE = EN ? MAXN : 1;   // energy accumulators only in the energy variant
  float ce[NE], re[NE];
#pragma unroll
  for (int o = 0; o < NE; o++) ce[o] = re[o] = 0.0f;
  for (int64_t pt = (int64_t)blockIdx.x * CORIOLIS_THREADS + threadIdx.x; pt < g.npt;
       pt += (int64_t)tiles * CORIOLIS_THREADS) {
    const int i = (int)(pt % g.n1), j = (int)(pt / g.n1);
    float2 x[MAXN];
#pragma unroll
    for (int o = 0; o < MAXN; o++) x[o] = o < n ? psi_j[base[o] + pt] : make_float2(0.0f, 0.0f);
    float2 tR = make_float2(0.0f, 0.0f), tr = make_float2(0.0f, 0.0f);
    if (pro || epi) {
      tR = __ldg(rotR + (int64_t)l * g.n1 + i);
      tr = __ldg(rotr + (int64_t)l * g.n2 + j);
    }
    if (pro) {
#pragma unroll
      for (int o = 0; o < MAXN; o++)
        if (o < n) {
          lift2c(x[o], tR);
          lift2c(x[o], tr);
        }
    }
    const float inv1 = __ldg(I1f + i);
    if (EN) {   // coupling energy of the incoming state
#pragma unroll
      for (int o = 0; o < NE; o++)
        if (o < n) {
          float c = Hd[o] * (x[o].x * x[o].x + x[o].y * x[o].y);
          if (o + 1 < n) c = fmaf(2.0f * Ho[o], x[o].x * x[o + 1].x + x[o].y * x[o + 1].y, c);
          ce[o] = fmaf(inv1, c, ce[o]);
        }
    }
    // y = V^T x: one pass over the members o, every a accumulating independently;
    // V is re-read from shared memory per point, two elements per load
    float2 y[MAXN];
#pragma unroll
    for (int a = 0; a < MAXN; a++) y[a] = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int o = 0; o < MAXN; o++) {
      if (o < n) {
#pragma unroll
        for (int a = 0; a < MAXN; a += 2)
          if (a < n) {
            const float4 v = lds_pair2(sV + 2 * (o * MAXN + a));
            y[a].x = fmaf(v.y, x[o].x, fmaf(v.x, x[o].x, y[a].x));
            y[a].y = fmaf(v.y, x[o].y, fmaf(v.x, x[o].y, y[a].y));
            y[a + 1].x = fmaf(v.w, x[o].x, fmaf(v.z, x[o].x, y[a + 1].x));
            y[a + 1].y = fmaf(v.w, x[o].y, fmaf(v.z, x[o].y, y[a + 1].y));
          }
      }
    }
#pragma unroll
    for (int a = 0; a < MAXN; a++)
      if (a < n) lift2c(y[a], __ldg(phl + gr.ph0 + (int64_t)a * g.n1 + i));
    // x = V y, each x[o] summed over a in ascending order (y beyond n is zero)
#pragma unroll
    for (int o = 0; o < MAXN; o++) {
      float2 acc = make_float2(0.0f, 0.0f);
      if (o < n) {
#pragma unroll
        for (int a = 0; a < MAXN; a += 2)
          if (a < n) {
            const float4 v = lds_pair2(sV + 2 * (o * MAXN + a));
            acc.x = fmaf(v.y, y[a].x, fmaf(v.x, y[a].x, acc.x));
            acc.y = fmaf(v.y, y[a].y, fmaf(v.x, y[a].y, acc.y));
            acc.x = fmaf(v.w, y[a + 1].x, fmaf(v.z, y[a + 1].x, acc.x));
            acc.y = fmaf(v.w, y[a + 1].y, fmaf(v.z, y[a + 1].y, acc.y));
          }
      }
      x[o] = acc;
    }
    const float rI = ll * (inv1 + __ldg(I2f + j));
#pragma unroll
    for (int o = 0; o < MAXN; o++) {
      if (o < n) {
        float2 v = x[o];
        if (epi) {
          lift2c(v, tR);
          lift2c(v, tr);
        }
        if constexpr (EN) re[o] = fmaf(rI, v.x * v.x + v.y * v.y, re[o]);
        psi_j[base[o] + pt] = v;
      }
    }
  }
  if constexpr (!EN) return;
  // per-Omega partials: shuffle tree per warp, then the warps in a fixed order
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 0; o < NE; o++) {
    if (o < n) {
      float c = ce[o], r = re[o];
      for (int s = 16; s > 0; s >>= 1) {
        c += __shfl_down_sync(0xffffffffu, c, s);
        r += __shfl_down_sync(0xffffffffu, r, s);
      }
      if (lane == 0) {
        red[warp][o] = c;
        red[warp][CORIOLIS_F32_MAXN + o] = r;
      }
    }
  }
  __syncthreads();
  for (int o = threadIdx.x; o < n; o += blockDim.x) {
    double c = 0.0, r = 0.0;
    for (int w = 0; w < CORIOLIS_THREADS / 32; w++) {
      c += (double)red[w][o];
      r += (double)red[w][CORIOLIS_F32_MAXN + o];
    }
    if (ce_part) ce_part[((int64_t)gid * ce_n + o) * tiles + blockIdx.x] = c;
    if (re_part) {
      const BlockDesc bd = blocks[gr.block_lo + o];
      re_part[(int64_t)(bd.slab0 + (l - bd.omega)) * tiles + blockIdx.x] = r;
    }
  }
}

int coriolis_f32_class(int n) {
  for (int c = 0; c < CORIOLIS_F32_CLASSES; c++)
    if (n <= CORIOLIS_F32_STEP * (c + 1)) return c;
  return -1;
}

// One launch for every group: each CTA runs the body compiled for its
// group's size class (at most 4, 8, ..., 24 blocks), so small groups
// do not pay for the largest one's unrolled loops.
template <int MAXC, bool EN>
__global__ void __launch_bounds__(CORIOLIS_THREADS) k_coriolis_f32(Grid g, float2 *__restrict__ psi_j,
                                                              const BlockDesc *__restrict__ blocks,
                                                              const CoriolisGroup *__restrict__ groups,
                                                              const float *__restrict__ Vh, const float *__restrict__ Vl,
                                                              const float2 *__restrict__ phl, const double *__restrict__ Hp,
                                                              const float2 *__restrict__ rotR, const float2 *__restrict__ rotr,
                                                              int pro, int epi, const float *__restrict__ I1f,
                                                              const float *__restrict__ I2f, double *__restrict__ ce_part,
                                                              double *__restrict__ re_part, int tiles, int ce_n,
                                                              const int *__restrict__ order, const int *status) {
  if (status && *status) return;
  constexpr int MAXN = CORIOLIS_F32_STEP * (MAXC + 1);
  __shared__ __align__(16) float sV[2 * MAXN * MAXN];
  __shared__ float Hd[MAXN], Ho[MAXN];
  __shared__ float red[CORIOLIS_THREADS / 32][2 * CORIOLIS_F32_MAXN];
  __shared__ int64_t base[MAXN];
  const int gid = order[blockIdx.y];
  const int cls = (groups[gid].n + CORIOLIS_F32_STEP - 1) / CORIOLIS_F32_STEP - 1;
#define QD_BODY(C)                                                                                       \
  coriolis_f32_body<CORIOLIS_F32_STEP * ((C) + 1), EN>(g, psi_j, blocks, groups, Vh, Vl, phl, Hp, rotR, rotr, \
                                                       pro, epi, I1f, I2f, ce_part, re_part, tiles, ce_n, gid,  \
                                                       sV, Hd, Ho, red, base)
  if (MAXC >= 5 && cls == 5) QD_BODY(MAXC >= 5 ? 5 : 0);
  else if (MAXC >= 4 && cls == 4) QD_BODY(MAXC >= 4 ? 4 : 0);
  else if (MAXC >= 3 && cls == 3) QD_BODY(MAXC >= 3 ? 3 : 0);
  else if (MAXC >= 2 && cls == 2) QD_BODY(MAXC >= 2 ? 2 : 0);
  else if (MAXC >= 1 && cls == 1) QD_BODY(MAXC >= 1 ? 1 : 0);
  else QD_BODY(0);
#undef QD_BODY
}

void launch_coriolis_f32(cudaStream_t s, const Grid &g, float2 *psi_j, const BlockDesc *blocks,
                         const CoriolisGroup *groups, const int *order, int n_groups, int max_n, const float *Vh,
                         const float *Vl, const float2 *phl, const double *H, const float2 *rotR, const float2 *rotr,
                         bool pro, bool epi, const float *I1f, const float *I2f, double *ce_part, double *re_part,
                         int tiles, const int *status) {
  if (n_groups == 0) return;
  const dim3 grid((unsigned)tiles, (unsigned)n_groups);
#define QD_COR32(C)                                                                                         \
  do {                                                                                                      \
    if (ce_part)                                                                                            \
      k_coriolis_f32<C, true><<<grid, CORIOLIS_THREADS, 0, s>>>(g, psi_j, blocks, groups, Vh, Vl, phl, H,    \
                                                                rotR, rotr, pro ? 1 : 0, epi ? 1 : 0, I1f, \
                                                                I2f, ce_part, re_part, tiles, max_n, order, \
                                                                status);                                   \
    else                                                                                                    \
      k_coriolis_f32<C, false><<<grid, CORIOLIS_THREADS, 0, s>>>(g, psi_j, blocks, groups, Vh, Vl, phl, H,   \
                                                                 rotR, rotr, pro ? 1 : 0, epi ? 1 : 0, I1f, \
                                                                 I2f, nullptr, nullptr, tiles, max_n, order, \
                                                                 status);                                   \
  } while (0)
  switch (coriolis_f32_class(max_n)) {
    case 0: QD_COR32(0); break;
    case 1: QD_COR32(1); break;
    case 2: QD_COR32(2); break;
    case 3: QD_COR32(3); break;
    case 4: QD_COR32(4); break;
    case 5: QD_COR32(5); break;
    default: throw Error{QD_ERR_UNSUPPORTED, "FP32 Coriolis: more than 24 coupled Omega blocks"};
  }
#undef QD_COR32
}

// half-step phase exp(-i dt e_a / (2 m1 R^2)) of every group as three-shear
// coefficients (applied twice), [ph0 + a n1 + i]
__global__ void k_build_coriolis_lift(Grid g, const CoriolisGroup *__restrict__ groups, const double *__restrict__ e,
                                      double dt, float2 *__restrict__ phl) {
  const CoriolisGroup gr = groups[blockIdx.y];
  const int64_t n = (int64_t)gr.n * g.n1;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(q / g.n1), i = (int)(q % g.n1);
    const double R = g.left1 + i * g.dr1;
    const double ang = -dt * e[gr.e0 + a] / (2 * g.m1 * R * R);
    const double r = remainder(ang, 2.0 * M_PI);
    const double h = 0.5 * r;
    phl[gr.ph0 + q] = make_float2((float)(-tan(0.5 * h)), (float)sin(h));
  }
}

void launch_build_coriolis_lift(cudaStream_t s, const Grid &g, const CoriolisGroup *groups, int n_groups,
                                const double *e, double dt, float2 *phl) {
  if (n_groups == 0) return;
  k_build_coriolis_lift<<<dim3(4, n_groups), 256, 0, s>>>(g, groups, e, dt, phl);
}

template <typename S>
void launch_coriolis(cudaStream_t s, const Grid &g, S *psi_j, const BlockDesc *blocks,
                     const CoriolisGroup *groups, int n_groups, int max_n, const double *V, const double2 *ph,
                     const double *H, double *ce_part, int ce_tiles, const double2 *tabE, const int *status,
                     const double2 *tabP) {
  if (n_groups == 0) return;
#define QD_COR(M) \
  launch_coriolis_n<M, S>(s, g, psi_j, blocks, groups, n_groups, max_n, V, ph, H, ce_part, ce_tiles, tabE, status, tabP)
  if (max_n > 48) throw Error{QD_ERR_UNSUPPORTED, "more than 48 coupled Omega blocks"};
  if constexpr (std::is_same<S, float2>::value) {
    // the mixed form uses this kernel only above the FP32 kernel's 24 blocks
    if (max_n <= 32) QD_COR(32);
    else QD_COR(48);
  } else {
    if (max_n <= 2) QD_COR(2);
    else if (max_n <= 4) QD_COR(4);
    else if (max_n <= 8) QD_COR(8);
    else if (max_n <= 16) QD_COR(16);
    else if (max_n <= 24) QD_COR(24);
    else if (max_n <= 32) QD_COR(32);
    else QD_COR(48);
  }
#undef QD_COR
}
template void launch_coriolis<double2>(cudaStream_t, const Grid &, double2 *, const BlockDesc *,
                                       const CoriolisGroup *, int, int, const double *, const double2 *,
                                       const double *, double *, int, const double2 *, const int *, const double2 *);
template void launch_coriolis<float2>(cudaStream_t, const Grid &, float2 *, const BlockDesc *, const CoriolisGroup *,
                                      int, int, const double *, const double2 *, const double *, double *, int,
                                      const double2 *, const int *, const double2 *);

}  // namespace qd
