// FP64 Coriolis kernel, instantiated per group-size bound MAXN in the
// k_coriolis_fp64_*.cu translation units so that the large, fully unrolled
// bodies compile in parallel; launch_coriolis in k_coriolis.cu dispatches.
//
// One thread owns one (l, R, r) point of one group, loads the whole Omega
// column, applies U = V diag(phase(R)) V^T as two real n x n products around
// the diagonal phase, and writes the column back in place (reference:
// _evolution_with_coriolis_, evolutionCUDAaux.cu:178-209, exponential of the
// tridiagonal Omega matrix of CoriolisMatrix.C:63-99).  The coupling energy
// (omegawavepacket.cu:503-553) is evaluated on the incoming values in the
// same pass.  Storage S is double2 (FP64 form) or float2 (mixed form above
// the FP32 kernel's limit); the arithmetic is FP64 either way.
#pragma once
#include "qd_internal.h"
#include "qd_device.cuh"

#include <type_traits>

namespace qd {

template <int MAXN, typename S>
__global__ void __launch_bounds__(CORIOLIS_THREADS) k_coriolis(Grid g, S *__restrict__ psi_j,
                                                          const BlockDesc *__restrict__ blocks,
                                                          const CoriolisGroup *__restrict__ groups,
                                                          const double *__restrict__ Vp, const double2 *__restrict__ php,
                                                          const double *__restrict__ Hp, double *__restrict__ ce_part,
                                                          int ce_tiles, int ce_n, const double2 *__restrict__ tabE,
                                                          const int *status, const double2 *__restrict__ tabP) {
  if (status && *status) return;
  __shared__ double Vs[MAXN * MAXN];
  __shared__ double Hd[MAXN], Ho[MAXN];
  __shared__ double red[32];
  const CoriolisGroup gr = groups[blockIdx.y];
  const int n = gr.n;
  for (int q = threadIdx.x; q < n * n; q += blockDim.x) Vs[q] = Vp[gr.v0 + q];
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    Hd[q] = Hp[gr.h0 + q * n + q];
    Ho[q] = q + 1 < n ? Hp[gr.h0 + q * n + q + 1] : 0.0;
  }
  __syncthreads();
  const int64_t pt = (int64_t)blockIdx.x * CORIOLIS_THREADS + threadIdx.x;
  const bool active = pt < g.npt;
  const int i = active ? (int)(pt % g.n1) : 0;
  // ptxas takes minutes over the fully unrolled 48-block body with complex64
  // storage; that variant keeps its outer loops rolled (its state spills anyway)
  constexpr int OUTER = (MAXN > 32 && std::is_same<S, float2>::value) ? 1 : MAXN;
  double2 x[MAXN];
  int64_t addr[MAXN];
#pragma unroll
  for (int o = 0; o < MAXN; o++) {
    if (o < n) {
      const BlockDesc bd = blocks[gr.block_lo + o];
      addr[o] = (int64_t)(bd.slab0 + (gr.l - bd.omega)) * g.npt + pt;
      x[o] = active ? load_c(psi_j + addr[o]) : make_double2(0.0, 0.0);
      if (tabP && active) x[o] = cmul(x[o], ldg2(tabP + (int64_t)gr.l * g.npt + pt));
    }
  }
  if (ce_part) {
    const double R = g.left1 + i * g.dr1;
    const double inv = 1.0 / (2 * g.m1 * R * R);
#pragma unroll OUTER
    for (int o = 0; o < MAXN; o++) {
      if (o < n) {
        double c = Hd[o] * inv * (x[o].x * x[o].x + x[o].y * x[o].y);
        if (o + 1 < n) c += 2.0 * Ho[o] * inv * (x[o].x * x[o + 1].x + x[o].y * x[o + 1].y);
        c = block_sum(active ? c : 0.0, red);
        if (threadIdx.x == 0)
          ce_part[((int64_t)blockIdx.y * ce_n + o) * ce_tiles + blockIdx.x] = c;
      }
    }
  }
  double2 y[MAXN];
#pragma unroll OUTER
  for (int a = 0; a < MAXN; a++) {
    if (a < n) {
      double2 acc = make_double2(0.0, 0.0);
#pragma unroll
      for (int o = 0; o < MAXN; o++)
        if (o < n) {
          const double v = Vs[o * n + a];
          acc.x = fma(v, x[o].x, acc.x);
          acc.y = fma(v, x[o].y, acc.y);
        }
      y[a] = cmul(acc, ldg2(php + gr.ph0 + (int64_t)a * g.n1 + i));
    }
  }
  if (!active) return;
#pragma unroll OUTER
  for (int o = 0; o < MAXN; o++) {
    if (o < n) {
      double2 acc = make_double2(0.0, 0.0);
#pragma unroll
      for (int a = 0; a < MAXN; a++)
        if (a < n) {
          const double v = Vs[o * n + a];
          acc.x = fma(v, y[a].x, acc.x);
          acc.y = fma(v, y[a].y, acc.y);
        }
      if (tabE) acc = cmul(acc, ldg2(tabE + (int64_t)gr.l * g.npt + pt));
      store_c(psi_j + addr[o], acc);
    }
  }
}

template <int MAXN, typename S>
void launch_coriolis_n(cudaStream_t s, const Grid &g, S *psi_j, const BlockDesc *blocks, const CoriolisGroup *groups,
                       int n_groups, int max_n, const double *V, const double2 *ph, const double *H, double *ce_part,
                       int ce_tiles, const double2 *tabE, const int *status, const double2 *tabP) {
  const dim3 grid((unsigned)coriolis_tiles(g), (unsigned)n_groups);
  k_coriolis<MAXN, S><<<grid, CORIOLIS_THREADS, 0, s>>>(g, psi_j, blocks, groups, V, ph, H, ce_part, ce_tiles, max_n,
                                                        tabE, status, tabP);
}

#define QD_CORIOLIS_N(M, S)                                                                                     \
  template void launch_coriolis_n<M, S>(cudaStream_t, const Grid &, S *, const BlockDesc *, const CoriolisGroup *, \
                                        int, int, const double *, const double2 *, const double *, double *, int,  \
                                        const double2 *, const int *, const double2 *)

}  // namespace qd
