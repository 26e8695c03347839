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
// The coupling energy (omegawavepacket.cu:503-553) is evaluated on the
// pre-update values in the same pass: sum over |Omega-Omega1| <= 1 of
// conj(psi^Omega) H_{Omega Omega1}/(2 m1 R^2) psi^Omega1, doubled off the
// diagonal and attributed to the lower Omega.
#include "qd_internal.h"
#include "qd_device.cuh"

namespace qd {

namespace {
constexpr int COR_THREADS = 128;
}

int coriolis_tiles(const Grid &g) { return (int)((g.npt + COR_THREADS - 1) / COR_THREADS); }

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

template <int MAXN, typename S>
__global__ void __launch_bounds__(COR_THREADS) k_coriolis(Grid g, S *__restrict__ psi_j,
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
  const int64_t pt = (int64_t)blockIdx.x * COR_THREADS + threadIdx.x;
  const bool active = pt < g.npt;
  const int i = active ? (int)(pt % g.n1) : 0;
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
#pragma unroll
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
#pragma unroll
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
#pragma unroll
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

template <typename S>
void launch_coriolis(cudaStream_t s, const Grid &g, S *psi_j, const BlockDesc *blocks,
                     const CoriolisGroup *groups, int n_groups, int max_n, const double *V, const double2 *ph,
                     const double *H, double *ce_part, int ce_tiles, const double2 *tabE, const int *status,
                     const double2 *tabP) {
  if (n_groups == 0) return;
  dim3 grid((unsigned)coriolis_tiles(g), (unsigned)n_groups);
#define QD_COR(M)                                                                                        \
  k_coriolis<M, S><<<grid, COR_THREADS, 0, s>>>(g, psi_j, blocks, groups, V, ph, H, ce_part, ce_tiles, max_n, \
                                             tabE, status, tabP)
  if (max_n <= 2) QD_COR(2);
  else if (max_n <= 4) QD_COR(4);
  else if (max_n <= 8) QD_COR(8);
  else if (max_n <= 16) QD_COR(16);
  else if (max_n <= 24) QD_COR(24);
  else if (max_n <= 32) QD_COR(32);
  else if (max_n <= 48) QD_COR(48);
  else throw Error{QD_ERR_UNSUPPORTED, "more than 48 coupled Omega blocks"};
#undef QD_COR
}
template void launch_coriolis<double2>(cudaStream_t, const Grid &, double2 *, const BlockDesc *,
                                       const CoriolisGroup *, int, int, const double *, const double2 *,
                                       const double *, double *, int, const double2 *, const int *, const double2 *);
template void launch_coriolis<float2>(cudaStream_t, const Grid &, float2 *, const BlockDesc *, const CoriolisGroup *,
                                      int, int, const double *, const double2 *, const double *, double *, int,
                                      const double2 *, const int *, const double2 *);

}  // namespace qd
