// FP64 theta <-> j Legendre contractions (SIMT DFMA).
//
// Reference: cublasZgemm with the real Legendre matrices stored as complex
// (omegawavepacket.cu:134-240), i.e. 4x the necessary flops.  Here the
// matrices stay real: C[pt][n] = sum_k A[pt][k] B[k][n] with complex A and real
// B, two real FMAs per term.  The theta-space phase (absorbing mask x
// exp(-iV dt), evolutionCUDAaux.cu:5-11,243-251) is applied while A is staged
// (forward), the rotational phase in the epilogue, and the backward epilogue
// reduces the module and potential energy (omegawavepacket.cu:76-132) from the
// values it stores.
#include "qd_internal.h"
#include "qd_device.cuh"

namespace qd {

namespace {
constexpr int BP = 64;   // points per CTA tile
constexpr int BN = 64;   // output columns per CTA tile
constexpr int BK = 16;   // contraction chunk
}

__global__ void __launch_bounds__(256) k_legendre_fwd_f64(Grid g, const double2 *__restrict__ psi_th,
                                                          double2 *__restrict__ psi_j, const double *__restrict__ Bf,
                                                          const BlockDesc *__restrict__ blocks,
                                                          const double2 *__restrict__ tabA,
                                                          const double2 *__restrict__ tabE, const int *status) {
  if (status && *status) return;
  __shared__ double2 As[BK][BP];
  __shared__ double Bs[BK][BN];
  const BlockDesc bd = blocks[blockIdx.z];
  const int K = g.nth;
  const int nl = bd.nl;
  const int n0 = blockIdx.y * BN;
  if (n0 >= nl) return;
  const int64_t pt0 = (int64_t)blockIdx.x * BP;
  const int tid = threadIdx.x, tm = tid & 15, tn = tid >> 4;
  const double2 *A = psi_th + (int64_t)blockIdx.z * K * g.npt;
  const double *B = Bf + bd.bmat0;

  double2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = make_double2(0.0, 0.0);

  for (int k0 = 0; k0 < K; k0 += BK) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int e = tid + 256 * r;
      const int kl = e / BP, pl = e % BP;
      const int k = k0 + kl;
      const int64_t pt = pt0 + pl;
      double2 v = make_double2(0.0, 0.0);
      if (k < K && pt < g.npt) {
        v = A[(int64_t)k * g.npt + pt];
        if (tabA) v = cmul(v, ldg2(tabA + (int64_t)k * g.npt + pt));
      }
      As[kl][pl] = v;
      const int nn = n0 + pl;
      Bs[kl][pl] = (k < K && nn < nl) ? __ldg(B + (int64_t)k * nl + nn) : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk++) {
      double2 a[4];
      double b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][tm + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tn + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
          acc[i][j].x = fma(a[i].x, b[j], acc[i][j].x);
          acc[i][j].y = fma(a[i].y, b[j], acc[i][j].y);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int n = n0 + tn + 16 * j;
    if (n >= nl) continue;
    const int l = bd.omega + n;
    double2 *C = psi_j + (int64_t)(bd.slab0 + n) * g.npt;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int64_t pt = pt0 + tm + 16 * i;
      if (pt >= g.npt) continue;
      double2 v = acc[i][j];
      if (tabE) v = cmul(v, ldg2(tabE + (int64_t)l * g.npt + pt));
      C[pt] = v;
    }
  }
}

void launch_legendre_fwd_f64(cudaStream_t s, const Grid &g, const double2 *psi_th, double2 *psi_j, const double *Bfwd,
                             const BlockDesc *blocks, int n_blocks, int max_nl, const double2 *tabA,
                             const double2 *tabE, const int *status) {
  dim3 grid((unsigned)((g.npt + BP - 1) / BP), (unsigned)((max_nl + BN - 1) / BN), (unsigned)n_blocks);
  k_legendre_fwd_f64<<<grid, 256, 0, s>>>(g, psi_th, psi_j, Bfwd, blocks, tabA, tabE, status);
}

int legendre_bwd_part_tiles(const Grid &g) {
  return (int)(((g.npt + BP - 1) / BP) * ((g.nth + BN - 1) / BN));
}

__global__ void __launch_bounds__(256) k_legendre_bwd_f64(Grid g, const double2 *__restrict__ psi_j,
                                                          double2 *__restrict__ psi_th, const double *__restrict__ Bb,
                                                          const BlockDesc *__restrict__ blocks,
                                                          const double2 *__restrict__ tabA,
                                                          const double *__restrict__ w, const double *__restrict__ pot,
                                                          double *__restrict__ part, int n_part_tiles,
                                                          const int *status) {
  if (status && *status) return;
  __shared__ double2 As[BK][BP];
  __shared__ double Bs[BK][BN];
  __shared__ double red[32];
  const BlockDesc bd = blocks[blockIdx.z];
  const int K = g.nth;       // output columns
  const int nl = bd.nl;      // contraction length
  const int k0 = blockIdx.y * BN;
  const int64_t pt0 = (int64_t)blockIdx.x * BP;
  const int tid = threadIdx.x, tm = tid & 15, tn = tid >> 4;
  const double *B = Bb + bd.bmat0;

  double2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = make_double2(0.0, 0.0);

  for (int c0 = 0; c0 < nl; c0 += BK) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int e = tid + 256 * r;
      const int cl = e / BP, pl = e % BP;
      const int c = c0 + cl;
      const int64_t pt = pt0 + pl;
      double2 v = make_double2(0.0, 0.0);
      if (c < nl && pt < g.npt) {
        v = psi_j[(int64_t)(bd.slab0 + c) * g.npt + pt];
        if (tabA) v = cmul(v, ldg2(tabA + (int64_t)(bd.omega + c) * g.npt + pt));
      }
      As[cl][pl] = v;
      const int kk = k0 + pl;
      Bs[cl][pl] = (c < nl && kk < K) ? __ldg(B + (int64_t)c * K + kk) : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int cc = 0; cc < BK; cc++) {
      double2 a[4];
      double b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[cc][tm + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[cc][tn + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
          acc[i][j].x = fma(a[i].x, b[j], acc[i][j].x);
          acc[i][j].y = fma(a[i].y, b[j], acc[i][j].y);
        }
    }
    __syncthreads();
  }
  double mod = 0.0, pe = 0.0;
  double2 *C = psi_th + (int64_t)blockIdx.z * K * g.npt;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int k = k0 + tn + 16 * j;
    if (k >= K) continue;
    const double wk = __ldg(w + k);
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int64_t pt = pt0 + tm + 16 * i;
      if (pt >= g.npt) continue;
      const double2 v = acc[i][j];
      C[(int64_t)k * g.npt + pt] = v;
      const double a2 = wk * (v.x * v.x + v.y * v.y);
      mod += a2;
      pe += a2 * __ldg(pot + (int64_t)k * g.npt + pt);
    }
  }
  mod = block_sum(mod, red);
  pe = block_sum(pe, red);
  if (tid == 0 && part) {
    const int64_t t = (int64_t)blockIdx.x + (int64_t)gridDim.x * blockIdx.y;
    part[((int64_t)blockIdx.z * n_part_tiles + t) * 2 + 0] = mod;
    part[((int64_t)blockIdx.z * n_part_tiles + t) * 2 + 1] = pe;
  }
}

void launch_legendre_bwd_f64(cudaStream_t s, const Grid &g, const double2 *psi_j, double2 *psi_th, const double *Bbwd,
                             const BlockDesc *blocks, int n_blocks, const double2 *tabA, const double *w,
                             const double *pot, double *part, int n_part_tiles, const int *status) {
  dim3 grid((unsigned)((g.npt + BP - 1) / BP), (unsigned)((g.nth + BN - 1) / BN), (unsigned)n_blocks);
  k_legendre_bwd_f64<<<grid, 256, 0, s>>>(g, psi_j, psi_th, Bbwd, blocks, tabA, w, pot, part, n_part_tiles, status);
}

}  // namespace qd
