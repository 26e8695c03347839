// Energy-resolved flux through the dividing surface r = r_s and the
// reaction probability P(E).
//
// The reference carries the CRP inputs (FH2main.m:182-191,
// matlabStructures.C:80-90) but computes nothing from them.  Definition used
// here (standard time-dependent flux analysis, hbar = 1):
//   psi(t_n) on the stencil rows = exp(-i V dt/2) psi_theta   (completes the
//     Strang half step that the merged V(dt) of the next step would apply),
//   A_E(R, x_k) += dt e^{i E t_n} psi(t_n; R, r_s, x_k),
//   D_E(R, x_k) += dt e^{i E t_n} d/dr psi(t_n; R, r_s, x_k)  (centred FD stencil),
//   P(E) = Im sum_{Omega,k,i} w_k dR conj(A_E) D_E / (2 pi mu_r |a(E)|^2),
// with |a(E)|^2 = CRP.eta_sq.  Per step only the stencil rows are read; the
// time-to-energy transform runs once per chunk of steps as a complex
// [n_E x chunk] x [chunk x surface] product accumulated in FP64.
#include "qd_internal.h"
#include "qd_device.cuh"
#include "qd_tail.cuh"

namespace qd {

// buf layout: [slot][block][2][nth][n1]
__global__ void k_flux_extract(Grid g, int n_grad, int n_ds, const double2 *__restrict__ psi_th,
                               const double2 *__restrict__ hv, const double *__restrict__ fd,
                               double2 *__restrict__ buf, int n_blocks, int slot, const int *status) {
  if (status && *status) return;
  const int b = blockIdx.y;
  const int h = (n_grad - 1) / 2;
  const int64_t ns = (int64_t)g.nth * g.n1;
  double2 *out = buf + ((int64_t)slot * n_blocks + b) * 2 * ns;
  const double2 *p = psi_th + (int64_t)b * g.nth * g.npt;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < ns; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % g.n1), k = (int)(q / g.n1);
    double2 A = make_double2(0.0, 0.0), D = make_double2(0.0, 0.0);
    for (int gg = 0; gg < n_grad; gg++) {
      const int j = n_ds - h + gg;
      const double2 v = cmul(p[((int64_t)k * g.n2 + j) * g.n1 + i],
                             ldg2(hv + ((int64_t)k * n_grad + gg) * g.n1 + i));
      const double c = __ldg(fd + gg);
      D.x = fma(c, v.x, D.x);
      D.y = fma(c, v.y, D.y);
      if (gg == h) A = v;
    }
    out[q] = A;
    out[ns + q] = D;
  }
}

void launch_flux_extract(cudaStream_t s, const Grid &g, const FluxConfig &f, const double2 *psi_th, int n_blocks,
                         const double2 *half_v, const double *fd, double2 *buf, int slot, const int *status) {
  const int64_t ns = (int64_t)g.nth * g.n1;
  dim3 grid(grid_for(ns, 256, 64), n_blocks);
  k_flux_extract<<<grid, 256, 0, s>>>(g, f.n_grad, f.n_ds, psi_th, half_v, fd, buf, n_blocks, slot, status);
}

// Mixed form of the surface extraction (FP32 on the c64 pool; qd_tail.cuh).
__global__ void __launch_bounds__(FLUX_GX *FLUX_GY) k_flux_extract_f32(FluxTileArgs f, const int *slot_p,
                                                                       const int *status) {
  if (status && *status) return;
  __shared__ float2 sD[FLUX_GY][FLUX_GX];
  __shared__ float2 sA[FLUX_GX];
  __shared__ int slot;
  if (threadIdx.x == 0 && threadIdx.y == 0) slot = *slot_p;
  flux_extract_tile(f, &slot, blockIdx.y, blockIdx.x, threadIdx.y * FLUX_GX + threadIdx.x, sD, sA);
}

void launch_flux_extract_f32(cudaStream_t s, const Grid &g, const FluxConfig &f, const float2 *psi_th, int n_blocks,
                             const float2 *half_v, const float *fd, float2 *buf, const int *slot, const int *status) {
  if (f.n_grad > FLUX_GY * FLUX_GMAX)
    throw Error{QD_ERR_UNSUPPORTED, "mixed-form flux: more than 32 stencil points"};
  const int64_t ns = (int64_t)g.nth * g.n1;
  dim3 grid((unsigned)((ns + FLUX_GX - 1) / FLUX_GX), (unsigned)n_blocks);
  k_flux_extract_f32<<<grid, dim3(FLUX_GX, FLUX_GY), 0, s>>>(flux_tile_args(g, f, psi_th, half_v, fd, buf, n_blocks),
                                                              slot, status);
}

// phase[n][E] = dt exp(i E (t0 + n dt))
__global__ void k_flux_phase(const double *__restrict__ E, int nE, int count, double t0, double dt,
                             double2 *__restrict__ phase) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nE * count) return;
  const int n = q / nE, e = q % nE;
  double s, c;
  sincos(E[e] * (t0 + n * dt), &s, &c);
  phase[q] = make_double2(dt * c, dt * s);
}

namespace {
constexpr int FLUX_EB = 8;        // energies per thread
constexpr int FLUX_THREADS = 128; // surface points per CTA
constexpr int FLUX_MAXC = 64;     // maximum chunk length

// dst[e ns] += v[e] for e < ne (FP64 accumulators; FP32 partial sums widened
// exactly with integer instructions).  The loads of a chunk of up to 16 energies
// issue together before their adds: one memory round trip per chunk, not one per
// energy.
__device__ inline double2 widen(float2 v) { return make_double2(f2d(v.x), f2d(v.y)); }
__device__ inline double2 widen(double2 v) { return v; }
// fresh: the accumulators hold no earlier sum yet (first transform of a call), so they are
// written without being read
template <int EB, typename T>
__device__ inline void flux_acc_add(double2 *__restrict__ dst, int64_t ns, int ne, const T *v, bool fresh) {
  constexpr int CH = EB < 8 ? EB : 8;
#pragma unroll
  for (int e1 = 0; e1 < EB; e1 += CH) {
    double2 old[CH];
#pragma unroll
    for (int u = 0; u < CH; u++)
      old[u] = e1 + u < ne && !fresh ? dst[(int64_t)(e1 + u) * ns] : make_double2(0.0, 0.0);
#pragma unroll
    for (int u = 0; u < CH; u++)
      if (e1 + u < ne) {
        const double2 w = widen(v[e1 + u]);
        old[u].x += w.x;
        old[u].y += w.y;
        dst[(int64_t)(e1 + u) * ns] = old[u];
      }
  }
}
}

// acc[b][c][E][k][i] += sum_n phase[n][E] buf[n][b][c][k][i]
__global__ void __launch_bounds__(FLUX_THREADS) k_flux_dft(int64_t ns2, int nE, int n_blocks, int count,
                                                           const double2 *__restrict__ buf,
                                                           const double2 *__restrict__ phase,
                                                           double2 *__restrict__ acc, const int *status) {
  if (status && *status) return;
  __shared__ double2 ph[FLUX_MAXC][FLUX_EB];
  const int b = blockIdx.z;
  const int e0 = blockIdx.y * FLUX_EB;
  for (int q = threadIdx.x; q < count * FLUX_EB; q += blockDim.x) {
    const int n = q / FLUX_EB, e = q % FLUX_EB;
    ph[n][e] = e0 + e < nE ? phase[(int64_t)n * nE + e0 + e] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  const int64_t s = (int64_t)blockIdx.x * FLUX_THREADS + threadIdx.x;   // over 2*nth*n1
  if (s >= ns2) return;
  double2 a[FLUX_EB];
#pragma unroll
  for (int e = 0; e < FLUX_EB; e++) a[e] = make_double2(0.0, 0.0);
  for (int n = 0; n < count; n++) {
    const double2 v = buf[((int64_t)n * n_blocks + b) * ns2 + s];
#pragma unroll
    for (int e = 0; e < FLUX_EB; e++) {
      const double2 p = ph[n][e];
      a[e].x = fma(p.x, v.x, fma(-p.y, v.y, a[e].x));
      a[e].y = fma(p.x, v.y, fma(p.y, v.x, a[e].y));
    }
  }
  const int64_t ns = ns2 / 2;
  const int c = (int)(s / ns);
  const int64_t kq = s % ns;
  flux_acc_add<FLUX_EB>(acc + (((int64_t)b * 2 + c) * nE + e0) * ns + kq, ns, min(FLUX_EB, nE - e0), a, false);
}

void launch_flux_dft(cudaStream_t s, const Grid &g, const FluxConfig &f, int n_blocks, const double2 *buf, int count,
                     const double *energies, double t0, double dt, double2 *phase_scratch, double2 *acc,
                     const int *status) {
  if (count <= 0) return;
  if (count > FLUX_MAXC) throw Error{QD_ERR_INVALID, "flux chunk above 64 steps"};
  const int nE = f.n_energies;
  k_flux_phase<<<(nE * count + 255) / 256, 256, 0, s>>>(energies, nE, count, t0, dt, phase_scratch);
  const int64_t ns2 = 2LL * g.nth * g.n1;
  dim3 grid((unsigned)((ns2 + FLUX_THREADS - 1) / FLUX_THREADS), (unsigned)((nE + FLUX_EB - 1) / FLUX_EB),
            (unsigned)n_blocks);
  k_flux_dft<<<grid, FLUX_THREADS, 0, s>>>(ns2, nE, n_blocks, count, buf, phase_scratch, acc, status);
}

// Same transform with the step count read from the device, so that it can sit
// inside a captured CUDA graph; the phase table holds rows n < *count_p.
__global__ void __launch_bounds__(FLUX_THREADS) k_flux_dft_dev(int64_t ns2, int nE, int n_blocks, const int *count_p,
                                                               int cap,
                                                               const double2 *__restrict__ buf,
                                                               const double2 *__restrict__ phase,
                                                               double2 *__restrict__ acc, const int *status,
                                                               const int *fresh) {
  if (status && *status) return;
  const bool fr = fresh && *fresh;
  const int count = min(min(*count_p, cap), FLUX_MAXC);
  if (count <= 0) return;
  __shared__ double2 ph[FLUX_MAXC][FLUX_EB];
  const int b = blockIdx.z;
  const int e0 = blockIdx.y * FLUX_EB;
  for (int q = threadIdx.x; q < count * FLUX_EB; q += blockDim.x) {
    const int n = q / FLUX_EB, e = q % FLUX_EB;
    ph[n][e] = e0 + e < nE ? phase[(int64_t)n * nE + e0 + e] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  const int64_t s = (int64_t)blockIdx.x * FLUX_THREADS + threadIdx.x;
  if (s >= ns2) return;
  double2 a[FLUX_EB];
#pragma unroll
  for (int e = 0; e < FLUX_EB; e++) a[e] = make_double2(0.0, 0.0);
  for (int n = 0; n < count; n++) {
    const double2 v = buf[((int64_t)n * n_blocks + b) * ns2 + s];
#pragma unroll
    for (int e = 0; e < FLUX_EB; e++) {
      const double2 p = ph[n][e];
      a[e].x = fma(p.x, v.x, fma(-p.y, v.y, a[e].x));
      a[e].y = fma(p.x, v.y, fma(p.y, v.x, a[e].y));
    }
  }
  const int64_t ns = ns2 / 2;
  const int c = (int)(s / ns);
  const int64_t kq = s % ns;
  flux_acc_add<FLUX_EB>(acc + (((int64_t)b * 2 + c) * nE + e0) * ns + kq, ns, min(FLUX_EB, nE - e0), a, fr);
}

// Mixed form of the transform: products and the chunk's partial sums in FP32
// (phases computed in FP64 and rounded once, surface values converted with
// integer instructions), each chunk's sum added into the FP64 accumulators.
// Eight energies per thread: the accumulator update is one round of eight
// loads per thread, and the grid (ns2 / 128 x nE / 8 CTAs of 80 registers, six
// per SM) keeps enough loads in flight; the kernel is bound by the latency of
// the 630 MB of FP64 accumulators it reads and writes per flush.
namespace {
constexpr int FLUX_EB32 = 8;
}

__global__ void __launch_bounds__(FLUX_THREADS, 6) k_flux_dft_f32(int64_t ns2, int nE, int n_blocks, const int *count_p,
                                                               int cap, const float2 *__restrict__ buf,
                                                               const double2 *__restrict__ phase,
                                                               double2 *__restrict__ acc, const int *status,
                                                               const int *fresh) {
  if (status && *status) return;
  const bool fr = fresh && *fresh;
  const int count = min(min(*count_p, cap), FLUX_MAXC);
  if (count <= 0) return;
  __shared__ float2 ph[FLUX_MAXC][FLUX_EB32];
  const int b = blockIdx.z;
  const int e0 = blockIdx.y * FLUX_EB32;
  for (int q = threadIdx.x; q < count * FLUX_EB32; q += blockDim.x) {
    const int n = q / FLUX_EB32, e = q % FLUX_EB32;
    const double2 v = e0 + e < nE ? phase[(int64_t)n * nE + e0 + e] : make_double2(0.0, 0.0);
    ph[n][e] = make_float2(d2f_rn(v.x), d2f_rn(v.y));
  }
  __syncthreads();
  const int64_t s = (int64_t)blockIdx.x * FLUX_THREADS + threadIdx.x;
  if (s >= ns2) return;
  float2 a[FLUX_EB32];
#pragma unroll
  for (int e = 0; e < FLUX_EB32; e++) a[e] = make_float2(0.0f, 0.0f);
  // unrolled so that several steps' surface values are loaded ahead of their use
#pragma unroll 8
  for (int n = 0; n < count; n++) {
    const float2 vd = buf[((int64_t)n * n_blocks + b) * ns2 + s];
    const float vx = vd.x, vy = vd.y;
#pragma unroll
    for (int e = 0; e < FLUX_EB32; e++) {
      const float2 p = ph[n][e];
      a[e].x = fmaf(p.x, vx, fmaf(-p.y, vy, a[e].x));
      a[e].y = fmaf(p.x, vy, fmaf(p.y, vx, a[e].y));
    }
  }
  const int64_t ns = ns2 / 2;
  const int c = (int)(s / ns);
  const int64_t kq = s % ns;
  flux_acc_add<FLUX_EB32>(acc + (((int64_t)b * 2 + c) * nE + e0) * ns + kq, ns, min(FLUX_EB32, nE - e0), a, fr);
}

void launch_flux_dft_f32(cudaStream_t s, int64_t ns2, int nE, int n_blocks, const int *count_p, int cap,
                         const float2 *buf, const double2 *phase, double2 *acc, const int *status, const int *fresh) {
  dim3 grid((unsigned)((ns2 + FLUX_THREADS - 1) / FLUX_THREADS), (unsigned)((nE + FLUX_EB32 - 1) / FLUX_EB32),
            (unsigned)n_blocks);
  k_flux_dft_f32<<<grid, FLUX_THREADS, 0, s>>>(ns2, nE, n_blocks, count_p, cap, buf, phase, acc, status, fresh);
}

// P(E) per problem: one CTA per (E, problem); accumulators still marked fresh hold
// no transform yet and count as zero
__global__ void k_flux_crp(Grid g, int nE, const int *__restrict__ pblock0, const double2 *__restrict__ acc,
                           const double *__restrict__ w, const double *__restrict__ eta_sq, double *__restrict__ crp,
                           const int *fresh) {
  __shared__ double red[32];
  const int e = blockIdx.x, pr = blockIdx.y;
  const int64_t ns = (int64_t)g.nth * g.n1;
  double s = 0.0;
  for (int b = pblock0[pr]; b < pblock0[pr + 1] && !(fresh && *fresh); b++) {
    const double2 *A = acc + (((int64_t)b * 2 + 0) * nE + e) * ns;
    const double2 *D = acc + (((int64_t)b * 2 + 1) * nE + e) * ns;
    for (int64_t q = threadIdx.x; q < ns; q += blockDim.x) {
      const double2 a = A[q], d = D[q];
      // Im(conj(a) d) = a.x d.y - a.y d.x
      s += w[q / g.n1] * (a.x * d.y - a.y * d.x);
    }
  }
  s = block_sum(s, red);
  if (threadIdx.x == 0)
    crp[(int64_t)pr * nE + e] = s * g.dr1 / (2.0 * M_PI * g.m2 * eta_sq[(int64_t)pr * nE + e]);
}

void launch_flux_crp(cudaStream_t s, const Grid &g, const FluxConfig &f, int n_problems, const int *block0_of_problem,
                     const double2 *acc, const double *w, const double *eta_sq, double *crp, const int *fresh) {
  dim3 grid((unsigned)f.n_energies, (unsigned)n_problems);
  k_flux_crp<<<grid, 256, 0, s>>>(g, f.n_energies, block0_of_problem, acc, w, eta_sq, crp, fresh);
}

}  // namespace qd
