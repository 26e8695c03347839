// Pointwise kernels: phase application, FP64 phase-table builders, energy
// finalisation and the norm guard.
//
// The reference evaluates exp(Complex(0,-dt)*x) per element on every call
// (evolutionCUDAaux.cu:5-54, complex.h:115).  Here each phase factor is
// evaluated once per run, in FP64 on the device, into a table; every step then
// multiplies by the table (one complex multiply per point instead of a sincos,
// which matters on a part whose FP64 rate is a small fraction of its FP32 rate).
#include "qd_internal.h"
#include "qd_device.cuh"
#include "qd_tail.cuh"

namespace qd {

template <typename S>
__global__ void k_theta_phase(S *__restrict__ psi, const double2 *__restrict__ tab, int64_t n_total,
                              int64_t n_per_block, const int *status) {
  if (status && *status) return;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_total; i += stride) {
    const int64_t t = i % n_per_block;
    store_c(psi + i, cmul(load_c(psi + i), ldg2(tab + t)));
  }
}

template <typename S>
void launch_theta_phase(cudaStream_t s, S *psi, const double2 *tab, int n_blocks, int64_t n_per_block,
                        const int *status) {
  const int64_t n = (int64_t)n_blocks * n_per_block;
  k_theta_phase<S><<<grid_for(n, 256), 256, 0, s>>>(psi, tab, n, n_per_block, status);
}
template void launch_theta_phase<double2>(cudaStream_t, double2 *, const double2 *, int, int64_t, const int *);
template void launch_theta_phase<float2>(cudaStream_t, float2 *, const double2 *, int, int64_t, const int *);

// c64 <-> c128 copies for the mixed form's host transfers (widening is exact,
// narrowing rounds to nearest)
__global__ void k_widen(const float2 *__restrict__ src, double2 *__restrict__ dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 v = src[i];
    dst[i] = make_double2(f2d(v.x), f2d(v.y));
  }
}
__global__ void k_narrow(const double2 *__restrict__ src, float2 *__restrict__ dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = src[i];
    dst[i] = make_float2(d2f_rn(v.x), d2f_rn(v.y));
  }
}
void launch_widen(cudaStream_t s, const float2 *src, double2 *dst, int64_t n) {
  if (n > 0) k_widen<<<grid_for(n, 256), 256, 0, s>>>(src, dst, n);
}
void launch_narrow(cudaStream_t s, const double2 *src, float2 *dst, int64_t n) {
  if (n > 0) k_narrow<<<grid_for(n, 256), 256, 0, s>>>(src, dst, n);
}

template <typename S>
__global__ void k_slab_phase(S *__restrict__ psi_j, const double2 *__restrict__ tab,
                             const SlabDesc *__restrict__ slabs, int64_t npt, const int *status) {
  if (status && *status) return;
  const int sl = blockIdx.y;
  const int l = slabs[sl].l;
  S *p = psi_j + (int64_t)sl * npt;
  const double2 *t = tab + (int64_t)l * npt;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npt; i += (int64_t)gridDim.x * blockDim.x)
    store_c(p + i, cmul(load_c(p + i), ldg2(t + i)));
}

template <typename S>
void launch_slab_phase(cudaStream_t s, S *psi_j, const double2 *tab, const SlabDesc *slabs, int n_slabs,
                       int64_t npt, const int *status) {
  if (n_slabs == 0) return;
  dim3 grid((unsigned)std::min<int64_t>((npt + 255) / 256, 64), n_slabs);
  k_slab_phase<S><<<grid, 256, 0, s>>>(psi_j, tab, slabs, npt, status);
}
template void launch_slab_phase<double2>(cudaStream_t, double2 *, const double2 *, const SlabDesc *, int, int64_t,
                                         const int *);
template void launch_slab_phase<float2>(cudaStream_t, float2 *, const double2 *, const SlabDesc *, int, int64_t,
                                        const int *);

// ------------------------------------------------------------------ tables
__global__ void k_build_theta_table(const double *__restrict__ pot, const double *__restrict__ d1,
                                    const double *__restrict__ d2, int n1, int n2, int64_t n, double dt,
                                    double2 *__restrict__ tab) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % n1);
    const int j = (int)((q / n1) % n2);
    double s, c;
    sincos(dt * pot[q], &s, &c);
    double m = 1.0;
    if (d1 && d2) m = d1[i] * d2[j];
    tab[q] = make_double2(m * c, -m * s);
  }
}

void launch_build_theta_table(cudaStream_t s, const Grid &g, const double *pot, const double *d1, const double *d2,
                              double dt, double2 *tab) {
  const int64_t n = g.npt * g.nth;
  k_build_theta_table<<<grid_for(n, 256), 256, 0, s>>>(pot, d1, d2, g.n1, g.n2, n, dt, tab);
}

// exp(-i dt l(l+1) (1/(2 m1 R_i^2) + 1/(2 m2 r_j^2)))   (evolutionCUDAaux.cu:33-54, cudaMath.h:150-157)
__global__ void k_build_rot_table(Grid g, double dt, double2 *__restrict__ tab) {
  const int64_t n = g.npt * (g.l_max + 1);
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % g.n1);
    const int j = (int)((q / g.n1) % g.n2);
    const int l = (int)(q / g.npt);
    const double R = g.left1 + i * g.dr1;
    const double r = g.left2 + j * g.dr2;
    const double I = 1.0 / (2 * g.m1 * R * R) + 1.0 / (2 * g.m2 * r * r);
    double s, c;
    sincos(dt * (double)l * (double)(l + 1) * I, &s, &c);
    tab[q] = make_double2(c, -s);
  }
}

void launch_build_rot_table(cudaStream_t s, const Grid &g, double dt, double2 *tab) {
  k_build_rot_table<<<grid_for(g.npt * (g.l_max + 1), 256), 256, 0, s>>>(g, dt, tab);
}

__global__ void k_build_kin_table(const double *__restrict__ T1, const double *__restrict__ T2, int n1, int64_t n,
                                  double dt, double2 *__restrict__ tab) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % n1);
    const int j = (int)(q / n1);
    double s, c;
    sincos(dt * (T1[i] + T2[j]), &s, &c);
    tab[q] = make_double2(c, -s);
  }
}

void launch_build_kin_table(cudaStream_t s, const Grid &g, const double *T1, const double *T2, double dt,
                            double2 *tab) {
  k_build_kin_table<<<grid_for(g.npt, 256), 256, 0, s>>>(T1, T2, g.n1, g.npt, dt, tab);
}

// exp(-i (dt/2) V) on the flux stencil rows: [k][g][i]
__global__ void k_build_half_v(Grid g, int n_grad, int n_ds, const double *__restrict__ pot, double dt,
                               double2 *__restrict__ hv) {
  const int h = (n_grad - 1) / 2;
  const int64_t n = (int64_t)g.nth * n_grad * g.n1;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % g.n1);
    const int gg = (int)((q / g.n1) % n_grad);
    const int k = (int)(q / ((int64_t)g.n1 * n_grad));
    const int j = n_ds - h + gg;
    double s, c;
    sincos(0.5 * dt * pot[((int64_t)k * g.n2 + j) * g.n1 + i], &s, &c);
    hv[q] = make_double2(c, -s);
  }
}

void launch_build_half_v(cudaStream_t s, const Grid &g, const FluxConfig &f, const double *pot, double dt,
                         double2 *half_v) {
  const int64_t n = (int64_t)g.nth * f.n_grad * g.n1;
  k_build_half_v<<<grid_for(n, 256), 256, 0, s>>>(g, f.n_grad, f.n_ds, pot, dt, half_v);
}

// ------------------------------------------------------- lifting tables
// Multiplication by exp(i a) is a rotation by a.  For the FP32 path it is
// applied as two rotations by a/2, each the three shears x += t y, y += s x,
// x += t y with t = -tan(a/4), s = sin(a/2) (|a/2| <= pi/2 after reducing a
// to (-pi, pi], so |t| <= 1).  Each shear has determinant exactly 1 whatever
// the rounding of t and s, so a factor applied every step cannot make the
// norm grow or decay systematically (a rounded e^{ia} in FP32 has
// |e^{ia}| = 1 +- 6e-8, which compounds over 10^4 steps).
__device__ inline float2 lift_coeffs(double a) {
  const double r = remainder(a, 2.0 * M_PI);
  const double h = 0.5 * r;
  return make_float2((float)(-tan(0.5 * h)), (float)sin(h));
}

__global__ void k_build_lift_theta(const double *__restrict__ pot, int64_t n, double dt, float2 *__restrict__ out) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    out[q] = lift_coeffs(-dt * pot[q]);
}

void launch_build_lift_theta(cudaStream_t s, const Grid &g, const double *pot, double dt, float2 *out) {
  const int64_t n = g.npt * g.nth;
  k_build_lift_theta<<<grid_for(n, 256), 256, 0, s>>>(pot, n, dt, out);
}

__global__ void k_build_lift_rot(int n, int l_max, double left, double dr, double mass, double dt,
                                 float2 *__restrict__ out) {
  const int64_t tot = (int64_t)(l_max + 1) * n;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % n), l = (int)(q / n);
    const double x = left + i * dr;
    out[q] = lift_coeffs(-dt * (double)l * (double)(l + 1) / (2.0 * mass * x * x));
  }
}

void launch_build_lift_rot(cudaStream_t s, int n, int l_max, double left, double dr, double mass, double dt,
                           float2 *out) {
  k_build_lift_rot<<<grid_for((int64_t)(l_max + 1) * n, 256), 256, 0, s>>>(n, l_max, left, dr, mass, dt, out);
}

__global__ void k_build_lift_kin(int n, const double *__restrict__ T, double dt, float2 *__restrict__ out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) out[q] = lift_coeffs(-dt * T[q]);
}

void launch_build_lift_kin(cudaStream_t s, int n, const double *T, double dt, float2 *out) {
  k_build_lift_kin<<<(n + 255) / 256, 256, 0, s>>>(n, T, dt, out);
}

__global__ void k_build_half_v_lift(Grid g, int n_grad, int n_ds, const double *__restrict__ pot, double dt,
                                    float2 *__restrict__ hv) {
  const int h = (n_grad - 1) / 2;
  const int64_t n = (int64_t)g.nth * n_grad * g.n1;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % g.n1);
    const int gg = (int)((q / g.n1) % n_grad);
    const int k = (int)(q / ((int64_t)g.n1 * n_grad));
    const int j = n_ds - h + gg;
    hv[q] = lift_coeffs(-0.5 * dt * pot[((int64_t)k * g.n2 + j) * g.n1 + i]);
  }
}

void launch_build_half_v_lift(cudaStream_t s, const Grid &g, const FluxConfig &f, const double *pot, double dt,
                              float2 *half_v) {
  const int64_t n = (int64_t)g.nth * f.n_grad * g.n1;
  k_build_half_v_lift<<<grid_for(n, 256), 256, 0, s>>>(g, f.n_grad, f.n_ds, pot, dt, half_v);
}

__global__ void k_build_float_tables(Grid g, const double *__restrict__ w, const double *__restrict__ pot,
                                     const double *__restrict__ d1, const double *__restrict__ d2,
                                     const double *__restrict__ T1, const double *__restrict__ T2, float *wf,
                                     float *wvf, float *d1f, float *d2f, float *T1f, float *T2f, float *I1f,
                                     float *I2f) {
  const int64_t n = g.npt * g.nth;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(q / g.npt);
    wvf[q] = (float)(w[k] * pot[q]);
    if (q < g.nth) wf[q] = (float)w[q];
    if (q < g.n1) {
      T1f[q] = (float)T1[q];
      const double R = g.left1 + (double)q * g.dr1;
      I1f[q] = (float)(1.0 / (2.0 * g.m1 * R * R));
      if (d1f) d1f[q] = (float)d1[q];
    }
    if (q < g.n2) {
      T2f[q] = (float)T2[q];
      const double r = g.left2 + (double)q * g.dr2;
      I2f[q] = (float)(1.0 / (2.0 * g.m2 * r * r));
      if (d2f) d2f[q] = (float)d2[q];
    }
  }
}

void launch_build_float_tables(cudaStream_t s, const Grid &g, const double *w, const double *pot, const double *d1,
                               const double *d2, const double *T1, const double *T2, float *wf, float *wvf,
                               float *d1f, float *d2f, float *T1f, float *T2f, float *I1f, float *I2f) {
  const int64_t n = g.npt * g.nth;
  k_build_float_tables<<<grid_for(n, 256), 256, 0, s>>>(g, w, pot, d1, d2, T1, T2, wf, wvf, d1f, d2f, T1f, T2f, I1f,
                                                       I2f);
}

// ------------------------------------------------------------ energies
// rotational energy partials: sum l(l+1) (I1_i + I2_j) |psi|^2 per (slab, tile)
template <typename S>
__global__ void k_rot_energy(Grid g, const S *__restrict__ psi_j, const SlabDesc *__restrict__ slabs,
                             double *__restrict__ re_part, int tiles, const int *status) {
  if (status && *status) return;
  __shared__ double red[32];
  const int sl = blockIdx.y;
  const double ll = (double)slabs[sl].l * (slabs[sl].l + 1);
  const S *p = psi_j + (int64_t)sl * g.npt;
  double acc = 0.0;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < g.npt; q += (int64_t)tiles * blockDim.x) {
    const int i = (int)(q % g.n1), j = (int)(q / g.n1);
    const double R = g.left1 + i * g.dr1, r = g.left2 + j * g.dr2;
    const double I = 1.0 / (2 * g.m1 * R * R) + 1.0 / (2 * g.m2 * r * r);
    const double2 v = load_c(p + q);
    acc += ll * I * (v.x * v.x + v.y * v.y);
  }
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) re_part[(int64_t)sl * tiles + blockIdx.x] = acc;
}

template <typename S>
void launch_rot_energy(cudaStream_t s, const Grid &g, const S *psi_j, const SlabDesc *slabs, int n_slabs,
                       double *re_part, int tiles, const int *status) {
  if (n_slabs == 0) return;
  k_rot_energy<S><<<dim3(tiles, n_slabs), 256, 0, s>>>(g, psi_j, slabs, re_part, tiles, status);
}
template void launch_rot_energy<double2>(cudaStream_t, const Grid &, const double2 *, const SlabDesc *, int,
                                         double *, int, const int *);
template void launch_rot_energy<float2>(cudaStream_t, const Grid &, const float2 *, const SlabDesc *, int, double *,
                                        int, const int *);

// Energy finalisation.  One CTA per Omega block loads all of that block's
// partials (module, potential, kinetic, rotational, Coriolis) in one pass,
// sums them in a fixed order (deterministic) and writes energies[b] and the
// step record; the last CTA to finish then applies the norm guard of
// print_energies (cudaOpenMP2.cu:425-445) per problem and, at the end of a
// full step, books the flux slot and advances the step counter.
// Coupling-energy partials are laid out [group][ce_n][tiles]; a block collects
// them from every group (one per l) of its problem that contains its Omega.
__global__ void __launch_bounds__(256) k_energy_finalize(FinalizeArgs a) {
  __shared__ double red[5][FIN_THREADS];
  __shared__ double tot[5];
  __shared__ bool last;
  __shared__ int hdr[3];
  const int tid = threadIdx.x;
  // everything this launch reads is loaded up front, once per CTA (the status words
  // share one L2 line), issued together with the partial sums; finalize_reduce's
  // barrier publishes them
  double eprev[6];
  if (tid == 0) {
    hdr[0] = *a.status;
    hdr[1] = *a.d_step;   // advanced only at the very end, after every CTA has read it
    hdr[2] = a.tail.flux_count ? *a.tail.flux_count : 0;
    for (int q = 0; q < 6; q++) eprev[q] = a.energies[blockIdx.x * 6 + q];
  }
  finalize_reduce(a, blockIdx.x, red, tot);
  const int st0 = hdr[0], step = hdr[1], fcount = tid == 0 ? hdr[2] : 0;
  if (st0) return;   // set before this launch: nothing is written, the counter is untouched
  double mod = 0.0;
  if (tid == 0) mod = finalize_write(a, blockIdx.x, step, tot, eprev);
  if (gridDim.x == 1) {
    if (tid != 0) return;
    bool bad = false;
    if (a.ep.have_mod && mod > 1.0 + a.norm_tol) {
      bad = true;
      if (atomicCAS(a.status, 0, QD_ERR_NORM) == 0) *a.status_step = step;
    }
    finalize_step_end(a, step, fcount, bad);
  } else {
    finalize_last_cta(a, step, fcount, &last);
  }
}

// Mixed form, one launch for the end of a step: CTAs [0, n_blocks) finalise one
// Omega block each (first in the grid, so that their serial reductions overlap
// the extraction), CTAs [n_blocks, n_blocks + nfx) extract the flux surface
// values (slot = the flux count before this step ends), and the last CTA to
// finish applies the norm guard and ends the step.
__global__ void __launch_bounds__(256) k_step_tail_mixed(FinalizeArgs a, FluxTileArgs f, int fx_tiles) {
  __shared__ double red[5][FIN_THREADS];
  __shared__ double tot[5];
  __shared__ float2 sD[FLUX_GY][FLUX_GX];
  __shared__ float2 sA[FLUX_GX];
  __shared__ bool last;
  __shared__ int hdr[4];
  const int tid = threadIdx.x;
  // the status words are read once per CTA (they share one L2 line) and in flight
  // together with the tile's own loads; the barrier inside the extraction or the
  // reduction publishes them, and nothing is written before they are checked
  double eprev[6];
  if (tid == 0) {
    hdr[0] = *a.status;
    hdr[1] = *a.d_step;
    hdr[2] = a.tail.flux_count ? *a.tail.flux_count : 0;
    // the flux slot, or -1: status already set, or the buffer is full (reported by the step end)
    hdr[3] = (hdr[0] == 0 && hdr[2] < a.tail.cap) ? hdr[2] : -1;
    if ((int)blockIdx.x < a.n_blocks)
      for (int q = 0; q < 6; q++) eprev[q] = a.energies[blockIdx.x * 6 + q];
  }
  if ((int)blockIdx.x >= a.n_blocks) {
    const int x = blockIdx.x - a.n_blocks;
    flux_extract_tile(f, &hdr[3], x / fx_tiles, x % fx_tiles, tid, sD, sA);
  } else {
    finalize_reduce(a, blockIdx.x, red, tot);
  }
  if (hdr[0]) return;   // set before this launch: uniform, the counter is untouched
  const int step = hdr[1], fcount = hdr[2];
  if ((int)blockIdx.x < a.n_blocks && tid == 0) finalize_write(a, blockIdx.x, step, tot, eprev);
  finalize_last_cta(a, step, fcount, &last);
}

void launch_energy_finalize2(cudaStream_t st, const Grid &g, const EnergyParts &ep, const BlockDesc *blocks,
                             const int *pblock0, int n_problems, const CoriolisGroup *groups, const int *pgroup0,
                             int ce_n, double *energies, double *rec, const int *d_step, int rec_base, int rec_cap,
                             double norm_tol, int *status, int *status_step, int n_blocks, unsigned *done,
                             const StepTail *tail, const FluxTileArgs *fx) {
  FinalizeArgs a{};
  a.g = g;
  a.ep = ep;
  a.blocks = blocks;
  a.pblock0 = pblock0;
  a.n_problems = n_problems;
  a.groups = groups;
  a.pgroup0 = pgroup0;
  a.ce_n = ce_n;
  a.energies = energies;
  a.rec = rec;
  a.d_step = const_cast<int *>(d_step);
  a.rec_base = rec_base;
  a.rec_cap = rec_cap;
  a.n_blocks = n_blocks;
  a.norm_tol = norm_tol;
  a.status = status;
  a.status_step = status_step;
  if (tail) a.tail = *tail;
  a.done = done;
  if (fx) {
    const int fx_tiles = (int)(((int64_t)g.nth * g.n1 + FLUX_GX - 1) / FLUX_GX);
    const int nfx = fx_tiles * n_blocks;
    k_step_tail_mixed<<<nfx + n_blocks, FLUX_GX * FLUX_GY, 0, st>>>(a, *fx, fx_tiles);
  } else {
    k_energy_finalize<<<n_blocks, 256, 0, st>>>(a);
  }
}

}  // namespace qd
