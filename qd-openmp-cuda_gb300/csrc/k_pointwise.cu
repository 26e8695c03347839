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
__global__ void __launch_bounds__(256) k_energy_finalize(Grid g, EnergyParts ep, const BlockDesc *__restrict__ blocks,
                                  const int *__restrict__ pblock0, int n_problems,
                                  const CoriolisGroup *__restrict__ groups, const int *__restrict__ pgroup0,
                                  int ce_n, double *__restrict__ energies, double *__restrict__ rec,
                                  int *__restrict__ d_step, int rec_base, int rec_cap, int n_blocks, double norm_tol,
                                  int *status, int *status_step, StepTail tail, unsigned *done) {
  constexpr int NW = 256 / 32;
  __shared__ double red[NW][2];
  __shared__ bool last;
  const int b = blockIdx.x, tid = threadIdx.x;
  // everything this launch reads is loaded up front: one round trip
  const int st0 = *status;
  const int step = *d_step;   // advanced only by the last CTA, after every CTA has read it
  const int fcount = (tid == 0 && tail.flux_count) ? *tail.flux_count : 0;
  const BlockDesc bd = blocks[b];
  // partial counts of this block: module/potential pairs, kinetic, rotational, Coriolis
  const int n0 = ep.have_mod ? ep.mod_pe_tiles : 0;
  const int n1 = ep.have_ke ? bd.nl * ep.ke_tiles : 0;
  const int n2 = ep.have_re ? bd.nl * ep.re_tiles : 0;
  // Coriolis: every group (one per l) of this problem, the tiles of this Omega where it is a member
  const int g_lo = (ep.have_ce && groups) ? pgroup0[bd.problem] : 0;
  const int n3 = (ep.have_ce && groups) ? (pgroup0[bd.problem + 1] - g_lo) * ep.ce_tiles : 0;
  const double2 *mp = reinterpret_cast<const double2 *>(ep.mod_pe) + (int64_t)b * ep.mod_pe_tiles;
  const double *kp = ep.ke + (int64_t)bd.slab0 * ep.ke_tiles;
  const double *rp = ep.re + (int64_t)bd.slab0 * ep.re_tiles;
  // two warps per quantity (warp-uniform branch, no divergence inside a loop),
  // so that each lane's loads are independent and issue together
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  const int wq = tid >> 6, l64 = tid & 63;
  if (wq == 0) {
#pragma unroll 8
    for (int t = l64; t < n0; t += 64) {
      const double2 v = mp[t];
      acc[0] += v.x;
      acc[1] += v.y;
    }
  } else if (wq == 1) {
#pragma unroll 8
    for (int t = l64; t < n1; t += 64) acc[2] += kp[t];
  } else if (wq == 2) {
#pragma unroll 8
    for (int t = l64; t < n2; t += 64) acc[3] += rp[t];
  } else {
#pragma unroll 4
    for (int q = l64; q < n3; q += 64) {
      const int gi = g_lo + q / ep.ce_tiles, tt = q - (q / ep.ce_tiles) * ep.ce_tiles;
      const int o = bd.omega - groups[gi].omega_lo;
      if (o >= 0 && o < groups[gi].n) acc[4] += ep.ce[((int64_t)gi * ce_n + o) * ep.ce_tiles + tt];
    }
  }
  // fixed-order reduction: each warp reduces only its own quantity (the
  // module/potential pair for the first pair of warps, one sum for the others),
  // then thread 0 adds the two warps of each quantity
  double v0 = wq == 0 ? acc[0] : acc[1 + wq], v1 = acc[1];
  for (int o = 16; o > 0; o >>= 1) {
    v0 += __shfl_down_sync(0xffffffffu, v0, o);
    if (wq == 0) v1 += __shfl_down_sync(0xffffffffu, v1, o);
  }
  if ((tid & 31) == 0) {
    red[tid >> 5][0] = v0;
    red[tid >> 5][1] = v1;
  }
  __syncthreads();
  if (st0) return;   // set before this launch: nothing is written, the counter is untouched
  double mod = 0.0;
  if (tid == 0) {
    const double tot[5] = {red[0][0] + red[1][0], red[0][1] + red[1][1], red[2][0] + red[3][0],
                           red[4][0] + red[5][0], red[6][0] + red[7][0]};
    const double dV = g.dr1 * g.dr2;
    double *e = energies + b * 6;
    double ev[6];
    ev[E_MODULE] = ep.have_mod ? tot[0] * dV : e[E_MODULE];
    ev[E_POTENTIAL] = ep.have_mod ? tot[1] * dV : e[E_POTENTIAL];
    ev[E_KINETIC] = ep.have_ke ? tot[2] * ep.ke_scale : e[E_KINETIC];
    ev[E_ROTATIONAL] = ep.have_re ? tot[3] * dV : e[E_ROTATIONAL];
    ev[E_CORIOLIS] = ep.have_ce ? tot[4] * dV : e[E_CORIOLIS];
    ev[E_TOTAL] = ev[E_POTENTIAL] + ev[E_KINETIC] + ev[E_ROTATIONAL] + ev[E_CORIOLIS];
    for (int q = 0; q < 6; q++) e[q] = ev[q];
    const int slot = step - rec_base;
    if (rec && slot >= 0 && slot < rec_cap)
      for (int q = 0; q < 6; q++) rec[((int64_t)slot * n_blocks + b) * 6 + q] = ev[q];
    mod = ev[E_MODULE];
  }
  // ---- end of step: norm guard per problem, flux slot, step counter
  bool bad = false;   // thread 0: this launch set the norm status
  if (gridDim.x == 1) {
    if (tid != 0) return;
    if (ep.have_mod && mod > 1.0 + norm_tol) {
      bad = true;
      if (atomicCAS(status, 0, QD_ERR_NORM) == 0) *status_step = step;
    }
  } else {
    if (tid == 0) {
      __threadfence();
      last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (ep.have_mod)
      for (int pr = tid; pr < n_problems; pr += 256) {
        double m = 0.0;
        for (int bb = pblock0[pr]; bb < pblock0[pr + 1]; bb++) m += __ldcg(energies + bb * 6 + E_MODULE);
        if (m > 1.0 + norm_tol && atomicCAS(status, 0, QD_ERR_NORM) == 0) *status_step = step;
      }
    __syncthreads();
    if (tid != 0) return;
    *done = 0u;
    bad = atomicAdd(status, 0) != 0;
  }
  if (tail.done && !bad) {
    if (tail.flux_count) {
      if (fcount >= tail.cap) {
        atomicCAS(status, 0, QD_ERR_INVALID);
        *tail.flux_slot = 0;
      } else {
        if (fcount == 0) *tail.flux_t0 = (step + 1) * tail.dt;
        *tail.flux_slot = fcount;
        *tail.flux_count = fcount + 1;
      }
    }
    *d_step = step + 1;
  }
}

void launch_energy_finalize2(cudaStream_t st, const Grid &g, const EnergyParts &ep, const BlockDesc *blocks,
                             const int *pblock0, int n_problems, const CoriolisGroup *groups, const int *pgroup0,
                             int ce_n, double *energies, double *rec, const int *d_step, int rec_base, int rec_cap,
                             double norm_tol, int *status, int *status_step, int n_blocks, unsigned *done,
                             const StepTail *tail) {
  StepTail t{};
  if (tail) t = *tail;
  k_energy_finalize<<<n_blocks, 256, 0, st>>>(g, ep, blocks, pblock0, n_problems, groups, pgroup0, ce_n,
                                                        energies, rec, const_cast<int *>(d_step), rec_base, rec_cap,
                                                        n_blocks, norm_tol, status, status_step, t, done);
}

}  // namespace qd
