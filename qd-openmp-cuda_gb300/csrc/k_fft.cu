// Batched 2-D FFT over (R, r) of every Legendre slab, fused with the kinetic
// phase, the kinetic-energy reduction, the 1/(n1 n2) scale, the epilogue
// rotational phase and the rotational-energy reduction.
//
// Reference: cufftPlanMany 2-D Z2Z {n2, n1} batched over l_max+1 slabs
// (wavepackets1device.cu:186-201), forward/inverse in place
// (omegawavepacket.cu:242-269), cublasZdscal by 1/(n1 n2), the kinetic kernel
// (evolutionCUDAaux.cu:13-31) and a per-slab ZDOTC loop for the kinetic energy
// (omegawavepacket.cu:364-395).  Sign conventions follow cuFFT: forward
// exp(-2 pi i jk/n), inverse exp(+2 pi i jk/n), both unnormalised.
//
// Algorithm: mixed-radix (4, 2, 3) Stockham autosort in shared memory, each
// stage reading all inputs to registers, a barrier, then writing the outputs
// in place.  Twiddles exp(-2 pi i t/n) are computed in FP64 on the host; the
// FP32 variant rounds them.  Three passes: rows (R, contiguous) forward;
// columns (r, stride n1) forward + kinetic phase + kinetic energy + inverse;
// rows inverse + scale + epilogue.
#include "qd_internal.h"
#include "qd_device.cuh"

#include <cooperative_groups.h>
#include <cmath>
#include <vector>

namespace cg = cooperative_groups;

namespace qd {

namespace {
constexpr int FFT_THREADS = 256;
constexpr int MAXV = 16;   // complex values per thread per stage

template <typename R> struct CT;
template <> struct CT<double> {
  using T = double2;
  static __device__ inline T make(double x, double y) { return make_double2(x, y); }
};
template <> struct CT<float> {
  using T = float2;
  static __device__ inline T make(float x, float y) { return make_float2(x, y); }
};

template <typename C> __device__ inline C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __device__ inline C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __device__ inline C cmulg(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}

template <typename R, int RAD>
__device__ inline void dft(typename CT<R>::T *v, bool inv) {
  using C = typename CT<R>::T;
  if (RAD == 2) {
    const C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if (RAD == 4) {
    const C a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    const C c = cadd(v[1], v[3]), d = csub(v[1], v[3]);
    C id;   // forward: -i d ; inverse: +i d
    if (!inv) { id.x = d.y; id.y = -d.x; } else { id.x = -d.y; id.y = d.x; }
    v[0] = cadd(a, c);
    v[2] = csub(a, c);
    v[1] = cadd(b, id);
    v[3] = csub(b, id);
  } else if (RAD == 3) {
    const R h = (R)0.86602540378443864676;   // sqrt(3)/2
    const C t = cadd(v[1], v[2]);
    const C x0 = v[0];
    v[0] = cadd(x0, t);
    C u;
    u.x = x0.x - (R)0.5 * t.x;
    u.y = x0.y - (R)0.5 * t.y;
    const C s = csub(v[1], v[2]);
    C w;   // forward: -i h s ; inverse: +i h s
    if (!inv) { w.x = h * s.y; w.y = -h * s.x; } else { w.x = -h * s.y; w.y = h * s.x; }
    v[1] = cadd(u, w);
    v[2] = csub(u, w);
  }
}

// One Stockham stage on nrows independent transforms of length N stored at
// buf[row*rs + x*es].  COLS selects which index varies fastest across threads
// so that shared-memory accesses stay contiguous.
template <typename R, int RAD, bool COLS, int THREADS = FFT_THREADS, int MV = MAXV>
__device__ inline void fft_stage(typename CT<R>::T *buf, int N, int nrows, int rs, int es, int Ns,
                                 const typename CT<R>::T *__restrict__ tw, bool inv, const FastDiv &fnbf,
                                 const FastDiv &fNs, const FastDiv &frows) {
  using C = typename CT<R>::T;
  constexpr int NB = (MV + RAD - 1) / RAD;
  const int nbf = N / RAD;
  const int total = nrows * nbf;
  const int tstep = N / (Ns * RAD);
  C v[NB][RAD];
  int dst_base[NB];
#pragma unroll
  for (int q = 0; q < NB; q++) {
    const int t = threadIdx.x + THREADS * q;
    if (t < total) {
      int row, jj;
      if (COLS) {
        const int qq = (int)fdiv(frows, (uint32_t)t);
        row = t - qq * nrows;
        jj = qq;
      } else {
        row = (int)fdiv(fnbf, (uint32_t)t);
        jj = t - row * nbf;
      }
      const int qn = (int)fdiv(fNs, (uint32_t)jj);
      const int k = jj - qn * Ns;
      dst_base[q] = row * rs + (qn * Ns * RAD + k) * es;
#pragma unroll
      for (int r = 0; r < RAD; r++) v[q][r] = buf[row * rs + (jj + r * nbf) * es];
      if (Ns > 1) {
#pragma unroll
        for (int r = 1; r < RAD; r++) {
          const int idx = r * k * tstep;
          C w = tw[idx];
          if constexpr (std::is_same<R, float>::value) {
            // twiddle as a three-shear rotation (determinant exactly 1): the
            // table holds (-tan(b/2), sin(b)) of b = the twiddle angle shifted
            // by pi where |angle| > pi/2 (then the vector is negated first)
            const bool flip = 4 * idx > N && 4 * idx < 3 * N;
            const float tt = inv ? -w.x : w.x, ss = inv ? -w.y : w.y;
            float x = v[q][r].x, y = v[q][r].y;
            if (flip) {
              x = -x;
              y = -y;
            }
            x = fmaf(tt, y, x);
            y = fmaf(ss, x, y);
            x = fmaf(tt, y, x);
            v[q][r].x = x;
            v[q][r].y = y;
          } else {
            if (inv) w.y = -w.y;
            v[q][r] = cmulg(v[q][r], w);
          }
        }
      }
      dft<R, RAD>(v[q], inv);
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NB; q++) {
    const int t = threadIdx.x + THREADS * q;
    if (t < total) {
#pragma unroll
      for (int r = 0; r < RAD; r++) buf[dst_base[q] + r * Ns * es] = v[q][r];
    }
  }
  __syncthreads();
}

// radix sequence of one transform length with the stage divisors precomputed
struct Radices {
  int n, nst;
  int rad[16];
  FastDiv nbf[16];   // n / rad[s]
  FastDiv ns[16];    // product of the radices before stage s
  FastDiv fn;        // n
};

template <typename R, bool COLS, int THREADS = FFT_THREADS, int MV = MAXV>
__device__ inline void fft_run(typename CT<R>::T *buf, const Radices &rd, int nrows, int rs, int es,
                               const typename CT<R>::T *__restrict__ tw, bool inv, const FastDiv &frows) {
  int Ns = 1;
  for (int s = 0; s < rd.nst; s++) {
    const int rad = rd.rad[s];
    if (rad == 4)
      fft_stage<R, 4, COLS, THREADS, MV>(buf, rd.n, nrows, rs, es, Ns, tw, inv, rd.nbf[s], rd.ns[s], frows);
    else if (rad == 2)
      fft_stage<R, 2, COLS, THREADS, MV>(buf, rd.n, nrows, rs, es, Ns, tw, inv, rd.nbf[s], rd.ns[s], frows);
    else
      fft_stage<R, 3, COLS, THREADS, MV>(buf, rd.n, nrows, rs, es, Ns, tw, inv, rd.nbf[s], rd.ns[s], frows);
    Ns *= rad;
  }
}

// rotation by 2*alpha from (t, s) = (-tan(alpha/2), sin(alpha)): two
// three-shear rotations, each of determinant exactly 1 in any rounding
__device__ inline void lift2(float &x, float &y, float2 ts) {
  x = fmaf(ts.x, y, x);
  y = fmaf(ts.y, x, y);
  x = fmaf(ts.x, y, x);
  x = fmaf(ts.x, y, x);
  y = fmaf(ts.y, x, y);
  x = fmaf(ts.x, y, x);
}

// storage (FP64) <-> arithmetic type; FP32 conversions use integer instructions
template <typename R> __device__ inline typename CT<R>::T from_d(double2 v) {
  if constexpr (std::is_same<R, float>::value)
    return make_float2(d2f_rn(v.x), d2f_rn(v.y));
  else
    return v;
}
__device__ inline double2 to_d(double2 v) { return v; }
__device__ inline double2 to_d(float2 v) { return make_double2(f2d(v.x), f2d(v.y)); }
// psi_j storage: c128 in the FP64 form, c64 in the mixed form (one rounding)
__device__ inline void store_psi(double2 *p, double2 v) { *p = v; }
__device__ inline void store_psi(float2 *p, double2 v) { *p = make_float2(d2f_rn(v.x), d2f_rn(v.y)); }
// FP32 result (x, y) times the transform scale: exact power of two in FP32, else
// the product formed in FP64 and rounded once
__device__ inline float2 scaled_c64(float x, float y, float fscale, double scale) {
  if (fscale != 0.0f) return make_float2(x * fscale, y * fscale);
  return make_float2(d2f_rn(f2d(x) * scale), d2f_rn(f2d(y) * scale));
}

}  // namespace

// ---------------------------------------------------------- rows forward
template <typename R>
__global__ void __launch_bounds__(FFT_THREADS, std::is_same<R, float>::value ? 2 : 1) k_fft_rows(typename CT<R>::T *__restrict__ psi, Radices rd, int nrows,
                                                          int n_rows_total, const typename CT<R>::T *__restrict__ tw,
                                                          int inv, Grid g, double scale,
                                                          const SlabDesc *__restrict__ slabs,
                                                          const double2 *__restrict__ tabE,
                                                          double *__restrict__ re_part, int re_tiles,
                                                          const int *status, const float2 *__restrict__ liftR,
                                                          const float2 *__restrict__ liftr, float fscale,
                                                          FastDiv fn2) {
  if (status && *status) return;
  using C = typename CT<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *buf = reinterpret_cast<C *>(smem_raw);
  __shared__ double red[32];
  const int N = rd.n;
  const int row0 = blockIdx.x * nrows;
  const int n = nrows * N;
  // FP32 path: the rotational phase as separable three-shear rotations,
  // before the forward transform or after the inverse one
  const bool lift = std::is_same<R, float>::value && liftR != nullptr;
  {
    // all of this thread's loads are issued before any is used
    C raw[MAXV];
#pragma unroll
    for (int u = 0; u < MAXV; u++) {
      const int e = threadIdx.x + FFT_THREADS * u;
      const int grow = row0 + (int)fdiv(rd.fn, (uint32_t)e);
      raw[u] = (e < n && grow < n_rows_total) ? psi[(int64_t)row0 * N + e] : CT<R>::make(0, 0);
    }
#pragma unroll
    for (int u = 0; u < MAXV; u++) {
      const int e = threadIdx.x + FFT_THREADS * u;
      if (e >= n) break;
      const int rl = (int)fdiv(rd.fn, (uint32_t)e);
      const int grow = row0 + rl;
      C v = raw[u];
      if (lift && !inv && grow < n_rows_total) {
        const int sl = (int)fdiv(fn2, (uint32_t)grow);
        const int l = slabs[sl].l, i = e - rl * N, j = grow - sl * g.n2;
        float x = (float)v.x, y = (float)v.y;
        lift2(x, y, __ldg(liftR + (int64_t)l * g.n1 + i));
        lift2(x, y, __ldg(liftr + (int64_t)l * g.n2 + j));
        v.x = x;
        v.y = y;
      }
      buf[e] = v;
    }
  }
  __syncthreads();
  fft_run<R, false>(buf, rd, nrows, N, 1, tw, inv != 0, rd.fn);
  double re = 0.0;
  float ref = 0.0f;
  for (int e = threadIdx.x; e < n; e += FFT_THREADS) {
    const int rl = (int)fdiv(rd.fn, (uint32_t)e);
    const int grow = row0 + rl;
    if (grow >= n_rows_total) continue;
    const int i = e - rl * N;
    const int sl = (int)fdiv(fn2, (uint32_t)grow);
    const int j = grow - sl * g.n2;
    if constexpr (std::is_same<R, float>::value) {
     if (inv) {
      float x = (float)buf[e].x, y = (float)buf[e].y;
      if (fscale != 0.0f) {   // exact FP32 scale (power of two)
        x *= fscale;
        y *= fscale;
      }
      const int l = slabs[sl].l;
      if (lift) {
        lift2(x, y, __ldg(liftR + (int64_t)l * g.n1 + i));
        lift2(x, y, __ldg(liftr + (int64_t)l * g.n2 + j));
      }
      if (re_part) {
        const float Rr = (float)(g.left1 + i * g.dr1), rr = (float)(g.left2 + j * g.dr2);
        const float I = 1.0f / (2.0f * (float)g.m1 * Rr * Rr) + 1.0f / (2.0f * (float)g.m2 * rr * rr);
        const float s2 = fscale != 0.0f ? 1.0f : (float)(scale * scale);
        ref = fmaf((float)l * (float)(l + 1) * I * s2, x * x + y * y, ref);
      }
      psi[(int64_t)grow * N + i] = fscale != 0.0f ? make_float2(x, y) : scaled_c64(x, y, 0.0f, scale);
      continue;
     }
    }
    double2 v = to_d(buf[e]);
    if (scale != 1.0) { v.x *= scale; v.y *= scale; }
    if (tabE) {
      const int l = slabs[sl].l;
      v = cmul(v, ldg2(tabE + (int64_t)l * g.npt + (int64_t)j * g.n1 + i));
    }
    if (re_part) {
      const int l = slabs[sl].l;
      const double Rr = g.left1 + i * g.dr1, rr = g.left2 + j * g.dr2;
      const double I = 1.0 / (2 * g.m1 * Rr * Rr) + 1.0 / (2 * g.m2 * rr * rr);
      re += (double)l * (l + 1) * I * (v.x * v.x + v.y * v.y);
    }
    store_psi(psi + (int64_t)grow * N + i, v);
  }
  if (re_part) {
    re = block_sum(re + (double)ref, red);
    if (threadIdx.x == 0) {
      const int64_t sl = row0 / g.n2;
      const int tile = (int)((row0 % g.n2) / nrows);
      re_part[sl * re_tiles + tile] = re;
    }
  }
}

// ------------------------------------- columns: forward, kinetic, inverse
template <typename R>
__global__ void __launch_bounds__(FFT_THREADS, std::is_same<R, float>::value ? 2 : 1) k_fft_cols(typename CT<R>::T *__restrict__ psi, Radices rd, int ncols, Grid g,
                                                          const typename CT<R>::T *__restrict__ tw,
                                                          const double2 *__restrict__ tab_kin,
                                                          const double *__restrict__ T1, const double *__restrict__ T2,
                                                          double *__restrict__ ke_part, int ke_tiles,
                                                          const int *status, const float2 *__restrict__ kinR,
                                                          const float2 *__restrict__ kinr, const float *__restrict__ T1f,
                                                          const float *__restrict__ T2f, FastDiv fncols) {
  if (status && *status) return;
  using C = typename CT<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *buf = reinterpret_cast<C *>(smem_raw);
  __shared__ double red[32];
  const int N = rd.n;                 // = n2
  const int tiles = g.n1 / ncols;
  const int64_t sl = blockIdx.x / tiles;
  const int tile = blockIdx.x % tiles;
  const int i0 = tile * ncols;
  C *p = psi + sl * g.npt + i0;
  const int n = ncols * N;
  {
    C raw[MAXV];
#pragma unroll
    for (int u = 0; u < MAXV; u++) {
      const int e = threadIdx.x + FFT_THREADS * u;
      const int t = (int)fdiv(fncols, (uint32_t)e);
      raw[u] = e < n ? p[(int64_t)t * g.n1 + (e - t * ncols)] : CT<R>::make(0, 0);
    }
#pragma unroll
    for (int u = 0; u < MAXV; u++) {
      const int e = threadIdx.x + FFT_THREADS * u;
      if (e < n) buf[e] = raw[u];
    }
  }
  __syncthreads();
  fft_run<R, true>(buf, rd, ncols, 1, ncols, tw, false, fncols);
  double ke = 0.0;
  float kef = 0.0f;
  for (int e = threadIdx.x; e < n; e += FFT_THREADS) {
    const int t = (int)fdiv(fncols, (uint32_t)e), c = e - t * ncols;
    if (std::is_same<R, float>::value && kinR) {
      float x = (float)buf[e].x, y = (float)buf[e].y;
      lift2(x, y, __ldg(kinR + i0 + c));
      lift2(x, y, __ldg(kinr + t));
      kef = fmaf(__ldg(T1f + i0 + c) + __ldg(T2f + t), x * x + y * y, kef);
      buf[e].x = x;
      buf[e].y = y;
      continue;
    }
    double2 v = to_d(buf[e]);
    v = cmul(v, ldg2(tab_kin + (int64_t)t * g.n1 + i0 + c));
    ke += (__ldg(T1 + i0 + c) + __ldg(T2 + t)) * (v.x * v.x + v.y * v.y);
    buf[e] = from_d<R>(v);
  }
  ke += (double)kef;
  __syncthreads();
  fft_run<R, true>(buf, rd, ncols, 1, ncols, tw, true, fncols);
  for (int e = threadIdx.x; e < n; e += FFT_THREADS) {
    const int t = (int)fdiv(fncols, (uint32_t)e), c = e - t * ncols;
    p[(int64_t)t * g.n1 + c] = buf[e];
  }
  if (ke_part) {
    ke = block_sum(ke, red);
    if (threadIdx.x == 0) ke_part[sl * ke_tiles + tile] = ke;
  }
}

// ------------------------------------------------- single-pass slab FFT (FP32)
// One thread-block cluster of C CTAs per Legendre slab.  CTA c owns the rows
// r in [c n2/C, (c+1) n2/C) in Xr and, after the first exchange, the columns
// kR in [c n1/C, (c+1) n1/C) in Xc; the exchange reads and writes the other
// CTAs' shared memory directly (distributed shared memory).  HBM sees one read
// and one write per point instead of three of each.
constexpr int SLAB_THREADS = 512;
constexpr int SLAB_MV = 8;   // values per thread per stage: n1 n2 / C <= 4096

__global__ void __launch_bounds__(SLAB_THREADS, 2) k_fft_slab_cluster(
    float2 *__restrict__ psi, Radices r1d, Radices r2d, int C, Grid g, const SlabDesc *__restrict__ slabs,
    const float2 *__restrict__ tw1, const float2 *__restrict__ tw2, FFTLift lf, double *__restrict__ ke_part,
    double *__restrict__ re_part, float fscale, double scale, FastDiv fcols, const int *status) {
  if (status && *status) return;   // uniform over the cluster: every CTA reads the same flag
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32];
  const int n1 = g.n1, n2 = g.n2;
  const int rows = n2 / C, cols = n1 / C;
  float2 *Xr = reinterpret_cast<float2 *>(smem_raw);   // [rows][n1]
  float2 *Xc = Xr + rows * n1;                          // [n2][cols]
  float2 *tws1 = Xc + n2 * cols;                        // twiddle shears of n1 and n2
  float2 *tws2 = tws1 + n1;
  for (int q = threadIdx.x; q < n1; q += SLAB_THREADS) tws1[q] = __ldg(tw1 + q);
  for (int q = threadIdx.x; q < n2; q += SLAB_THREADS) tws2[q] = __ldg(tw2 + q);
  const int c = (int)cluster.block_rank();
  const int sl = blockIdx.x / C;
  const int l = slabs[sl].l;
  float2 *P = psi + (int64_t)sl * g.npt;
  const int r0 = c * rows, k0 = c * cols;
  const int n = rows * n1;   // == n2 * cols
  const int tid = threadIdx.x;

  // 1. rows -> Xr (FP32), rotational phase before the forward transform
  {
    float2 raw[SLAB_MV];
#pragma unroll
    for (int u = 0; u < SLAB_MV; u++) {
      const int e = tid + SLAB_THREADS * u;
      raw[u] = e < n ? __ldcs(P + (int64_t)r0 * n1 + e) : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int u = 0; u < SLAB_MV; u++) {
      const int e = tid + SLAB_THREADS * u;
      if (e >= n) break;
      float x = raw[u].x, y = raw[u].y;
      if (lf.proR) {
        const int rl = (int)fdiv(r1d.fn, (uint32_t)e);
        const int i = e - rl * n1;
        lift2(x, y, __ldg(lf.proR + (int64_t)l * n1 + i));
        lift2(x, y, __ldg(lf.pror + (int64_t)l * n2 + r0 + rl));
      }
      Xr[e] = make_float2(x, y);
    }
  }
  __syncthreads();
  fft_run<float, false, SLAB_THREADS, SLAB_MV>(Xr, r1d, rows, n1, 1, tws1, false, r1d.fn);
  cluster.sync();
  // 2. gather the columns of this CTA from every CTA's rows (all loads issued first)
  {
    float2 v[SLAB_MV];
#pragma unroll
    for (int u = 0; u < SLAB_MV; u++) {
      const int e = tid + SLAB_THREADS * u;
      if (e < n) {
        const int t = (int)fdiv(fcols, (uint32_t)e), cc = e - t * cols;
        const int owner = t / rows;
        const float2 *src = cluster.map_shared_rank(Xr, owner);
        v[u] = src[(t - owner * rows) * n1 + k0 + cc];
      }
    }
#pragma unroll
    for (int u = 0; u < SLAB_MV; u++) {
      const int e = tid + SLAB_THREADS * u;
      if (e < n) Xc[e] = v[u];
    }
  }
  __syncthreads();
  fft_run<float, true, SLAB_THREADS, SLAB_MV>(Xc, r2d, cols, 1, cols, tws2, false, fcols);
  float kef = 0.0f;
  for (int e = tid; e < n; e += SLAB_THREADS) {
    const int t = (int)fdiv(fcols, (uint32_t)e), cc = e - t * cols;
    float x = Xc[e].x, y = Xc[e].y;
    lift2(x, y, __ldg(lf.kinR + k0 + cc));
    lift2(x, y, __ldg(lf.kinr + t));
    kef = fmaf(__ldg(lf.T1f + k0 + cc) + __ldg(lf.T2f + t), x * x + y * y, kef);
    Xc[e] = make_float2(x, y);
  }
  __syncthreads();
  fft_run<float, true, SLAB_THREADS, SLAB_MV>(Xc, r2d, cols, 1, cols, tws2, true, fcols);
  cluster.sync();   // every CTA has finished reading the rows it gathered
  // 3. scatter the columns back into the owners' rows
  for (int e = tid; e < n; e += SLAB_THREADS) {
    const int t = (int)fdiv(fcols, (uint32_t)e), cc = e - t * cols;
    const int owner = t / rows;
    float2 *dst = cluster.map_shared_rank(Xr, owner);
    dst[(t - owner * rows) * n1 + k0 + cc] = Xc[e];
  }
  cluster.sync();   // every scatter into this CTA's rows has landed
  fft_run<float, false, SLAB_THREADS, SLAB_MV>(Xr, r1d, rows, n1, 1, tws1, true, r1d.fn);
  // 4. scale, rotational phase after the inverse transform, rotational energy, store
  float ref = 0.0f;
  const float lls2 = (float)l * (float)(l + 1) * (fscale != 0.0f ? 1.0f : (float)(scale * scale));
  for (int e = tid; e < n; e += SLAB_THREADS) {
    const int rl = (int)fdiv(r1d.fn, (uint32_t)e);
    const int i = e - rl * n1, j = r0 + rl;
    float x = Xr[e].x, y = Xr[e].y;
    if (fscale != 0.0f) {
      x *= fscale;
      y *= fscale;
    }
    if (lf.epiR) {
      lift2(x, y, __ldg(lf.epiR + (int64_t)l * n1 + i));
      lift2(x, y, __ldg(lf.epir + (int64_t)l * n2 + j));
    }
    if (re_part) {
      const float I = __ldg(lf.I1f + i) + __ldg(lf.I2f + j);
      ref = fmaf(lls2 * I, x * x + y * y, ref);
    }
    __stcs(P + (int64_t)r0 * n1 + e, fscale != 0.0f ? make_float2(x, y) : scaled_c64(x, y, 0.0f, scale));
  }
  const double ke = block_sum((double)kef, red);
  const double re = block_sum((double)ref, red);
  if (tid == 0) {
    if (ke_part) ke_part[(int64_t)sl * C + c] = ke;
    if (re_part) re_part[(int64_t)sl * C + c] = re;
  }
}

// ------------------------------------ separable single-pass slab FFT (FP32)
// The kinetic propagator is separable: with F = F1 (x) F2 and the phase
// K = K1 (x) K2,  F^-1 K F = (F1^-1 K1 F1) (x) (F2^-1 K2 F2).  So each slab is
// propagated by a complete forward-phase-inverse 1-D pass along R on every
// row, then one along r on every column, with a single cluster exchange in
// between (the 2-D form needs two).  Each 1-D transform of length N = A B is
// done in registers: B threads hold A values each, a length-A DFT with
// constant twiddles, the twiddles W_N^(j k1), one exchange through shared
// memory, then A/B length-B DFTs per thread; the inverse retraces the steps.
// Kinetic energy: sum (T1 + T2) |psi^|^2 over the 2-D spectrum equals
// n2 sum T1 |F1 psi|^2 + (1/n1) sum T2 |F2 (n1 A1 psi)|^2, A1 the unitary row
// propagator, so each pass accumulates its own term.
namespace {
// t = -tan(theta/2), s = sin(theta) of theta = u pi/24 (units of 7.5 degrees), u = 1..11
__device__ __forceinline__ float rot_tan_half(int u) {
  constexpr float T[12] = {0.0f, 6.554346281523822093e-02f, 1.316524975873958336e-01f, 1.989123673796580061e-01f,
                           2.679491924311226958e-01f, 3.394542588633758240e-01f, 4.142135623730950345e-01f,
                           4.931454260313040683e-01f, 5.773502691896257311e-01f, 6.681786379192988790e-01f,
                           7.673269879789603731e-01f, 8.769764629927567778e-01f};
  return T[u];
}
__device__ __forceinline__ float rot_sin(int u) {
  constexpr float S[12] = {0.0f, 1.305261922200515734e-01f, 2.588190451025207395e-01f, 3.826834323650897818e-01f,
                           0.5f, 6.087614290087206559e-01f, 7.071067811865474617e-01f, 7.933533402912351651e-01f,
                           8.660254037844385966e-01f, 9.238795325112867385e-01f, 9.659258262890683122e-01f,
                           9.914448613738103822e-01f};
  return S[u];
}

// v *= exp(i u pi/24) for a compile-time-known integer u (after unrolling):
// exact for multiples of pi/2, a three-shear rotation otherwise
__device__ __forceinline__ void rot48(float2 &v, int u) {
  u = ((u % 48) + 48) % 48;
  if (u > 24) u -= 48;   // (-24, 24]
  if (u > 12 || u < -12) {
    v.x = -v.x;
    v.y = -v.y;
    u += u > 0 ? -24 : 24;
  }
  if (u == 0) return;
  if (u == 12) {   // * i
    const float x = v.x;
    v.x = -v.y;
    v.y = x;
    return;
  }
  if (u == -12) {   // * -i
    const float x = v.x;
    v.x = v.y;
    v.y = -x;
    return;
  }
  const int a = u > 0 ? u : -u;
  const float t = u > 0 ? -rot_tan_half(a) : rot_tan_half(a);
  const float s = u > 0 ? rot_sin(a) : -rot_sin(a);
  float x = v.x, y = v.y;
  x = fmaf(t, y, x);
  y = fmaf(s, x, y);
  x = fmaf(t, y, x);
  v.x = x;
  v.y = y;
}

// In-register DFT of N values in natural order, N | 48 (products of 2, 3, 4);
// forward exp(-2 pi i jk/N), inverse exp(+2 pi i jk/N), unnormalised.
// N = P Q with P = 4 (or 3, 2): length-P DFTs over the stride-Q subsequences,
// twiddles W_N^(q k1) as exact rotations, then length-Q DFTs.
template <int N, bool INV> struct RegDFT {
  static __device__ __forceinline__ void run(float2 *v) {
    static_assert(48 % N == 0, "register DFT length divides 48");
    constexpr int P = (N % 4 == 0) ? 4 : ((N % 3 == 0) ? 3 : 2);
    constexpr int Q = N / P;
    float2 a[Q][P];
#pragma unroll
    for (int q = 0; q < Q; q++) {
#pragma unroll
      for (int p = 0; p < P; p++) a[q][p] = v[q + Q * p];
      RegDFT<P, INV>::run(a[q]);
#pragma unroll
      for (int k1 = 1; k1 < P; k1++) rot48(a[q][k1], (INV ? 48 : -48) * q * k1 / N);
    }
#pragma unroll
    for (int k1 = 0; k1 < P; k1++) {
      float2 b[Q];
#pragma unroll
      for (int q = 0; q < Q; q++) b[q] = a[q][k1];
      RegDFT<Q, INV>::run(b);
#pragma unroll
      for (int k2 = 0; k2 < Q; k2++) v[k1 + P * k2] = b[k2];
    }
  }
};
template <bool INV> struct RegDFT<1, INV> {
  static __device__ __forceinline__ void run(float2 *) {}
};
template <bool INV> struct RegDFT<2, INV> {
  static __device__ __forceinline__ void run(float2 *v) {
    const float2 a = v[0], b = v[1];
    v[0] = make_float2(a.x + b.x, a.y + b.y);
    v[1] = make_float2(a.x - b.x, a.y - b.y);
  }
};
template <bool INV> struct RegDFT<3, INV> {
  // sqrt(3)/2 as an FP32 pair: h s is formed to ~2^-48, so the butterfly
  // carries no fixed FP32 constant error (which would bias the norm)
  static __device__ __forceinline__ void run(float2 *v) {
    constexpr float H_HI = 0.8660253882408142f, H_LO = 1.5543625053737742e-08f;
    const float2 t = make_float2(v[1].x + v[2].x, v[1].y + v[2].y);
    const float2 d = make_float2(v[1].x - v[2].x, v[1].y - v[2].y);
    const float2 x0 = v[0];
    const float2 u = make_float2(fmaf(-0.5f, t.x, x0.x), fmaf(-0.5f, t.y, x0.y));
    const float hx = fmaf(H_LO, d.x, H_HI * d.x), hy = fmaf(H_LO, d.y, H_HI * d.y);
    // forward: w = -i h d ; inverse: +i h d
    const float2 w = INV ? make_float2(-hy, hx) : make_float2(hy, -hx);
    v[0] = make_float2(x0.x + t.x, x0.y + t.y);
    v[1] = make_float2(u.x + w.x, u.y + w.y);
    v[2] = make_float2(u.x - w.x, u.y - w.y);
  }
};
template <bool INV> struct RegDFT<4, INV> {
  static __device__ __forceinline__ void run(float2 *v) { dft<float, 4>(v, INV); }
};

// v *= W_n^(+-e) given its table entry w (three shears, see fft_stage)
__device__ __forceinline__ void tw_rotate(float2 &v, float2 w, int e, int n, bool inv) {
  if (e == 0) return;
  const float tt = inv ? -w.x : w.x, ss = inv ? -w.y : w.y;
  float x = v.x, y = v.y;
  if (4 * e > n && 4 * e < 3 * n) {
    x = -x;
    y = -y;
  }
  x = fmaf(tt, y, x);
  y = fmaf(ss, x, y);
  x = fmaf(tt, y, x);
  v.x = x;
  v.y = y;
}
// v *= W_n^(+-e) from the shared twiddle table indexed by e
__device__ __forceinline__ void tw_apply(float2 &v, const float2 *tab, int e, int n, bool inv) {
  if (e != 0) tw_rotate(v, tab[e], e, n, inv);
}
}  // namespace

// Layout: cluster of C CTAs per slab.  CTA c owns rows r in [c RPC, (c+1) RPC)
// (RPC = THREADS / B1, B1 threads per row) and columns R in [c CPC, (c+1) CPC)
// (CPC = n1 / C, B2 threads per column).  Row region of local row q: RS
// floats2 at Xr + q RS, used as the row transposition buffer and then as the
// row the other CTAs gather from.  Column transposition buffer Sc[k1][j][col].
// PIPE: a persistent grid of clusters walks the slabs (slab = cluster index +
// k x clusters); each thread loads its rows of the next slab into registers
// right after the current slab's rows are in shared memory, so that load
// overlaps the column phase.  Otherwise one cluster per slab.
template <int A, int B1, int B2, int THREADS, bool PIPE>
__global__ void __launch_bounds__(THREADS, PIPE ? 2 : (THREADS <= 256 ? 3 : 1))
    k_fft_slab_sep(float2 *__restrict__ psi, Grid g, const SlabDesc *__restrict__ slabs, int n_slabs,
                   const float2 *__restrict__ tw1, const float2 *__restrict__ tw2, FFTLift lf,
                   double *__restrict__ ke_part, double *__restrict__ re_part, float fscale, double scale,
                   const int *status) {
  constexpr int N1 = A * B1, N2 = A * B2;
  constexpr int RPC = THREADS / B1;
  constexpr int C = N2 / RPC;
  constexpr int CPC = N1 / C;
  constexpr int RS = A * (B1 + 1);
  static_assert(THREADS % B1 == 0 && N2 % RPC == 0 && N1 % C == 0 && CPC * B2 == THREADS, "slab tiling");
  static_assert(A % B1 == 0 && A % B2 == 0 && 32 % B1 == 0, "transform factors");
  if (status && *status) return;   // uniform over the cluster
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32];
  float2 *Xr = reinterpret_cast<float2 *>(smem_raw);
  float2 *Sc = Xr + RPC * RS;
  float2 *t1 = Sc + A * B2 * CPC;
  float2 *t2 = t1 + N1;
  const int tid = threadIdx.x;
  const int c = (int)cluster.block_rank();
  const int ncl = PIPE ? (int)(gridDim.x / C) : n_slabs;
  const int q = tid / B1, j = tid % B1;   // row phase: thread j of local row q
  const int r = c * RPC + q;
  float2 v[A];
  int sl = blockIdx.x / C;
  if (sl < n_slabs) {
    const float2 *src = psi + (int64_t)sl * g.npt + (int64_t)r * N1 + j;
#pragma unroll
    for (int m = 0; m < A; m++) v[m] = __ldcs(src + B1 * m);
  }
  for (int p = tid; p < N1; p += THREADS) t1[p] = __ldg(tw1 + p);
  for (int p = tid; p < N2; p += THREADS) t2[p] = __ldg(tw2 + p);
  __syncthreads();   // twiddle tables
  for (; sl < n_slabs; sl += ncl) {
  const int l = slabs[sl].l;
  float2 *P = psi + (int64_t)sl * g.npt;
  float ke1 = 0.0f, ke2 = 0.0f, ref = 0.0f;

  // ======== rows: thread j of row group q holds x[j + B1 m], m < A
  {
    if (lf.proR) {
      const float2 pr = __ldg(lf.pror + (int64_t)l * N2 + r);
#pragma unroll
      for (int m = 0; m < A; m++) {
        lift2(v[m].x, v[m].y, __ldg(lf.proR + (int64_t)l * N1 + j + B1 * m));
        lift2(v[m].x, v[m].y, pr);
      }
    }
    float2 *G = Xr + q * RS;
    RegDFT<A, false>::run(v);
#pragma unroll
    for (int k1 = 1; k1 < A; k1++) tw_apply(v[k1], t1, j * k1, N1, false);
#pragma unroll
    for (int k1 = 0; k1 < A; k1++) G[k1 * (B1 + 1) + j] = v[k1];
    __syncwarp();
    // thread t now takes k1 = t + B1 h, h < A / B1, over all j
    float2 w[A];
#pragma unroll
    for (int h = 0; h < A / B1; h++)
#pragma unroll
      for (int jj = 0; jj < B1; jj++) w[h * B1 + jj] = G[(j + B1 * h) * (B1 + 1) + jj];
#pragma unroll
    for (int h = 0; h < A / B1; h++) {
      RegDFT<B1, false>::run(w + h * B1);
#pragma unroll
      for (int k2 = 0; k2 < B1; k2++) {   // frequency kR = k1 + A k2
        const int kR = j + B1 * h + A * k2;
        float2 &z = w[h * B1 + k2];
        ke1 = fmaf(__ldg(lf.T1f + kR), z.x * z.x + z.y * z.y, ke1);
        lift2(z.x, z.y, __ldg(lf.kinR + kR));
      }
      RegDFT<B1, true>::run(w + h * B1);
#pragma unroll
      for (int jj = 1; jj < B1; jj++) tw_apply(w[h * B1 + jj], t1, jj * (j + B1 * h), N1, true);
    }
    __syncwarp();
#pragma unroll
    for (int h = 0; h < A / B1; h++)
#pragma unroll
      for (int jj = 0; jj < B1; jj++) G[(j + B1 * h) * (B1 + 1) + jj] = w[h * B1 + jj];
    __syncwarp();
#pragma unroll
    for (int k1 = 0; k1 < A; k1++) v[k1] = G[k1 * (B1 + 1) + j];
    RegDFT<A, true>::run(v);
    __syncwarp();
#pragma unroll
    for (int m = 0; m < A; m++) G[j + B1 * m] = v[m];
  }
  cluster.sync();   // every row of the slab is in its owner's shared memory
  float2 vn[PIPE ? A : 1];
  if (PIPE && sl + ncl < n_slabs) {   // the next slab's rows, in flight during the column phase
    const float2 *src = psi + (int64_t)(sl + ncl) * g.npt + (int64_t)r * N1 + j;
#pragma unroll
    for (int m = 0; m < (PIPE ? A : 1); m++) vn[m] = __ldcs(src + B1 * m);
  }

  // ======== columns: thread jc of column col holds x[r = jc + B2 m], m < A
  const int col = tid % CPC, jc = tid / CPC;
  const int R = c * CPC + col;
#pragma unroll
  for (int m = 0; m < A; m++) {
    const int rr = jc + B2 * m;
    const int owner = rr / RPC;
    const float2 *src = cluster.map_shared_rank(Xr, owner);
    v[m] = src[(rr - owner * RPC) * RS + R];
  }
  RegDFT<A, false>::run(v);
  // the gathered values are consumed: other CTAs may finish once all arrive
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
#pragma unroll
  for (int k1 = 1; k1 < A; k1++) tw_apply(v[k1], t2, jc * k1, N2, false);
#pragma unroll
  for (int k1 = 0; k1 < A; k1++) Sc[(k1 * B2 + jc) * CPC + col] = v[k1];
  __syncthreads();
  {
    float2 w[A];
#pragma unroll
    for (int h = 0; h < A / B2; h++)
#pragma unroll
      for (int jj = 0; jj < B2; jj++) w[h * B2 + jj] = Sc[((jc + B2 * h) * B2 + jj) * CPC + col];
#pragma unroll
    for (int h = 0; h < A / B2; h++) {
      RegDFT<B2, false>::run(w + h * B2);
#pragma unroll
      for (int k2 = 0; k2 < B2; k2++) {   // frequency kr = k1 + A k2
        const int kr = jc + B2 * h + A * k2;
        float2 &z = w[h * B2 + k2];
        ke2 = fmaf(__ldg(lf.T2f + kr), z.x * z.x + z.y * z.y, ke2);
        lift2(z.x, z.y, __ldg(lf.kinr + kr));
      }
      RegDFT<B2, true>::run(w + h * B2);
#pragma unroll
      for (int jj = 1; jj < B2; jj++) tw_apply(w[h * B2 + jj], t2, jj * (jc + B2 * h), N2, true);
    }
    __syncthreads();
#pragma unroll
    for (int h = 0; h < A / B2; h++)
#pragma unroll
      for (int jj = 0; jj < B2; jj++) Sc[((jc + B2 * h) * B2 + jj) * CPC + col] = w[h * B2 + jj];
  }
  __syncthreads();
#pragma unroll
  for (int k1 = 0; k1 < A; k1++) v[k1] = Sc[(k1 * B2 + jc) * CPC + col];
  RegDFT<A, true>::run(v);

  // ======== scale, rotational phase after the inverse transform, rotational energy, store
  const float lls2 = (float)l * (float)(l + 1) * (fscale != 0.0f ? 1.0f : (float)(scale * scale));
  const float2 eR = lf.epiR ? __ldg(lf.epiR + (int64_t)l * N1 + R) : make_float2(0.0f, 0.0f);
  const float I1 = re_part ? __ldg(lf.I1f + R) : 0.0f;
#pragma unroll
  for (int m = 0; m < A; m++) {
    const int rr = jc + B2 * m;
    float x = v[m].x, y = v[m].y;
    if (fscale != 0.0f) {
      x *= fscale;
      y *= fscale;
    }
    if (lf.epiR) {
      lift2(x, y, eR);
      lift2(x, y, __ldg(lf.epir + (int64_t)l * N2 + rr));
    }
    if (re_part) ref = fmaf(lls2 * (I1 + __ldg(lf.I2f + rr)), x * x + y * y, ref);
    __stcs(P + (int64_t)rr * N1 + R, fscale != 0.0f ? make_float2(x, y) : scaled_c64(x, y, 0.0f, scale));
  }
  // partial sums: FP32 within a warp and across warps, in a fixed order
  float kew = fmaf((float)N2, ke1, ke2 * (1.0f / (float)N1)), rew = ref;
  for (int o = 16; o > 0; o >>= 1) {
    kew += __shfl_down_sync(0xffffffffu, kew, o);
    rew += __shfl_down_sync(0xffffffffu, rew, o);
  }
  float2 *red2 = reinterpret_cast<float2 *>(red);
  if ((tid & 31) == 0) red2[tid >> 5] = make_float2(kew, rew);
  __syncthreads();
  if (tid == 0) {   // FP32 over the warps (FP64 conversions would queue on the slow FP64 pipe)
    float ke = 0.0f, re = 0.0f;
    for (int w = 0; w < THREADS / 32; w++) {
      ke += red2[w].x;
      re += red2[w].y;
    }
    if (ke_part) ke_part[(int64_t)sl * C + c] = (double)ke;
    if (re_part) re_part[(int64_t)sl * C + c] = (double)re;
  }
  // no CTA leaves, or rewrites its rows, while another may still read them
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
  if (PIPE) {
#pragma unroll
    for (int m = 0; m < (PIPE ? A : 1); m++) v[m] = vn[m];
  }
  }
}

// ---------------------------------------------------------- two-pass form
// The separable transform as two independent passes with no cluster: a row pass
// (rotational phase before the transform, forward row FFT, kinetic phase along R and
// its energy, inverse) writes each slab back in natural order, where it stays in L2,
// and a column pass (forward column FFT, kinetic phase along r and its energy,
// inverse, scale, epilogue phase, rotational energy) finishes it.  Same arithmetic as
// k_fft_slab_sep; what changes is that no CTA waits for another (no cluster barrier,
// no distributed-shared-memory gather), and every table a CTA needs (per-l phases,
// kinetic phase and energy weights, twiddles) is fetched into shared memory right at its
// start, beside the slab's own loads.
//
// Row transposition buffer: element (a, b), a < A, b < B1, of a row at a B1 + (b ^ (a mod
// B1)) (an XOR swizzle instead of padding), rows RS apart; the twiddle table W^(a b)
// uses the same swizzle, so the forward (a uniform in a half-warp) and inverse (b
// uniform) lookups are both free of bank conflicts.
template <int A, int B1>
constexpr int split_row_stride() {
  return A * B1 + (B1 == 16 ? 0 : B1);
}
// W resident warps per SM (24: about 80 registers a thread, 32: 64)
template <int A, int B1, int B2, int T, int W>
__global__ void __launch_bounds__(T, W * 32 / T)
    k_fft_split_rows(float2 *__restrict__ psi, Grid g, const SlabDesc *__restrict__ slabs,
                     const float2 *__restrict__ tw1, FFTLift lf, double *__restrict__ ke_part, int ke_tiles,
                     const int *status) {
  constexpr int N1 = A * B1, N2 = A * B2;
  constexpr int RPC = T / B1;   // rows per CTA
  constexpr int CR = N2 / RPC;  // CTAs per slab
  constexpr int RS = split_row_stride<A, B1>();
  static_assert(T % B1 == 0 && N2 % RPC == 0 && A % B1 == 0 && 32 % B1 == 0 && N1 % 16 == 0, "row tiling");
  if (status && *status) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ float red[T / 32];
  float2 *tw = reinterpret_cast<float2 *>(smem_raw);
  float2 *X = tw + N1;
  float2 *pro = X + RPC * RS;
  float2 *kin = pro + N1;
  float *t1s = reinterpret_cast<float *>(kin + N1);
  const int tid = threadIdx.x;
  const int sl = blockIdx.x / CR, c = blockIdx.x % CR;
  const int l = __ldg(&slabs[sl].l);
  const int q = tid / B1, j = tid % B1;
  const int r = c * RPC + q;
  float2 *row = psi + (int64_t)sl * g.npt + (int64_t)r * N1;
  float2 v[A];
#pragma unroll
  for (int m = 0; m < A; m++) v[m] = __ldcs(row + j + B1 * m);
  for (int p = tid; p < N1; p += T) {
    const int a = p / B1, b = (p % B1) ^ (a % B1);
    tw[p] = __ldg(tw1 + a * b);
    if (lf.proR) pro[p] = __ldg(lf.proR + (int64_t)l * N1 + p);
    kin[p] = __ldg(lf.kinR + p);
    t1s[p] = __ldg(lf.T1f + p);
  }
  const float2 pr = lf.proR ? __ldg(lf.pror + (int64_t)l * N2 + r) : make_float2(0.0f, 0.0f);
  __syncthreads();

  if (lf.proR) {
#pragma unroll
    for (int m = 0; m < A; m++) {
      lift2(v[m].x, v[m].y, pro[j + B1 * m]);
      lift2(v[m].x, v[m].y, pr);
    }
  }
  float2 *G = X + q * RS;
  float ke1 = 0.0f;
  RegDFT<A, false>::run(v);
#pragma unroll
  for (int k1 = 1; k1 < A; k1++) tw_rotate(v[k1], tw[k1 * B1 + (j ^ (k1 % B1))], j * k1, N1, false);
#pragma unroll
  for (int k1 = 0; k1 < A; k1++) G[k1 * B1 + (j ^ (k1 % B1))] = v[k1];
  __syncwarp();
  float2 w[A];
#pragma unroll
  for (int h = 0; h < A / B1; h++)
#pragma unroll
    for (int jj = 0; jj < B1; jj++) w[h * B1 + jj] = G[(j + B1 * h) * B1 + (jj ^ j)];
#pragma unroll
  for (int h = 0; h < A / B1; h++) {
    RegDFT<B1, false>::run(w + h * B1);
#pragma unroll
    for (int k2 = 0; k2 < B1; k2++) {   // frequency kR = k1 + A k2
      const int kR = j + B1 * h + A * k2;
      float2 &z = w[h * B1 + k2];
      ke1 = fmaf(t1s[kR], z.x * z.x + z.y * z.y, ke1);
      lift2(z.x, z.y, kin[kR]);
    }
    RegDFT<B1, true>::run(w + h * B1);
#pragma unroll
    for (int jj = 1; jj < B1; jj++) {
      const int a = j + B1 * h;
      tw_rotate(w[h * B1 + jj], tw[a * B1 + (jj ^ j)], a * jj, N1, true);
    }
  }
  __syncwarp();
#pragma unroll
  for (int h = 0; h < A / B1; h++)
#pragma unroll
    for (int jj = 0; jj < B1; jj++) G[(j + B1 * h) * B1 + (jj ^ j)] = w[h * B1 + jj];
  __syncwarp();
#pragma unroll
  for (int k1 = 0; k1 < A; k1++) v[k1] = G[k1 * B1 + (j ^ (k1 % B1))];
  RegDFT<A, true>::run(v);
#pragma unroll
  for (int m = 0; m < A; m++) row[j + B1 * m] = v[m];   // natural order; read back by the column pass

  float kew = (float)N2 * ke1;
  for (int o = 16; o > 0; o >>= 1) kew += __shfl_down_sync(0xffffffffu, kew, o);
  if ((tid & 31) == 0) red[tid >> 5] = kew;
  __syncthreads();
  if (tid == 0) {   // FP32 over the warps, in a fixed order
    float ke = 0.0f;
    for (int wi = 0; wi < T / 32; wi++) ke += red[wi];
    if (ke_part) ke_part[(int64_t)sl * ke_tiles + c] = (double)ke;
  }
}

template <int A, int B1, int B2, int T, int W>
__global__ void __launch_bounds__(T, W * 32 / T)
    k_fft_split_cols(float2 *__restrict__ psi, Grid g, const SlabDesc *__restrict__ slabs,
                     const float2 *__restrict__ tw2, FFTLift lf, double *__restrict__ ke_part, int ke_tiles,
                     double *__restrict__ re_part, int re_tiles, float fscale, double scale, const int *status) {
  constexpr int N1 = A * B1, N2 = A * B2;
  constexpr int CPC = T / B2;        // columns per CTA
  constexpr int CC = N1 / CPC;       // CTAs per slab
  static_assert(T % B2 == 0 && N1 % CPC == 0 && A % B2 == 0, "column tiling");
  static_assert(N2 / (T / B1) == CC, "both passes have A B1 B2 / T CTAs per slab");
  if (status && *status) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ float2 red[T / 32];
  float2 *t2 = reinterpret_cast<float2 *>(smem_raw);
  float2 *Sc = t2 + N2;
  float2 *epi = Sc + A * B2 * CPC;
  float2 *kin = epi + N2;
  float *i2 = reinterpret_cast<float *>(kin + N2);
  float *t2s = i2 + N2;
  const int tid = threadIdx.x;
  const int sl = blockIdx.x / CC, c = blockIdx.x % CC;
  const int l = __ldg(&slabs[sl].l);
  const int col = tid % CPC, jc = tid / CPC;
  const int R = c * CPC + col;
  float2 *P = psi + (int64_t)sl * g.npt;
  for (int p = tid; p < N2; p += T) {
    t2[p] = __ldg(tw2 + p);
    if (lf.epiR) epi[p] = __ldg(lf.epir + (int64_t)l * N2 + p);
    if (re_part) i2[p] = __ldg(lf.I2f + p);
    kin[p] = __ldg(lf.kinr + p);
    t2s[p] = __ldg(lf.T2f + p);
  }
  const float2 eR = lf.epiR ? __ldg(lf.epiR + (int64_t)l * N1 + R) : make_float2(0.0f, 0.0f);
  const float I1 = re_part ? __ldg(lf.I1f + R) : 0.0f;
  float2 v[A];
#pragma unroll
  for (int m = 0; m < A; m++) v[m] = __ldcs(P + (int64_t)(jc + B2 * m) * N1 + R);
  __syncthreads();

  float ke2 = 0.0f, ref = 0.0f;
  RegDFT<A, false>::run(v);
#pragma unroll
  for (int k1 = 1; k1 < A; k1++) tw_apply(v[k1], t2, jc * k1, N2, false);
#pragma unroll
  for (int k1 = 0; k1 < A; k1++) Sc[(k1 * B2 + jc) * CPC + col] = v[k1];
  __syncthreads();
  {
    float2 w[A];
#pragma unroll
    for (int h = 0; h < A / B2; h++)
#pragma unroll
      for (int jj = 0; jj < B2; jj++) w[h * B2 + jj] = Sc[((jc + B2 * h) * B2 + jj) * CPC + col];
#pragma unroll
    for (int h = 0; h < A / B2; h++) {
      RegDFT<B2, false>::run(w + h * B2);
#pragma unroll
      for (int k2 = 0; k2 < B2; k2++) {   // frequency kr = k1 + A k2
        const int kr = jc + B2 * h + A * k2;
        float2 &z = w[h * B2 + k2];
        ke2 = fmaf(t2s[kr], z.x * z.x + z.y * z.y, ke2);
        lift2(z.x, z.y, kin[kr]);
      }
      RegDFT<B2, true>::run(w + h * B2);
#pragma unroll
      for (int jj = 1; jj < B2; jj++) tw_apply(w[h * B2 + jj], t2, jj * (jc + B2 * h), N2, true);
    }
    __syncthreads();
#pragma unroll
    for (int h = 0; h < A / B2; h++)
#pragma unroll
      for (int jj = 0; jj < B2; jj++) Sc[((jc + B2 * h) * B2 + jj) * CPC + col] = w[h * B2 + jj];
  }
  __syncthreads();
#pragma unroll
  for (int k1 = 0; k1 < A; k1++) v[k1] = Sc[(k1 * B2 + jc) * CPC + col];
  RegDFT<A, true>::run(v);

  // scale, rotational phase after the inverse transform, rotational energy, store
  const float lls2 = (float)l * (float)(l + 1) * (fscale != 0.0f ? 1.0f : (float)(scale * scale));
#pragma unroll
  for (int m = 0; m < A; m++) {
    const int rr = jc + B2 * m;
    float x = v[m].x, y = v[m].y;
    if (fscale != 0.0f) {
      x *= fscale;
      y *= fscale;
    }
    if (lf.epiR) {
      lift2(x, y, eR);
      lift2(x, y, epi[rr]);
    }
    if (re_part) ref = fmaf(lls2 * (I1 + i2[rr]), x * x + y * y, ref);
    __stcs(P + (int64_t)rr * N1 + R, fscale != 0.0f ? make_float2(x, y) : scaled_c64(x, y, 0.0f, scale));
  }
  float kew = ke2 * (1.0f / (float)N1), rew = ref;
  for (int o = 16; o > 0; o >>= 1) {
    kew += __shfl_down_sync(0xffffffffu, kew, o);
    rew += __shfl_down_sync(0xffffffffu, rew, o);
  }
  if ((tid & 31) == 0) red[tid >> 5] = make_float2(kew, rew);
  __syncthreads();
  if (tid == 0) {
    float ke = 0.0f, re = 0.0f;
    for (int wi = 0; wi < T / 32; wi++) {
      ke += red[wi].x;
      re += red[wi].y;
    }
    // the row pass's CTA c left its kinetic partial in this slot: one partial per CTA pair
    if (ke_part) ke_part[(int64_t)sl * ke_tiles + c] += (double)ke;
    if (re_part) re_part[(int64_t)sl * re_tiles + c] = (double)re;
  }
}

namespace {
// instantiations of the separable slab FFT: (n1, n2) -> (A, B1, B2, threads, mode).  Mode 0:
// one cluster per slab (C = A B2 B1 / threads CTAs); 1: a persistent grid of such clusters;
// 2 and 3: the two-pass form (row pass, then column pass, no cluster) built for 24 and 32
// resident warps per SM.  Several thread counts exist for the production grids; the
// autotuner times them on the session's own slabs.
struct SepShape {
  int n1, n2, A, B1, B2, threads, mode;
};
constexpr SepShape kSepShapes[] = {
    {256, 128, 16, 16, 8, 256, 0},
    {192, 96, 24, 8, 4, 96, 0},
    {64, 32, 8, 8, 4, 128, 0},
    {32, 16, 8, 4, 2, 32, 0},
    {16, 8, 4, 4, 2, 32, 0},
    {256, 128, 16, 16, 8, 512, 0},
    {256, 128, 16, 16, 8, 128, 0},
    {192, 96, 24, 8, 4, 192, 0},
    {192, 96, 24, 8, 4, 384, 0},
    {256, 128, 16, 16, 8, 256, 1},
    {192, 96, 24, 8, 4, 192, 1},
    {192, 96, 24, 8, 4, 96, 1},
    {256, 128, 16, 16, 8, 256, 2},
    {256, 128, 16, 16, 8, 256, 3},
    {256, 128, 16, 16, 8, 128, 3},
    {192, 96, 24, 8, 4, 192, 2},
    {192, 96, 24, 8, 4, 96, 2},
    {192, 96, 24, 8, 4, 192, 3},
};
constexpr int kNumSep = (int)(sizeof(kSepShapes) / sizeof(kSepShapes[0]));

template <int A, int B1, int B2, int T>
size_t sep_smem_bytes() {
  constexpr int RPC = T / B1, C = A * B2 / RPC, CPC = A * B1 / C;
  return ((size_t)RPC * A * (B1 + 1) + (size_t)A * B2 * CPC + A * B1 + A * B2) * sizeof(float2);
}
template <int A, int B1, int B2, int T>
int sep_cluster() {
  return A * B2 / (T / B1);
}
// two-pass form: shared memory of each pass, CTAs per slab of each pass
template <int A, int B1, int B2, int T>
size_t split_rows_smem() {
  return (size_t)A * B1 * sizeof(float2) + ((size_t)(T / B1) * split_row_stride<A, B1>() + 2 * A * B1) * sizeof(float2) +
         (size_t)A * B1 * sizeof(float);
}
template <int A, int B1, int B2, int T>
size_t split_cols_smem() {
  return (size_t)A * B2 * sizeof(float2) + ((size_t)A * B2 * (T / B2) + 2 * A * B2) * sizeof(float2) +
         2 * (size_t)A * B2 * sizeof(float);
}
template <int A, int B1, int B2, int T>
constexpr int split_row_ctas() {
  return A * B2 / (T / B1);
}
template <int A, int B1, int B2, int T>
constexpr int split_col_ctas() {
  return A * B1 / (T / B2);
}

// kinetic-energy and rotational-energy partials per slab: one per CTA of the cluster, or one
// per CTA of the column pass (its CTA c adds the row pass's CTA c to its own kinetic partial)
template <int A, int B1, int B2, int T, int MODE>
int shape_ke_tiles() {
  if constexpr (MODE >= 2)
    return split_col_ctas<A, B1, B2, T>();
  else
    return sep_cluster<A, B1, B2, T>();
}
template <int A, int B1, int B2, int T, int MODE>
int shape_re_tiles() {
  if constexpr (MODE >= 2)
    return split_col_ctas<A, B1, B2, T>();
  else
    return sep_cluster<A, B1, B2, T>();
}

template <int A, int B1, int B2, int T, int MODE>
void sep_set_attr() {
  if constexpr (MODE >= 2) {
    constexpr int W = MODE == 2 ? 24 : 32;
    QD_CUDA(cudaFuncSetAttribute(k_fft_split_rows<A, B1, B2, T, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)split_rows_smem<A, B1, B2, T>()));
    QD_CUDA(cudaFuncSetAttribute(k_fft_split_cols<A, B1, B2, T, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)split_cols_smem<A, B1, B2, T>()));
  } else {
    QD_CUDA(cudaFuncSetAttribute(k_fft_slab_sep<A, B1, B2, T, MODE == 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sep_smem_bytes<A, B1, B2, T>()));
    if (sep_cluster<A, B1, B2, T>() > 8)
      QD_CUDA(cudaFuncSetAttribute(k_fft_slab_sep<A, B1, B2, T, MODE == 1>,
                                   cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  }
}

template <int A, int B1, int B2, int T, bool PIPE>
void sep_launch(cudaStream_t s, const Grid &g, const FFTPlan &p, float2 *psi_j, const SlabDesc *slabs, int n_slabs,
                const FFTLift &lf, double *ke_part, double *re_part, float fscale, double scale, const int *status) {
  const int C = sep_cluster<A, B1, B2, T>();
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)(n_slabs * C));
  cfg.blockDim = dim3(T);
  cfg.dynamicSmemBytes = sep_smem_bytes<A, B1, B2, T>();
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (PIPE) {
    // as many clusters as fit on the device at once (all of them resident: the slab loop
    // needs no cluster to wait for another), at most one per slab
    static int resident[64] = {};   // per instantiation, per device
    int dev = 0;
    QD_CUDA(cudaGetDevice(&dev));
    int &n = resident[dev & 63];
    if (n == 0) {
      int k = 0;
      n = cudaOccupancyMaxActiveClusters(&k, k_fft_slab_sep<A, B1, B2, T, PIPE>, &cfg) == cudaSuccess && k > 0 ? k : -1;
      if (n < 0) cudaGetLastError();
    }
    if (n > 0) cfg.gridDim = dim3((unsigned)(std::min(n_slabs, n) * C));
  }
  QD_CUDA(cudaLaunchKernelEx(&cfg, k_fft_slab_sep<A, B1, B2, T, PIPE>, psi_j, g, slabs, n_slabs,
                             (const float2 *)p.tw1_f, (const float2 *)p.tw2_f, lf, ke_part, re_part, fscale, scale,
                             status));
}

template <int A, int B1, int B2, int T, int W>
void split_launch(cudaStream_t s, const Grid &g, const FFTPlan &p, float2 *psi_j, const SlabDesc *slabs, int n_slabs,
                  const FFTLift &lf, double *ke_part, double *re_part, float fscale, double scale, const int *status) {
  const int ke_tiles = shape_ke_tiles<A, B1, B2, T, 2>(), re_tiles = shape_re_tiles<A, B1, B2, T, 2>();
  k_fft_split_rows<A, B1, B2, T, W>
      <<<(unsigned)(n_slabs * split_row_ctas<A, B1, B2, T>()), T, split_rows_smem<A, B1, B2, T>(), s>>>(
          psi_j, g, slabs, (const float2 *)p.tw1_f, lf, ke_part, ke_tiles, status);
  QD_CUDA(cudaGetLastError());
  k_fft_split_cols<A, B1, B2, T, W>
      <<<(unsigned)(n_slabs * split_col_ctas<A, B1, B2, T>()), T, split_cols_smem<A, B1, B2, T>(), s>>>(
          psi_j, g, slabs, (const float2 *)p.tw2_f, lf, ke_part, ke_tiles, re_part, re_tiles, fscale, scale, status);
  QD_CUDA(cudaGetLastError());
}

#define QD_SEP_CASES(X)     \
  X(0, 16, 16, 8, 256, 0)   \
  X(1, 24, 8, 4, 96, 0)     \
  X(2, 8, 8, 4, 128, 0)     \
  X(3, 8, 4, 2, 32, 0)      \
  X(4, 4, 4, 2, 32, 0)      \
  X(5, 16, 16, 8, 512, 0)   \
  X(6, 16, 16, 8, 128, 0)   \
  X(7, 24, 8, 4, 192, 0)    \
  X(8, 24, 8, 4, 384, 0)    \
  X(9, 16, 16, 8, 256, 1)   \
  X(10, 24, 8, 4, 192, 1)   \
  X(11, 24, 8, 4, 96, 1)    \
  X(12, 16, 16, 8, 256, 2)  \
  X(13, 16, 16, 8, 256, 3)  \
  X(14, 16, 16, 8, 128, 3)  \
  X(15, 24, 8, 4, 192, 2)   \
  X(16, 24, 8, 4, 96, 2)    \
  X(17, 24, 8, 4, 192, 3)

void sep_dispatch_attr(int id) {
  switch (id) {
#define QD_X(i, a, b1, b2, t, mode) \
  case i: sep_set_attr<a, b1, b2, t, mode>(); break;
    QD_SEP_CASES(QD_X)
#undef QD_X
  }
}
int sep_dispatch_ke_tiles(int id) {
  switch (id) {
#define QD_X(i, a, b1, b2, t, mode) \
  case i: return shape_ke_tiles<a, b1, b2, t, mode>();
    QD_SEP_CASES(QD_X)
#undef QD_X
  }
  return 0;
}
int sep_dispatch_re_tiles(int id) {
  switch (id) {
#define QD_X(i, a, b1, b2, t, mode) \
  case i: return shape_re_tiles<a, b1, b2, t, mode>();
    QD_SEP_CASES(QD_X)
#undef QD_X
  }
  return 0;
}
void sep_dispatch_launch(int id, cudaStream_t s, const Grid &g, const FFTPlan &p, float2 *psi_j,
                         const SlabDesc *slabs, int n_slabs, const FFTLift &lf, double *ke_part, double *re_part,
                         float fscale, double scale, const int *status) {
  switch (id) {
#define QD_X(i, a, b1, b2, t, mode)                                                                               \
  case i:                                                                                                          \
    if constexpr (mode >= 2)                                                                                       \
      split_launch<a, b1, b2, t, mode == 2 ? 24 : 32>(s, g, p, psi_j, slabs, n_slabs, lf, ke_part, re_part, fscale, \
                                                      scale, status);                                              \
    else                                                                                                           \
      sep_launch<a, b1, b2, t, mode == 1>(s, g, p, psi_j, slabs, n_slabs, lf, ke_part, re_part, fscale, scale,    \
                                          status);                                                                 \
    break;
    QD_SEP_CASES(QD_X)
#undef QD_X
  }
}
}  // namespace

// ------------------------------------------------------------- host side
bool fft_factor(int n, int *rad, int *nst) {
  int k = 0;
  int m = n;
  while (m % 4 == 0) { rad[k++] = 4; m /= 4; }
  while (m % 2 == 0) { rad[k++] = 2; m /= 2; }
  while (m % 3 == 0) { rad[k++] = 3; m /= 3; }
  *nst = k;
  return m == 1 && k <= 16;
}

static int largest_divisor_at_most(int n, int cap) {
  for (int d = std::min(n, cap); d >= 1; d--)
    if (n % d == 0) return d;
  return 1;
}

// Cluster size of the single-pass FP32 slab FFT: the smallest C in {1,2,4,8}
// dividing n1 and n2 whose two FP32 buffers (2 n1 n2 / C * 8 bytes) fit in
// 100 KB and whose per-thread stage load stays within MAXV; 0 = not usable.
static int choose_cluster(int n1, int n2) {
  for (int C = 1; C <= 8; C *= 2) {
    if (n1 % C || n2 % C) continue;
    const int64_t per = (int64_t)n1 * n2 / C;
    if ((per * 2 + n1 + n2) * 8 > 100 * 1024) continue;
    if (per > (int64_t)SLAB_THREADS * SLAB_MV) continue;
    return C;
  }
  return 0;
}

void fft_plan_init(FFTPlan &p, int n1, int n2) {
  p.n1 = n1;
  p.n2 = n2;
  if (!fft_factor(n1, p.rad1, &p.nst1) || !fft_factor(n2, p.rad2, &p.nst2))
    throw Error{QD_ERR_UNSUPPORTED, "FFT grid sizes must factor into 2 and 3"};
  if (n1 > FFT_THREADS * MAXV || n2 > FFT_THREADS * MAXV)
    throw Error{QD_ERR_UNSUPPORTED, "FFT grid size above 4096"};
  p.cluster = choose_cluster(n1, n2);
  p.sep = -1;
  p.sep_ke_tiles = p.sep_re_tiles = 0;
  // mixed-form candidates in order of preference without timing: separable shapes
  // (first instantiated first), the two-exchange cluster kernel, the three-pass kernels
  p.n_cand = 0;
  for (int q = 0; q < kNumSep && p.n_cand < FFT_MAX_CANDIDATES - 2; q++)
    if (kSepShapes[q].n1 == n1 && kSepShapes[q].n2 == n2) p.cand[p.n_cand++] = FFT_SEP0 + q;
  if (p.cluster) p.cand[p.n_cand++] = FFT_CLUSTER;
  p.cand[p.n_cand++] = FFT_THREE_PASS;
  fft_plan_choose(p, p.cand[0]);
  p.rows_per_cta = largest_divisor_at_most(n2, std::max(1, FFT_THREADS * MAXV / n1));
  p.rows_per_cta = std::min(p.rows_per_cta, largest_divisor_at_most(n2, 64));
  p.cols_per_cta = largest_divisor_at_most(n1, std::min(32, std::max(1, FFT_THREADS * MAXV / n2)));
  // FP64 twiddles exp(-2 pi i t/n); FP32 twiddles as three-shear rotation
  // coefficients (-tan(b/2), sin(b)) with b the angle reduced to [-pi/2, pi/2]
  // by a shift of pi where 4t lies strictly between n and 3n
  auto make = [](int n, double2 **d, float2 **f) {
    std::vector<double2> hd(n);
    std::vector<float2> hf(n);
    for (int t = 0; t < n; t++) {
      const double a = -2.0 * M_PI * (double)t / (double)n;
      hd[t] = make_double2(std::cos(a), std::sin(a));
      double b = std::remainder(a, 2.0 * M_PI);
      if (4LL * t > n && 4LL * t < 3LL * n) b += b > 0 ? -M_PI : M_PI;
      hf[t] = make_float2((float)(-std::tan(0.5 * b)), (float)std::sin(b));
    }
    QD_CUDA(cudaMalloc(d, n * sizeof(double2)));
    QD_CUDA(cudaMalloc(f, n * sizeof(float2)));
    QD_CUDA(cudaMemcpy(*d, hd.data(), n * sizeof(double2), cudaMemcpyHostToDevice));
    QD_CUDA(cudaMemcpy(*f, hf.data(), n * sizeof(float2), cudaMemcpyHostToDevice));
  };
  make(n1, &p.tw1_d, &p.tw1_f);
  make(n2, &p.tw2_d, &p.tw2_f);
  // shared-memory opt-in, set outside any stream capture
  QD_CUDA(cudaFuncSetAttribute(k_fft_rows<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  QD_CUDA(cudaFuncSetAttribute(k_fft_cols<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  QD_CUDA(cudaFuncSetAttribute(k_fft_rows<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  QD_CUDA(cudaFuncSetAttribute(k_fft_cols<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  QD_CUDA(cudaFuncSetAttribute(k_fft_slab_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  if (p.cluster > 1)
    QD_CUDA(cudaFuncSetAttribute(k_fft_slab_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 0));
  for (int q = 0; q < p.n_cand; q++)
    if (p.cand[q] >= FFT_SEP0) sep_dispatch_attr(p.cand[q] - FFT_SEP0);
}

void fft_plan_choose(FFTPlan &p, int choice) {
  p.choice = choice;
  p.sep = choice >= FFT_SEP0 ? choice - FFT_SEP0 : -1;
  p.sep_ke_tiles = p.sep >= 0 ? sep_dispatch_ke_tiles(p.sep) : 0;
  p.sep_re_tiles = p.sep >= 0 ? sep_dispatch_re_tiles(p.sep) : 0;
  p.use_cluster = choice == FFT_CLUSTER;
}

std::string fft_choice_name(int choice) {
  std::string name;
  if (choice >= FFT_SEP0) {
    const SepShape &q = kSepShapes[choice - FFT_SEP0];
    name = "separable A=" + std::to_string(q.A) + " B1=" + std::to_string(q.B1) + " B2=" + std::to_string(q.B2) +
           " threads=" + std::to_string(q.threads) +
           (q.mode >= 2 ? std::string(q.mode == 2 ? " two-pass 24 warps/SM" : " two-pass 32 warps/SM")
                        : " cluster=" + std::to_string(sep_dispatch_ke_tiles(choice - FFT_SEP0)) +
                              (q.mode == 1 ? " persistent" : ""));
  } else {
    name = choice == FFT_CLUSTER ? "cluster two-exchange" : "three-pass";
  }
  return name + " [" + std::to_string(choice) + "]";
}

void fft_plan_free(FFTPlan &p) {
  cudaFree(p.tw1_d);
  cudaFree(p.tw1_f);
  cudaFree(p.tw2_d);
  cudaFree(p.tw2_f);
  p.tw1_d = p.tw2_d = nullptr;
  p.tw1_f = p.tw2_f = nullptr;
}

// partial-sum tiles per slab: the single-pass FP32 form writes one per CTA of
// the cluster, the two-pass form one per CTA of the column pass, the three-pass
// forms one per column / row tile
int fft_col_tiles(const FFTPlan &p, int precision) {
  if (precision == QD_PRECISION_MIXED && p.sep >= 0) return p.sep_ke_tiles;
  return (precision == QD_PRECISION_MIXED && p.use_cluster) ? p.cluster : p.n1 / p.cols_per_cta;
}
int fft_row_tiles(const FFTPlan &p, int precision) {
  if (precision == QD_PRECISION_MIXED && p.sep >= 0) return p.sep_re_tiles;
  return (precision == QD_PRECISION_MIXED && p.use_cluster) ? p.cluster : p.n2 / p.rows_per_cta;
}
// kernel launches of the mixed form's FFT stage: one for the single-pass kernels, two for the
// two-pass form, three for the three-pass kernels
int fft_mixed_launches(const FFTPlan &p) {
  if (p.sep >= 0) return kSepShapes[p.sep].mode >= 2 ? 2 : 1;
  return p.use_cluster ? 1 : 3;
}
// partial-sum tiles per slab of any mixed-form candidate (buffers sized for tuning)
int fft_max_tiles(const FFTPlan &p) {
  int t = std::max(p.n1 / p.cols_per_cta, p.n2 / p.rows_per_cta);
  for (int q = 0; q < p.n_cand; q++) {
    if (p.cand[q] >= FFT_SEP0) t = std::max(t, sep_dispatch_ke_tiles(p.cand[q] - FFT_SEP0));
    if (p.cand[q] == FFT_CLUSTER) t = std::max(t, p.cluster);
  }
  return t;
}



template <typename R>
static void launch_fft_kinetic_t(cudaStream_t s, const Grid &g, const FFTPlan &p, typename CT<R>::T *psi_j,
                                 const SlabDesc *slabs, int n_slabs, const double2 *tab_kin, const double *T1,
                                 const double *T2, double *ke_part, const double2 *tabE, double *re_part,
                                 const int *status, const FFTLift *lf) {
  using C = typename CT<R>::T;
  auto radices = [](int n, int nst, const int *rad) {
    Radices r{};
    r.n = n;
    r.nst = nst;
    r.fn = make_fastdiv((uint32_t)n);
    int ns = 1;
    for (int q = 0; q < nst; q++) {
      r.rad[q] = rad[q];
      r.nbf[q] = make_fastdiv((uint32_t)(n / rad[q]));
      r.ns[q] = make_fastdiv((uint32_t)ns);
      ns *= rad[q];
    }
    return r;
  };
  const Radices r1 = radices(p.n1, p.nst1, p.rad1), r2 = radices(p.n2, p.nst2, p.rad2);
  const FastDiv fn2 = make_fastdiv((uint32_t)g.n2), fncols = make_fastdiv((uint32_t)p.cols_per_cta);
  const C *tw1 = std::is_same<R, double>::value ? (const C *)p.tw1_d : (const C *)p.tw1_f;
  const C *tw2 = std::is_same<R, double>::value ? (const C *)p.tw2_d : (const C *)p.tw2_f;
  const int rows = n_slabs * g.n2;
  const size_t sm_rows = (size_t)p.rows_per_cta * p.n1 * sizeof(C);
  const size_t sm_cols = (size_t)p.cols_per_cta * p.n2 * sizeof(C);
  const unsigned nrow_ctas = (unsigned)(rows / p.rows_per_cta);
  const double scale = 1.0 / ((double)g.n1 * g.n2);
  const bool pow2 = ((g.n1 * g.n2) & (g.n1 * g.n2 - 1)) == 0;
  const float fscale = pow2 ? (float)scale : 0.0f;
  if constexpr (std::is_same<R, float>::value) {
  if (p.sep >= 0 && lf && lf->kinR) {
    sep_dispatch_launch(p.sep, s, g, p, psi_j, slabs, n_slabs, *lf, ke_part, re_part, fscale, scale, status);
    prof_mark(s, "fft_slab");
    return;
  }
  if (p.use_cluster && lf && lf->kinR) {
    const int C = p.cluster;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)(n_slabs * C));
    cfg.blockDim = dim3(SLAB_THREADS);
    cfg.dynamicSmemBytes = ((size_t)2 * g.n1 * g.n2 / C + g.n1 + g.n2) * sizeof(float2);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    QD_CUDA(cudaLaunchKernelEx(&cfg, k_fft_slab_cluster, psi_j, r1, r2, C, g, slabs, p.tw1_f, p.tw2_f, *lf, ke_part,
                               re_part, fscale, scale, make_fastdiv((uint32_t)(g.n1 / C)), status));
    prof_mark(s, "fft_slab");
    return;
  }
  }
  k_fft_rows<R><<<nrow_ctas, FFT_THREADS, sm_rows, s>>>(psi_j, r1, p.rows_per_cta, rows, tw1, 0, g, 1.0, slabs,
                                                        nullptr, nullptr, 0, status, lf ? lf->proR : nullptr,
                                                        lf ? lf->pror : nullptr, 0.0f, fn2);
  prof_mark(s, "fft_rows_forward");
  const unsigned ncol_ctas = (unsigned)(n_slabs * (p.n1 / p.cols_per_cta));
  k_fft_cols<R><<<ncol_ctas, FFT_THREADS, sm_cols, s>>>(psi_j, r2, p.cols_per_cta, g, tw2, tab_kin, T1, T2, ke_part,
                                                        fft_col_tiles(p, QD_PRECISION_FP64), status, lf ? lf->kinR : nullptr,
                                                        lf ? lf->kinr : nullptr, lf ? lf->T1f : nullptr,
                                                        lf ? lf->T2f : nullptr, fncols);
  prof_mark(s, "fft_cols_kinetic");
  k_fft_rows<R><<<nrow_ctas, FFT_THREADS, sm_rows, s>>>(psi_j, r1, p.rows_per_cta, rows, tw1, 1, g, scale, slabs,
                                                        tabE, re_part, fft_row_tiles(p, QD_PRECISION_FP64), status,
                                                        lf ? lf->epiR : nullptr, lf ? lf->epir : nullptr, fscale, fn2);
  prof_mark(s, "fft_rows_inverse");
}

void launch_fft_kinetic(cudaStream_t s, const Grid &g, const FFTPlan &p, double2 *psi_j, const SlabDesc *slabs,
                        int n_slabs, const double2 *tab_kin, const double *T1, const double *T2, double *ke_part,
                        const double2 *tabE, double *re_part, const int *status) {
  if (n_slabs == 0) return;
  launch_fft_kinetic_t<double>(s, g, p, psi_j, slabs, n_slabs, tab_kin, T1, T2, ke_part, tabE, re_part, status,
                               nullptr);
}

void launch_fft_kinetic(cudaStream_t s, const Grid &g, const FFTPlan &p, float2 *psi_j, const SlabDesc *slabs,
                        int n_slabs, double *ke_part, double *re_part, const int *status, const FFTLift *lift) {
  if (n_slabs == 0) return;
  launch_fft_kinetic_t<float>(s, g, p, psi_j, slabs, n_slabs, nullptr, nullptr, nullptr, ke_part, nullptr, re_part,
                              status, lift);
}

}  // namespace qd
