// Device pieces shared by the energy finalisation, the mixed-form surface
// extraction and the fused end-of-step kernel of the mixed form.
#pragma once
#include "qd_internal.h"
#include "qd_device.cuh"

namespace qd {

// rotation by 2 alpha from (t, s) = (-tan(alpha/2), sin(alpha)): two
// three-shear rotations, each of determinant exactly 1
__device__ inline void lift2f(float &x, float &y, float2 ts) {
  x = fmaf(ts.x, y, x);
  y = fmaf(ts.y, x, y);
  x = fmaf(ts.x, y, x);
  x = fmaf(ts.x, y, x);
  y = fmaf(ts.y, x, y);
  x = fmaf(ts.x, y, x);
}

// ------------------------------------------------------- surface extraction
// One CTA of FLUX_GX x FLUX_GY threads (linear index tid = ty FLUX_GX + tx):
// thread row ty handles the stencil rows gg = ty, ty + FLUX_GY, ... of FLUX_GX
// consecutive surface points (i fastest: coalesced loads); the rows' partial
// derivatives are summed in a fixed order through shared memory.  Values are
// psi on the stencil rows after exp(-i V dt/2) (three-shear rotations), the
// centre row's value and the FD derivative, stored in slot `slot`.
constexpr int FLUX_GX = 64, FLUX_GY = 4, FLUX_GMAX = 8;   // n_grad <= FLUX_GY * FLUX_GMAX
struct FluxTileArgs {
  Grid g;
  int n_grad, n_ds, n_blocks;
  const float2 *psi_th;   // c64 theta-space pool
  const float2 *hv;       // [k][gg][i] three-shear coefficients of exp(-i V dt/2)
  const float *fd;        // FD weights / dr2
  float2 *buf;            // [slot][block][A, dA/dr][k][i]
};
inline FluxTileArgs flux_tile_args(const Grid &g, const FluxConfig &fc, const float2 *psi_th, const float2 *hv,
                                   const float *fd, float2 *buf, int n_blocks) {
  FluxTileArgs f{};
  f.g = g;
  f.n_grad = fc.n_grad;
  f.n_ds = fc.n_ds;
  f.n_blocks = n_blocks;
  f.psi_th = psi_th;
  f.hv = hv;
  f.fd = fd;
  f.buf = buf;
  return f;
}
__device__ inline void flux_extract_tile(const FluxTileArgs &f, int slot, int b, int xtile, int tid,
                                         float2 (*sD)[FLUX_GX], float2 *sA) {
  const Grid &g = f.g;
  const int tx = tid % FLUX_GX, ty = tid / FLUX_GX;
  const int h = (f.n_grad - 1) / 2;
  const int64_t ns = (int64_t)g.nth * g.n1;
  float2 *out = f.buf + ((int64_t)slot * f.n_blocks + b) * 2 * ns;
  const float2 *p = f.psi_th + (int64_t)b * g.nth * g.npt;
  const int64_t q = (int64_t)xtile * FLUX_GX + tx;
  float Dx = 0.0f, Dy = 0.0f;
  if (q < ns) {
    const int i = (int)(q % g.n1), k = (int)(q / g.n1);
    float2 a[FLUX_GMAX];
    float2 ts[FLUX_GMAX];
#pragma unroll
    for (int u = 0; u < FLUX_GMAX; u++) {
      const int gg = ty + FLUX_GY * u;
      if (gg < f.n_grad) {
        a[u] = p[((int64_t)k * g.n2 + (f.n_ds - h + gg)) * g.n1 + i];
        ts[u] = __ldg(f.hv + ((int64_t)k * f.n_grad + gg) * g.n1 + i);
      }
    }
#pragma unroll
    for (int u = 0; u < FLUX_GMAX; u++) {
      const int gg = ty + FLUX_GY * u;
      if (gg < f.n_grad) {
        float x = a[u].x, y = a[u].y;
        lift2f(x, y, ts[u]);
        const float c = __ldg(f.fd + gg);
        Dx = fmaf(c, x, Dx);
        Dy = fmaf(c, y, Dy);
        if (gg == h) sA[tx] = make_float2(x, y);
      }
    }
  }
  sD[ty][tx] = make_float2(Dx, Dy);
  __syncthreads();
  if (ty == 0 && q < ns) {
    float2 D = sD[0][tx];
#pragma unroll
    for (int y = 1; y < FLUX_GY; y++) {
      D.x += sD[y][tx].x;
      D.y += sD[y][tx].y;
    }
    out[q] = sA[tx];
    out[ns + q] = D;
  }
}

// ------------------------------------------------------ energy finalisation
struct FinalizeArgs {
  Grid g;
  EnergyParts ep;
  const BlockDesc *blocks;
  const int *pblock0;
  int n_problems;
  const CoriolisGroup *groups;
  const int *pgroup0;
  int ce_n;
  double *energies, *rec;
  int *d_step;
  int rec_base, rec_cap, n_blocks;
  double norm_tol;
  int *status, *status_step;
  StepTail tail;
  unsigned *done;
};

// All partials of block b, 256 threads (two warps per quantity: module/potential,
// kinetic, rotational, Coriolis), reduced in a fixed order into red[8][2].
__device__ inline void finalize_reduce(const FinalizeArgs &a, int b, double (*red)[2]) {
  const int tid = threadIdx.x;
  const EnergyParts &ep = a.ep;
  const BlockDesc bd = a.blocks[b];
  const int n0 = ep.have_mod ? ep.mod_pe_tiles : 0;
  const int n1 = ep.have_ke ? bd.nl * ep.ke_tiles : 0;
  const int n2 = ep.have_re ? bd.nl * ep.re_tiles : 0;
  // Coriolis: every group (one per l) of this problem, the tiles of this Omega where it is a member
  const int g_lo = (ep.have_ce && a.groups) ? a.pgroup0[bd.problem] : 0;
  const int n3 = (ep.have_ce && a.groups) ? (a.pgroup0[bd.problem + 1] - g_lo) * ep.ce_tiles : 0;
  const double2 *mp = reinterpret_cast<const double2 *>(ep.mod_pe) + (int64_t)b * ep.mod_pe_tiles;
  const double *kp = ep.ke + (int64_t)bd.slab0 * ep.ke_tiles;
  const double *rp = ep.re + (int64_t)bd.slab0 * ep.re_tiles;
  // warp-uniform branches, no divergence inside a loop: each lane's loads issue together
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
      const int o = bd.omega - a.groups[gi].omega_lo;
      if (o >= 0 && o < a.groups[gi].n) acc[4] += ep.ce[((int64_t)gi * a.ce_n + o) * ep.ce_tiles + tt];
    }
  }
  // each warp reduces only its own quantity; thread 0 later adds the two warps of each
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
}

// Thread 0: energies[b] (totals included) and the step record; returns the module.
__device__ inline double finalize_write(const FinalizeArgs &a, int b, int step, const double (*red)[2]) {
  const EnergyParts &ep = a.ep;
  const double tot[5] = {red[0][0] + red[1][0], red[0][1] + red[1][1], red[2][0] + red[3][0],
                         red[4][0] + red[5][0], red[6][0] + red[7][0]};
  const double dV = a.g.dr1 * a.g.dr2;
  double *e = a.energies + b * 6;
  double ev[6];
  ev[E_MODULE] = ep.have_mod ? tot[0] * dV : e[E_MODULE];
  ev[E_POTENTIAL] = ep.have_mod ? tot[1] * dV : e[E_POTENTIAL];
  ev[E_KINETIC] = ep.have_ke ? tot[2] * ep.ke_scale : e[E_KINETIC];
  ev[E_ROTATIONAL] = ep.have_re ? tot[3] * dV : e[E_ROTATIONAL];
  ev[E_CORIOLIS] = ep.have_ce ? tot[4] * dV : e[E_CORIOLIS];
  ev[E_TOTAL] = ev[E_POTENTIAL] + ev[E_KINETIC] + ev[E_ROTATIONAL] + ev[E_CORIOLIS];
  for (int q = 0; q < 6; q++) e[q] = ev[q];
  const int slot = step - a.rec_base;
  if (a.rec && slot >= 0 && slot < a.rec_cap)
    for (int q = 0; q < 6; q++) a.rec[((int64_t)slot * a.n_blocks + b) * 6 + q] = ev[q];
  return ev[E_MODULE];
}

// Thread 0 at the very end of a step (no other CTA of the launch still runs):
// flux slot and t0 of this step, then the step counter.  `bad`: the norm guard
// tripped in this launch.
__device__ inline void finalize_step_end(const FinalizeArgs &a, int step, int fcount, bool bad) {
  const StepTail &t = a.tail;
  if (!t.done || bad) return;
  if (t.flux_count) {
    if (fcount >= t.cap) {
      atomicCAS(a.status, 0, QD_ERR_INVALID);
      *t.flux_slot = 0;
    } else {
      if (fcount == 0) *t.flux_t0 = (step + 1) * t.dt;
      *t.flux_slot = fcount;
      *t.flux_count = fcount + 1;
    }
  }
  *a.d_step = step + 1;
}

// Multi-CTA end: the last CTA to arrive applies the norm guard per problem and
// ends the step.  Every thread of every CTA calls this once.
__device__ inline void finalize_last_cta(const FinalizeArgs &a, int step, int fcount, bool *last) {
  const int tid = threadIdx.x;
  if (tid == 0) {
    __threadfence();
    *last = atomicAdd(a.done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!*last) return;
  __threadfence();
  if (a.ep.have_mod)
    for (int pr = tid; pr < a.n_problems; pr += blockDim.x) {
      double m = 0.0;
      for (int bb = a.pblock0[pr]; bb < a.pblock0[pr + 1]; bb++) m += __ldcg(a.energies + bb * 6 + E_MODULE);
      if (m > 1.0 + a.norm_tol && atomicCAS(a.status, 0, QD_ERR_NORM) == 0) *a.status_step = step;
    }
  __syncthreads();
  if (tid != 0) return;
  *a.done = 0u;
  finalize_step_end(a, step, fcount, atomicAdd(a.status, 0) != 0);
}

}  // namespace qd
