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
// slot_sh: shared word written by thread 0 before the call and read only after
// the tile's barrier (so its global source need not be waited for first); a
// negative slot writes nothing.
__device__ inline void flux_extract_tile(const FluxTileArgs &f, const int *slot_sh, int b, int xtile, int tid,
                                         float2 (*sD)[FLUX_GX], float2 *sA) {
  const Grid &g = f.g;
  const int tx = tid % FLUX_GX, ty = tid / FLUX_GX;
  const int h = (f.n_grad - 1) / 2;
  const int64_t ns = (int64_t)g.nth * g.n1;
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
  const int slot = *slot_sh;
  if (ty == 0 && q < ns && slot >= 0) {
    float2 *out = f.buf + ((int64_t)slot * f.n_blocks + b) * 2 * ns;
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

// All partials of block b, summed by the CTA's 256 threads into tot[5] (module,
// potential, kinetic, rotational, Coriolis), deterministically: thread t loads
// elements t, t + 256, ... of every partial array (a chunk's loads in flight
// together) and adds the ones that exist; warp q then sums quantity q's 256
// per-thread values from shared memory in a fixed order.  The FP64 pipe runs
// at 1/64 of FP32 on this part, so the CTA adds each value once: no zero
// padding and no all-lane shuffle trees over the 256 threads.
constexpr int FIN_THREADS = 256;
__device__ inline void finalize_reduce(const FinalizeArgs &a, int b, double (*red)[FIN_THREADS], double *tot) {
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
  constexpr int T = FIN_THREADS, U = 4;
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  const int nmax = max(max(n0, n1), max(n2, n3));
  for (int t0 = tid; t0 < nmax; t0 += T * U) {
    double2 vm[U];
    double vk[U], vr[U], vc[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int t = t0 + u * T;
      vm[u] = t < n0 ? mp[t] : make_double2(0.0, 0.0);
      vk[u] = t < n1 ? kp[t] : 0.0;
      vr[u] = t < n2 ? rp[t] : 0.0;
      vc[u] = 0.0;
      if (t < n3) {
        const int gi = g_lo + t / ep.ce_tiles, tt = t - (t / ep.ce_tiles) * ep.ce_tiles;
        const int o = bd.omega - a.groups[gi].omega_lo;
        if (o >= 0 && o < a.groups[gi].n) vc[u] = ep.ce[((int64_t)gi * a.ce_n + o) * ep.ce_tiles + tt];
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int t = t0 + u * T;
      if (t < n0) {
        acc[0] += vm[u].x;
        acc[1] += vm[u].y;
      }
      if (t < n1) acc[2] += vk[u];
      if (t < n2) acc[3] += vr[u];
      if (t < n3) acc[4] += vc[u];
    }
  }
#pragma unroll
  for (int q = 0; q < 5; q++) red[q][tid] = acc[q];
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31;
  if (warp < 5) {
    double v = 0.0;
#pragma unroll
    for (int i = 0; i < T / 32; i++) v += red[warp][lane + 32 * i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) tot[warp] = v;
  }
  __syncthreads();
}

// Thread 0: energies[b] (totals included) and the step record; returns the module.
// eprev: energies[b] as loaded at the start (kept for quantities not computed here).
__device__ inline double finalize_write(const FinalizeArgs &a, int b, int step, const double *tot,
                                        const double *eprev) {
  const EnergyParts &ep = a.ep;
  const double dV = a.g.dr1 * a.g.dr2;
  double *e = a.energies + b * 6;
  double ev[6];
  ev[E_MODULE] = ep.have_mod ? tot[0] * dV : eprev[E_MODULE];
  ev[E_POTENTIAL] = ep.have_mod ? tot[1] * dV : eprev[E_POTENTIAL];
  ev[E_KINETIC] = ep.have_ke ? tot[2] * ep.ke_scale : eprev[E_KINETIC];
  ev[E_ROTATIONAL] = ep.have_re ? tot[3] * dV : eprev[E_ROTATIONAL];
  ev[E_CORIOLIS] = ep.have_ce ? tot[4] * dV : eprev[E_CORIOLIS];
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
