// Mixed-precision theta <-> j Legendre contraction on the 5th-generation
// tensor cores (tcgen05, sm_103a).
//
// Reference: the two cublasZgemm calls of omegawavepacket.cu:200-240.  The
// contraction is a real GEMM over the interleaved view of psi: rows
// m = 2*point + {re, im}, so C[m][n] = sum_k A[m][k] B[n][k] with B the real
// (weighted) associated-Legendre matrix.
//
// Precision (3-term BF16 split, exact accumulation): each row m of A is scaled
// by a power of two s_m >= max_k |A[m][k]| and each column n of B by t_n, so
// |a|, |b| <= 1.  Three integer slices are taken by round-to-nearest,
//   i0 = rn(256 a), i1 = rn(256 (256 a - i0)), i2 = rn(256 (... - i1)),
// with |i0| <= 256, |i1|, |i2| <= 128: every slice is an integer that BF16
// holds exactly.  Products of slices are grouped by order,
//   D0 = sum_k i0 j0,  D1 = sum_k (i0 j1 + i1 j0),  D2 = sum_k (i0 j2 + i1 j1 + i2 j0),
// each an integer below 96 * 81920 < 2^24 for K <= 192, so the three FP32
// TMEM accumulators hold them exactly whatever the tensor core's internal
// rounding.  C = s_m t_n 2^-16 (D0 + 2^-8 (D1 + 2^-8 D2)) is then formed with
// two round-to-nearest FP32 operations.  (A single accumulator of all six
// products loses about 2e-6 of the norm per forward+backward pair to biased
// accumulation rounding; the exact form has no such bias.)
//
// The kernel (k_legendre_tc_ws) is persistent and warp-specialised: one CTA
// per SM walks a contiguous range of (block, 64-point tile) pairs, M = 128
// real rows each.  Eight producer warps load the tile from the c64 pool (with
// an L2 prefetch of the next tile; forward: absorbing mask and exp(-iV dt) as
// an exactly area-preserving three-shear rotation), stage it in FP32, scale
// and slice every row into the SWIZZLE_NONE K-major canonical layout; one
// consumer thread issues the tcgen05.mma chain (four MMAs per K = 16 step) and
// commits to an mbarrier; eight consumer warps read their rows (TMEM lanes)
// back with tcgen05.ld 32x32b, recombine, and store c64.  The backward
// epilogue also reduces the module and potential energy per tile.
//
// The backward contraction runs in a second form (TA) where the A slices live
// in TMEM (tcgen05.mma reads A from tensor memory: row m in lane m, BF16 element
// k in column k / 2, even k in the low half) beside the accumulators.  The
// shared memory that frees holds two raw staging buffers, filled by cp.async one
// tile ahead, so each tile's load overlaps the previous tile's slicing; the
// producer warps also drain a quarter of the previous tile's accumulator columns
// after slicing, once the consumers have published that tile's tables.
#include <cuda_bf16.h>


#include "qd_internal.h"
#include "qd_device.cuh"
#include "qd_mbarrier.cuh"
#include "qd_tcgen05.cuh"

namespace qd {

namespace {
constexpr int TC_POINTS = 64;        // 128 real rows

__host__ __device__ inline int round16(int x) { return (x + 15) & ~15; }

// products a_i * b_j with i + j <= 2
__constant__ int c_pair_a[6] = {0, 0, 1, 0, 1, 2};
__constant__ int c_pair_b[6] = {0, 1, 0, 2, 1, 0};
}  // namespace

// byte size of the B image of one block: 3 terms x Npad x Kpad BF16
__host__ __device__ inline int64_t tc_bimg_bytes(int Np, int Kp) { return 3LL * Np * Kp * 2; }

// TMEM columns for three Np-wide accumulators (power of two >= 32)
__host__ __device__ inline uint32_t tc_tmem_cols(int Np) {
  const int need = 3 * Np;
  return need <= 32 ? 32u : need <= 64 ? 64u : need <= 128 ? 128u : need <= 256 ? 256u : 512u;
}

// ---------------------------------------------------------------------------
// B images: element (n, k) of term t at t*Np*Kp*2 + (n/8)*SBO + (k/8)*128 +
// (n%8)*16 + (k%8)*2 bytes with SBO = Kp/8*128 (SWIZZLE_NONE, K-major).
// fwd: B(n = l, k = theta) = w_k P_l(x_k) = Bf[k*nl + n]
// bwd: B(n = theta, k = l) = P_l(x_n)     = Bb[k*nth + n]
// One CTA per (block, column n): the column scale t_n = 2^e (smallest power
// of two >= max_k |B(n, k)|) and the three integer slices of B(n, k)/t_n.
__global__ void k_build_tc_bimage(const BlockDesc *__restrict__ blocks, const double *__restrict__ Bsrc, int nth,
                                  int fwd, const int64_t *__restrict__ img_off, uint16_t *__restrict__ img,
                                  float *__restrict__ bscale) {
  __shared__ double red[32];
  const BlockDesc bd = blocks[blockIdx.y];
  const int Kv = fwd ? nth : bd.nl, Nv = fwd ? bd.nl : nth;
  const int Kp = (Kv + 15) & ~15, Np = (Nv + 15) & ~15;
  const int n = blockIdx.x;
  if (n >= Np) return;
  uint16_t *out = img + img_off[blockIdx.y] / 2;
  const int SBOe = Kp / 8 * 64;   // in elements
  auto val = [&](int k) -> double {
    if (n >= Nv || k >= Kv) return 0.0;
    return fwd ? Bsrc[bd.bmat0 + (int64_t)k * bd.nl + n] : Bsrc[bd.bmat0 + (int64_t)k * nth + n];
  };
  // block-wide max |B(n, :)| (max via -sum of negated maxima is not needed: use a
  // shared reduction with fmax)
  double mx = 0.0;
  for (int k = threadIdx.x; k < Kp; k += blockDim.x) mx = fmax(mx, fabs(val(k)));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x + 31) / 32; w++) m = fmax(m, red[w]);
    red[0] = m;
  }
  __syncthreads();
  mx = red[0];
  int e = 0;
  if (mx > 0.0) frexp(mx, &e);          // mx = f 2^e, f in [0.5, 1)  ->  |B| / 2^e < 1
  const double inv = ldexp(1.0, -e);
  if (threadIdx.x == 0) bscale[(int64_t)blockIdx.y * 256 + n] = (float)ldexp(1.0, e);
  for (int k = threadIdx.x; k < Kp; k += blockDim.x) {
    const double b = val(k) * inv * 256.0;
    const double i0 = rint(b);
    const double r1 = (b - i0) * 256.0;
    const double i1 = rint(r1);
    const double i2 = rint((r1 - i1) * 256.0);
    const int64_t el = (int64_t)(n / 8) * SBOe + (k / 8) * 64 + (n % 8) * 8 + (k % 8);
    out[el] = __bfloat16_as_ushort(__double2bfloat16(i0));
    out[(int64_t)Np * Kp + el] = __bfloat16_as_ushort(__double2bfloat16(i1));
    out[2LL * Np * Kp + el] = __bfloat16_as_ushort(__double2bfloat16(i2));
  }
}

struct TcArgs {
  Grid g;
  const float2 *A;           // fwd: psi_theta pool, bwd: psi_j pool (both c64)
  float2 *C;                 // fwd: psi_j pool, bwd: psi_theta pool
  const BlockDesc *blocks;
  const uint16_t *bimg;      // B images
  const int64_t *bimg_off;   // per block byte offset
  const float *bscale;       // per block (x256) column scales t_n
  const float2 *vph;         // fwd: half-angle shears of exp(-iV dt) [k][p] (may be null)
  const float *d1, *d2;      // fwd: absorbing masks (may be null)
  const float *w;            // bwd: quadrature weights
  const float *wv;           // bwd: w_k V(k, p) [k][p]
  double *part;              // bwd: [b][tile][2]
  int n_part_tiles;
  const int *status;
  int *status_w;
};

// rotation by 2*alpha given (t, s) = (-tan(alpha/2), sin(alpha)): two
// three-shear rotations, each of determinant exactly 1
__device__ inline void rot_lift2(float &x, float &y, float2 ts) {
  x = fmaf(ts.x, y, x);
  y = fmaf(ts.y, x, y);
  x = fmaf(ts.x, y, x);
  x = fmaf(ts.x, y, x);
  y = fmaf(ts.y, x, y);
  x = fmaf(ts.x, y, x);
}


// ---------------------------------------------------------------------------
// Persistent, warp-specialised form.  Each CTA walks a contiguous range of
// (block, 64-point tile) pairs.  Warps 0-7 (producers) stage and slice tile
// t+1 while warps 8-15 (consumers) drain tile t from TMEM; consumer thread
// MMA_ISSUER issues the MMA chain of each tile.  Three mbarriers carry the
// hand-offs:
//   slices_ready (256 producer arrivals)  -> the MMA may read A/B slices
//   mma_done     (tcgen05.commit)         -> TMEM holds tile t; A/B reusable
//   tmem_free    (256 consumer arrivals)  -> the next MMA may overwrite TMEM
// Every wait is bounded (1 s, qd_mbarrier.cuh); a timeout sets QD_ERR_TIMEOUT
// in the status word and the CTA stops issuing work, waits (bounded) for its
// MMAs, frees TMEM and returns.
__device__ inline void named_bar(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
struct TcTile {
  int b, mt, Kv, Nv, Kp, Np;
  uint32_t SBO, A_TERM, B_TERM;
};

template <bool FWD>
__device__ inline TcTile tc_tile(const TcArgs &P, int tt, int mtiles) {
  TcTile t;
  t.b = tt / mtiles;
  t.mt = tt - t.b * mtiles;
  const int nl = P.blocks[t.b].nl;
  t.Kv = FWD ? P.g.nth : nl;
  t.Nv = FWD ? nl : P.g.nth;
  t.Kp = round16(t.Kv);
  t.Np = round16(t.Nv);
  t.SBO = (uint32_t)(t.Kp / 8 * 128);
  t.A_TERM = 16u * t.SBO;
  t.B_TERM = (uint32_t)(t.Np / 8) * t.SBO;
  return t;
}

constexpr int WS_THREADS = 512;      // 8 producer warps + 8 consumer warps
// FP32 staging of one A tile, k-major: element (k, point pl, re/im c) at
// k * TC_LDM + pl + TC_IM * c.  With TC_LDM = 2 (mod 32) and TC_IM = 8 (mod 32)
// the loader's stores (32 consecutive points) and the slicer's loads (8
// points x re/im x two k-groups 8 apart) fall in 32 distinct banks.
constexpr int TC_LDM = 162, TC_IM = 72;
// raw staging of the A-in-TMEM form: row k of a tile's c64 values as 128 interleaved floats
// (re, im of point 0, ...), rows TC_LDR floats apart (8-byte aligned rows for the copies)
constexpr int TC_LDR = 130;
// first TMEM column of the A slices in that form (after the three Np-wide accumulators)
__host__ __device__ inline uint32_t tc_a_col0(int np_max) { return (uint32_t)((3 * np_max + 31) & ~31); }
// consumer thread that issues the MMA chain: not thread 0, which forms the
// backward kernel's per-tile module/potential sums after each epilogue
constexpr int MMA_ISSUER = 32;
constexpr int WS_PROD = 256;

// TA (backward only): the A slices live in TMEM instead of shared memory (tcgen05.mma reads A
// from tensor memory), which frees the shared memory for two raw staging buffers: the producers
// copy tile t+1 in with cp.async while they slice tile t, so a tile's load and its slicing
// overlap instead of following each other.
template <bool FWD, bool TA = false>
__global__ void __launch_bounds__(WS_THREADS, 1) k_legendre_tc_ws(TcArgs P, int mtiles, int n_tiles, int kp_max,
                                                                   int np_max) {
  static_assert(!(FWD && TA), "A in TMEM: backward contraction only");
  if (P.status && *P.status) return;
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t mb_ready, mb_done, mb_free;
  __shared__ uint64_t mb_tab;   // A-in-TMEM form: a tile's tables and w V are in shared memory
  __shared__ uint32_t tmem_base_s;
  __shared__ float srow_s[2][128];
  __shared__ float red_s[16];
  // column scales and (backward) weights of the tile's block; in the A-in-TMEM form one set per
  // tile parity, since the producers drain tile t - 1 while the consumers set up tile t
  __shared__ float tsc_s[TA ? 2 : 1][256], w_s[TA ? 2 : 1][256];
  __shared__ int abort_p, abort_c, n_issued;
  __shared__ float rmax_s[TA ? 2 : 1][128];   // A-in-TMEM form: the two k halves' row maxima
  __shared__ float redp_s[16];                // A-in-TMEM form: the producers' energy partials
  const Grid &g = P.g;
  const uint32_t a_term_max = TA ? 0u : 16u * (uint32_t)(kp_max / 8 * 128);
  const uint32_t b_term_max = (uint32_t)(np_max / 8) * (uint32_t)(kp_max / 8 * 128);
  unsigned char *sA = smem;
  unsigned char *sB = smem + 3 * a_term_max;
  float *sF = reinterpret_cast<float *>(sB + 3 * b_term_max);
  // backward: w V of the tile, [n][64 points] (two, by tile parity, in the A-in-TMEM form)
  float *sWV = sF + (TA ? 2 * kp_max * TC_LDR : kp_max * TC_LDM);
  const uint32_t a_col0 = TA ? tc_a_col0(np_max) : 0u;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t ncols = 512;
  const int t_begin = (int)((int64_t)blockIdx.x * n_tiles / gridDim.x);
  const int t_end = (int)((int64_t)(blockIdx.x + 1) * n_tiles / gridDim.x);

  if (warp == 0) tmem_alloc(smem_u32(&tmem_base_s), ncols);
  if (tid == 0) {
    mbar_init(smem_u32(&mb_ready), WS_PROD);
    mbar_init(smem_u32(&mb_done), 1);
    mbar_init(smem_u32(&mb_free), TA ? WS_THREADS : WS_THREADS - WS_PROD);   // A in TMEM: both groups drain
    mbar_init(smem_u32(&mb_tab), WS_THREADS - WS_PROD);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_p = 0;
    abort_c = 0;
    n_issued = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;

  // Drain of one tile's accumulators by one warp: TMEM lanes of quarter qd (rows m = 32 qd +
  // lane), 16-column chunks n0 = 16 grp, 16 grp + stride, ...; recombination, c64 store and
  // (backward) the module and potential partials.
  auto drain = [&](const TcTile &T, const BlockDesc &bd, int itd, int qd, int grp, int stride, float &mod,
                   float &pe) {
    const int m = 32 * qd + lane;
    const int pl = m >> 1, c = m & 1;
    const int64_t p = (int64_t)T.mt * TC_POINTS + pl;
    const int par = TA ? (itd & 1) : 0;
    const float srow = srow_s[itd & 1][m];
    const float *tsc = tsc_s[par];
    const float *wq = w_s[par];
    const float *wv = sWV + (TA ? par * np_max * TC_POINTS : 0);
    float *Cf = reinterpret_cast<float *>(P.C);
    const uint32_t trow = tmem + ((uint32_t)(32 * qd) << 16);
    for (int n0 = 16 * grp; n0 < T.Np; n0 += stride) {
      uint32_t r0[16], r1[16], r2[16];
      tmem_ld16(trow + (uint32_t)n0, r0);
      tmem_ld16(trow + (uint32_t)(T.Np + n0), r1);
      tmem_ld16(trow + (uint32_t)(2 * T.Np + n0), r2);
      tmem_wait_ld();   // one wait for the three loads
      float d0[16], d1[16], d2[16];
#pragma unroll
      for (int q = 0; q < 16; q++) {
        reg_after_wait(r0[q]);
        reg_after_wait(r1[q]);
        reg_after_wait(r2[q]);
        d0[q] = __uint_as_float(r0[q]);
        d1[q] = __uint_as_float(r1[q]);
        d2[q] = __uint_as_float(r2[q]);
      }
      if (p < g.npt) {
#pragma unroll
        for (int q = 0; q < 16; q++) {
          const int n = n0 + q;
          const float v = fmaf(fmaf(d2[q], 0.00390625f, d1[q]), 0.00390625f, d0[q]) * (srow * tsc[n]);
          if (n < T.Nv) {
            if (FWD) {
              Cf[2 * ((int64_t)(bd.slab0 + n) * g.npt + p) + c] = v;
            } else {
              Cf[2 * (((int64_t)T.b * g.nth + n) * g.npt + p) + c] = v;
              const float v2 = v * v;
              mod = fmaf(wq[n], v2, mod);
              pe = fmaf(wv[n * TC_POINTS + pl], v2, pe);
            }
          }
        }
      }
    }
  };
  // A-in-TMEM form: the producers' share of tile itd's drain (column chunks 2 + kh of four, after
  // the consumers' two), its module and potential partial (slot 2 mt + 1 of the tile), release
  auto producer_drain = [&](int ttd, int itd) {
    const TcTile T = tc_tile<false>(P, ttd, mtiles);
    const BlockDesc bd = P.blocks[T.b];
    // the consumers have set up this tile's column scales, weights and w V
    if (tid == 0 && !mbar_wait_bounded(smem_u32(&mb_tab), (uint32_t)(itd & 1))) {
      if (P.status_w) atomicCAS(P.status_w, 0, QD_ERR_TIMEOUT);
      abort_p = 1;
    }
    named_bar(1, WS_PROD);
    if (abort_p) return;
    float mod = 0.0f, pe = 0.0f;
    drain(T, bd, itd, warp & 3, 2 + (warp >> 2), 64, mod, pe);
    tc_fence_before();
    mbar_arrive(smem_u32(&mb_free));
    if (P.part) {
      for (int o = 16; o > 0; o >>= 1) {
        mod += __shfl_down_sync(0xffffffffu, mod, o);
        pe += __shfl_down_sync(0xffffffffu, pe, o);
      }
      if (lane == 0) {
        redp_s[warp] = mod;
        redp_s[8 + warp] = pe;
      }
      named_bar(1, WS_PROD);
      if (tid == 0) {
        float ms = 0.0f, ps = 0.0f;
        for (int q = 0; q < 8; q++) {
          ms += redp_s[q];
          ps += redp_s[8 + q];
        }
        P.part[((int64_t)T.b * P.n_part_tiles + 2 * T.mt + 1) * 2 + 0] = (double)ms;
        P.part[((int64_t)T.b * P.n_part_tiles + 2 * T.mt + 1) * 2 + 1] = (double)ps;
      }
      named_bar(1, WS_PROD);   // redp_s is rewritten only after thread 0 has read it
    }
  };

  if (TA && tid < WS_PROD) {
    // =============================== producers, A in TMEM: 256 threads; thread (w, lane)
    // slices row m = 32 (w & 3) + lane (its warp's TMEM lanes) over half of the k range
    // raw copy of tile tt into staging buffer buf: row k holds the 64 points' (re, im)
    auto issue = [&](int tt, int buf) {
      const TcTile T = tc_tile<false>(P, tt, mtiles);
      const BlockDesc bd = P.blocks[T.b];
      const int64_t p0 = (int64_t)T.mt * TC_POINTS;
      const float2 *A = P.A + (int64_t)bd.slab0 * g.npt;
      float *dst = sF + buf * kp_max * TC_LDR;
      for (int q = tid; q < T.Kp * TC_POINTS; q += WS_PROD) {
        const int k = q / TC_POINTS, pl = q % TC_POINTS;
        const int64_t pp = p0 + pl;
        float *d = dst + k * TC_LDR + 2 * pl;
        if (k < T.Kv && pp < g.npt)
          asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(d)), "l"(A + (int64_t)k * g.npt + pp)
                       : "memory");
        else
          *reinterpret_cast<float2 *>(d) = make_float2(0.0f, 0.0f);
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    };
    if (t_begin < t_end) issue(t_begin, 0);
    int cur_b = -1;
    const int qd = warp & 3, kh = warp >> 2;
    const int m = 32 * qd + lane;
    for (int tt = t_begin, it = 0; tt < t_end; tt++, it++) {
      const TcTile T = tc_tile<false>(P, tt, mtiles);
      const int buf = it & 1;
      if (tt + 1 < t_end) {
        issue(tt + 1, buf ^ 1);
        asm volatile("cp.async.wait_group 1;" ::: "memory");   // this thread's copies of tile tt
      } else {
        asm volatile("cp.async.wait_group 0;" ::: "memory");
      }
      named_bar(1, WS_PROD);   // ... and every producer's
      // the MMA of the previous tile must be done before A (TMEM) and B are rewritten
      if (tid == 0 && it > 0 && !mbar_wait_bounded(smem_u32(&mb_done), (uint32_t)((it - 1) & 1))) {
        if (P.status_w) atomicCAS(P.status_w, 0, QD_ERR_TIMEOUT);
        abort_p = 1;
      }
      named_bar(1, WS_PROD);
      tc_fence_after();
      if (abort_p) {
        asm volatile("cp.async.wait_group 0;" ::: "memory");   // no copy lands after the CTA is gone
        break;
      }
      if (T.b != cur_b) {
        const uint4 *src = reinterpret_cast<const uint4 *>(P.bimg + P.bimg_off[T.b] / 2);
        uint4 *dst = reinterpret_cast<uint4 *>(sB);
        const int n16 = (int)(tc_bimg_bytes(T.Np, T.Kp) / 16);
        for (int q = tid; q < n16; q += WS_PROD) dst[q] = __ldg(src + q);
        cur_b = T.b;
      }
      const float *row = sF + buf * kp_max * TC_LDR + m;   // element k at row[k * TC_LDR]
      const int KH = T.Kp / 2, k0 = kh * KH;               // KH: a multiple of 8
      float mx = 0.0f;
      for (int k = k0; k < k0 + KH; k++) mx = fmaxf(mx, fabsf(row[k * TC_LDR]));
      rmax_s[kh][m] = mx;
      named_bar(1, WS_PROD);
      mx = fmaxf(rmax_s[0][m], rmax_s[1][m]);
      // mx = f 2^e, f in [0.5, 1): row scale 2^e, slices of a = 256 x / 2^e
      const int e = mx >= 1e-30f ? (int)((__float_as_uint(mx) >> 23) & 0xffu) - 126 : 0;
      const float inv = mx >= 1e-30f ? __uint_as_float((uint32_t)(127 + 8 - e) << 23) : 0.0f;
      if (kh == 0) srow_s[it & 1][m] = __uint_as_float((uint32_t)(127 + e - 16) << 23);
      auto rne = [](float x) { return __fsub_rn(__fadd_rn(x, 12582912.0f), 12582912.0f); };
      const uint32_t tl = tmem + ((uint32_t)(32 * qd) << 16) + a_col0;
      for (int kg = 0; kg < KH / 8; kg++) {
        uint32_t w[3][4];
#pragma unroll
        for (int e2 = 0; e2 < 4; e2++) {
          uint32_t b[3][2];
#pragma unroll
          for (int h = 0; h < 2; h++) {
            const float a = __fmul_rn(row[(k0 + kg * 8 + 2 * e2 + h) * TC_LDR], inv);
            const float i0 = rne(a);
            const float r1 = __fmul_rn(__fsub_rn(a, i0), 256.0f);
            const float i1 = rne(r1);
            const float i2 = rne(__fmul_rn(__fsub_rn(r1, i1), 256.0f));
            b[0][h] = __float_as_uint(i0);
            b[1][h] = __float_as_uint(i1);
            b[2][h] = __float_as_uint(i2);
          }
#pragma unroll
          for (int t = 0; t < 3; t++) w[t][e2] = __byte_perm(b[t][0], b[t][1], 0x7632);   // even k low
        }
#pragma unroll
        for (int t = 0; t < 3; t++) tmem_st4(tl + (uint32_t)(t * KH + (k0 + kg * 8) / 2), w[t]);
      }
      tmem_wait_st();
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // the B image, when rewritten
      tc_fence_before();
      mbar_arrive(smem_u32(&mb_ready));
      // the previous tile's accumulators are complete (its MMA was waited for above): drain a share
      if (it > 0) producer_drain(tt - 1, it - 1);
      named_bar(1, WS_PROD);   // the staging buffer and rmax_s are rewritten only after every producer is done
    }
    // the last tile's share, once its MMA is done
    if (!abort_p && t_end > t_begin) {
      const int itl = t_end - 1 - t_begin;
      if (tid == 0 && !mbar_wait_bounded(smem_u32(&mb_done), (uint32_t)(itl & 1))) {
        if (P.status_w) atomicCAS(P.status_w, 0, QD_ERR_TIMEOUT);
        abort_p = 1;
      }
      named_bar(1, WS_PROD);
      if (!abort_p) {
        tc_fence_after();
        producer_drain(t_end - 1, itl);
      }
    }
  } else if (tid < WS_PROD) {
    // =============================== producers: 256 threads, two per row
    int cur_b = -1;
    for (int tt = t_begin, it = 0; tt < t_end; tt++, it++) {
      const TcTile T = tc_tile<FWD>(P, tt, mtiles);
      const BlockDesc bd = P.blocks[T.b];
      const int64_t p0 = (int64_t)T.mt * TC_POINTS;
      const float2 *A = P.A + (FWD ? (int64_t)T.b * g.nth * g.npt : (int64_t)bd.slab0 * g.npt);
      // L2 prefetch of the next tile (128-byte lines of its k rows)
      if (tt + 1 < t_end) {
        const TcTile Tn = tc_tile<FWD>(P, tt + 1, mtiles);
        const BlockDesc bn = P.blocks[Tn.b];
        const float2 *An = P.A + (FWD ? (int64_t)Tn.b * g.nth * g.npt : (int64_t)bn.slab0 * g.npt);
        const int64_t pn = (int64_t)Tn.mt * TC_POINTS;
        constexpr int LPR = 4;                          // 128-byte lines per k row: 64 points x 8 B
        constexpr int PPL = TC_POINTS / LPR;            // points per line
        const int lines = Tn.Kv * LPR;
        for (int q = tid; q < lines; q += WS_PROD) {
          const int k = q / LPR, ln = q % LPR;
          const int64_t pp = pn + ln * PPL;
          if (pp < g.npt) asm volatile("prefetch.global.L2 [%0];" ::"l"(An + (int64_t)k * g.npt + pp));
          if (FWD && P.vph && pp < g.npt)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(P.vph + (int64_t)k * g.npt + pp));
        }
      }
      // phase 1: A tile -> FP32 rows in sF
      {
        const int pl = tid % TC_POINTS;
        const int64_t p = p0 + pl;
        float msk = 1.0f;
        if (FWD && P.d1 && p < g.npt) msk = P.d1[(int)(p % g.n1)] * P.d2[(int)(p / g.n1)];
        constexpr int U = 24;   // all of a 96-row tile's loads (and shears) in flight in one batch
        const int nk = T.Kp / 4;   // this thread's k values: tid/64 + 4u
        for (int u0 = 0; u0 < nk; u0 += U) {
          float2 v[U];
          float2 ts[U];
#pragma unroll
          for (int u = 0; u < U; u++) {
            const int k = tid / TC_POINTS + 4 * (u0 + u);
            const bool in = u0 + u < nk && k < T.Kv && p < g.npt;
            v[u] = in ? A[(int64_t)k * g.npt + p] : make_float2(0.0f, 0.0f);
            if (FWD) ts[u] = (in && P.vph) ? __ldg(P.vph + (int64_t)k * g.npt + p) : make_float2(0.0f, 0.0f);
          }
#pragma unroll
          for (int u = 0; u < U; u++) {
            if (u0 + u >= nk) break;
            const int k = tid / TC_POINTS + 4 * (u0 + u);
            float x = v[u].x, y = v[u].y;
            if (FWD) {
              x *= msk;
              y *= msk;
              if (P.vph) rot_lift2(x, y, ts[u]);
            }
            sF[k * TC_LDM + pl] = x;
            sF[k * TC_LDM + TC_IM + pl] = y;
          }
        }
      }
      named_bar(1, WS_PROD);
      // the MMA of the previous tile must be done before A (and B) are rewritten;
      // one thread waits and the group decides together (no divergent exit)
      if (tid == 0 && it > 0 && !mbar_wait_bounded(smem_u32(&mb_done), (uint32_t)((it - 1) & 1))) {
        if (P.status_w) atomicCAS(P.status_w, 0, QD_ERR_TIMEOUT);
        abort_p = 1;
      }
      named_bar(1, WS_PROD);
      if (abort_p) break;
      if (T.b != cur_b) {
        const uint4 *src = reinterpret_cast<const uint4 *>(P.bimg + P.bimg_off[T.b] / 2);
        uint4 *dst = reinterpret_cast<uint4 *>(sB);
        const int n16 = (int)(tc_bimg_bytes(T.Np, T.Kp) / 16);
        for (int q = tid; q < n16; q += WS_PROD) dst[q] = __ldg(src + q);
        cur_b = T.b;
      }
      // phase 2: lanes l and l+16 of warp w scale row m = 16 w + l and slice the even and
      // the odd k groups; each group of 8 lanes then writes 128 contiguous image bytes
      {
        const int m = 16 * warp + (lane & 15), half = lane >> 4;
        const float *row = sF + (m >> 1) + TC_IM * (m & 1);   // element k at row[k * TC_LDM]
        float mx = 0.0f;
        for (int kg = half; kg < T.Kp / 8; kg += 2)
#pragma unroll
          for (int e8 = 0; e8 < 8; e8++) mx = fmaxf(mx, fabsf(row[(kg * 8 + e8) * TC_LDM]));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 16));
        // mx = f 2^e, f in [0.5, 1): row scale 2^e, slices of a = 256 x / 2^e
        const int e = mx >= 1e-30f ? (int)((__float_as_uint(mx) >> 23) & 0xffu) - 126 : 0;
        const float inv = mx >= 1e-30f ? __uint_as_float((uint32_t)(127 + 8 - e) << 23) : 0.0f;
        if (half == 0) srow_s[it & 1][m] = __uint_as_float((uint32_t)(127 + e - 16) << 23);
        const uint32_t orow = (uint32_t)(m / 8) * T.SBO + (m % 8) * 16;
        // round to nearest even integer for |x| <= 2^22: (x + 1.5 2^23) - 1.5 2^23
        auto rne = [](float x) { return __fsub_rn(__fadd_rn(x, 12582912.0f), 12582912.0f); };
        for (int kg = half; kg < T.Kp / 8; kg += 2) {
          uint32_t w[3][4];
#pragma unroll
          for (int e2 = 0; e2 < 4; e2++) {
            uint32_t b[3][2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
              const float a = __fmul_rn(row[(kg * 8 + 2 * e2 + h) * TC_LDM], inv);
              const float i0 = rne(a);
              const float r1 = __fmul_rn(__fsub_rn(a, i0), 256.0f);
              const float i1 = rne(r1);
              const float i2 = rne(__fmul_rn(__fsub_rn(r1, i1), 256.0f));
              // |i| <= 256 integers: the BF16 encoding is the upper half of the FP32 one
              b[0][h] = __float_as_uint(i0);
              b[1][h] = __float_as_uint(i1);
              b[2][h] = __float_as_uint(i2);
            }
#pragma unroll
            for (int t = 0; t < 3; t++) w[t][e2] = __byte_perm(b[t][0], b[t][1], 0x7632);
          }
#pragma unroll
          for (int t = 0; t < 3; t++)
            *reinterpret_cast<uint4 *>(sA + t * T.A_TERM + orow + kg * 128) =
                make_uint4(w[t][0], w[t][1], w[t][2], w[t][3]);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(smem_u32(&mb_ready));
      named_bar(1, WS_PROD);   // sF is rewritten only after every producer has sliced
    }
  } else {
    // =============================== consumers: 256 threads (+ the MMA issuer, thread 256)
    const int ctid = tid - WS_PROD, cw = warp - WS_PROD / 32;
    const int quarter = warp & 3, chalf = cw >> 2;
    int cons_b = -1;
    for (int tt = t_begin, it = 0; tt < t_end; tt++, it++) {
      const TcTile T = tc_tile<FWD>(P, tt, mtiles);
      const BlockDesc bd = P.blocks[T.b];
      // backward: the tile's w V values [n][64 points], copied asynchronously into
      // shared memory before the MMA wait, 16 bytes (4 points) per copy spread over
      // all consumer threads (a 4-byte copy per point where the tile ends early)
      if (!FWD) {
        const int64_t p0 = (int64_t)T.mt * TC_POINTS;
        for (int q = ctid; q < T.Nv * (TC_POINTS / 4); q += WS_THREADS - WS_PROD) {
          const int n = q / (TC_POINTS / 4), c4 = 4 * (q % (TC_POINTS / 4));
          const float *src = P.wv + (int64_t)n * g.npt + p0 + c4;
          const uint32_t dst = smem_u32(sWV + (TA ? (it & 1) * np_max * TC_POINTS : 0) + n * TC_POINTS + c4);
          if (p0 + c4 + 4 <= g.npt) {
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
          } else {
            for (int e = 0; e < 4 && p0 + c4 + e < g.npt; e++)
              asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst + 4 * e), "l"(src + e) : "memory");
          }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
      }
      if (ctid == MMA_ISSUER) {
        bool ok = mbar_wait_bounded(smem_u32(&mb_ready), (uint32_t)(it & 1));
        if (ok && it > 0) ok = mbar_wait_bounded(smem_u32(&mb_free), (uint32_t)((it - 1) & 1));
        if (!ok) {
          if (P.status_w) atomicCAS(P.status_w, 0, QD_ERR_TIMEOUT);
          abort_c = 1;
        } else {
          tc_fence_after();
          const uint32_t idesc = make_idesc(128, T.Np);
          const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
          if (TA) {
            // A term t of k step s: TMEM columns a_col0 + t Kp/2 + 8 s (16 BF16 values)
            const uint32_t ta = tmem + a_col0, KH = (uint32_t)(T.Kp / 2);
            if (2 * T.Np <= 256) {
              const uint32_t idesc2 = make_idesc(128, 2 * T.Np);
              for (int s = 0; s < T.Kp / 16; s++) {
                const uint32_t acc = s > 0 ? 1u : 0u;
                const uint64_t bd0 = make_desc(b0 + s * 256, 128, T.SBO);
                mma_bf16_ta(tmem, ta + 8 * s, bd0, idesc2, acc);
                mma_bf16_ta(tmem + (uint32_t)(2 * T.Np), ta + 8 * s,
                            make_desc(b0 + 2 * T.B_TERM + s * 256, 128, T.SBO), idesc, acc);
                mma_bf16_ta(tmem + (uint32_t)T.Np, ta + KH + 8 * s, bd0, idesc2, 1u);
                mma_bf16_ta(tmem + (uint32_t)(2 * T.Np), ta + 2 * KH + 8 * s, bd0, idesc, 1u);
              }
            } else {
              for (int s = 0; s < T.Kp / 16; s++) {
#pragma unroll
                for (int q = 0; q < 6; q++) {
                  const int d = c_pair_a[q] + c_pair_b[q];
                  const uint64_t bdsc = make_desc(b0 + c_pair_b[q] * T.B_TERM + s * 256, 128, T.SBO);
                  const bool first = s == 0 && (q == 0 || q == 1 || q == 3);
                  mma_bf16_ta(tmem + (uint32_t)(d * T.Np), ta + c_pair_a[q] * KH + 8 * s, bdsc, idesc,
                              first ? 0u : 1u);
                }
              }
            }
          } else if (2 * T.Np <= 256) {
            // B0 and B1 are adjacent in shared memory and D0, D1, D2 in TMEM, so
            // A0 [B0 B1] -> [D0 D1] and A1 [B0 B1] -> [D1 D2] are single N = 2 Np
            // MMAs: four per k step instead of six, same sums
            const uint32_t idesc2 = make_idesc(128, 2 * T.Np);
            for (int s = 0; s < T.Kp / 16; s++) {
              const uint32_t acc = s > 0 ? 1u : 0u;
              const uint64_t bd0 = make_desc(b0 + s * 256, 128, T.SBO);
              mma_bf16(tmem, make_desc(a0 + s * 256, 128, T.SBO), bd0, idesc2, acc);
              mma_bf16(tmem + (uint32_t)(2 * T.Np), make_desc(a0 + s * 256, 128, T.SBO),
                       make_desc(b0 + 2 * T.B_TERM + s * 256, 128, T.SBO), idesc, acc);
              mma_bf16(tmem + (uint32_t)T.Np, make_desc(a0 + T.A_TERM + s * 256, 128, T.SBO), bd0, idesc2, 1u);
              mma_bf16(tmem + (uint32_t)(2 * T.Np), make_desc(a0 + 2 * T.A_TERM + s * 256, 128, T.SBO), bd0, idesc,
                       1u);
            }
          } else {
            for (int s = 0; s < T.Kp / 16; s++) {
#pragma unroll
              for (int q = 0; q < 6; q++) {
                const int d = c_pair_a[q] + c_pair_b[q];
                const uint64_t ad = make_desc(a0 + c_pair_a[q] * T.A_TERM + s * 256, 128, T.SBO);
                const uint64_t bdsc = make_desc(b0 + c_pair_b[q] * T.B_TERM + s * 256, 128, T.SBO);
                const bool first = s == 0 && (q == 0 || q == 1 || q == 3);
                mma_bf16(tmem + (uint32_t)(d * T.Np), ad, bdsc, idesc, first ? 0u : 1u);
              }
            }
          }
          mma_commit(smem_u32(&mb_done));
          n_issued = it + 1;
          // this thread observes completion for the group
          if (!mbar_wait_bounded(smem_u32(&mb_done), (uint32_t)(it & 1))) {
            if (P.status_w) atomicCAS(P.status_w, 0, QD_ERR_TIMEOUT);
            abort_c = 1;
          }
        }
        tc_fence_before();
      }
      __syncwarp();
      if (!FWD) asm volatile("cp.async.wait_all;" ::: "memory");   // this thread's w V copies have landed
      named_bar(2, WS_THREADS - WS_PROD);                          // ... and so have everyone's
      if (abort_c) break;
      if (TA || T.b != cons_b) {   // the A-in-TMEM form keeps one set per tile parity
        const int par = TA ? (it & 1) : 0;
        for (int n = ctid; n < 256; n += WS_THREADS - WS_PROD) {
          tsc_s[par][n] = n < T.Np ? __ldg(P.bscale + (int64_t)T.b * 256 + n) : 0.0f;
          if (!FWD) w_s[par][n] = n < T.Nv ? __ldg(P.w + n) : 0.0f;
        }
        cons_b = T.b;
        named_bar(2, WS_THREADS - WS_PROD);
      }
      if (TA) mbar_arrive(smem_u32(&mb_tab));   // the producers may drain their share of this tile now
      tc_fence_after();
      float mod = 0.0f, pe = 0.0f;
      // the consumers' share: column chunks chalf of two, or (A in TMEM) of four with the producers
      drain(T, bd, it, quarter, chalf, TA ? 64 : 32, mod, pe);
      tc_fence_before();
      mbar_arrive(smem_u32(&mb_free));
      __syncwarp();
      if (!FWD && P.part) {
        // fixed-order reduction over the 256 consumer threads
        for (int o = 16; o > 0; o >>= 1) {
          mod += __shfl_down_sync(0xffffffffu, mod, o);
          pe += __shfl_down_sync(0xffffffffu, pe, o);
        }
        if (lane == 0) {
          red_s[cw] = mod;
          red_s[8 + cw] = pe;
        }
        named_bar(2, WS_THREADS - WS_PROD);   // also: every consumer is done with the w V tile
        if (ctid == 0) {   // red_s is next written after the next tile's MMA barrier
          float ms = 0.0f, ps = 0.0f;
          for (int q = 0; q < 8; q++) {
            ms += red_s[q];
            ps += red_s[8 + q];
          }
          const int64_t slot = (int64_t)T.b * P.n_part_tiles + (TA ? 2 * T.mt : T.mt);
          P.part[slot * 2 + 0] = (double)ms;
          P.part[slot * 2 + 1] = (double)ps;
        }
      } else if (!FWD) {
        named_bar(2, WS_THREADS - WS_PROD);   // every consumer is done with the w V tile
      }
    }
  }
  // ---- drain: after a timeout, wait (bounded) for the last MMA chain issued
  __syncthreads();
  if (tid == WS_PROD + MMA_ISSUER && (abort_p || abort_c) && n_issued > 0)
    mbar_wait_bounded(smem_u32(&mb_done), (uint32_t)((n_issued - 1) & 1));
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, ncols);
  }
}

// Dynamic shared memory of the persistent kernel: the BF16 slices of A and B,
// the FP32 staging rows and (backward) the w V tile, and at least 120 KB so
// that one CTA (holding all 512 TMEM columns) runs per SM.
size_t tc_ws_smem_bytes(bool fwd, int kp_max, int np_max) {
  const size_t need = (size_t)3 * 16 * (kp_max / 8 * 128) + (size_t)tc_bimg_bytes(np_max, kp_max) +
                      (size_t)kp_max * TC_LDM * 4 + (fwd ? 0 : (size_t)np_max * TC_POINTS * 4);
  return std::max(need, (size_t)120 * 1024);
}

bool tc_shape_ok(bool fwd, int Kp, int Np) {
  return Kp <= 192 && Np <= 160 && tc_ws_smem_bytes(fwd, Kp, Np) <= 220 * 1024;
}

// The backward contraction with its A slices in TMEM: the B slices, two raw staging buffers and
// two w V tiles in shared memory; usable when the accumulators and the A slices share the 512
// TMEM columns.
static size_t tc_ta_smem_bytes(int kp_max, int np_max) {
  const size_t need = (size_t)tc_bimg_bytes(np_max, kp_max) + (size_t)2 * kp_max * TC_LDR * 4 +
                      (size_t)2 * np_max * TC_POINTS * 4;
  return std::max(need, (size_t)120 * 1024);
}
static bool tc_ta_ok(int kp_max, int np_max) {
  return tc_a_col0(np_max) + 3u * (uint32_t)(kp_max / 2) <= 512u && tc_ta_smem_bytes(kp_max, np_max) <= 220 * 1024;
}

int legendre_tc_part_tiles(const Grid &g) { return (int)((g.npt + TC_POINTS - 1) / TC_POINTS); }
// module/potential partial slots per block of the backward contraction: one per tile, or two in
// the A-in-TMEM form (the consumers' and the producers' share of each tile's drain)
int legendre_tc_part_slots(const Grid &g, int max_nl) {
  return legendre_tc_part_tiles(g) * (tc_ta_ok(round16(max_nl), round16(g.nth)) ? 2 : 1);
}


void launch_legendre_tc_ws(cudaStream_t s, bool fwd, const TcArgs &a, int n_blocks, int kp_max, int np_max) {
  const int mtiles = legendre_tc_part_tiles(a.g);
  const int n_tiles = mtiles * n_blocks;
  int dev = 0, sms = 0;
  QD_CUDA(cudaGetDevice(&dev));
  QD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int grid = std::min(n_tiles, sms);
  if (fwd)
    k_legendre_tc_ws<true><<<grid, WS_THREADS, tc_ws_smem_bytes(true, kp_max, np_max), s>>>(a, mtiles, n_tiles,
                                                                                             kp_max, np_max);
  else if (tc_ta_ok(kp_max, np_max))
    k_legendre_tc_ws<false, true><<<grid, WS_THREADS, tc_ta_smem_bytes(kp_max, np_max), s>>>(a, mtiles, n_tiles,
                                                                                              kp_max, np_max);
  else
    k_legendre_tc_ws<false><<<grid, WS_THREADS, tc_ws_smem_bytes(false, kp_max, np_max), s>>>(a, mtiles, n_tiles,
                                                                                              kp_max, np_max);
}


void launch_legendre_tc_fwd(cudaStream_t s, const Grid &g, const float2 *psi_th, float2 *psi_j,
                            const BlockDesc *blocks, int n_blocks, const uint16_t *img, const int64_t *img_off,
                            const float2 *vph, const float *d1f, const float *d2f, size_t smem, const int *status,
                            int *status_w, const float *bscale, int max_nl) {
  TcArgs a{};
  a.bscale = bscale;
  a.g = g;
  a.A = psi_th;
  a.C = psi_j;
  a.blocks = blocks;
  a.bimg = img;
  a.bimg_off = img_off;
  a.vph = vph;
  a.d1 = d1f;
  a.d2 = d2f;
  a.status = status;
  a.status_w = status_w;
  (void)smem;
  launch_legendre_tc_ws(s, true, a, n_blocks, round16(g.nth), round16(max_nl));
}

void launch_legendre_tc_bwd(cudaStream_t s, const Grid &g, const float2 *psi_j, float2 *psi_th,
                            const BlockDesc *blocks, int n_blocks, const uint16_t *img, const int64_t *img_off,
                            const float *wf, const float *wvf, double *part, int n_part_tiles, size_t smem,
                            const int *status, int *status_w, const float *bscale, int max_nl) {
  TcArgs a{};
  a.bscale = bscale;
  a.g = g;
  a.A = psi_j;
  a.C = psi_th;
  a.blocks = blocks;
  a.bimg = img;
  a.bimg_off = img_off;
  a.w = wf;
  a.wv = wvf;
  a.part = part;
  a.n_part_tiles = n_part_tiles;
  a.status = status;
  a.status_w = status_w;
  (void)smem;
  launch_legendre_tc_ws(s, false, a, n_blocks, round16(max_nl), round16(g.nth));
}

void tc_set_smem_limit(size_t bytes) {
  QD_CUDA(cudaFuncSetAttribute(k_legendre_tc_ws<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  QD_CUDA(cudaFuncSetAttribute(k_legendre_tc_ws<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  QD_CUDA(cudaFuncSetAttribute(k_legendre_tc_ws<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)bytes));
}

void launch_build_tc_bimage(cudaStream_t s, const BlockDesc *blocks, int n_blocks, const double *Bsrc, int nth,
                            bool fwd, const int64_t *img_off, uint16_t *img, float *bscale, int max_np) {
  k_build_tc_bimage<<<dim3(max_np, n_blocks), 128, 0, s>>>(blocks, Bsrc, nth, fwd ? 1 : 0, img_off, img, bscale);
}

}  // namespace qd
