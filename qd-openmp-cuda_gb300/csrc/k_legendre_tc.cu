// Mixed-precision theta <-> j Legendre contraction on the 5th-generation
// tensor cores (tcgen05, sm_103a).
//
// Reference: the two cublasZgemm calls of omegawavepacket.cu:200-240.  The
// contraction is a real GEMM over the interleaved view of psi: rows
// m = 2*point + {re, im}, so C[m][n] = sum_k A[m][k] B[n][k] with B the real
// (weighted) associated-Legendre matrix.
//
// Precision: every FP32 value x is split into three BF16 terms
// x = a0 + a1 + a2 (a1 = bf16(x - a0), a2 = bf16(x - a0 - a1)); the products
// a_i b_j with i + j <= 2 (six of them) are accumulated in one FP32 TMEM
// accumulator, which reproduces an FP32-accurate product.  B (constant per
// Omega block) is split once at set-up, in FP64, into its shared-memory image.
//
// Per CTA: 64 points (M = 128 real rows) x all N columns.  Four warps stage
// the A tile (FP64 load -> FP32 -> forward: absorbing mask and exp(-iV dt) as
// an exactly area-preserving three-shear rotation -> BF16x3 split) into the
// SWIZZLE_NONE K-major canonical layout; one thread issues the tcgen05.mma
// chain; the commit arrives on an mbarrier; the four warps read their 32 TMEM
// lanes back (tcgen05.ld 32x32b), convert to FP64 and store.  The backward
// epilogue also reduces the module and potential energy.
#include <cuda_bf16.h>

#include "qd_internal.h"
#include "qd_device.cuh"

namespace qd {

namespace {
constexpr int TC_THREADS = 128;
constexpr int TC_POINTS = 64;        // 128 real rows
constexpr uint64_t WAIT_NS = 1000000000ull;   // give up waiting for the MMA chain after 1 s

__device__ inline uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

__device__ inline uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// SWIZZLE_NONE, K-major shared-memory matrix descriptor (tcgen05 form):
// start address, leading byte offset (between core matrices along K), stride
// byte offset (between 8-row groups), descriptor version 1 at bits 46-47.
__device__ inline uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// kind::f16 instruction descriptor: D = F32, A = B = BF16, both K-major.
__host__ __device__ inline uint32_t make_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ inline void mbar_init(uint32_t a, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ inline bool mbar_try_wait(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ inline void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ inline void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ inline void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ inline void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ inline void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ inline void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ inline void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 16; q++) v[q] = __uint_as_float(r[q]);
}

__device__ inline void split3(float x, uint16_t &a0, uint16_t &a1, uint16_t &a2) {
  const __nv_bfloat16 b0 = __float2bfloat16_rn(x);
  float r = x - __bfloat162float(b0);
  const __nv_bfloat16 b1 = __float2bfloat16_rn(r);
  r = r - __bfloat162float(b1);
  const __nv_bfloat16 b2 = __float2bfloat16_rn(r);
  a0 = __bfloat16_as_ushort(b0);
  a1 = __bfloat16_as_ushort(b1);
  a2 = __bfloat16_as_ushort(b2);
}

__device__ inline int round16(int x) { return (x + 15) & ~15; }

// products a_i * b_j with i + j <= 2
__constant__ int c_pair_a[6] = {0, 0, 1, 0, 1, 2};
__constant__ int c_pair_b[6] = {0, 1, 0, 2, 1, 0};
}  // namespace

// byte size of the B image of one block: 3 terms x Npad x Kpad BF16
__host__ __device__ inline int64_t tc_bimg_bytes(int Np, int Kp) { return 3LL * Np * Kp * 2; }

// ---------------------------------------------------------------------------
// B images: element (n, k) of term t at t*Np*Kp*2 + (n/8)*SBO + (k/8)*128 +
// (n%8)*16 + (k%8)*2 bytes with SBO = Kp/8*128 (SWIZZLE_NONE, K-major).
// fwd: B(n = l, k = theta) = w_k P_l(x_k) = Bf[k*nl + n]
// bwd: B(n = theta, k = l) = P_l(x_n)     = Bb[k*nth + n]
__global__ void k_build_tc_bimage(const BlockDesc *__restrict__ blocks, const double *__restrict__ Bsrc, int nth,
                                  int fwd, const int64_t *__restrict__ img_off, uint16_t *__restrict__ img) {
  const BlockDesc bd = blocks[blockIdx.y];
  const int Kv = fwd ? nth : bd.nl, Nv = fwd ? bd.nl : nth;
  const int Kp = (Kv + 15) & ~15, Np = (Nv + 15) & ~15;
  uint16_t *out = img + img_off[blockIdx.y] / 2;
  const int SBOe = Kp / 8 * 64;   // in elements
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < Np * Kp; q += gridDim.x * blockDim.x) {
    const int n = q / Kp, k = q % Kp;
    double b = 0.0;
    if (n < Nv && k < Kv) b = fwd ? Bsrc[bd.bmat0 + (int64_t)k * bd.nl + n] : Bsrc[bd.bmat0 + (int64_t)k * nth + n];
    const __nv_bfloat16 b0 = __double2bfloat16(b);
    const double r1 = b - (double)__bfloat162float(b0);
    const __nv_bfloat16 b1 = __double2bfloat16(r1);
    const double r2 = r1 - (double)__bfloat162float(b1);
    const __nv_bfloat16 b2 = __double2bfloat16(r2);
    const int64_t e = (int64_t)(n / 8) * SBOe + (k / 8) * 64 + (n % 8) * 8 + (k % 8);
    out[e] = __bfloat16_as_ushort(b0);
    out[(int64_t)Np * Kp + e] = __bfloat16_as_ushort(b1);
    out[2LL * Np * Kp + e] = __bfloat16_as_ushort(b2);
  }
}

struct TcArgs {
  Grid g;
  const double2 *A;          // fwd: psi_theta pool, bwd: psi_j pool
  double2 *C;                // fwd: psi_j pool, bwd: psi_theta pool
  const BlockDesc *blocks;
  const uint16_t *bimg;      // B images
  const int64_t *bimg_off;   // per block byte offset
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

template <bool FWD>
__global__ void __launch_bounds__(TC_THREADS, 1) k_legendre_tc(TcArgs P) {
  if (P.status && *P.status) return;
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_base_s;
  __shared__ double red[32];
  const BlockDesc bd = P.blocks[blockIdx.y];
  const Grid &g = P.g;
  const int Kv = FWD ? g.nth : bd.nl, Nv = FWD ? bd.nl : g.nth;
  const int Kp = round16(Kv), Np = round16(Nv);
  const uint32_t SBO_A = (uint32_t)(Kp / 8 * 128), SBO_B = SBO_A;
  const uint32_t A_TERM = 16u * SBO_A;                 // 128 rows
  const uint32_t B_TERM = (uint32_t)(Np / 8) * SBO_B;
  unsigned char *sA = smem;
  unsigned char *sB = smem + 3 * A_TERM;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t p0 = (int64_t)blockIdx.x * TC_POINTS;
  const uint32_t ncols = Np <= 32 ? 32 : (Np <= 64 ? 64 : (Np <= 128 ? 128 : 256));

  if (warp == 0) tmem_alloc(smem_u32(&tmem_base_s), ncols);
  if (tid == 0) {
    mbar_init(smem_u32(&mbar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }

  // ---- B image -> shared memory
  {
    const uint4 *src = reinterpret_cast<const uint4 *>(P.bimg + P.bimg_off[blockIdx.y] / 2);
    uint4 *dst = reinterpret_cast<uint4 *>(sB);
    const int n16 = (int)(tc_bimg_bytes(Np, Kp) / 16);
    for (int q = tid; q < n16; q += TC_THREADS) dst[q] = __ldg(src + q);
  }
  // ---- A tile: (point, group of 8 k) items
  {
    const double2 *A = FWD ? P.A + (int64_t)blockIdx.y * g.nth * g.npt : P.A + (int64_t)bd.slab0 * g.npt;
    const int kgs = Kp / 8;
    for (int it = tid; it < TC_POINTS * kgs; it += TC_THREADS) {
      const int pl = it % TC_POINTS, kg = it / TC_POINTS;
      const int64_t p = p0 + pl;
      uint32_t wre[3][4], wim[3][4];
      float msk = 1.0f;
      if (FWD && P.d1 && p < g.npt) msk = P.d1[p % g.n1] * P.d2[p / g.n1];
#pragma unroll
      for (int e = 0; e < 8; e++) {
        const int k = kg * 8 + e;
        float x = 0.0f, y = 0.0f;
        if (k < Kv && p < g.npt) {
          const double2 v = A[(int64_t)k * g.npt + p];
          x = (float)v.x;
          y = (float)v.y;
          if (FWD) {
            x *= msk;
            y *= msk;
            if (P.vph) rot_lift2(x, y, __ldg(P.vph + (int64_t)k * g.npt + p));
          }
        }
        uint16_t a[3], b[3];
        split3(x, a[0], a[1], a[2]);
        split3(y, b[0], b[1], b[2]);
#pragma unroll
        for (int t = 0; t < 3; t++) {
          if (e & 1) {
            wre[t][e >> 1] |= (uint32_t)a[t] << 16;
            wim[t][e >> 1] |= (uint32_t)b[t] << 16;
          } else {
            wre[t][e >> 1] = a[t];
            wim[t][e >> 1] = b[t];
          }
        }
      }
      const int mre = 2 * pl, mim = 2 * pl + 1;
      const uint32_t ore = (uint32_t)(mre / 8) * SBO_A + (mre % 8) * 16 + kg * 128;
      const uint32_t oim = (uint32_t)(mim / 8) * SBO_A + (mim % 8) * 16 + kg * 128;
#pragma unroll
      for (int t = 0; t < 3; t++) {
        *reinterpret_cast<uint4 *>(sA + t * A_TERM + ore) = make_uint4(wre[t][0], wre[t][1], wre[t][2], wre[t][3]);
        *reinterpret_cast<uint4 *>(sA + t * A_TERM + oim) = make_uint4(wim[t][0], wim[t][1], wim[t][2], wim[t][3]);
      }
    }
  }
  // make the generic-proxy shared stores visible to the tensor core (async proxy)
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;

  if (tid == 0) {
    const uint32_t idesc = make_idesc(128, Np);
    const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
    for (int s = 0; s < Kp / 16; s++) {
#pragma unroll
      for (int q = 0; q < 6; q++) {
        const uint64_t ad = make_desc(a0 + c_pair_a[q] * A_TERM + s * 256, 128, SBO_A);
        const uint64_t bdsc = make_desc(b0 + c_pair_b[q] * B_TERM + s * 256, 128, SBO_B);
        mma_bf16(tmem, ad, bdsc, idesc, (s | q) != 0);
      }
    }
    mma_commit(smem_u32(&mbar));
  }
  // ---- wait for the MMA chain (bounded in wall-clock time); on a timeout
  // flag the error, wait once more (bounded) for the chain, free TMEM, return
  bool ok = false;
  {
    const uint64_t t0 = globaltimer();
    while (!(ok = mbar_try_wait(smem_u32(&mbar), 0)))
      if (globaltimer() - t0 > WAIT_NS) break;
  }
  if (!ok) {
    if (tid == 0 && P.status_w) atomicCAS(P.status_w, 0, QD_ERR_CUDA);
    const uint64_t t0 = globaltimer();
    while (!mbar_try_wait(smem_u32(&mbar), 0))
      if (globaltimer() - t0 > WAIT_NS) break;
  }
  tc_fence_after();

  // ---- epilogue: warp w owns TMEM lanes (rows) 32w .. 32w+31
  const int m = 32 * warp + lane;
  const int pl = m >> 1, c = m & 1;
  const int64_t p = p0 + pl;
  float mod = 0.0f, pe = 0.0f;
  double *Cd = reinterpret_cast<double *>(P.C);
  for (int n0 = 0; n0 < Np; n0 += 16) {
    float v[16];
    tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)n0, v);
    if (!ok || p >= g.npt) continue;
#pragma unroll
    for (int q = 0; q < 16; q++) {
      const int n = n0 + q;
      if (n >= Nv) break;
      if (FWD) {
        Cd[2 * ((int64_t)(bd.slab0 + n) * g.npt + p) + c] = (double)v[q];
      } else {
        Cd[2 * (((int64_t)blockIdx.y * g.nth + n) * g.npt + p) + c] = (double)v[q];
        const float v2 = v[q] * v[q];
        mod = fmaf(__ldg(P.w + n), v2, mod);
        pe = fmaf(__ldg(P.wv + (int64_t)n * g.npt + p), v2, pe);
      }
    }
  }
  if (!FWD && P.part) {
    const double m2 = block_sum((double)mod, red);
    const double p2 = block_sum((double)pe, red);
    if (tid == 0) {
      P.part[((int64_t)blockIdx.y * P.n_part_tiles + blockIdx.x) * 2 + 0] = m2;
      P.part[((int64_t)blockIdx.y * P.n_part_tiles + blockIdx.x) * 2 + 1] = p2;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, ncols);
  }
}

// Dynamic shared memory of one launch: the A and B tiles, and at least
// ncols * 456 bytes so that no more than 512/ncols CTAs share an SM (the
// TMEM columns that their allocations need never exceed the SM's 512).
size_t tc_smem_bytes(int Kp, int Np) {
  const size_t need = (size_t)3 * 16 * (Kp / 8 * 128) + (size_t)tc_bimg_bytes(Np, Kp);
  const size_t ncols = Np <= 32 ? 32 : (Np <= 64 ? 64 : (Np <= 128 ? 128 : 256));
  return std::max(need, ncols * 456 + 1024);
}

int legendre_tc_part_tiles(const Grid &g) { return (int)((g.npt + TC_POINTS - 1) / TC_POINTS); }

void launch_legendre_tc_fwd(cudaStream_t s, const Grid &g, const double2 *psi_th, double2 *psi_j,
                            const BlockDesc *blocks, int n_blocks, const uint16_t *img, const int64_t *img_off,
                            const float2 *vph, const float *d1f, const float *d2f, size_t smem, const int *status,
                            int *status_w) {
  TcArgs a{};
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
  dim3 grid((unsigned)legendre_tc_part_tiles(g), (unsigned)n_blocks);
  k_legendre_tc<true><<<grid, TC_THREADS, smem, s>>>(a);
}

void launch_legendre_tc_bwd(cudaStream_t s, const Grid &g, const double2 *psi_j, double2 *psi_th,
                            const BlockDesc *blocks, int n_blocks, const uint16_t *img, const int64_t *img_off,
                            const float *wf, const float *wvf, double *part, int n_part_tiles, size_t smem,
                            const int *status, int *status_w) {
  TcArgs a{};
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
  dim3 grid((unsigned)legendre_tc_part_tiles(g), (unsigned)n_blocks);
  k_legendre_tc<false><<<grid, TC_THREADS, smem, s>>>(a);
}

void tc_set_smem_limit(size_t bytes) {
  QD_CUDA(cudaFuncSetAttribute(k_legendre_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  QD_CUDA(cudaFuncSetAttribute(k_legendre_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

void launch_build_tc_bimage(cudaStream_t s, const BlockDesc *blocks, int n_blocks, const double *Bsrc, int nth,
                            bool fwd, const int64_t *img_off, uint16_t *img) {
  k_build_tc_bimage<<<dim3(8, n_blocks), 256, 0, s>>>(blocks, Bsrc, nth, fwd ? 1 : 0, img_off, img);
}

}  // namespace qd
