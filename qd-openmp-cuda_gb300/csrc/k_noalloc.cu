// Rotational energy of one Omega block without any device allocation.
//
// Same quantity as the session's rotational-energy reduction (the
// QD_STAGE_ENERGIES path): dr1 dr2 sum_l l(l+1) sum_{R,r} (1/(2 m1 R^2) +
// 1/(2 m2 r^2)) |psi_l(R, r)|^2.  The per-CTA partial sums, which the session
// keeps in memory it allocates with cudaMalloc, live here in a file-scope
// device array instead, so that a caller whose device memory is all owned by
// someone else (a framework's caching allocator such as PyTorch's or MATLAB's
// gpuArray pool, or a loop in which the implicit device synchronisation of
// cudaMalloc is not allowed) can still call it with only its own input and
// output buffers.
#include "qd_internal.h"
#include "qd_device.cuh"

namespace qd {

namespace {
// Partial sums of the most recent call: at most QD_NOALLOC_MAX_PARTIALS
// doubles (512 KiB), held by every GPU that loads the library until exit.
constexpr int QD_NOALLOC_MAX_PARTIALS = 65536;
constexpr int NOALLOC_TILES = 16;     // CTAs per Legendre slab
constexpr int NOALLOC_THREADS = 256;
static __device__ __align__(256) double g_rot_energy_scratch[QD_NOALLOC_MAX_PARTIALS];

// Device address of the scratch array in the current device's context.  In host
// code the array's name is only a host-side stand-in, never a device address, so
// every call looks the address up again: that is cheap, allocates nothing, and
// stays right after a cudaDeviceReset or under a different context on the device,
// where an address cached from an earlier call would no longer be valid.
double *scratch_for_current_device() {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_rot_energy_scratch);
  if (e != cudaSuccess)
    throw Error{QD_ERR_CUDA, std::string("cudaGetSymbolAddress(rotational-energy scratch): ") + cudaGetErrorString(e)};
  return static_cast<double *>(p);
}
}  // namespace

// Partials of slab s (l = omega + s) over a strided tile of its points.
__global__ void k_rot_energy_block(Grid g, const double2 *__restrict__ psi_j, int omega, double *__restrict__ part) {
  __shared__ double red[32];
  const int sl = blockIdx.y;
  const double l = (double)(omega + sl);
  const double ll = l * (l + 1.0);
  const double2 *p = psi_j + (int64_t)sl * g.npt;
  double acc = 0.0;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < g.npt;
       q += (int64_t)NOALLOC_TILES * blockDim.x) {
    const int i = (int)(q % g.n1), j = (int)(q / g.n1);
    const double R = g.left1 + i * g.dr1, r = g.left2 + j * g.dr2;
    const double I = 1.0 / (2 * g.m1 * R * R) + 1.0 / (2 * g.m2 * r * r);
    const double2 v = p[q];
    acc += ll * I * (v.x * v.x + v.y * v.y);
  }
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) part[(int64_t)sl * NOALLOC_TILES + blockIdx.x] = acc;
}

// One CTA: fixed-order sum of the partials, scaled by dr1 dr2.
__global__ void k_rot_energy_sum(const double *__restrict__ part, int n, double scale, double *__restrict__ out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int q = threadIdx.x; q < n; q += blockDim.x) s += part[q];
  s = block_sum(s, red);
  if (threadIdx.x == 0) *out = s * scale;
}

}  // namespace qd

extern "C" int qd_rotational_energy_noalloc(const double *psi_j, int32_t n1, int32_t n2, int32_t omega, int32_t l_max,
                                            double r1_left, double r1_dr, double r1_mass, double r2_left, double r2_dr,
                                            double r2_mass, double *rotational_energy, void *stream) {
  using namespace qd;
  try {
    set_error("");
    QD_REQUIRE(psi_j && rotational_energy, "psi_j && rotational_energy");
    QD_REQUIRE(n1 > 0 && n2 > 0 && omega >= 0 && l_max >= omega, "n1, n2 > 0 and 0 <= omega <= l_max");
    QD_REQUIRE(r1_dr > 0 && r2_dr > 0 && r1_mass > 0 && r2_mass > 0 && r1_left > 0 && r2_left > 0,
               "positive radial grids and masses");
    const int n_slabs = l_max - omega + 1;
    if ((int64_t)n_slabs * NOALLOC_TILES > QD_NOALLOC_MAX_PARTIALS)
      throw Error{QD_ERR_INVALID, "qd_rotational_energy_noalloc: l_max - omega + 1 = " + std::to_string(n_slabs) +
                                      " slabs exceed the fixed scratch of " +
                                      std::to_string(QD_NOALLOC_MAX_PARTIALS / NOALLOC_TILES) + " slabs"};
    double *scratch = scratch_for_current_device();
    Grid g{};
    g.n1 = n1;
    g.n2 = n2;
    g.npt = (int64_t)n1 * n2;
    g.left1 = r1_left;
    g.dr1 = r1_dr;
    g.m1 = r1_mass;
    g.left2 = r2_left;
    g.dr2 = r2_dr;
    g.m2 = r2_mass;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // every partial slot that the sum reads is written by this call first.  The
    // launches report through their own return codes, so an error left pending by
    // the caller's earlier work is neither cleared nor reported as this call's.
    const double2 *psi = reinterpret_cast<const double2 *>(psi_j);
    void *block_args[] = {&g, &psi, &omega, &scratch};
    cudaError_t e = cudaLaunchKernel(reinterpret_cast<const void *>(&k_rot_energy_block),
                                     dim3(NOALLOC_TILES, n_slabs), dim3(NOALLOC_THREADS), block_args, 0, st);
    if (e != cudaSuccess) throw Error{QD_ERR_CUDA, std::string("rotational-energy partials: ") + cudaGetErrorString(e)};
    int n_part = n_slabs * NOALLOC_TILES;
    double scale = r1_dr * r2_dr;
    const double *part = scratch;
    void *sum_args[] = {&part, &n_part, &scale, &rotational_energy};
    e = cudaLaunchKernel(reinterpret_cast<const void *>(&k_rot_energy_sum), dim3(1), dim3(NOALLOC_THREADS), sum_args,
                         0, st);
    if (e != cudaSuccess) throw Error{QD_ERR_CUDA, std::string("rotational-energy sum: ") + cudaGetErrorString(e)};
    return QD_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.status;
  }
}
