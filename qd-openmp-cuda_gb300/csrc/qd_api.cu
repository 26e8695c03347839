// C ABI and host engine of the GB300 split-operator propagator.
//
// Reference entry: mexFunction (cudaOpenMPEvolution.C:15-79) -> CudaOpenMPQMMD
// (cudaOpenMP2.cu:23-127) -> test_multiple_cards (cudaOpenMP2.cu:328-390).
// The multi-GPU orchestration (OpenMP threads per device, P2P Coriolis
// exchange) is replaced by one session on one device holding every Omega block
// of every problem resident in HBM; each stage is one launch over all blocks,
// and steps are replayed from CUDA graphs.
#include "qd_internal.h"
#include "qd_device.cuh"
#include "qd_tail.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <sstream>
#include <string>
#include <vector>

namespace qd {

static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }

struct Profiler {
  cudaEvent_t start = nullptr;
  std::vector<cudaEvent_t> ev;
  std::vector<std::string> names;
};
static thread_local Profiler *g_prof = nullptr;

void prof_mark(cudaStream_t s, const char *name) {
  if (!g_prof) return;
  cudaEvent_t e;
  QD_CUDA(cudaEventCreate(&e));
  QD_CUDA(cudaEventRecord(e, s));
  g_prof->ev.push_back(e);
  g_prof->names.push_back(name);
}

// ------------------------------------------------------- Coriolis matrices
// Tridiagonal Omega matrix of setup_coriolis_matrix (CoriolisMatrix.C:63-99):
// diagonal J(J+1) - 2 Omega^2, off-diagonal -lambda(J,Omega) lambda(l,Omega)
// sqrt(1 + delta_{Omega,0}), lambda(J,Omega) = sqrt(J(J+1) - Omega(Omega+1))
// for J >= Omega (CoriolisMatrix.C:23-33).
static double lam(int J, int omega) {
  return J >= omega ? std::sqrt(J * (J + 1.0) - omega * (omega + 1.0)) : 0.0;
}

// Cyclic Jacobi diagonalisation of a small symmetric matrix (row-major a[n*n]).
// Returns eigenvalues ascending in e and eigenvectors as columns of v
// (v[p*n + a] = component p of vector a), the layout dstev writes.
static void jacobi_eigen(int n, std::vector<double> a, std::vector<double> &e, std::vector<double> &v) {
  v.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) v[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, diag = 0.0;
    for (int p = 0; p < n; p++)
      for (int q = 0; q < n; q++) (p == q ? diag : off) += a[(size_t)p * n + q] * a[(size_t)p * n + q];
    if (off <= 1e-32 * std::max(diag, 1e-300)) break;
    for (int p = 0; p < n - 1; p++)
      for (int q = p + 1; q < n; q++) {
        const double apq = a[(size_t)p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double app = a[(size_t)p * n + p], aqq = a[(size_t)q * n + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; k++) {   // A <- A J (columns p, q)
          const double akp = a[(size_t)k * n + p], akq = a[(size_t)k * n + q];
          a[(size_t)k * n + p] = c * akp - s * akq;
          a[(size_t)k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; k++) {   // A <- J^T A (rows p, q)
          const double apk = a[(size_t)p * n + k], aqk = a[(size_t)q * n + k];
          a[(size_t)p * n + k] = c * apk - s * aqk;
          a[(size_t)q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; k++) {   // V <- V J
          const double vkp = v[(size_t)k * n + p], vkq = v[(size_t)k * n + q];
          v[(size_t)k * n + p] = c * vkp - s * vkq;
          v[(size_t)k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  e.resize(n);
  for (int i = 0; i < n; i++) e[i] = a[(size_t)i * n + i];
  std::vector<int> idx(n);
  for (int i = 0; i < n; i++) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int x, int y) { return e[x] < e[y]; });
  std::vector<double> e2(n), v2((size_t)n * n);
  for (int k = 0; k < n; k++) {
    e2[k] = e[idx[k]];
    for (int p = 0; p < n; p++) v2[(size_t)p * n + k] = v[(size_t)p * n + idx[k]];
  }
  e.swap(e2);
  v.swap(v2);
}

// ------------------------------------------------------------- validation
struct ProblemHost {
  qd_fh2data *d;
  int J, parity, l_max, n_omegas, omega_min, omega_cap;
  bool coupled;
  std::vector<int> omegas;
};

static void validate_problem(qd_fh2data *d, ProblemHost &ph) {
  QD_REQUIRE(d != nullptr, "FH2Data != NULL");
  QD_REQUIRE(d->r1.n > 0 && d->r2.n > 0 && d->theta.n > 0, "grid sizes > 0");
  QD_REQUIRE(d->r1.dr > 0 && d->r2.dr > 0, "r1.dr > 0 && r2.dr > 0");
  QD_REQUIRE(d->r1.mass > 0 && d->r2.mass > 0, "masses > 0");
  QD_REQUIRE(d->r1.left > 0 && d->r2.left > 0, "radial grids start above 0 (1/R^2 terms)");
  QD_REQUIRE(d->theta.x && d->theta.w, "theta.x && theta.w");
  QD_REQUIRE(d->pot, "pot");
  QD_REQUIRE(d->time.total_steps >= 0, "time.total_steps >= 0");
  QD_REQUIRE(std::isfinite(d->time.time_step), "time.time_step finite");
  QD_REQUIRE(d->time.steps >= 0, "time.steps >= 0");
  if (d->r1.n % 2 || d->r2.n % 2)
    throw Error{QD_ERR_UNSUPPORTED, "r1.n and r2.n must be even (FFT kinetic table, cudaMath.h:117-130)"};
  const qd_omega_states &om = d->OmegaStates;
  QD_REQUIRE(om.J >= 0, "OmegaStates.J >= 0");
  if (om.J == 0) QD_REQUIRE(om.parity == 0, "p == 0 when J == 0 (CoriolisMatrix.C:52)");
  QD_REQUIRE(om.l_max >= 0, "l_max >= 0");
  QD_REQUIRE(om.n_omegas >= 1 && om.omegas, "omegas");
  QD_REQUIRE(om.n_omegas_max >= om.n_omegas, "n_omegas_max >= omegas.size() (matlabStructures.C:128)");
  QD_REQUIRE(d->theta.n >= om.l_max + 1, "theta.n >= l_max + 1 (Gauss-Legendre exactness)");
  QD_REQUIRE(om.associated_legendres && om.wave_packets, "associated_legendres && wave_packets");
  const int omega_min = om.J == 0 ? 0 : ((om.J + om.parity) % 2 == 0 ? 0 : 1);
  QD_REQUIRE(om.omegas[0] == omega_min, "omegas[0] == (J+p)%2 (OmegaList.m)");
  for (int i = 1; i < om.n_omegas; i++) QD_REQUIRE(om.omegas[i] == om.omegas[i - 1] + 1, "consecutive omegas");
  const int omega_last = om.omegas[om.n_omegas - 1];
  QD_REQUIRE(omega_last <= std::min(om.J, om.l_max), "omega <= min(J, l_max)");
  QD_REQUIRE(om.n_cols >= om.l_max - omega_min + 1, "associated_legendres columns >= l_max - omega_min + 1");
  const qd_crp &c = d->CRP;
  if (c.calculate_CRP) {
    QD_REQUIRE(c.energies && c.eta_sq && c.CRP, "CRP.energies && CRP.eta_sq && CRP.CRP");
    QD_REQUIRE(c.n_energies > 0, "CRP.n_energies > 0");
    QD_REQUIRE(c.n_gradient_points >= 3 && c.n_gradient_points % 2 == 1, "CRP.n_gradient_points odd >= 3");
    const int h = (c.n_gradient_points - 1) / 2;
    QD_REQUIRE(c.n_dividing_surface - h >= 0 && c.n_dividing_surface + h < d->r2.n,
               "flux stencil inside the r2 grid");
    for (int e = 0; e < c.n_energies; e++) QD_REQUIRE(c.eta_sq[e] > 0, "CRP.eta_sq > 0");
  }
  if (d->options.wave_to_matlab)
    QD_REQUIRE(d->options.steps_to_copy_psi_from_device_to_host > 0, "steps_to_copy_psi_from_device_to_host > 0");
  QD_REQUIRE(d->options.precision == QD_PRECISION_FP64 || d->options.precision == QD_PRECISION_MIXED,
             "options.precision in {0, 1}");
  ph.d = d;
  ph.J = om.J;
  ph.parity = om.parity;
  ph.l_max = om.l_max;
  ph.n_omegas = om.n_omegas;
  ph.omega_min = omega_min;
  ph.omegas.assign(om.omegas, om.omegas + om.n_omegas);
  ph.omega_cap = omega_last;
  ph.coupled = om.J > 0;
}

static void validate_batch(qd_fh2data *const *pr, int n, std::vector<ProblemHost> &out) {
  QD_REQUIRE(pr != nullptr && n >= 1, "n_problems >= 1");
  out.resize(n);
  for (int i = 0; i < n; i++) validate_problem(pr[i], out[i]);
  const qd_fh2data *a = pr[0];
  for (int i = 1; i < n; i++) {
    const qd_fh2data *b = pr[i];
    QD_REQUIRE(a->r1.n == b->r1.n && a->r2.n == b->r2.n && a->theta.n == b->theta.n, "batch: same grids");
    QD_REQUIRE(a->r1.left == b->r1.left && a->r1.dr == b->r1.dr && a->r1.mass == b->r1.mass, "batch: same r1");
    QD_REQUIRE(a->r2.left == b->r2.left && a->r2.dr == b->r2.dr && a->r2.mass == b->r2.mass, "batch: same r2");
    QD_REQUIRE(a->OmegaStates.l_max == b->OmegaStates.l_max, "batch: same l_max");
    QD_REQUIRE(a->time.time_step == b->time.time_step && a->time.steps == b->time.steps &&
                   a->time.total_steps == b->time.total_steps,
               "batch: same time");
    QD_REQUIRE(a->options.precision == b->options.precision, "batch: same precision");
    QD_REQUIRE(a->CRP.calculate_CRP == b->CRP.calculate_CRP, "batch: same CRP switch");
    const size_t npot = (size_t)a->r1.n * a->r2.n * a->theta.n;
    QD_REQUIRE(a->pot == b->pot || std::memcmp(a->pot, b->pot, npot * sizeof(double)) == 0, "batch: same pot");
    QD_REQUIRE((a->dump1.dump == nullptr) == (b->dump1.dump == nullptr) &&
                   (a->dump2.dump == nullptr) == (b->dump2.dump == nullptr),
               "batch: same masks");
    if (a->CRP.calculate_CRP) {
      QD_REQUIRE(a->CRP.n_energies == b->CRP.n_energies && a->CRP.n_dividing_surface == b->CRP.n_dividing_surface &&
                     a->CRP.n_gradient_points == b->CRP.n_gradient_points,
                 "batch: same CRP shape");
      QD_REQUIRE(std::memcmp(a->CRP.energies, b->CRP.energies, a->CRP.n_energies * sizeof(double)) == 0,
                 "batch: same CRP energies");
    }
  }
}

// first-derivative weights of the centred n-point stencil (Fornberg 1988)
static std::vector<double> fd_weights(int n) {
  const int h = (n - 1) / 2;
  std::vector<double> x(n);
  for (int i = 0; i < n; i++) x[i] = i - h;
  std::vector<std::vector<double>> c(n, std::vector<double>(2, 0.0));
  double c1 = 1.0, c4 = x[0];
  c[0][0] = 1.0;
  for (int i = 1; i < n; i++) {
    const int mn = std::min(i, 1);
    double c2 = 1.0;
    const double c5 = c4;
    c4 = x[i];
    for (int j = 0; j < i; j++) {
      const double c3 = x[i] - x[j];
      c2 *= c3;
      if (j == i - 1) {
        for (int k = mn; k > 0; k--) c[i][k] = c1 * (k * c[i - 1][k - 1] - c5 * c[i - 1][k]) / c2;
        c[i][0] = -c1 * c5 * c[i - 1][0] / c2;
      }
      for (int k = mn; k > 0; k--) c[j][k] = (c4 * c[j][k] - k * c[j][k - 1]) / c3;
      c[j][0] = c4 * c[j][0] / c3;
    }
    c1 = c2;
  }
  std::vector<double> w(n);
  for (int i = 0; i < n; i++) w[i] = c[i][1];
  return w;
}

// Device memory of one session: a few cudaMalloc chunks of growing size (16 MiB
// doubling, or the request when larger), sub-allocated 256-byte aligned and
// released together.  A session makes about 60 buffers; this keeps the
// allocation (and the device synchronisation of cudaFree) to a handful of calls.
struct Arena {
  std::vector<void *> chunks;
  char *cur = nullptr;
  size_t left = 0, next = (size_t)16 << 20, total = 0;
  void *take(size_t bytes) {
    bytes = (bytes + 255) & ~(size_t)255;
    if (bytes > left) {
      const size_t chunk = std::max(bytes, next);
      next = std::min(next * 2, (size_t)1 << 30);
      void *p = nullptr;
      QD_CUDA(cudaMalloc(&p, chunk));
      chunks.push_back(p);
      cur = static_cast<char *>(p);
      left = chunk;
      total += chunk;
    }
    void *r = cur;
    cur += bytes;
    left -= bytes;
    return r;
  }
  ~Arena() {
    for (void *p : chunks) cudaFree(p);
  }
};

template <typename T> static T *dalloc(size_t n) {
  T *p = nullptr;
  if (n == 0) return nullptr;
  QD_CUDA(cudaMalloc(&p, n * sizeof(T)));
  return p;
}
template <typename T> static T *dupload(const T *h, size_t n, cudaStream_t s) {
  T *p = dalloc<T>(n);
  if (n) QD_CUDA(cudaMemcpyAsync(p, h, n * sizeof(T), cudaMemcpyHostToDevice, s));
  return p;
}

__global__ void k_step_end(int *step, const int *status, int *flux_count, double *flux_t0, double dt,
                           int flux_on);
__global__ void k_flux_begin(const int *step, int *flux_count, double *flux_t0, double dt, int *slot_out, int cap,
                             int *status);

}  // namespace qd

using namespace qd;

// ------------------------------------------------------------------ session
struct qd_session {
  qd::Arena arena;   // every device buffer of the session (released last)
  int device = 0;
  cudaStream_t stream = nullptr;
  Grid g{};
  int precision = 0;
  double dt = 0.0;
  double norm_tol = 1e-10;
  int n_problems = 0, n_blocks = 0, n_slabs = 0, max_nl = 0;
  bool any_coupled = false, has_mask = false;
  std::vector<ProblemHost> probs;
  std::vector<BlockDesc> h_blocks;
  std::vector<SlabDesc> h_slabs;
  std::vector<int> h_pblock0;
  BlockDesc *d_blocks = nullptr;
  SlabDesc *d_slabs = nullptr;
  int *d_pblock0 = nullptr;
  // coupled / uncoupled slab lists (epilogue tables differ)
  double2 *psi_th = nullptr, *psi_j = nullptr;   // FP64 form: both pools in c128
  // mixed form: both pools in c64 (every value the mixed step writes is an
  // FP32 number); host transfers widen/narrow through xfer (c128)
  float2 *psi_thf = nullptr, *psi_jf = nullptr;
  double2 *xfer = nullptr;
  int64_t xfer_elems = 0;
  double *pot = nullptr, *w = nullptr, *T1 = nullptr, *T2 = nullptr, *I1 = nullptr, *I2 = nullptr;
  double *d1 = nullptr, *d2 = nullptr;
  double2 *tab_v = nullptr, *tab_v0 = nullptr, *tab_rot2 = nullptr, *tab_rot4 = nullptr, *tab_kin = nullptr;
  double *Bf = nullptr, *Bb = nullptr;
  // Coriolis
  std::vector<CoriolisGroup> h_groups;
  CoriolisGroup *d_groups = nullptr;
  int n_groups = 0, max_group_n = 1;
  double *cor_V = nullptr, *cor_e = nullptr, *cor_H = nullptr;
  double2 *cor_ph = nullptr;
  // mixed form with at most CORIOLIS_F32_MAXN coupled blocks: FP32 Coriolis
  bool cor_f32 = false;
  float *cor_Vh = nullptr, *cor_Vl = nullptr;
  float2 *cor_phl = nullptr;
  int *cor_order = nullptr;   // group indices, largest groups first
  std::vector<int> h_pgroup0;
  int *d_pgroup0 = nullptr;
  // energies
  double *part_modpe = nullptr, *part_ke = nullptr, *part_re = nullptr, *part_ce = nullptr;
  int t_modpe = 0, t_ke = 0, t_re = 0, t_ce = 0;
  double *energies = nullptr;     // [n_blocks][6]
  double *rec = nullptr;          // [rec_cap][n_blocks][6]
  int rec_cap = 0, rec_base = 0;
  int *status = nullptr, *status_step = nullptr, *d_step = nullptr;
  // flux
  FluxConfig flux{};
  double2 *flux_buf = nullptr, *flux_acc = nullptr, *flux_phase = nullptr, *half_v = nullptr;
  float2 *flux_buf_f = nullptr;   // mixed form: surface buffer in c64 (FP32 values)
  double *fd = nullptr, *flux_E = nullptr, *flux_eta = nullptr, *crp = nullptr, *flux_t0 = nullptr;
  int *flux_count = nullptr, *flux_slot = nullptr;
  int *flux_fresh = nullptr;   // nonzero: the accumulators hold no transform of this call yet
  unsigned *step_done = nullptr;
  float2 *half_v_lift = nullptr;
  float *fdf = nullptr;
  int flux_pending = 0;
  FFTPlan fft{};
  // mixed form: tensor-core Legendre images and FP32 three-shear tables
  uint16_t *img_f = nullptr, *img_b = nullptr;
  float *bscale_f = nullptr, *bscale_b = nullptr;
  int64_t *imgoff_f = nullptr, *imgoff_b = nullptr;
  size_t smem_f = 0, smem_b = 0;
  float2 *vph = nullptr, *vph0 = nullptr, *lrotR = nullptr, *lrotr = nullptr, *lkinR = nullptr, *lkinr = nullptr;
  float *wf = nullptr, *wvf = nullptr, *d1f = nullptr, *d2f = nullptr, *T1f = nullptr, *T2f = nullptr;
  float *I1f = nullptr, *I2f = nullptr;
  int steps = 0;   // host mirror of time.steps
  int launches_per_step = 0;
  // end of a call: the download stream (psi beside the flux transform), the event that
  // ends the steps (also: the potential comparison at the start), and the status words and
  // the comparison flag read back through pinned memory
  cudaStream_t stream_dl = nullptr;
  cudaEvent_t ev_steps = nullptr;
  int *h_status = nullptr;   // [status, status step, potential differs]
  cudaGraphExec_t graph_chunk = nullptr;
  int graph_steps = 0;
  // reuse across qd_evolve calls of the same shape: the key, host copies of the
  // small inputs the tables were built from, a staging buffer and a flag for the
  // on-device comparison of the potential
  std::vector<double> key;
  std::vector<double> h_w, h_d1, h_d2, h_Bf, h_Bb;
  double *pot_stage = nullptr;
  int *d_flag = nullptr;
  double *rec_buf = nullptr;
  size_t rec_buf_cap = 0;
  std::string tuning;   // what the autotuner chose (qd_session_tuning)
  // energy-record arguments the step graph was captured with
  double *graph_rec = nullptr;
  int graph_rec_base = 0, graph_rec_cap = 0;
  // graphs of 2^k steps (k = 1..5) without a flux transform, for runs shorter than a chunk;
  // built together, with the energy-record arguments they were captured with
  static constexpr int N_POW_GRAPHS = 5;
  cudaGraphExec_t graph_pow[N_POW_GRAPHS + 1] = {};
  double *pow_rec = nullptr;
  int pow_rec_base = 0, pow_rec_cap = 0;

  template <typename T> T *alloc(size_t n) { return n ? static_cast<T *>(arena.take(n * sizeof(T))) : nullptr; }
  template <typename T> T *upload(const T *h, size_t n) {
    T *p = alloc<T>(n);
    if (n) QD_CUDA(cudaMemcpyAsync(p, h, n * sizeof(T), cudaMemcpyHostToDevice, stream));
    return p;
  }

  ~qd_session();
};

namespace qd {

__global__ void k_step_end(int *step, const int *status, int *, double *, double, int) {
  if (*status) return;
  *step += 1;
}

// sets the flux slot for this step; records t0 when the chunk starts.  A full
// buffer (which the host scheduling never produces) stops the run with an
// error status instead of writing past the buffer.
__global__ void k_flux_begin(const int *step, int *flux_count, double *flux_t0, double dt, int *slot_out, int cap,
                             int *status) {
  const int c = *flux_count;
  if (c >= cap) {
    atomicCAS(status, 0, QD_ERR_INVALID);
    *slot_out = 0;
    return;
  }
  if (c == 0) *flux_t0 = (*step + 1) * dt;
  *slot_out = c;
  *flux_count = c + 1;
}

// flux extract with a device-side slot
template <typename S>
__global__ void k_flux_extract_dev(Grid g, int n_grad, int n_ds, const S *__restrict__ psi_th,
                                   const double2 *__restrict__ hv, const double *__restrict__ fd,
                                   double2 *__restrict__ buf, int n_blocks, const int *slot_p, const int *status) {
  if (status && *status) return;
  const int slot = *slot_p;
  const int b = blockIdx.y;
  const int h = (n_grad - 1) / 2;
  const int64_t ns = (int64_t)g.nth * g.n1;
  double2 *out = buf + ((int64_t)slot * n_blocks + b) * 2 * ns;
  const S *p = psi_th + (int64_t)b * g.nth * g.npt;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < ns; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % g.n1), k = (int)(q / g.n1);
    double2 A = make_double2(0.0, 0.0), D = make_double2(0.0, 0.0);
    constexpr int GB = 8;   // stencil rows loaded together
    for (int g0 = 0; g0 < n_grad; g0 += GB) {
      double2 av[GB], mv[GB];
#pragma unroll
      for (int u = 0; u < GB; u++)
        if (g0 + u < n_grad) {
          av[u] = load_c(p + ((int64_t)k * g.n2 + (n_ds - h + g0 + u)) * g.n1 + i);
          mv[u] = hv[((int64_t)k * n_grad + g0 + u) * g.n1 + i];
        }
#pragma unroll
      for (int u = 0; u < GB; u++)
        if (g0 + u < n_grad) {
          const double2 a = av[u], m = mv[u];
          const double2 v = make_double2(a.x * m.x - a.y * m.y, a.x * m.y + a.y * m.x);
          const double c = fd[g0 + u];
          D.x = fma(c, v.x, D.x);
          D.y = fma(c, v.y, D.y);
          if (g0 + u == h) A = v;
        }
    }
    out[q] = A;
    out[ns + q] = D;
  }
}

// phase[n][E] = dt exp(i E (t0 + n dt)) for n < count (device count and t0)
__global__ void k_flux_phase_dev(const double *__restrict__ E, int nE, int cap, const int *count_p,
                                 const double *t0_p, double dt, double2 *__restrict__ phase) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nE * cap) return;
  const int n = q / nE, e = q % nE;
  if (n >= *count_p) return;
  double s, c;
  sincos(E[e] * (*t0_p + n * dt), &s, &c);
  phase[q] = make_double2(dt * c, dt * s);
}

// after a transform: the buffer is empty, and the accumulators hold a sum (when it ran)
__global__ void k_flux_reset(int *count, int *fresh, const int *status) {
  if (*count > 0 && !*status) *fresh = 0;
  *count = 0;
}

}  // namespace qd

qd_session::~qd_session() {
  if (graph_chunk) cudaGraphExecDestroy(graph_chunk);
  for (cudaGraphExec_t &e : graph_pow)
    if (e) cudaGraphExecDestroy(e);
  fft_plan_free(fft);
  if (stream) {
    cudaStreamSynchronize(stream);
    cudaStreamDestroy(stream);
  }
  if (stream_dl) {
    cudaStreamSynchronize(stream_dl);
    cudaStreamDestroy(stream_dl);
  }
  if (ev_steps) cudaEventDestroy(ev_steps);
  if (h_status) cudaFreeHost(h_status);
  // the arena's chunks are released by its destructor
}

namespace qd {

// flux DFT reading count/t0 from the device (graph friendly)
__global__ void k_flux_dft_dev(int64_t ns2, int nE, int n_blocks, const int *count_p, int cap,
                               const double2 *__restrict__ buf, const double2 *__restrict__ phase,
                               double2 *__restrict__ acc, const int *status, const int *fresh);

static void enqueue_flux_dft(qd_session *s) {
  const int nE = s->flux.n_energies;
  const int cap = s->flux.chunk;
  k_flux_phase_dev<<<(nE * cap + 255) / 256, 256, 0, s->stream>>>(s->flux_E, nE, cap, s->flux_count, s->flux_t0,
                                                                   s->dt, s->flux_phase);
  prof_mark(s->stream, "flux_phase");
  const int64_t ns2 = 2LL * s->g.nth * s->g.n1;
  if (s->precision == QD_PRECISION_MIXED) {
    launch_flux_dft_f32(s->stream, ns2, nE, s->n_blocks, s->flux_count, cap, s->flux_buf_f, s->flux_phase,
                        s->flux_acc, s->status, s->flux_fresh);
  } else {
    dim3 grid((unsigned)((ns2 + 127) / 128), (unsigned)((nE + 7) / 8), (unsigned)s->n_blocks);
    k_flux_dft_dev<<<grid, 128, 0, s->stream>>>(ns2, nE, s->n_blocks, s->flux_count, cap, s->flux_buf,
                                                 s->flux_phase, s->flux_acc, s->status, s->flux_fresh);
  }
  prof_mark(s->stream, "flux_dft");
  k_flux_reset<<<1, 1, 0, s->stream>>>(s->flux_count, s->flux_fresh, s->status);
  prof_mark(s->stream, "flux_reset");
}

static EnergyParts energy_parts(qd_session *s, bool mod, bool ke, bool re, bool ce) {
  EnergyParts ep{};
  ep.mod_pe = s->part_modpe;
  ep.mod_pe_tiles = s->t_modpe;
  ep.ke = s->part_ke;
  ep.ke_tiles = s->t_ke;
  ep.re = s->part_re;
  ep.re_tiles = s->t_re;
  ep.ce = s->part_ce;
  ep.ce_tiles = s->t_ce;
  ep.have_mod = mod;
  ep.have_ke = ke;
  ep.have_re = re;
  ep.have_ce = ce;
  ep.ke_scale = s->g.dr1 * s->g.dr2 / ((double)s->g.n1 * s->g.n2);
  return ep;
}

static void enqueue_tail(qd_session *s);

// Mixed form of the same step on the c64 pools: tensor-core Legendre
// contractions, the separable FP32 slab FFT, FP32 Coriolis (FP64-exact
// operator) and FP32 three-shear phases; energies and flux accumulate in FP64.
static void enqueue_step_mixed(qd_session *s, bool first) {
  cudaStream_t st = s->stream;
  const Grid &g = s->g;
  launch_legendre_tc_fwd(st, g, s->psi_thf, s->psi_jf, s->d_blocks, s->n_blocks, s->img_f, s->imgoff_f,
                         first ? s->vph0 : s->vph, s->d1f, s->d2f, s->smem_f, s->status, s->status, s->bscale_f, s->max_nl);
  prof_mark(st, "legendre_forward");
  if (s->cor_f32) {
    launch_coriolis_f32(st, g, s->psi_jf, s->d_blocks, s->d_groups, s->cor_order, s->n_groups,
                        s->max_group_n, s->cor_Vh,
                        s->cor_Vl, s->cor_phl, s->cor_H, s->lrotR, s->lrotr, true, true, s->I1f, s->I2f, nullptr,
                        nullptr, s->t_ce, s->status);
    prof_mark(st, "coriolis");
  } else if (s->any_coupled) {
    launch_coriolis(st, g, s->psi_jf, s->d_blocks, s->d_groups, s->n_groups, s->max_group_n, s->cor_V, s->cor_ph,
                    s->cor_H, nullptr, s->t_ce, s->tab_rot4, s->status, s->tab_rot4);
    prof_mark(st, "coriolis");
  }
  FFTLift lf{};
  lf.proR = s->any_coupled ? nullptr : s->lrotR;
  lf.pror = s->any_coupled ? nullptr : s->lrotr;
  lf.epiR = s->lrotR;
  lf.epir = s->lrotr;
  lf.kinR = s->lkinR;
  lf.kinr = s->lkinr;
  lf.T1f = s->T1f;
  lf.T2f = s->T2f;
  lf.I1f = s->I1f;
  lf.I2f = s->I2f;
  launch_fft_kinetic(st, g, s->fft, s->psi_jf, s->d_slabs, s->n_slabs, s->part_ke,
                     s->any_coupled ? nullptr : s->part_re, s->status, &lf);
  if (s->cor_f32) {
    // coupling energy of the incoming state, rotational energy of the outgoing one
    launch_coriolis_f32(st, g, s->psi_jf, s->d_blocks, s->d_groups, s->cor_order, s->n_groups,
                        s->max_group_n, s->cor_Vh,
                        s->cor_Vl, s->cor_phl, s->cor_H, s->lrotR, s->lrotr, false, true, s->I1f, s->I2f,
                        s->part_ce, s->part_re, s->t_ce, s->status);
    prof_mark(st, "coriolis_energy");
  } else if (s->any_coupled) {
    launch_coriolis(st, g, s->psi_jf, s->d_blocks, s->d_groups, s->n_groups, s->max_group_n, s->cor_V, s->cor_ph,
                    s->cor_H, s->part_ce, s->t_ce, s->tab_rot4, s->status);
    prof_mark(st, "coriolis_energy");
    launch_rot_energy(st, g, s->psi_jf, s->d_slabs, s->n_slabs, s->part_re, s->t_re, s->status);
    prof_mark(st, "rotational_energy");
  }
  launch_legendre_tc_bwd(st, g, s->psi_jf, s->psi_thf, s->d_blocks, s->n_blocks, s->img_b, s->imgoff_b, s->wf, s->wvf,
                         s->part_modpe, s->t_modpe, s->smem_b, s->status, s->status, s->bscale_b, s->max_nl);
  prof_mark(st, "legendre_backward");
  enqueue_tail(s);
}

// One full time step, sequence of test_multiple_cards (cudaOpenMP2.cu:338-386).
static void enqueue_step(qd_session *s, bool first) {
  if (s->precision == QD_PRECISION_MIXED) {
    enqueue_step_mixed(s, first);
    return;
  }
  cudaStream_t st = s->stream;
  const Grid &g = s->g;
  const double2 *tabA = first ? s->tab_v0 : s->tab_v;
  // dump_wavepacket + evolution_with_potential(-dt/2 at step 0) + potential(dt) -> prologue,
  // forward_legendre_transform, rotational(dt/4) [x2 fused when uncoupled] -> epilogue
  launch_legendre_fwd_f64(st, g, s->psi_th, s->psi_j, s->Bf, s->d_blocks, s->n_blocks, s->max_nl, tabA,
                          s->any_coupled ? s->tab_rot4 : s->tab_rot2, s->status);
  prof_mark(st, "legendre_forward");
  if (s->any_coupled) {
    // evolution_with_coriolis(dt/2) + rotational(dt/4)
    launch_coriolis(st, g, s->psi_j, s->d_blocks, s->d_groups, s->n_groups, s->max_group_n, s->cor_V, s->cor_ph,
                    s->cor_H, nullptr, s->t_ce, s->tab_rot4, s->status);
    prof_mark(st, "coriolis");
  }
  // forward FFT, kinetic(dt), kinetic energy, backward FFT + scale, rotational(dt/4)
  launch_fft_kinetic(st, g, s->fft, s->psi_j, s->d_slabs, s->n_slabs, s->tab_kin, s->T1, s->T2, s->part_ke,
                     s->any_coupled ? s->tab_rot4 : s->tab_rot2, s->any_coupled ? nullptr : s->part_re, s->status);
  if (s->any_coupled) {
    // evolution_with_coriolis(dt/2, energy) + rotational(dt/4), then the rotational energy
    launch_coriolis(st, g, s->psi_j, s->d_blocks, s->d_groups, s->n_groups, s->max_group_n, s->cor_V, s->cor_ph,
                    s->cor_H, s->part_ce, s->t_ce, s->tab_rot4, s->status);
    prof_mark(st, "coriolis_energy");
    launch_rot_energy(st, g, s->psi_j, s->d_slabs, s->n_slabs, s->part_re, s->t_re, s->status);
    prof_mark(st, "rotational_energy");
  }
  // backward_legendre_transform + potential energy + module
  launch_legendre_bwd_f64(st, g, s->psi_j, s->psi_th, s->Bb, s->d_blocks, s->n_blocks, nullptr, s->w, s->pot,
                          s->part_modpe, s->t_modpe, s->status);
  prof_mark(st, "legendre_backward");
  enqueue_tail(s);
}

// energies, norm guard, flux surface values, step counter
static void enqueue_tail(qd_session *s) {
  cudaStream_t st = s->stream;
  const Grid &g = s->g;
  EnergyParts ep = energy_parts(s, true, true, true, s->any_coupled);
  StepTail tail{};
  tail.done = s->step_done;
  if (s->flux.enabled) {
    tail.flux_count = s->flux_count;
    tail.flux_slot = s->flux_slot;
    tail.flux_t0 = s->flux_t0;
    tail.cap = s->flux.chunk;
    tail.dt = s->dt;
  }
  if (s->flux.enabled && s->precision == QD_PRECISION_MIXED) {
    // mixed form: surface extraction and energy finalisation in one launch
    const FluxTileArgs fx = flux_tile_args(g, s->flux, s->psi_thf, s->half_v_lift, s->fdf, s->flux_buf_f, s->n_blocks);
    launch_energy_finalize2(st, g, ep, s->d_blocks, s->d_pblock0, s->n_problems, s->d_groups, s->d_pgroup0,
                            s->max_group_n, s->energies, s->rec, s->d_step, s->rec_base, s->rec_cap, s->norm_tol,
                            s->status, s->status_step, s->n_blocks, s->step_done, &tail, &fx);
    prof_mark(st, "step_tail");
    return;
  }
  launch_energy_finalize2(st, g, ep, s->d_blocks, s->d_pblock0, s->n_problems, s->d_groups, s->d_pgroup0,
                          s->max_group_n, s->energies, s->rec, s->d_step, s->rec_base, s->rec_cap, s->norm_tol,
                          s->status, s->status_step, s->n_blocks, s->step_done, &tail);
  prof_mark(st, "energy_finalize");
  if (s->flux.enabled) {
    const int64_t ns = (int64_t)g.nth * g.n1;
    dim3 grid((unsigned)((ns + 127) / 128), (unsigned)s->n_blocks);
    k_flux_extract_dev<<<grid, 128, 0, st>>>(g, s->flux.n_grad, s->flux.n_ds, s->psi_th, s->half_v, s->fd,
                                             s->flux_buf, s->n_blocks, s->flux_slot, s->status);
    prof_mark(st, "flux_extract");
  }
}

static int count_launches_per_step(qd_session *s) {
  const int fft = s->precision == QD_PRECISION_MIXED ? fft_mixed_launches(s->fft) : 3;
  int n = 1 + fft + 1 + 1;   // fwd, fft, bwd, end of step (energies, norm guard, step counter)
  if (s->cor_f32) n += 2;              // coriolis x2 (rotational energy fused)
  else if (s->any_coupled) n += 3;     // coriolis x2, rot energy
  if (s->flux.enabled && s->precision != QD_PRECISION_MIXED) n += 1;   // surface extraction (fused in the mixed form)
  return n;
}

}  // namespace qd

// theta-space pool <-> host memory in c128.  The FP64 form copies directly;
// the mixed form narrows (round to nearest) or widens (exact) through the
// c128 staging buffer, chunk by chunk in stream order.
static void theta_from_host(qd_session *s, int64_t off, int64_t n, const double *host) {
  cudaStream_t st = s->stream;
  if (!s->psi_thf) {
    QD_CUDA(cudaMemcpyAsync(s->psi_th + off, host, n * sizeof(double2), cudaMemcpyHostToDevice, st));
    return;
  }
  for (int64_t q = 0; q < n; q += s->xfer_elems) {
    const int64_t m = std::min(s->xfer_elems, n - q);
    QD_CUDA(cudaMemcpyAsync(s->xfer, host + 2 * q, m * sizeof(double2), cudaMemcpyHostToDevice, st));
    launch_narrow(st, s->xfer, s->psi_thf + off + q, m);
  }
}
static void theta_to_host(qd_session *s, int64_t off, int64_t n, double *host, cudaStream_t st) {
  if (!s->psi_thf) {
    QD_CUDA(cudaMemcpyAsync(host, s->psi_th + off, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    return;
  }
  for (int64_t q = 0; q < n; q += s->xfer_elems) {
    const int64_t m = std::min(s->xfer_elems, n - q);
    launch_widen(st, s->psi_thf + off + q, s->xfer, m);
    QD_CUDA(cudaMemcpyAsync(host + 2 * q, s->xfer, m * sizeof(double2), cudaMemcpyDeviceToHost, st));
  }
}

// ------------------------------------------------------------ create
// Everything the device state of a batch depends on besides the per-call inputs
// (wave packets, potential, masks, quadrature weights, Legendre matrices, CRP
// energies, |a(E)|^2 and accumulators): sizes, grids, time step, precision,
// the Omega lists and the flux surface.  Two calls with equal keys can share
// one session's buffers, tables and step graph.
static std::vector<double> session_key(qd_fh2data *const *pr, int n) {
  std::vector<double> k;
  int dev = 0;
  cudaGetDevice(&dev);
  const qd_fh2data *d = pr[0];
  k.insert(k.end(), {(double)dev, (double)n, (double)d->r1.n, d->r1.left, d->r1.dr, d->r1.mass, (double)d->r2.n,
                     d->r2.left, d->r2.dr, d->r2.mass, (double)d->theta.n, (double)d->OmegaStates.l_max,
                     d->time.time_step, (double)d->options.precision, (double)(d->dump1.dump && d->dump2.dump),
                     (double)d->CRP.calculate_CRP});
  if (d->CRP.calculate_CRP)
    k.insert(k.end(), {(double)d->CRP.n_energies, (double)d->CRP.n_gradient_points, (double)d->CRP.n_dividing_surface});
  for (int p = 0; p < n; p++) {
    const qd_omega_states &om = pr[p]->OmegaStates;
    k.insert(k.end(), {(double)om.J, (double)om.parity, (double)om.n_omegas});
    for (int i = 0; i < om.n_omegas; i++) k.push_back((double)om.omegas[i]);
  }
  return k;
}

__global__ void k_differs(const double *__restrict__ a, const double *__restrict__ b, int64_t n, int *flag) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    if (__double_as_longlong(a[q]) != __double_as_longlong(b[q])) {
      *flag = 1;
      return;
    }
}

// ------------------------------------------------------------- autotuner
// The mixed form's 2-D FFT has several kernels for a grid: separable shapes with
// different CTA and cluster sizes, the two-exchange cluster kernel and the
// three-pass kernels (FFTPlan::cand).  The first session of a key (device
// architecture and SM count, grid, slab count, coupled or not) times each
// candidate on its own slab pool, zeroed before any input is loaded: one
// warm-up launch, then three launches between CUDA events; the fastest is kept.
// Choices live in a process-wide map and, when a cache file is named
// (options.autotune_cache, else the QD_AUTOTUNE_CACHE environment variable), in
// that file: one line "<key>\t<choice>\t<microseconds>" per key, read before
// tuning and appended after it.
static std::mutex g_tune_mutex;
static std::map<std::string, std::pair<int, double>> *g_tune = nullptr;   // never freed
static std::set<std::string> *g_tune_read = nullptr;

static std::string tune_key(qd_session *s) {
  int cc_major = 0, cc_minor = 0, sms = 0;
  cudaDeviceGetAttribute(&cc_major, cudaDevAttrComputeCapabilityMajor, s->device);
  cudaDeviceGetAttribute(&cc_minor, cudaDevAttrComputeCapabilityMinor, s->device);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
  std::ostringstream k;
  k << "fft_mixed sm" << cc_major << cc_minor << "x" << sms << " grid " << s->g.n1 << "x" << s->g.n2 << " slabs "
    << s->n_slabs << " coupled " << (s->any_coupled ? 1 : 0);
  return k.str();
}

static const char *tune_path(const qd_fh2data *d) {
  if (d->options.autotune_cache && *d->options.autotune_cache) return d->options.autotune_cache;
  const char *e = std::getenv("QD_AUTOTUNE_CACHE");
  return e && *e ? e : nullptr;
}

// reads the cache file once per path into the map (caller holds g_tune_mutex)
static void tune_read_file(const char *path) {
  if (!path) return;
  if (!g_tune_read) g_tune_read = new std::set<std::string>();
  if (!g_tune_read->insert(path).second) return;
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line)) {
    const size_t a = line.find('\t'), b = line.find('\t', a == std::string::npos ? a : a + 1);
    if (a == std::string::npos || b == std::string::npos) continue;
    try {
      (*g_tune)[line.substr(0, a)] = {std::stoi(line.substr(a + 1, b - a - 1)), std::stod(line.substr(b + 1))};
    } catch (const std::exception &) {
      // a malformed line is skipped
    }
  }
}

static void autotune_fft(qd_session *s, const qd_fh2data *d0) {
  FFTPlan &p = s->fft;
  if (s->precision != QD_PRECISION_MIXED || p.n_cand <= 1) {
    s->tuning = "fft: " + fft_choice_name(p.choice) + " (only candidate)";
    return;
  }
  const std::string key = tune_key(s);
  const char *path = tune_path(d0);
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    if (!g_tune) g_tune = new std::map<std::string, std::pair<int, double>>();
    tune_read_file(path);
    auto it = g_tune->find(key);
    if (it != g_tune->end())
      for (int q = 0; q < p.n_cand; q++)
        if (p.cand[q] == it->second.first) {
          fft_plan_choose(p, it->second.first);
          s->tuning = "fft: " + fft_choice_name(p.choice) + " (cached, " + std::to_string(it->second.second) + " us)";
          return;
        }
  }
  // time every candidate on the zeroed slab pool
  cudaStream_t st = s->stream;
  const Grid &g = s->g;
  QD_CUDA(cudaMemsetAsync(s->psi_jf, 0, (size_t)s->n_slabs * g.npt * sizeof(float2), st));
  for (float *t : {s->T1f, s->I1f}) QD_CUDA(cudaMemsetAsync(t, 0, (size_t)g.n1 * sizeof(float), st));
  for (float *t : {s->T2f, s->I2f}) QD_CUDA(cudaMemsetAsync(t, 0, (size_t)g.n2 * sizeof(float), st));
  const int tiles = fft_max_tiles(p);
  double *ke = s->alloc<double>((size_t)s->n_slabs * tiles);
  double *re = s->alloc<double>((size_t)s->n_slabs * tiles);
  FFTLift lf{};
  lf.proR = s->any_coupled ? nullptr : s->lrotR;
  lf.pror = s->any_coupled ? nullptr : s->lrotr;
  lf.epiR = s->lrotR;
  lf.epir = s->lrotr;
  lf.kinR = s->lkinR;
  lf.kinr = s->lkinr;
  lf.T1f = s->T1f;
  lf.T2f = s->T2f;
  lf.I1f = s->I1f;
  lf.I2f = s->I2f;
  // each candidate: two warm-up launches, then seven launches between events; the median
  // launch time decides (the shapes of one grid differ by a few percent, about the spread of
  // a three-launch average)
  constexpr int TUNE_REPS = 7;
  cudaEvent_t ev[TUNE_REPS + 1];
  for (cudaEvent_t &e : ev) QD_CUDA(cudaEventCreate(&e));
  int best = -1;
  double best_us = 0.0;
  std::string report;
  for (int q = 0; q < p.n_cand; q++) {
    fft_plan_choose(p, p.cand[q]);
    double us = -1.0;
    try {
      for (int r = 0; r < 2 + TUNE_REPS; r++) {
        if (r >= 2) QD_CUDA(cudaEventRecord(ev[r - 2], st));
        launch_fft_kinetic(st, g, p, s->psi_jf, s->d_slabs, s->n_slabs, ke, s->any_coupled ? nullptr : re, s->status,
                           &lf);
      }
      QD_CUDA(cudaEventRecord(ev[TUNE_REPS], st));
      QD_CUDA(cudaEventSynchronize(ev[TUNE_REPS]));
      float ms[TUNE_REPS];
      for (int r = 0; r < TUNE_REPS; r++) QD_CUDA(cudaEventElapsedTime(&ms[r], ev[r], ev[r + 1]));
      std::sort(ms, ms + TUNE_REPS);
      us = 1e3 * ms[TUNE_REPS / 2];
    } catch (const Error &) {
      cudaGetLastError();   // a candidate that cannot launch here is skipped
      QD_CUDA(cudaStreamSynchronize(st));
    }
    report += (q ? ", " : "") + fft_choice_name(p.cand[q]) + " = " + (us < 0 ? std::string("n/a") : std::to_string(us));
    if (us >= 0 && (best < 0 || us < best_us)) {
      best = p.cand[q];
      best_us = us;
    }
  }
  for (cudaEvent_t e : ev) cudaEventDestroy(e);
  if (best < 0) throw Error{QD_ERR_CUDA, "autotuner: no FFT kernel could run on this device"};
  fft_plan_choose(p, best);
  s->tuning = "fft: " + fft_choice_name(best) + " (tuned: " + report + " us)";
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  (*g_tune)[key] = {best, best_us};
  if (path) {
    std::ofstream f(path, std::ios::app);
    if (f) f << key << '\t' << best << '\t' << best_us << '\n';
  }
}

// Layout, buffers and the tables that depend only on the key.
static void session_build(qd_session *s, qd_fh2data *const *problems, int n_problems) {
  validate_batch(problems, n_problems, s->probs);
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
    throw Error{QD_ERR_NO_DEVICE, "no CUDA device"};
  QD_CUDA(cudaGetDevice(&s->device));
  QD_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  QD_CUDA(cudaStreamCreateWithFlags(&s->stream_dl, cudaStreamNonBlocking));
  QD_CUDA(cudaEventCreateWithFlags(&s->ev_steps, cudaEventDisableTiming));
  QD_CUDA(cudaMallocHost(&s->h_status, 3 * sizeof(int)));
  s->key = session_key(problems, n_problems);
  cudaStream_t st = s->stream;
  const qd_fh2data *d0 = problems[0];
  Grid &g = s->g;
  g.n1 = d0->r1.n;
  g.n2 = d0->r2.n;
  g.nth = d0->theta.n;
  g.l_max = d0->OmegaStates.l_max;
  g.npt = (int64_t)g.n1 * g.n2;
  g.dr1 = d0->r1.dr;
  g.dr2 = d0->r2.dr;
  g.m1 = d0->r1.mass;
  g.m2 = d0->r2.mass;
  g.left1 = d0->r1.left;
  g.left2 = d0->r2.left;
  s->precision = d0->options.precision;
  s->dt = d0->time.time_step;
  s->norm_tol = s->precision == QD_PRECISION_MIXED ? 1e-4 : 1e-10;
  s->n_problems = n_problems;
  fft_plan_init(s->fft, g.n1, g.n2);

  // blocks and slabs
  int slab = 0;
  int64_t bmat = 0;
  s->h_pblock0.push_back(0);
  for (int p = 0; p < n_problems; p++) {
    ProblemHost &ph = s->probs[p];
    if (ph.coupled) s->any_coupled = true;
    for (int o : ph.omegas) {
      BlockDesc bd{};
      bd.problem = p;
      bd.omega = o;
      bd.nl = g.l_max - o + 1;
      bd.slab0 = slab;
      bd.bmat0 = bmat;
      for (int l = o; l <= g.l_max; l++) s->h_slabs.push_back(SlabDesc{(int32_t)s->h_blocks.size(), l});
      slab += bd.nl;
      bmat += (int64_t)bd.nl * g.nth;
      s->max_nl = std::max(s->max_nl, bd.nl);
      s->h_blocks.push_back(bd);
    }
    s->h_pblock0.push_back((int)s->h_blocks.size());
  }
  s->n_blocks = (int)s->h_blocks.size();
  s->n_slabs = slab;
  s->d_blocks = s->upload(s->h_blocks.data(), s->h_blocks.size());
  s->d_slabs = s->upload(s->h_slabs.data(), s->h_slabs.size());
  s->d_pblock0 = s->upload(s->h_pblock0.data(), s->h_pblock0.size());

  // wave packets: the mixed form keeps both pools in c64 (every value its step
  // writes there, tensor-core epilogues and FP32 FFT, is an FP32 number)
  const int64_t nth_pt = g.npt * g.nth;
  if (s->precision == QD_PRECISION_MIXED) {
    s->psi_thf = s->alloc<float2>((size_t)s->n_blocks * nth_pt);
    s->psi_jf = s->alloc<float2>((size_t)s->n_slabs * g.npt);
    s->xfer_elems = std::min<int64_t>((int64_t)s->n_blocks * nth_pt, (int64_t)1 << 25);
    s->xfer = s->alloc<double2>((size_t)s->xfer_elems);
  } else {
    s->psi_th = s->alloc<double2>((size_t)s->n_blocks * nth_pt);
    s->psi_j = s->alloc<double2>((size_t)s->n_slabs * g.npt);
  }

  // tables of the key: kinetic, rotational, inverse inertia
  std::vector<double> T1(g.n1), T2(g.n2);
  auto kin = [](int n, double dr, double mass, std::vector<double> &T) {
    const double two_pi_xl = 2 * M_PI / (n * dr);   // cudaMath.h:117-130
    for (int i = 0; i < n; i++) {
      const double k = two_pi_xl * (i <= n / 2 ? i : i - n);
      T[i] = k * k / (mass + mass);
    }
  };
  kin(g.n1, g.dr1, g.m1, T1);
  kin(g.n2, g.dr2, g.m2, T2);
  s->T1 = s->upload(T1.data(), T1.size());
  s->T2 = s->upload(T2.data(), T2.size());
  s->pot = s->alloc<double>((size_t)nth_pt);
  s->pot_stage = s->alloc<double>((size_t)nth_pt);
  s->d_flag = s->alloc<int>(1);
  s->w = s->alloc<double>((size_t)g.nth);
  s->has_mask = d0->dump1.dump && d0->dump2.dump;   // MatlabData::dump_wavepacket (matlabData.h:27)
  if (s->has_mask) {
    s->d1 = s->alloc<double>((size_t)g.n1);
    s->d2 = s->alloc<double>((size_t)g.n2);
  }
  const bool fp64 = s->precision == QD_PRECISION_FP64;
  if (fp64) {
    s->tab_v = s->alloc<double2>((size_t)nth_pt);
    s->tab_v0 = s->alloc<double2>((size_t)nth_pt);
  }
  const int64_t nrot = g.npt * (g.l_max + 1);
  if (s->any_coupled) {
    s->tab_rot4 = s->alloc<double2>((size_t)nrot);
    launch_build_rot_table(st, g, 0.25 * s->dt, s->tab_rot4);
  } else if (fp64) {
    s->tab_rot2 = s->alloc<double2>((size_t)nrot);
    launch_build_rot_table(st, g, 0.5 * s->dt, s->tab_rot2);
  }
  s->tab_kin = s->alloc<double2>((size_t)g.npt);
  launch_build_kin_table(st, g, s->T1, s->T2, s->dt, s->tab_kin);
  // FP32 tables (the mixed form; also used by mixed-precision stage calls)
  s->wf = s->alloc<float>((size_t)g.nth);
  s->wvf = s->alloc<float>((size_t)nth_pt);
  s->T1f = s->alloc<float>((size_t)g.n1);
  s->T2f = s->alloc<float>((size_t)g.n2);
  s->I1f = s->alloc<float>((size_t)g.n1);
  s->I2f = s->alloc<float>((size_t)g.n2);
  if (s->has_mask) {
    s->d1f = s->alloc<float>((size_t)g.n1);
    s->d2f = s->alloc<float>((size_t)g.n2);
  }
  if (!fp64) {
    s->vph = s->alloc<float2>((size_t)nth_pt);
    s->vph0 = s->alloc<float2>((size_t)nth_pt);
    const double drot = (s->any_coupled ? 0.25 : 0.5) * s->dt;
    s->lrotR = s->alloc<float2>((size_t)(g.l_max + 1) * g.n1);
    s->lrotr = s->alloc<float2>((size_t)(g.l_max + 1) * g.n2);
    launch_build_lift_rot(st, g.n1, g.l_max, g.left1, g.dr1, g.m1, drot, s->lrotR);
    launch_build_lift_rot(st, g.n2, g.l_max, g.left2, g.dr2, g.m2, drot, s->lrotr);
    s->lkinR = s->alloc<float2>((size_t)g.n1);
    s->lkinr = s->alloc<float2>((size_t)g.n2);
    launch_build_lift_kin(st, g.n1, s->T1, s->dt, s->lkinR);
    launch_build_lift_kin(st, g.n2, s->T2, s->dt, s->lkinr);
  }

  // Legendre matrices (filled per call): forward B = w_k P (k, n) as [k][n];
  // backward P as [n][k]; their tensor-core images (BF16x3 split, shared-memory layout)
  s->h_Bf.assign((size_t)bmat, 0.0);
  s->h_Bb.assign((size_t)bmat, 0.0);
  s->Bf = s->alloc<double>((size_t)bmat);
  s->Bb = s->alloc<double>((size_t)bmat);
  {
    auto r16 = [](int x) { return (x + 15) & ~15; };
    std::vector<int64_t> of, ob;
    int64_t tf = 0, tb = 0;
    for (const BlockDesc &bd : s->h_blocks) {
      of.push_back(tf);
      tf += 3LL * r16(bd.nl) * r16(g.nth) * 2;
      s->smem_f = std::max(s->smem_f, tc_ws_smem_bytes(true, r16(g.nth), r16(bd.nl)));
      ob.push_back(tb);
      tb += 3LL * r16(g.nth) * r16(bd.nl) * 2;
      s->smem_b = std::max(s->smem_b, tc_ws_smem_bytes(false, r16(bd.nl), r16(g.nth)));
    }
    bool ok = true;
    for (const BlockDesc &bd : s->h_blocks)
      ok = ok && tc_shape_ok(true, r16(g.nth), r16(bd.nl)) && tc_shape_ok(false, r16(bd.nl), r16(g.nth));
    if (!ok) {
      if (s->precision == QD_PRECISION_MIXED)
        throw Error{QD_ERR_UNSUPPORTED, "mixed form: n_theta and l_max+1 above the tensor-core tile limit "
                                        "(contraction <= 192, columns <= 160)"};
    } else {
      tc_set_smem_limit(std::max(s->smem_f, s->smem_b));
      s->imgoff_f = s->upload(of.data(), of.size());
      s->imgoff_b = s->upload(ob.data(), ob.size());
      s->img_f = s->alloc<uint16_t>((size_t)tf / 2);
      s->img_b = s->alloc<uint16_t>((size_t)tb / 2);
      s->bscale_f = s->alloc<float>((size_t)s->n_blocks * 256);
      s->bscale_b = s->alloc<float>((size_t)s->n_blocks * 256);
    }
  }

  // Coriolis groups (cudaOpenMP2.cu:158-209): one per (problem, l >= omega_min)
  if (s->any_coupled) {
    std::vector<double> V, E, H;
    s->h_pgroup0.push_back(0);
    int64_t ph0 = 0;
    for (int p = 0; p < n_problems; p++) {
      const ProblemHost &ph = s->probs[p];
      // J = 0 problems of a coupled batch get 1x1 zero matrices: identity
      // coupling, but their second rotational quarter step still applies
      for (int l = ph.omega_min; l <= g.l_max; l++) {
        const int omax = std::min(std::min(ph.J, l), ph.omega_cap);
        const int n = omax - ph.omega_min + 1;
        if (n < 1) continue;
        std::vector<double> a((size_t)n * n, 0.0);
        for (int k = 0; k < n; k++) {
          const int om = k + ph.omega_min;
          a[(size_t)k * n + k] = ph.J * (ph.J + 1.0) - 2.0 * om * om;
          if (k + 1 < n) {
            const double off = -lam(ph.J, om) * lam(l, om) * std::sqrt(1.0 + (om == 0 ? 1.0 : 0.0));
            a[(size_t)k * n + k + 1] = off;
            a[(size_t)(k + 1) * n + k] = off;
          }
        }
        std::vector<double> e, v;
        jacobi_eigen(n, a, e, v);
        CoriolisGroup gr{};
        gr.l = l;
        gr.n = n;
        gr.block_lo = s->h_pblock0[p];
        gr.omega_lo = ph.omega_min;
        gr.v0 = (int64_t)V.size();
        gr.e0 = (int64_t)E.size();
        gr.h0 = (int64_t)H.size();
        gr.ph0 = ph0;
        ph0 += (int64_t)n * g.n1;
        V.insert(V.end(), v.begin(), v.end());
        E.insert(E.end(), e.begin(), e.end());
        H.insert(H.end(), a.begin(), a.end());
        s->h_groups.push_back(gr);
        s->max_group_n = std::max(s->max_group_n, n);
      }
      s->h_pgroup0.push_back((int)s->h_groups.size());
    }
    s->n_groups = (int)s->h_groups.size();
    s->d_groups = s->upload(s->h_groups.data(), s->h_groups.size());
    s->d_pgroup0 = s->upload(s->h_pgroup0.data(), s->h_pgroup0.size());
    s->cor_V = s->upload(V.data(), V.size());
    s->cor_e = s->upload(E.data(), E.size());
    s->cor_H = s->upload(H.data(), H.size());
    s->cor_ph = s->alloc<double2>((size_t)ph0);
    launch_build_coriolis_phase(st, g, s->d_groups, s->n_groups, s->max_group_n, s->cor_e, 0.5 * s->dt, s->cor_ph);
    if (s->precision == QD_PRECISION_MIXED && s->max_group_n <= CORIOLIS_F32_MAXN) {
      // eigenvectors as FP32 pairs (hi + lo) and the phases as three-shear coefficients
      std::vector<float> vh(V.size()), vl(V.size());
      for (size_t q = 0; q < V.size(); q++) {
        vh[q] = (float)V[q];
        vl[q] = (float)(V[q] - (double)vh[q]);
      }
      s->cor_Vh = s->upload(vh.data(), vh.size());
      s->cor_Vl = s->upload(vl.data(), vl.size());
      s->cor_phl = s->alloc<float2>((size_t)ph0);
      launch_build_coriolis_lift(st, g, s->d_groups, s->n_groups, s->cor_e, 0.5 * s->dt, s->cor_phl);
      std::vector<int> order;
      for (int c = CORIOLIS_F32_CLASSES - 1; c >= 0; c--)
        for (int gi = 0; gi < s->n_groups; gi++)
          if (coriolis_f32_class(s->h_groups[gi].n) == c) order.push_back(gi);
      s->cor_order = s->upload(order.data(), order.size());
      s->cor_f32 = true;
    }
  }

  // the mixed form's FFT kernel for this grid and slab count (the partial-sum tiles below follow it)
  autotune_fft(s, d0);

  // energies and partials
  s->t_modpe = s->precision == QD_PRECISION_MIXED ? legendre_tc_part_slots(g, s->max_nl) : legendre_bwd_part_tiles(g);
  s->t_ke = fft_col_tiles(s->fft, s->precision);
  // CTAs per group of the FP32 Coriolis passes: twice the base while the groups are few (one
  // coupled problem has about l_max of them), the base for batched runs with thousands, where
  // more tiles only add partial sums
  const int cor_tiles = s->n_groups < CORIOLIS_F32_FEW_GROUPS ? 2 * CORIOLIS_F32_TILES : CORIOLIS_F32_TILES;
  s->t_re = s->any_coupled ? (s->cor_f32 ? cor_tiles : CORIOLIS_F32_TILES) : fft_row_tiles(s->fft, s->precision);
  s->t_ce = s->cor_f32 ? cor_tiles : coriolis_tiles(g);
  s->part_modpe = s->alloc<double>((size_t)s->n_blocks * s->t_modpe * 2);
  s->part_ke = s->alloc<double>((size_t)s->n_slabs * s->t_ke);
  s->part_re = s->alloc<double>((size_t)s->n_slabs * s->t_re);
  if (s->any_coupled) s->part_ce = s->alloc<double>((size_t)std::max(1, s->n_groups) * s->max_group_n * s->t_ce);
  s->energies = s->alloc<double>((size_t)s->n_blocks * 6);
  s->status = s->alloc<int>(1);
  s->status_step = s->alloc<int>(1);
  s->d_step = s->alloc<int>(1);
  s->step_done = s->alloc<unsigned>(1);

  // flux
  const qd_crp &c = d0->CRP;
  s->flux.enabled = c.calculate_CRP != 0;
  if (s->flux.enabled) {
    if (s->precision == QD_PRECISION_MIXED && c.n_gradient_points > 32)
      throw Error{QD_ERR_UNSUPPORTED, "mixed form: CRP.n_gradient_points above 32"};
    s->flux.n_energies = c.n_energies;
    s->flux.n_grad = c.n_gradient_points;
    s->flux.n_ds = c.n_dividing_surface;
    s->flux.chunk = 64;   // steps per flux DFT flush (and per CUDA graph)
    const int64_t ns = (int64_t)g.nth * g.n1;
    if (s->precision == QD_PRECISION_MIXED)
      s->flux_buf_f = s->alloc<float2>((size_t)s->flux.chunk * s->n_blocks * 2 * ns);
    else
      s->flux_buf = s->alloc<double2>((size_t)s->flux.chunk * s->n_blocks * 2 * ns);
    s->flux_acc = s->alloc<double2>((size_t)s->n_blocks * 2 * c.n_energies * ns);
    s->flux_fresh = s->alloc<int>(1);
    s->flux_phase = s->alloc<double2>((size_t)s->flux.chunk * c.n_energies);
    s->half_v = s->alloc<double2>((size_t)g.nth * c.n_gradient_points * g.n1);
    std::vector<double> fdw = fd_weights(c.n_gradient_points);
    for (double &x : fdw) x /= g.dr2;
    s->fd = s->upload(fdw.data(), fdw.size());
    s->flux_E = s->alloc<double>((size_t)c.n_energies);
    s->flux_eta = s->alloc<double>((size_t)n_problems * c.n_energies);
    s->crp = s->alloc<double>((size_t)n_problems * c.n_energies);
    s->flux_t0 = s->alloc<double>(1);
    s->flux_count = s->alloc<int>(1);
    s->flux_slot = s->alloc<int>(1);
    if (s->precision == QD_PRECISION_MIXED) {
      s->half_v_lift = s->alloc<float2>((size_t)g.nth * c.n_gradient_points * g.n1);
      std::vector<float> fdw32(fdw.begin(), fdw.end());
      s->fdf = s->upload(fdw32.data(), fdw32.size());
    }
  }
  s->launches_per_step = count_launches_per_step(s);
}

// Per-call inputs of a session: the wave packets, the potential, masks,
// quadrature weights and Legendre matrices (with the tables built from them),
// the CRP inputs and the counters.  On a reused session (`reuse`) the tables
// are rebuilt only when their inputs changed: the potential is compared on the
// device (bit for bit, against the copy the tables were built from), the small
// inputs on the host.
static void session_load(qd_session *s, qd_fh2data *const *problems, int n_problems, bool reuse) {
  if (reuse) validate_batch(problems, n_problems, s->probs);
  cudaStream_t st = s->stream;
  const Grid &g = s->g;
  const qd_fh2data *d0 = problems[0];
  const int64_t nth_pt = g.npt * g.nth;
  const bool fp64 = s->precision == QD_PRECISION_FP64;
  s->steps = d0->time.steps;
  for (int p = 0; p < n_problems; p++) s->probs[p].d = problems[p];

  // potential: compared on the device with the one the tables hold
  bool pot_changed = !reuse;
  if (reuse) {
    QD_CUDA(cudaMemcpyAsync(s->pot_stage, d0->pot, (size_t)nth_pt * sizeof(double), cudaMemcpyHostToDevice, st));
    QD_CUDA(cudaMemsetAsync(s->d_flag, 0, sizeof(int), st));
    k_differs<<<grid_for(nth_pt, 256, 152 * 8), 256, 0, st>>>(s->pot_stage, s->pot, nth_pt, s->d_flag);
    // the flag is read as soon as the comparison ends, while the wave packets upload
    QD_CUDA(cudaMemcpyAsync(s->h_status + 2, s->d_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    QD_CUDA(cudaEventRecord(s->ev_steps, st));
  } else {
    QD_CUDA(cudaMemcpyAsync(s->pot, d0->pot, (size_t)nth_pt * sizeof(double), cudaMemcpyHostToDevice, st));
  }
  // wave packets (uploads overlap the host work below)
  for (int p = 0; p < n_problems; p++)
    theta_from_host(s, (int64_t)s->h_pblock0[p] * nth_pt, (int64_t)s->probs[p].n_omegas * nth_pt,
                    problems[p]->OmegaStates.wave_packets);
  // small inputs, compared on the host
  auto same = [](const std::vector<double> &h, const double *x, size_t n) {
    return h.size() == n && (n == 0 || std::memcmp(h.data(), x, n * sizeof(double)) == 0);
  };
  const bool w_changed = !reuse || !same(s->h_w, d0->theta.w, (size_t)g.nth);
  const bool mask_changed =
      s->has_mask && (!reuse || !same(s->h_d1, d0->dump1.dump, (size_t)g.n1) || !same(s->h_d2, d0->dump2.dump, (size_t)g.n2));
  if (w_changed) {
    s->h_w.assign(d0->theta.w, d0->theta.w + g.nth);
    QD_CUDA(cudaMemcpyAsync(s->w, s->h_w.data(), g.nth * sizeof(double), cudaMemcpyHostToDevice, st));
  }
  if (mask_changed) {
    s->h_d1.assign(d0->dump1.dump, d0->dump1.dump + g.n1);
    s->h_d2.assign(d0->dump2.dump, d0->dump2.dump + g.n2);
    QD_CUDA(cudaMemcpyAsync(s->d1, s->h_d1.data(), g.n1 * sizeof(double), cudaMemcpyHostToDevice, st));
    QD_CUDA(cudaMemcpyAsync(s->d2, s->h_d2.data(), g.n2 * sizeof(double), cudaMemcpyHostToDevice, st));
  }
  // Legendre matrices of every block
  std::vector<double> Bf(s->h_Bf.size()), Bb(s->h_Bb.size());
  for (int b = 0; b < s->n_blocks; b++) {
    const BlockDesc &bd = s->h_blocks[b];
    const ProblemHost &ph = s->probs[bd.problem];
    const qd_omega_states &om = ph.d->OmegaStates;
    const int bi = b - s->h_pblock0[bd.problem];
    for (int n = 0; n < bd.nl; n++)
      for (int k = 0; k < g.nth; k++) {
        const double P = om.associated_legendres[((int64_t)bi * om.n_cols + n) * g.nth + k];
        Bf[bd.bmat0 + (int64_t)k * bd.nl + n] = ph.d->theta.w[k] * P;
        Bb[bd.bmat0 + (int64_t)n * g.nth + k] = P;
      }
  }
  const bool legendre_changed = !reuse || Bf != s->h_Bf || Bb != s->h_Bb;
  if (legendre_changed) {
    s->h_Bf.swap(Bf);
    s->h_Bb.swap(Bb);
    QD_CUDA(cudaMemcpyAsync(s->Bf, s->h_Bf.data(), s->h_Bf.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    QD_CUDA(cudaMemcpyAsync(s->Bb, s->h_Bb.data(), s->h_Bb.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    if (s->img_f) {
      launch_build_tc_bimage(st, s->d_blocks, s->n_blocks, s->Bf, g.nth, true, s->imgoff_f, s->img_f, s->bscale_f,
                             (s->max_nl + 15) & ~15);
      launch_build_tc_bimage(st, s->d_blocks, s->n_blocks, s->Bb, g.nth, false, s->imgoff_b, s->img_b, s->bscale_b,
                             (g.nth + 15) & ~15);
    }
  }
  if (reuse) {
    QD_CUDA(cudaEventSynchronize(s->ev_steps));
    if (s->h_status[2]) {
      pot_changed = true;
      QD_CUDA(cudaMemcpyAsync(s->pot, s->pot_stage, (size_t)nth_pt * sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
  }
  // tables of the potential, masks and weights
  if (fp64 && (pot_changed || mask_changed)) {
    launch_build_theta_table(st, g, s->pot, s->d1, s->d2, s->dt, s->tab_v);
    launch_build_theta_table(st, g, s->pot, s->d1, s->d2, 0.5 * s->dt, s->tab_v0);
  }
  if (pot_changed || mask_changed || w_changed)
    launch_build_float_tables(st, g, s->w, s->pot, s->d1, s->d2, s->T1, s->T2, s->wf, s->wvf, s->d1f, s->d2f, s->T1f,
                              s->T2f, s->I1f, s->I2f);
  if (!fp64 && pot_changed) {
    launch_build_lift_theta(st, g, s->pot, s->dt, s->vph);
    launch_build_lift_theta(st, g, s->pot, 0.5 * s->dt, s->vph0);
  }
  // counters and energies
  QD_CUDA(cudaMemsetAsync(s->energies, 0, (size_t)s->n_blocks * 6 * sizeof(double), st));
  QD_CUDA(cudaMemsetAsync(s->step_done, 0, sizeof(unsigned), st));
  QD_CUDA(cudaMemsetAsync(s->status, 0, sizeof(int), st));
  QD_CUDA(cudaMemsetAsync(s->status_step, 0, sizeof(int), st));
  QD_CUDA(cudaMemcpyAsync(s->d_step, &s->steps, sizeof(int), cudaMemcpyHostToDevice, st));
  s->rec = nullptr;
  s->rec_cap = 0;
  s->rec_base = 0;
  // flux inputs
  s->flux_pending = 0;
  if (s->flux.enabled) {
    const qd_crp &c = d0->CRP;
    const int64_t ns = (int64_t)g.nth * g.n1;
    QD_CUDA(cudaMemcpyAsync(s->flux_E, c.energies, (size_t)c.n_energies * sizeof(double), cudaMemcpyHostToDevice, st));
    for (int p = 0; p < n_problems; p++)
      QD_CUDA(cudaMemcpyAsync(s->flux_eta + (size_t)p * c.n_energies, problems[p]->CRP.eta_sq,
                              (size_t)c.n_energies * sizeof(double), cudaMemcpyHostToDevice, st));
    QD_CUDA(cudaMemsetAsync(s->flux_count, 0, sizeof(int), st));
    if (pot_changed) {
      launch_build_half_v(st, g, s->flux, s->pot, s->dt, s->half_v);
      if (s->half_v_lift) launch_build_half_v_lift(st, g, s->flux, s->pot, s->dt, s->half_v_lift);
    }
    // accumulators: the caller's sums, or none (the first transform writes them, P(E)
    // before it is zero); all problems of a batch either pass theirs or none
    bool any_acc = false, all_acc = true;
    for (int p = 0; p < n_problems; p++) {
      any_acc = any_acc || problems[p]->CRP.accumulators;
      all_acc = all_acc && problems[p]->CRP.accumulators;
    }
    for (int p = 0; p < n_problems && any_acc; p++) {
      double2 *dst = s->flux_acc + (int64_t)s->h_pblock0[p] * 2 * c.n_energies * ns;
      const size_t bytes = (size_t)s->probs[p].n_omegas * 2 * c.n_energies * ns * sizeof(double2);
      if (problems[p]->CRP.accumulators)
        QD_CUDA(cudaMemcpyAsync(dst, problems[p]->CRP.accumulators, bytes, cudaMemcpyHostToDevice, st));
      else if (!all_acc)
        QD_CUDA(cudaMemsetAsync(dst, 0, bytes, st));
    }
    QD_CUDA(cudaMemsetAsync(s->flux_fresh, any_acc ? 0 : 1, sizeof(int), st));
  }
  QD_CUDA(cudaGetLastError());
}

static void session_create(qd_session *s, qd_fh2data *const *problems, int n_problems) {
  session_build(s, problems, n_problems);
  session_load(s, problems, n_problems, false);
  QD_CUDA(cudaStreamSynchronize(s->stream));
  QD_CUDA(cudaGetLastError());
}

// -------------------------------------------------------------- running
static void throw_status(int st, int stp) {
  if (st == QD_ERR_NORM)
    throw Error{st, "Total module error: norm above 1 at step " + std::to_string(stp) +
                        " (print_energies, cudaOpenMP2.cu:437-440)"};
  if (st == QD_ERR_TIMEOUT)
    throw Error{st, "a device-side wait gave up after 1 s: a tensor-core contraction's pipeline stalled"};
  if (st == QD_ERR_INVALID) throw Error{st, "flux surface buffer full (more steps buffered than its capacity)"};
  if (st) throw Error{st, "device status " + std::to_string(st)};
}
static void check_status(qd_session *s) {
  QD_CUDA(cudaStreamSynchronize(s->stream));
  QD_CUDA(cudaGetLastError());
  int st = 0, stp = 0;
  QD_CUDA(cudaMemcpy(&st, s->status, sizeof(int), cudaMemcpyDeviceToHost));
  if (st == QD_ERR_NORM) QD_CUDA(cudaMemcpy(&stp, s->status_step, sizeof(int), cudaMemcpyDeviceToHost));
  throw_status(st, stp);
}

static void flush_flux(qd_session *s) {
  if (s->flux.enabled && s->flux_pending > 0) {
    enqueue_flux_dft(s);
    s->flux_pending = 0;
  }
}

// steps (and, with flux, the transform of a full chunk) captured into one graph
static void capture_steps(qd_session *s, int steps, bool with_flux, cudaGraphExec_t *exec) {
  if (*exec) {
    cudaGraphExecDestroy(*exec);
    *exec = nullptr;
  }
  cudaGraph_t graph;
  QD_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  try {
    for (int i = 0; i < steps; i++) enqueue_step(s, false);
    if (with_flux) enqueue_flux_dft(s);
  } catch (...) {
    cudaStreamEndCapture(s->stream, &graph);
    throw;
  }
  QD_CUDA(cudaStreamEndCapture(s->stream, &graph));
  QD_CUDA(cudaGraphInstantiate(exec, graph, 0));
  cudaGraphDestroy(graph);
}

static void build_pow_graphs(qd_session *s) {
  for (int k = 1; k <= qd_session::N_POW_GRAPHS; k++) capture_steps(s, 1 << k, false, &s->graph_pow[k]);
  s->pow_rec = s->rec;
  s->pow_rec_base = s->rec_base;
  s->pow_rec_cap = s->rec_cap;
}

static void build_chunk_graph(qd_session *s, int steps) {
  capture_steps(s, steps, s->flux.enabled, &s->graph_chunk);
  s->graph_steps = steps;
  s->graph_rec = s->rec;
  s->graph_rec_base = s->rec_base;
  s->graph_rec_cap = s->rec_cap;
}

// Enqueue n steps without host synchronisation.
static void run_steps(qd_session *s, int n) {
  const int chunk = s->flux.enabled ? s->flux.chunk : 32;
  while (n > 0) {
    if (s->steps == 0) {
      // first step: V(-dt/2) folded into the prologue table (cudaOpenMP2.cu:344)
      enqueue_step(s, true);
      s->steps++;
      n--;
      // flush step 0's surface values at once, so that later steps align with whole graph chunks
      if (s->flux.enabled && ++s->flux_pending > 0) flush_flux(s);
      continue;
    }
    if (n >= chunk && s->flux_pending == 0) {
      if (!s->graph_chunk || s->graph_steps != chunk || s->graph_rec != s->rec || s->graph_rec_base != s->rec_base ||
          s->graph_rec_cap != s->rec_cap)
        build_chunk_graph(s, chunk);
      QD_CUDA(cudaGraphLaunch(s->graph_chunk, s->stream));
      s->steps += chunk;
      n -= chunk;
      continue;
    }
    // shorter runs (up to the next flux transform): the largest 2^k-step graph that fits
    const int room = s->flux.enabled ? s->flux.chunk - s->flux_pending : chunk;
    const int m = std::min(n, room);
    if (m >= 2) {
      if (!s->graph_pow[1] || s->pow_rec != s->rec || s->pow_rec_base != s->rec_base || s->pow_rec_cap != s->rec_cap)
        build_pow_graphs(s);
      int k = qd_session::N_POW_GRAPHS;
      while ((1 << k) > m) k--;
      QD_CUDA(cudaGraphLaunch(s->graph_pow[k], s->stream));
      s->steps += 1 << k;
      n -= 1 << k;
      if (s->flux.enabled && (s->flux_pending += 1 << k) == s->flux.chunk) flush_flux(s);
      continue;
    }
    enqueue_step(s, false);
    s->steps++;
    n--;
    if (s->flux.enabled && ++s->flux_pending == s->flux.chunk) flush_flux(s);
  }
}

static void download_psi(qd_session *s, qd_fh2data *const *problems, int n, cudaStream_t st) {
  const int64_t nth_pt = s->g.npt * s->g.nth;
  for (int p = 0; p < n; p++)
    theta_to_host(s, (int64_t)s->h_pblock0[p] * nth_pt, (int64_t)s->probs[p].n_omegas * nth_pt,
                  problems[p]->OmegaStates.wave_packets, st);
  QD_CUDA(cudaStreamSynchronize(st));
}

// P(E) of the accumulators (the flux transform of the buffered steps is already enqueued)
static void download_crp(qd_session *s, qd_fh2data *const *problems, int n) {
  if (!s->flux.enabled) return;
  const int nE = s->flux.n_energies;
  const int64_t ns = (int64_t)s->g.nth * s->g.n1;
  for (int p = 0; p < n; p++) {
    QD_CUDA(cudaMemcpyAsync(problems[p]->CRP.CRP, s->crp + (int64_t)p * nE, nE * sizeof(double),
                            cudaMemcpyDeviceToHost, s->stream));
    if (problems[p]->CRP.accumulators)
      QD_CUDA(cudaMemcpyAsync(problems[p]->CRP.accumulators, s->flux_acc + (int64_t)s->h_pblock0[p] * 2 * nE * ns,
                              (size_t)s->probs[p].n_omegas * 2 * nE * ns * sizeof(double2), cudaMemcpyDeviceToHost,
                              s->stream));
  }
  QD_CUDA(cudaStreamSynchronize(s->stream));
}

static void print_energies(qd_session *s, const std::vector<double> &e) {
  double total_module = 0.0, total_energy = 0.0;
  for (int b = 0; b < s->n_blocks; b++) {
    std::printf(" %d %.12f %.12f %.12f %.12f %.12f %.12f\n", s->h_blocks[b].omega, e[b * 6 + 0], e[b * 6 + 1],
                e[b * 6 + 2], e[b * 6 + 3], e[b * 6 + 4], e[b * 6 + 5]);
    total_module += e[b * 6 + 0];
    total_energy += e[b * 6 + 5];
  }
  std::printf(" Total: %.12f %.12f\n", total_module, total_energy);
}

// ------------------------------------------------------- session reuse
// One idle session per device is kept after a qd_evolve call for the next call
// with the same key (session_key): its buffers, key tables and step graph are
// reused and only the per-call inputs are loaded again (session_load).  A
// session whose device memory exceeds the limit (QD_SESSION_CACHE_BYTES, default
// 8 GiB; 0 turns reuse off) is released at the end of its call instead.
// qd_release_session_cache() releases the kept sessions.
constexpr int CACHE_DEVICES = 64;
static std::mutex g_cache_mutex;
static qd_session *g_cache[CACHE_DEVICES] = {};   // released by qd_release_session_cache, else at exit

static size_t cache_limit() {
  const char *e = std::getenv("QD_SESSION_CACHE_BYTES");
  if (e && *e) return (size_t)std::strtoull(e, nullptr, 10);
  return (size_t)8 << 30;
}

static std::unique_ptr<qd_session> acquire_session(qd_fh2data *const *problems, int n) {
  std::vector<ProblemHost> checked;
  validate_batch(problems, n, checked);   // before reading any array the key names
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < CACHE_DEVICES) {
    const std::vector<double> key = session_key(problems, n);
    std::unique_ptr<qd_session> hit;
    {
      std::lock_guard<std::mutex> lock(g_cache_mutex);
      if (g_cache[dev] && g_cache[dev]->key == key) {
        hit.reset(g_cache[dev]);
        g_cache[dev] = nullptr;
      }
    }
    if (hit) {
      session_load(hit.get(), problems, n, true);
      return hit;
    }
  }
  std::unique_ptr<qd_session> s(new qd_session());
  session_create(s.get(), problems, n);
  return s;
}

static void park_session(std::unique_ptr<qd_session> s) {
  const int dev = s->device;
  if (dev < 0 || dev >= CACHE_DEVICES || s->arena.total > cache_limit()) return;
  qd_session *old = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_cache_mutex);
    old = g_cache[dev];
    g_cache[dev] = s.release();
  }
  delete old;
}

static void release_session_cache() {
  std::vector<qd_session *> all;
  {
    std::lock_guard<std::mutex> lock(g_cache_mutex);
    for (qd_session *&c : g_cache)
      if (c) {
        all.push_back(c);
        c = nullptr;
      }
  }
  for (qd_session *c : all) {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(c->device);
    delete c;
    cudaSetDevice(cur);
  }
}

// The evolution loop of test_multiple_cards with callbacks and outputs.
static void evolve(qd_fh2data *const *problems, int n, qd_callback cb, void *user) {
  std::unique_ptr<qd_session> s = acquire_session(problems, n);
  const qd_fh2data *d0 = problems[0];
  const int total = d0->time.total_steps;
  const qd_options &op = d0->options;
  const bool want_rec = op.energies != nullptr;
  if (want_rec && total > 0) {
    const size_t need = (size_t)total * s->n_blocks * 6;
    if (s->rec_buf_cap < need) {
      s->rec_buf = s->alloc<double>(need);
      s->rec_buf_cap = need;
    }
    s->rec_cap = total;
    s->rec_base = s->steps;
    s->rec = s->rec_buf;
  }
  const int every = op.wave_to_matlab ? op.steps_to_copy_psi_from_device_to_host : 0;
  int done = 0;
  while (done < total) {
    // run until the next host-side event: callback step, print, or end
    int seg = total - done;
    if (op.print_energies) seg = 1;
    if (every > 0) {
      // callback fires after the step whose pre-increment counter is a multiple of `every`
      const int k = s->steps;   // counter value at the start of the next step
      const int next = ((k + every - 1) / every) * every;   // first counter >= k divisible by every
      seg = std::min(seg, next - k + 1);
    }
    const int before = s->steps;
    run_steps(s.get(), seg);
    done += seg;
    const int last = s->steps - 1;   // counter value of the last completed step
    const bool cb_now = every > 0 && last >= before && last % every == 0;
    // the status of the last segment is read by the end of the call, beside the downloads
    if (done < total || op.print_energies || cb_now) check_status(s.get());
    if (op.print_energies) {
      std::vector<double> e((size_t)s->n_blocks * 6);
      QD_CUDA(cudaMemcpy(e.data(), s->energies, e.size() * sizeof(double), cudaMemcpyDeviceToHost));
      std::printf("\n Step: %d\n", s->steps - 1);
      print_energies(s.get(), e);
    }
    if (cb_now) {
      download_psi(s.get(), problems, n, s->stream);
      for (int p = 0; p < n; p++) problems[p]->time.steps = last;
      if (cb) {
        for (int p = 0; p < n; p++)
          if (cb(problems[p], user) != 0) throw Error{QD_ERR_CALLBACK, "wave_to_matlab callback returned an error"};
      }
    }
  }
  // End of the call.  The download stream reads the status words once the steps are
  // done, while the main stream runs the flux transform of the buffered steps and
  // P(E); psi is copied out only when the status is clean, beside that transform.
  QD_CUDA(cudaEventRecord(s->ev_steps, s->stream));
  QD_CUDA(cudaStreamWaitEvent(s->stream_dl, s->ev_steps, 0));
  QD_CUDA(cudaMemcpyAsync(s->h_status, s->status, sizeof(int), cudaMemcpyDeviceToHost, s->stream_dl));
  QD_CUDA(cudaMemcpyAsync(s->h_status + 1, s->status_step, sizeof(int), cudaMemcpyDeviceToHost, s->stream_dl));
  if (s->flux.enabled) {
    flush_flux(s.get());
    launch_flux_crp(s->stream, s->g, s->flux, s->n_problems, s->d_pblock0, s->flux_acc, s->w, s->flux_eta, s->crp,
                    s->flux_fresh);
  }
  QD_CUDA(cudaStreamSynchronize(s->stream_dl));
  QD_CUDA(cudaGetLastError());
  if (s->h_status[0]) {
    QD_CUDA(cudaStreamSynchronize(s->stream));
    throw_status(s->h_status[0], s->h_status[1]);
  }
  download_psi(s.get(), problems, n, s->stream_dl);
  download_crp(s.get(), problems, n);
  for (int p = 0; p < n; p++) problems[p]->time.steps = s->steps;
  if (want_rec && total > 0) {
    std::vector<double> r((size_t)total * s->n_blocks * 6);
    QD_CUDA(cudaMemcpy(r.data(), s->rec, r.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int p = 0; p < n; p++) {
      double *out = problems[p]->options.energies;
      if (!out) continue;
      const int nb = s->probs[p].n_omegas, b0 = s->h_pblock0[p];
      for (int t = 0; t < total; t++)
        std::memcpy(out + ((size_t)t * nb) * 6, &r[((size_t)t * s->n_blocks + b0) * 6], (size_t)nb * 6 * sizeof(double));
    }
  }
  park_session(std::move(s));
}

// ---------------------------------------------------------------- C ABI
#define QD_GUARD(...)                                    \
  try {                                                  \
    qd::set_error("");                                   \
    __VA_ARGS__;                                         \
    return QD_OK;                                        \
  } catch (const qd::Error &e) {                         \
    qd::set_error(e.msg);                                \
    return e.status;                                     \
  } catch (const std::bad_alloc &) {                     \
    qd::set_error("host allocation failed");             \
    return QD_ERR_NOMEM;                                 \
  } catch (const std::exception &e) {                    \
    qd::set_error(e.what());                             \
    return QD_ERR_INVALID;                               \
  }

extern "C" {

int qd_version(void) { return QD_VERSION; }

const char *qd_last_error(void) { return qd::g_last_error.c_str(); }

int qd_evolve(qd_fh2data *data, qd_callback cb, void *user) {
  QD_GUARD({
    qd_fh2data *p[1] = {data};
    evolve(p, 1, cb, user);
  })
}

int qd_evolve_batch(qd_fh2data *const *problems, int32_t n_problems, qd_callback cb, void *user) {
  QD_GUARD(evolve(problems, n_problems, cb, user))
}

int qd_session_create(qd_fh2data *const *problems, int32_t n_problems, qd_session **out) {
  QD_GUARD({
    QD_REQUIRE(out != nullptr, "out != NULL");
    *out = nullptr;
    std::unique_ptr<qd_session> s(new qd_session());
    session_create(s.get(), problems, n_problems);
    *out = s.release();
  })
}

int qd_release_session_cache(void) { QD_GUARD(release_session_cache()) }

int qd_session_destroy(qd_session *s) {
  QD_GUARD(delete s)
}

int qd_session_run(qd_session *s, int32_t n_steps) {
  QD_GUARD({
    QD_REQUIRE(s && n_steps >= 0, "session && n_steps >= 0");
    run_steps(s, n_steps);
    QD_CUDA(cudaGetLastError());
  })
}

int qd_session_synchronize(qd_session *s) {
  QD_GUARD({
    QD_REQUIRE(s, "session");
    check_status(s);
  })
}

int qd_session_flush(qd_session *s) {
  QD_GUARD({
    QD_REQUIRE(s, "session");
    flush_flux(s);
    QD_CUDA(cudaGetLastError());
  })
}

int qd_session_download(qd_session *s, qd_fh2data *const *problems, int32_t n_problems) {
  QD_GUARD({
    QD_REQUIRE(s && problems && n_problems == s->n_problems, "session download: same problem count");
    check_status(s);
    download_psi(s, problems, n_problems, s->stream);
    if (s->flux.enabled) {
      flush_flux(s);
      launch_flux_crp(s->stream, s->g, s->flux, s->n_problems, s->d_pblock0, s->flux_acc, s->w, s->flux_eta, s->crp,
                    s->flux_fresh);
    }
    download_crp(s, problems, n_problems);
    for (int p = 0; p < n_problems; p++) problems[p]->time.steps = s->steps;
  })
}

int qd_session_upload(qd_session *s, qd_fh2data *const *problems, int32_t n_problems) {
  QD_GUARD({
    QD_REQUIRE(s && problems && n_problems == s->n_problems, "session upload: same problem count");
    const int64_t nth_pt = s->g.npt * s->g.nth;
    for (int p = 0; p < n_problems; p++)
      theta_from_host(s, (int64_t)s->h_pblock0[p] * nth_pt, (int64_t)s->probs[p].n_omegas * nth_pt,
                      problems[p]->OmegaStates.wave_packets);
  })
}

void *qd_session_stream(qd_session *s) { return s ? (void *)s->stream : nullptr; }

int qd_session_info(qd_session *s, int32_t *n_blocks, int32_t *launches_per_step) {
  QD_GUARD({
    QD_REQUIRE(s, "session");
    if (n_blocks) *n_blocks = s->n_blocks;
    if (launches_per_step) *launches_per_step = s->launches_per_step;
  })
}

int qd_session_apply(qd_session *s, int32_t stage, double dt) {
  QD_GUARD({
    QD_REQUIRE(s, "session");
    cudaStream_t st = s->stream;
    const Grid &g = s->g;
    double2 *tab = nullptr;
    auto scratch_tab = [&](int64_t n) {
      double2 *t = dalloc<double2>((size_t)n);
      return t;
    };
    switch (stage) {
      case QD_STAGE_DUMP: {
        if (!s->has_mask) break;
        tab = scratch_tab(g.npt * g.nth);
        std::vector<double> zero((size_t)g.npt * g.nth, 0.0);
        double *z = dupload(zero.data(), zero.size(), st);
        launch_build_theta_table(st, g, z, s->d1, s->d2, 0.0, tab);
        if (s->psi_thf)
          launch_theta_phase(st, s->psi_thf, tab, s->n_blocks, g.npt * g.nth, s->status);
        else
          launch_theta_phase(st, s->psi_th, tab, s->n_blocks, g.npt * g.nth, s->status);
        QD_CUDA(cudaStreamSynchronize(st));
        cudaFree(z);
        break;
      }
      case QD_STAGE_POTENTIAL:
        tab = scratch_tab(g.npt * g.nth);
        launch_build_theta_table(st, g, s->pot, nullptr, nullptr, dt, tab);
        if (s->psi_thf)
          launch_theta_phase(st, s->psi_thf, tab, s->n_blocks, g.npt * g.nth, s->status);
        else
          launch_theta_phase(st, s->psi_th, tab, s->n_blocks, g.npt * g.nth, s->status);
        break;
      case QD_STAGE_FORWARD_LEGENDRE:
        if (s->precision == QD_PRECISION_MIXED)
          launch_legendre_tc_fwd(st, g, s->psi_thf, s->psi_jf, s->d_blocks, s->n_blocks, s->img_f, s->imgoff_f, nullptr,
                                 nullptr, nullptr, s->smem_f, s->status, s->status, s->bscale_f, s->max_nl);
        else
          launch_legendre_fwd_f64(st, g, s->psi_th, s->psi_j, s->Bf, s->d_blocks, s->n_blocks, s->max_nl, nullptr,
                                  nullptr, s->status);
        break;
      case QD_STAGE_BACKWARD_LEGENDRE:
        if (s->precision == QD_PRECISION_MIXED)
          launch_legendre_tc_bwd(st, g, s->psi_jf, s->psi_thf, s->d_blocks, s->n_blocks, s->img_b, s->imgoff_b, s->wf,
                                 s->wvf, s->part_modpe, s->t_modpe, s->smem_b, s->status, s->status, s->bscale_b, s->max_nl);
        else
          launch_legendre_bwd_f64(st, g, s->psi_j, s->psi_th, s->Bb, s->d_blocks, s->n_blocks, nullptr, s->w, s->pot,
                                  s->part_modpe, s->t_modpe, s->status);
        break;
      case QD_STAGE_ROTATIONAL:
        tab = scratch_tab(g.npt * (g.l_max + 1));
        launch_build_rot_table(st, g, dt, tab);
        if (s->psi_jf)
          launch_slab_phase(st, s->psi_jf, tab, s->d_slabs, s->n_slabs, g.npt, s->status);
        else
          launch_slab_phase(st, s->psi_j, tab, s->d_slabs, s->n_slabs, g.npt, s->status);
        break;
      case QD_STAGE_CORIOLIS:
      case QD_STAGE_CORIOLIS_ENERGY: {
        if (!s->any_coupled) break;
        double2 *ph = dalloc<double2>((size_t)s->h_groups.back().ph0 + (size_t)s->h_groups.back().n * g.n1);
        launch_build_coriolis_phase(st, g, s->d_groups, s->n_groups, s->max_group_n, s->cor_e, dt, ph);
        const bool en = stage == QD_STAGE_CORIOLIS_ENERGY;
        float2 *phl = nullptr;
        if (s->cor_f32) {
          phl = dalloc<float2>((size_t)s->h_groups.back().ph0 + (size_t)s->h_groups.back().n * g.n1);
          launch_build_coriolis_lift(st, g, s->d_groups, s->n_groups, s->cor_e, dt, phl);
          launch_coriolis_f32(st, g, s->psi_jf, s->d_blocks, s->d_groups, s->cor_order, s->n_groups,
                        s->max_group_n, s->cor_Vh,
                              s->cor_Vl, phl, s->cor_H, nullptr, nullptr, false, false, s->I1f, s->I2f,
                              en ? s->part_ce : nullptr, nullptr, s->t_ce, s->status);
        } else if (s->psi_jf)
          launch_coriolis(st, g, s->psi_jf, s->d_blocks, s->d_groups, s->n_groups, s->max_group_n, s->cor_V, ph,
                          s->cor_H, en ? s->part_ce : nullptr, s->t_ce, nullptr, s->status);
        else
          launch_coriolis(st, g, s->psi_j, s->d_blocks, s->d_groups, s->n_groups, s->max_group_n, s->cor_V, ph,
                          s->cor_H, en ? s->part_ce : nullptr, s->t_ce, nullptr, s->status);
        if (en) {
          EnergyParts ep = energy_parts(s, false, false, false, true);
          launch_energy_finalize2(st, g, ep, s->d_blocks, s->d_pblock0, s->n_problems, s->d_groups, s->d_pgroup0,
                                  s->max_group_n, s->energies, nullptr, s->d_step, 0, 0, 1e300, s->status,
                                  s->status_step, s->n_blocks, s->step_done);
        }
        QD_CUDA(cudaStreamSynchronize(st));
        cudaFree(ph);
        if (phl) cudaFree(phl);
        break;
      }
      case QD_STAGE_FFT_KINETIC: {
        tab = scratch_tab(g.npt);
        launch_build_kin_table(st, g, s->T1, s->T2, dt, tab);
        FFTLift lf{};
        float2 *kR = nullptr, *kr = nullptr;
        if (s->precision == QD_PRECISION_MIXED) {
          kR = dalloc<float2>((size_t)g.n1);
          kr = dalloc<float2>((size_t)g.n2);
          launch_build_lift_kin(st, g.n1, s->T1, dt, kR);
          launch_build_lift_kin(st, g.n2, s->T2, dt, kr);
          lf.kinR = kR;
          lf.kinr = kr;
          lf.T1f = s->T1f;
          lf.T2f = s->T2f;
          lf.I1f = s->I1f;
          lf.I2f = s->I2f;
        }
        if (s->psi_jf)
          launch_fft_kinetic(st, g, s->fft, s->psi_jf, s->d_slabs, s->n_slabs, s->part_ke, nullptr, s->status, &lf);
        else
          launch_fft_kinetic(st, g, s->fft, s->psi_j, s->d_slabs, s->n_slabs, tab, s->T1, s->T2, s->part_ke, nullptr,
                             nullptr, s->status);
        QD_CUDA(cudaStreamSynchronize(st));
        if (kR) cudaFree(kR);
        if (kr) cudaFree(kr);
        EnergyParts ep = energy_parts(s, false, true, false, false);
        launch_energy_finalize2(st, g, ep, s->d_blocks, s->d_pblock0, s->n_problems, s->d_groups, s->d_pgroup0,
                                s->max_group_n, s->energies, nullptr, s->d_step, 0, 0, 1e300, s->status,
                                s->status_step, s->n_blocks, s->step_done);
        break;
      }
      case QD_STAGE_ENERGIES: {
        const int t_re_saved = s->t_re;
        if (s->psi_jf)
          launch_rot_energy(st, g, s->psi_jf, s->d_slabs, s->n_slabs, s->part_re, s->t_re, s->status);
        else
          launch_rot_energy(st, g, s->psi_j, s->d_slabs, s->n_slabs, s->part_re, s->t_re, s->status);
        // module and potential energy come from a backward contraction into psi_theta
        EnergyParts ep = energy_parts(s, true, false, true, false);
        ep.re_tiles = t_re_saved;
        launch_energy_finalize2(st, g, ep, s->d_blocks, s->d_pblock0, s->n_problems, s->d_groups, s->d_pgroup0,
                                s->max_group_n, s->energies, nullptr, s->d_step, 0, 0, 1e300, s->status,
                                s->status_step, s->n_blocks, s->step_done);
        break;
      }
      case QD_STAGE_FLUX: {
        QD_REQUIRE(s->flux.enabled, "CRP.calculate_CRP");
        k_flux_begin<<<1, 1, 0, st>>>(s->d_step, s->flux_count, s->flux_t0, s->dt, s->flux_slot, s->flux.chunk,
                                  s->status);
        const int64_t ns = (int64_t)g.nth * g.n1;
        dim3 grid((unsigned)std::min<int64_t>((ns + 255) / 256, 64), (unsigned)s->n_blocks);
        if (s->psi_thf)
          launch_flux_extract_f32(st, g, s->flux, s->psi_thf, s->n_blocks, s->half_v_lift, s->fdf, s->flux_buf_f,
                                  s->flux_slot, s->status);
        else
          k_flux_extract_dev<<<grid, 256, 0, st>>>(g, s->flux.n_grad, s->flux.n_ds, s->psi_th, s->half_v, s->fd,
                                                   s->flux_buf, s->n_blocks, s->flux_slot, s->status);
        k_step_end<<<1, 1, 0, st>>>(s->d_step, s->status, nullptr, nullptr, 0.0, 0);
        s->steps++;
        if (++s->flux_pending == s->flux.chunk) flush_flux(s);
        break;
      }
      default:
        throw Error{QD_ERR_INVALID, "unknown stage"};
    }
    QD_CUDA(cudaStreamSynchronize(st));
    if (tab) cudaFree(tab);
    QD_CUDA(cudaGetLastError());
  })
}

int qd_session_get_psi(qd_session *s, int32_t which, int32_t block, double *host_out, size_t n_doubles) {
  QD_GUARD({
    QD_REQUIRE(s && host_out && block >= 0 && block < s->n_blocks, "session, block");
    const BlockDesc &bd = s->h_blocks[block];
    const size_t n = which == 0 ? (size_t)s->g.npt * s->g.nth : (size_t)s->g.npt * bd.nl;
    QD_REQUIRE(n_doubles == 2 * n, "buffer size");
    QD_CUDA(cudaStreamSynchronize(s->stream));
    if (which == 0) {
      theta_to_host(s, (int64_t)block * n, (int64_t)n, host_out, s->stream);
      QD_CUDA(cudaStreamSynchronize(s->stream));
    } else if (s->psi_jf) {   // mixed form: c64 pool, widened exactly
      std::vector<float2> tmp(n);
      QD_CUDA(cudaMemcpy(tmp.data(), s->psi_jf + (int64_t)bd.slab0 * s->g.npt, n * sizeof(float2),
                         cudaMemcpyDeviceToHost));
      for (size_t q = 0; q < n; q++) {
        host_out[2 * q] = tmp[q].x;
        host_out[2 * q + 1] = tmp[q].y;
      }
    } else {
      QD_CUDA(cudaMemcpy(host_out, s->psi_j + (int64_t)bd.slab0 * s->g.npt, n * sizeof(double2),
                         cudaMemcpyDeviceToHost));
    }
  })
}

int qd_session_set_psi(qd_session *s, int32_t which, int32_t block, const double *host_in, size_t n_doubles) {
  QD_GUARD({
    QD_REQUIRE(s && host_in && block >= 0 && block < s->n_blocks, "session, block");
    const BlockDesc &bd = s->h_blocks[block];
    const size_t n = which == 0 ? (size_t)s->g.npt * s->g.nth : (size_t)s->g.npt * bd.nl;
    QD_REQUIRE(n_doubles == 2 * n, "buffer size");
    QD_CUDA(cudaStreamSynchronize(s->stream));
    if (which == 0) {
      theta_from_host(s, (int64_t)block * n, (int64_t)n, host_in);
      QD_CUDA(cudaStreamSynchronize(s->stream));
    } else if (s->psi_jf) {   // mixed form: c64 pool, rounded to nearest
      std::vector<float2> tmp(n);
      for (size_t q = 0; q < n; q++) tmp[q] = make_float2((float)host_in[2 * q], (float)host_in[2 * q + 1]);
      QD_CUDA(cudaMemcpy(s->psi_jf + (int64_t)bd.slab0 * s->g.npt, tmp.data(), n * sizeof(float2),
                         cudaMemcpyHostToDevice));
    } else {
      QD_CUDA(cudaMemcpy(s->psi_j + (int64_t)bd.slab0 * s->g.npt, host_in, n * sizeof(double2),
                         cudaMemcpyHostToDevice));
    }
  })
}

int qd_session_profile(qd_session *s, int32_t n_steps, char *names, size_t names_cap, double *avg_ms,
                       int32_t *launches_per_step, int32_t max_kernels, int32_t *n_kernels) {
  Profiler prof;
  struct Reset {
    Profiler *p;
    ~Reset() {
      g_prof = nullptr;
      if (p->start) cudaEventDestroy(p->start);
      for (cudaEvent_t e : p->ev) cudaEventDestroy(e);
    }
  } reset{&prof};
  QD_GUARD({
    QD_REQUIRE(s && n_steps > 0 && names && avg_ms && launches_per_step && n_kernels, "profile arguments");
    QD_CUDA(cudaStreamSynchronize(s->stream));
    flush_flux(s);
    QD_CUDA(cudaEventCreate(&prof.start));
    QD_CUDA(cudaEventRecord(prof.start, s->stream));
    g_prof = &prof;
    for (int i = 0; i < n_steps; i++) {
      enqueue_step(s, false);
      s->steps++;
      if (s->flux.enabled && ++s->flux_pending == s->flux.chunk) flush_flux(s);
    }
    g_prof = nullptr;
    check_status(s);
    std::vector<std::string> order;
    std::vector<double> tot;
    std::vector<int> cnt;
    cudaEvent_t prev = prof.start;
    for (size_t i = 0; i < prof.ev.size(); i++) {
      float ms = 0;
      QD_CUDA(cudaEventElapsedTime(&ms, prev, prof.ev[i]));
      prev = prof.ev[i];
      size_t k = 0;
      while (k < order.size() && order[k] != prof.names[i]) k++;
      if (k == order.size()) {
        order.push_back(prof.names[i]);
        tot.push_back(0.0);
        cnt.push_back(0);
      }
      tot[k] += ms;
      cnt[k] += 1;
    }
    QD_REQUIRE((int)order.size() <= max_kernels, "max_kernels too small");
    std::string joined;
    for (size_t k = 0; k < order.size(); k++) {
      avg_ms[k] = tot[k] / cnt[k];
      launches_per_step[k] = cnt[k];
      joined += order[k];
      if (k + 1 < order.size()) joined += "\n";
    }
    QD_REQUIRE(joined.size() + 1 <= names_cap, "names buffer too small");
    std::memcpy(names, joined.c_str(), joined.size() + 1);
    *n_kernels = (int32_t)order.size();
  })
}

int qd_device_fma_peaks(double *fp64_tflops, double *fp32_tflops) {
  QD_GUARD({
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) throw Error{QD_ERR_NO_DEVICE, "no CUDA device"};
    if (fp64_tflops) *fp64_tflops = measure_fp64_tflops();
    if (fp32_tflops) *fp32_tflops = measure_fp32_tflops();
  })
}

int qd_session_tuning(qd_session *s, char *text, size_t text_cap) {
  QD_GUARD({
    QD_REQUIRE(s && text && text_cap > s->tuning.size(), "session, text buffer large enough");
    std::memcpy(text, s->tuning.c_str(), s->tuning.size() + 1);
  })
}

int qd_device_dmma_peak(double *fp64_tensor_tflops) {
  QD_GUARD({
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) throw Error{QD_ERR_NO_DEVICE, "no CUDA device"};
    QD_REQUIRE(fp64_tensor_tflops, "fp64_tensor_tflops");
    *fp64_tensor_tflops = measure_dmma_tflops();
  })
}

int qd_device_wait_selftest(double budget_ms, int32_t arrive) {
  QD_GUARD({
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) throw Error{QD_ERR_NO_DEVICE, "no CUDA device"};
    device_wait_selftest(budget_ms, arrive);
  })
}

int qd_session_get_energies(qd_session *s, double *host_out, size_t n_doubles) {
  QD_GUARD({
    QD_REQUIRE(s && host_out && n_doubles == (size_t)s->n_blocks * 6, "session, buffer size");
    QD_CUDA(cudaStreamSynchronize(s->stream));
    QD_CUDA(cudaMemcpy(host_out, s->energies, n_doubles * sizeof(double), cudaMemcpyDeviceToHost));
  })
}

}  // extern "C"
