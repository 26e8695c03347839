// Internal declarations shared by the host engine and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>

#include "../../include/qd.h"

namespace qd {

// ------------------------------------------------------------------ errors
void set_error(const std::string &msg);
struct Error {
  int status;
  std::string msg;
};

#define QD_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      throw ::qd::Error{e_ == cudaErrorMemoryAllocation ? QD_ERR_NOMEM : QD_ERR_CUDA,   \
                        std::string(#call) + ": " + cudaGetErrorString(e_)};            \
  } while (0)

#define QD_REQUIRE(cond, msg)                                                           \
  do {                                                                                  \
    if (!(cond)) throw ::qd::Error{QD_ERR_INVALID, std::string("insist failed: ") + (msg)}; \
  } while (0)

// ------------------------------------------------------------- device data
// One Omega block (one helicity of one total-J problem).
struct BlockDesc {
  int32_t problem;
  int32_t omega;
  int32_t nl;      // l_max - omega + 1 Legendre slabs
  int32_t slab0;   // global index of its first Legendre slab
  int64_t bmat0;   // offset (doubles) of its Legendre matrices in the B pools
};

// Legendre-space slab: one (block, l) pair, n1*n2 complex values.
struct SlabDesc {
  int32_t block;
  int32_t l;
};

// One Coriolis coupling group: a fixed l of one problem, coupling the
// blocks with omega in [omega_lo, omega_hi].
struct CoriolisGroup {
  int32_t l;
  int32_t n;          // omega_hi - omega_lo + 1
  int32_t block_lo;   // block index of omega_lo
  int32_t omega_lo;
  int64_t v0;         // offset (double) of the eigenvectors V[n][n] (V[p*n+a] = component p of vector a)
  int64_t e0;         // offset (double) of the eigenvalues e[n]
  int64_t ph0;        // offset (double2) of exp(-i dt e_a/(2 m1 R_i^2)) as ph[a][n1]
  int64_t h0;         // offset (double) of the matrix H[n][n] (coupling energy)
};

struct FluxConfig {
  int enabled;
  int n_energies;
  int n_grad;
  int n_ds;
  int chunk;           // steps buffered between time-to-energy transforms
};

enum { E_MODULE = 0, E_POTENTIAL = 1, E_KINETIC = 2, E_ROTATIONAL = 3, E_CORIOLIS = 4, E_TOTAL = 5 };

// --------------------------------------------------------------- profiling
// When a profiler is active on this thread, every launch wrapper records a
// named CUDA event on its stream right after the launch.
void prof_mark(cudaStream_t s, const char *name);
double measure_fp64_tflops();
double measure_dmma_tflops();
void device_wait_selftest(double budget_ms, int arrive);
double measure_fp32_tflops();

// ------------------------------------------------------------ kernel API
// All launches take the session stream.  Pointers are device pointers.
struct Grid {
  int n1, n2, nth, l_max;
  int64_t npt;          // n1*n2
  double dr1, dr2, m1, m2, left1, left2;
};

// theta-space phase: psi[b][k][j][i] *= tab[k][j][i] for every block; psi c128 or c64
template <typename S>
void launch_theta_phase(cudaStream_t s, S *psi, const double2 *tab, int n_blocks, int64_t n_per_block,
                        const int *status);
// c64 -> c128 (exact) and c128 -> c64 (round to nearest) element copies
void launch_widen(cudaStream_t s, const float2 *src, double2 *dst, int64_t n);
void launch_narrow(cudaStream_t s, const double2 *src, float2 *dst, int64_t n);

// j-space phase: slab s (l = slabs[s].l) *= tab[l][j][i]; psi_j c128 or c64
template <typename S>
void launch_slab_phase(cudaStream_t s, S *psi_j, const double2 *tab, const SlabDesc *slabs, int n_slabs,
                       int64_t npt, const int *status);

// FP64 Legendre contractions (SIMT DFMA).
// forward: psi_j(slab0_b+n) = sum_k wP_b[k][n] (tabA[k] * psi_th[b][k]);  tabA may be null;
//          epilogue multiplies by tabE[l] (may be null)
void launch_legendre_fwd_f64(cudaStream_t s, const Grid &g, const double2 *psi_th, double2 *psi_j,
                             const double *Bfwd, const BlockDesc *blocks, int n_blocks, int max_nl,
                             const double2 *tabA, const double2 *tabE, const int *status);
// backward: psi_th[b][k] = sum_n P_b[n][k] (tabA[l] * psi_j(slab0_b+n)); tabA may be null.
//           partial sums of module and potential energy per CTA -> part[b][tile][2]
void launch_legendre_bwd_f64(cudaStream_t s, const Grid &g, const double2 *psi_j, double2 *psi_th,
                             const double *Bbwd, const BlockDesc *blocks, int n_blocks,
                             const double2 *tabA, const double *w, const double *pot,
                             double *part, int n_part_tiles, const int *status);
int legendre_bwd_part_tiles(const Grid &g);

// 2-D FFT over (R, r) of every Legendre slab with the kinetic phase between
// the passes.  precision: 0 = FP64 butterflies, 1 = FP32 butterflies.
constexpr int FFT_MAX_CANDIDATES = 12;
constexpr int FFT_THREE_PASS = 0, FFT_CLUSTER = 1, FFT_SEP0 = 2;
struct FFTPlan {
  int n1, n2;
  int rad1[16], nst1;
  int rad2[16], nst2;
  double2 *tw1_d;  float2 *tw1_f;   // exp(-2 pi i t / n1), t < n1
  double2 *tw2_d;  float2 *tw2_f;
  int rows_per_cta;
  int cols_per_cta;
  int cluster;   // CTAs per slab of the single-pass FP32 FFT (0: three-pass form)
  int sep;           // shape index of the separable single-pass FP32 FFT, -1: none
  int sep_ke_tiles;  // its kinetic-energy partials per slab
  int sep_re_tiles;  // its rotational-energy partials per slab
  int use_cluster;   // the two-exchange cluster kernel is the mixed form's FFT
  // mixed-form FFT kernels that fit this grid (FFT_SEP0 + shape, FFT_CLUSTER,
  // FFT_THREE_PASS) and the one in use (fft_plan_choose; the autotuner times them)
  int cand[FFT_MAX_CANDIDATES];
  int n_cand;
  int choice;
};
void fft_plan_choose(FFTPlan &p, int choice);
std::string fft_choice_name(int choice);
int fft_max_tiles(const FFTPlan &p);
int fft_mixed_launches(const FFTPlan &p);
// FP32 three-shear phase tables of the mixed form (float2 (t, s) per entry,
// see lift tables below); null entries are skipped.
struct FFTLift {
  const float2 *proR, *pror;   // [l][n1], [l][n2]: rotational phase before the forward transform
  const float2 *epiR, *epir;   // after the inverse transform
  const float2 *kinR, *kinr;   // [n1], [n2]: kinetic phase
  const float *T1f, *T2f;      // kinetic energy tables in FP32
  const float *I1f, *I2f;      // 1/(2 m R^2), 1/(2 m r^2) in FP32 (rotational energy)
};
bool fft_factor(int n, int *rad, int *nst);
void fft_plan_init(FFTPlan &p, int n1, int n2);
void fft_plan_free(FFTPlan &p);
// FP64 form: forward rows -> cols (fwd, kinetic, KE partials, inv) -> rows
// inverse with scale 1/(n1 n2) and the epilogue phase tabE (may be null) and
// rotational energy partials (when re_part is non-null).
void launch_fft_kinetic(cudaStream_t s, const Grid &g, const FFTPlan &p, double2 *psi_j, const SlabDesc *slabs,
                        int n_slabs, const double2 *tab_kin, const double *T1, const double *T2, double *ke_part,
                        const double2 *tabE, double *re_part, const int *status);
// Mixed form: FP32 transforms on the c64 psi_j pool with the three-shear phases
// of lift (kinetic, and the rotational phase before/after when set).
void launch_fft_kinetic(cudaStream_t s, const Grid &g, const FFTPlan &p, float2 *psi_j, const SlabDesc *slabs,
                        int n_slabs, double *ke_part, double *re_part, const int *status, const FFTLift *lift);
int fft_col_tiles(const FFTPlan &p, int precision);
int fft_row_tiles(const FFTPlan &p, int precision);

// rotational energy partials only (for stage-by-stage use)
template <typename S>
void launch_rot_energy(cudaStream_t s, const Grid &g, const S *psi_j, const SlabDesc *slabs, int n_slabs,
                       double *re_part, int tiles, const int *status);

// Coriolis: in-place psi_l^Omega <- sum_Omega1 U_l[Omega][Omega1](R) psi_l^Omega1 per group,
// optional coupling-energy partials per block (computed on the input psi),
// optional epilogue phase tabE[l] (may be null).
// psi_j is double2 (FP64 form) or float2 (mixed form; arithmetic stays FP64).
template <typename S>
void launch_coriolis(cudaStream_t s, const Grid &g, S *psi_j, const BlockDesc *blocks,
                     const CoriolisGroup *groups, int n_groups, int max_n, const double *V,
                     const double2 *ph, const double *H, double *ce_part, int ce_tiles,
                     const double2 *tabE, const int *status, const double2 *tabP = nullptr);
void launch_build_coriolis_phase(cudaStream_t s, const Grid &g, const CoriolisGroup *groups, int n_groups,
                                 int max_n, const double *e, double dt, double2 *ph);
int coriolis_tiles(const Grid &g);
constexpr int CORIOLIS_THREADS = 128;    // points per CTA of the Coriolis kernels
// one FP64 kernel variant for groups of at most MAXN blocks (instantiated in k_coriolis_fp64_*.cu)
template <int MAXN, typename S>
void launch_coriolis_n(cudaStream_t s, const Grid &g, S *psi_j, const BlockDesc *blocks, const CoriolisGroup *groups,
                       int n_groups, int max_n, const double *V, const double2 *ph, const double *H, double *ce_part,
                       int ce_tiles, const double2 *tabE, const int *status, const double2 *tabP);
// Mixed form (FP32 arithmetic, c64 pool, at most CORIOLIS_F32_MAXN coupled
// blocks): V = Vh + Vl as FP32 pairs, phases as three-shear coefficients
// (phl from launch_build_coriolis_lift; rotR/rotr the dt/4 rotational phase,
// applied before when pro, after when epi); optional coupling-energy partials
// [group][omega][tiles] and rotational-energy partials [slab][tiles] of the
// outgoing state.
constexpr int CORIOLIS_F32_MAXN = 24;
constexpr int CORIOLIS_F32_STEP = 4;     // size classes of at most 4, 8, ..., 24 blocks (one body each)
constexpr int CORIOLIS_F32_CLASSES = 6;
constexpr int CORIOLIS_F32_TILES = 16;   // CTAs per group (its partial tiles), doubled below
constexpr int CORIOLIS_F32_FEW_GROUPS = 512;   // ... this many groups
int coriolis_f32_class(int n);           // size class of a group of n blocks, -1 above the limit
// order: the group indices, largest groups first
void launch_coriolis_f32(cudaStream_t s, const Grid &g, float2 *psi_j, const BlockDesc *blocks,
                         const CoriolisGroup *groups, const int *order, int n_groups, int max_n, const float *Vh,
                         const float *Vl, const float2 *phl, const double *H, const float2 *rotR, const float2 *rotr,
                         bool pro, bool epi, const float *I1f, const float *I2f, double *ce_part, double *re_part,
                         int tiles, const int *status);
void launch_build_coriolis_lift(cudaStream_t s, const Grid &g, const CoriolisGroup *groups, int n_groups,
                                const double *e, double dt, float2 *phl);

// Energy finalisation: sums partial arrays per block in a fixed order,
// writes energies[b][6] (and rec if non-null), applies the norm guard.
struct EnergyParts {
  const double *mod_pe;  int mod_pe_tiles;    // [b][tiles][2]
  const double *ke;      int ke_tiles;        // [slab][tiles]
  const double *re;      int re_tiles;        // [slab][tiles]
  const double *ce;      int ce_tiles;        // [b][tiles]
  int have_ke, have_re, have_ce, have_mod;
  double ke_scale;   // dr1 dr2 / (n1 n2): kinetic partials are sums over the unnormalised spectrum
};
// End-of-step bookkeeping done by the last CTA of the energy finalisation:
// flux slot and t0 of this step (when flux_count is set) and the step counter.
struct StepTail {
  unsigned *done;      // non-null: advance the step (end of a full step)
  int *flux_count, *flux_slot;
  double *flux_t0;
  int cap;
  double dt;
};
// With fx (mixed form, end of a full step) the surface extraction runs in the
// same launch (k_step_tail_mixed); fx is defined in qd_tail.cuh.
struct FluxTileArgs;
void launch_energy_finalize2(cudaStream_t st, const Grid &g, const EnergyParts &ep, const BlockDesc *blocks,
                             const int *pblock0, int n_problems, const CoriolisGroup *groups, const int *pgroup0,
                             int ce_n, double *energies, double *rec, const int *d_step, int rec_base, int rec_cap,
                             double norm_tol, int *status, int *status_step, int n_blocks, unsigned *done,
                             const StepTail *tail = nullptr, const FluxTileArgs *fx = nullptr);
void launch_build_half_v_lift(cudaStream_t s, const Grid &g, const FluxConfig &f, const double *pot, double dt,
                              float2 *half_v);
void launch_flux_extract_f32(cudaStream_t s, const Grid &g, const FluxConfig &f, const float2 *psi_th,
                             int n_blocks, const float2 *half_v, const float *fd, float2 *buf, const int *slot,
                             const int *status);

// flux: extract surface values (A, dA/dr) into buf[slot], then DFT chunks
void launch_flux_extract(cudaStream_t s, const Grid &g, const FluxConfig &f, const double2 *psi_th,
                         int n_blocks, const double2 *half_v, const double *fd, double2 *buf, int slot,
                         const int *status);
void launch_flux_dft(cudaStream_t s, const Grid &g, const FluxConfig &f, int n_blocks, const double2 *buf,
                     int count, const double *energies, double t0, double dt, double2 *phase_scratch,
                     double2 *acc, const int *status);
void launch_flux_dft_f32(cudaStream_t s, int64_t ns2, int nE, int n_blocks, const int *count_p, int cap,
                         const float2 *buf, const double2 *phase, double2 *acc, const int *status, const int *fresh);
void launch_flux_crp(cudaStream_t s, const Grid &g, const FluxConfig &f, int n_problems,
                     const int *block0_of_problem, const double2 *acc, const double *w, const double *eta_sq,
                     double *crp, const int *fresh);

// table builders (FP64 on the device)
void launch_build_theta_table(cudaStream_t s, const Grid &g, const double *pot, const double *d1,
                              const double *d2, double dt, double2 *tab);
void launch_build_rot_table(cudaStream_t s, const Grid &g, double dt, double2 *tab);
void launch_build_kin_table(cudaStream_t s, const Grid &g, const double *T1, const double *T2, double dt,
                            double2 *tab);
// Lifting tables: entry = (-tan(a/4), sin(a/2)) of the rotation angle a =
// -scale * f (reduced to (-pi, pi]), applied as two half-angle three-shear
// rotations.
//   theta:  f = V[k][p] (with scale dt)                      -> [nth][npt]
//   rot:    f = l(l+1)/(2 m R^2) per coordinate              -> [l_max+1][n]
//   kin:    f = T[i]                                          -> [n]
void launch_build_lift_theta(cudaStream_t s, const Grid &g, const double *pot, double dt, float2 *out);
void launch_build_lift_rot(cudaStream_t s, int n, int l_max, double left, double dr, double mass, double dt,
                           float2 *out);
void launch_build_lift_kin(cudaStream_t s, int n, const double *T, double dt, float2 *out);
void launch_build_float_tables(cudaStream_t s, const Grid &g, const double *w, const double *pot, const double *d1,
                               const double *d2, const double *T1, const double *T2, float *wf, float *wvf,
                               float *d1f, float *d2f, float *T1f, float *T2f, float *I1f, float *I2f);

// tcgen05 BF16x3 Legendre contraction
struct TcArgs;
size_t tc_ws_smem_bytes(bool fwd, int kp_max, int np_max);
bool tc_shape_ok(bool fwd, int Kp, int Np);
void tc_set_smem_limit(size_t bytes);
void launch_build_tc_bimage(cudaStream_t s, const BlockDesc *blocks, int n_blocks, const double *Bsrc, int nth,
                            bool fwd, const int64_t *img_off, uint16_t *img, float *bscale, int max_np);
void launch_legendre_tc_fwd(cudaStream_t s, const Grid &g, const float2 *psi_th, float2 *psi_j,
                            const BlockDesc *blocks, int n_blocks, const uint16_t *img, const int64_t *img_off,
                            const float2 *vph, const float *d1f, const float *d2f, size_t smem, const int *status,
                            int *status_w, const float *bscale, int max_nl);
void launch_legendre_tc_bwd(cudaStream_t s, const Grid &g, const float2 *psi_j, float2 *psi_th,
                            const BlockDesc *blocks, int n_blocks, const uint16_t *img, const int64_t *img_off,
                            const float *wf, const float *wvf, double *part, int n_part_tiles, size_t smem,
                            const int *status, int *status_w, const float *bscale, int max_nl);
int legendre_tc_part_tiles(const Grid &g);
int legendre_tc_part_slots(const Grid &g, int max_nl);

void launch_build_half_v(cudaStream_t s, const Grid &g, const FluxConfig &f, const double *pot, double dt,
                         double2 *half_v);

}  // namespace qd
