/*
 * qd.h - C ABI of the GB300 split-operator wavepacket propagator.
 *
 * Drop-in boundary for the reference's MATLAB entry point
 *   void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
 * (cudaOpenMPEvolution.C:15-79), invoked from MATLAB as
 * cudaOpenMPEvolution(FH2Data) (FH2main.m:213).  The structs below carry the
 * same fields, with the same names, types and column-major layouts, as the
 * MATLAB struct the reference unmarshals (matlabStructures.C:17-153).  All
 * array pointers are borrowed caller memory; the library never frees them.
 * Outputs are written in place, as in the reference: the Omega wave packets
 * (omegawavepacket.cu:271-280), time.steps (matlabStructures.C:42) and
 * CRP.CRP.
 *
 * Every entry point returns a qd_status; none calls exit().  The text of the
 * last error of the calling thread is available from qd_last_error().
 * Plain C: no CUDA or C++ types appear in any signature.
 */
#ifndef QD_H
#define QD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QD_VERSION 10000 /* 1.0.0 */

typedef enum qd_status {
  QD_OK = 0,
  QD_ERR_INVALID = 1,     /* malformed input (the reference's insist() failures) */
  QD_ERR_CUDA = 2,        /* CUDA runtime / driver error */
  QD_ERR_NOMEM = 3,       /* device or host allocation failed */
  QD_ERR_NORM = 4,        /* norm guard: total module > 1 (cudaOpenMP2.cu:437-440) */
  QD_ERR_CALLBACK = 5,    /* the wave_to_matlab callback returned non-zero */
  QD_ERR_UNSUPPORTED = 6, /* valid input the library does not handle (e.g. odd FFT grid) */
  QD_ERR_NO_DEVICE = 7,   /* no CUDA device, or not an sm_103 device */
  QD_ERR_TIMEOUT = 8      /* a bounded device-side wait gave up (a kernel's
                             pipeline stalled); the context stays usable */
} qd_status;

typedef enum qd_precision {
  QD_PRECISION_FP64 = 0,  /* every stage in FP64 */
  QD_PRECISION_MIXED = 1  /* Legendre contraction as an exact 3-term BF16 split on
                             tensor cores, FFT, phases and Coriolis in FP32 (phases
                             as determinant-1 rotations), wave packets held as
                             complex64 on the device; tables, norms, energies and
                             flux accumulators in FP64.  Inputs and outputs stay
                             complex128. */
} qd_precision;

/* r1 (R) and r2 (r): matlabStructures.C:17-23 */
typedef struct qd_radial_coordinate {
  int32_t n;
  double left;
  double dr;
  double mass;
} qd_radial_coordinate;

/* theta: matlabStructures.C:25-37.  associated_legendre is (m+1) x n, parsed
   but not used by the time step (as in the reference). */
typedef struct qd_angle_coordinate {
  int32_t n;
  int32_t m;
  const double *x;
  const double *w;
  const double *associated_legendre;
} qd_angle_coordinate;

/* time: matlabStructures.C:39-44.  steps is in/out. */
typedef struct qd_evolution_time {
  int32_t total_steps;
  double time_step;
  int32_t steps;
} qd_evolution_time;

/* options: matlabStructures.C:46-58, plus optional extensions after
   use_p2p_async (zero-initialise to get the reference's behaviour). */
typedef struct qd_options {
  const char *wave_to_matlab; /* callback is invoked only when non-NULL */
  const char *test_name;
  int32_t steps_to_copy_psi_from_device_to_host;
  int32_t use_p2p_async;      /* accepted and ignored: one GPU, no peer copies */
  /* extensions */
  int32_t precision;          /* qd_precision */
  int32_t print_energies;     /* 1: print per-step energies like the reference */
  double *energies;           /* optional out: [total_steps][n_omegas][6] =
                                 module, potential, kinetic, rotational,
                                 coriolis, total (wavepackets1device.cu:442-451) */
  const char *autotune_cache; /* optional file of the autotuner's kernel choices
                                 (NULL: the QD_AUTOTUNE_CACHE environment
                                 variable, else kept in the process only) */
} qd_options;

/* dump1 / dump2 absorbing masks: matlabStructures.C:67-72 (NULL = absent) */
typedef struct qd_dump_function {
  const double *dump;
} qd_dump_function;

/* CRP: matlabStructures.C:80-90.  The reference parses these fields and never
   uses them; here calculate_CRP != 0 turns on the flux analysis and CRP
   receives P(E). */
typedef struct qd_crp {
  const double *energies;     /* [n_energies] total energies */
  const double *eta_sq;       /* [n_energies] |a(E)|^2 of the initial packet */
  double *CRP;                /* [n_energies] out */
  int32_t n_dividing_surface; /* index of r_s on the r2 grid */
  int32_t n_gradient_points;  /* odd stencil width of d/dr at r_s */
  int32_t n_energies;
  int32_t calculate_CRP;
  /* extension: optional in/out time-to-energy accumulators so that a run split
     over several calls continues exactly; layout
     [n_omegas][2][n_energies][n_theta][n1] complex (interleaved doubles) */
  double *accumulators;
} qd_crp;

/* OmegaStates: matlabStructures.C:92-153 */
typedef struct qd_omega_states {
  int32_t J;
  int32_t parity;
  int32_t l_max;
  int32_t n_omegas_max;
  int32_t n_omegas;                   /* number of entries in omegas */
  const int32_t *omegas;              /* consecutive helicities starting at
                                         (J+parity)%2 (OmegaList.m:2-16) */
  const double *associated_legendres; /* [n_theta][n_cols][n_omegas] MATLAB order;
                                         block i uses its first l_max-omega_i+1
                                         columns (matlabStructures.C:112-132) */
  int32_t n_cols;                     /* columns per block = l_max - omegas[0] + 1 */
  double *wave_packets;               /* [2*n1][n2][n_theta][n_omegas] in/out */
} qd_omega_states;

/* FH2Data: the struct passed to cudaOpenMPEvolution (FH2main.m:195-206) */
typedef struct qd_fh2data {
  qd_radial_coordinate r1;
  qd_radial_coordinate r2;
  qd_angle_coordinate theta;
  const double *pot;          /* [n1][n2][n_theta] MATLAB order */
  const double *psi;          /* passed by FH2main.m, unused (as in the reference) */
  qd_evolution_time time;
  qd_options options;
  qd_dump_function dump1;
  qd_dump_function dump2;
  qd_crp CRP;
  qd_omega_states OmegaStates;
} qd_fh2data;

/* Callback standing in for mexCallMATLAB(options.wave_to_matlab)
   (wave2matlab.C:19-26, cudaOpenMP2.cu:380-384): called with the wave packets
   already copied back into OmegaStates.wave_packets.  Non-zero return aborts
   with QD_ERR_CALLBACK. */
typedef int (*qd_callback)(qd_fh2data *data, void *user);

/* ---------------------------------------------------------------- core API */

/* Replaces mexFunction / cudaOpenMPEvolution(FH2Data) (cudaOpenMPEvolution.C:15-79):
   runs time.total_steps steps of CudaOpenMPQMMD::test_multiple_cards
   (cudaOpenMP2.cu:328-390) on the current CUDA device. */
int qd_evolve(qd_fh2data *data, qd_callback cb, void *user);

/* Batched partial waves: n_problems independent FH2Data structs (one per total
   J) that share r1, r2, theta, pot, dump1, dump2, time and options, stepped
   together (each stage one launch over every Omega block of every problem). */
int qd_evolve_batch(qd_fh2data *const *problems, int32_t n_problems, qd_callback cb, void *user);

/* qd_evolve and qd_evolve_batch keep the device state of their last call on
   each device (up to QD_SESSION_CACHE_BYTES of device memory, default 8 GiB;
   the environment variable set to 0 turns this off) and reuse it for the next
   call with the same grids, time step, precision, Omega lists and flux
   surface: only the wave packets and the inputs that changed are loaded again.
   This releases the kept state and its device memory. */
int qd_release_session_cache(void);

/* Last error message of the calling thread ("" if none). */
const char *qd_last_error(void);

/* QD_VERSION of the loaded library. */
int qd_version(void);

/* ---------------------------------------------------------- session API
 * A session keeps every Omega block resident in HBM between calls: the
 * pieces of qd_evolve, for benchmarking and for stage-by-stage checking.
 * The reference's per-stage methods (omegawavepacket.h:79-126) map to
 * qd_session_apply stages.
 */
typedef struct qd_session qd_session;

int qd_session_create(qd_fh2data *const *problems, int32_t n_problems, qd_session **out);
int qd_session_destroy(qd_session *s);
/* enqueue n_steps full time steps on the session stream (no host sync) */
int qd_session_run(qd_session *s, int32_t n_steps);
int qd_session_synchronize(qd_session *s);
/* enqueue the time-to-energy transform of the flux surface values buffered by
   the steps run so far (it otherwise runs once per 64 steps, and before any
   download), so that a timed region can hold exactly its own steps' flux work;
   no host sync.  A no-op without CRP.calculate_CRP or with nothing buffered. */
int qd_session_flush(qd_session *s);
/* copy psi (theta space), time.steps, CRP and energies back into the structs */
int qd_session_download(qd_session *s, qd_fh2data *const *problems, int32_t n_problems);
/* upload psi (theta space) from the structs again */
int qd_session_upload(qd_session *s, qd_fh2data *const *problems, int32_t n_problems);
/* opaque cudaStream_t of the session */
void *qd_session_stream(qd_session *s);
/* total Omega blocks and kernel launches per regular time step */
int qd_session_info(qd_session *s, int32_t *n_blocks, int32_t *launches_per_step);

typedef enum qd_stage {
  QD_STAGE_DUMP = 0,              /* dump_wavepacket (omegawavepacket.cu:491-501) */
  QD_STAGE_POTENTIAL = 1,         /* evolution_with_potential(dt) (:314-328) */
  QD_STAGE_FORWARD_LEGENDRE = 2,  /* forward_legendre_transform (:200-219) */
  QD_STAGE_BACKWARD_LEGENDRE = 3, /* backward_legendre_transform (:221-240) */
  QD_STAGE_ROTATIONAL = 4,        /* evolution_with_rotational(dt) (:347-362) */
  QD_STAGE_CORIOLIS = 5,          /* evolution_with_coriolis(dt) (cudaOpenMP2.cu:392-423) */
  QD_STAGE_CORIOLIS_ENERGY = 6,   /* evolution_with_coriolis(dt, 1) */
  QD_STAGE_FFT_KINETIC = 7,       /* forward FFT, kinetic(dt), kinetic energy,
                                     backward FFT + scale (:242-269, :330-345, :364-395) */
  QD_STAGE_ENERGIES = 8,          /* rotational, potential energies and module */
  QD_STAGE_FLUX = 9               /* accumulate the flux at time (steps+1)*dt */
} qd_stage;

int qd_session_apply(qd_session *s, int32_t stage, double dt);

/* state access for one Omega block (global block index over all problems):
   which = 0: theta-space psi [n_theta][n2][n1] complex,
   which = 1: Legendre-space psi [l_max-omega+1][n2][n1] complex */
int qd_session_get_psi(qd_session *s, int32_t which, int32_t block, double *host_out, size_t n_doubles);
int qd_session_set_psi(qd_session *s, int32_t which, int32_t block, const double *host_in, size_t n_doubles);
/* energies of the last completed step or stage: [n_blocks][6] */
int qd_session_get_energies(qd_session *s, double *host_out, size_t n_doubles);

/* ------------------------------------------------------ allocation-free call */

/* Rotational energy of one Omega block, computed without allocating any device
   memory.  It has no counterpart in the reference.  It is for callers that
   cannot call cudaMalloc: code whose device memory is all owned by another
   allocator (a framework's caching pool such as PyTorch's or MATLAB gpuArray's)
   or a loop in which the device synchronisation of cudaMalloc is not allowed.
   psi_j: device pointer to the block's Legendre-space slabs l = omega..l_max,
   [l_max-omega+1][n2][n1] complex (interleaved doubles).  rotational_energy:
   device pointer to one double, receiving dr1 dr2 sum_l l(l+1)
   sum (1/(2 m1 R^2) + 1/(2 m2 r^2)) |psi_l|^2, the same quantity as the
   session's rotational energy.  stream: a cudaStream_t, or NULL for the default
   stream.  The per-CTA partial sums live in a fixed 512 KiB device array of the
   library (every GPU that loads the library holds it until exit), so
   l_max - omega + 1 may be at most 4096; larger values return QD_ERR_INVALID.
   All calls share that array, so calls that overlap on the GPU (on different
   streams, or on different host threads) race.  Every call looks up the
   array's device address in the current device's context (no allocation); the
   first call on a device may also load the library's device code, so make it
   before any stream capture. */
int qd_rotational_energy_noalloc(const double *psi_j, int32_t n1, int32_t n2, int32_t omega, int32_t l_max,
                                 double r1_left, double r1_dr, double r1_mass, double r2_left, double r2_dr,
                                 double r2_mass, double *rotational_energy, void *stream);

/* ------------------------------------------------------------ diagnostics */

/* Runs n_steps regular time steps eagerly with a CUDA event after every
   kernel launch on the session stream and reports, per kernel name, the mean
   duration of one launch (ms) and its number of launches over the n_steps.
   names receives the kernel names separated by '\n'. */
int qd_session_profile(qd_session *s, int32_t n_steps, char *names, size_t names_cap, double *avg_ms,
                       int32_t *launches, int32_t max_kernels, int32_t *n_kernels);

/* What the autotuner chose for this session's mixed-form FFT (kernel, and the
   measured microseconds per launch of every candidate, or "cached"), as text. */
int qd_session_tuning(qd_session *s, char *text, size_t text_cap);

/* Measured FP64 tensor-core throughput of the current device (TFLOP/s, 2
   flops per FMA) from a register-resident loop of mma.sync m8n8k4 f64 (DMMA),
   to compare with the DFMA figure of qd_device_fma_peaks. */
int qd_device_dmma_peak(double *fp64_tensor_tflops);

/* Self-test of the bounded device-side wait that every pipelined kernel of the
   library uses: one CTA waits on an mbarrier with a budget of budget_ms.  With
   arrive = 0 nothing ever arrives, the wait gives up after the budget and the
   call returns QD_ERR_TIMEOUT (the device status word the kernels set); with
   arrive = 1 a second thread arrives and the call returns QD_OK.  Either way
   the kernel ends and the context stays usable. */
int qd_device_wait_selftest(double budget_ms, int32_t arrive);

/* Measured FP64 fused-multiply-add throughput of the current device
   (TFLOP/s, 2 flops per FMA) from a register-resident DFMA loop, and the
   same for FP32 FMA. */
int qd_device_fma_peaks(double *fp64_tflops, double *fp32_tflops);

#ifdef __cplusplus
}
#endif

#endif /* QD_H */
