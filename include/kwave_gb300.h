/* C ABI of the GB300 k-space first-order time loop (libkwave_gb300.so).
 *
 * The library replaces the time loop of k-wave-python's native solver
 * (kwave/solvers/kspace_solver.py, Simulation.setup :205-241, Simulation.step
 * :691-747, Simulation.run :749-778), reached from kspaceFirstOrder2D/3D
 * (kwave/kspaceFirstOrder2D.py:215-218, kwave/kspaceFirstOrder3D.py:208-211)
 * through kwave/solvers/native.py:6-30 (run_python_backend).
 *
 * Conventions: plain host pointers and sizes; grids are C order with axis 0 = x
 * and the last axis contiguous; all device memory belongs to the plan.  Every
 * call returns KW_OK (0) or an error code; kw_last_error() gives the
 * thread-local message of the last failure.
 */
#ifndef KWAVE_GB300_H
#define KWAVE_GB300_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum {
  KW_OK = 0,
  KW_ERR_INVALID = 1,      /* bad argument / descriptor (reference raises ValueError) */
  KW_ERR_CUDA = 2,         /* CUDA runtime failure */
  KW_ERR_OOM = 3,          /* device allocation failed */
  KW_ERR_UNSUPPORTED = 4,  /* e.g. FFT length with a prime factor above 7 */
  KW_ERR_STATE = 5         /* call out of order (e.g. run before finalize) */
};

/* Grid, time axis and physics switches.  Mirrors what Simulation.setup derives
 * (kspace_solver.py:205-241, :363-550). */
typedef struct kw_grid_desc {
  int32_t ndim;          /* 2 or 3 */
  int32_t shape[3];      /* N_x, N_y, N_z (unused entries 1) */
  int32_t Nt;            /* number of time steps (kgrid.Nt) */
  int32_t record_start;  /* 0-based first recorded step (sensor.record_start_index - 1) */
  double spacing[3];     /* d_x, d_y, d_z [m] */
  double dt;             /* [s] */
  double c_ref;          /* max(c0), kspace_solver.py:231 */
  int32_t use_sg;        /* staggered grid shifts (kspace_solver.py:440-447) */
  int32_t use_kspace;    /* kappa / source_kappa (kspace_solver.py:429-435) */
  int32_t absorb_mode;   /* 0 none, 1 power law (fractional Laplacian), 2 Stokes (y = 2) */
  int32_t dispersion;    /* 1: power-law dispersion term enabled (kspace_solver.py:500-524) */
  int32_t nonlinear;     /* 1: B/A enabled (kspace_solver.py:526-550) */
  int32_t flags;         /* KW_DESC_* bits */
  double alpha_power;    /* y */
} kw_grid_desc;

/* kw_grid_desc.flags: run every pass with the shared-memory FFT kernels that
 * take their length at run time, so that kw_batch can fold the plan's passes
 * into grouped launches with other plans of any size. */
enum { KW_DESC_GENERIC_FFT = 1 };

/* Grid-valued inputs.  n == 0 (or host == NULL) selects the scalar. */
enum {
  KW_F_C0 = 0,       /* sound speed c0 */
  KW_F_RHO0 = 1,     /* density rho0 */
  KW_F_DTRSG0 = 2,   /* dt / rho0 staggered along x (kspace_solver.py:657-666) */
  KW_F_DTRSG1 = 3,   /* ... along y */
  KW_F_DTRSG2 = 4,   /* ... along z */
  KW_F_BONA = 5,     /* B/A */
  KW_F_TAU = 6,      /* absorption coefficient tau (kspace_solver.py:494-497) */
  KW_F_ETA = 7,      /* dispersion coefficient eta (kspace_solver.py:522) */
  KW_F_P0 = 8        /* initial pressure, already smoothed if requested */
};

/* One-dimensional per-axis tables (length N_axis; complex tables hold 2*N floats
 * re,im interleaved). */
enum {
  KW_T_K = 0,        /* 2 pi fftfreq(N, d) (kspace_solver.py:419) */
  KW_T_PML = 1,      /* PML, non-staggered (kwave/utils/pml.py:6-64) */
  KW_T_PMLSG = 2,    /* PML, staggered */
  KW_T_OPGRAD = 3,   /* i k e^{+i k d/2} (Hermitian part), without kappa (complex) */
  KW_T_OPDIV = 4,    /* i k e^{-i k d/2} (Hermitian part), without kappa (complex) */
  KW_T_UNSTAG = 5,   /* e^{-i k d/2} (Hermitian part) (kspace_solver.py:677) (complex) */
  KW_T_WCOORD = 6    /* p0 smoothing: squared window coordinate along the axis, FFT order */
};

/* Source slots: KW_S_P0..2 = pressure source injected into rho_x/y/z, already
 * scaled per axis (kspace_solver.py:597-624); KW_S_U0..2 = velocity sources. */
enum { KW_S_P0 = 0, KW_S_P1 = 1, KW_S_P2 = 2, KW_S_U0 = 3, KW_S_U1 = 4, KW_S_U2 = 5 };
/* Source modes (kspace_solver.py:86-114). */
enum { KW_SRC_DIRICHLET = 0, KW_SRC_ADDITIVE = 1, KW_SRC_ADDITIVE_NC = 2 };

/* Recorded series.  Stored time-major on the device; read back sensor-major. */
enum {
  KW_R_P = 0,
  KW_R_UX_ST = 1, KW_R_UY_ST = 2, KW_R_UZ_ST = 3,  /* staggered u (kspace_solver.py:744-745) */
  KW_R_UX = 4, KW_R_UY = 5, KW_R_UZ = 6            /* u shifted to the pressure grid (:740-743) */
};
/* Fields readable after a run. */
enum { KW_FLD_P = 0, KW_FLD_U0 = 1, KW_FLD_U1 = 2, KW_FLD_U2 = 3, KW_FLD_RHO0 = 4, KW_FLD_RHO1 = 5, KW_FLD_RHO2 = 6 };
/* Aggregates over the recorded time axis (kspace_solver.py:824-837). */
enum { KW_AGG_MAX = 0, KW_AGG_MIN = 1, KW_AGG_RMS = 2 };

typedef struct kw_plan kw_plan;

/* Library version (major*10000 + minor*100 + patch). */
int32_t kw_version(void);
/* Thread-local message of the last failing call ("" if none). */
const char* kw_last_error(void);
/* Device properties of the current CUDA device. */
int32_t kw_device_query(int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor, uint64_t* free_bytes);

/* Simulation.__init__/setup (kspace_solver.py:135-241): validates the grid and
 * the FFT lengths. */
int32_t kw_plan_create(const kw_grid_desc* desc, kw_plan** out);
/* _expand_to_grid of medium/p0 inputs (kspace_solver.py:48-57, 228-230, 680-687). */
int32_t kw_plan_set_field(kw_plan* plan, int32_t field, const float* host, int64_t n, float scalar);
/* _setup_pml / _setup_kspace_operators tables (kspace_solver.py:363-447). */
int32_t kw_plan_set_table(kw_plan* plan, int32_t table, int32_t axis, const float* host, int64_t n_floats);
/* _build_source_op (kspace_solver.py:60-114): flat C-order mask indices and the
 * scaled signal, (n_rows, length) row-major; n_rows == 1 broadcasts. */
int32_t kw_plan_set_source(kw_plan* plan, int32_t slot, int32_t mode, const int64_t* mask_index, int32_t n_points,
                           const float* signal, int32_t n_rows, int32_t length);
/* _setup_sensor_mask (kspace_solver.py:243-326): flat C-order grid indices that
 * are sampled every recorded step, and which series to record (bit r set =
 * record series r of KW_R_*). */
int32_t kw_plan_set_sensor(kw_plan* plan, const int64_t* slot_index, int32_t n_slots, int32_t record_mask);
/* Cartesian sensors (kspace_solver.py:328-361): point s is
 * sum_c weight[s*n_corners+c] * sample[slot[s*n_corners+c]]. */
int32_t kw_plan_set_sensor_interp(kw_plan* plan, int32_t n_points, int32_t n_corners, const int32_t* slot,
                                  const double* weight);
/* Smooth p0 on the device before the first step (kwave/utils/filters.py:549-615,
 * restore_max=True): p0 <- (max|p0| / max|p0_s|) p0_s with
 * p0_s = Re F^-1[W F[p0]], W(k) = window(min(sqrt(sum_i c_i^2), radius)) where c_i are
 * the KW_T_WCOORD tables and window is linearly interpolated from n samples on
 * [-radius, radius] (the rotated Blackman window of kwave/utils/signals.py:222-283). */
int32_t kw_plan_set_p0_smoothing(kw_plan* plan, const float* window, int32_t n, double radius);
/* Derive on the device, at kw_plan_finalize, the medium grids that the host
 * would otherwise compute and upload (kspace_solver.py:655-666, :471-524):
 *   what & 1: dt / rho0 on the three staggered grids (KW_F_DTRSG0..2) from the
 *             KW_F_RHO0 grid, as the reference forms them in float32;
 *   what & 2: tau = -2 a c0^(y-1) (power law) or -2 a c0 (Stokes);
 *   what & 4: eta = 2 a c0^y tan(pi y / 2);
 * with a = db2neper(alpha, y) (kwave/utils/conversion.py:20-35) from `alpha`
 * (n = grid size values, dB/(MHz^y cm)) or the scalar alpha_s when alpha is
 * NULL.  absorb_mode: 1 power law, 2 Stokes.  Fields derived this way must
 * not also be set with kw_plan_set_field. */
int32_t kw_plan_derive_medium(kw_plan* plan, int32_t what, const float* alpha, int64_t n, double alpha_s,
                              double alpha_power, int32_t absorb_mode);
/* Replaces the initial pressure of a finalized plan that was given a p0 grid
 * (n = N_total values) and rewinds it to t = 0 as kw_plan_reset does, keeping
 * everything else uploaded.  No counterpart in the reference, where a new p0
 * means a new Simulation; iterative reconstructions run many forward passes
 * that differ only in p0. */
int32_t kw_plan_update_p0(kw_plan* plan, const float* host, int64_t n);
/* Replaces the signal of a source slot of a finalized plan (same shape as
 * given to kw_plan_set_source, already scaled the same way); the mask and
 * mode stay.  Call kw_plan_reset before running from t = 0 again.  No
 * counterpart in the reference (a new Simulation per signal there); used to
 * run many time-reversal passes on one plan. */
int32_t kw_plan_update_source(kw_plan* plan, int32_t slot, const float* signal, int32_t n_rows, int32_t length);
/* Allocates device memory, uploads all inputs and resets the state to t = 0. */
int32_t kw_plan_finalize(kw_plan* plan);
/* Advances min(nsteps, Nt - t) steps of Simulation.step (kspace_solver.py:691-747)
 * on `stream` (a cudaStream_t, NULL = default stream); returns after enqueueing.
 * Steps with the same launch sequence run as one CUDA graph, captured on first
 * use and replayed with the step index held on the device; the last step of a
 * call, the t = 0 initial-condition step and every step while timing is on are
 * plain launches.  Use one stream per plan. */
int32_t kw_plan_run(kw_plan* plan, int32_t nsteps, void* stream);
/* Autotuner of the run-time-length FFT kernels (the lengths that are not
 * powers of two): times `nsteps` graph steps after the t = 0 step (at least
 * 2, at most Nt - 1) for each candidate launch geometry -- tile columns T in
 * {2, 4, 8, 16} of the axis passes, rows per block R in {R0/2, R0, 2 R0} of
 * the row stages -- keeps the fastest and rewinds the plan to t = 0
 * (kw_plan_reset).  The plan must be at
 * t = 0.  Results are bit-identical for every choice.  *T_out / *R_out (may be
 * NULL) receive the geometry in use; plans without such kernels are left as
 * they are. */
int32_t kw_plan_autotune(kw_plan* plan, int32_t nsteps, void* stream, int32_t* T_out, int32_t* R_out);
/* Adjoint of the time loop (no counterpart in the reference): the gradient
 * with respect to p0 of sum over sensor points and recorded steps of
 * residual * recorded p, i.e. the transposed time loop applied to `residual`
 * (sensor-major (n_slots, Nt - record_start): one row per recorded grid
 * point -- the sensor points of a binary sensor, the interpolation corners of
 * a Cartesian one, whose residual the caller takes back through the
 * transposed interpolation weights).  For the lossless, source-free loop
 * with a sensor recording p and smoothing off; `grad` receives N_total
 * float32 (C order).  With residual = recorded p - observed data it is the gradient of
 * 1/2 ||recorded p - observed||^2.  The plan is reset (t = 0, zero state)
 * before and after; its uploaded medium, PML and sensor are used. */
int32_t kw_plan_adjoint_p0(kw_plan* plan, const float* residual, int64_t n, float* grad, void* stream);
/* Checkpoints of the forward run for kw_plan_adjoint's sound-speed gradient
 * (no counterpart in the reference): with interval K > 0, kw_plan_run keeps
 * the state carried between steps (u_i, rho_i and the spectrum of p) after
 * every step t with t % K == 0, in ceil(Nt / K) device slots of
 * (2 D N_total + 2 spectrum) floats each; K = 1 keeps every step (no
 * recomputation), larger K trades memory for rerunning up to K - 1 steps per
 * segment.  0 frees them.  The plan must be at t = 0. */
int32_t kw_plan_set_checkpoints(kw_plan* plan, int32_t interval);
/* Adjoint of the time loop with both gradients (no counterpart in the
 * reference): as kw_plan_adjoint_p0 for grad_p0; when grad_c is not NULL it
 * also receives the gradient with respect to the sound speed c0 (N_total
 * float32) of sum(residual * recorded p), with c_ref (PML, kappa) held at the
 * plan's value.  That needs the forward run of this plan from t = 0 to Nt
 * with p0 set, smoothing off and checkpoints on (kw_plan_set_checkpoints):
 * the forward density sum of every step is regenerated segment by segment
 * from the checkpoints while the transposed steps run backwards.  The result
 * does not depend on the interval: the regenerated steps are the forward's
 * own steps, bit for bit.  The plan is reset (t = 0) afterwards. */
int32_t kw_plan_adjoint(kw_plan* plan, const float* residual, int64_t n, float* grad_p0, float* grad_c, void* stream);
/* Failure-detection test of the bounded device waits (off by default; no
 * counterpart in the reference).  While enabled, the velocity stage's bulk-fed
 * row kernel withholds, in its first CTA, the first copy its consumers wait
 * for, and its waits give up after 20 ms instead of 2 s: the consumers time
 * out, leave together, and the next kw_plan_sync returns KW_ERR_CUDA with the
 * timeout message.  Nothing faults and no wait is unbounded; the plan's
 * results are invalid until it is reset.  Needs a power-of-two last axis of
 * 128 to 2048 points (the bulk-fed row stages). */
int32_t kw_plan_set_wait_test(kw_plan* plan, int32_t enable);
/* enable == 0: every step as plain launches (default 1; the environment
 * variable KWAVE_GB300_GRAPHS=0 sets 0 at kw_plan_finalize). */
int32_t kw_plan_set_graphs(kw_plan* plan, int32_t enable);
/* Batch of independent finalized plans (any sizes, media, sources, sensors;
 * no counterpart in the reference, which runs one Simulation at a time).
 * kw_batch_run advances every plan by min(nsteps, Nt - t) steps; each step of
 * all plans whose steps are graph steps is ONE graph launch.  Inside it the
 * passes of plans created with KW_DESC_GENERIC_FFT are grouped: the k-th
 * launch of every such plan's step runs in one grouped launch; other plans
 * join as parallel branches holding their own step graphs.  Plans keep their
 * own state, results and read functions.  Destroy the batch before its plans. */
typedef struct kw_batch kw_batch;
int32_t kw_batch_create(kw_plan* const* plans, int32_t n, kw_batch** out);
int32_t kw_batch_run(kw_batch* batch, int32_t nsteps, void* stream);
/* Batch autotuner: one launch geometry of the run-time-length kernels for all
 * members (T in {2, 4, 8, 16}, R = R0 * {1/2, 1, 2} of each member), each
 * candidate timed on `nsteps` graph steps after the t = 0 step of the batch
 * itself (fewer if a member is shorter; no tuning below 2); keeps the fastest
 * and rewinds every plan to t = 0.  Every plan must be at t = 0.  Results are
 * bit-identical for every choice. */
int32_t kw_batch_autotune(kw_batch* batch, int32_t nsteps, void* stream, int32_t* T_out, int32_t* R_num,
                          int32_t* R_den);
/* Schedule of the run-time-length shared-memory FFTs.  0-2: Stockham stages
 * with the factors in the order 0: 4, 2, 3, 5, 7 (default), 1: 5, 3, 7, 4, 2,
 * 2: 3, 4, 5, 2, 7.  3: the two-level schedule (two passes of register DFTs)
 * for lengths n1 n2 with both factors 5-smooth and at most 20, schedule 0 for
 * the other lengths.  Every schedule computes the same transform; they differ
 * in speed and in rounding (results stay within the 1e-5 parity bar; they are
 * not bit-identical across schedules).  No counterpart in the reference. */
int32_t kw_plan_set_radix_order(kw_plan* plan, int32_t order);
/* The same schedule for every member of a batch (drops the batch's graphs;
 * members keep their time index). */
int32_t kw_batch_set_radix_order(kw_batch* batch, int32_t order);
/* Batch radix autotuner: times each schedule on `nsteps` graph steps of the
 * whole batch after the t = 0 step (every member on the same schedule), keeps
 * the fastest and rewinds every plan to t = 0; *order_out (may be NULL)
 * receives it.  Run after kw_batch_autotune when both are wanted. */
int32_t kw_batch_autotune_radix(kw_batch* batch, int32_t nsteps, void* stream, int32_t* order_out);
/* Runs of steps with an unchanged launch sequence (no source switching on or
 * off, no record start, not the last step) run as ONE launch of a graph that
 * loops over the batch's step graph on the device: a conditional while node
 * whose body is the step graph followed by a one-thread kernel counting the
 * passes (cudaGraphSetConditional).  Runs shorter than 4 steps, and every
 * step when enable == 0 (or KWAVE_GB300_BATCH_LOOPS=0 at kw_batch_create),
 * are one launch each.  Results are bit-identical either way.  No
 * counterpart in the reference. */
int32_t kw_batch_set_loops(kw_batch* batch, int32_t enable);
/* Graph launches issued by kw_batch_run for the batch's steps since its
 * creation (one per loop run or per single step). */
int32_t kw_batch_graph_launches(const kw_batch* batch, int64_t* count);
/* Kernels launched through the batch and its plans since their creation (a
 * grouped launch over several plans counts once). */
int32_t kw_batch_launch_count(const kw_batch* batch, int64_t* count);
int32_t kw_batch_destroy(kw_batch* batch);
/* Waits for the plan's work on `stream`. */
int32_t kw_plan_sync(kw_plan* plan, void* stream);
/* Current step index t. */
int32_t kw_plan_time_index(const kw_plan* plan, int32_t* t);
/* Recorded series, sensor-major (n_points, n_recorded_steps) float32, the layout
 * of sensor_data[...] in kspace_solver.py:663-668. */
int32_t kw_plan_read_series(kw_plan* plan, int32_t series, float* host, int64_t n);
/* Aggregate over recorded steps (max/min/rms), n_points float32. */
int32_t kw_plan_read_aggregate(kw_plan* plan, int32_t series, int32_t kind, float* host, int64_t n);
/* Whole field (p, u_i or rho_i), C order, N_total float32. */
int32_t kw_plan_read_field(kw_plan* plan, int32_t field, float* host, int64_t n);
/* Device pointer of a field (valid until kw_plan_destroy). */
int32_t kw_plan_field_device_ptr(kw_plan* plan, int32_t field, void** dptr);
/* Zeroes the state and the recorded series and rewinds to t = 0, keeping the
 * uploaded medium, sources and sensor (a fresh Simulation.setup()). */
int32_t kw_plan_reset(kw_plan* plan);
/* Launch classes for timing: axis pass with operators, plain axis pass, and
 * the row stages INIT, U, RHO, EOS. */
enum { KW_K_AXIS_OPS = 0, KW_K_AXIS_PLAIN = 1, KW_K_ROWS_INIT = 2, KW_K_ROWS_U = 3, KW_K_ROWS_RHO = 4,
       KW_K_ROWS_EOS = 5, KW_K_NCLASS = 6 };
/* enable != 0: bracket every launch with CUDA events on its stream (clears
 * previous timings). */
int32_t kw_plan_set_timing(kw_plan* plan, int32_t enable);
/* Synchronises and returns, per launch class, the summed kernel time [ms] and
 * the number of launches since timing was enabled (arrays of KW_K_NCLASS). */
int32_t kw_plan_read_timing(kw_plan* plan, double* ms, int64_t* count);
/* Number of kernels the plan has launched since creation. */
int32_t kw_plan_launch_count(const kw_plan* plan, int64_t* count);
/* Spectral derivative along `axis` without any device allocation (no
 * counterpart in the reference; it computes what Simulation._diff(f,
 * op_grad_list[axis]) computes, kwave/solvers/kspace_solver.py:781-796 with the
 * operator of :440-447):
 *     out = Re F^-1[ kappa(|k|) (i k_a e^{+i k_a d_a/2}) F[f] ],
 *     kappa = sin(kappa_coef |k|) / (kappa_coef |k|)  (kappa_coef = c_ref dt / 2; 0 gives kappa = 1),
 * with the shift factor dropped when use_sg == 0.  f and out are caller-owned
 * device buffers of N_total float32 (C order).
 * For callers that cannot let a library allocate device memory: custom
 * operators of frameworks that own all device memory (PyTorch, JAX/XLA,
 * TensorRT plugins) and real-time pipelines that forbid allocation once
 * running.  The half-spectrum scratch is a static 16 MiB device array
 * (2,097,152 complex values: the grid must satisfy N0*N1*Hp (3-D) or N0*Hp
 * (2-D) <= 2,097,152 with Hp = N_last/2 + 1 rounded up to even, e.g. square
 * grids up to 2040^2 and cubes up to 159^3), held by every
 * GPU that loads the library until exit; larger grids return
 * KW_ERR_UNSUPPORTED.  The first call on a device resolves the array's address
 * and sets kernel attributes (make it before any stream capture).  All calls
 * share the array: calls that overlap on the GPU race and must be serialised
 * by the caller.  Work is enqueued on `stream` (NULL = default stream). */
int32_t kw_gradient_noalloc(const float* f, float* out, int32_t ndim, const int32_t* shape, const double* spacing,
                            int32_t axis, double kappa_coef, int32_t use_sg, void* stream);
/* ---- learned warm start (no counterpart in the reference) ----------------
 * Kernels of a BF16 U-Net with FP32 accumulation on the 5th-generation tensor
 * cores (tcgen05.mma with the accumulator in tensor memory), trained and run
 * by kwave_gb300.warmstart.  Its input is a time-reversal image
 * (kwave/reconstruction/time_reversal.py:129-150), its output an initial
 * pressure estimate that adjoint iterations refine.  All pointers are device
 * pointers owned by the caller; activations are bf16 NHWC, parameters and
 * gradients f32; every call enqueues on `stream` (NULL = default stream). */
/* C[M][N] (f32) = sum_k A[m][k] B[n][k], A and B row-major bf16, K % 8 == 0. */
int32_t kw_umma_gemm(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K, void* stream);
/* C[M][N] (f32) = sum_k A[k][m] B[k][n] on MN-major shared-memory tiles (A and
 * B row-major bf16 with M and N contiguous), M % 8 == 0, N % 8 == 0. */
int32_t kw_umma_gemm_mn(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K, void* stream);
/* 3x3 convolution, stride 1, zero padding: y[p][co] = act(bias[co] + sum over
 * taps and input channels of w[co][tap][ci] x[p + tap][ci]), where the input is
 * x1 (nb, H, W, c1) followed along channels by x2 (nb, H/2, W/2, c2) read with
 * nearest-neighbour upsampling (c2 = 0: x1 alone).  c1, c2 and cout
 * multiples of 8; act = ReLU when relu != 0.  Output to y (bf16) and/or
 * yf (f32), (nb, H, W, cout).  With the output gradient as x1 and the weights
 * from kw_unet_flip_weights it is the data gradient. */
int32_t kw_conv3x3(const void* x1, int32_t c1, const void* x2, int32_t c2, int32_t nb, int32_t H, int32_t W,
                   const void* w, const float* bias, int32_t cout, int32_t relu, void* y, float* yf, void* stream);
/* Weight gradient of kw_conv3x3: dw[co][tap][ci] += sum over pixels of
 * dz[p][co] x[p + tap][ci] (x as in kw_conv3x3), cout a multiple of 8. */
int32_t kw_conv3x3_wgrad(const void* x1, int32_t c1, const void* x2, int32_t c2, int32_t nb, int32_t H, int32_t W,
                         const void* dz, int32_t cout, float* dw, void* stream);
/* 2x2 average pooling (nb, H, W, C) -> (nb, H/2, W/2, C), and its gradient
 * (dx = dy/4 on each child, plus `add` when not NULL). */
int32_t kw_unet_avgpool2(const void* x, void* y, int32_t nb, int32_t H, int32_t W, int32_t C, void* stream);
int32_t kw_unet_avgpool2_bwd(const void* dy, void* dx, int32_t nb, int32_t H, int32_t W, int32_t C, const void* add,
                             void* stream);
/* dz = dy where y > 0, else 0 (ReLU gradient), n bf16 values. */
int32_t kw_unet_relu_grad(const void* dy, const void* y, void* dz, int64_t n, void* stream);
/* Gradient of a concatenated input (nb, H, W, C1 + C2): channels < C1 to d1
 * (plus add1 when not NULL), the rest summed over each 2x2 block to d2
 * (nb, H/2, W/2, C2), the gradient of the nearest-neighbour upsampling. */
int32_t kw_unet_split_concat_grad(const void* dcat, int32_t nb, int32_t H, int32_t W, int32_t C1, int32_t C2, void* d1,
                                  const void* add1, void* d2, void* stream);
/* wt[ci][8 - tap][co] = w[co][tap][ci] (bf16): the data-gradient weights. */
int32_t kw_unet_flip_weights(const void* w, void* wt, int32_t cout, int32_t cin, void* stream);
/* db[c] += sum over npix pixels of dz[p][c]. */
int32_t kw_unet_bias_grad(const void* dz, float* db, int64_t npix, int32_t C, void* stream);
/* Residual-form estimate e[p] = out[p][0] + s img[p] (out (npix, cout) f32,
 * img (npix) f32): kw_unet_residual_out writes e; kw_unet_mse_grad adds
 * sum (e - target)^2 to *loss and writes dout[p][0] = scale (e - target),
 * the other channels 0 (bf16). */
int32_t kw_unet_mse_grad(const float* out, int32_t cout, const float* img, float s, const float* target, void* dout,
                         int64_t npix, float scale, float* loss, void* stream);
int32_t kw_unet_residual_out(const float* out, int32_t cout, const float* img, float s, float* e, int64_t npix,
                             void* stream);
/* Adam step (bias-corrected, step >= 1) on f32 parameters w with moments m, v
 * and gradient g; wb (may be NULL) receives the bf16 copy. */
int32_t kw_unet_adam(float* w, float* m, float* v, const float* g, void* wb, int64_t n, float lr, float b1, float b2,
                     float eps, int32_t step, void* stream);
/* f32 image (npix) -> bf16 NHWC with C channels: channel 0 = scale * image, others 0. */
int32_t kw_unet_image_to_nhwc(const float* img, void* x, int64_t npix, int32_t C, float scale, void* stream);
/* Frees all device memory of the plan. */
int32_t kw_plan_destroy(kw_plan* plan);

#ifdef __cplusplus
}
#endif
#endif
