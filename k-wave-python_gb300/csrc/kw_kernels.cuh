// Kernels of the k-space first-order time loop.
//
// Spectral layout.  A real field of shape (N0[, N1], L), C order, is held in
// "row spectra": every row of L reals along the last axis becomes H = L/2 + 1
// complex values (numpy rfft convention), stored with a row stride Hp = H
// rounded up to an even count (16-byte aligned rows).  The other axes are then
// transformed in place as complex sequences.
//
// Two kernel families:
//   * k_axis  : complex FFT along a strided axis (axis 0, or axis 1 of a 3-D
//               grid), in place.  In "ops" mode it runs forward FFT, multiplies
//               by a spectral operator, runs the inverse FFT and stores, for
//               one or more (input, output, operator) jobs.  The operators
//               (gradient, divergence, fractional Laplacian, source kappa,
//               unstagger shift) are evaluated on the fly from 1-D tables.
//   * k_rows  : one stage of the time step on whole rows along the last axis:
//               C2R of the stage's inputs, the real-space physics of that
//               stage (velocity update, split-density update, equation of
//               state, sources, sensor sampling), and R2C of the outputs.
#pragma once
#include "kw_fft.cuh"

#define KW_NBUF 12
// spectral buffers: S0..S2 work spectra, P = spectrum of p, SRCP / SRCU0..2 =
// k-space corrected source fields, US0..2 = velocity shifted to the pressure grid
enum KwBuf { B_S0 = 0, B_P = 3, B_SRCP = 4, B_SRCU0 = 5, B_US0 = 8 };
#define KW_MAX_JOBS 8
#define KW_NREAL 5

// ST_RHO_PL: ST_RHO with power-law absorption on the register row kernels,
// where rho_sum holds the density sum of the previous step (written by ST_INIT
// and by every ST_RHO_PL) and supplies the nonlinear factor.
// ST_ADJ_*: the transposed step of the lossless time loop (run-time-length
// row kernels only); p, u_i, rho_i then hold the adjoint state and rec[0] the
// sensor residual.
enum KwStage { ST_INIT = 0, ST_U = 1, ST_RHO = 2, ST_EOS = 3, ST_SRC = 4, ST_UREC = 5, ST_P0FFT = 6, ST_P0BACK = 7,
               ST_RHO_PL = 8, ST_ADJ_A = 9, ST_ADJ_B = 10, ST_ADJ_C = 11, ST_ADJ_D = 12, ST_ADJ_E = 13 };
enum KwOp { OP_GRAD = 0, OP_DIV = 1, OP_NAB1 = 2, OP_NAB2 = 3, OP_SKAPPA = 4, OP_UNSTAG = 5, OP_WIN = 6 };
enum KwSrcMode { SRC_DIRICHLET = 0, SRC_ADDITIVE = 1, SRC_ADDITIVE_NC = 2 };

struct KwSrcDev {
  int active;            // 0 = no source in this slot
  int mode;              // KwSrcMode
  int nsig;              // signal rows (1 = broadcast)
  int len;               // signal length in steps
  const int* row_ptr;    // per grid row: first entry (nrows + 1)
  const int4* ent;       // (row, pos, point, 0) sorted by row
  const float* sig;      // time-major [len][nsig], pre-scaled
};

struct RowsParams {
  int stage, init;
  int ndim, N0, N1, L, H, Hp, Mfft, even;
  int nrows, R;
  int t, rec_row, write_p;
  int ex_stride;         // register-FFT rows: exchange region per row (complex values)
  int srcp_on;           // k-space corrected pressure source active at this step
  int srcu_on[3];        // k-space corrected velocity source active at this step
  int rec_us;            // bit a: record u_a shifted to the pressure grid at this step
  int init_r2c;          // ST_U with init: also transform u (for recording at t = 0)
  float inv_d[3];        // 1 / d_i (pressure source correction per density component)
  float2* S[KW_NBUF];    // spectral buffers (KwBuf)
  float* u[3];
  float* rho[3];
  float* p;
  float* rho_sum;
  const float* p0;
  float* p0w;             // ST_P0FFT reads it, ST_P0BACK writes the smoothed p0 into it
  const float* p0_scale;  // restore-max factor applied to p0 in ST_INIT (nullptr: 1)
  const float* c0;
  float c0_s;
  const float* rho0;
  float rho0_s;
  const float* dtrsg[3];
  float dtrsg_s[3];
  const float* bona;
  float bona_s;
  const float* tau;
  float tau_s;
  const float* eta;
  float eta_s;
  int absorb, disp, nonlin;
  float dt;
  const float* pml[3];
  const float* pmlsg[3];
  const float2* tw;       // Mfft twiddles
  const float2* twpost;   // exp(-2 pi i k / L), k <= L/2 (even L)
  KwFftLen flen;
  KwSrcDev src[6];        // p into rho_0..2, then u_0..2
  const int* sens_row_ptr;
  const int4* sens_ent;   // (row, pos, slot, 0)
  int nslots;
  float* rec[7];
  KwDivU dM, dL, dH;      // division by Mfft, L and H (generic row kernels)
  // inside a replayed step graph: the plan's device step counter; t and
  // rec_row are then offsets added to it (nullptr: t and rec_row as given)
  const int* tdev;
  // adjoint with the sound-speed gradient: fsum = forward density sum
  // sum_i rho_i of the step being transposed (ST_ADJ_A), gacc = accumulator of
  // the c^2 gradient, turned into the c gradient by ST_ADJ_E (nullptr: off)
  const float* fsum;
  float* gacc;
  // failure-detection test (kw_plan_set_wait_test): the bulk-fed row stage's
  // CTA 0 withholds its first copy, and its bounded waits give up after
  // wait_ns (0: the normal limit), so that the timeout path runs
  int withhold;
  unsigned long long wait_ns;
};

// step index and record column of a row-stage launch
__device__ __forceinline__ int kw_step_t(const RowsParams& P) { return P.tdev ? P.t + *P.tdev : P.t; }
__device__ __forceinline__ int kw_rec_row(const RowsParams& P) { return P.tdev ? P.rec_row + *P.tdev : P.rec_row; }

struct AxisJob {
  int in, out, op, axis;
};

struct AxisParams {
  float2* bufs[KW_NBUF];
  int n;
  long long xs;   // element stride along the axis
  long long os;   // stride between outer blocks (blockIdx.y)
  int ncols;      // contiguous positions per outer block
  int T;          // positions per tile
  int mode;       // 0 plain forward, 1 plain inverse, 2 ops
  int plain[KW_NBUF];
  int njobs;
  AxisJob jobs[KW_MAX_JOBS];
  KwFftLen flen;
  const float2* tw;
  int ndim, H, Hp;
  const float* k[3];
  const float2* fg[3];
  const float2* fd[3];
  const float2* us[3];
  const float* wc[3];   // p0 smoothing: squared window coordinates (FFT order)
  const float* wtab;    // window samples on [-wrad, wrad]
  int wlen;
  float wrad;
  float kcoef;    // c_ref * dt / 2
  int use_kspace;
  float pow1, pow2;
  float scale;    // 1 / N_total
};

// Spectral operator for one column (ky, kz fixed) of the axis-0 pass.
struct ColK {
  int a1, a2;
  bool valid;
  float ky2, kz2;
};

__device__ __forceinline__ ColK col_geometry(const AxisParams& A, int c) {
  ColK g;
  if (A.ndim == 3) {
    g.a1 = c / A.Hp;
    g.a2 = c - g.a1 * A.Hp;
    g.valid = g.a2 < A.H;
    const float ky = A.k[1][g.a1];
    const float kz = g.valid ? A.k[2][g.a2] : 0.f;
    g.ky2 = __fmul_rn(ky, ky);
    g.kz2 = __fmul_rn(kz, kz);
  } else {
    g.a1 = c;
    g.a2 = 0;
    g.valid = c < A.H;
    const float ky = g.valid ? A.k[1][c] : 0.f;
    g.ky2 = __fmul_rn(ky, ky);
    g.kz2 = 0.f;
  }
  return g;
}

// Host launchers of the generic-length kernels (kw_generic.cuh: k_rows,
// k_axis and their grouped forms, 256 threads per block), one set per FFT
// schedule family F: 0 the Stockham stages (kw_kernels.cu), 1 the two-level
// schedule for plans whose KwFftLen.n1 != 0 (kw_generic_fft2.cu).
#define KW_GENERIC_DECL(F)                                                                                        \
  cudaError_t kw_generic_attr_##F(int smem_max);                                                                  \
  cudaError_t kw_rows_launch_##F(dim3 grid, size_t smem, cudaStream_t st, const RowsParams& P);                   \
  cudaError_t kw_axis_launch_##F(dim3 grid, size_t smem, cudaStream_t st, const AxisParams& A);                   \
  cudaError_t kw_rows_group_launch_##F(int nblk, size_t smem, cudaStream_t st, const RowsParams* Ps, const int4* blk, \
                                       int n);                                                                    \
  cudaError_t kw_axis_group_launch_##F(int nblk, size_t smem, cudaStream_t st, const AxisParams* Ps, const int4* blk, \
                                       int n);
KW_GENERIC_DECL(0)
KW_GENERIC_DECL(1)
// Register-FFT variants for power-of-two lengths 64..1024, launched through
// these host helpers (defined next to the template instantiations).
bool kw_reg_shape(int n, int* E, int* P);
cudaError_t kw_axis_reg_attr(int n);
cudaError_t kw_rows_v2_attr(int m);
cudaError_t kw_axis_reg_launch(int n, dim3 grid, size_t smem, cudaStream_t st, const AxisParams& A);
// register-resident row stages (kw_rows_reg.cu), 128 threads per block
cudaError_t kw_rows_v2_launch(int m, int stage, dim3 grid, size_t smem, cudaStream_t st, const RowsParams& Q);

// Persistent TMA-fed axis passes (kw_axis_tma.cu), power-of-two lengths 64..1024.
void* kw_tma_plan_create();
void kw_tma_plan_destroy(void* h);
bool kw_tma_supported(int n);
bool kw_tma_encode(void* h, int axis, int b, void* base, int ncols, int n, long long xs, int nouter, long long os, int P);
cudaError_t kw_tma_attr(int n, int axis, bool small);
// operator passes along `axis` on small tiles (set before encoding the maps)
void kw_tma_set_small(void* h, int axis, bool small);
bool kw_tma_small_wanted(int n, int ncols, int nsm);
// pdl != 0: launched as a programmatic dependent of the previous kernel of the
// stream (its prologue overlaps that kernel's tail)
cudaError_t kw_tma_launch(void* h, int axis, int n, int nouter, int nb, int nsm, cudaStream_t st, const AxisParams& A,
                          int pdl);
// Window value of the p0 smoothing at squared radius r2 (linear interpolation).
__device__ __forceinline__ float window_at(const float* tab, int n, float rad, float r2) {
  float r = sqrtf(r2);
  if (r > rad) r = rad;
  const float pos = (r + rad) / (2.f * rad) * (float)(n - 1);
  int i0 = (int)pos;
  if (i0 > n - 2) i0 = n - 2;
  const float f = pos - (float)i0;
  return tab[i0] + f * (tab[i0 + 1] - tab[i0]);
}

// max |x| over n values, as float bits folded into *out with atomicMax (n > 0)
__global__ void k_absmax(const float* __restrict__ x, long long n, unsigned int* out);
// out = a / b for two float bit patterns (restore-max factor)
__global__ void k_ratio(const unsigned int* a, const unsigned int* b, float* out);
// device step counter of a plan: set before a run of graph steps, advanced by
// the last node of each step graph
__global__ void k_step_set(int* tdev, int t);
// out = rho_0 + rho_1 (+ rho_2): the forward density sum, in the step's order
__global__ void k_density_sum(float* __restrict__ out, const float* __restrict__ r0, const float* __restrict__ r1,
                              const float* __restrict__ r2, long long n);
__global__ void k_step_tick(int* tdev);
__global__ void k_loop_set(int* left, int n);
__global__ void k_loop_tick(cudaGraphConditionalHandle h, int* left);
__global__ void k_step_tick_group(int* const* tdev, int n);
// Medium grids derived on the device (kw_plan_derive_medium); any output may be null.
struct DeriveParams {
  int ndim, N[3];
  long long ntot;
  float dt_f;          // dt as float32
  int use_sg;
  const float* rho0;
  const float* c0;
  float c0_s;
  const float* alpha;  // null: alpha_s
  double alpha_s;
  double y, db_fac, db_div, tan_fac;  // (1e-6 / (2 pi))^y, 20 log10(e), tan(pi y / 2)
  float db_fac_f;
  int absorb;          // 1 power law, 2 Stokes
  float* dtrsg[3];
  float* tau;
  float* eta;
};
__global__ void k_derive_medium(const __grid_constant__ DeriveParams D);
// Returns and clears the device error word (nonzero: a bounded device wait timed out).
int kw_device_error_take();
// Device address of that word on the current device (nullptr on failure).
int* kw_device_error_ptr();
// Velocity and power-law density stages fed by bulk copies (kw_rows_tma.cu),
// power-of-two row lengths; stage is ST_U or ST_RHO_PL.
cudaError_t kw_rows_tma_attr(int m, int Hp, int ex_stride);
cudaError_t kw_rows_tma_launch(int m, int stage, int nsm, cudaStream_t st, const RowsParams& Q, int* err, int pdl);
__global__ void k_series_gather(const float* __restrict__ rec, int nrec, int nslots, int npts, int ncorner,
                                const int* __restrict__ slot, const double* __restrict__ w, float* __restrict__ out);
__global__ void k_series_reduce(const float* __restrict__ series, int npts, int nrec, int kind, float* __restrict__ out);
