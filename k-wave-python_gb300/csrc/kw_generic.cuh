// Generic-length kernels of the k-space first-order time loop: the row stages
// (k_rows) and axis passes (k_axis) for any 2,3,5,7-smooth length, and their
// grouped forms over several plans.  SCHED selects the FFT family compiled
// into a kernel (kw_fft.cuh: fft_smem): 0 the Stockham stages, instantiated
// in kw_kernels.cu; 1 the two-level register schedule, instantiated in
// kw_generic_fft2.cu.  The physics is the same code for both.
//
// Arithmetic order inside the physics follows kwave/solvers/kspace_solver.py
// (Simulation.step, :691-747) operation by operation, with explicit
// round-to-nearest intrinsics so that the compiler does not contract the
// reference's separate multiplies and adds into FMAs.
#pragma once
#include "kw_kernels.cuh"

// ---------------------------------------------------------------------------
// spectral operators (kspace_solver.py:408-447, :811-816)
// ---------------------------------------------------------------------------
static __device__ __forceinline__ float2 axis_op(const AxisParams& P, const AxisJob& J, int x, int c, bool& valid) {
  int a1, a2 = 0;
  float kk;
  const float kx = P.k[0][x];
  if (P.ndim == 3) {
    a1 = c / P.Hp;
    a2 = c - a1 * P.Hp;
    valid = a2 < P.H;
    if (!valid) return make_float2(0.f, 0.f);
    const float ky = P.k[1][a1], kz = P.k[2][a2];
    kk = __fadd_rn(__fadd_rn(__fmul_rn(kx, kx), __fmul_rn(ky, ky)), __fmul_rn(kz, kz));
  } else {
    a1 = c;
    valid = a1 < P.H;
    if (!valid) return make_float2(0.f, 0.f);
    const float ky = P.k[1][a1];
    kk = __fadd_rn(__fmul_rn(kx, kx), __fmul_rn(ky, ky));
  }
  const float kmag = sqrtf(kk);
  const int ai = (J.axis == 0) ? x : (J.axis == 1 ? a1 : a2);
  float2 v;
  switch (J.op) {
    case OP_GRAD:
    case OP_DIV: {
      float kappa = 1.f;
      if (P.use_kspace) {
        const float arg = P.kcoef * kmag;
        kappa = (arg == 0.f) ? 1.f : sinf(arg) / arg;
      }
      const float2 f = (J.op == OP_GRAD) ? P.fg[J.axis][ai] : P.fd[J.axis][ai];
      v = make_float2(f.x * kappa, f.y * kappa);
      break;
    }
    case OP_NAB1:
    case OP_NAB2: {
      const float e = (J.op == OP_NAB1) ? P.pow1 : P.pow2;
      v = make_float2(kmag == 0.f ? 0.f : powf(kmag, e), 0.f);
      break;
    }
    case OP_SKAPPA:
      v = make_float2(P.use_kspace ? cosf(P.kcoef * kmag) : 1.f, 0.f);
      break;
    case OP_WIN: {
      float r2 = P.wc[0][x] + P.wc[1][a1];
      if (P.ndim == 3) r2 += P.wc[2][a2];
      v = make_float2(window_at(P.wtab, P.wlen, P.wrad, r2), 0.f);
      break;
    }
    default:
      v = P.us[J.axis][ai];
      break;
  }
  return make_float2(v.x * P.scale, v.y * P.scale);
}

// ---------------------------------------------------------------------------
// strided-axis FFT kernel
// ---------------------------------------------------------------------------
// One block (bx, by, bz) of an axis pass.
// L2 prefetch of an axis tile: rows x < n of the nc positions at base + x xs.
static __device__ __forceinline__ void axis_prefetch(const float2* buf, long long base, long long xs, int n, int nc) {
  for (int x = threadIdx.x; x < n; x += blockDim.x) {
    const float2* a = buf + base + (long long)x * xs;
    const float2* e = a + (nc - 1);
    asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
    if (((uintptr_t)a >> 7) != ((uintptr_t)e >> 7)) asm volatile("prefetch.global.L2 [%0];" ::"l"(e));
  }
}

template <int SCHED>
static __device__ __forceinline__ void axis_block(const AxisParams& P, int bx, int by, int bz) {
  extern __shared__ float4 smem_f4[];
  float2* sm = reinterpret_cast<float2*>(smem_f4);
  const int n = P.n, T = P.T;
  float2* tw = sm;
  float2* A = sm + n;
  float2* B = A + (size_t)n * T;
  float2* C = B + (size_t)n * T;
  kw_load_twiddles(tw, P.tw, P.flen);
  const int lgT = __ffs(T) - 1;  // T is a power of two
  const int c0 = bx * T;
  const int nc = min(T, P.ncols - c0);
  const long long base = (long long)by * P.os + c0;
  const int tot = n * T;

  if (P.mode < 2) {
    float2* buf = P.bufs[P.plain[bz]];
    const bool inv = P.mode == 1;
    if (nc > 0) axis_prefetch(buf, base, P.xs, n, nc);
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
      const int x = i >> lgT, cc = i & (T - 1);
      float2 v = make_float2(0.f, 0.f);
      if (cc < nc) v = buf[base + (long long)x * P.xs + cc];
      A[i] = inv ? cconj(v) : v;
    }
    float2* res = fft_smem<true, SCHED>(A, B, P.flen, T, T, 1, tw);
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
      const int x = i >> lgT, cc = i & (T - 1);
      if (cc < nc) {
        const float2 v = res[i];
        buf[base + (long long)x * P.xs + cc] = inv ? cconj(v) : v;
      }
    }
    return;
  }

  if (nc > 0)
    for (int j = 0; j < P.njobs; ++j) {
      bool seen = false;
      for (int i = 0; i < j; ++i) seen = seen || P.jobs[i].in == P.jobs[j].in;
      if (!seen) axis_prefetch(P.bufs[P.jobs[j].in], base, P.xs, n, nc);
    }
  int cur = -1;
  float2* X = A;
  for (int j = 0; j < P.njobs; ++j) {
    const AxisJob J = P.jobs[j];
    if (J.in != cur) {
      const float2* in = P.bufs[J.in];
      for (int i = threadIdx.x; i < tot; i += blockDim.x) {
        const int x = i >> lgT, cc = i & (T - 1);
        A[i] = (cc < nc) ? in[base + (long long)x * P.xs + cc] : make_float2(0.f, 0.f);
      }
      X = fft_smem<true, SCHED>(A, B, P.flen, T, T, 1, tw);
      cur = J.in;
    }
    float2* Y = (X == A) ? B : A;
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
      const int x = i >> lgT, cc = i & (T - 1);
      float2 v = make_float2(0.f, 0.f);
      if (cc < nc) {
        bool valid;
        const float2 op = axis_op(P, J, x, c0 + cc, valid);
        if (valid) v = cconj(cmul(op, X[i]));
      }
      Y[i] = v;
    }
    float2* res = fft_smem<true, SCHED>(Y, C, P.flen, T, T, 1, tw);
    float2* out = P.bufs[J.out];
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
      const int x = i >> lgT, cc = i & (T - 1);
      if (cc < nc) out[base + (long long)x * P.xs + cc] = cconj(res[i]);
    }
    __syncthreads();
  }
}

template <int SCHED>
__global__ void __launch_bounds__(256) k_axis(const __grid_constant__ AxisParams P) {
  axis_block<SCHED>(P, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ---------------------------------------------------------------------------
// grouped launches: one launch runs the same kind of pass for several plans.
// blk[i] = (first block of member i, grid x, grid y, 0), blk[n].x = total
// blocks; each block copies its member's parameters into shared memory.
// ---------------------------------------------------------------------------
static __device__ __forceinline__ int group_member(const int4* __restrict__ blk, int n) {
  __shared__ int s_member;
  if (threadIdx.x == 0) {
    int lo = 0, hi = n - 1;
    const int b = blockIdx.x;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (blk[mid].x <= b)
        lo = mid;
      else
        hi = mid - 1;
    }
    s_member = lo;
  }
  __syncthreads();
  return s_member;
}

template <class T>
static __device__ __forceinline__ void copy_params(T& dst, const T* __restrict__ src) {
  static_assert(sizeof(T) % 4 == 0, "parameter block size");
  const int* s = reinterpret_cast<const int*>(src);
  int* d = reinterpret_cast<int*>(&dst);
  for (int w = threadIdx.x; w < (int)(sizeof(T) / 4); w += blockDim.x) d[w] = s[w];
  __syncthreads();
}

template <int SCHED>
__global__ void __launch_bounds__(256) k_axis_group(const AxisParams* __restrict__ Ps, const int4* __restrict__ blk,
                                                    int n) {
  __shared__ __align__(16) AxisParams sp;
  const int i = group_member(blk, n);
  copy_params(sp, Ps + i);
  const int4 g = blk[i];
  const int b = blockIdx.x - g.x;
  axis_block<SCHED>(sp, b % g.y, (b / g.y) % g.z, b / (g.y * g.z));
}

// ---------------------------------------------------------------------------
// row helpers (block-wide)
// ---------------------------------------------------------------------------
struct RowSmem {
  float2* tw;
  float2* twp;
  float2* A;
  float2* B;
  float* rb[KW_NREAL];
};

// C2R of R rows of spectral buffer S into rbuf (unnormalised: L * x).
template <int SCHED>
static __device__ void rows_c2r(const RowsParams& P, const RowSmem& s, const float2* __restrict__ S, float* rbuf, int r0,
                         int nr) {
  const int M = P.Mfft, L = P.L, R = P.R;
  const int tot = R * M;
  for (int i = threadIdx.x; i < tot; i += blockDim.x) {
    const int row = kw_divu(i, P.dM), k = i - row * M;
    float2 z = make_float2(0.f, 0.f);
    if (row < nr) {
      const float2* sr = S + (long long)(r0 + row) * P.Hp;
      if (P.even) {
        const float2 xk = sr[k];
        const float2 xc = cconj(sr[M - k]);
        const float2 e = cadd(xk, xc);
        const float2 o = cmul(csub(xk, xc), cconj(s.twp[k]));
        z = make_float2(e.x - o.y, e.y + o.x);
      } else {
        z = (k < P.H) ? sr[k] : cconj(sr[L - k]);
      }
    }
    s.A[i] = cconj(z);
  }
  float2* res = fft_smem<false, SCHED>(s.A, s.B, P.flen, R, 1, M, s.tw);
  for (int i = threadIdx.x; i < tot; i += blockDim.x) {
    const int row = kw_divu(i, P.dM), n = i - row * M;
    const float2 v = res[i];
    if (P.even) {
      rbuf[row * L + 2 * n] = v.x;
      rbuf[row * L + 2 * n + 1] = -v.y;
    } else {
      rbuf[row * L + n] = v.x;
    }
  }
  __syncthreads();
}

// R2C of rbuf rows into spectral buffer S.
template <int SCHED>
static __device__ void rows_r2c(const RowsParams& P, const RowSmem& s, const float* rbuf, float2* __restrict__ S, int r0,
                         int nr) {
  const int M = P.Mfft, L = P.L, R = P.R, H = P.H;
  const int tot = R * M;
  for (int i = threadIdx.x; i < tot; i += blockDim.x) {
    const int row = kw_divu(i, P.dM), n = i - row * M;
    s.A[i] = P.even ? make_float2(rbuf[row * L + 2 * n], rbuf[row * L + 2 * n + 1]) : make_float2(rbuf[row * L + n], 0.f);
  }
  float2* res = fft_smem<false, SCHED>(s.A, s.B, P.flen, R, 1, M, s.tw);
  const int toth = R * H;
  for (int i = threadIdx.x; i < toth; i += blockDim.x) {
    const int row = kw_divu(i, P.dH), k = i - row * H;
    if (row >= nr) continue;
    float2 X;
    if (P.even) {
      const float2 zk = res[row * M + (k == M ? 0 : k)];
      const float2 zc = cconj(res[row * M + (k == 0 ? 0 : M - k)]);
      const float2 e = cscale(cadd(zk, zc), 0.5f);
      const float2 d = csub(zk, zc);
      const float2 o = make_float2(0.5f * d.y, -0.5f * d.x);
      X = cadd(e, cmul(s.twp[k], o));
    } else {
      X = res[row * L + k];
    }
    S[(long long)(r0 + row) * P.Hp + k] = X;
  }
  __syncthreads();
}

static __device__ __forceinline__ int axis_index(const RowsParams& P, int axis, int grow, int z) {
  if (axis == P.ndim - 1) return z;
  if (axis == 0) return (P.ndim == 3) ? grow / P.N1 : grow;
  return grow % P.N1;  // axis 1 of a 3-D grid
}

static __device__ __forceinline__ float fld(const float* p, float s, long long g) { return p ? p[g] : s; }

// Apply a sparse source to rbuf for the block's rows (kspace_solver.py:86-109).
static __device__ void apply_source(const RowsParams& P, const KwSrcDev& S, float* rbuf, int r0, int nr) {
  const int t = kw_step_t(P);
  if (!S.active || t >= S.len) return;
  const int e0 = S.row_ptr[r0], e1 = S.row_ptr[r0 + nr];
  for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const int4 en = S.ent[e];
    const float val = S.sig[(long long)t * S.nsig + (S.nsig == 1 ? 0 : en.z)];
    float& f = rbuf[(en.x - r0) * P.L + en.y];
    if (S.mode == SRC_DIRICHLET)
      f = val;
    else
      f = __fadd_rn(f, val);
  }
}

// Scatter a source's values at step t into a zeroed rbuf (the field whose
// k-space corrected version is added, kspace_solver.py:93-101).
static __device__ void scatter_source(const RowsParams& P, const KwSrcDev& S, float* rbuf, int r0, int nr) {
  const int t = kw_step_t(P);
  const int e0 = S.row_ptr[r0], e1 = S.row_ptr[r0 + nr];
  for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const int4 en = S.ent[e];
    rbuf[(en.x - r0) * P.L + en.y] = S.sig[(long long)t * S.nsig + (S.nsig == 1 ? 0 : en.z)];
  }
}

static __device__ void record_samples(const RowsParams& P, const float* rbuf, float* rec, int r0, int nr) {
  const int rr = kw_rec_row(P);
  if (rec == nullptr || rr < 0 || P.sens_row_ptr == nullptr) return;
  const int e0 = P.sens_row_ptr[r0], e1 = P.sens_row_ptr[r0 + nr];
  float* out = rec + (long long)rr * P.nslots;
  for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const int4 en = P.sens_ent[e];
    out[en.z] = rbuf[(en.x - r0) * P.L + en.y];
  }
}

// lp += S^T r at this block's sensor points (binary sensor: one slot per grid
// point; r is time-major in rec[0], row kw_rec_row(P)).
static __device__ void add_residual(const RowsParams& P, float* rbuf, int r0, int nr) {
  const int rr = kw_rec_row(P);
  const float* res = P.rec[0];
  if (res == nullptr || rr < 0 || P.sens_row_ptr == nullptr) return;
  const int e0 = P.sens_row_ptr[r0], e1 = P.sens_row_ptr[r0 + nr];
  const float* in = res + (long long)rr * P.nslots;
  for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const int4 en = P.sens_ent[e];
    float& f = rbuf[(en.x - r0) * P.L + en.y];
    f = __fadd_rn(f, in[en.z]);
  }
}

// ---------------------------------------------------------------------------
// row stage kernels: one physics body, two row-FFT implementations
// ---------------------------------------------------------------------------
// Row transforms through the shared-memory Stockham stages (any 2,3,5,7-smooth length).
template <int SCHED>
struct GenericRowFFT {
  RowSmem s;
  __device__ void c2r(const RowsParams& P, const float2* S, float* rbuf, int r0, int nr) const {
    rows_c2r<SCHED>(P, s, S, rbuf, r0, nr);
  }
  __device__ void r2c(const RowsParams& P, const float* rbuf, float2* S, int r0, int nr) const {
    rows_r2c<SCHED>(P, s, rbuf, S, r0, nr);
  }
};

// Transposed step of the lossless, source-free time loop
// (kspace_solver.py:700-723 with alpha = 0, B/A = 0).  With G_i = Re F^-1
// [op_grad_i F .], D_i = Re F^-1[op_div_i F .] and G_i^T = -D_i, one step
// back from the adjoint (lp, lu_i, lr_i) of the state after step t is
//   ADJ_A: lp += S^T r_t; lr_i' = lr_i + c^2 lp; lr_i <- m_i^2 lr_i';
//          S_i <- F[b m_i lr_i']                       (b = dt rho0)
//   (x/y passes: S_i <- op_grad_i S_i)
//   ADJ_B: lu_i' = lu_i + F^-1 S_i; lu_i <- sg_i^2 lu_i'; S_i <- F[a_i sg_i lu_i']
//   (passes: S_i <- op_div_i S_i)
//   ADJ_C: lp = sum_i F^-1 S_i
// and the transpose of the t = 0 override p = p0, rho_i = p0 / (c^2 D),
// u_i = (a_i / 2) G_i p0 gives the gradient with respect to p0:
//   ADJ_D: lp += S^T r_0; S_i <- F[(a_i / 2) lu_i]   (passes: op_div)
//   ADJ_E: g = lp + sum_i lr_i / (c^2 D) - sum_i F^-1 S_i   (into p)
// With the sound-speed gradient on (gacc set), ADJ_A also accumulates
// gacc += fsum_t lp' (fsum_t = forward sum_i rho_i after step t, so that
// p_t = c^2 fsum_t), and ADJ_E turns the c^2 gradient into the c gradient:
//   gacc <- 2 c (gacc - p0 sum_i lr_i / (c^4 D)).
template <class RF>
static __device__ __forceinline__ void adjoint_body(const RowsParams& P, const RF& rf, float* const* rb, int r0, int nr) {
  const int L = P.L, R = P.R;
  const int tot = R * L;
  const int D = P.ndim;
  if (P.stage == ST_ADJ_A || P.stage == ST_ADJ_D) {
    float* lpb = rb[D];
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
      const int row = kw_divu(i, P.dL), z = i - row * L;
      if (row < nr) lpb[i] = P.p[(long long)(r0 + row) * L + z];
    }
    __syncthreads();
    add_residual(P, lpb, r0, nr);
    __syncthreads();
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
      const int row = kw_divu(i, P.dL), z = i - row * L;
      if (row >= nr) continue;
      const long long g = (long long)(r0 + row) * L + z;
      const float lp = lpb[i];
      if (P.stage == ST_ADJ_A) {
        if (P.gacc) P.gacc[g] = __fmaf_rn(P.fsum[g], lp, P.gacc[g]);
        const float c = fld(P.c0, P.c0_s, g);
        const float c2 = __fmul_rn(c, c);
        const float b = __fmul_rn(P.dt, fld(P.rho0, P.rho0_s, g));
        for (int a = 0; a < D; ++a) {
          const float pm = P.pml[a][axis_index(P, a, r0 + row, z)];
          const float lr = __fadd_rn(P.rho[a][g], __fmul_rn(c2, lp));
          P.rho[a][g] = __fmul_rn(__fmul_rn(pm, pm), lr);
          rb[a][i] = __fmul_rn(__fmul_rn(b, pm), lr);
        }
      } else {
        P.p[g] = lp;
        for (int a = 0; a < D; ++a)
          rb[a][i] = __fmul_rn(__fmul_rn(fld(P.dtrsg[a], P.dtrsg_s[a], g), 0.5f), P.u[a][g]);
      }
    }
    __syncthreads();
    for (int a = 0; a < D; ++a) rf.r2c(P, rb[a], P.S[a], r0, nr);
    return;
  }
  if (P.stage == ST_ADJ_B) {
    for (int a = 0; a < D; ++a) {
      rf.c2r(P, P.S[a], rb[0], r0, nr);
      for (int i = threadIdx.x; i < tot; i += blockDim.x) {
        const int row = kw_divu(i, P.dL), z = i - row * L;
        if (row >= nr) continue;
        const long long g = (long long)(r0 + row) * L + z;
        const float sg = P.pmlsg[a][axis_index(P, a, r0 + row, z)];
        const float lu = __fadd_rn(P.u[a][g], rb[0][i]);
        P.u[a][g] = __fmul_rn(__fmul_rn(sg, sg), lu);
        rb[0][i] = __fmul_rn(__fmul_rn(fld(P.dtrsg[a], P.dtrsg_s[a], g), sg), lu);
      }
      __syncthreads();
      rf.r2c(P, rb[0], P.S[a], r0, nr);
      __syncthreads();
    }
    return;
  }
  // ST_ADJ_C / ST_ADJ_E
  for (int a = 0; a < D; ++a) rf.c2r(P, P.S[a], rb[a], r0, nr);
  for (int i = threadIdx.x; i < tot; i += blockDim.x) {
    const int row = kw_divu(i, P.dL), z = i - row * L;
    if (row >= nr) continue;
    const long long g = (long long)(r0 + row) * L + z;
    float s = rb[0][i];
    for (int a = 1; a < D; ++a) s = __fadd_rn(s, rb[a][i]);
    if (P.stage == ST_ADJ_C) {
      P.p[g] = s;
    } else {
      const float c = fld(P.c0, P.c0_s, g);
      const float den = __fmul_rn(__fmul_rn(c, c), (float)D);
      float acc = P.p[g];
      for (int a = 0; a < D; ++a) acc = __fadd_rn(acc, __fdiv_rn(P.rho[a][g], den));
      P.p[g] = __fsub_rn(acc, s);
      if (P.gacc) {
        float lr = P.rho[0][g];
        for (int a = 1; a < D; ++a) lr = __fadd_rn(lr, P.rho[a][g]);
        const float ov = __fdiv_rn(__fmul_rn(P.p0[g], lr), __fmul_rn(den, __fmul_rn(c, c)));
        P.gacc[g] = __fmul_rn(__fmul_rn(2.f, c), __fsub_rn(P.gacc[g], ov));
      }
    }
  }
}

// The stage physics of one block of R rows; rb[q] are R*L real buffers in
// shared memory.  Every rf call starts and ends with a block-wide barrier.
// ---------------------------------------------------------------------------
// L2 prefetch of a block's inputs.  The element loops of the generic kernels
// issue one global load per element and iteration, so a block otherwise waits
// on DRAM latency iteration after iteration; prefetching the block's ranges
// when it starts turns those waits into L2 hits.
// ---------------------------------------------------------------------------
// The 128-byte lines of [base + off, base + off + nbytes) (base may be null).
// The first line is rounded down to its 128-byte boundary, which stays inside
// an allocation that starts 256-byte aligned.
static __device__ __forceinline__ void pf_lines(const void* base, long long off, long long nbytes) {
  if (base == nullptr || nbytes <= 0) return;
  const uintptr_t a0 = ((uintptr_t)base + (uintptr_t)off) & ~(uintptr_t)127;
  const uintptr_t a1 = (uintptr_t)base + (uintptr_t)(off + nbytes);
  for (uintptr_t a = a0 + (uintptr_t)threadIdx.x * 128; a < a1; a += (uintptr_t)blockDim.x * 128)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
}

// Rows r0 .. r0 + nr - 1 of the arrays a row stage reads.
static __device__ __forceinline__ void rows_prefetch(const RowsParams& P, int r0, int nr) {
  const long long sro = (long long)r0 * P.Hp * 8, srn = (long long)nr * P.Hp * 8;
  const long long fro = (long long)r0 * P.L * 4, frn = (long long)nr * P.L * 4;
  const int D = P.ndim;
  if (P.stage == ST_U) {
    for (int a = 0; a < D; ++a) {
      pf_lines(P.S[a], sro, srn);
      if (!P.init) pf_lines(P.u[a], fro, frn);
      pf_lines(P.dtrsg[a], fro, frn);
    }
  } else if (P.stage == ST_RHO) {
    for (int a = 0; a < D; ++a) {
      pf_lines(P.S[a], sro, srn);
      pf_lines(P.rho[a], fro, frn);
    }
    pf_lines(P.rho0, fro, frn);
    if (P.absorb != 1) {
      pf_lines(P.c0, fro, frn);
      if (P.absorb == 2) pf_lines(P.tau, fro, frn);
      if (P.nonlin) pf_lines(P.bona, fro, frn);
    }
  } else if (P.stage == ST_EOS) {
    pf_lines(P.S[0], sro, srn);
    if (P.disp) pf_lines(P.S[1], sro, srn);
    pf_lines(P.rho_sum, fro, frn);
    pf_lines(P.c0, fro, frn);
    pf_lines(P.tau, fro, frn);
    if (P.disp) pf_lines(P.eta, fro, frn);
    if (P.nonlin) {
      pf_lines(P.rho0, fro, frn);
      pf_lines(P.bona, fro, frn);
    }
  }
}

template <class RF>
static __device__ __forceinline__ void rows_body(const RowsParams& P, const RF& rf, float* const* rb, int bx) {
  const int L = P.L, R = P.R;
  const int r0 = bx * R;
  const int nr = min(R, P.nrows - r0);
  const int tot = R * L;
  const int D = P.ndim;
  if (nr > 0) rows_prefetch(P, r0, nr);

  if (P.stage == ST_INIT) {
    // t = 0 with p0: p = p0, rho_i = p0 / (c0^2 D) (kspace_solver.py:729-733)
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
      const int row = kw_divu(i, P.dL), z = i - row * L;
      if (row >= nr) continue;
      const long long g = (long long)(r0 + row) * L + z;
      const float pv = P.p0_scale ? __fmul_rn(P.p0[g], *P.p0_scale) : P.p0[g];
      const float c = fld(P.c0, P.c0_s, g);
      const float c2 = __fmul_rn(c, c);
      const float r = __fdiv_rn(pv, __fmul_rn(c2, (float)D));
      for (int a = 0; a < D; ++a) P.rho[a][g] = r;
      if (P.write_p) P.p[g] = pv;
      rb[0][i] = pv;
    }
    __syncthreads();
    record_samples(P, rb[0], P.rec[0], r0, nr);
    rf.r2c(P, rb[0], P.S[3], r0, nr);
    return;
  }

  if (P.stage == ST_U) {
    // momentum: u_i = pml_sg (pml_sg u_i - dt/rho_sg g_i) (kspace_solver.py:703-707)
    for (int a = 0; a < D; ++a) {
      rf.c2r(P, P.S[a], rb[0], r0, nr);
      float* u = P.u[a];
      for (int i = threadIdx.x; i < tot; i += blockDim.x) {
        const int row = kw_divu(i, P.dL), z = i - row * L;
        if (row >= nr) continue;
        const long long g = (long long)(r0 + row) * L + z;
        const float gr = rb[0][i];
        const float dtr = fld(P.dtrsg[a], P.dtrsg_s[a], g);
        float nu;
        if (P.init) {
          nu = __fmul_rn(__fmul_rn(dtr, 0.5f), gr);
        } else {
          const float sg = P.pmlsg[a][axis_index(P, a, r0 + row, z)];
          nu = __fmul_rn(sg, __fsub_rn(__fmul_rn(sg, u[g]), __fmul_rn(dtr, gr)));
        }
        rb[0][i] = nu;
      }
      __syncthreads();
      if (!P.init) {
        if (P.srcu_on[a]) {
          // u_i += Re F^-1[source_kappa F[s_i]] (kspace_solver.py:91-98)
          rf.c2r(P, P.S[B_SRCU0 + a], rb[1], r0, nr);
          for (int i = threadIdx.x; i < tot; i += blockDim.x) rb[0][i] = __fadd_rn(rb[0][i], rb[1][i]);
        } else {
          apply_source(P, P.src[3 + a], rb[0], r0, nr);
        }
      }
      __syncthreads();
      for (int i = threadIdx.x; i < tot; i += blockDim.x) {
        const int row = kw_divu(i, P.dL), z = i - row * L;
        if (row >= nr) continue;
        u[(long long)(r0 + row) * L + z] = rb[0][i];
      }
      record_samples(P, rb[0], P.rec[1 + a], r0, nr);
      if (!P.init || P.init_r2c) rf.r2c(P, rb[0], P.S[a], r0, nr);
      __syncthreads();
    }
    return;
  }

  if (P.stage == ST_RHO) {
    // mass conservation with split density (kspace_solver.py:709-717)
    for (int a = 0; a < D; ++a) rf.c2r(P, P.S[a], rb[a], r0, nr);
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
      const int row = kw_divu(i, P.dL), z = i - row * L;
      if (row >= nr) continue;
      const long long g = (long long)(r0 + row) * L + z;
      const float r0v = fld(P.rho0, P.rho0_s, g);
      float nl = 1.f;
      if (P.nonlin) {
        float sr = P.rho[0][g];
        for (int a = 1; a < D; ++a) sr = __fadd_rn(sr, P.rho[a][g]);
        nl = __fdiv_rn(__fadd_rn(__fmul_rn(2.f, sr), r0v), r0v);
      }
      float div = 0.f;
      const float dtr0 = __fmul_rn(P.dt, r0v);
      for (int a = 0; a < D; ++a) {
        const float du = rb[a][i];
        div = __fadd_rn(div, du);
        const float pm = P.pml[a][axis_index(P, a, r0 + row, z)];
        const float term = __fmul_rn(__fmul_rn(dtr0, du), nl);
        rb[a][i] = __fmul_rn(pm, __fsub_rn(__fmul_rn(pm, P.rho[a][g]), term));
      }
      rb[3][i] = div;
    }
    __syncthreads();
    if (P.srcp_on) {
      // rho_i += Re F^-1[source_kappa F[s]] / d_i (kspace_solver.py:91-98, scale :619-624)
      rf.c2r(P, P.S[B_SRCP], rb[4], r0, nr);
      for (int i = threadIdx.x; i < tot; i += blockDim.x)
        for (int a = 0; a < D; ++a) rb[a][i] = __fadd_rn(rb[a][i], __fmul_rn(rb[4][i], P.inv_d[a]));
    } else {
      for (int a = 0; a < D; ++a) apply_source(P, P.src[a], rb[a], r0, nr);
    }
    __syncthreads();
    const bool powerlaw = P.absorb == 1;
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
      const int row = kw_divu(i, P.dL), z = i - row * L;
      if (row >= nr) continue;
      const long long g = (long long)(r0 + row) * L + z;
      float rs = rb[0][i];
      P.rho[0][g] = rs;
      for (int a = 1; a < D; ++a) {
        const float ra = rb[a][i];
        P.rho[a][g] = ra;
        rs = __fadd_rn(rs, ra);
      }
      const float div = rb[3][i];
      const float r0v = fld(P.rho0, P.rho0_s, g);
      if (powerlaw) {
        P.rho_sum[g] = rs;
        rb[0][i] = __fmul_rn(r0v, div);
        rb[1][i] = rs;
      } else {
        // equation of state without fractional Laplacians (kspace_solver.py:719-723)
        const float c = fld(P.c0, P.c0_s, g);
        const float c2 = __fmul_rn(c, c);
        float acc = rs;
        if (P.absorb == 2) acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(fld(P.tau, P.tau_s, g), r0v), div));
        if (P.nonlin) {
          const float nlt = __fdiv_rn(__fmul_rn(fld(P.bona, P.bona_s, g), __fmul_rn(rs, rs)), __fmul_rn(2.f, r0v));
          acc = __fadd_rn(acc, nlt);
        }
        const float pv = __fmul_rn(c2, acc);
        if (P.write_p) P.p[g] = pv;
        rb[0][i] = pv;
      }
    }
    __syncthreads();
    if (powerlaw) {
      rf.r2c(P, rb[0], P.S[0], r0, nr);
      if (P.disp) rf.r2c(P, rb[1], P.S[1], r0, nr);
    } else {
      record_samples(P, rb[0], P.rec[0], r0, nr);
      rf.r2c(P, rb[0], P.S[3], r0, nr);
    }
    if (P.rec_us) {
      // velocity on the pressure grid, Re F^-1[e^{-i k d/2} F[u_i]] (kspace_solver.py:740-743)
      for (int a = 0; a < D; ++a) {
        if (!(P.rec_us & (1 << a))) continue;
        rf.c2r(P, P.S[B_US0 + a], rb[4], r0, nr);
        record_samples(P, rb[4], P.rec[4 + a], r0, nr);
        __syncthreads();
      }
    }
    return;
  }

  if (P.stage == ST_SRC) {
    // scattered source fields of this step, transformed for the source-kappa pass
    if (P.srcp_on) {
      for (int i = threadIdx.x; i < tot; i += blockDim.x) rb[0][i] = 0.f;
      __syncthreads();
      scatter_source(P, P.src[0], rb[0], r0, nr);
      __syncthreads();
      rf.r2c(P, rb[0], P.S[B_SRCP], r0, nr);
    }
    for (int a = 0; a < D; ++a) {
      if (!P.srcu_on[a]) continue;
      for (int i = threadIdx.x; i < tot; i += blockDim.x) rb[0][i] = 0.f;
      __syncthreads();
      scatter_source(P, P.src[3 + a], rb[0], r0, nr);
      __syncthreads();
      rf.r2c(P, rb[0], P.S[B_SRCU0 + a], r0, nr);
    }
    return;
  }

  if (P.stage == ST_P0FFT) {
    // spectrum of p0 for the smoothing window
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
      const int row = kw_divu(i, P.dL), z = i - row * L;
      rb[0][i] = (row < nr) ? P.p0w[(long long)(r0 + row) * L + z] : 0.f;
    }
    __syncthreads();
    rf.r2c(P, rb[0], P.S[B_P], r0, nr);
    return;
  }

  if (P.stage == ST_P0BACK) {
    rf.c2r(P, P.S[B_P], rb[0], r0, nr);
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
      const int row = kw_divu(i, P.dL), z = i - row * L;
      if (row < nr) P.p0w[(long long)(r0 + row) * L + z] = rb[0][i];
    }
    return;
  }

  if (P.stage >= ST_ADJ_A) {
    adjoint_body(P, rf, rb, r0, nr);
    return;
  }

  if (P.stage == ST_UREC) {
    for (int a = 0; a < D; ++a) {
      if (!(P.rec_us & (1 << a))) continue;
      rf.c2r(P, P.S[B_US0 + a], rb[0], r0, nr);
      record_samples(P, rb[0], P.rec[4 + a], r0, nr);
      __syncthreads();
    }
    return;
  }

  // ST_EOS: p = c0^2 (rho + tau F^-1[nabla1 F[rho0 div]] - eta F^-1[nabla2 F[rho]] + B/A rho^2 / (2 rho0))
  rf.c2r(P, P.S[0], rb[0], r0, nr);
  if (P.disp) rf.c2r(P, P.S[1], rb[1], r0, nr);
  for (int i = threadIdx.x; i < tot; i += blockDim.x) {
    const int row = kw_divu(i, P.dL), z = i - row * L;
    if (row >= nr) continue;
    const long long g = (long long)(r0 + row) * L + z;
    const float rs = P.rho_sum[g];
    const float c = fld(P.c0, P.c0_s, g);
    const float c2 = __fmul_rn(c, c);
    float acc = __fadd_rn(rs, __fmul_rn(fld(P.tau, P.tau_s, g), rb[0][i]));
    if (P.disp) acc = __fsub_rn(acc, __fmul_rn(fld(P.eta, P.eta_s, g), rb[1][i]));
    if (P.nonlin) {
      const float r0v = fld(P.rho0, P.rho0_s, g);
      const float nlt = __fdiv_rn(__fmul_rn(fld(P.bona, P.bona_s, g), __fmul_rn(rs, rs)), __fmul_rn(2.f, r0v));
      acc = __fadd_rn(acc, nlt);
    }
    const float pv = __fmul_rn(c2, acc);
    if (P.write_p) P.p[g] = pv;
    rb[0][i] = pv;
  }
  __syncthreads();
  record_samples(P, rb[0], P.rec[0], r0, nr);
  rf.r2c(P, rb[0], P.S[3], r0, nr);
}

template <int SCHED>
static __device__ __forceinline__ void rows_block(const RowsParams& P, int bx) {
  extern __shared__ float4 smem_f4[];
  const int M = P.Mfft, L = P.L, R = P.R;
  GenericRowFFT<SCHED> rf;
  RowSmem& s = rf.s;
  s.tw = reinterpret_cast<float2*>(smem_f4);
  s.twp = s.tw + M;
  s.A = s.twp + (L / 2 + 1);
  s.B = s.A + (size_t)R * M;
  float* rbase = reinterpret_cast<float*>(s.B + (size_t)R * M);
  for (int q = 0; q < KW_NREAL; ++q) s.rb[q] = rbase + (size_t)q * R * L;
  kw_load_twiddles(s.tw, P.tw, P.flen);
  if (P.even)
    for (int i = threadIdx.x; i <= L / 2; i += blockDim.x) s.twp[i] = P.twpost[i];
  __syncthreads();  // the row transforms read twp before their first barrier
  rows_body(P, rf, s.rb, bx);
}

template <int SCHED>
__global__ void __launch_bounds__(256) k_rows(const __grid_constant__ RowsParams P) {
  rows_block<SCHED>(P, blockIdx.x);
}

template <int SCHED>
__global__ void __launch_bounds__(256) k_rows_group(const RowsParams* __restrict__ Ps, const int4* __restrict__ blk,
                                                    int n) {
  __shared__ __align__(16) RowsParams sp;
  const int i = group_member(blk, n);
  copy_params(sp, Ps + i);
  rows_block<SCHED>(sp, blockIdx.x - blk[i].x);
}

// Host launchers of schedule family F (declared in kw_kernels.cuh); expanded
// once in the translation unit that instantiates F.
#define KW_GENERIC_DEFINE(F)                                                                                      \
  cudaError_t kw_generic_attr_##F(int smem_max) {                                                                 \
    cudaError_t e = cudaFuncSetAttribute(k_rows<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max);       \
    if (e == cudaSuccess)                                                                                         \
      e = cudaFuncSetAttribute(k_axis<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max);                 \
    if (e == cudaSuccess)                                                                                         \
      e = cudaFuncSetAttribute(k_rows_group<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max);           \
    if (e == cudaSuccess)                                                                                         \
      e = cudaFuncSetAttribute(k_axis_group<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max);           \
    return e;                                                                                                     \
  }                                                                                                               \
  cudaError_t kw_rows_launch_##F(dim3 grid, size_t smem, cudaStream_t st, const RowsParams& P) {                  \
    k_rows<F><<<grid, 256, smem, st>>>(P);                                                                        \
    return cudaGetLastError();                                                                                    \
  }                                                                                                               \
  cudaError_t kw_axis_launch_##F(dim3 grid, size_t smem, cudaStream_t st, const AxisParams& A) {                  \
    k_axis<F><<<grid, 256, smem, st>>>(A);                                                                        \
    return cudaGetLastError();                                                                                    \
  }                                                                                                               \
  cudaError_t kw_rows_group_launch_##F(int nblk, size_t smem, cudaStream_t st, const RowsParams* Ps, const int4* blk, \
                                       int n) {                                                                   \
    k_rows_group<F><<<nblk, 256, smem, st>>>(Ps, blk, n);                                                         \
    return cudaGetLastError();                                                                                    \
  }                                                                                                               \
  cudaError_t kw_axis_group_launch_##F(int nblk, size_t smem, cudaStream_t st, const AxisParams* Ps, const int4* blk, \
                                       int n) {                                                                   \
    k_axis_group<F><<<nblk, 256, smem, st>>>(Ps, blk, n);                                                         \
    return cudaGetLastError();                                                                                    \
  }
