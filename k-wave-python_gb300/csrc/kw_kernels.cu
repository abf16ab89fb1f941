// Kernels of the k-space first-order time loop (see kw_kernels.cuh).
//
// Arithmetic order inside the physics follows kwave/solvers/kspace_solver.py
// (Simulation.step, :691-747) operation by operation, with explicit
// round-to-nearest intrinsics so that the compiler does not contract the
// reference's separate multiplies and adds into FMAs.
#include "kw_generic.cuh"
#include "kw_regfft.cuh"

// The generic-length row and axis kernels (kw_generic.cuh), Stockham schedule.
KW_GENERIC_DEFINE(0)

__global__ void k_step_tick_group(int* const* __restrict__ tdev, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) *tdev[i] += 1;
}

// ---------------------------------------------------------------------------
// register-FFT variants for power-of-two lengths (kw_regfft.cuh)
// ---------------------------------------------------------------------------
// Spectral operator value at x-frequency index x of a column (register axis pass).
__device__ __forceinline__ float2 col_op(const AxisParams& A, const AxisJob& J, int x, const ColK& g) {
  const float kx = A.k[0][x];
  float kk = __fadd_rn(__fmul_rn(kx, kx), g.ky2);
  if (A.ndim == 3) kk = __fadd_rn(kk, g.kz2);
  const float kmag = sqrtf(kk);
  const int ai = (J.axis == 0) ? x : (J.axis == 1 ? g.a1 : g.a2);
  float2 v;
  switch (J.op) {
    case OP_GRAD:
    case OP_DIV: {
      float kappa = 1.f;
      if (A.use_kspace) {
        const float arg = A.kcoef * kmag;
        kappa = (arg == 0.f) ? 1.f : sinf(arg) / arg;
      }
      const float2 f = (J.op == OP_GRAD) ? A.fg[J.axis][ai] : A.fd[J.axis][ai];
      v = make_float2(f.x * kappa, f.y * kappa);
      break;
    }
    case OP_NAB1:
    case OP_NAB2: {
      const float e = (J.op == OP_NAB1) ? A.pow1 : A.pow2;
      v = make_float2(kmag == 0.f ? 0.f : powf(kmag, e), 0.f);
      break;
    }
    case OP_SKAPPA:
      v = make_float2(A.use_kspace ? cosf(A.kcoef * kmag) : 1.f, 0.f);
      break;
    case OP_WIN: {
      float r2 = A.wc[0][x] + A.wc[1][g.a1];
      if (A.ndim == 3) r2 += A.wc[2][g.a2];
      v = make_float2(window_at(A.wtab, A.wlen, A.wrad, r2), 0.f);
      break;
    }
    default:
      v = A.us[J.axis][ai];
      break;
  }
  return make_float2(v.x * A.scale, v.y * A.scale);
}

// Strided axis: T = 256 / P columns per block, P threads per column.
template <int E, int P>
__global__ void __launch_bounds__(256) k_axis_reg(const __grid_constant__ AxisParams A) {
  constexpr int N = E * P, T = 256 / P, RS = N + E + 1;
  extern __shared__ float4 smem_f4[];
  float2* tw = reinterpret_cast<float2*>(smem_f4);
  float2* ex = tw + N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = A.tw[i];
  __syncthreads();
  const int cc = threadIdx.x % T, t = threadIdx.x / T;
  const int c0 = blockIdx.x * T;
  const bool act = cc < A.ncols - c0;
  const long long base = (long long)blockIdx.y * A.os + c0 + cc;
  const long long xs = A.xs;
  float2* sm = ex + cc * RS;
  auto sync = [] __device__() { __syncthreads(); };
  if (A.mode < 2) {
    float2* buf = A.bufs[A.plain[blockIdx.z]];
    float2 v[E];
    if (A.mode == 0) {
#pragma unroll
      for (int j = 0; j < E; ++j) v[j] = act ? buf[base + (t + P * j) * xs] : make_float2(0.f, 0.f);
      kwreg::Reg<E, P>::fwd(v, t, sm, 1, tw, sync);
      if (act) {
#pragma unroll
        for (int m = 0; m < E / P; ++m)
#pragma unroll
          for (int k2 = 0; k2 < P; ++k2) buf[base + (t + P * m + E * k2) * xs] = v[m * P + k2];
      }
    } else {
#pragma unroll
      for (int m = 0; m < E / P; ++m)
#pragma unroll
        for (int k2 = 0; k2 < P; ++k2)
          v[m * P + k2] = act ? cconj(buf[base + (t + P * m + E * k2) * xs]) : make_float2(0.f, 0.f);
      kwreg::Reg<E, P>::rev(v, t, sm, 1, tw, sync);
      if (act) {
#pragma unroll
        for (int j = 0; j < E; ++j) buf[base + (t + P * j) * xs] = cconj(v[j]);
      }
    }
    return;
  }
  const ColK g = col_geometry(A, act ? c0 + cc : c0);
  int cur = -1;
  float2 X[E];
  for (int jj = 0; jj < A.njobs; ++jj) {
    const AxisJob J = A.jobs[jj];
    if (J.in != cur) {
      const float2* in = A.bufs[J.in];
#pragma unroll
      for (int j = 0; j < E; ++j) X[j] = act ? in[base + (t + P * j) * xs] : make_float2(0.f, 0.f);
      kwreg::Reg<E, P>::fwd(X, t, sm, 1, tw, sync);
      cur = J.in;
    }
    float2 Y[E];
#pragma unroll
    for (int m = 0; m < E / P; ++m)
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) {
        float2 y = make_float2(0.f, 0.f);
        if (act && g.valid) y = cconj(cmul(col_op(A, J, t + P * m + E * k2, g), X[m * P + k2]));
        Y[m * P + k2] = y;
      }
    kwreg::Reg<E, P>::rev(Y, t, sm, 1, tw, sync);
    if (act) {
      float2* out = A.bufs[J.out];
#pragma unroll
      for (int j = 0; j < E; ++j) out[base + (t + P * j) * xs] = cconj(Y[j]);
    }
  }
}

// Host-side dispatch of the register kernels (launched from this translation
// unit, where the templates are instantiated).
bool kw_reg_shape(int n, int* E, int* P) {
  switch (n) {
    case 64: *E = 16; *P = 4; return true;
    case 128: *E = 16; *P = 8; return true;
    case 256: *E = 16; *P = 16; return true;
    case 512: *E = 32; *P = 16; return true;
    case 1024: *E = 32; *P = 32; return true;
    default: return false;
  }
}

#define KW_REG_SWITCH(n, CALL)             \
  switch (n) {                             \
    case 64: return CALL(16, 4);           \
    case 128: return CALL(16, 8);          \
    case 256: return CALL(16, 16);         \
    case 512: return CALL(32, 16);         \
    case 1024: return CALL(32, 32);        \
    default: return cudaErrorInvalidValue; \
  }

cudaError_t kw_axis_reg_attr(int n) {
#define KW_A(E, P) cudaFuncSetAttribute(k_axis_reg<E, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024)
  KW_REG_SWITCH(n, KW_A)
#undef KW_A
}

cudaError_t kw_axis_reg_launch(int n, dim3 grid, size_t smem, cudaStream_t st, const AxisParams& A) {
#define KW_A(E, P) (k_axis_reg<E, P><<<grid, 256, smem, st>>>(A), cudaGetLastError())
  KW_REG_SWITCH(n, KW_A)
#undef KW_A
}


// ---------------------------------------------------------------------------
// device step counter of replayed step graphs
// ---------------------------------------------------------------------------
__global__ void k_density_sum(float* __restrict__ out, const float* __restrict__ r0, const float* __restrict__ r1,
                              const float* __restrict__ r2, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float s = __fadd_rn(r0[i], r1[i]);
    if (r2) s = __fadd_rn(s, r2[i]);
    out[i] = s;
  }
}

__global__ void k_step_set(int* tdev, int t) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *tdev = t;
}

__global__ void k_loop_set(int* left, int n) { *left = n; }

// End of one pass through a loop graph's body: count the pass and keep the
// while-condition set while passes remain.
__global__ void k_loop_tick(cudaGraphConditionalHandle h, int* left) {
  const int v = --(*left);
  cudaGraphSetConditional(h, v > 0 ? 1u : 0u);
}

__global__ void k_step_tick(int* tdev) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *tdev += 1;
}

// ---------------------------------------------------------------------------
// p0 smoothing helpers (kwave/utils/filters.py:613-614, restore_max)
// ---------------------------------------------------------------------------
__global__ void k_absmax(const float* __restrict__ x, long long n, unsigned int* out) {
  float m = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(x[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

__global__ void k_ratio(const unsigned int* a, const unsigned int* b, float* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const float den = __uint_as_float(*b);
    *out = den > 0.f ? __uint_as_float(*a) / den : 1.f;
  }
}

// ---------------------------------------------------------------------------
// recorder post-processing (kspace_solver.py:335-359, :824-837)
// ---------------------------------------------------------------------------
// out[pt][t] = sum_c w[pt][c] * rec[t][slot[pt][c]]  (ncorner == 0: out[pt][t] = rec[t][pt])
__global__ void k_series_gather(const float* __restrict__ rec, int nrec, int nslots, int npts, int ncorner,
                                const int* __restrict__ slot, const double* __restrict__ w, float* __restrict__ out) {
  const long long tot = (long long)npts * nrec;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const int pt = (int)(i / nrec), t = (int)(i - (long long)pt * nrec);
    if (ncorner == 0) {
      out[i] = rec[(long long)t * nslots + pt];
    } else {
      double acc = 0.0;
      for (int c = 0; c < ncorner; ++c)
        acc += w[(long long)pt * ncorner + c] * (double)rec[(long long)t * nslots + slot[(long long)pt * ncorner + c]];
      out[i] = (float)acc;
    }
  }
}

__global__ void k_series_reduce(const float* __restrict__ series, int npts, int nrec, int kind, float* __restrict__ out) {
  const int pt = blockIdx.x * blockDim.x + threadIdx.x;
  if (pt >= npts) return;
  const float* s = series + (long long)pt * nrec;
  if (kind == 2) {
    double acc = 0.0;
    for (int t = 0; t < nrec; ++t) {
      const float v = s[t];
      const float v2 = v * v;
      acc += (double)v2;
    }
    out[pt] = sqrtf((float)(acc / nrec));
  } else {
    float m = s[0];
    for (int t = 1; t < nrec; ++t) m = (kind == 0) ? fmaxf(m, s[t]) : fminf(m, s[t]);
    out[pt] = m;
  }
}

// Medium grids of the time loop derived from c0 / rho0 / alpha on the device,
// following the reference's float32 arithmetic (kspace_solver.py:655-666 with
// float32 rho0: rho_sg = 0.5 (rho_i + rho_i+1), the last plane copied, then
// dt / rho_sg; :471-524 and kwave/utils/conversion.py:20-35 for tau / eta,
// whose db2neper divides by a float64 scalar, so they are formed in double).
__global__ void k_derive_medium(const __grid_constant__ DeriveParams D) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long st[3] = {1, 1, 1};
  if (D.ndim == 3) {
    st[0] = (long long)D.N[1] * D.N[2];
    st[1] = D.N[2];
  } else {
    st[0] = D.N[1];
  }
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < D.ntot; i += stride) {
    if (D.dtrsg[0]) {
      const float r = D.rho0[i];
      long long rem = i;
      for (int a = 0; a < D.ndim; ++a) {
        const long long ca = rem / st[a];
        rem -= ca * st[a];
        float rs = r;
        if (D.use_sg && ca < D.N[a] - 1) rs = __fmul_rn(0.5f, __fadd_rn(r, D.rho0[i + st[a]]));
        D.dtrsg[a][i] = __fdiv_rn(D.dt_f, rs);
      }
    }
    if (D.tau || D.eta) {
      const float c = D.c0 ? D.c0[i] : D.c0_s;
      double a_np;
      if (D.alpha) {
        // float32 array arithmetic of db2neper up to its float64 divisor
        a_np = (double)__fmul_rn(__fmul_rn(100.f, D.alpha[i]), D.db_fac_f) / D.db_div;
      } else {
        a_np = 100.0 * D.alpha_s * D.db_fac / D.db_div;
      }
      if (D.tau) {
        const double cp = (D.absorb == 2) ? (double)c : (double)powf(c, (float)(D.y - 1.0));
        D.tau[i] = (float)(-2.0 * a_np * cp);
      }
      if (D.eta) D.eta[i] = (float)(2.0 * a_np * (double)powf(c, (float)D.y) * D.tan_fac);
    }
  }
}
