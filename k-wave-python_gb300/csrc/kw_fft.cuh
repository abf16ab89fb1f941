// Shared-memory Stockham FFT building blocks for the k-space solver.
//
// Every transform here is a forward, unnormalised DFT
//     X[k] = sum_n x[n] exp(-2 pi i k n / N)
// computed as a sequence of Stockham autosort stages of radix 2, 3, 4, 5 or 7
// (no bit reversal).  Inverse transforms are taken as conj(DFT(conj(x))), so
// the conjugations fold into the load/store of the caller.  Normalisation is
// left to the caller: the spectral operators carry the 1/N of the full N-D
// inverse transform.
//
// Stage s with radix r and p = product of the radices of earlier stages maps
// butterfly j (0 <= j < N/r), k = j mod p:
//     y_t = in[j + t N/r] * w^(t k N/(p r)),  t < r
//     out[(j - k) r + k + q p] = sum_t y_t exp(-2 pi i t q / r),  q < r
// with w = exp(-2 pi i / N) read from a per-length table computed in FP64 on
// the host and stored in FP32.
//
// A length that factors as N = n1 n2 with both factors in KW_FFT2_SIZES can
// instead take the two-level schedule (fft2_smem): n1 register DFTs of n2
// points, one twiddle multiply, n2 register DFTs of n1 points; two passes
// over shared memory instead of one per radix.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <utility>

#define KW_MAX_STAGES 16
#define KW_RADIX_ORDERS 4  // FFT schedules a plan can use: three Stockham radix orders (kw_plan.cu:
                           // kRadixOrders) and the two-level schedule

// x / d for 0 <= x < 2^31 and 1 <= d < 2^31 as a multiply-high, an add and a
// shift: m = floor(2^32 (2^l - d) / d) + 1 with l = ceil(log2 d) (the
// round-up reciprocal of Granlund and Montgomery, "Division by invariant
// integers using multiplication", PLDI 1994).
struct KwDivU {
  uint32_t m, s;
};

__host__ __device__ inline KwDivU kw_divu_make(uint32_t d) {
  uint32_t l = 0;
  while ((1ull << l) < d) ++l;
  KwDivU r;
  r.s = l;
  r.m = (uint32_t)(((((unsigned long long)1 << l) - d) << 32) / d + 1);
  return r;
}

__device__ __forceinline__ int kw_divu(int x, KwDivU D) {
  return (int)((__umulhi((uint32_t)x, D.m) + (uint32_t)x) >> D.s);
}

struct KwFftLen {
  int n;                      // transform length
  int nst;                    // number of stages
  int radix[KW_MAX_STAGES];   // radices in stage order
  KwDivU dt[KW_MAX_STAGES];   // stage s: division by n / radix[s]
  KwDivU dp[KW_MAX_STAGES];   // stage s: division by the product of the earlier radices
  int n1, n2;                 // two-level schedule n = n1 n2 (n1 = 0: Stockham stages)
  KwDivU d1, d2;              // division by n1, by n2
};

// Fill the per-stage divisors once the radices are set (Stockham schedule).
inline void kw_fft_len_finish(KwFftLen& f) {
  int p = 1;
  for (int s = 0; s < f.nst; ++s) {
    f.dt[s] = kw_divu_make((uint32_t)(f.n / f.radix[s]));
    f.dp[s] = kw_divu_make((uint32_t)p);
    p *= f.radix[s];
  }
  f.n1 = f.n2 = 0;
  f.d1 = f.d2 = kw_divu_make(1);
}

// Sizes of the register DFTs of the two-level schedule: the 5-smooth sizes up
// to 20, so that lengths up to 400 qualify.  (Sizes up to 32 would take every
// 5-smooth length up to 1024, but the 24..32-point DFTs raise the row and axis
// kernels from 64 to 106-128 registers.)
#define KW_FFT2_SIZES(X) X(2) X(3) X(4) X(5) X(6) X(8) X(9) X(10) X(12) X(15) X(16) X(18) X(20)

inline bool kw_fft2_size_ok(int n) {
  switch (n) {
#define KW_FFT2_CASE(N) case N:
    KW_FFT2_SIZES(KW_FFT2_CASE)
#undef KW_FFT2_CASE
    return true;
    default:
      return false;
  }
}

// Two-level schedule for n when n = n1 n2 with both factors register-DFT
// sizes: the most balanced split (smallest larger factor), n1 <= n2.  Keeps
// the Stockham fields as they are; returns false (and leaves n1 = 0) when no
// split exists.
inline bool kw_fft_len_two_level(KwFftLen& f) {
  const int n = f.n;
  int best = 0;
  for (int a = 2; a * a <= n; ++a)
    if (n % a == 0 && kw_fft2_size_ok(a) && kw_fft2_size_ok(n / a)) best = a;
  if (!best) return false;
  f.n1 = best;
  f.n2 = n / best;
  f.d1 = kw_divu_make((uint32_t)f.n1);
  f.d2 = kw_divu_make((uint32_t)f.n2);
  return true;
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(__fsub_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                     __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by -i
__device__ __forceinline__ float2 cmul_mi(float2 a) { return make_float2(a.y, -a.x); }

// Small forward DFTs in registers.  Constants are cos/sin of 2 pi / r.
template <int R>
__device__ __forceinline__ void dft_small(float2* v);

template <>
__device__ __forceinline__ void dft_small<2>(float2* v) {
  float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <>
__device__ __forceinline__ void dft_small<4>(float2* v) {
  float2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
  float2 b0 = cadd(v[1], v[3]), b1 = cmul_mi(csub(v[1], v[3]));
  v[0] = cadd(a0, b0);
  v[2] = csub(a0, b0);
  v[1] = cadd(a1, b1);
  v[3] = csub(a1, b1);
}

template <>
__device__ __forceinline__ void dft_small<3>(float2* v) {
  const float c1 = -0.5f;
  const float s1 = 0.86602540378443864676f;  // sin(2 pi / 3)
  float2 a = v[0], b = v[1], c = v[2];
  float2 s = cadd(b, c), d = csub(b, c);
  v[0] = cadd(a, s);
  float2 m = make_float2(a.x + c1 * s.x, a.y + c1 * s.y);
  // forward: -i * s1 * d
  float2 e = make_float2(s1 * d.y, -s1 * d.x);
  v[1] = cadd(m, e);
  v[2] = csub(m, e);
}

template <>
__device__ __forceinline__ void dft_small<5>(float2* v) {
  const float c1 = 0.30901699437494742410f;   // cos(2 pi / 5)
  const float c2 = -0.80901699437494742410f;  // cos(4 pi / 5)
  const float s1 = 0.95105651629515357212f;   // sin(2 pi / 5)
  const float s2 = 0.58778525229247312917f;   // sin(4 pi / 5)
  float2 x0 = v[0];
  float2 a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
  float2 a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
  v[0] = make_float2(x0.x + a1.x + a2.x, x0.y + a1.y + a2.y);
  float2 m1 = make_float2(x0.x + c1 * a1.x + c2 * a2.x, x0.y + c1 * a1.y + c2 * a2.y);
  float2 m2 = make_float2(x0.x + c2 * a1.x + c1 * a2.x, x0.y + c2 * a1.y + c1 * a2.y);
  // forward: -i * (s1 b1 + s2 b2), -i * (s2 b1 - s1 b2)
  float2 n1 = make_float2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y);
  float2 n2 = make_float2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y);
  float2 e1 = cmul_mi(n1), e2 = cmul_mi(n2);
  v[1] = cadd(m1, e1);
  v[4] = csub(m1, e1);
  v[2] = cadd(m2, e2);
  v[3] = csub(m2, e2);
}

template <>
__device__ __forceinline__ void dft_small<7>(float2* v) {
  const float c1 = 0.62348980185873353053f;   // cos(2 pi / 7)
  const float c2 = -0.22252093395631440429f;  // cos(4 pi / 7)
  const float c3 = -0.90096886790241912624f;  // cos(6 pi / 7)
  const float s1 = 0.78183148246802980871f;   // sin(2 pi / 7)
  const float s2 = 0.97492791218182360702f;   // sin(4 pi / 7)
  const float s3 = 0.43388373911755812048f;   // sin(6 pi / 7)
  float2 x0 = v[0];
  float2 a1 = cadd(v[1], v[6]), b1 = csub(v[1], v[6]);
  float2 a2 = cadd(v[2], v[5]), b2 = csub(v[2], v[5]);
  float2 a3 = cadd(v[3], v[4]), b3 = csub(v[3], v[4]);
  v[0] = make_float2(x0.x + a1.x + a2.x + a3.x, x0.y + a1.y + a2.y + a3.y);
  float2 m1 = make_float2(x0.x + c1 * a1.x + c2 * a2.x + c3 * a3.x, x0.y + c1 * a1.y + c2 * a2.y + c3 * a3.y);
  float2 m2 = make_float2(x0.x + c2 * a1.x + c3 * a2.x + c1 * a3.x, x0.y + c2 * a1.y + c3 * a2.y + c1 * a3.y);
  float2 m3 = make_float2(x0.x + c3 * a1.x + c1 * a2.x + c2 * a3.x, x0.y + c3 * a1.y + c1 * a2.y + c2 * a3.y);
  float2 n1 = make_float2(s1 * b1.x + s2 * b2.x + s3 * b3.x, s1 * b1.y + s2 * b2.y + s3 * b3.y);
  float2 n2 = make_float2(s2 * b1.x - s3 * b2.x - s1 * b3.x, s2 * b1.y - s3 * b2.y - s1 * b3.y);
  float2 n3 = make_float2(s3 * b1.x - s1 * b2.x + s2 * b3.x, s3 * b1.y - s1 * b2.y + s2 * b3.y);
  float2 e1 = cmul_mi(n1), e2 = cmul_mi(n2), e3 = cmul_mi(n3);
  v[1] = cadd(m1, e1);
  v[6] = csub(m1, e1);
  v[2] = cadd(m2, e2);
  v[5] = csub(m2, e2);
  v[3] = cadd(m3, e3);
  v[4] = csub(m3, e3);
}

// ---------------------------------------------------------------------------
// register DFTs with compile-time twiddles
// ---------------------------------------------------------------------------
// cos (want_sin = false) or sin of 2 pi k / n in double precision, by its
// Taylor series after reducing the angle to [-pi, pi]; evaluated by the
// compiler for the constant twiddles of the register DFTs.
__host__ __device__ constexpr double kw_ct_trig(int k, int n, bool want_sin) {
  k %= n;
  if (k < 0) k += n;
  double x = 6.28318530717958647692528676656 * (double)k / (double)n;
  if (x > 3.14159265358979323846264338328) x -= 6.28318530717958647692528676656;
  const double x2 = x * x;
  double term = want_sin ? x : 1.0, sum = term;
  for (int i = 1; i < 30; ++i) {
    const double a = want_sin ? 2.0 * i : 2.0 * i - 1.0, b = want_sin ? 2.0 * i + 1.0 : 2.0 * i;
    term = -term * x2 / (a * b);
    sum += term;
  }
  return sum;
}

// v * exp(-2 pi i K / N) with the constant folded in.
template <int K, int N>
__device__ __forceinline__ float2 kw_twc(float2 v) {
  constexpr int k = ((K % N) + N) % N;
  if constexpr (k == 0) {
    return v;
  } else if constexpr (4 * k == N) {
    return make_float2(v.y, -v.x);
  } else if constexpr (2 * k == N) {
    return make_float2(-v.x, -v.y);
  } else if constexpr (4 * k == 3 * N) {
    return make_float2(-v.y, v.x);
  } else {
    constexpr float c = (float)kw_ct_trig(k, N, false);
    constexpr float s = (float)-kw_ct_trig(k, N, true);
    return make_float2(fmaf(v.x, c, -v.y * s), fmaf(v.x, s, v.y * c));
  }
}

template <int N, int R, int M, int... E>
__device__ __forceinline__ void kw_tw_block(float2 (&sub)[R][M], std::integer_sequence<int, E...>) {
  ((sub[E / M][E % M] = kw_twc<(E / M) * (E % M), N>(sub[E / M][E % M])), ...);
}

// Forward DFT of N points held in registers: decimation in time over the
// first radix R of N (4, 2, 3, 5, 7 in that order of preference), the R
// sub-DFTs of N / R points recursively, constant twiddles w_N^(j k'), then
// radix-R butterflies; X[k' + (N/R) q] = sum_j w_R^(j q) w_N^(j k') Y_j[k'].
template <int N>
__device__ __forceinline__ void dft_reg(float2 (&v)[N]) {
  if constexpr (N == 1) {
  } else if constexpr (N == 2 || N == 3 || N == 4 || N == 5 || N == 7) {
    dft_small<N>(v);
  } else {
    constexpr int R = (N % 4 == 0) ? 4 : (N % 2 == 0) ? 2 : (N % 3 == 0) ? 3 : (N % 5 == 0) ? 5 : 7;
    constexpr int M = N / R;
    float2 sub[R][M];
#pragma unroll
    for (int j = 0; j < R; ++j)
#pragma unroll
      for (int i = 0; i < M; ++i) sub[j][i] = v[j + R * i];
#pragma unroll
    for (int j = 0; j < R; ++j) dft_reg<M>(sub[j]);
    kw_tw_block<N, R, M>(sub, std::make_integer_sequence<int, R * M>{});
#pragma unroll
    for (int k = 0; k < M; ++k) {
      float2 t[R];
#pragma unroll
      for (int j = 0; j < R; ++j) t[j] = sub[j][k];
      dft_small<R>(t);
#pragma unroll
      for (int q = 0; q < R; ++q) v[k + M * q] = t[q];
    }
  }
}

__device__ __forceinline__ float2 cmul_fma(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// ---------------------------------------------------------------------------
// two-level schedule: n = n1 n2, x = x1 + n1 x2, k = k2 + n2 k1
//   pass 1: Y[x1][k2] = w_n^(x1 k2) sum_x2 x[x1 + n1 x2] w_n2^(x2 k2)
//   pass 2: X[k2 + n2 k1] = sum_x1 Y[x1][k2] w_n1^(x1 k1)
// Element x of sequence b lives at (x xs + b bs).  Y[x1][k2] is kept in the
// scratch buffer at position n1 k2 + ((x1 + sk k2) mod n1), sk = 1 for even
// n1: pass 1's stores (consecutive x1) and pass 2's loads (consecutive k2)
// then both fall on distinct banks.  The twiddles come from a shared-memory
// table in [k2][x1] order (kw_load_twiddles), read along x1.
// BATCH_FAST: consecutive threads walk consecutive b (B a power of two).
// ---------------------------------------------------------------------------
template <int N2, bool BATCH_FAST>
__device__ __forceinline__ void fft2_pass1(const float2* __restrict__ a, float2* __restrict__ o, const KwFftLen& L,
                                           int B, int lgB, int xs, int bs, const float2* __restrict__ tw) {
  const int n1 = L.n1;
  const int items = B * n1;
  const bool sk = (n1 & 1) == 0;
  const int step = n1 * xs;
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    int b, x1;
    if (BATCH_FAST) {
      b = it & (B - 1);
      x1 = it >> lgB;
    } else {
      b = kw_divu(it, L.d1);
      x1 = it - b * n1;
    }
    const float2* src = a + x1 * xs + b * bs;
    float2 v[N2];
#pragma unroll
    for (int x2 = 0; x2 < N2; ++x2) v[x2] = src[x2 * step];
    dft_reg<N2>(v);
    float2* dst = o + b * bs;
    int r = x1;
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) {
      const float2 w = (k2 == 0) ? v[0] : cmul_fma(v[k2], tw[k2 * n1 + x1]);
      dst[(k2 * n1 + r) * xs] = w;
      if (sk) r = (r + 1 == n1) ? 0 : r + 1;
    }
  }
}

template <int N1, bool BATCH_FAST>
__device__ __forceinline__ void fft2_pass2(const float2* __restrict__ o, float2* __restrict__ a, const KwFftLen& L,
                                           int B, int lgB, int xs, int bs) {
  const int n2 = L.n2;
  const int items = B * n2;
  constexpr bool sk = (N1 & 1) == 0;
  const int ostep = n2 * xs;
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    int b, k2;
    if (BATCH_FAST) {
      b = it & (B - 1);
      k2 = it >> lgB;
    } else {
      b = kw_divu(it, L.d2);
      k2 = it - b * n2;
    }
    const float2* src = o + b * bs + k2 * N1 * xs;
    float2 v[N1];
    int r = sk ? k2 % N1 : 0;
#pragma unroll
    for (int x1 = 0; x1 < N1; ++x1) {
      v[x1] = src[(sk ? r : x1) * xs];
      if (sk) r = (r + 1 == N1) ? 0 : r + 1;
    }
    dft_reg<N1>(v);
    float2* dst = a + b * bs + k2 * xs;
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) dst[k1 * ostep] = v[k1];
  }
}

// Full forward FFT of B sequences in `a` on the two-level schedule; `b` is
// scratch of the same size; the result is left in `a`.  Contains
// __syncthreads(); every thread of the block must call it.
template <bool BATCH_FAST>
__device__ __noinline__ float2* fft2_smem(float2* a, float2* b, const KwFftLen& L, int B, int xs, int bs,
                                          const float2* __restrict__ tw) {
  const int lgB = __ffs(B) - 1;
  __syncthreads();
  switch (L.n2) {
#define KW_FFT2_P1(N) \
  case N: fft2_pass1<N, BATCH_FAST>(a, b, L, B, lgB, xs, bs, tw); break;
    KW_FFT2_SIZES(KW_FFT2_P1)
#undef KW_FFT2_P1
    default: break;
  }
  __syncthreads();
  switch (L.n1) {
#define KW_FFT2_P2(N) \
  case N: fft2_pass2<N, BATCH_FAST>(b, a, L, B, lgB, xs, bs); break;
    KW_FFT2_SIZES(KW_FFT2_P2)
#undef KW_FFT2_P2
    default: break;
  }
  __syncthreads();
  return a;
}

// Shared-memory twiddle table of a length: w^i in index order for the
// Stockham stages, or w^(x1 k2) at [k2 n1 + x1] for the two-level schedule
// (x1 k2 < n, so the entries come from the same global table).  The caller
// synchronises before the first transform.
__device__ __forceinline__ void kw_load_twiddles(float2* s, const float2* __restrict__ g, const KwFftLen& L) {
  const int n = L.n;
  if (L.n1 == 0) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) s[i] = g[i];
  } else {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const int k2 = kw_divu(i, L.d1), x1 = i - k2 * L.n1;
      s[i] = g[x1 * k2];
    }
  }
}

// One Stockham stage over a batch of B sequences.
// Element x of sequence b lives at buf[x * xs + b * bs].
// BATCH_FAST: consecutive threads walk consecutive b (interleaved layouts),
// otherwise consecutive j (row-contiguous layouts).
// BATCH_FAST needs B to be a power of two (lgB = log2 B).
template <int R, bool BATCH_FAST>
__device__ __forceinline__ void stockham_stage(const float2* __restrict__ in, float2* __restrict__ out, int n, int p,
                                               int B, int lgB, KwDivU dT, KwDivU dp, int xs, int bs,
                                               const float2* __restrict__ tw, int tid, int nth) {
  const int T = n / R;
  const int tstep = n / (p * R);
  const int total = T * B;
  for (int idx = tid; idx < total; idx += nth) {
    int b, j;
    if (BATCH_FAST) {
      b = idx & (B - 1);
      j = idx >> lgB;
    } else {
      b = kw_divu(idx, dT);
      j = idx - b * T;
    }
    const int k = j - kw_divu(j, dp) * p;
    float2 v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = in[(j + t * T) * xs + b * bs];
    if (p > 1) {
#pragma unroll
      for (int t = 1; t < R; ++t) v[t] = cmul(v[t], tw[t * k * tstep]);
    }
    dft_small<R>(v);
    const int ob = (j - k) * R + k;
#pragma unroll
    for (int q = 0; q < R; ++q) out[(ob + q * p) * xs + b * bs] = v[q];
  }
}

// Full forward FFT of B sequences held in shared memory on the Stockham
// stages.  Data start in `a`; `b` is scratch of the same size.  Returns the
// buffer holding the result.  Contains __syncthreads(); every thread of the
// block must call it.  BATCH_FAST layouts need B to be a power of two.
template <bool BATCH_FAST>
__device__ float2* fft_stockham(float2* a, float2* b, const KwFftLen& L, int B, int xs, int bs,
                                const float2* __restrict__ tw) {
  const int tid = threadIdx.x, nth = blockDim.x;
  const int lgB = __ffs(B) - 1;
  int p = 1;
  float2* src = a;
  float2* dst = b;
  for (int s = 0; s < L.nst; ++s) {
    __syncthreads();
    const int r = L.radix[s];
    const KwDivU dT = L.dt[s], dp = L.dp[s];
    switch (r) {
      case 4: stockham_stage<4, BATCH_FAST>(src, dst, L.n, p, B, lgB, dT, dp, xs, bs, tw, tid, nth); break;
      case 2: stockham_stage<2, BATCH_FAST>(src, dst, L.n, p, B, lgB, dT, dp, xs, bs, tw, tid, nth); break;
      case 3: stockham_stage<3, BATCH_FAST>(src, dst, L.n, p, B, lgB, dT, dp, xs, bs, tw, tid, nth); break;
      case 5: stockham_stage<5, BATCH_FAST>(src, dst, L.n, p, B, lgB, dT, dp, xs, bs, tw, tid, nth); break;
      default: stockham_stage<7, BATCH_FAST>(src, dst, L.n, p, B, lgB, dT, dp, xs, bs, tw, tid, nth); break;
    }
    p *= r;
    float2* t = src;
    src = dst;
    dst = t;
  }
  __syncthreads();
  return src;
}

// The FFT of a kernel instantiated for one schedule family: SCHED 0 the
// Stockham stages (L.n1 == 0), SCHED 1 the two-level schedule (L.n1 != 0).
// Separate instantiations keep each kernel's register count to its own
// schedule's.
template <bool BATCH_FAST, int SCHED = 0>
__device__ __forceinline__ float2* fft_smem(float2* a, float2* b, const KwFftLen& L, int B, int xs, int bs,
                                            const float2* __restrict__ tw) {
  if constexpr (SCHED == 1)
    return fft2_smem<BATCH_FAST>(a, b, L, B, xs, bs, tw);
  else
    return fft_stockham<BATCH_FAST>(a, b, L, B, xs, bs, tw);
}
