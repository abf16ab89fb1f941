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
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define KW_MAX_STAGES 16
#define KW_RADIX_ORDERS 3  // radix schedules a plan can use (kw_plan.cu: kRadixOrders)

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
};

// Fill the per-stage divisors once the radices are set.
inline void kw_fft_len_finish(KwFftLen& f) {
  int p = 1;
  for (int s = 0; s < f.nst; ++s) {
    f.dt[s] = kw_divu_make((uint32_t)(f.n / f.radix[s]));
    f.dp[s] = kw_divu_make((uint32_t)p);
    p *= f.radix[s];
  }
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

// Full forward FFT of B sequences held in shared memory.  Data start in `a`;
// `b` is scratch of the same size.  Returns the buffer holding the result.
// Contains __syncthreads(); every thread of the block must call it.
// BATCH_FAST layouts need B to be a power of two.
template <bool BATCH_FAST>
__device__ float2* fft_smem(float2* a, float2* b, const KwFftLen& L, int B, int xs, int bs,
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
