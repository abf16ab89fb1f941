// Register-resident FFTs for power-of-two lengths N = E * P (64 <= N <= 1024).
//
// One transform is computed by P threads that each hold E complex values
// (P divides E).  Index maps (Cooley-Tukey, n = t + P j, k = k1 + E k2):
//
//   fwd(): in  thread t holds x[t + P j],            j  < E   ("strided" layout)
//          out thread t holds X[k1 + E k2] at v[m P + k2],
//                 k1 = t + P m (m < E/P), k2 < P      ("frequency" layout)
//          = E-point DFTs in registers, twiddle W_N^{t k1}, one transpose
//            through shared memory, P-point DFTs in registers.
//   rev(): the exact reverse data flow (frequency layout in, strided layout
//          out) with forward DFTs; rev(conj X) conjugated gives N * IDFT(X).
//
// All DFTs are forward and unnormalised; twiddles come from a table
// tw[j] = exp(-2 pi i j / N) held in shared memory.  Small DFTs (2, 4, 8, 16,
// 32) are fully unrolled Cooley-Tukey with constant twiddles.
#pragma once
#include "kw_fft.cuh"

namespace kwreg {

// complex multiply with fused multiply-adds (FFT-internal arithmetic)
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// sin(x)/x from its Taylor series in x^2 (Horner form), |x| < 3; relative
// error below 1e-7 there.  Larger arguments use sinf.
__device__ __forceinline__ float sinc_taylor(float x) {
  if (!(x < 3.0f)) return sinf(x) / x;
  const float y = x * x;
  float s = 1.0f;
#pragma unroll
  for (int n = 10; n >= 1; --n) s = fmaf(-y * (1.0f / float((2 * n) * (2 * n + 1))), s, 1.0f);
  return s;
}

// sin(x)/x from the same series given y = x^2 < 9
__device__ __forceinline__ float sinc_taylor_sq(float y) {
  float s = 1.0f;
#pragma unroll
  for (int n = 10; n >= 1; --n) s = fmaf(-y * (1.0f / float((2 * n) * (2 * n + 1))), s, 1.0f);
  return s;
}

// cos/sin(2 pi j / 32), j = 0..31 (constant twiddles of the small DFTs)
__device__ __forceinline__ float2 w32(int j) {
  // exp(-2 pi i j / 32)
  constexpr float c[8] = {1.0f, 0.98078528040323044913f, 0.92387953251128675613f, 0.83146961230254523708f,
                          0.70710678118654752440f, 0.55557023301960222474f, 0.38268343236508977173f,
                          0.19509032201612826785f};
  j &= 31;
  // cos(2 pi j/32) and sin(2 pi j/32) from the first octant table by symmetry
  const int q = j >> 3, r = j & 7;
  float cs, sn;
  if (r == 0) {
    cs = c[0];
    sn = 0.f;
  } else {
    cs = c[r];
    sn = c[8 - r];
  }
  float C, S;
  switch (q) {
    case 0: C = cs; S = sn; break;
    case 1: C = -sn; S = cs; break;
    case 2: C = -cs; S = -sn; break;
    default: C = sn; S = -cs; break;
  }
  return make_float2(C, -S);
}

// Complex add / subtract as packed two-lane float operations (FADD2 / FFMA2
// on sm_100+): one instruction each, component-wise identical to the scalar
// forms (a - b is formed as b * (-1) + a, which is exact before the rounding).
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

template <int R>
struct Dft;

template <>
struct Dft<1> {
  __device__ __forceinline__ static void run(float2*) {}
};
template <>
struct Dft<2> {
  __device__ __forceinline__ static void run(float2* v) {
    const float2 a = v[0], b = v[1];
    v[0] = padd(a, b);
    v[1] = psub(a, b);
  }
};
template <>
struct Dft<4> {
  __device__ __forceinline__ static void run(float2* v) {
    const float2 a0 = padd(v[0], v[2]), a1 = psub(v[0], v[2]);
    const float2 b0 = padd(v[1], v[3]), d = psub(v[1], v[3]);
    v[0] = padd(a0, b0);
    v[2] = psub(a0, b0);
    // a1 -/+ i d
    v[1] = make_float2(a1.x + d.y, a1.y - d.x);
    v[3] = make_float2(a1.x - d.y, a1.y + d.x);
  }
};

// N = N1 * N2 in registers: n = N2 n1 + n2, k = k1 + N1 k2.
template <int N1, int N2>
struct DftCT {
  static constexpr int N = N1 * N2;
  __device__ __forceinline__ static void run(float2* v) {
    float2 a[N];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) {
      float2 t[N1];
#pragma unroll
      for (int n1 = 0; n1 < N1; ++n1) t[n1] = v[N2 * n1 + n2];
      Dft<N1>::run(t);
#pragma unroll
      for (int k1 = 0; k1 < N1; ++k1) {
        const int e = (n2 * k1 * (32 / N)) & 31;
        a[k1 * N2 + n2] = (n2 * k1 == 0) ? t[k1] : cmulf(t[k1], w32(e));
      }
    }
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) {
      float2 s[N2];
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) s[n2] = a[k1 * N2 + n2];
      Dft<N2>::run(s);
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) v[k1 + N1 * k2] = s[k2];
    }
  }
};

template <>
struct Dft<8> {
  __device__ __forceinline__ static void run(float2* v) { DftCT<4, 2>::run(v); }
};
template <>
struct Dft<16> {
  __device__ __forceinline__ static void run(float2* v) { DftCT<4, 4>::run(v); }
};
template <>
struct Dft<32> {
  __device__ __forceinline__ static void run(float2* v) { DftCT<8, 4>::run(v); }
};

// Two-level transform of one sequence by P cooperating threads.
// sm: this sequence's exchange region of at least N + E slots, addressed as
// sm[idx * ss] (ss = stride between consecutive slots); rows of the exchanged
// matrices are padded by one slot against shared-memory bank conflicts.  The
// caller supplies the synchronisation of the P threads (sync()).
template <int E, int P>
struct Reg {
  static constexpr int N = E * P;
  static_assert(E % P == 0, "P must divide E");

  template <class Sync>
  __device__ __forceinline__ static void fwd(float2 (&v)[E], int t, float2* sm, int ss, const float2* tw, Sync sync) {
    Dft<E>::run(v);
#pragma unroll
    for (int k1 = 1; k1 < E; ++k1) v[k1] = cmulf(v[k1], tw[t * k1]);
#pragma unroll
    for (int k1 = 0; k1 < E; ++k1) sm[(k1 * (P + 1) + t) * ss] = v[k1];
    sync();
#pragma unroll
    for (int m = 0; m < E / P; ++m) {
      float2 s[P];
      const int k1 = t + P * m;
#pragma unroll
      for (int n2 = 0; n2 < P; ++n2) s[n2] = sm[(k1 * (P + 1) + n2) * ss];
      Dft<P>::run(s);
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) v[m * P + k2] = s[k2];
    }
    sync();
  }

  template <class Sync>
  __device__ __forceinline__ static void rev(float2 (&v)[E], int t, float2* sm, int ss, const float2* tw, Sync sync) {
#pragma unroll
    for (int m = 0; m < E / P; ++m) {
      float2 s[P];
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) s[k2] = v[m * P + k2];
      Dft<P>::run(s);
      const int k1 = t + P * m;
#pragma unroll
      for (int n2 = 0; n2 < P; ++n2) {
        const float2 w = (n2 * k1 == 0) ? make_float2(1.f, 0.f) : tw[n2 * k1];
        sm[(n2 * (E + 1) + k1) * ss] = cmulf(s[n2], w);
      }
    }
    sync();
#pragma unroll
    for (int k1 = 0; k1 < E; ++k1) v[k1] = sm[(t * (E + 1) + k1) * ss];
    sync();
    Dft<E>::run(v);
  }

  // Per-thread twiddle rows: twf[k1] = W_N^{t k1} (k1 < E) for fwd_t,
  // twr[m P + n2] = W_N^{n2 (t + P m)} (n2 < P, m < E / P) for rev_t, each row
  // 16-byte aligned and read two values per load.
  static constexpr int TW_ROW = E + 2;  // row stride (complex): aligned, bank-spread
  __device__ __forceinline__ static void build_rows(float2* twf, float2* twr, const float2* tw, int tid, int nthr) {
    for (int i = tid; i < P * E; i += nthr) {
      const int t = i / E, k = i - t * E;
      twf[t * TW_ROW + k] = tw[t * k];
      const int m = k / P, n2 = k - m * P;
      twr[t * TW_ROW + k] = tw[n2 * (t + P * m)];
    }
  }

  template <class Sync>
  __device__ __forceinline__ static void fwd_t(float2 (&v)[E], int t, float2* sm, int ss, const float2* twf, Sync sync) {
    Dft<E>::run(v);
    const float4* w4 = reinterpret_cast<const float4*>(twf);
#pragma unroll
    for (int h = 0; h < E / 2; ++h) {
      const float4 w = w4[h];
      if (h > 0) v[2 * h] = cmulf(v[2 * h], make_float2(w.x, w.y));
      v[2 * h + 1] = cmulf(v[2 * h + 1], make_float2(w.z, w.w));
    }
#pragma unroll
    for (int k1 = 0; k1 < E; ++k1) sm[(k1 * (P + 1) + t) * ss] = v[k1];
    sync();
#pragma unroll
    for (int m = 0; m < E / P; ++m) {
      float2 s[P];
      const int k1 = t + P * m;
#pragma unroll
      for (int n2 = 0; n2 < P; ++n2) s[n2] = sm[(k1 * (P + 1) + n2) * ss];
      Dft<P>::run(s);
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) v[m * P + k2] = s[k2];
    }
    sync();
  }

  template <class Sync>
  __device__ __forceinline__ static void rev_t(float2 (&v)[E], int t, float2* sm, int ss, const float2* twr, Sync sync) {
    const float4* w4 = reinterpret_cast<const float4*>(twr);
#pragma unroll
    for (int m = 0; m < E / P; ++m) {
      float2 s[P];
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) s[k2] = v[m * P + k2];
      Dft<P>::run(s);
      const int k1 = t + P * m;
#pragma unroll
      for (int h = 0; h < P / 2; ++h) {
        const float4 w = w4[(m * P) / 2 + h];
        const int n2 = 2 * h;
        sm[(n2 * (E + 1) + k1) * ss] = n2 == 0 ? s[n2] : cmulf(s[n2], make_float2(w.x, w.y));
        sm[((n2 + 1) * (E + 1) + k1) * ss] = cmulf(s[n2 + 1], make_float2(w.z, w.w));
      }
    }
    sync();
#pragma unroll
    for (int k1 = 0; k1 < E; ++k1) v[k1] = sm[(t * (E + 1) + k1) * ss];
    sync();
    Dft<E>::run(v);
  }
};

}  // namespace kwreg
