// Persistent, warp-specialised strided-axis FFT pass (power-of-two lengths).
//
// One or more CTAs per SM.  The last warp is the producer: its elected lane
// streams tiles of T columns x N points of a spectral buffer into a ring of
// NST shared-memory stages with TMA (cp.async.bulk.tensor, box T x min(N,256)),
// completion tracked by "full" mbarriers.  The other warps are consumers: they
// copy a stage into registers, release it on its "empty" mbarrier, run the
// register FFT (kw_regfft.cuh), apply the spectral operators and store the
// results with coalesced global stores.  Loads therefore run NST tiles ahead
// of compute.
//
// Work units: in operator mode one unit is a tile and its items are the
// distinct input buffers of the jobs; in plain mode one unit is (buffer,
// outer index, tile).  Producer and consumers walk the same unit/item sequence.
//
// KIND fixes the pass at compile time so that each instantiation carries only
// its own arithmetic:
//   KK_PLAIN  forward or inverse transforms of whole buffers (no operator);
//   KK_GEN    any job list (operator chosen per job at run time);
//   KK_GRAD   one input, D jobs: out a = gradient along axis a (the common
//             kappa(|k|) / N is folded into the spectrum once; the y and z
//             gradients share one inverse transform, their 1-D operators
//             being constant along x);
//   KK_DIV    D inputs, job a: in a -> out a, derivative along axis a; kappa
//             is evaluated once per tile and kept in registers for all items;
//   KK_NAB    one or two inputs: in 0 -> |k|^pow1, in 1 -> |k|^pow2;
//             log2 |k|^2 is evaluated once per tile.
//
// All mbarrier waits are bounded (2 s).  A timeout sets the error word the
// host passes in (TmaWork::err), the consumers agree on it through a
// reducing barrier and leave together, and thread 0 waits (bounded) for loads
// still in flight before the CTA exits.
#pragma once
#include "kw_kernels.cuh"
#include "kw_regfft.cuh"
#include "kw_tma.cuh"

enum KwTmaKind { KK_PLAIN = 0, KK_GEN = 1, KK_GRAD = 2, KK_DIV = 3, KK_NAB = 4 };

struct TmaMaps {
  CUtensorMap m[KW_NBUF];  // one per spectral buffer (KwBuf) for the pass's axis
};

struct TmaWork {
  int ntile;   // column tiles per outer block
  int nouter;  // outer blocks (x planes for the 3-D y pass)
  int nunits;
  int nitems;  // items per unit
  int inp[KW_MAX_JOBS];  // operator mode: distinct input buffers in job order
  int* err;    // device error word (set on a wait timeout)
  // the grid stride gridDim.x as (buffer, outer, tile) digits, for the
  // division-free walk over units (UnitPos)
  int st_tile, st_outer, st_b;
  int pdl;     // host: launch as a programmatic dependent of the previous kernel
};

// Position (b, outer, tile) of unit u = b * nouter * ntile + outer * ntile +
// tile, advanced by the grid stride without divisions.
struct UnitPos {
  int u, tile, outer, b;
  __device__ __forceinline__ void init(int u0, const TmaWork& W) {
    u = u0;
    tile = u0 % W.ntile;
    const int rest = u0 / W.ntile;
    outer = rest % W.nouter;
    b = rest / W.nouter;
  }
  __device__ __forceinline__ void next(const TmaWork& W) {
    u += gridDim.x;
    tile += W.st_tile;
    int c = tile >= W.ntile;
    if (c) tile -= W.ntile;
    outer += W.st_outer + c;
    c = outer >= W.nouter;
    if (c) outer -= W.nouter;
    b += W.st_b + c;
  }
};

namespace kwtmak {

constexpr uint64_t kWaitLimitNs = 2000000000ull;

// OR-reduction of pred over the n consumer threads (named barrier 1)
__device__ __forceinline__ bool consumers_any(bool pred, int n) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.or.pred p, 1, %2, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(r)
      : "r"((uint32_t)pred), "r"(n)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ float kappa_of(const AxisParams& A, float kmag) {
  if (!A.use_kspace) return 1.f;
  return kwreg::sinc_taylor(A.kcoef * kmag);
}

// kappa from |k|^2: sinc(c dt |k| / 2) with the series taken in its square
// (no square root unless the argument is large)
__device__ __forceinline__ float kappa_kk(const AxisParams& A, float kk) {
  if (!A.use_kspace) return 1.f;
  const float y = (A.kcoef * A.kcoef) * kk;
  if (!(y < 9.0f)) {
    const float x = sqrtf(y);
    return sinf(x) / x;
  }
  return kwreg::sinc_taylor_sq(y);
}

__device__ __forceinline__ float kk_of(const float* k0s, int ndim, int x, const ColK& g) {
  const float kx = k0s[x];
  float kk = __fadd_rn(__fmul_rn(kx, kx), g.ky2);
  if (ndim == 3) kk = __fadd_rn(kk, g.kz2);
  return kk;
}

__device__ __forceinline__ float kmag_of(const float* k0s, int ndim, int x, const ColK& g) {
  return sqrtf(kk_of(k0s, ndim, x, g));
}

// The x-axis operator tables (shared or global memory).
struct TabX {
  const float2* grad;
  const float2* div;
  const float2* unstag;
};

// Operator OP of job J at x-frequency index x of column g (OP known at compile
// time, so each job's element loop carries only its own arithmetic).  fcol is
// the job's 1-D factor when it acts along y or z.  With full == false only the
// 1-D factor of a gradient/divergence is returned (kappa and 1/N already folded
// into the spectrum).
template <int OP>
__device__ __forceinline__ float2 op_value(const AxisParams& A, const AxisJob& J, int x, const ColK& g,
                                           const float* k0s, const TabX& f0s, float2 fcol, bool full) {
  float2 op = make_float2(0.f, 0.f);
  if constexpr (OP == OP_GRAD || OP == OP_DIV) {
    const float2 f = (J.axis == 0) ? (OP == OP_GRAD ? f0s.grad[x] : f0s.div[x]) : fcol;
    if (!full) return f;
    const float kp = kappa_of(A, kmag_of(k0s, A.ndim, x, g)) * A.scale;
    return make_float2(f.x * kp, f.y * kp);
  } else if constexpr (OP == OP_NAB1 || OP == OP_NAB2) {
    const float km = kmag_of(k0s, A.ndim, x, g);
    op = make_float2(km == 0.f ? 0.f : powf(km, OP == OP_NAB1 ? A.pow1 : A.pow2), 0.f);
  } else if constexpr (OP == OP_SKAPPA) {
    op = make_float2(A.use_kspace ? cosf(A.kcoef * kmag_of(k0s, A.ndim, x, g)) : 1.f, 0.f);
  } else if constexpr (OP == OP_WIN) {
    float r2 = A.wc[0][x] + A.wc[1][g.a1];
    if (A.ndim == 3) r2 += A.wc[2][g.a2];
    op = make_float2(window_at(A.wtab, A.wlen, A.wrad, r2), 0.f);
  } else {
    op = (J.axis == 0) ? f0s.unstag[x] : fcol;
  }
  return make_float2(op.x * A.scale, op.y * A.scale);
}

// y[r] = conj(op * v[r]) over the thread's frequencies, for operator OP.
template <int OP, int E, int P>
__device__ __forceinline__ void apply_op(const AxisParams& A, const AxisJob& J, int t, const ColK& g, const float* k0s,
                                         const TabX& f0s, float2 fcol, bool full, bool on, const float2 (&v)[E],
                                         float2 (&y)[E]) {
#pragma unroll
  for (int m = 0; m < E / P; ++m)
#pragma unroll
    for (int k2 = 0; k2 < P; ++k2) {
      const int r = m * P + k2;
      const float2 op = op_value<OP>(A, J, t + P * m + E * k2, g, k0s, f0s, fcol, full);
      y[r] = on ? cconj(kwreg::cmulf(op, v[r])) : make_float2(0.f, 0.f);
    }
}

template <int E, int P>
__device__ __forceinline__ void apply_job(const AxisParams& A, const AxisJob& J, int t, const ColK& g, const float* k0s,
                                          const TabX& f0s, float2 fcol, bool full, bool on, const float2 (&v)[E],
                                          float2 (&y)[E]) {
  switch (J.op) {
    case OP_GRAD: apply_op<OP_GRAD, E, P>(A, J, t, g, k0s, f0s, fcol, full, on, v, y); break;
    case OP_DIV: apply_op<OP_DIV, E, P>(A, J, t, g, k0s, f0s, fcol, full, on, v, y); break;
    case OP_NAB1: apply_op<OP_NAB1, E, P>(A, J, t, g, k0s, f0s, fcol, full, on, v, y); break;
    case OP_NAB2: apply_op<OP_NAB2, E, P>(A, J, t, g, k0s, f0s, fcol, full, on, v, y); break;
    case OP_SKAPPA: apply_op<OP_SKAPPA, E, P>(A, J, t, g, k0s, f0s, fcol, full, on, v, y); break;
    case OP_WIN: apply_op<OP_WIN, E, P>(A, J, t, g, k0s, f0s, fcol, full, on, v, y); break;
    default: apply_op<OP_UNSTAG, E, P>(A, J, t, g, k0s, f0s, fcol, full, on, v, y); break;
  }
}

// The column-constant 1-D factor of an operator along axis 1 or 2.
__device__ __forceinline__ float2 col_factor_of(const AxisParams& A, int op, int axis, const ColK& g) {
  if (axis == 0 || !g.valid) return make_float2(0.f, 0.f);
  const int ai = (axis == 1) ? g.a1 : g.a2;
  switch (op) {
    case OP_GRAD: return A.fg[axis][ai];
    case OP_DIV: return A.fd[axis][ai];
    case OP_UNSTAG: return A.us[axis][ai];
    default: return make_float2(0.f, 0.f);
  }
}

__device__ __forceinline__ float2 col_factor(const AxisParams& A, const AxisJob& J, const ColK& g) {
  return col_factor_of(A, J.op, J.axis, g);
}

// Inverse transform of y (frequency layout) and store of column cc to `out`.
template <int E, int P, class Sync>
__device__ __forceinline__ void rev_store(float2 (&y)[E], int t, float2* exr, const float2* twr, Sync sync, bool act,
                                          float2* out, uint32_t base, uint32_t xs) {
  kwreg::Reg<E, P>::rev_t(y, t, exr, 1, twr, sync);
  if (act) {
#pragma unroll
    for (int j = 0; j < E; ++j) out[base + (t + P * j) * xs] = cconj(y[j]);
  }
}

}  // namespace kwtmak

// Stride (complex values) between the exchange regions of adjacent columns.
// Consumer thread tid = t * T + cc; a half warp holds 16 / T values of t for
// each of T columns, and its 64-bit exchange accesses hit bank pairs
// (cc * RS + t) mod 16.  With T = 8 they are distinct when RS = 2 (mod 16);
// with T >= 16 (one t per half warp) when RS is odd.  N + E + 1 is odd.
__host__ __device__ constexpr int kw_tma_rs(int N, int E, int T) {
  return T == 8 ? N + E + 1 + ((2 - (N + E + 1) % 16) + 16) % 16 : N + E + 1;
}

// T columns per tile, CT = T * P consumer threads plus one producer warp.
template <int E, int P, int NST, int MINB, int T, int KIND>
__global__ void __launch_bounds__(T * P + 32, MINB)
    k_axis_tma(const __grid_constant__ AxisParams A, const __grid_constant__ TmaMaps maps, const TmaWork W) {
  using namespace kwtmak;
  constexpr int N = E * P, RS = kw_tma_rs(E * P, E, T), CT = T * P;
  constexpr bool OPS = KIND != KK_PLAIN;
  // kinds whose single result per item goes back through the stage slot and a TMA store
  constexpr bool TSTORE = KIND == KK_PLAIN || KIND == KK_DIV || KIND == KK_NAB;
  constexpr uint32_t kStageBytes = N * T * sizeof(float2);
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  float2* stages = reinterpret_cast<float2*>(smem_raw);  // NST * N * T
  float2* ex = stages + (size_t)NST * N * T;             // T * RS
  // per-thread twiddle rows of the forward and inverse transforms (Reg::build_rows)
  constexpr int TWR = kwreg::Reg<E, P>::TW_ROW;
  float2* twf = ex + (size_t)T * RS;                     // P * TWR
  float2* twrt = twf + P * TWR;                          // P * TWR
  // x-axis tables (k, op_grad, op_div, unstag) in shared memory when they fit
  constexpr bool kTablesInSmem = N <= 512 && KIND != KK_PLAIN;
  constexpr int NT = kTablesInSmem ? N : 0;
  float* k0t = reinterpret_cast<float*>(twrt + P * TWR);
  float2* f0t = reinterpret_cast<float2*>(k0t + NT);
  uint64_t* full = reinterpret_cast<uint64_t*>(f0t + 3 * NT);
  uint64_t* empty = full + NST;
  int* counters = reinterpret_cast<int*>(empty + NST);  // [0] issued, [1] consumed

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      kwtma::mbar_init(&full[s], 1);
      // tile-store kinds: the slot is freed by the thread that stores it back with TMA
      kwtma::mbar_init(&empty[s], TSTORE ? 1 : CT / 32);
    }
    counters[0] = counters[1] = 0;
    kwtma::fence_barrier_init();
  }
  kwreg::Reg<E, P>::build_rows(twf, twrt, A.tw, tid, blockDim.x);
  for (int i = tid; i < N; i += blockDim.x) {
    if (kTablesInSmem && OPS) {
      k0t[i] = A.k[0][i];
      f0t[i] = A.fg[0][i];
      f0t[N + i] = A.fd[0][i];
      f0t[2 * N + i] = A.us[0] ? A.us[0][i] : make_float2(0.f, 0.f);
    }
  }
  __syncthreads();
  // everything above reads only tables; the spectra come from the previous launch
  kwtma::grid_dep_wait();
  kwtma::grid_dep_launch();
  const float* k0s = kTablesInSmem ? k0t : A.k[0];
  const TabX f0s{kTablesInSmem ? f0t : A.fg[0], kTablesInSmem ? f0t + N : A.fd[0], kTablesInSmem ? f0t + 2 * N : A.us[0]};

  if (warp == CT / 32) {
    // ---------------- producer ----------------
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      UnitPos up;
      for (up.init(blockIdx.x, W); up.u < W.nunits && ok; up.next(W)) {
        const int tile = up.tile, outer = up.outer, b = up.b;
        for (int q = 0; q < W.nitems; ++q, ++it) {
          const int buf = OPS ? W.inp[q] : A.plain[b];
          const uint32_t s = it % NST, k = it / NST;
          if (k > 0 && !kwtma::mbar_wait(&empty[s], (k - 1) & 1, kWaitLimitNs)) {
            atomicExch(W.err, 1);
            ok = false;
            break;
          }
          kwtma::mbar_arrive_expect_tx(&full[s], kStageBytes);
          float2* dst = stages + (size_t)s * N * T;
#pragma unroll
          for (int n0 = 0; n0 < N; n0 += 256) kwtma::tma_load_3d(dst + n0 * T, &maps.m[buf], tile * T, n0, outer, &full[s]);
        }
      }
      counters[0] = (int)it;
    }
  } else {
    // ---------------- consumers ----------------
    const int cc = tid % T, t = tid / T;
    auto sync = [] __device__() { kwtma::named_sync(CT); };
    const float2* tw = twf + t * TWR;   // this thread's forward twiddles
    const float2* twr = twrt + t * TWR;  // and inverse twiddles
    float2* exr = ex + cc * RS;
    uint32_t it = 0;
    bool aborted = false;
    // per-tile operator cache (KK_DIV: kappa / N; KK_NAB: log2 |k|^2, -inf at k = 0)
    constexpr int NC = (KIND == KK_DIV || KIND == KK_NAB) ? E : 1;
    float kc[NC];
    UnitPos up;
    for (up.init(blockIdx.x, W); up.u < W.nunits && !aborted; up.next(W)) {
      const int tile = up.tile, outer = up.outer, b = up.b;
      const int c0 = tile * T;
      const bool act = cc < A.ncols - c0;
      // 32-bit element offsets (the host uses this pass only for spectra below 2^31 elements)
      const uint32_t base = (uint32_t)outer * (uint32_t)A.os + (uint32_t)(c0 + cc);
      const uint32_t xs = (uint32_t)A.xs;
      ColK g;
      if constexpr (OPS) g = col_geometry(A, act ? c0 + cc : c0);
      const bool on = OPS && act && g.valid;
      for (int q = 0; q < W.nitems; ++q, ++it) {
        const uint32_t s = it % NST, k = it / NST;
        const bool got = kwtma::mbar_wait(&full[s], k & 1, kWaitLimitNs);
        if (consumers_any(!got, CT)) {
          if (tid == 0) atomicExch(W.err, 2);
          aborted = true;
          break;
        }
        const float2* st = stages + (size_t)s * N * T;
        float2 v[E];
        if (!OPS && A.mode == 1) {
#pragma unroll
          for (int m = 0; m < E / P; ++m)
#pragma unroll
            for (int k2 = 0; k2 < P; ++k2) v[m * P + k2] = cconj(st[(t + P * m + E * k2) * T + cc]);
        } else {
#pragma unroll
          for (int j = 0; j < E; ++j) v[j] = st[(t + P * j) * T + cc];
        }
        if constexpr (!TSTORE) {
          __syncwarp();
          if (lane == 0) kwtma::mbar_arrive(&empty[s]);
        }
        // write the item's result (inverse-transformed, conjugated back) into
        // the slot and store it with TMA to buffer `ob`; frees the slot
        auto store_rev = [&](float2 (&y)[E], int ob) {
          float2* so = stages + (size_t)s * N * T;
          kwreg::Reg<E, P>::rev_t(y, t, exr, 1, twr, sync);
#pragma unroll
          for (int j = 0; j < E; ++j) so[(t + P * j) * T + cc] = cconj(y[j]);
          kwtma::fence_proxy_async_smem();
          kwtma::named_sync(CT);
          if (tid == 0) {
#pragma unroll
            for (int n0 = 0; n0 < N; n0 += 256) kwtma::tma_store_3d(&maps.m[ob], so + n0 * T, tile * T, n0, outer);
            kwtma::bulk_commit();
            kwtma::bulk_wait_read_all();
            kwtma::mbar_arrive(&empty[s]);
          }
        };

        if constexpr (KIND == KK_PLAIN) {
          // transform, write the results back into the stage slot in the
          // tile's layout and store the tile with TMA (the slot is freed once
          // the store has read it)
          float2* so = stages + (size_t)s * N * T;
          if (A.mode == 0) {
            kwreg::Reg<E, P>::fwd_t(v, t, exr, 1, tw, sync);
#pragma unroll
            for (int m = 0; m < E / P; ++m)
#pragma unroll
              for (int k2 = 0; k2 < P; ++k2) so[(t + P * m + E * k2) * T + cc] = v[m * P + k2];
          } else {
            kwreg::Reg<E, P>::rev_t(v, t, exr, 1, twr, sync);
#pragma unroll
            for (int j = 0; j < E; ++j) so[(t + P * j) * T + cc] = cconj(v[j]);
          }
          kwtma::fence_proxy_async_smem();
          kwtma::named_sync(CT);
          if (tid == 0) {
            const CUtensorMap* map = &maps.m[A.plain[b]];
#pragma unroll
            for (int n0 = 0; n0 < N; n0 += 256) kwtma::tma_store_3d(map, so + n0 * T, tile * T, n0, outer);
            kwtma::bulk_commit();
            kwtma::bulk_wait_read_all();
            kwtma::mbar_arrive(&empty[s]);
          }
        } else if constexpr (KIND == KK_GRAD) {
          kwreg::Reg<E, P>::fwd_t(v, t, exr, 1, tw, sync);
          // the D gradients share kappa(|k|) / N: fold it into the spectrum once
#pragma unroll
          for (int m = 0; m < E / P; ++m)
#pragma unroll
            for (int k2 = 0; k2 < P; ++k2) {
              const float kp = kappa_kk(A, kk_of(k0s, A.ndim, t + P * m + E * k2, g)) * A.scale;
              v[m * P + k2] = make_float2(v[m * P + k2].x * kp, v[m * P + k2].y * kp);
            }
          // x derivative: its 1-D operator varies along x
          {
            float2 y[E];
#pragma unroll
            for (int m = 0; m < E / P; ++m)
#pragma unroll
              for (int k2 = 0; k2 < P; ++k2) {
                const int r = m * P + k2;
                y[r] = on ? cconj(kwreg::cmulf(f0s.grad[t + P * m + E * k2], v[r])) : make_float2(0.f, 0.f);
              }
            rev_store<E, P>(y, t, exr, twr, sync, act, A.bufs[0], base, xs);
          }
          // y and z derivatives: their 1-D operators are constant along x and
          // commute with the x transform, so one inverse transform of
          // kappa F / N serves both: out_a = op_a(column) * G
#pragma unroll
          for (int r = 0; r < E; ++r) v[r] = on ? cconj(v[r]) : make_float2(0.f, 0.f);
          kwreg::Reg<E, P>::rev_t(v, t, exr, 1, twr, sync);
          if (act) {
#pragma unroll 1
            for (int a = 1; a < A.ndim; ++a) {
              const float2 fcol = col_factor_of(A, OP_GRAD, a, g);
              float2* out = A.bufs[a];
#pragma unroll
              for (int j = 0; j < E; ++j) out[base + (t + P * j) * xs] = kwreg::cmulf(fcol, cconj(v[j]));
            }
          }
        } else if constexpr (KIND == KK_DIV) {
          // item q is the velocity spectrum of axis q; its derivative replaces it
          kwreg::Reg<E, P>::fwd_t(v, t, exr, 1, tw, sync);
          if (q == 0) {
#pragma unroll
            for (int m = 0; m < E / P; ++m)
#pragma unroll
              for (int k2 = 0; k2 < P; ++k2)
                kc[m * P + k2] = kappa_kk(A, kk_of(k0s, A.ndim, t + P * m + E * k2, g)) * A.scale;
          }
          const float2 fcol = col_factor_of(A, OP_DIV, q, g);
#pragma unroll
          for (int m = 0; m < E / P; ++m)
#pragma unroll
            for (int k2 = 0; k2 < P; ++k2) {
              const int r = m * P + k2;
              const float2 f = (q == 0) ? f0s.div[t + P * m + E * k2] : fcol;
              const float2 op = make_float2(f.x * kc[r], f.y * kc[r]);
              v[r] = on ? cconj(kwreg::cmulf(op, v[r])) : make_float2(0.f, 0.f);
            }
          store_rev(v, W.inp[q]);
        } else if constexpr (KIND == KK_NAB) {
          // item 0: |k|^pow1 on buffer 0, item 1: |k|^pow2 on buffer 1 (0 at k = 0)
          kwreg::Reg<E, P>::fwd_t(v, t, exr, 1, tw, sync);
          if (q == 0) {
#pragma unroll
            for (int m = 0; m < E / P; ++m)
#pragma unroll
              for (int k2 = 0; k2 < P; ++k2) kc[m * P + k2] = log2f(kk_of(k0s, A.ndim, t + P * m + E * k2, g));
          }
          const float hp = 0.5f * (q == 0 ? A.pow1 : A.pow2);
#pragma unroll
          for (int r = 0; r < E; ++r) {
            const float val = (kc[r] == -INFINITY) ? 0.f : exp2f(hp * kc[r]);
            const float2 op = make_float2(val * A.scale, 0.f);
            v[r] = on ? cconj(kwreg::cmulf(op, v[r])) : make_float2(0.f, 0.f);
          }
          store_rev(v, W.inp[q]);
        } else {
          // generic operator mode: forward FFT of this input, then every job reading it
          kwreg::Reg<E, P>::fwd_t(v, t, exr, 1, tw, sync);
          const int in = W.inp[q];
          int nj = 0, jlast = 0;
          bool all_kappa = true;
          for (int jj = 0; jj < A.njobs; ++jj)
            if (A.jobs[jj].in == in) {
              ++nj;
              jlast = jj;
              all_kappa &= (A.jobs[jj].op == OP_GRAD || A.jobs[jj].op == OP_DIV);
            }
          if (nj == 1) {
            // one job: multiply in place
            const AxisJob J = A.jobs[jlast];
            const float2 fcol = col_factor(A, J, g);
            apply_job<E, P>(A, J, t, g, k0s, f0s, fcol, true, on, v, v);
            rev_store<E, P>(v, t, exr, twr, sync, act, A.bufs[J.out], base, xs);
            continue;
          }
          if (all_kappa) {
            // the jobs share kappa(|k|) / N: fold it into the spectrum once
#pragma unroll
            for (int m = 0; m < E / P; ++m)
#pragma unroll
              for (int k2 = 0; k2 < P; ++k2) {
                const float kp = kappa_of(A, kmag_of(k0s, A.ndim, t + P * m + E * k2, g)) * A.scale;
                v[m * P + k2] = make_float2(v[m * P + k2].x * kp, v[m * P + k2].y * kp);
              }
          }
          for (int jj = 0; jj < A.njobs; ++jj) {
            const AxisJob J = A.jobs[jj];
            if (J.in != in) continue;
            const float2 fcol = col_factor(A, J, g);
            float2 y[E];
            apply_job<E, P>(A, J, t, g, k0s, f0s, fcol, !all_kappa, on, v, y);
            rev_store<E, P>(y, t, exr, twr, sync, act, A.bufs[J.out], base, xs);
          }
        }
      }
    }
    if (tid == 0) {
      counters[1] = (int)it;
      if constexpr (TSTORE) kwtma::bulk_wait_all();  // tile stores complete before the CTA exits
    }
  }
  __syncthreads();
  // loads issued but never consumed (only after a timeout): wait for them, bounded
  if (tid == 0) {
    for (int i = counters[1]; i < counters[0]; ++i) {
      const uint32_t s = (uint32_t)i % NST, k = (uint32_t)i / NST;
      if (!kwtma::mbar_wait(&full[s], k & 1, kWaitLimitNs)) break;
    }
  }
}

// ---------------------------------------------------------------------------
// launch geometry (shared by the host side of every translation unit)
// ---------------------------------------------------------------------------

// (E, P) of a pass: plain passes of length 256 use 32 points per thread and 8
// threads per column (16-column tiles, 128-byte rows); everything else the
// register-FFT shape of the length (kw_reg_shape).
inline bool kw_tma_shape(int n, int kind, int* E, int* P) {
  if (n == 256 && kind == KK_PLAIN) {
    *E = 32;
    *P = 8;
    return true;
  }
  return kw_reg_shape(n, E, P);
}

// Tile width: lengths up to 256 use tiles of 128 / P columns (128 consumer
// threads plus the producer warp) at three CTAs per SM, which leaves each
// thread 128 registers; 512 and 1024 use 256 / P columns at one CTA per SM.
inline bool kw_tma_narrow(int n, int axis, int kind) { return n <= 256; }
// Small tiles (operator passes of lengths 128..512): one warp of consumers
// (32 / P columns) at four CTAs per SM, for grids with too few columns to
// give every SM a tile at the normal width (2-D grids up to 512 columns).
inline bool kw_tma_small_ok(int n, int kind) { return kind != KK_PLAIN && (n == 128 || n == 256 || n == 512); }
inline int kw_tma_tile_cols(int n, int P, int axis, int kind, bool small = false) {
  return small ? 32 / P : kw_tma_narrow(n, axis, kind) ? 128 / P : 256 / P;
}
inline int kw_tma_per_sm(int n, int axis, int kind, bool small = false) {
  return small ? 4 : (n == 256 && kind == KK_PLAIN) ? 2 : kw_tma_narrow(n, axis, kind) ? 3 : 1;
}

// Stages of the TMA ring (a third stage measured no faster for the plain passes).
inline int kw_tma_stages(int n, int kind) { return 2; }
#define KW_NST_S 2

inline size_t kw_tma_smem(int n, int E, int P, int axis, int kind, bool small = false) {
  const int T = kw_tma_tile_cols(n, P, axis, kind, small), RS = kw_tma_rs(n, E, T), NST = kw_tma_stages(n, kind);
  const size_t nt = (n <= 512 && kind != KK_PLAIN) ? (size_t)n : 0;
  return sizeof(float2) * ((size_t)NST * n * T + (size_t)T * RS + 2 * (size_t)P * (E + 2) + 3 * nt) + sizeof(float) * nt +
         2 * NST * sizeof(uint64_t) + 16;
}

// Instantiation table: (E, P, stages, CTAs per SM, tile columns) per length.
#define KW_TMA_SWITCH(n, narrow_, CALL)      \
  switch (n) {                               \
    case 64: return CALL(16, 4, KW_NST_S, 3, 32);   \
    case 128: return CALL(16, 8, KW_NST_S, 3, 16);  \
    case 256:                                       \
      if constexpr (KIND == KK_PLAIN) return CALL(32, 8, KW_NST_S, 2, 16); \
      return CALL(16, 16, KW_NST_S, 3, 8);          \
    case 512: return CALL(32, 16, 2, 1, 16); \
    case 1024: return CALL(32, 32, 2, 1, 8); \
    default: return cudaErrorInvalidValue;   \
  }

// Small-tile instantiations (kw_tma_small_ok): T = 32 / P, 4 CTAs per SM.
#define KW_TMA_SWITCH_SMALL(n, CALL)                 \
  switch (n) {                                       \
    case 128: return CALL(16, 8, KW_NST_S, 4, 4);    \
    case 256: return CALL(16, 16, KW_NST_S, 4, 2);   \
    case 512: return CALL(32, 16, 2, 4, 2);          \
    default: return cudaErrorInvalidValue;           \
  }

// Attribute set-up and launch of one KIND (instantiated in the translation
// unit that calls them).
template <int KIND>
cudaError_t kw_tma_attr_kind(int n, int axis, bool small) {
  int E, P;
  if (!kw_tma_shape(n, KIND, &E, &P)) return cudaErrorInvalidValue;
  const int smem = (int)kw_tma_smem(n, E, P, axis, KIND, small);
#define KW_T(E_, P_, S_, B_, T_) \
  cudaFuncSetAttribute(k_axis_tma<E_, P_, S_, B_, T_, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)
  if constexpr (KIND != KK_PLAIN) {
    if (small) KW_TMA_SWITCH_SMALL(n, KW_T)
  }
  KW_TMA_SWITCH(n, 0, KW_T)
#undef KW_T
}

template <int KIND>
cudaError_t kw_tma_launch_kind(int n, int axis, int grid, size_t smem, cudaStream_t st, const AxisParams& A,
                               const TmaMaps& maps, const TmaWork& W, bool small) {
#define KW_T(E_, P_, S_, B_, T_)                                                                              \
  kwtma::launch_k(k_axis_tma<E_, P_, S_, B_, T_, KIND>, dim3(grid), dim3(T_ * P_ + 32), smem, st, W.pdl != 0, A, \
                  maps, W)
  if constexpr (KIND != KK_PLAIN) {
    if (small) KW_TMA_SWITCH_SMALL(n, KW_T)
  }
  KW_TMA_SWITCH(n, 0, KW_T)
#undef KW_T
}

// Per-kind entry points.  Each is defined (KW_TMA_DEFINE_KIND) in the
// translation unit that instantiates that kind, so that the kinds compile in
// parallel.
#define KW_TMA_DECLARE_KIND(name)                                                                             \
  cudaError_t kw_tma_attr_##name(int n, int axis, bool small);                                                \
  cudaError_t kw_tma_launch_##name(int n, int axis, int grid, size_t smem, cudaStream_t st, const AxisParams& A, \
                                   const TmaMaps& maps, const TmaWork& W, bool small);
#define KW_TMA_DEFINE_KIND(name, KIND)                                                                         \
  cudaError_t kw_tma_attr_##name(int n, int axis, bool small) { return kw_tma_attr_kind<KIND>(n, axis, small); } \
  cudaError_t kw_tma_launch_##name(int n, int axis, int grid, size_t smem, cudaStream_t st, const AxisParams& A, \
                                   const TmaMaps& maps, const TmaWork& W, bool small) {                        \
    return kw_tma_launch_kind<KIND>(n, axis, grid, smem, st, A, maps, W, small);                               \
  }
KW_TMA_DECLARE_KIND(plain)
KW_TMA_DECLARE_KIND(gen)
KW_TMA_DECLARE_KIND(grad)
KW_TMA_DECLARE_KIND(div)
KW_TMA_DECLARE_KIND(nab)
