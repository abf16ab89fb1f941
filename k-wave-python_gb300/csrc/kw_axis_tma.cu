// Persistent, warp-specialised strided-axis FFT pass (power-of-two lengths).
//
// One CTA per SM.  Warp 8 is the producer: its elected lane streams tiles of
// T columns x N points of a spectral buffer into a ring of NST shared-memory
// stages with TMA (cp.async.bulk.tensor, box T x min(N,256)), completion
// tracked by "full" mbarriers.  Warps 0-7 are consumers: they copy a stage
// into registers, release it on its "empty" mbarrier, run the register FFT
// (kw_regfft.cuh), apply the spectral operators and store the results with
// coalesced global stores.  Loads therefore run NST tiles ahead of compute.
//
// Work units: in operator mode one unit is a tile and its items are the
// distinct input buffers of the jobs; in plain mode one unit is (buffer,
// outer index, tile).  Producer and consumers walk the same unit/item sequence.
//
// All mbarrier waits are bounded (2 s).  A timeout sets g_kw_device_error,
// the consumers agree on it through a reducing barrier and leave together,
// and thread 0 waits (bounded) for loads still in flight before the CTA exits.
#include <cstdlib>

#include "kw_kernels.cuh"
#include "kw_regfft.cuh"
#include "kw_tma.cuh"

__device__ int g_kw_device_error;

namespace {

constexpr uint64_t kWaitLimitNs = 2000000000ull;

struct TmaMaps {
  CUtensorMap m[KW_NBUF];  // one per spectral buffer (KwBuf) for the pass's axis
};

struct TmaWork {
  int ntile;   // column tiles per outer block
  int nouter;  // outer blocks (x planes for the 3-D y pass)
  int nunits;
  int nitems;  // items per unit
  int inp[KW_MAX_JOBS];  // operator mode: distinct input buffers in job order
};

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

__device__ __forceinline__ float kmag_of(const float* k0s, int ndim, int x, const ColK& g) {
  const float kx = k0s[x];
  float kk = __fadd_rn(__fmul_rn(kx, kx), g.ky2);
  if (ndim == 3) kk = __fadd_rn(kk, g.kz2);
  return sqrtf(kk);
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
  float2 op;
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

// The column-constant 1-D factor of job J (axis 1 or 2).
__device__ __forceinline__ float2 col_factor(const AxisParams& A, const AxisJob& J, const ColK& g) {
  if (J.axis == 0 || !g.valid) return make_float2(0.f, 0.f);
  const int ai = (J.axis == 1) ? g.a1 : g.a2;
  switch (J.op) {
    case OP_GRAD: return A.fg[J.axis][ai];
    case OP_DIV: return A.fd[J.axis][ai];
    case OP_UNSTAG: return A.us[J.axis][ai];
    default: return make_float2(0.f, 0.f);
  }
}

}  // namespace

// T columns per tile, CT = T * P consumer threads plus one producer warp.
// OPS selects the operator pass (A.mode == 2) or the plain transforms, so that
// each instantiation carries only one of the two code paths.
template <int E, int P, int NST, int MINB, int T, bool OPS>
__global__ void __launch_bounds__(T * P + 32, MINB)
    k_axis_tma(const __grid_constant__ AxisParams A, const __grid_constant__ TmaMaps maps, const TmaWork W) {
  constexpr int N = E * P, RS = N + E + 1, CT = T * P;
  constexpr uint32_t kStageBytes = N * T * sizeof(float2);
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  float2* stages = reinterpret_cast<float2*>(smem_raw);  // NST * N * T
  float2* ex = stages + (size_t)NST * N * T;             // T * RS
  float2* tw = ex + (size_t)T * RS;                      // N
  // x-axis tables (k, op_grad, op_div, unstag) in shared memory when they fit
  constexpr bool kTablesInSmem = N <= 512;
  constexpr int NT = kTablesInSmem ? N : 0;
  float* k0t = reinterpret_cast<float*>(tw + N);
  float2* f0t = reinterpret_cast<float2*>(k0t + NT);
  uint64_t* full = reinterpret_cast<uint64_t*>(f0t + 3 * NT);
  uint64_t* empty = full + NST;
  int* counters = reinterpret_cast<int*>(empty + NST);  // [0] issued, [1] consumed

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      kwtma::mbar_init(&full[s], 1);
      kwtma::mbar_init(&empty[s], CT / 32);
    }
    counters[0] = counters[1] = 0;
    kwtma::fence_barrier_init();
  }
  for (int i = tid; i < N; i += blockDim.x) {
    tw[i] = A.tw[i];
    if (kTablesInSmem && A.mode == 2) {
      k0t[i] = A.k[0][i];
      f0t[i] = A.fg[0][i];
      f0t[N + i] = A.fd[0][i];
      f0t[2 * N + i] = A.us[0] ? A.us[0][i] : make_float2(0.f, 0.f);
    }
  }
  __syncthreads();
  const float* k0s = kTablesInSmem ? k0t : A.k[0];
  const TabX f0s{kTablesInSmem ? f0t : A.fg[0], kTablesInSmem ? f0t + N : A.fd[0], kTablesInSmem ? f0t + 2 * N : A.us[0]};

  constexpr bool plain = !OPS;
  if (warp == CT / 32) {
    // ---------------- producer ----------------
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int u = blockIdx.x; u < W.nunits && ok; u += gridDim.x) {
        const int tile = u % W.ntile;
        const int rest = u / W.ntile;
        const int outer = rest % W.nouter;
        const int b = rest / W.nouter;
        for (int q = 0; q < W.nitems; ++q, ++it) {
          const int buf = OPS ? W.inp[q] : A.plain[b];
          const uint32_t s = it % NST, k = it / NST;
          if (k > 0 && !kwtma::mbar_wait(&empty[s], (k - 1) & 1, kWaitLimitNs)) {
            atomicExch(&g_kw_device_error, 1);
            ok = false;
            break;
          }
          kwtma::mbar_arrive_expect_tx(&full[s], kStageBytes);
          float2* dst = stages + (size_t)s * N * T;
#pragma unroll
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
    uint32_t it = 0;
    bool aborted = false;
    for (int u = blockIdx.x; u < W.nunits && !aborted; u += gridDim.x) {
      const int tile = u % W.ntile;
      const int rest = u / W.ntile;
      const int outer = rest % W.nouter;
      const int b = rest / W.nouter;
      const int c0 = tile * T;
      const bool act = cc < A.ncols - c0;
      const long long base = (long long)outer * A.os + c0 + cc;
      const long long xs = A.xs;
      ColK g;
      if constexpr (OPS) g = col_geometry(A, act ? c0 + cc : c0);
      for (int q = 0; q < W.nitems; ++q, ++it) {
        const uint32_t s = it % NST, k = it / NST;
        const bool got = kwtma::mbar_wait(&full[s], k & 1, kWaitLimitNs);
        if (consumers_any(!got, CT)) {
          if (tid == 0) atomicExch(&g_kw_device_error, 2);
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
        __syncwarp();
        if (lane == 0) kwtma::mbar_arrive(&empty[s]);

        if constexpr (!OPS) {
          float2* buf = A.bufs[A.plain[b]];
          if (A.mode == 0) {
            kwreg::Reg<E, P>::fwd(v, t, ex + cc * RS, 1, tw, sync);
            if (act) {
#pragma unroll
              for (int m = 0; m < E / P; ++m)
#pragma unroll
                for (int k2 = 0; k2 < P; ++k2) buf[base + (t + P * m + E * k2) * xs] = v[m * P + k2];
            }
          } else {
            kwreg::Reg<E, P>::rev(v, t, ex + cc * RS, 1, tw, sync);
            if (act) {
#pragma unroll
              for (int j = 0; j < E; ++j) buf[base + (t + P * j) * xs] = cconj(v[j]);
            }
          }
        } else {
        // operator mode: forward FFT of this input, then every job reading it
        kwreg::Reg<E, P>::fwd(v, t, ex + cc * RS, 1, tw, sync);
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
          apply_job<E, P>(A, J, t, g, k0s, f0s, fcol, true, act && g.valid, v, v);
          kwreg::Reg<E, P>::rev(v, t, ex + cc * RS, 1, tw, sync);
          if (act) {
            float2* out = A.bufs[J.out];
#pragma unroll
            for (int j = 0; j < E; ++j) out[base + (t + P * j) * xs] = cconj(v[j]);
          }
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
          apply_job<E, P>(A, J, t, g, k0s, f0s, fcol, !all_kappa, act && g.valid, v, y);
          kwreg::Reg<E, P>::rev(y, t, ex + cc * RS, 1, tw, sync);
          if (act) {
            float2* out = A.bufs[J.out];
#pragma unroll
            for (int j = 0; j < E; ++j) out[base + (t + P * j) * xs] = cconj(y[j]);
          }
        }
        }
      }
    }
    if (tid == 0) counters[1] = (int)it;
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
// host side
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// Two variants: 4 stages at one CTA per SM, or (lengths <= 256) 2 stages at
// two CTAs per SM.
static int g_axis_variant = -1;
static int axis_variant() {
  if (g_axis_variant < 0) {
    const char* e = getenv("KWAVE_GB300_AXIS_2CTA");
    g_axis_variant = (e && e[0] == '0') ? 0 : 1;
  }
  return g_axis_variant;
}
static int stages_for(int n) { return (n <= 256 && !axis_variant()) ? 4 : 2; }

// Tile width: plain passes along y of a 3-D grid (axis 1) use narrow 8-column
// tiles at three CTAs per SM for length 256; everything else 256 / P columns.
static bool narrow(int n, int axis) { return n == 256 && axis == 1 && axis_variant(); }
static int tile_cols(int n, int P, int axis) { return narrow(n, axis) ? 8 : 256 / P; }

static size_t tma_smem(int n, int E, int P, int axis) {
  const int T = tile_cols(n, P, axis), RS = n + E + 1;
  const size_t nt = n <= 512 ? (size_t)n : 0;
  return sizeof(float2) * ((size_t)stages_for(n) * n * T + (size_t)T * RS + n + 3 * nt) + sizeof(float) * nt +
         2 * 4 * sizeof(uint64_t) + 16;
}

// Tensor-map storage for one plan: 2 axes x 4 buffers.
struct KwTmaPlan {
  TmaMaps maps[2];
};

void* kw_tma_plan_create() { return new KwTmaPlan(); }
void kw_tma_plan_destroy(void* h) { delete static_cast<KwTmaPlan*>(h); }

// Describe buffer `b` for a pass along `axis`: a 3-D tensor of 8-byte elements
// (ncols contiguous, n along the axis with stride xs, nouter with stride os).
bool kw_tma_encode(void* h, int axis, int b, void* base, int ncols, int n, long long xs, int nouter, long long os,
                   int P) {
  KwTmaPlan* tp = static_cast<KwTmaPlan*>(h);
  EncodeTiledFn fn = encode_fn();
  if (!fn || !base) return false;
  const int T = tile_cols(n, P, axis);
  cuuint64_t dims[3] = {(cuuint64_t)ncols, (cuuint64_t)n, (cuuint64_t)nouter};
  cuuint64_t strides[2] = {(cuuint64_t)xs * 8, (cuuint64_t)(nouter > 1 ? os : xs * n) * 8};
  cuuint32_t box[3] = {(cuuint32_t)T, (cuuint32_t)(n < 256 ? n : 256), 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(&tp->maps[axis].m[b], CU_TENSOR_MAP_DATA_TYPE_INT64, 3, base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

bool kw_tma_supported(int n) {
  int E, P;
  return encode_fn() != nullptr && kw_reg_shape(n, &E, &P);
}

#define KW_TMA_SWITCH(n, CALL)                                                           \
  switch (n) {                                                                           \
    case 64: return axis_variant() ? CALL(16, 4, 2, 2, 64) : CALL(16, 4, 4, 1, 64);       \
    case 128: return axis_variant() ? CALL(16, 8, 2, 2, 32) : CALL(16, 8, 4, 1, 32);      \
    case 256:                                                                            \
      if (narrow(n, axis)) return CALL(16, 16, 2, 3, 8);                                 \
      return axis_variant() ? CALL(16, 16, 2, 2, 16) : CALL(16, 16, 4, 1, 16);            \
    case 512: return CALL(32, 16, 2, 1, 16);                                             \
    case 1024: return CALL(32, 32, 2, 1, 8);                                             \
    default: return cudaErrorInvalidValue;                                               \
  }

cudaError_t kw_tma_attr(int n, int axis) {
  int E, P;
  if (!kw_reg_shape(n, &E, &P)) return cudaErrorInvalidValue;
  const int smem = (int)tma_smem(n, E, P, axis);
#define KW_T(E_, P_, S_, B_, T_)                                                                                 \
  (cudaFuncSetAttribute(k_axis_tma<E_, P_, S_, B_, T_, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != \
           cudaSuccess                                                                                           \
       ? cudaGetLastError()                                                                                      \
       : cudaFuncSetAttribute(k_axis_tma<E_, P_, S_, B_, T_, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem))
  KW_TMA_SWITCH(n, KW_T)
#undef KW_T
}

// Launch one persistent pass along `axis` (0: operator or plain pass along x;
// 1: plain pass along y of a 3-D grid) over `nb` plain buffers or A's jobs.
cudaError_t kw_tma_launch(void* h, int axis, int n, int nouter, int nb, int nsm, cudaStream_t st, const AxisParams& A) {
  KwTmaPlan* tp = static_cast<KwTmaPlan*>(h);
  int E, P;
  if (!kw_reg_shape(n, &E, &P)) return cudaErrorInvalidValue;
  const int T = tile_cols(n, P, axis);
  TmaWork W;
  W.ntile = (A.ncols + T - 1) / T;
  W.nouter = nouter;
  if (A.mode < 2) {
    W.nitems = 1;
    W.nunits = W.ntile * nouter * nb;
  } else {
    int ni = 0;
    for (int j = 0; j < A.njobs; ++j) {
      bool seen = false;
      for (int q = 0; q < ni; ++q) seen |= (W.inp[q] == A.jobs[j].in);
      if (!seen) W.inp[ni++] = A.jobs[j].in;
    }
    W.nitems = ni;
    W.nunits = W.ntile * nouter;
  }
  const int per_sm = narrow(n, axis) ? 3 : ((n <= 256 && axis_variant()) ? 2 : 1);
  const int grid = W.nunits < nsm * per_sm ? W.nunits : nsm * per_sm;
  const size_t smem = tma_smem(n, E, P, axis);
#define KW_T(E_, P_, S_, B_, T_)                                                                          \
  ((A.mode == 2 ? k_axis_tma<E_, P_, S_, B_, T_, true><<<grid, T_ * P_ + 32, smem, st>>>(A, tp->maps[axis], W) \
                : k_axis_tma<E_, P_, S_, B_, T_, false><<<grid, T_ * P_ + 32, smem, st>>>(A, tp->maps[axis], W)), \
   cudaGetLastError())
  KW_TMA_SWITCH(n, KW_T)
#undef KW_T
}

int kw_device_error_take() {
  int v = 0, z = 0;
  if (cudaMemcpyFromSymbol(&v, g_kw_device_error, sizeof(int)) != cudaSuccess) return -1;
  if (v) cudaMemcpyToSymbol(g_kw_device_error, &z, sizeof(int));
  return v;
}
