// kw_gradient_noalloc: the k-space spectral derivative of the time loop,
// Re F^-1[ kappa(|k|) * i k_a e^{+i k_a d_a / 2} * F[f] ], computed without any
// device allocation.
//
// Who needs this: callers whose device memory must come from their own
// allocator or from a pool sized up front, and who therefore cannot let a
// library call cudaMalloc -- a custom operator inside a framework that owns
// the device memory (PyTorch, JAX/XLA, a TensorRT plugin), or a real-time
// pipeline that forbids allocation once it is running.  They pass the input
// and output buffers; the half-spectrum scratch and the small 1-D tables live
// in file-scope static __device__ arrays of this file.
//
// Limits and sharing rules:
//   * the scratch holds KW_NOALLOC_MAX_SPECTRUM complex values (16 MiB); a
//     grid needs (N_total / N_last) * Hp of them, Hp = (N_last/2 + 1) rounded
//     up to even, so N0*N1*Hp (3-D) or N0*Hp (2-D) must not exceed 2,097,152:
//     square grids up to 2040^2 in 2-D and cubes up to 159^3 in 3-D.  Larger grids are
//     rejected with KW_ERR_UNSUPPORTED.  Every GPU that loads the library holds
//     these arrays until the process exits.
//   * all calls share the arrays, and each call leaves its own values behind.
//     Every value a call reads is written earlier in the same call, so nothing
//     needs clearing, but calls whose work overlaps on the GPU (different
//     streams, or different host threads on one device) race on the arrays
//     and must be serialised by the caller.
//   * the first call on a device resolves the arrays' device addresses
//     (cudaGetSymbolAddress) and sets kernel attributes, with that device
//     current; make that first call before any stream capture.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/kwave_gb300.h"
#include "kw_kernels.cuh"

int kw_internal_fail(int code, const char* msg);

#define KW_NOALLOC_MAX_SPECTRUM (1 << 21)
#define KW_NOALLOC_MAX_N 4096

static __device__ __align__(256) float2 g_na_spectrum[KW_NOALLOC_MAX_SPECTRUM];
static __device__ __align__(256) float2 g_na_twiddle[3][KW_NOALLOC_MAX_N];   // axis 0, axis 1, row FFT
static __device__ __align__(256) float2 g_na_twpost[KW_NOALLOC_MAX_N / 2 + 1];
static __device__ __align__(256) float g_na_k[3][KW_NOALLOC_MAX_N];
static __device__ __align__(256) float2 g_na_op[3][KW_NOALLOC_MAX_N];

namespace {

struct NaDevice {
  bool ready = false;
  float2* spectrum = nullptr;
  float2* twiddle = nullptr;
  float2* twpost = nullptr;
  float* k = nullptr;
  float2* op = nullptr;
};

constexpr int kMaxDevices = 64;
NaDevice g_na_dev[kMaxDevices];
std::mutex g_na_mu;

int na_err(int code, const char* msg) { return kw_internal_fail(code, msg); }

#define NA_CK(call)                                       \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) {                              \
      char b_[512];                                       \
      snprintf(b_, sizeof(b_), "%s: %s", #call, cudaGetErrorString(e_)); \
      return na_err(KW_ERR_CUDA, b_);                     \
    }                                                     \
  } while (0)

bool na_factor(int n, KwFftLen& f) {
  f.n = n;
  f.nst = 0;
  int m = n;
  const int rs[5] = {4, 2, 3, 5, 7};
  for (int r : rs)
    while (m % r == 0 && m > 1) {
      if (f.nst >= KW_MAX_STAGES) return false;
      f.radix[f.nst++] = r;
      m /= r;
    }
  kw_fft_len_finish(f);
  return m == 1;
}

// Per-device set-up: device addresses of the static arrays (host code may not
// use the symbols themselves) and the shared-memory attributes of the kernels.
int na_setup(int dev, NaDevice** out);

}  // namespace

// ---------------------------------------------------------------------------
// device code
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 na_twiddle(long long j, long long n) {
  double s, c;
  sincospi(-2.0 * (double)j / (double)n, &s, &c);
  return make_float2((float)c, (float)s);
}

// 1-D tables: twiddles, k vectors (2 pi fftfreq), and the derivative operator
// along `axis` (Hermitian part: real at an even-length Nyquist bin).
__global__ void k_na_tables(int ndim, int n0, int n1, int n2, double d0, double d1, double d2, int axis, int use_sg,
                            int M, int L) {
  const int N[3] = {n0, n1, n2};
  const double d[3] = {d0, d1, d2};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < KW_NOALLOC_MAX_N; i += gridDim.x * blockDim.x) {
    for (int a = 0; a < ndim; ++a) {
      const int n = N[a];
      if (i >= n) continue;
      if (a < ndim - 1) g_na_twiddle[a][i] = na_twiddle(i, n);
      const int j = (i <= (n - 1) / 2) ? i : i - n;
      const float k32 = (float)(2.0 * M_PI * ((double)j / ((double)n * d[a])));
      g_na_k[a][i] = k32;
      if (a == axis) {
        const double kk = (double)k32;
        double re = 0.0, im = kk;  // i k
        if (use_sg) {
          double s, c;
          sincos(kk * d[a] / 2.0, &s, &c);
          re = -kk * s;
          im = kk * c;
        }
        if ((n % 2) == 0 && i == n / 2) im = 0.0;
        g_na_op[a][i] = make_float2((float)re, (float)im);
      }
    }
    if (i < M) g_na_twiddle[2][i] = na_twiddle(i, M);
    if (i <= L / 2) g_na_twpost[i] = na_twiddle(i, L);
  }
}

// Rows along the last axis: real rows of `f` -> half spectra (dir = 0), or
// half spectra -> real rows of `out` (dir = 1, unnormalised: L * x).
__global__ void __launch_bounds__(256) k_na_rows(const float* __restrict__ f, float* __restrict__ out,
                                                 float2* __restrict__ spec, int dir, int nrows, int L, int H, int Hp,
                                                 int M, int even, int R, KwFftLen flen, const float2* __restrict__ tw_g,
                                                 const float2* __restrict__ twp_g) {
  extern __shared__ float4 na_smem[];
  float2* tw = reinterpret_cast<float2*>(na_smem);
  float2* twp = tw + M;
  float2* A = twp + (L / 2 + 1);
  float2* B = A + (size_t)R * M;
  for (int i = threadIdx.x; i < M; i += blockDim.x) tw[i] = tw_g[i];
  if (even)
    for (int i = threadIdx.x; i <= L / 2; i += blockDim.x) twp[i] = twp_g[i];
  __syncthreads();
  const int r0 = blockIdx.x * R;
  const int nr = min(R, nrows - r0);
  const int tot = R * M;
  if (dir == 0) {
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
      const int row = i / M, n = i - row * M;
      float2 v = make_float2(0.f, 0.f);
      if (row < nr) {
        const float* fr = f + (long long)(r0 + row) * L;
        v = even ? make_float2(fr[2 * n], fr[2 * n + 1]) : make_float2(fr[n], 0.f);
      }
      A[i] = v;
    }
    float2* res = fft_smem<false>(A, B, flen, R, 1, M, tw);
    for (int i = threadIdx.x; i < R * H; i += blockDim.x) {
      const int row = i / H, k = i - row * H;
      if (row >= nr) continue;
      float2 X;
      if (even) {
        const float2 zk = res[row * M + (k == M ? 0 : k)];
        const float2 zc = cconj(res[row * M + (k == 0 ? 0 : M - k)]);
        const float2 e = cscale(cadd(zk, zc), 0.5f);
        const float2 dd = csub(zk, zc);
        const float2 o = make_float2(0.5f * dd.y, -0.5f * dd.x);
        X = cadd(e, cmul(twp[k], o));
      } else {
        X = res[row * L + k];
      }
      spec[(long long)(r0 + row) * Hp + k] = X;
    }
    return;
  }
  for (int i = threadIdx.x; i < tot; i += blockDim.x) {
    const int row = i / M, k = i - row * M;
    float2 z = make_float2(0.f, 0.f);
    if (row < nr) {
      const float2* sr = spec + (long long)(r0 + row) * Hp;
      if (even) {
        const float2 xk = sr[k];
        const float2 xc = cconj(sr[M - k]);
        const float2 e = cadd(xk, xc);
        const float2 o = cmul(csub(xk, xc), cconj(twp[k]));
        z = make_float2(e.x - o.y, e.y + o.x);
      } else {
        z = (k < H) ? sr[k] : cconj(sr[L - k]);
      }
    }
    A[i] = cconj(z);
  }
  float2* res = fft_smem<false>(A, B, flen, R, 1, M, tw);
  for (int i = threadIdx.x; i < tot; i += blockDim.x) {
    const int row = i / M, n = i - row * M;
    if (row >= nr) continue;
    float* orow = out + (long long)(r0 + row) * L;
    const float2 v = res[i];
    if (even) {
      orow[2 * n] = v.x;
      orow[2 * n + 1] = -v.y;
    } else {
      orow[n] = v.x;
    }
  }
}

namespace {

int na_setup(int dev, NaDevice** out) {
  std::lock_guard<std::mutex> lock(g_na_mu);
  NaDevice& d = g_na_dev[dev];
  if (!d.ready) {
    NA_CK(cudaGetSymbolAddress((void**)&d.spectrum, g_na_spectrum));
    NA_CK(cudaGetSymbolAddress((void**)&d.twiddle, g_na_twiddle));
    NA_CK(cudaGetSymbolAddress((void**)&d.twpost, g_na_twpost));
    NA_CK(cudaGetSymbolAddress((void**)&d.k, g_na_k));
    NA_CK(cudaGetSymbolAddress((void**)&d.op, g_na_op));
    NA_CK(kw_generic_attr_0(200 * 1024));
    NA_CK(cudaFuncSetAttribute(k_na_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    d.ready = true;
  }
  *out = &d;
  return KW_OK;
}

}  // namespace

extern "C" int32_t kw_gradient_noalloc(const float* f, float* out, int32_t ndim, const int32_t* shape,
                                       const double* spacing, int32_t axis, double kappa_coef, int32_t use_sg,
                                       void* stream) {
  if (!f || !out || !shape || !spacing) return na_err(KW_ERR_INVALID, "kw_gradient_noalloc: null argument");
  if (ndim != 2 && ndim != 3) return na_err(KW_ERR_UNSUPPORTED, "kw_gradient_noalloc: only 2-D and 3-D grids");
  if (axis < 0 || axis >= ndim) return na_err(KW_ERR_INVALID, "kw_gradient_noalloc: axis outside [0, ndim)");
  int N[3] = {1, 1, 1};
  double d[3] = {1.0, 1.0, 1.0};
  long long ntot = 1;
  for (int a = 0; a < ndim; ++a) {
    N[a] = shape[a];
    d[a] = spacing[a];
    if (N[a] < 2 || N[a] > KW_NOALLOC_MAX_N)
      return na_err(KW_ERR_UNSUPPORTED, "kw_gradient_noalloc: every grid size must lie in [2, 4096]");
    if (!(d[a] > 0.0)) return na_err(KW_ERR_INVALID, "kw_gradient_noalloc: grid spacing must be positive");
    ntot *= N[a];
  }
  const int L = N[ndim - 1];
  const int H = L / 2 + 1, Hp = (H + 1) & ~1;
  const int even = (L % 2) == 0;
  const int M = even ? L / 2 : L;
  const long long nrows = ntot / L;
  if (nrows * Hp > KW_NOALLOC_MAX_SPECTRUM) {
    char b[256];
    snprintf(b, sizeof(b),
             "kw_gradient_noalloc: grid needs %lld spectrum values, the static scratch holds %d (16 MiB); "
             "use the plan API for larger grids",
             nrows * Hp, KW_NOALLOC_MAX_SPECTRUM);
    return na_err(KW_ERR_UNSUPPORTED, b);
  }
  KwFftLen fl_row, fl_ax[2];
  if (!na_factor(M, fl_row)) return na_err(KW_ERR_UNSUPPORTED, "kw_gradient_noalloc: FFT length has a prime factor above 7");
  for (int a = 0; a < ndim - 1; ++a)
    if (!na_factor(N[a], fl_ax[a]))
      return na_err(KW_ERR_UNSUPPORTED, "kw_gradient_noalloc: FFT length has a prime factor above 7");

  int dev = 0;
  NA_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return na_err(KW_ERR_UNSUPPORTED, "kw_gradient_noalloc: device index too large");
  NaDevice* D;
  int rc = na_setup(dev, &D);
  if (rc) return rc;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);

  k_na_tables<<<16, 256, 0, st>>>(ndim, N[0], N[1], N[2], d[0], d[1], d[2], axis, use_sg, M, L);
  NA_CK(cudaGetLastError());

  const int R = (L >= 2048) ? 1 : (2048 / L > 16 ? 16 : 2048 / L);
  const size_t smem_rows = sizeof(float2) * ((size_t)M + L / 2 + 1 + 2 * (size_t)R * M);
  const int grid_rows = (int)((nrows + R - 1) / R);
  float2* tw_row = D->twiddle + 2 * KW_NOALLOC_MAX_N;
  k_na_rows<<<grid_rows, 256, smem_rows, st>>>(f, nullptr, D->spectrum, 0, (int)nrows, L, H, Hp, M, even, R, fl_row,
                                               tw_row, D->twpost);
  NA_CK(cudaGetLastError());

  // strided axes: forward along axis 1 (3-D), operator pass along axis 0, inverse along axis 1
  AxisParams A;
  memset(&A, 0, sizeof(A));
  A.bufs[3] = D->spectrum;
  A.ndim = ndim;
  A.H = H;
  A.Hp = Hp;
  for (int a = 0; a < ndim; ++a) {
    A.k[a] = D->k + (size_t)a * KW_NOALLOC_MAX_N;
    A.fg[a] = A.fd[a] = A.us[a] = D->op + (size_t)a * KW_NOALLOC_MAX_N;
  }
  A.kcoef = (float)kappa_coef;
  A.use_kspace = kappa_coef != 0.0;
  A.scale = (float)(1.0 / (double)ntot);
  auto tile = [](int n) {
    int T = 16;
    while (T > 1 && (size_t)3 * n * T * sizeof(float2) > 100 * 1024) T /= 2;
    return T;
  };
  auto axis_geom = [&](int a) {
    A.n = N[a];
    A.flen = fl_ax[a];
    A.tw = D->twiddle + (size_t)a * KW_NOALLOC_MAX_N;
    A.T = tile(N[a]);
    if (ndim == 3 && a == 0) {
      A.xs = (long long)N[1] * Hp;
      A.os = 0;
      A.ncols = N[1] * Hp;
    } else if (ndim == 3) {
      A.xs = Hp;
      A.os = (long long)N[1] * Hp;
      A.ncols = Hp;
    } else {
      A.xs = Hp;
      A.os = 0;
      A.ncols = Hp;
    }
  };
  auto plain = [&](int inv) -> int {
    axis_geom(1);
    A.mode = inv;
    A.njobs = 0;
    A.plain[0] = 3;
    dim3 g((A.ncols + A.T - 1) / A.T, N[0], 1);
    NA_CK(kw_axis_launch_0(g, sizeof(float2) * ((size_t)A.n + 2 * (size_t)A.n * A.T), st, A));
    NA_CK(cudaGetLastError());
    return KW_OK;
  };
  if (ndim == 3 && (rc = plain(0))) return rc;
  axis_geom(0);
  A.mode = 2;
  A.njobs = 1;
  A.jobs[0] = AxisJob{3, 3, OP_GRAD, axis};
  {
    dim3 g((A.ncols + A.T - 1) / A.T, 1, 1);
    NA_CK(kw_axis_launch_0(g, sizeof(float2) * ((size_t)A.n + 3 * (size_t)A.n * A.T), st, A));
    NA_CK(cudaGetLastError());
  }
  if (ndim == 3 && (rc = plain(1))) return rc;

  k_na_rows<<<grid_rows, 256, smem_rows, st>>>(nullptr, out, D->spectrum, 1, (int)nrows, L, H, Hp, M, even, R, fl_row,
                                               tw_row, D->twpost);
  NA_CK(cudaGetLastError());
  return KW_OK;
}
