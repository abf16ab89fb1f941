// Host side of the TMA-fed axis pass: tensor maps, pass-kind selection and
// launch geometry, and the device error word of the bounded waits.  The
// kernel itself is kw_axis_tma.cuh; its instantiations live in
// kw_axis_tma_plain.cu (plain transforms), kw_axis_tma_ops.cu (generic and
// gradient passes) and kw_axis_tma_ops2.cu (divergence and fractional-
// Laplacian passes).
#include "kw_axis_tma.cuh"

// Set by a device wait that timed out; read and cleared by
// kw_device_error_take().  Kernels get its address through TmaWork::err.
__device__ int g_kw_device_error;

static int* device_error_ptr() {
  static int* ptrs[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!ptrs[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_kw_device_error) != cudaSuccess) return nullptr;
    ptrs[dev] = static_cast<int*>(p);
  }
  return ptrs[dev];
}

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

// Tensor-map storage for one plan: 2 axes x 4 buffers.
struct KwTmaPlan {
  TmaMaps maps[2];
  bool small[2] = {false, false};  // operator passes along the axis on small tiles
};

void* kw_tma_plan_create() { return new KwTmaPlan(); }
void kw_tma_set_small(void* h, int axis, bool small) { static_cast<KwTmaPlan*>(h)->small[axis] = small; }

// Small tiles for an operator pass of length n over ncols columns (one outer
// block) when the normal tile width gives fewer tiles than SMs.
bool kw_tma_small_wanted(int n, int ncols, int nsm) {
  int E, P;
  if (!kw_tma_small_ok(n, KK_GEN) || !kw_tma_shape(n, KK_GEN, &E, &P)) return false;
  const int T = kw_tma_tile_cols(n, P, 0, KK_GEN);
  return (ncols + T - 1) / T < nsm;
}
void kw_tma_plan_destroy(void* h) { delete static_cast<KwTmaPlan*>(h); }

// Describe buffer `b` for a pass along `axis`: a 3-D tensor of 8-byte elements
// (ncols contiguous, n along the axis with stride xs, nouter with stride os).
bool kw_tma_encode(void* h, int axis, int b, void* base, int ncols, int n, long long xs, int nouter, long long os,
                   int P) {
  KwTmaPlan* tp = static_cast<KwTmaPlan*>(h);
  EncodeTiledFn fn = encode_fn();
  if (!fn || !base) return false;
  const int kind = axis == 1 ? KK_PLAIN : KK_GEN;
  int Ek, Pk;
  if (!kw_tma_shape(n, kind, &Ek, &Pk)) return false;
  (void)P;
  const int T = kw_tma_tile_cols(n, Pk, axis, kind, tp->small[axis]);
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

// Pass kind of an operator job list (see kw_axis_tma.cuh).
static int ops_kind(const AxisParams& A) {
  const int D = A.ndim;
  bool grad = A.njobs == D, div = A.njobs == D;
  for (int j = 0; j < A.njobs; ++j) {
    const AxisJob& J = A.jobs[j];
    grad &= J.in == B_P && J.out == j && J.op == OP_GRAD && J.axis == j;
    div &= J.in == j && J.out == j && J.op == OP_DIV && J.axis == j;
  }
  if (grad) return KK_GRAD;
  if (div) return KK_DIV;
  bool nab = A.njobs >= 1 && A.njobs <= 2;
  for (int j = 0; j < A.njobs; ++j) {
    const AxisJob& J = A.jobs[j];
    nab &= J.in == j && J.out == j && J.op == (j == 0 ? OP_NAB1 : OP_NAB2);
  }
  return nab ? KK_NAB : KK_GEN;
}

cudaError_t kw_tma_attr(int n, int axis, bool small) {
  cudaError_t e = kw_tma_attr_plain(n, axis, false);
  if (e != cudaSuccess || axis != 0) return e;
  if ((e = kw_tma_attr_gen(n, 0, small)) != cudaSuccess) return e;
  if ((e = kw_tma_attr_grad(n, 0, small)) != cudaSuccess) return e;
  if ((e = kw_tma_attr_div(n, 0, small)) != cudaSuccess) return e;
  return kw_tma_attr_nab(n, 0, small);
}

// Launch one persistent pass along `axis` (0: operator or plain pass along x;
// 1: plain pass along y of a 3-D grid) over `nb` plain buffers or A's jobs.
cudaError_t kw_tma_launch(void* h, int axis, int n, int nouter, int nb, int nsm, cudaStream_t st, const AxisParams& A,
                          int pdl) {
  KwTmaPlan* tp = static_cast<KwTmaPlan*>(h);
  int E, P;
  const int kind = A.mode < 2 ? KK_PLAIN : ops_kind(A);
  if (!kw_tma_shape(n, kind, &E, &P)) return cudaErrorInvalidValue;
  const bool small = tp->small[axis] && kind != KK_PLAIN;
  const int T = kw_tma_tile_cols(n, P, axis, kind, small);
  TmaWork W;
  W.pdl = pdl;
  W.err = device_error_ptr();
  if (!W.err) return cudaErrorInvalidSymbol;
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
  const int per_sm = kw_tma_per_sm(n, axis, kind, small);
  const int grid = W.nunits < nsm * per_sm ? W.nunits : nsm * per_sm;
  W.st_tile = grid % W.ntile;
  W.st_outer = (grid / W.ntile) % W.nouter;
  W.st_b = grid / W.ntile / W.nouter;
  const size_t smem = kw_tma_smem(n, E, P, axis, kind, small);
  const TmaMaps& maps = tp->maps[axis];
  switch (kind) {
    case KK_PLAIN: return kw_tma_launch_plain(n, axis, grid, smem, st, A, maps, W, false);
    case KK_GRAD: return kw_tma_launch_grad(n, axis, grid, smem, st, A, maps, W, small);
    case KK_DIV: return kw_tma_launch_div(n, axis, grid, smem, st, A, maps, W, small);
    case KK_NAB: return kw_tma_launch_nab(n, axis, grid, smem, st, A, maps, W, small);
    default: return kw_tma_launch_gen(n, axis, grid, smem, st, A, maps, W, small);
  }
}

int* kw_device_error_ptr() { return device_error_ptr(); }

int kw_device_error_take() {
  int v = 0, z = 0;
  if (cudaMemcpyFromSymbol(&v, g_kw_device_error, sizeof(int)) != cudaSuccess) return -1;
  if (v) cudaMemcpyToSymbol(g_kw_device_error, &z, sizeof(int));
  return v;
}
