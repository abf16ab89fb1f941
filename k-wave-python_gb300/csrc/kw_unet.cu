// Kernels of the learned warm start: a BF16 U-Net (FP32 accumulation) that
// maps a time-reversal image to an initial-pressure estimate, trained and run
// with this file's kernels only.  The reference has no counterpart; its input
// is the image of kwave/reconstruction/time_reversal.py:129-150.
//
// Tensor-core core (k_umma): one CTA of 128 threads computes a 128 x NT tile
// D[m][n] = sum_k A(m, k) B(n, k) on the 5th-generation tensor cores:
//   * the 128 threads gather 64-wide K chunks of A and B (bf16) into a
//     two-stage shared-memory ring, in the canonical K-major layout without
//     swizzle (core matrices of 8 rows x 16 bytes, 128 contiguous bytes each;
//     LBO = 128 bytes between core matrices along K, SBO = 1024 bytes between
//     8-row groups);
//   * one thread issues tcgen05.mma (kind::f16, bf16 x bf16 -> f32, M = 128,
//     N = NT, K = 16 per instruction) into an accumulator in tensor memory
//     (TMEM, allocated by warp 0) and tcgen05.commit's each stage to an
//     mbarrier, which the gatherers wait on before refilling that stage;
//   * the epilogue reads the accumulator with tcgen05.ld (warp w owns TMEM
//     lanes 32w..32w+31, one D row per thread).
// Every mbarrier wait is bounded (2 s of global time); a timeout sets the
// device error word, skips the epilogue and still frees the TMEM.
//
// Persistent convolution (k_conv_tma): the halo-tile convolution of one
// full-resolution input whose weights fit shared memory runs on persistent,
// warp-specialised CTAs instead -- a producer lane streams each tile's halo
// with 4-D TMA boxes into a shared-memory ring, one lane issues the MMAs into
// two TMEM accumulators, four warps drain the other accumulator.
//
// Gathers:
//   GEMM   A = row-major [M][K], B = row-major [N][K] (tests of the core)
//   CONV   3x3 convolution, stride 1, zero padding, NHWC bf16: m = output
//          pixel, n = output channel, k = (tap, input channel); the input is
//          one tensor or the concatenation of a full-resolution tensor and a
//          half-resolution one read through nearest-neighbour upsampling (the
//          decoder's skip + upsampled input).  The data gradient of a 3x3
//          convolution is the same gather with the flipped, transposed
//          weights and the output gradient as input.
//   WGRAD  weight gradient, k = pixel (split over CTAs, partial tiles added
//          with red.add): by default m = (tap, input channel), n = output
//          channel on MN-major tiles -- both operands are contiguous along m
//          and n in the NHWC tensors, so their 16-byte groups are copied as
//          they are (instruction descriptor bits 15/16; LBO = 128 bytes between
//          K core matrices, SBO = 1024 bytes between 8-element groups); the
//          K-major form (m = output channel) transposes 8 x 8 blocks in
//          registers instead.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/kwave_gb300.h"
#include "kw_tma.cuh"

int kw_internal_fail(int code, const char* msg);
int* kw_device_error_ptr();

namespace {

using kwtma::mbar_init;
using kwtma::mbar_wait;
using kwtma::smem_u32;

constexpr int kThreads = 128;
constexpr int kBM = 128;            // tile rows (TMEM lanes)
constexpr int kBK = 64;             // K chunk per stage (bf16: 128 bytes per row)
constexpr int kMaxNT = 256;         // tile columns (TMEM columns)
constexpr uint32_t kSBO = 1024;     // 8-row group stride in a stage tile
constexpr uint32_t kLBO = 128;      // K-adjacent core matrix stride
constexpr int kATile = kBM * kBK * 2;         // 16 KB
constexpr uint64_t kWaitNs = 2000000000ull;
constexpr int kErrUmmaTimeout = 0x55;

// tcgen05 shared-memory matrix descriptor: K-major, no swizzle; lbo = bytes
// between core matrices adjacent along K, sbo = bytes between 8-row groups.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo = kLBO, uint32_t sbo = kSBO) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of the 5th-generation tensor cores
  return d;                // base offset 0, swizzle mode 0 (none)
}

// Halo-tile convolution (mode 3): a tile is 128 consecutive pixels of one
// image row; a stage holds, for 16 input channels, the 3-row x 130-column
// halo around them (two 8-channel groups of 16-byte pixel chunks, rows of
// pixels contiguous) and the 9 taps' weights for those channels.  The nine
// taps' A operands are the same halo at nine start addresses: with one pixel
// per 16-byte row of the core matrices (SBO 128 bytes), a shift by one pixel
// is 16 bytes and by one row 130 x 16 bytes.
constexpr int kHaloCols = 130;
constexpr uint32_t kHaloGroup = 3 * kHaloCols * 16;           // bytes of one 8-channel group
constexpr uint32_t kAHalo = ((2 * kHaloGroup + 127) / 128) * 128;  // A stage bytes (16 channels)

// Instruction descriptor of kind::f16: D f32, A and B bf16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// The same with both operands MN-major (bits 15 and 16: A and B transposed).
__host__ __device__ constexpr uint32_t idesc_bf16_mn(int M, int N) { return idesc_bf16(M, N) | (1u << 15) | (1u << 16); }

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void umma_bf16(uint32_t taddr, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(taddr),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive f32 columns of this thread's TMEM lane into v[0..15]
// without waiting (tmem_wait_ld before using them).
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, float* v) {
  uint32_t* r = reinterpret_cast<uint32_t*>(v);
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 16 consecutive f32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Byte offset of the 16-byte chunk (row r, 8-wide K group kc) in a stage tile.
__device__ __forceinline__ uint32_t chunk_off(int r, int kc) {
  return (uint32_t)((r >> 3) * kSBO + kc * kLBO + (r & 7) * 16);
}

__device__ __forceinline__ uint4 ldg16(const void* p) { return __ldg(reinterpret_cast<const uint4*>(p)); }

// Word w (0..3) of a uint4, w known at compile time after unrolling.
__device__ __forceinline__ uint32_t word_of(const uint4& v, int w) {
  return w == 0 ? v.x : w == 1 ? v.y : w == 2 ? v.z : v.w;
}

// 8 x 8 bf16 transpose: in[j] holds 8 values of row j; out[i] gets element i
// of every row.  Word q of out[i] pairs element i of rows 2q and 2q + 1,
// picked with byte permutes (low halves for even i, high halves for odd i).
__device__ __forceinline__ void transpose8(const uint4 (&in)[8], uint4 (&out)[8]) {
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const uint32_t sel = (i & 1) ? 0x7632u : 0x5410u;
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) w[q] = __byte_perm(word_of(in[2 * q], i >> 1), word_of(in[2 * q + 1], i >> 1), sel);
    out[i] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// gather policies
// ---------------------------------------------------------------------------
struct UmmaArgs {
  int mode;  // 0 GEMM, 1 CONV, 2 WGRAD, 3 CONV on halo tiles, 4 GEMM of MN-major operands, 5 WGRAD MN-major
  int M, N, K;
  int NT;    // tile columns (multiple of 16, <= 256)
  // GEMM
  const __nv_bfloat16* A;
  const __nv_bfloat16* B;
  float* C;
  // CONV / WGRAD geometry
  int nb, H, W;       // batch, output height and width (= input height and width)
  int C1, C2;         // channels of the full-resolution input and of the half-resolution one (0: none)
  const __nv_bfloat16* X1;
  const __nv_bfloat16* X2;
  const __nv_bfloat16* Wt;   // CONV weights [N][9][C1 + C2]
  const float* bias;         // CONV: per output channel (may be null)
  int relu;                  // CONV: apply ReLU
  __nv_bfloat16* Y;          // CONV output [pixels][N] bf16 (may be null)
  float* Yf;                 // CONV output [pixels][N] f32 (may be null)
  const __nv_bfloat16* dZ;   // WGRAD: output gradient [pixels][M]
  float* dW;                 // WGRAD: [M][N] f32, accumulated
  int ksplit;                // WGRAD: pixels per CTA; CONV split over K: K values per CTA (multiple of 64, 0: no split)
};

// 16-byte chunk of the convolution input at pixel (b, y, x) of the output
// grid shifted by tap, channels ci..ci+7 (zero outside the image); bimg is the
// index of the image's first pixel, b * H * W.
__device__ __forceinline__ uint4 conv_chunk_at(const UmmaArgs& a, int bimg, int y, int x, int tap, int ci) {
  y += tap / 3 - 1;
  x += tap % 3 - 1;
  if (tap >= 9 || y < 0 || y >= a.H || x < 0 || x >= a.W) return make_uint4(0, 0, 0, 0);
  if (ci < a.C1) return ldg16(a.X1 + ((long long)bimg + y * a.W + x) * a.C1 + ci);
  const int w2 = a.W >> 1;
  return ldg16(a.X2 + ((long long)(bimg >> 2) + (y >> 1) * w2 + (x >> 1)) * a.C2 + (ci - a.C1));
}

// Per-thread state of the CONV operand gathers.  Thread tid fills the 8-wide
// K group kc = (tid >> 3) & 7 of the tile rows r_i = (2 i + (tid >> 6)) * 8 +
// (tid & 7), i < 8, in every chunk: their output pixels are decomposed once
// per tile, and the group's (tap, channel) advances by 64 per chunk without
// divisions.
struct ConvRows {
  int bimg[8];  // b * H * W of the row's pixel, -1 beyond the batch
  int yx[8];    // y << 16 | x
  int tap, ci;
  __device__ __forceinline__ void init(const UmmaArgs& a, int m0, int kbeg) {
    const int tid = threadIdx.x, hw = a.H * a.W;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int m = m0 + (2 * i + (tid >> 6)) * 8 + (tid & 7);
      if (m < a.M) {
        const int b = m / hw, rem = m - b * hw;
        bimg[i] = b * hw;
        yx[i] = ((rem / a.W) << 16) | (rem % a.W);
      } else {
        bimg[i] = -1;
        yx[i] = 0;
      }
    }
    const int cin = a.C1 + a.C2, k = kbeg + ((tid >> 3) & 7) * 8;
    tap = k / cin;
    ci = k - tap * cin;
  }
  __device__ __forceinline__ void advance(int cin) {
    ci += kBK;
    while (ci >= cin) {
      ci -= cin;
      ++tap;
    }
  }
};

// Fill stage tiles for K chunk k0 (all 128 threads).
__device__ __forceinline__ void fill_stage(const UmmaArgs& a, unsigned char* sA, unsigned char* sB, int m0, int n0,
                                           int k0, ConvRows& cr) {
  const int tid = threadIdx.x;
  if (a.mode == 5) {
    // weight gradient on MN-major tiles: m = (tap, input channel), n = output
    // channel, k = pixel; A(p, m) = input[p + tap][ci], B(p, n) = dz[p][co]:
    // both 8-wide groups are 16 contiguous bytes of the NHWC tensors, copied
    // as they are (chunk layout as in mode 4)
    const int k = tid & 63;
    const int p = k0 + k;
    const bool pin = p < a.K;
    int bimg = 0, y = 0, x = 0;
    if (pin) {
      const int hw = a.H * a.W;
      const int b = p / hw, rem = p - b * hw;
      bimg = b * hw;
      y = rem / a.W;
      x = rem - y * a.W;
    }
    const int cin = a.C1 + a.C2;
#pragma unroll
    for (int it = 0; it < 8; ++it) {
      const int g = it * 2 + (tid >> 6);
      const int m = m0 + g * 8;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (pin && m < a.M) {
        const int tap = m / cin;
        v = conv_chunk_at(a, bimg, y, x, tap, m - tap * cin);
      }
      *reinterpret_cast<uint4*>(sA + g * 1024 + (k >> 3) * 128 + (k & 7) * 16) = v;
    }
    for (int c = tid; c < a.NT * 8; c += kThreads) {
      const int kk = c & 63, g = c >> 6;
      const int n = n0 + g * 8, pp = k0 + kk;
      const uint4 v = (n < a.N && pp < a.K) ? ldg16(a.dZ + (long long)pp * a.N + n) : make_uint4(0, 0, 0, 0);
      *reinterpret_cast<uint4*>(sB + g * 1024 + (kk >> 3) * 128 + (kk & 7) * 16) = v;
    }
    return;
  }
  if (a.mode == 4) {
    // MN-major tiles: A[k][m], B[k][n] row-major; chunk (8-row group g of M or N,
    // k) = 8 consecutive m (n) at one k, stored at g * 1024 + (k / 8) * 128 + (k % 8) * 16
#pragma unroll
    for (int it = 0; it < 8; ++it) {
      const int c = it * kThreads + tid;
      const int k = c & 63, g = c >> 6;
      const int m = m0 + g * 8, kk = k0 + k;
      const uint4 v = (m < a.M && kk < a.K) ? ldg16(a.A + (long long)kk * a.M + m) : make_uint4(0, 0, 0, 0);
      *reinterpret_cast<uint4*>(sA + g * 1024 + (k >> 3) * 128 + (k & 7) * 16) = v;
    }
    for (int c = tid; c < a.NT * 8; c += kThreads) {
      const int k = c & 63, g = c >> 6;
      const int n = n0 + g * 8, kk = k0 + k;
      const uint4 v = (n < a.N && kk < a.K) ? ldg16(a.B + (long long)kk * a.N + n) : make_uint4(0, 0, 0, 0);
      *reinterpret_cast<uint4*>(sB + g * 1024 + (k >> 3) * 128 + (k & 7) * 16) = v;
    }
    return;
  }
  if (a.mode == 2) {
    // WGRAD: A(co, p) = dZ[p][co], B((tap, ci), p) = input[p + tap][ci]; 8 x 8 blocks transposed
    {
      const int cb = tid >> 3, pb = tid & 7;  // 16 channel blocks x 8 pixel blocks
      uint4 in[8], out[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int p = k0 + pb * 8 + j;
        const int co = m0 + cb * 8;
        in[j] = (p < a.K && co < a.M) ? ldg16(a.dZ + (long long)p * a.M + co) : make_uint4(0, 0, 0, 0);
      }
      transpose8(in, out);
#pragma unroll
      for (int i = 0; i < 8; ++i) *reinterpret_cast<uint4*>(sA + chunk_off(cb * 8 + i, pb)) = out[i];
    }
    const int nblk = (a.NT >> 3) * 8;
    const int cin = a.C1 + a.C2, hw = a.H * a.W;
    for (int q = tid; q < nblk; q += kThreads) {
      const int nb8 = q >> 3, pb = q & 7;
      const int n = n0 + nb8 * 8;
      const int tap = n / cin, ci = n - tap * cin;
      // the block's 8 consecutive pixels, walked from the first without divisions
      const int p0 = k0 + pb * 8;
      int b = p0 / hw, rem = p0 - b * hw;
      int y = rem / a.W, x = rem - y * a.W;
      uint4 in[8], out[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        in[j] = (p0 + j < a.K && n < a.N) ? conv_chunk_at(a, b * hw, y, x, tap, ci) : make_uint4(0, 0, 0, 0);
        if (++x == a.W) {
          x = 0;
          if (++y == a.H) {
            y = 0;
            ++b;
          }
        }
      }
      transpose8(in, out);
#pragma unroll
      for (int i = 0; i < 8; ++i) *reinterpret_cast<uint4*>(sB + chunk_off(nb8 * 8 + i, pb)) = out[i];
    }
    return;
  }
  // GEMM / CONV: A rows are output rows (pixels), 8 K groups of 8 per row;
  // this thread's group is kc, its rows those of ConvRows
  const int kc = (tid >> 3) & 7;
  if (a.mode == 0) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = (2 * i + (tid >> 6)) * 8 + (tid & 7);
      const int m = m0 + r, k = k0 + kc * 8;
      const uint4 v = (m < a.M && k < a.K) ? ldg16(a.A + (long long)m * a.K + k) : make_uint4(0, 0, 0, 0);
      *reinterpret_cast<uint4*>(sA + chunk_off(r, kc)) = v;
    }
  } else {
    uint4 v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
      v[i] = cr.bimg[i] < 0 ? make_uint4(0, 0, 0, 0)
                            : conv_chunk_at(a, cr.bimg[i], cr.yx[i] >> 16, cr.yx[i] & 0xFFFF, cr.tap, cr.ci);
#pragma unroll
    for (int i = 0; i < 8; ++i)
      *reinterpret_cast<uint4*>(sA + chunk_off((2 * i + (tid >> 6)) * 8 + (tid & 7), kc)) = v[i];
    cr.advance(a.C1 + a.C2);
  }
  const __nv_bfloat16* Bm = a.mode == 0 ? a.B : a.Wt;
  for (int c = tid; c < a.NT * 8; c += kThreads) {
    const int r = (c >> 6) * 8 + (c & 7), kc = (c >> 3) & 7;
    const int n = n0 + r, k = k0 + kc * 8;
    const uint4 v = (n < a.N && k < a.K) ? ldg16(Bm + (long long)n * a.K + k) : make_uint4(0, 0, 0, 0);
    *reinterpret_cast<uint4*>(sB + chunk_off(r, kc)) = v;
  }
}

// Fill a halo stage: A halo of channels ci0..ci0+15 around pixels (y, x0..x0+127)
// of image bimg, and the 9 taps x NT output channels of weights for them.
__device__ __forceinline__ void fill_halo(const UmmaArgs& a, unsigned char* sA, unsigned char* sB, int bimg, int y,
                                          int x0, int n0, int ci0) {
  const int tid = threadIdx.x;
  for (int q = tid; q < 2 * 3 * kHaloCols; q += kThreads) {
    const int kg = q / (3 * kHaloCols), rem = q - kg * (3 * kHaloCols);
    const int r = rem / kHaloCols, col = rem - r * kHaloCols;
    const int yy = y + r - 1, xx = x0 + col - 1, ci = ci0 + kg * 8;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (yy >= 0 && yy < a.H && xx >= 0 && xx < a.W) {
      if (ci < a.C1)
        v = ldg16(a.X1 + ((long long)bimg + yy * a.W + xx) * a.C1 + ci);
      else
        v = ldg16(a.X2 + ((long long)(bimg >> 2) + (yy >> 1) * (a.W >> 1) + (xx >> 1)) * a.C2 + (ci - a.C1));
    }
    *reinterpret_cast<uint4*>(sA + kg * kHaloGroup + rem * 16) = v;
  }
  const int cin = a.C1 + a.C2;
  for (int q = tid; q < 18 * a.NT; q += kThreads) {
    const int kg = q & 1, nt = q >> 1;
    const int n = nt / 9, tap = nt - n * 9;
    const uint4 v = (n0 + n < a.N) ? ldg16(a.Wt + ((long long)(n0 + n) * 9 + tap) * cin + ci0 + kg * 8)
                                   : make_uint4(0, 0, 0, 0);
    *reinterpret_cast<uint4*>(sB + ((tap * 2 + kg) * a.NT + n) * 16) = v;
  }
}

__global__ void __launch_bounds__(kThreads) k_umma(UmmaArgs a, int* err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  // stage s: A at base + s astage, B at base + 2 astage + s bstage
  const bool halo = a.mode == 3;
  const uint32_t astage = halo ? kAHalo : (uint32_t)kATile;
  const uint32_t bstage = halo ? (uint32_t)a.NT * 288u : (uint32_t)a.NT * (kBK * 2);
  uint64_t* bar = reinterpret_cast<uint64_t*>(base + 2 * astage + 2 * bstage);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
  __shared__ int s_fail;

  const int tid = threadIdx.x, warp = tid >> 5;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * a.NT;
  const uint32_t ncols = a.NT <= 32 ? 32 : a.NT <= 64 ? 64 : a.NT <= 128 ? 128 : 256;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    s_fail = 0;
    kwtma::fence_barrier_init();
  }
  if (warp == 0) tmem_alloc(tslot, ncols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  int kbeg = 0, kend = a.K;
  if (a.mode == 2 || a.mode == 5 || (a.mode == 1 && a.ksplit > 0)) {
    kbeg = blockIdx.z * a.ksplit;
    kend = min(a.K, kbeg + a.ksplit);
  }
  const int nchunks = halo ? (a.C1 + a.C2) / 16 : (kend - kbeg + kBK - 1) / kBK;
  // MN-major tiles (modes 4, 5): 8-element groups along M / N 1024 bytes apart
  // (SBO), K core matrices 128 bytes apart (LBO), as in the K-major layout
  const bool mn = a.mode == 4 || a.mode == 5;
  const uint32_t idesc = mn ? idesc_bf16_mn(kBM, a.NT) : idesc_bf16(kBM, a.NT);
  int hb = 0, hy = 0, hx = 0;  // halo tiles: image, row and first column of the tile
  if (halo) {
    const int hw = a.H * a.W;
    hb = (m0 / hw) * hw;
    hy = (m0 - hb) / a.W;
    hx = m0 - hb - hy * a.W;
  }
  ConvRows cr;
  if (a.mode == 1) cr.init(a, m0, kbeg);
  bool ok = true;
  for (int c = 0; c < nchunks && ok; ++c) {
    const int s = c & 1;
    if (c >= 2) {
      if (!mbar_wait(&bar[s], ((c - 2) >> 1) & 1, kWaitNs)) ok = false;
      if (__syncthreads_or(!ok)) {
        ok = false;
        break;
      }
    }
    unsigned char* sAs = base + s * astage;
    unsigned char* sBs = base + 2 * astage + s * bstage;
    if (halo)
      fill_halo(a, sAs, sBs, hb, hy, hx, n0, c * 16);
    else
      fill_stage(a, sAs, sBs, m0, n0, kbeg + c * kBK, cr);
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint32_t ab = smem_u32(sAs), bb = smem_u32(sBs);
      if (halo) {
        // tap (dy, dx): the halo from row 1 + dy, column 1 + dx; the tap's weights
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
          const uint32_t aoff = (uint32_t)(((tap / 3) * kHaloCols + (tap % 3)) * 16);
          umma_bf16(tmem, smem_desc(ab + aoff, kHaloGroup, 128), smem_desc(bb + tap * 2 * a.NT * 16, a.NT * 16, 128),
                    idesc, (c | tap) != 0);
        }
      } else if (mn) {
#pragma unroll
        for (int kk = 0; kk < kBK / 16; ++kk)
          umma_bf16(tmem, smem_desc(ab + kk * 256, 128, 1024), smem_desc(bb + kk * 256, 128, 1024), idesc,
                    (c | kk) != 0);
      } else {
#pragma unroll
        for (int kk = 0; kk < kBK / 16; ++kk)
          umma_bf16(tmem, smem_desc(ab + kk * 2 * kLBO), smem_desc(bb + kk * 2 * kLBO), idesc, (c | kk) != 0);
      }
      umma_commit(&bar[s]);
    }
  }
  if (ok && nchunks > 0) {
    const int L = nchunks - 1;
    if (!mbar_wait(&bar[L & 1], (L >> 1) & 1, kWaitNs)) ok = false;
  }
  if (!ok) s_fail = 1;
  __syncthreads();
  tc_fence_after();
  if (!s_fail && nchunks > 0) {
    const int r = warp * 32 + (tid & 31);
    const int m = m0 + r;
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    for (int j0 = 0; j0 < a.NT; j0 += 16) {
      float v[16];
      tmem_ld16(trow + (uint32_t)j0, v);
      if (m >= a.M) continue;
      if (a.mode == 0 || a.mode == 4) {
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (n0 + j0 + j < a.N) a.C[(long long)m * a.N + n0 + j0 + j] = v[j];
      } else if (a.mode == 1 && a.ksplit > 0) {
        // CONV split over K: this CTA's partial sums; bias, ReLU and the
        // stores follow in k_conv_finish
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int n = n0 + j0 + j;
          if (n < a.N) atomicAdd(a.C + (long long)m * a.N + n, v[j]);
        }
      } else if (a.mode == 1 || a.mode == 3) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int n = n0 + j0 + j;
          float y = v[j] + ((a.bias && n < a.N) ? a.bias[n] : 0.f);
          if (a.relu) y = fmaxf(y, 0.f);
          v[j] = y;
        }
        const long long o = (long long)m * a.N + n0 + j0;
        if (n0 + j0 + 16 <= a.N) {
          if (a.Y) {
            uint32_t w[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
              w[q] = *reinterpret_cast<const uint32_t*>(&h);
            }
            *reinterpret_cast<uint4*>(a.Y + o) = make_uint4(w[0], w[1], w[2], w[3]);
            *reinterpret_cast<uint4*>(a.Y + o + 8) = make_uint4(w[4], w[5], w[6], w[7]);
          }
          if (a.Yf) {
#pragma unroll
            for (int q = 0; q < 4; ++q)
              *reinterpret_cast<float4*>(a.Yf + o + 4 * q) = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
          }
        } else {
          for (int j = 0; j < 16 && n0 + j0 + j < a.N; ++j) {
            if (a.Y) a.Y[o + j] = __float2bfloat16_rn(v[j]);
            if (a.Yf) a.Yf[o + j] = v[j];
          }
        }
      } else if (a.mode == 5) {
        // WGRAD on MN-major tiles: row m = (tap, ci), column n = co -> dW[co][tap][ci]
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int n = n0 + j0 + j;
          if (n < a.N) atomicAdd(a.dW + (long long)n * a.M + m, v[j]);
        }
      } else {
        // WGRAD: add this pixel range's partial tile
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int n = n0 + j0 + j;
          if (n < a.N) atomicAdd(a.dW + (long long)m * a.N + n, v[j]);
        }
      }
    }
  }
  if (s_fail && tid == 0 && err) atomicCAS(err, 0, kErrUmmaTimeout);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, ncols);
}

// ---------------------------------------------------------------------------
// persistent, TMA-fed convolution on halo tiles (k_conv_tma)
// ---------------------------------------------------------------------------
// The same halo-tile convolution as k_umma mode 3 for one full-resolution
// input (no concatenation) whose weights fit shared memory, restructured so
// that staging, tensor-core work and the epilogue overlap:
//   * the CTA is persistent over tiles blockIdx.x, blockIdx.x + gridDim.x, ...
//     (a tile: 128 pixels of a.rows = 1 or 2 image rows, all output
//     channels; two rows stage each input row for two outputs instead of
//     three);
//   * the weights of all input channels stay in shared memory for the whole
//     kernel, in the B layout of mode 3 ([16-channel group][tap][8-channel
//     half][output channel][8 channels]);
//   * warp 4 (one lane) is the producer: per group of a.gc channels of a
//     tile it loads the (rows + 2) x 130-pixel halo with one 4-D TMA box
//     (tensor map over the NHWC input, whole pixels as swizzled rows, zero
//     fill outside the image) into a ring of a.stages stages (chosen per
//     launch), completion on full[s];
//   * warp 5 (one lane) issues nine tcgen05.mma per 16 channels and output
//     row (row rr reads the halo from row rr on) into the tile's accumulators in
//     one of two TMEM buffers, commits each group to empty[s] (the producer
//     may refill the stage) and each finished tile to tfull[b];
//   * warps 0-3 read accumulator b (warp w: TMEM lanes 32w..32w+31), apply
//     bias and ReLU, store bf16 and/or f32 rows, and arrive on tempty[b] so
//     that the tile after next may overwrite it.
// Every wait is bounded; a timeout sets s_fail, every role leaves its loop,
// the producer waits (bounded) for its last copies and the MMA lane for its
// last MMAs before the CTA frees its TMEM.
constexpr int kCtThreads = 192;
constexpr int kCtMaxStages = 4;

// A stage is the halo of one channel group of gc = 16, 32 or 64 channels for
// a tile of `rows` image rows: (rows + 2) x 130 pixels of gc * 2 bytes, one
// TMA box written in the K-major swizzled layout of that row width (32-, 64-
// or 128-byte swizzle: each pixel is one row of the tensor-core operand, its
// 16-byte chunks permuted by the shared-memory address bits of the row).  The
// tensor cores apply the same permutation from the absolute address, so the
// nine taps stay nine descriptor start addresses, whole pixel rows apart,
// with base offset 0 (verified on the GPU for all three widths and row shifts
// that are not multiples of the 8-row swizzle atom).  Stages start 1024-byte
// aligned.
__host__ __device__ inline uint32_t conv_tma_box(int rows, int gc) {
  return (uint32_t)((rows + 2) * kHaloCols * gc * 2);
}
__host__ __device__ inline uint32_t conv_tma_stage(int rows, int gc) { return (conv_tma_box(rows, gc) + 1023u) & ~1023u; }
// tcgen05 layout code of a K-major swizzle for rows of `rowbytes` bytes
__host__ __device__ inline uint32_t conv_tma_layout(int rowbytes) {
  return rowbytes == 128 ? 2u : rowbytes == 64 ? 4u : 6u;
}

// Shared-memory descriptor of a swizzled K-major operand (rows of rowbytes,
// 8-row atoms rowbytes * 8 apart; LBO unused within the atom).
__device__ __forceinline__ uint64_t smem_desc_swz(uint32_t addr, uint32_t rowbytes) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(((8 * rowbytes) >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)conv_tma_layout((int)rowbytes) << 61;
  return d;
}

struct ConvTmaArgs {
  int nb, H, W, C1, N, NT;  // NT: N rounded up to 16 (one column tile)
  int rows;                 // image rows per tile (1 or 2; H % rows == 0)
  int gc;                   // channels per stage (16, 32 or 64; C1 % gc == 0)
  int ntiles;               // nb * (H / rows) * (W / 128)
  int stages;               // depth of the halo ring (2..kCtMaxStages)
  const __nv_bfloat16* Wt;  // [N][9][C1]
  const float* bias;
  int relu;
  __nv_bfloat16* Y;
  float* Yf;
};

__host__ __device__ inline uint32_t conv_tma_wbytes(int C1, int NT) { return (uint32_t)(9 * C1 * NT * 2); }

// two tiles' accumulators of `rows` x NT columns
__host__ __device__ inline uint32_t conv_tma_tmem_cols(int NT, int rows) {
  const int c = 2 * rows * NT;
  return c <= 32 ? 32 : c <= 64 ? 64 : c <= 128 ? 128 : c <= 256 ? 256 : 512;
}

__global__ void __launch_bounds__(kCtThreads) k_conv_tma(const __grid_constant__ CUtensorMap xmap, ConvTmaArgs a,
                                                         int* err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int groups = a.C1 / a.gc, k16 = a.gc / 16;
  const uint32_t wbytes = conv_tma_wbytes(a.C1, a.NT);
  const int S = a.stages, R = a.rows;
  const uint32_t rowbytes = (uint32_t)a.gc * 2, stage_bytes = conv_tma_stage(R, a.gc);
  unsigned char* sW = base;
  float* sBias = reinterpret_cast<float*>(base + ((wbytes + 1023) & ~1023u));
  unsigned char* sH = reinterpret_cast<unsigned char*>(sBias) + 1024;
  uint64_t* full = reinterpret_cast<uint64_t*>(sH + S * stage_bytes);
  uint64_t* empty = full + S;
  uint64_t* tfull = empty + S;
  uint64_t* tempty = tfull + 2;
  uint64_t* done = tempty + 2;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  __shared__ volatile int s_fail;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t ncols = conv_tma_tmem_cols(a.NT, R);
  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 128);
    }
    mbar_init(done, 1);
    s_fail = 0;
    kwtma::fence_barrier_init();
  }
  if (warp == 0) tmem_alloc(tslot, ncols);
  // weights of every 16-channel group: [c][tap][half][n][8 channels]
  const int wrows = (a.C1 / 16) * 18 * a.NT;  // every 16-channel chunk
  for (int q = tid; q < wrows; q += kCtThreads) {
    const int c = q / (18 * a.NT), r = q - c * 18 * a.NT;
    const int th = r / a.NT, n = r - th * a.NT;
    const int tap = th >> 1, half = th & 1;
    const uint4 v = (n < a.N) ? ldg16(a.Wt + ((long long)n * 9 + tap) * a.C1 + c * 16 + half * 8)
                              : make_uint4(0, 0, 0, 0);
    *reinterpret_cast<uint4*>(sW + (uint32_t)q * 16) = v;
  }
  for (int n = tid; n < a.NT; n += kCtThreads) sBias[n] = (a.bias && n < a.N) ? a.bias[n] : 0.f;
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const int segs = a.W / 128;

  if (warp == 4) {
    if (lane == 0) {
      // producer, TMA: two 4-D boxes per stage
      int q = 0;
      for (int t = blockIdx.x; t < a.ntiles && !s_fail; t += gridDim.x) {
        const int seg = t % segs, blk = t / segs;
        const int hb = a.H / R;
        const int y = (blk % hb) * R, b = blk / hb;
        for (int c = 0; c < groups; ++c, ++q) {
          const int s = q % S;
          if (q >= S && !mbar_wait(&empty[s], ((q / S) - 1) & 1, kWaitNs)) {
            s_fail = 1;
            break;
          }
          if (s_fail) break;
          kwtma::mbar_arrive_expect_tx(&full[s], conv_tma_box(R, a.gc));
          kwtma::tma_load_4d(sH + s * stage_bytes, &xmap, c * a.gc, seg * 128 - 1, y - 1, b, &full[s]);
        }
      }
      // the last use of each stage: its copies must have landed before the CTA ends
      for (int k = q - 1; k >= 0 && k >= q - S; --k)
        if (!mbar_wait(&full[k % S], (k / S) & 1, kWaitNs)) s_fail = 1;
    }
  } else if (warp == 5) {
    if (lane == 0) {
      // tensor-core issuer
      const uint32_t idesc = idesc_bf16(kBM, a.NT);
      int q = 0, i = 0;
      for (int t = blockIdx.x; t < a.ntiles && !s_fail; t += gridDim.x, ++i) {
        const int b = i & 1;
        if (i >= 2 && !mbar_wait(&tempty[b], ((i >> 1) - 1) & 1, kWaitNs)) {
          s_fail = 1;
          break;
        }
        tc_fence_after();
        const uint32_t acc = tmem + (uint32_t)(b * R * a.NT);
        bool ok = true;
        for (int c = 0; c < groups; ++c, ++q) {
          const int s = q % S;
          if (!mbar_wait(&full[s], (q / S) & 1, kWaitNs) || s_fail) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t ab = smem_u32(sH + s * stage_bytes);
          // output row rr of the tile: halo rows rr .. rr + 2, accumulator rr;
          // 16 channels per MMA, 32 bytes further along the pixel row
          for (int rr = 0; rr < R; ++rr) {
            for (int kk = 0; kk < k16; ++kk) {
              const uint32_t bb = smem_u32(sW + (uint32_t)(c * k16 + kk) * 18 * a.NT * 16);
#pragma unroll
              for (int tap = 0; tap < 9; ++tap) {
                const uint32_t aoff = (uint32_t)((tap / 3 + rr) * kHaloCols + (tap % 3)) * rowbytes + kk * 32;
                umma_bf16(acc + (uint32_t)(rr * a.NT), smem_desc_swz(ab + aoff, rowbytes),
                          smem_desc(bb + tap * 2 * a.NT * 16, a.NT * 16, 128), idesc, (c | kk | tap) != 0);
              }
            }
          }
          umma_commit(&empty[s]);
        }
        if (!ok) {
          s_fail = 1;
          break;
        }
        umma_commit(&tfull[b]);
      }
      // every MMA issued by this thread has completed before the TMEM is freed
      umma_commit(done);
      if (!mbar_wait(done, 0, kWaitNs)) s_fail = 1;
    }
  } else {
    // epilogue: warps 0-3, one accumulator row per thread
    int i = 0;
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x, ++i) {
      const int b = i & 1;
      // the warp leaves together: tcgen05.ld below is warp-collective
      const bool ok = mbar_wait(&tfull[b], (i >> 1) & 1, kWaitNs);
      if (__any_sync(0xffffffffu, !ok || s_fail)) {
        s_fail = 1;
        break;
      }
      tc_fence_after();
      const int r = warp * 32 + lane;
      const int seg = t % segs, blk = t / segs;
      const int hb = a.H / R;
      const int y0 = (blk % hb) * R, bimg = blk / hb;
      // the tile's R rows x NT columns as one list of 16-column groups (a group
      // never straddles two rows, NT being a multiple of 16); up to four
      // groups per TMEM round trip, their loads in flight together
      const int ngroups = R * (a.NT / 16), gpr = a.NT / 16;
      const uint32_t tlane = tmem + (uint32_t)(b * R * a.NT) + ((uint32_t)(warp * 32) << 16);
      for (int g0 = 0; g0 < ngroups; g0 += 4) {
        float vv[64];
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (g0 + q < ngroups) tmem_ld16_nowait(tlane + (uint32_t)((g0 + q) * 16), vv + q * 16);
        tmem_wait_ld();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (g0 + q >= ngroups) break;
          const int rr = (g0 + q) / gpr, j0 = ((g0 + q) - rr * gpr) * 16;
          const long long m = ((long long)(bimg * a.H + y0 + rr) * a.W + seg * 128) + r;
          float* v = vv + q * 16;
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            float yv = v[j] + sBias[j0 + j];
            if (a.relu) yv = fmaxf(yv, 0.f);
            v[j] = yv;
          }
          const long long o = m * a.N + j0;
          if (j0 + 16 <= a.N) {
            if (a.Y) {
              uint32_t w[8];
#pragma unroll
              for (int qq = 0; qq < 8; ++qq) {
                const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * qq], v[2 * qq + 1]);
                w[qq] = *reinterpret_cast<const uint32_t*>(&h);
              }
              *reinterpret_cast<uint4*>(a.Y + o) = make_uint4(w[0], w[1], w[2], w[3]);
              *reinterpret_cast<uint4*>(a.Y + o + 8) = make_uint4(w[4], w[5], w[6], w[7]);
            }
            if (a.Yf) {
#pragma unroll
              for (int qq = 0; qq < 4; ++qq)
                *reinterpret_cast<float4*>(a.Yf + o + 4 * qq) =
                    make_float4(v[4 * qq], v[4 * qq + 1], v[4 * qq + 2], v[4 * qq + 3]);
            }
          } else {
            for (int j = 0; j < 16 && j0 + j < a.N; ++j) {
              if (a.Y) a.Y[o + j] = __float2bfloat16_rn(v[j]);
              if (a.Yf) a.Yf[o + j] = v[j];
            }
          }
        }
      }
      tc_fence_before();
      kwtma::mbar_arrive(&tempty[b]);
    }
  }
  __syncthreads();
  if (s_fail && tid == 0 && err) atomicCAS(err, 0, kErrUmmaTimeout);
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, ncols);
}

// Bias, ReLU and stores of a convolution whose K range was split over CTAs:
// acc holds the sums of the partial tiles, [pixels][n] f32.
__global__ void k_conv_finish(const float* __restrict__ acc, const float* __restrict__ bias, int relu,
                              __nv_bfloat16* __restrict__ y, float* __restrict__ yf, long long total, int n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    float v = acc[i] + (bias ? bias[i % n] : 0.f);
    if (relu) v = fmaxf(v, 0.f);
    if (y) y[i] = __float2bfloat16_rn(v);
    if (yf) yf[i] = v;
  }
}

// ---------------------------------------------------------------------------
// elementwise kernels of the network (bf16 NHWC activations, f32 parameters)
// ---------------------------------------------------------------------------
// 2 x 2 average pooling, NHWC.
__global__ void k_avgpool2(const __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ y, int nb, int H, int W,
                           int C) {
  const int h2 = H / 2, w2 = W / 2;
  const long long n = (long long)nb * h2 * w2 * C;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    long long q = i / C;
    const int xo = (int)(q % w2);
    q /= w2;
    const int yo = (int)(q % h2);
    const int b = (int)(q / h2);
    const long long r0 = (((long long)b * H + 2 * yo) * W + 2 * xo) * C + c;
    const float s = __bfloat162float(x[r0]) + __bfloat162float(x[r0 + C]) + __bfloat162float(x[r0 + (long long)W * C]) +
                    __bfloat162float(x[r0 + (long long)W * C + C]);
    y[i] = __float2bfloat16_rn(0.25f * s);
  }
}

// Gradient of 2 x 2 average pooling, added into dx (f32 accumulation buffer or
// bf16 with add = 0 meaning overwrite).
__global__ void k_avgpool2_bwd(const __nv_bfloat16* __restrict__ dy, __nv_bfloat16* __restrict__ dx, int nb, int H,
                               int W, int C, const __nv_bfloat16* __restrict__ add) {
  const long long n = (long long)nb * H * W * C;
  const int h2 = H / 2, w2 = W / 2;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    long long q = i / C;
    const int x = (int)(q % W);
    q /= W;
    const int yy = (int)(q % H);
    const int b = (int)(q / H);
    float g = 0.25f * __bfloat162float(dy[(((long long)b * h2 + yy / 2) * w2 + x / 2) * C + c]);
    if (add) g += __bfloat162float(add[i]);
    dx[i] = __float2bfloat16_rn(g);
  }
}

// dz = dy * (y > 0) (ReLU gradient), all [n] bf16.
__global__ void k_relu_grad(const __nv_bfloat16* __restrict__ dy, const __nv_bfloat16* __restrict__ y,
                            __nv_bfloat16* __restrict__ dz, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dz[i] = __bfloat162float(y[i]) > 0.f ? dy[i] : __float2bfloat16_rn(0.f);
}

// Split the data gradient of a concatenated input [pixels][C1 + C2] into the
// full-resolution part (added to d1, [pixels][C1]; add1 may be null) and the
// half-resolution part summed over its 2 x 2 nearest-neighbour children (d2,
// [pixels/4][C2]).
__global__ void k_split_concat_grad(const __nv_bfloat16* __restrict__ dcat, int nb, int H, int W, int C1, int C2,
                                    __nv_bfloat16* __restrict__ d1, const __nv_bfloat16* __restrict__ add1,
                                    __nv_bfloat16* __restrict__ d2) {
  const int C = C1 + C2;
  const long long n1 = (long long)nb * H * W * C1;
  const int h2 = H / 2, w2 = W / 2;
  const long long n2 = (long long)nb * h2 * w2 * C2;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n1 + n2;
       i += (long long)gridDim.x * blockDim.x) {
    if (i < n1) {
      const long long p = i / C1;
      const int c = (int)(i % C1);
      float g = __bfloat162float(dcat[p * C + c]);
      if (add1) g += __bfloat162float(add1[i]);
      d1[i] = __float2bfloat16_rn(g);
    } else {
      const long long j = i - n1;
      const int c = (int)(j % C2);
      long long q = j / C2;
      const int xo = (int)(q % w2);
      q /= w2;
      const int yo = (int)(q % h2);
      const int b = (int)(q / h2);
      float g = 0.f;
#pragma unroll
      for (int dy = 0; dy < 2; ++dy)
#pragma unroll
        for (int dx = 0; dx < 2; ++dx) {
          const long long p = ((long long)b * H + 2 * yo + dy) * W + 2 * xo + dx;
          g += __bfloat162float(dcat[p * C + C1 + c]);
        }
      d2[j] = __float2bfloat16_rn(g);
    }
  }
}

// Flipped, transposed weights for the data gradient: wt[ci][8 - tap][co] = w[co][tap][ci].
__global__ void k_flip_weights(const __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wt, int cout, int cin) {
  const long long n = (long long)cout * 9 * cin;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int ci = (int)(i % cin);
    const int tap = (int)((i / cin) % 9);
    const int co = (int)(i / (9LL * cin));
    wt[((long long)ci * 9 + (8 - tap)) * cout + co] = w[i];
  }
}

// Bias gradient: db[c] += sum over pixels of dz[p][c].  Each block sums a
// range of pixels with coalesced loads (consecutive threads read consecutive
// elements of the NHWC rows; C divides 256 or is a multiple of it), reduces
// per channel in shared memory and adds one value per channel (red.add).
__global__ void k_bias_grad(const __nv_bfloat16* __restrict__ dz, float* __restrict__ db, long long npix, int C,
                            long long pix_per_block) {
  __shared__ float acc[256];
  const long long p0 = (long long)blockIdx.x * pix_per_block;
  const long long p1 = min(npix, p0 + pix_per_block);
  const long long e0 = p0 * C, e1 = p1 * C;
  if (C <= 256 && 256 % C == 0) {
    // thread t always meets channel t % C
    float s = 0.f;
    for (long long e = e0 + threadIdx.x; e < e1; e += 256) s += __bfloat162float(dz[e]);
    acc[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < C) {
      float t = 0.f;
      for (int j = threadIdx.x; j < 256; j += C) t += acc[j];
      atomicAdd(db + threadIdx.x, t);
    }
  } else {
    for (int c = threadIdx.x; c < C; c += blockDim.x) {
      float t = 0.f;
      for (long long p = p0; p < p1; ++p) t += __bfloat162float(dz[p * C + c]);
      atomicAdd(db + c, t);
    }
  }
}

// Loss of the network output in residual form: the estimate is
// e = out[p][0] + s img[p] (out [pixels][cout] f32, img and target [pixels]
// f32); *loss += sum (e - target)^2 and dout[p][0] = scale (e - target), the
// other channels 0 (bf16).
__global__ void k_mse_grad(const float* __restrict__ out, int cout, const float* __restrict__ img, float s,
                           const float* __restrict__ target, __nv_bfloat16* __restrict__ dout, long long npix,
                           float scale, float* loss) {
  float acc = 0.f;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x) {
    const float d = __fmaf_rn(s, img[p], out[p * cout]) - target[p];
    acc += d * d;
    dout[p * cout] = __float2bfloat16_rn(d * scale);
    for (int c = 1; c < cout; ++c) dout[p * cout + c] = __float2bfloat16_rn(0.f);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

// The estimate of the residual form: e[p] = out[p][0] + s img[p].
__global__ void k_residual_out(const float* __restrict__ out, int cout, const float* __restrict__ img, float s,
                               float* __restrict__ e, long long npix) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x)
    e[p] = __fmaf_rn(s, img[p], out[p * cout]);
}

// Adam step on f32 master parameters, with the bf16 copy the kernels read.
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v, const float* __restrict__ g,
                       __nv_bfloat16* __restrict__ wb, long long n, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16_rn(wi);
  }
}

// f32 image [pixels] -> bf16 NHWC with C channels, the image in channel 0 (scaled).
__global__ void k_image_to_nhwc(const float* __restrict__ img, __nv_bfloat16* __restrict__ x, long long npix, int C,
                                float scale) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x)
    for (int c = 0; c < C; ++c) x[p * C + c] = __float2bfloat16_rn(c == 0 ? img[p] * scale : 0.f);
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
namespace {

int g_umma_attr_dev = -1;

int umma_fail(int code, const char* msg) { return kw_internal_fail(code, msg); }

// Dynamic shared memory of a launch: the two A stages, two B stages of the
// launch's tile width, barriers and alignment slack -- at least enough that no
// more CTAs share an SM than its 512 TMEM columns hold (256-column tiles: 2
// CTAs, 128-column tiles: 4), so that tcgen05.alloc never has to wait.
int umma_smem(int NT, bool halo = false) {
  const int need = halo ? 2 * (int)kAHalo + 2 * NT * 288 + 64 + 1024 : 2 * kATile + 2 * NT * kBK * 2 + 64 + 1024;
  const int ncols = NT <= 32 ? 32 : NT <= 64 ? 64 : NT <= 128 ? 128 : 256;
  const int floor_bytes = ncols == 256 ? 80 * 1024 : ncols == 128 ? 48 * 1024 : 0;
  return need > floor_bytes ? need : floor_bytes;
}

int umma_launch(UmmaArgs& a, dim3 grid, cudaStream_t st) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return umma_fail(KW_ERR_CUDA, "cudaGetDevice failed");
  const int smem = umma_smem(a.NT, a.mode == 3);
  if (g_umma_attr_dev != dev) {
    const int most = std::max(umma_smem(kMaxNT), umma_smem(kMaxNT, true));
    if (cudaFuncSetAttribute(k_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, most) != cudaSuccess)
      return umma_fail(KW_ERR_CUDA, "k_umma: cannot set the shared-memory size");
    g_umma_attr_dev = dev;
  }
  k_umma<<<grid, kThreads, smem, st>>>(a, kw_device_error_ptr());
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    char buf[256];
    snprintf(buf, sizeof buf, "k_umma launch: %s", cudaGetErrorString(e));
    return umma_fail(KW_ERR_CUDA, buf);
  }
  return KW_OK;
}

int tile_cols(int n) {
  const int r = (n + 15) / 16 * 16;
  return r > kMaxNT ? kMaxNT : r;
}

// --- persistent TMA-fed convolution (k_conv_tma) ---------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn conv_encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

int conv_tma_smem(int C1, int NT, int stages, int rows, int gc) {
  return 1024 + (int)((conv_tma_wbytes(C1, NT) + 1023) & ~1023u) + 1024 + stages * (int)conv_tma_stage(rows, gc) + 256;
}

int g_conv_tma_attr_dev = -1;
constexpr int kConvTmaMaxSmem = 220 * 1024;

// Run the convolution on k_conv_tma if it applies: one full-resolution input
// of 16-channel groups, rows of a multiple of 128 pixels, at most 256 output
// channels, weights and the halo ring within the shared-memory budget.
// Returns KW_OK when launched, 1 when the caller should use k_umma.
int conv_tma_try(const UmmaArgs& u, cudaStream_t st) {
  static const bool enabled = [] {
    const char* env = getenv("KWAVE_GB300_CONV_TMA");
    return !(env && env[0] == '0');
  }();
  if (!enabled || u.C2 != 0 || u.W % 128 || u.C1 % 16 || u.NT > kMaxNT || u.N > u.NT) return 1;
  // ring depth: the most CTAs per SM (shared memory, 512 TMEM columns, at
  // most 4), then the deepest ring that keeps that count
  // tiles of two image rows where the four accumulators fit TMEM: each input
  // row is staged for two output rows instead of three
  // channels per stage: the widest swizzle row (64 channels = 128 bytes) that divides C1
  const int gc = u.C1 % 64 == 0 ? 64 : u.C1 % 32 == 0 ? 32 : 16;
  int rows = (u.H % 2 == 0 && 4 * u.NT <= 512) ? 2 : 1;
  int stages = 0, per_sm = 0;
  for (; rows >= 1 && stages == 0; --rows) {
    const int by_tmem = 512 / (int)conv_tma_tmem_cols(u.NT, rows);
    for (int sdepth = 2; sdepth <= kCtMaxStages; ++sdepth) {
      const int sm = conv_tma_smem(u.C1, u.NT, sdepth, rows, gc);
      if (sm > kConvTmaMaxSmem) break;
      const int k = std::min(std::min((227 * 1024) / (sm + 1024), by_tmem), 4);
      if (k >= per_sm) {
        per_sm = k;
        stages = sdepth;
      }
    }
    if (stages) break;
  }
  if (stages == 0 || per_sm == 0 || rows < 1) return 1;
  const int smem = conv_tma_smem(u.C1, u.NT, stages, rows, gc);
  EncodeTiledFn fn = conv_encode_fn();
  if (!fn) return 1;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return umma_fail(KW_ERR_CUDA, "k_conv_tma: device query failed");
  CUtensorMap map;
  const cuuint64_t C = (cuuint64_t)u.C1, W = (cuuint64_t)u.W, H = (cuuint64_t)u.H;
  cuuint64_t dims[4] = {C, W, H, (cuuint64_t)u.nb};
  cuuint64_t strides[3] = {C * 2, W * C * 2, H * W * C * 2};
  cuuint32_t box[4] = {(cuuint32_t)gc, (cuuint32_t)kHaloCols, (cuuint32_t)(rows + 2), 1};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUtensorMapSwizzle swz = gc == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : gc == 32 ? CU_TENSOR_MAP_SWIZZLE_64B
                                                                                 : CU_TENSOR_MAP_SWIZZLE_32B;
  if (fn(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16*>(u.X1), dims, strides, box, estr,
         CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
      CUDA_SUCCESS)
    return 1;
  if (g_conv_tma_attr_dev != dev) {
    if (cudaFuncSetAttribute(k_conv_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, kConvTmaMaxSmem) != cudaSuccess)
      return umma_fail(KW_ERR_CUDA, "k_conv_tma: cannot set the shared-memory size");
    g_conv_tma_attr_dev = dev;
  }
  ConvTmaArgs a;
  a.nb = u.nb;
  a.H = u.H;
  a.W = u.W;
  a.C1 = u.C1;
  a.N = u.N;
  a.NT = u.NT;
  a.rows = rows;
  a.gc = gc;
  a.ntiles = u.nb * (u.H / rows) * (u.W / 128);
  a.stages = stages;
  a.Wt = u.Wt;
  a.bias = u.bias;
  a.relu = u.relu;
  a.Y = u.Y;
  a.Yf = u.Yf;
  const int grid = std::min(a.ntiles, nsm * per_sm);
  k_conv_tma<<<grid, kCtThreads, smem, st>>>(map, a, kw_device_error_ptr());
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    char buf[256];
    snprintf(buf, sizeof buf, "k_conv_tma launch: %s", cudaGetErrorString(e));
    return umma_fail(KW_ERR_CUDA, buf);
  }
  return KW_OK;
}

inline int grid1(long long n) {
  long long g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : g > 4096 ? 4096 : g);
}

}  // namespace

extern "C" {

int32_t kw_umma_gemm(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K, void* stream) {
  if (!A || !B || !C) return umma_fail(KW_ERR_INVALID, "kw_umma_gemm: null argument");
  if (M <= 0 || N <= 0 || K <= 0 || K % 8) return umma_fail(KW_ERR_INVALID, "kw_umma_gemm: M, N, K > 0 and K % 8 == 0");
  UmmaArgs a;
  memset(&a, 0, sizeof a);
  a.mode = 0;
  a.M = M;
  a.N = N;
  a.K = K;
  a.NT = tile_cols(N);
  a.A = static_cast<const __nv_bfloat16*>(A);
  a.B = static_cast<const __nv_bfloat16*>(B);
  a.C = C;
  return umma_launch(a, dim3((N + a.NT - 1) / a.NT, (M + kBM - 1) / kBM), static_cast<cudaStream_t>(stream));
}

int32_t kw_umma_gemm_mn(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K, void* stream) {
  if (!A || !B || !C) return umma_fail(KW_ERR_INVALID, "kw_umma_gemm_mn: null argument");
  if (M <= 0 || N <= 0 || K <= 0 || M % 8 || N % 8)
    return umma_fail(KW_ERR_INVALID, "kw_umma_gemm_mn: M, N, K > 0, M % 8 == 0 and N % 8 == 0");
  UmmaArgs a;
  memset(&a, 0, sizeof a);
  a.mode = 4;
  a.M = M;
  a.N = N;
  a.K = K;
  a.NT = tile_cols(N);
  a.A = static_cast<const __nv_bfloat16*>(A);
  a.B = static_cast<const __nv_bfloat16*>(B);
  a.C = C;
  return umma_launch(a, dim3((N + a.NT - 1) / a.NT, (M + kBM - 1) / kBM), static_cast<cudaStream_t>(stream));
}

int32_t kw_conv3x3(const void* x1, int32_t c1, const void* x2, int32_t c2, int32_t nb, int32_t H, int32_t W,
                   const void* w, const float* bias, int32_t cout, int32_t relu, void* y, float* yf, void* stream) {
  if (!x1 || !w || (!y && !yf)) return umma_fail(KW_ERR_INVALID, "kw_conv3x3: null argument");
  if (c1 <= 0 || c1 % 8 || c2 < 0 || c2 % 8 || (c2 && !x2) || cout <= 0 || cout % 8)
    return umma_fail(KW_ERR_INVALID, "kw_conv3x3: channel counts must be multiples of 8");
  if (nb <= 0 || H <= 0 || W <= 0 || (c2 && (H % 2 || W % 2)))
    return umma_fail(KW_ERR_INVALID, "kw_conv3x3: bad geometry");
  UmmaArgs a;
  memset(&a, 0, sizeof a);
  // 3x3 convolutions on rows of a multiple of 128 pixels with 16-channel
  // inputs run on halo tiles (KWAVE_GB300_CONV_HALO=0: the gather tiles)
  static const bool halo_ok = [] {
    const char* env = getenv("KWAVE_GB300_CONV_HALO");
    return !(env && env[0] == '0');
  }();
  a.mode = (halo_ok && W % 128 == 0 && c1 % 16 == 0 && c2 % 16 == 0) ? 3 : 1;
  a.nb = nb;
  a.H = H;
  a.W = W;
  a.C1 = c1;
  a.C2 = c2;
  a.M = nb * H * W;
  a.N = cout;
  a.K = 9 * (c1 + c2);
  a.NT = tile_cols(cout);
  a.X1 = static_cast<const __nv_bfloat16*>(x1);
  a.X2 = static_cast<const __nv_bfloat16*>(x2);
  a.Wt = static_cast<const __nv_bfloat16*>(w);
  a.bias = bias;
  a.relu = relu;
  a.Y = static_cast<__nv_bfloat16*>(y);
  a.Yf = yf;
  // halo tiles of one input: the persistent TMA-fed kernel when it applies
  // (KWAVE_GB300_CONV_TMA=0: always k_umma)
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (a.mode == 3) {
    const int rc = conv_tma_try(a, st);
    if (rc != 1) return rc;
  }
  const int ntile = (cout + a.NT - 1) / a.NT, mtile = (a.M + kBM - 1) / kBM;
  // gather tiles that leave SMs idle (small images, many channels): the K
  // range is split over CTAs whose partial tiles are added in f32 scratch,
  // then bias, ReLU and the stores run as one elementwise pass
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return umma_fail(KW_ERR_CUDA, "kw_conv3x3: device query failed");
  const int nchunk = (a.K + kBK - 1) / kBK;
  int split = 1;
  if (a.mode == 1 && ntile * mtile < nsm) split = std::min((2 * nsm + ntile * mtile - 1) / (ntile * mtile), nchunk / 2);
  if (split <= 1) return umma_launch(a, dim3(ntile, mtile), st);
  const int per = (nchunk + split - 1) / split;
  split = (nchunk + per - 1) / per;
  float* acc = nullptr;
  const size_t bytes = (size_t)a.M * cout * sizeof(float);
  if (cudaMallocAsync(reinterpret_cast<void**>(&acc), bytes, st) != cudaSuccess)
    return umma_fail(KW_ERR_OOM, "kw_conv3x3: split-K scratch");
  int rc = KW_OK;
  if (cudaMemsetAsync(acc, 0, bytes, st) != cudaSuccess) rc = umma_fail(KW_ERR_CUDA, "kw_conv3x3: scratch clear");
  if (!rc) {
    a.ksplit = per * kBK;
    a.C = acc;
    rc = umma_launch(a, dim3(ntile, mtile, split), st);
  }
  if (!rc) {
    const long long total = (long long)a.M * cout;
    k_conv_finish<<<grid1(total), 256, 0, st>>>(acc, bias, relu, a.Y, a.Yf, total, cout);
    if (cudaGetLastError() != cudaSuccess) rc = umma_fail(KW_ERR_CUDA, "kw_conv3x3: finish launch");
  }
  cudaFreeAsync(acc, st);
  return rc;
}

int32_t kw_conv3x3_wgrad(const void* x1, int32_t c1, const void* x2, int32_t c2, int32_t nb, int32_t H, int32_t W,
                         const void* dz, int32_t cout, float* dw, void* stream) {
  if (!x1 || !dz || !dw) return umma_fail(KW_ERR_INVALID, "kw_conv3x3_wgrad: null argument");
  if (c1 <= 0 || c1 % 8 || c2 < 0 || c2 % 8 || (c2 && !x2) || cout <= 0 || cout % 8)
    return umma_fail(KW_ERR_INVALID, "kw_conv3x3_wgrad: channels must be multiples of 8");
  // MN-major tiles (rows (tap, input channel), columns output channels) unless
  // KWAVE_GB300_WGRAD_MN=0 selects the transposing K-major tiles
  static const bool mn_ok = [] {
    const char* env = getenv("KWAVE_GB300_WGRAD_MN");
    return !(env && env[0] == '0');
  }();
  UmmaArgs a;
  memset(&a, 0, sizeof a);
  a.mode = mn_ok ? 5 : 2;
  a.nb = nb;
  a.H = H;
  a.W = W;
  a.C1 = c1;
  a.C2 = c2;
  a.M = mn_ok ? 9 * (c1 + c2) : cout;
  a.N = mn_ok ? cout : 9 * (c1 + c2);
  a.K = nb * H * W;
  a.NT = tile_cols(a.N);
  a.X1 = static_cast<const __nv_bfloat16*>(x1);
  a.X2 = static_cast<const __nv_bfloat16*>(x2);
  a.dZ = static_cast<const __nv_bfloat16*>(dz);
  a.dW = dw;
  const int ntile = (a.N + a.NT - 1) / a.NT, mtile = (a.M + kBM - 1) / kBM;
  // split the pixels so that the grid covers the GPU a few times over
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  long long want = 4LL * nsm / (ntile * mtile);
  if (want < 1) want = 1;
  long long per = ((long long)a.K + want - 1) / want;
  per = (per + kBK - 1) / kBK * kBK;
  if (per < 4 * kBK) per = 4 * kBK;
  a.ksplit = (int)per;
  const int nsplit = (int)((a.K + per - 1) / per);
  return umma_launch(a, dim3(ntile, mtile, nsplit), static_cast<cudaStream_t>(stream));
}

#define KW_UNET_CK()                                                                 \
  do {                                                                              \
    const cudaError_t e_ = cudaGetLastError();                                      \
    if (e_ != cudaSuccess) return umma_fail(KW_ERR_CUDA, cudaGetErrorString(e_));   \
  } while (0)

int32_t kw_unet_avgpool2(const void* x, void* y, int32_t nb, int32_t H, int32_t W, int32_t C, void* stream) {
  if (!x || !y || H % 2 || W % 2) return umma_fail(KW_ERR_INVALID, "kw_unet_avgpool2: bad argument");
  k_avgpool2<<<grid1((long long)nb * H * W * C / 4), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(x), static_cast<__nv_bfloat16*>(y), nb, H, W, C);
  KW_UNET_CK();
  return KW_OK;
}

int32_t kw_unet_avgpool2_bwd(const void* dy, void* dx, int32_t nb, int32_t H, int32_t W, int32_t C, const void* add,
                             void* stream) {
  if (!dy || !dx || H % 2 || W % 2) return umma_fail(KW_ERR_INVALID, "kw_unet_avgpool2_bwd: bad argument");
  k_avgpool2_bwd<<<grid1((long long)nb * H * W * C), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(dy), static_cast<__nv_bfloat16*>(dx), nb, H, W, C,
      static_cast<const __nv_bfloat16*>(add));
  KW_UNET_CK();
  return KW_OK;
}

int32_t kw_unet_relu_grad(const void* dy, const void* y, void* dz, int64_t n, void* stream) {
  if (!dy || !y || !dz) return umma_fail(KW_ERR_INVALID, "kw_unet_relu_grad: null argument");
  k_relu_grad<<<grid1(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(dy), static_cast<const __nv_bfloat16*>(y), static_cast<__nv_bfloat16*>(dz), n);
  KW_UNET_CK();
  return KW_OK;
}

int32_t kw_unet_split_concat_grad(const void* dcat, int32_t nb, int32_t H, int32_t W, int32_t C1, int32_t C2, void* d1,
                                  const void* add1, void* d2, void* stream) {
  if (!dcat || !d1 || !d2 || H % 2 || W % 2) return umma_fail(KW_ERR_INVALID, "kw_unet_split_concat_grad: bad argument");
  k_split_concat_grad<<<grid1((long long)nb * H * W * C1 + (long long)nb * H * W * C2 / 4), 256, 0,
                        static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(dcat), nb, H, W, C1, C2, static_cast<__nv_bfloat16*>(d1),
      static_cast<const __nv_bfloat16*>(add1), static_cast<__nv_bfloat16*>(d2));
  KW_UNET_CK();
  return KW_OK;
}

int32_t kw_unet_flip_weights(const void* w, void* wt, int32_t cout, int32_t cin, void* stream) {
  if (!w || !wt) return umma_fail(KW_ERR_INVALID, "kw_unet_flip_weights: null argument");
  k_flip_weights<<<grid1((long long)cout * 9 * cin), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(w), static_cast<__nv_bfloat16*>(wt), cout, cin);
  KW_UNET_CK();
  return KW_OK;
}

int32_t kw_unet_bias_grad(const void* dz, float* db, int64_t npix, int32_t C, void* stream) {
  if (!dz || !db) return umma_fail(KW_ERR_INVALID, "kw_unet_bias_grad: null argument");
  const long long per = 1024;  // pixels per block
  k_bias_grad<<<(int)((npix + per - 1) / per), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(dz), db, npix, C, per);
  KW_UNET_CK();
  return KW_OK;
}

int32_t kw_unet_mse_grad(const float* out, int32_t cout, const float* img, float s, const float* target, void* dout,
                         int64_t npix, float scale, float* loss, void* stream) {
  if (!out || !img || !target || !dout || !loss) return umma_fail(KW_ERR_INVALID, "kw_unet_mse_grad: null argument");
  k_mse_grad<<<grid1(npix), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      out, cout, img, s, target, static_cast<__nv_bfloat16*>(dout), npix, scale, loss);
  KW_UNET_CK();
  return KW_OK;
}

int32_t kw_unet_residual_out(const float* out, int32_t cout, const float* img, float s, float* e, int64_t npix,
                             void* stream) {
  if (!out || !img || !e) return umma_fail(KW_ERR_INVALID, "kw_unet_residual_out: null argument");
  k_residual_out<<<grid1(npix), 256, 0, static_cast<cudaStream_t>(stream)>>>(out, cout, img, s, e, npix);
  KW_UNET_CK();
  return KW_OK;
}

int32_t kw_unet_adam(float* w, float* m, float* v, const float* g, void* wb, int64_t n, float lr, float b1, float b2,
                     float eps, int32_t step, void* stream) {
  if (!w || !m || !v || !g || step < 1) return umma_fail(KW_ERR_INVALID, "kw_unet_adam: bad argument");
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<grid1(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(w, m, v, g, static_cast<__nv_bfloat16*>(wb), n, lr, b1,
                                                                   b2, eps, c1, c2);
  KW_UNET_CK();
  return KW_OK;
}

int32_t kw_unet_image_to_nhwc(const float* img, void* x, int64_t npix, int32_t C, float scale, void* stream) {
  if (!img || !x || C < 1) return umma_fail(KW_ERR_INVALID, "kw_unet_image_to_nhwc: bad argument");
  k_image_to_nhwc<<<grid1(npix), 256, 0, static_cast<cudaStream_t>(stream)>>>(img, static_cast<__nv_bfloat16*>(x),
                                                                              npix, C, scale);
  KW_UNET_CK();
  return KW_OK;
}

}  // extern "C"
