// Velocity stage fed by bulk copies (power-of-two row lengths).
//
// The register row kernel (kw_rows_reg.cuh) loads its inputs with ordinary
// global loads; with its register budget a warp keeps only a few of them in
// flight, so it waits on memory latency.  Here a persistent CTA streams, for
// each block of R rows and each component a, the three arrays the velocity
// update reads -- the rows of the gradient spectrum S_a, of u_a and of
// dt/rho_sg_a -- into a ring of shared-memory slots with 1-D bulk copies
// (cp.async.bulk, mbarrier completion), issued by one producer lane up to
// NST copies ahead.  The 128 consumer threads (P per row) run the same
// arithmetic as ST_U of the register kernel, reading the staged rows:
//   u_a = pml_sg (pml_sg u_a - dt/rho_sg_a g_a)     (kspace_solver.py:703-707)
// and write u_a and its spectrum to global memory.
//
// Used for the ordinary velocity update (not the t = 0 half step, not with
// k-space corrected velocity sources or velocity-on-pressure-grid records:
// those keep the register kernel).  All waits are bounded (2 s) and report
// through the device error word, as in the TMA axis pass.
#include "kw_rows_reg.cuh"
#include "kw_tma.cuh"

namespace {

constexpr uint64_t kRowWaitNs = 2000000000ull;

__device__ __forceinline__ bool consumers_any_rows(bool pred, int n) {
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

}  // namespace

template <int E, int P, int NST>
__global__ void __launch_bounds__(160, 2) k_rows_u_tma(const __grid_constant__ RowsParams Q, int* err) {
  using namespace kwrows;
  constexpr int M = E * P, R = 128 / P, CT = 128;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int D = Q.ndim;
  const int Hp = Q.Hp;
  const uint32_t spec_row = (uint32_t)Hp * 8u, fld_row = (uint32_t)M * 8u;  // bytes per row
  const uint32_t slot_bytes = ((R * (spec_row > fld_row ? spec_row : fld_row)) + 127u) & ~127u;
  unsigned char* slots = smem_raw;
  float2* tw = reinterpret_cast<float2*>(slots + (size_t)NST * slot_bytes);
  float2* twp = tw + M;
  float2* ex = twp + (M + 1);
  uint64_t* full = reinterpret_cast<uint64_t*>((reinterpret_cast<uintptr_t>(ex + R * Q.ex_stride) + 7) & ~uintptr_t(7));
  uint64_t* empty = full + NST;
  int* counters = reinterpret_cast<int*>(empty + NST);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      kwtma::mbar_init(&full[s], 1);
      kwtma::mbar_init(&empty[s], CT / 32);
    }
    counters[0] = counters[1] = 0;
    kwtma::fence_barrier_init();
  }
  for (int i = tid; i < M; i += blockDim.x) tw[i] = Q.tw[i];
  for (int i = tid; i <= M; i += blockDim.x) twp[i] = Q.twpost[i];
  __syncthreads();

  const int nblk = (Q.nrows + R - 1) / R;
  const bool has_dtr = Q.dtrsg[0] != nullptr;
  const int per_a = has_dtr ? 3 : 2;

  if (warp == CT / 32) {
    // ---------------- producer ----------------
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int rb = blockIdx.x; rb < nblk && ok; rb += gridDim.x) {
        const int r0 = rb * R, nr = min(R, Q.nrows - r0);
        for (int a = 0; a < D && ok; ++a) {
          for (int q = 0; q < per_a; ++q, ++it) {
            const uint32_t s = it % NST, k = it / NST;
            if (k > 0 && !kwtma::mbar_wait(&empty[s], (k - 1) & 1, kRowWaitNs)) {
              atomicExch(err, 3);
              ok = false;
              break;
            }
            const void* src;
            uint32_t bytes;
            if (q == 0) {
              src = Q.S[a] + (size_t)r0 * Hp;
              bytes = (uint32_t)nr * spec_row;
            } else {
              src = reinterpret_cast<const float2*>(q == 1 ? Q.u[a] : Q.dtrsg[a]) + (size_t)r0 * M;
              bytes = (uint32_t)nr * fld_row;
            }
            kwtma::mbar_arrive_expect_tx(&full[s], bytes);
            kwtma::bulk_load(slots + (size_t)s * slot_bytes, src, bytes, &full[s]);
          }
        }
      }
      counters[0] = (int)it;
    }
  } else {
    // ---------------- consumers ----------------
    const int row = tid / P, t = tid % P;
    uint32_t it = 0;
    bool aborted = false;
    float2 v[E];
    for (int rb = blockIdx.x; rb < nblk && !aborted; rb += gridDim.x) {
      const int grow = rb * R + row;
      RowCtx<E, P> c{Q, tw, twp, ex + row * Q.ex_stride, row, t, grow, grow < Q.nrows, (uint32_t)grow * (uint32_t)M};
      c.gx = D == 3 ? grow / Q.N1 : grow;
      c.gy = D == 3 ? grow - c.gx * Q.N1 : 0;
      for (int a = 0; a < D && !aborted; ++a) {
        // gradient spectrum rows -> register pairs
        uint32_t s = it % NST;
        bool got = kwtma::mbar_wait(&full[s], (it / NST) & 1, kRowWaitNs);
        if (consumers_any_rows(!got, CT)) {
          if (tid == 0) atomicExch(err, 4);
          aborted = true;
          break;
        }
        const float2* srow = reinterpret_cast<const float2*>(slots + (size_t)s * slot_bytes) + row * Hp;
        // read the staged row into registers, then free the slot
        {
#pragma unroll
          for (int m = 0; m < E / P; ++m)
#pragma unroll
            for (int k2 = 0; k2 < P; ++k2) {
              const int k = t + P * m + E * k2;
              float2 z = make_float2(0.f, 0.f);
              if (c.ok) {
                const float2 xk = srow[k];
                const float2 xc = cconj(srow[M - k]);
                const float2 e = cadd(xk, xc);
                const float2 o = kwreg::cmulf(csub(xk, xc), cconj(twp[k]));
                z = make_float2(e.x - o.y, e.y + o.x);
              }
              v[m * P + k2] = cconj(z);
            }
        }
        __syncwarp();
        if (lane == 0) kwtma::mbar_arrive(&empty[s]);
        ++it;
        kwreg::Reg<E, P>::rev(v, t, c.exr, 1, tw, [] __device__() { __syncwarp(); });
#pragma unroll
        for (int j = 0; j < E; ++j) v[j].y = -v[j].y;
        // u_a and dt/rho_sg_a rows
        const uint32_t su = it % NST;
        got = kwtma::mbar_wait(&full[su], (it / NST) & 1, kRowWaitNs);
        uint32_t sd = su;
        if (has_dtr) {
          sd = (it + 1) % NST;
          got = got && kwtma::mbar_wait(&full[sd], ((it + 1) / NST) & 1, kRowWaitNs);
        }
        if (consumers_any_rows(!got, CT)) {
          if (tid == 0) atomicExch(err, 4);
          aborted = true;
          break;
        }
        const float2* urow = reinterpret_cast<const float2*>(slots + (size_t)su * slot_bytes) + row * M;
        const float2* drow = reinterpret_cast<const float2*>(slots + (size_t)sd * slot_bytes) + row * M;
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const int n = t + P * j;
          if (!c.ok) continue;
          const float2 g = v[j];
          const float2 dtr = has_dtr ? drow[n] : make_float2(Q.dtrsg_s[a], Q.dtrsg_s[a]);
          const float2 sg = c.pml2(Q.pmlsg[a], a, n);
          const float2 u = urow[n];
          v[j] = make_float2(__fmul_rn(sg.x, __fsub_rn(__fmul_rn(sg.x, u.x), __fmul_rn(dtr.x, g.x))),
                             __fmul_rn(sg.y, __fsub_rn(__fmul_rn(sg.y, u.y), __fmul_rn(dtr.y, g.y))));
        }
        __syncwarp();
        if (lane == 0) {
          kwtma::mbar_arrive(&empty[su]);
          if (has_dtr) kwtma::mbar_arrive(&empty[sd]);
        }
        it += has_dtr ? 2 : 1;
        c.source(Q.src[3 + a], v);
        if (c.ok) {
#pragma unroll
          for (int j = 0; j < E; ++j) st2(Q.u[a], c.rbase + t + P * j, v[j]);
        }
        c.record(v, Q.rec[1 + a]);
        c.r2c(v, Q.S[a]);
      }
    }
    if (tid == 0) counters[1] = (int)it;
  }
  __syncthreads();
  // copies issued but never consumed (only after a timeout): wait for them, bounded
  if (tid == 0) {
    for (int i = counters[1]; i < counters[0]; ++i) {
      const uint32_t s = (uint32_t)i % NST, k = (uint32_t)i / NST;
      if (!kwtma::mbar_wait(&full[s], k & 1, kRowWaitNs)) break;
    }
  }
}

static constexpr int kRowNst = 4;

static size_t rows_u_tma_smem(int M, int E, int P, int Hp, int ex_stride) {
  const int R = 128 / P;
  const size_t spec_row = (size_t)Hp * 8, fld_row = (size_t)M * 8;
  const size_t slot = ((R * (spec_row > fld_row ? spec_row : fld_row)) + 127) & ~(size_t)127;
  return kRowNst * slot + sizeof(float2) * (2 * (size_t)M + 1 + (size_t)R * ex_stride) + 8 + 2 * kRowNst * 8 + 16;
}

#define KW_RU_SWITCH(m, CALL)              \
  switch (m) {                             \
    case 64: return CALL(16, 4);           \
    case 128: return CALL(16, 8);          \
    case 256: return CALL(16, 16);         \
    case 512: return CALL(32, 16);         \
    case 1024: return CALL(32, 32);        \
    default: return cudaErrorInvalidValue; \
  }

cudaError_t kw_rows_u_tma_attr(int m, int Hp, int ex_stride) {
  int E, P;
  if (!kw_reg_shape(m, &E, &P)) return cudaErrorInvalidValue;
  const int smem = (int)rows_u_tma_smem(m, E, P, Hp, ex_stride);
#define KW_R(E_, P_) cudaFuncSetAttribute(k_rows_u_tma<E_, P_, kRowNst>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)
  KW_RU_SWITCH(m, KW_R)
#undef KW_R
}

cudaError_t kw_rows_u_tma_launch(int m, int nsm, cudaStream_t st, const RowsParams& Q, int* err) {
  int E, P;
  if (!kw_reg_shape(m, &E, &P)) return cudaErrorInvalidValue;
  const int R = 128 / P, nblk = (Q.nrows + R - 1) / R;
  const int grid = nblk < 2 * nsm ? nblk : 2 * nsm;
  const size_t smem = rows_u_tma_smem(m, E, P, Q.Hp, Q.ex_stride);
#define KW_R(E_, P_) (k_rows_u_tma<E_, P_, kRowNst><<<grid, 160, smem, st>>>(Q, err), cudaGetLastError())
  KW_RU_SWITCH(m, KW_R)
#undef KW_R
}
