// Row stages fed by bulk copies (power-of-two row lengths).
//
// The register row kernel (kw_rows_reg.cuh) loads its inputs with ordinary
// global loads; with its register budget a warp keeps only a few of them in
// flight, so it waits on memory latency.  Here a persistent CTA streams, for
// each block of R rows, the arrays the stage reads -- spectrum rows and
// field rows, each a contiguous range -- into a ring of shared-memory slots
// with 1-D bulk copies (cp.async.bulk, mbarrier completion), issued by one
// producer lane up to NST copies ahead.  The 128 consumer threads (P per row)
// run the same arithmetic as the register kernel's stage, reading the staged
// rows, and write their outputs to global memory.
//
//   ST_U      per component a: S_a, u_a, dt/rho_sg_a (if a grid)
//             u_a = pml_sg (pml_sg u_a - dt/rho_sg_a g_a)   (kspace_solver.py:703-707)
//   ST_RHO_PL rho0 (if a grid), sum rho (if nonlinear), then per component a:
//             S_a, rho_a; split-density update with power-law absorption
//             (kspace_solver.py:709-717, :498, :524), as the register
//             kernel's ST_RHO_PL
//   ST_EOS    the two fractional-Laplacian spectra, sum rho, tau, eta, rho0,
//             B/A, c0 (those that are grids); equation of state with
//             absorption and dispersion (kspace_solver.py:719-723)
//
// Launches with k-space corrected sources, velocity-on-pressure-grid records
// or the t = 0 half step keep the register kernel.  All waits are bounded
// (2 s) and report through the device error word, as in the TMA axis pass.
#include "kw_rows_reg.cuh"
#include "kw_tma.cuh"

namespace {

constexpr uint64_t kRowWaitNs = 2000000000ull;
// Ring depth and resident CTAs per SM per stage: the density stage keeps its
// density-sum slots in shared memory and needs more registers (2 CTAs, 4
// slots); the velocity and EOS stages run 3 CTAs of 3 slots.
__host__ __device__ constexpr int row_nst(int stage) { return stage == ST_RHO_PL ? 2 : 3; }
__host__ __device__ constexpr int row_ctas(int stage) { return 3; }

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

// The idx-th array a block of rows of stage STAGE reads, in stream order:
// base pointer and whether it is a spectrum (else a real field).  Arrays that
// are absent (scalar medium values) are skipped by the caller.
template <int STAGE>
__device__ __forceinline__ const void* row_load(const RowsParams& Q, int idx, bool& spec) {
  const int D = Q.ndim;
  if constexpr (STAGE == ST_U) {
    const int a = idx / 3, q = idx - 3 * a;
    spec = q == 0;
    return q == 0 ? (const void*)Q.S[a] : q == 1 ? (const void*)Q.u[a] : (const void*)Q.dtrsg[a];
  } else if constexpr (STAGE == ST_EOS) {
    spec = idx < 2;
    switch (idx) {
      case 0: return Q.S[0];
      case 1: return Q.disp ? Q.S[1] : nullptr;
      case 2: return Q.rho_sum;
      case 3: return Q.tau;
      case 4: return Q.disp ? Q.eta : nullptr;
      case 5: return Q.nonlin ? Q.rho0 : nullptr;
      case 6: return Q.nonlin ? Q.bona : nullptr;
      default: return Q.c0;
    }
  } else {
    if (idx == 0) {
      spec = false;
      return Q.rho0;
    }
    if (idx == 1) {
      spec = false;
      return Q.nonlin ? Q.rho_sum : nullptr;
    }
    if (idx == 2 + 2 * D) {
      spec = false;
      return Q.rho0;  // again, for rho0 * div
    }
    const int a = (idx - 2) >> 1, q = (idx - 2) & 1;
    spec = q == 0;
    return q == 0 ? (const void*)Q.S[a] : (const void*)Q.rho[a];
  }
}

template <int STAGE>
__device__ __forceinline__ int row_nloads(const RowsParams& Q) {
  return STAGE == ST_U ? 3 * Q.ndim : STAGE == ST_EOS ? 8 : 3 + 2 * Q.ndim;
}

}  // namespace

template <int E, int P, int NST, int STAGE>
__global__ void __launch_bounds__(160, row_ctas(STAGE)) k_rows_tma(const __grid_constant__ RowsParams Q, int* err) {
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
  // ST_RHO_PL: the new density sum accumulates in this thread's slots
  // (rsm[j * 128 + thread]) instead of registers
  float2* rsm = ex + R * Q.ex_stride;
  constexpr int NRS = STAGE == ST_RHO_PL ? 128 * E : 0;
  // the stage's PML profile along the last axis (2 M reals), read per element
  float* pmlz = reinterpret_cast<float*>(rsm + NRS);
  uint64_t* full = reinterpret_cast<uint64_t*>((reinterpret_cast<uintptr_t>(pmlz + 2 * M) + 7) & ~uintptr_t(7));
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
  if constexpr (STAGE == ST_U || STAGE == ST_RHO_PL) {
    const float* src = STAGE == ST_U ? Q.pmlsg[D - 1] : Q.pml[D - 1];
    for (int i = tid; i < 2 * M; i += blockDim.x) pmlz[i] = src[i];
  }
  __syncthreads();
  // everything above reads only tables; the fields come from the previous launch
  kwtma::grid_dep_wait();
  kwtma::grid_dep_launch();

  const int nblk = (Q.nrows + R - 1) / R;
  const int nload = row_nloads<STAGE>(Q);
  const uint64_t wait_ns = Q.wait_ns ? Q.wait_ns : kRowWaitNs;

  if (warp == CT / 32) {
    // ---------------- producer ----------------
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int rb = blockIdx.x; rb < nblk && ok; rb += gridDim.x) {
        const int r0 = rb * R, nr = min(R, Q.nrows - r0);
        for (int idx = 0; idx < nload; ++idx) {
          bool spec;
          const void* base = row_load<STAGE>(Q, idx, spec);
          if (!base) continue;
          const uint32_t s = it % NST, k = it / NST;
          if (Q.withhold && blockIdx.x == 0) {
            // failure-detection test: no copy is issued, the consumers' wait for it runs out
            ok = false;
            break;
          }
          if (k > 0 && !kwtma::mbar_wait(&empty[s], (k - 1) & 1, wait_ns)) {
            atomicExch(err, 3);
            ok = false;
            break;
          }
          const void* src = spec ? (const void*)(reinterpret_cast<const float2*>(base) + (size_t)r0 * Hp)
                                 : (const void*)(reinterpret_cast<const float2*>(base) + (size_t)r0 * M);
          const uint32_t bytes = (uint32_t)nr * (spec ? spec_row : fld_row);
          kwtma::mbar_arrive_expect_tx(&full[s], bytes);
          kwtma::bulk_load(slots + (size_t)s * slot_bytes, src, bytes, &full[s]);
          ++it;
        }
      }
      counters[0] = (int)it;
    }
  } else {
    // ---------------- consumers ----------------
    const int row = tid / P, t = tid % P;
    uint32_t it = 0;
    bool aborted = false;
    // wait for item `i` (bounded; all consumers agree on a timeout)
    auto wait_item = [&](uint32_t i) -> const float2* {
      const uint32_t s = i % NST;
      const bool got = kwtma::mbar_wait(&full[s], (i / NST) & 1, wait_ns);
      if (consumers_any_rows(!got, CT)) {
        if (tid == 0) atomicExch(err, 4);
        aborted = true;
        return nullptr;
      }
      return reinterpret_cast<const float2*>(slots + (size_t)s * slot_bytes);
    };
    auto release = [&](uint32_t i) {
      __syncwarp();
      if (lane == 0) kwtma::mbar_arrive(&empty[i % NST]);
    };
    float2 v[E];
    for (int rb = blockIdx.x; rb < nblk && !aborted; rb += gridDim.x) {
      const int grow = rb * R + row;
      RowCtx<E, P> c{Q, tw, twp, ex + row * Q.ex_stride, row, t, grow, grow < Q.nrows, (uint32_t)grow * (uint32_t)M};
      c.gx = D == 3 ? grow / Q.N1 : grow;
      c.gy = D == 3 ? grow - c.gx * Q.N1 : 0;

      if constexpr (STAGE == ST_U) {
        const bool has_dtr = Q.dtrsg[0] != nullptr;
        for (int a = 0; a < D; ++a) {
          const float2* ss = wait_item(it);
          if (!ss) break;
          c.c2r_row(ss + row * Hp, v);  // reads the slot before its transform's first exchange
          release(it);
          ++it;
          const float2* su = wait_item(it);
          if (!su) break;
          const float2* sd = su;
          if (has_dtr) {
            sd = wait_item(it + 1);
            if (!sd) break;
          }
          const float2* urow = su + row * M;
          const float2* drow = sd + row * M;
#pragma unroll
          for (int j = 0; j < E; ++j) {
            const int n = t + P * j;
            if (!c.ok) continue;
            const float2 g = v[j];
            const float2 dtr = has_dtr ? drow[n] : make_float2(Q.dtrsg_s[a], Q.dtrsg_s[a]);
            const float2 sg = c.pml2(a == D - 1 ? pmlz : Q.pmlsg[a], a, n);
            const float2 u = urow[n];
            v[j] = make_float2(__fmul_rn(sg.x, __fsub_rn(__fmul_rn(sg.x, u.x), __fmul_rn(dtr.x, g.x))),
                               __fmul_rn(sg.y, __fsub_rn(__fmul_rn(sg.y, u.y), __fmul_rn(dtr.y, g.y))));
          }
          release(it);
          if (has_dtr) release(it + 1);
          it += has_dtr ? 2 : 1;
          c.source(Q.src[3 + a], v);
          if (c.ok) {
#pragma unroll
            for (int j = 0; j < E; ++j) st2(Q.u[a], c.rbase + t + P * j, v[j]);
          }
          c.record(v, Q.rec[1 + a]);
          c.r2c(v, Q.S[a]);
        }
      } else if constexpr (STAGE == ST_EOS) {
        // p = c0^2 (sum rho + tau L1 - eta L2 + B/A (sum rho)^2 / (2 rho0)), the
        // terms added in the register kernel's order; each field row is read
        // once and its slot released before the next is waited for
        float2 w[E], rsum[E];
        const float2* sp = wait_item(it);
        if (!sp) break;
        c.c2r_row(sp + row * Hp, v);
        release(it++);
        if (Q.disp) {
          sp = wait_item(it);
          if (!sp) break;
          c.c2r_row(sp + row * Hp, w);
          release(it++);
        }
        sp = wait_item(it);
        if (!sp) break;
#pragma unroll
        for (int j = 0; j < E; ++j) rsum[j] = sp[row * M + t + P * j];
        release(it++);
        const float2* sf = nullptr;
        if (Q.tau) {
          sf = wait_item(it);
          if (!sf) break;
        }
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const float2 tau = sf ? sf[row * M + t + P * j] : make_float2(Q.tau_s, Q.tau_s);
          v[j] = make_float2(__fadd_rn(rsum[j].x, __fmul_rn(tau.x, v[j].x)), __fadd_rn(rsum[j].y, __fmul_rn(tau.y, v[j].y)));
        }
        if (sf) release(it++);
        if (Q.disp) {
          sf = nullptr;
          if (Q.eta) {
            sf = wait_item(it);
            if (!sf) break;
          }
#pragma unroll
          for (int j = 0; j < E; ++j) {
            const float2 eta = sf ? sf[row * M + t + P * j] : make_float2(Q.eta_s, Q.eta_s);
            v[j] = make_float2(__fsub_rn(v[j].x, __fmul_rn(eta.x, w[j].x)), __fsub_rn(v[j].y, __fmul_rn(eta.y, w[j].y)));
          }
          if (sf) release(it++);
        }
        if (Q.nonlin) {
          const float2* sr0 = nullptr;
          const float2* sb = nullptr;
          const uint32_t i0 = it;
          if (Q.rho0) {
            sr0 = wait_item(it++);
            if (!sr0) break;
          }
          if (Q.bona) {
            sb = wait_item(it++);
            if (!sb) break;
          }
#pragma unroll
          for (int j = 0; j < E; ++j) {
            const int n = row * M + t + P * j;
            const float2 r0v = sr0 ? sr0[n] : make_float2(Q.rho0_s, Q.rho0_s);
            const float2 b = sb ? sb[n] : make_float2(Q.bona_s, Q.bona_s);
            v[j] = make_float2(
                __fadd_rn(v[j].x, __fdiv_rn(__fmul_rn(b.x, __fmul_rn(rsum[j].x, rsum[j].x)), __fmul_rn(2.f, r0v.x))),
                __fadd_rn(v[j].y, __fdiv_rn(__fmul_rn(b.y, __fmul_rn(rsum[j].y, rsum[j].y)), __fmul_rn(2.f, r0v.y))));
          }
          for (uint32_t i = i0; i < it; ++i) release(i);
        }
        sf = nullptr;
        if (Q.c0) {
          sf = wait_item(it);
          if (!sf) break;
        }
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const float2 cc = sf ? sf[row * M + t + P * j] : make_float2(Q.c0_s, Q.c0_s);
          v[j] = c.ok ? make_float2(__fmul_rn(__fmul_rn(cc.x, cc.x), v[j].x), __fmul_rn(__fmul_rn(cc.y, cc.y), v[j].y))
                      : make_float2(0.f, 0.f);
          if (c.ok && Q.write_p) st2(Q.p, c.rbase + t + P * j, v[j]);
        }
        if (sf) release(it++);
        c.record(v, Q.rec[0]);
        c.r2c(v, Q.S[3]);
      } else {
        // w = dt rho0 (2 sum rho + rho0) / rho0 per pair (nonlinear factor from
        // the previous step's density sum), rho0 kept for rho0 * div
        float2 w[E], div[E];
        const float2* s0 = nullptr;
        const float2* s1 = nullptr;
        const uint32_t i0 = it;
        if (Q.rho0) {
          s0 = wait_item(it++);
          if (!s0) break;
        }
        if (Q.nonlin) {
          s1 = wait_item(it++);
          if (!s1) break;
        }
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const int n = t + P * j;
          const float2 r0 = s0 ? s0[row * M + n] : make_float2(Q.rho0_s, Q.rho0_s);
          w[j] = make_float2(__fmul_rn(Q.dt, r0.x), __fmul_rn(Q.dt, r0.y));
          if (Q.nonlin) {
            const float2 sr = s1[row * M + n];
            w[j] = make_float2(__fmul_rn(w[j].x, __fdiv_rn(__fadd_rn(__fmul_rn(2.f, sr.x), r0.x), r0.x)),
                               __fmul_rn(w[j].y, __fdiv_rn(__fadd_rn(__fmul_rn(2.f, sr.y), r0.y), r0.y)));
          }
        }
        for (uint32_t i = i0; i < it; ++i) release(i);
        for (int a = 0; a < D; ++a) {
          const float2* ss = wait_item(it);
          if (!ss) break;
          c.c2r_row(ss + row * Hp, v);
          release(it);
          ++it;
          const float2* sr = wait_item(it);
          if (!sr) break;
          const float2* rrow = sr + row * M;
#pragma unroll
          for (int j = 0; j < E; ++j) {
            const int n = t + P * j;
            const float2 du = v[j];
            const float2 d0 = (a == 0) ? make_float2(0.f, 0.f) : div[j];
            div[j] = make_float2(__fadd_rn(d0.x, du.x), __fadd_rn(d0.y, du.y));
            if (!c.ok) continue;
            const float2 pm = c.pml2(a == D - 1 ? pmlz : Q.pml[a], a, n);
            const float2 ro = rrow[n];
            const float tx = __fmul_rn(w[j].x, du.x);
            const float ty = __fmul_rn(w[j].y, du.y);
            v[j] = make_float2(__fmul_rn(pm.x, __fsub_rn(__fmul_rn(pm.x, ro.x), tx)),
                               __fmul_rn(pm.y, __fsub_rn(__fmul_rn(pm.y, ro.y), ty)));
          }
          release(it);
          ++it;
          c.source(Q.src[a], v);
#pragma unroll
          for (int j = 0; j < E; ++j) {
            if (c.ok) st2(Q.rho[a], c.rbase + t + P * j, v[j]);
            float2* rp = rsm + j * CT + tid;
            const float2 r = (a == 0) ? v[j] : *rp;
            *rp = (a == 0) ? r : make_float2(__fadd_rn(r.x, v[j].x), __fadd_rn(r.y, v[j].y));
          }
        }
        if (aborted) break;
        const float2* s2 = nullptr;
        if (Q.rho0) {
          s2 = wait_item(it);
          if (!s2) break;
        }
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const float2 r0 = s2 ? s2[row * M + t + P * j] : make_float2(Q.rho0_s, Q.rho0_s);
          v[j] = c.ok ? make_float2(__fmul_rn(r0.x, div[j].x), __fmul_rn(r0.y, div[j].y)) : make_float2(0.f, 0.f);
        }
        if (s2) release(it++);
        c.r2c(v, Q.S[0]);
#pragma unroll
        for (int j = 0; j < E; ++j) {
          v[j] = rsm[j * CT + tid];
          if (c.ok) st2(Q.rho_sum, c.rbase + t + P * j, v[j]);
        }
        if (Q.disp) c.r2c(v, Q.S[1]);
      }
    }
    if (tid == 0) counters[1] = (int)it;
  }
  __syncthreads();
  // copies issued but never consumed (only after a timeout): wait for them, bounded
  if (tid == 0) {
    for (int i = counters[1]; i < counters[0]; ++i) {
      const uint32_t s = (uint32_t)i % NST, k = (uint32_t)i / NST;
      if (!kwtma::mbar_wait(&full[s], k & 1, wait_ns)) break;
    }
  }
}

static size_t rows_tma_smem(int stage, int M, int E, int P, int Hp, int ex_stride) {
  const int R = 128 / P;
  const size_t spec_row = (size_t)Hp * 8, fld_row = (size_t)M * 8;
  const size_t slot = ((R * (spec_row > fld_row ? spec_row : fld_row)) + 127) & ~(size_t)127;
  const size_t nrs = stage == ST_RHO_PL ? (size_t)128 * E : 0;
  const int nst = row_nst(stage);
  return nst * slot + sizeof(float2) * (2 * (size_t)M + 1 + (size_t)R * ex_stride + nrs) + sizeof(float) * 2 * M + 8 +
         2 * nst * 8 + 16;
}

#define KW_RT_SWITCH(m, CALL)              \
  switch (m) {                             \
    case 64: return CALL(16, 4);           \
    case 128: return CALL(16, 8);          \
    case 256: return CALL(16, 16);         \
    case 512: return CALL(32, 16);         \
    case 1024: return CALL(32, 32);        \
    default: return cudaErrorInvalidValue; \
  }

template <int STAGE>
static cudaError_t rows_tma_attr(int m, int Hp, int ex_stride) {
  int E, P;
  if (!kw_reg_shape(m, &E, &P)) return cudaErrorInvalidValue;
  const int smem = (int)rows_tma_smem(STAGE, m, E, P, Hp, ex_stride);
#define KW_R(E_, P_) \
  cudaFuncSetAttribute(k_rows_tma<E_, P_, row_nst(STAGE), STAGE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)
  KW_RT_SWITCH(m, KW_R)
#undef KW_R
}

template <int STAGE>
static cudaError_t rows_tma_launch(int m, int nsm, cudaStream_t st, const RowsParams& Q, int* err, int pdl) {
  int E, P;
  if (!kw_reg_shape(m, &E, &P)) return cudaErrorInvalidValue;
  const int R = 128 / P, nblk = (Q.nrows + R - 1) / R;
  const int per_sm = row_ctas(STAGE);
  const int grid = nblk < per_sm * nsm ? nblk : per_sm * nsm;
  const size_t smem = rows_tma_smem(STAGE, m, E, P, Q.Hp, Q.ex_stride);
#define KW_R(E_, P_) \
  kwtma::launch_k(k_rows_tma<E_, P_, row_nst(STAGE), STAGE>, dim3(grid), dim3(160), smem, st, pdl != 0, Q, err)
  KW_RT_SWITCH(m, KW_R)
#undef KW_R
}

cudaError_t kw_rows_tma_attr(int m, int Hp, int ex_stride) {
  cudaError_t e = rows_tma_attr<ST_U>(m, Hp, ex_stride);
  if (e == cudaSuccess) e = rows_tma_attr<ST_RHO_PL>(m, Hp, ex_stride);
  return e == cudaSuccess ? rows_tma_attr<ST_EOS>(m, Hp, ex_stride) : e;
}

cudaError_t kw_rows_tma_launch(int m, int stage, int nsm, cudaStream_t st, const RowsParams& Q, int* err, int pdl) {
  if (stage == ST_U) return rows_tma_launch<ST_U>(m, nsm, st, Q, err, pdl);
  if (stage == ST_RHO_PL) return rows_tma_launch<ST_RHO_PL>(m, nsm, st, Q, err, pdl);
  if (stage == ST_EOS) return rows_tma_launch<ST_EOS>(m, nsm, st, Q, err, pdl);
  return cudaErrorInvalidValue;
}
