// Row stages of the time step for power-of-two last-axis lengths, with all
// real-space physics held in registers in the layout of the row FFT.
//
// P consecutive threads own one row of L = 2M reals; thread t owns the float2
// pairs n = t + P j (j < E), i.e. reals 2n and 2n+1.  The inverse row
// transform (half spectrum -> reals) leaves exactly these pairs in registers
// and the forward transform starts from them, so the physics between them
// (velocity update, split-density update, equation of state, sources,
// sensors) needs no shared-memory staging: fields are read and written as
// float2 straight from global memory.  Shared memory holds only twiddles and
// the per-row FFT exchange regions.
//
// The arithmetic and its order follow kwave/solvers/kspace_solver.py
// (Simulation.step, :691-747) as the generic row kernel does.
#pragma once
#include "kw_kernels.cuh"
#include "kw_regfft.cuh"

namespace kwrows {

// pair indices are 32-bit: the host uses these kernels only for grids below 2^32 cells
__device__ __forceinline__ float2 ld2(const float* p, uint32_t i) { return reinterpret_cast<const float2*>(p)[i]; }
__device__ __forceinline__ void st2(float* p, uint32_t i, float2 v) { reinterpret_cast<float2*>(p)[i] = v; }
__device__ __forceinline__ float2 fld2(const float* p, float s, uint32_t i) {
  return p ? ld2(p, i) : make_float2(s, s);
}

template <int E, int P>
struct RowCtx {
  static constexpr int M = E * P;
  const RowsParams& Q;
  const float2* tw;
  const float2* twp;
  float2* exr;      // this row's exchange region
  int row, t, grow;
  bool ok;          // row < nrows
  uint32_t rbase;   // float2 index of the row's first pair
  int gx, gy;       // the row's x and (3-D) y index

  // half-spectrum row -> register pairs (unnormalised: L * x)
  __device__ __forceinline__ void c2r(const float2* S, float2 (&v)[E]) const {
    c2r_row(S + (uint32_t)(ok ? grow : 0) * (uint32_t)Q.Hp, v);
  }

  // the same from the row's H values at sr (global or shared memory)
  __device__ __forceinline__ void c2r_row(const float2* sr, float2 (&v)[E]) const {
#pragma unroll
    for (int m = 0; m < E / P; ++m)
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) {
        const int k = t + P * m + E * k2;
        float2 z = make_float2(0.f, 0.f);
        if (ok) {
          const float2 xk = sr[k];
          const float2 xc = cconj(sr[M - k]);
          const float2 e = cadd(xk, xc);
          const float2 o = kwreg::cmulf(csub(xk, xc), cconj(twp[k]));
          z = make_float2(e.x - o.y, e.y + o.x);
        }
        v[m * P + k2] = cconj(z);
      }
    kwreg::Reg<E, P>::rev(v, t, exr, 1, tw, [] __device__() { __syncwarp(); });
#pragma unroll
    for (int j = 0; j < E; ++j) v[j].y = -v[j].y;
  }

  // register pairs -> half-spectrum row
  __device__ __forceinline__ void r2c(float2 (&v)[E], float2* S) const {
    kwreg::Reg<E, P>::fwd(v, t, exr, 1, tw, [] __device__() { __syncwarp(); });
#pragma unroll
    for (int m = 0; m < E / P; ++m)
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) exr[t + P * m + E * k2] = v[m * P + k2];
    __syncwarp();
    if (ok) {
      float2* so = S + (uint32_t)grow * (uint32_t)Q.Hp;
      for (int k = t; k <= M; k += P) {
        const float2 zk = exr[k == M ? 0 : k];
        const float2 zc = cconj(exr[k == 0 ? 0 : M - k]);
        const float2 e = cscale(cadd(zk, zc), 0.5f);
        const float2 d = csub(zk, zc);
        const float2 o = make_float2(0.5f * d.y, -0.5f * d.x);
        so[k] = cadd(e, kwreg::cmulf(twp[k], o));
      }
    }
    __syncwarp();
  }

  // PML factors of the two reals of pair n along `axis`
  __device__ __forceinline__ float2 pml2(const float* tab, int axis, int n) const {
    if (axis == Q.ndim - 1) return ld2(tab, n);
    const int idx = (axis == 0) ? gx : gy;
    const float s = tab[idx];
    return make_float2(s, s);
  }

  // sparse source on this row (kspace_solver.py:86-109): owner thread updates its pair
  __device__ __forceinline__ void source(const KwSrcDev& S, float2 (&v)[E]) const {
    const int ts = kw_step_t(Q);
    if (!S.active || ts >= S.len || !ok) return;
    const int e0 = S.row_ptr[grow], e1 = S.row_ptr[grow + 1];
    for (int e = e0; e < e1; ++e) {
      const int4 en = S.ent[e];
      const int n = en.y >> 1;
      if ((n % P) != t) continue;
      const int jj = n / P;
      const float val = S.sig[(long long)ts * S.nsig + (S.nsig == 1 ? 0 : en.z)];
#pragma unroll
      for (int j = 0; j < E; ++j)
        if (j == jj) {
          float& f = (en.y & 1) ? v[j].y : v[j].x;
          f = (S.mode == SRC_DIRICHLET) ? val : __fadd_rn(f, val);
        }
    }
  }

  // values of a source at step t on this row, zero elsewhere (the field whose
  // k-space corrected version is added)
  __device__ __forceinline__ void scatter(const KwSrcDev& S, float2 (&v)[E]) const {
#pragma unroll
    for (int j = 0; j < E; ++j) v[j] = make_float2(0.f, 0.f);
    if (!ok) return;
    const int ts = kw_step_t(Q);
    const int e0 = S.row_ptr[grow], e1 = S.row_ptr[grow + 1];
    for (int e = e0; e < e1; ++e) {
      const int4 en = S.ent[e];
      const int n = en.y >> 1;
      if ((n % P) != t) continue;
      const int jj = n / P;
      const float val = S.sig[(long long)ts * S.nsig + (S.nsig == 1 ? 0 : en.z)];
#pragma unroll
      for (int j = 0; j < E; ++j)
        if (j == jj) {
          if (en.y & 1)
            v[j].y = val;
          else
            v[j].x = val;
        }
    }
  }

  __device__ __forceinline__ void record(const float2 (&v)[E], float* rec) const {
    const int rr = kw_rec_row(Q);
    if (rec == nullptr || rr < 0 || Q.sens_row_ptr == nullptr || !ok) return;
    const int e0 = Q.sens_row_ptr[grow], e1 = Q.sens_row_ptr[grow + 1];
    float* out = rec + (long long)rr * Q.nslots;
    for (int e = e0; e < e1; ++e) {
      const int4 en = Q.sens_ent[e];
      const int n = en.y >> 1;
      if ((n % P) != t) continue;
      const int jj = n / P;
      float val = 0.f;
#pragma unroll
      for (int j = 0; j < E; ++j)
        if (j == jj) val = (en.y & 1) ? v[j].y : v[j].x;
      out[en.z] = val;
    }
  }

  // v += S^T r at this row's sensor points (binary sensor: one slot per grid
  // point; r is time-major in rec[0], row kw_rec_row(Q))
  __device__ __forceinline__ void add_residual(float2 (&v)[E]) const {
    const int rr = kw_rec_row(Q);
    const float* res = Q.rec[0];
    if (res == nullptr || rr < 0 || Q.sens_row_ptr == nullptr || !ok) return;
    const int e0 = Q.sens_row_ptr[grow], e1 = Q.sens_row_ptr[grow + 1];
    const float* in = res + (long long)rr * Q.nslots;
    for (int e = e0; e < e1; ++e) {
      const int4 en = Q.sens_ent[e];
      const int n = en.y >> 1;
      if ((n % P) != t) continue;
      const int jj = n / P;
      const float val = in[en.z];
#pragma unroll
      for (int j = 0; j < E; ++j)
        if (j == jj) {
          float& f = (en.y & 1) ? v[j].y : v[j].x;
          f = __fadd_rn(f, val);
        }
    }
  }
};

// velocity on the pressure grid, Re F^-1[e^{-i k d/2} F[u_i]] (kspace_solver.py:740-743)
template <int E, int P>
__device__ __forceinline__ void record_unstaggered(const RowCtx<E, P>& c, const RowsParams& Q, float2 (&v)[E]) {
  if (!Q.rec_us) return;
  for (int a = 0; a < Q.ndim; ++a) {
    if (!(Q.rec_us & (1 << a))) continue;
    c.c2r(Q.S[B_US0 + a], v);
    c.record(v, Q.rec[4 + a]);
  }
}

// Bulk prefetch into L2 of one contiguous byte range (16-byte aligned start
// and size; no completion to wait for).
__device__ __forceinline__ void l2_prefetch(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Lane `lane` of warp 0 prefetches into L2 one of the arrays that component
// `comp` of the density stage (or the equation of state) reads for this block's rows [r0, r0 + R): the rows of
// a block are contiguous in every row-major array, so one bulk prefetch per
// array covers them.  Component 0 also brings the arrays shared by all
// components; each later component is prefetched while the previous one is
// computed, so that only about one component's data per block is in flight.
template <int STAGE>
__device__ __forceinline__ void prefetch_block(const RowsParams& Q, int r0, int lane, int comp) {
  const int nr = min(Q.R, Q.nrows - r0);
  if (nr <= 0 || comp >= Q.ndim) return;
  const uint32_t sb = (uint32_t)nr * Q.Hp * 8u, fb = (uint32_t)nr * Q.L * 4u;
  const long long so = (long long)r0 * Q.Hp, fo = (long long)r0 * Q.L;
  const void* p = nullptr;
  uint32_t bytes = 0;
  auto spec = [&](int b) { p = Q.S[b] + so; bytes = sb; };
  auto fld = [&](const float* f) { if (f) { p = f + fo; bytes = fb; } };
  if constexpr (STAGE == ST_RHO_PL || STAGE == ST_RHO) {
    if (lane == 0) spec(comp);
    else if (lane == 1) fld(Q.rho[comp]);
    else if (comp == 0 && lane == 2) fld(Q.rho0);
    else if (comp == 0 && lane == 3 && STAGE == ST_RHO_PL && Q.nonlin) fld(Q.rho_sum);
    else if (comp == 0 && lane == 3 && STAGE == ST_RHO) fld(Q.c0);
  } else if constexpr (STAGE == ST_EOS) {
    if (comp != 0) return;
    if (lane == 0) spec(0);
    else if (lane == 1 && Q.disp) spec(1);
    else if (lane == 2) fld(Q.rho_sum);
    else if (lane == 3) fld(Q.c0);
    else if (lane == 4) fld(Q.tau);
    else if (lane == 5 && Q.disp) fld(Q.eta);
    else if (lane == 6 && Q.nonlin) fld(Q.rho0);
    else if (lane == 7 && Q.nonlin) fld(Q.bona);
  }
  if (p && bytes) l2_prefetch(p, bytes);
}

}  // namespace kwrows

// EXTRA: this launch has k-space corrected sources or records the velocity on
// the pressure grid; without it those paths are compiled out, which keeps the
// common launch at its smaller register budget.
// Resident blocks per SM each stage is compiled for (register budget
// 65536 / (128 * blocks)): velocity 72, power-law density 128, equation of
// state 96, generic density 168, the rest 128.
constexpr int kw_rows_min_blocks(int stage) {
  return stage == ST_U ? 7 : stage == ST_RHO_PL ? 4 : stage == ST_EOS ? 5 : stage == ST_RHO ? 3 : 4;
}

template <int E, int P, int STAGE, bool EXTRA>
__global__ void __launch_bounds__(128, kw_rows_min_blocks(STAGE)) k_rows_v2(const __grid_constant__ RowsParams Q) {
  constexpr int M = E * P;
  extern __shared__ float4 smem_f4[];
  float2* tw = reinterpret_cast<float2*>(smem_f4);
  float2* twp = tw + M;
  float2* ex = twp + (M + 1);
  if (threadIdx.x < 32) kwrows::prefetch_block<STAGE>(Q, blockIdx.x * (blockDim.x / P), threadIdx.x, 0);
  for (int i = threadIdx.x; i < M; i += blockDim.x) tw[i] = Q.tw[i];
  for (int i = threadIdx.x; i <= M; i += blockDim.x) twp[i] = Q.twpost[i];
  __syncthreads();

  const int row = threadIdx.x / P, t = threadIdx.x % P;
  const int R = blockDim.x / P;
  const int grow = blockIdx.x * R + row;
  using namespace kwrows;
  RowCtx<E, P> c{Q, tw, twp, ex + row * Q.ex_stride, row, t, grow, grow < Q.nrows, (uint32_t)grow * (uint32_t)M};
  c.gx = Q.ndim == 3 ? grow / Q.N1 : grow;
  c.gy = Q.ndim == 3 ? grow - c.gx * Q.N1 : 0;
  const int D = Q.ndim;
  float2 v[E];

  if constexpr (STAGE == ST_INIT) {
    // t = 0 with p0: p = p0, rho_i = p0 / (c0^2 D) (kspace_solver.py:729-733)
#pragma unroll
    for (int j = 0; j < E; ++j) {
      const uint32_t i = c.rbase + t + P * j;
      float2 pv = make_float2(0.f, 0.f);
      if (c.ok) {
        pv = ld2(Q.p0, i);
        if (Q.p0_scale) {
          const float sc = *Q.p0_scale;
          pv = make_float2(__fmul_rn(pv.x, sc), __fmul_rn(pv.y, sc));
        }
        const float2 cc = fld2(Q.c0, Q.c0_s, i);
        const float2 r = make_float2(__fdiv_rn(pv.x, __fmul_rn(__fmul_rn(cc.x, cc.x), (float)D)),
                                     __fdiv_rn(pv.y, __fmul_rn(__fmul_rn(cc.y, cc.y), (float)D)));
        for (int a = 0; a < D; ++a) st2(Q.rho[a], i, r);
        if (Q.rho_sum) {
          // the density sum in the order the density stage adds the components
          float2 sr = r;
          for (int a = 1; a < D; ++a) sr = make_float2(__fadd_rn(sr.x, r.x), __fadd_rn(sr.y, r.y));
          st2(Q.rho_sum, i, sr);
        }
        if (Q.write_p) st2(Q.p, i, pv);
      }
      v[j] = pv;
    }
    c.record(v, Q.rec[0]);
    c.r2c(v, Q.S[3]);
    return;
  }

  if constexpr (STAGE == ST_U) {
    // u_i = pml_sg (pml_sg u_i - dt/rho_sg g_i) (kspace_solver.py:703-707)
    for (int a = 0; a < D; ++a) {
      if (threadIdx.x < 32) prefetch_block<STAGE>(Q, blockIdx.x * (blockDim.x / P), threadIdx.x, a + 1);
      c.c2r(Q.S[a], v);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        const int n = t + P * j;
        const uint32_t i = c.rbase + n;
        if (!c.ok) continue;
        const float2 g = v[j];
        const float2 dtr = fld2(Q.dtrsg[a], Q.dtrsg_s[a], i);
        if (Q.init) {
          v[j] = make_float2(__fmul_rn(__fmul_rn(dtr.x, 0.5f), g.x), __fmul_rn(__fmul_rn(dtr.y, 0.5f), g.y));
        } else {
          const float2 sg = c.pml2(Q.pmlsg[a], a, n);
          const float2 u = ld2(Q.u[a], i);
          v[j] = make_float2(__fmul_rn(sg.x, __fsub_rn(__fmul_rn(sg.x, u.x), __fmul_rn(dtr.x, g.x))),
                             __fmul_rn(sg.y, __fsub_rn(__fmul_rn(sg.y, u.y), __fmul_rn(dtr.y, g.y))));
        }
      }
      if (!Q.init) {
        if (EXTRA && Q.srcu_on[a]) {
          // u_i += Re F^-1[source_kappa F[s_i]] (kspace_solver.py:91-98)
          float2 w[E];
          c.c2r(Q.S[B_SRCU0 + a], w);
#pragma unroll
          for (int j = 0; j < E; ++j) v[j] = make_float2(__fadd_rn(v[j].x, w[j].x), __fadd_rn(v[j].y, w[j].y));
        } else {
          c.source(Q.src[3 + a], v);
        }
      }
      if (c.ok) {
#pragma unroll
        for (int j = 0; j < E; ++j) st2(Q.u[a], c.rbase + t + P * j, v[j]);
      }
      c.record(v, Q.rec[1 + a]);
      if (!Q.init || Q.init_r2c) c.r2c(v, Q.S[a]);
    }
    return;
  }

  if constexpr (STAGE == ST_RHO) {
    // mass conservation with split density (kspace_solver.py:709-717)
    float2 nl[E], div[E], rs[E];
#pragma unroll
    for (int j = 0; j < E; ++j) {
      nl[j] = make_float2(1.f, 1.f);
      div[j] = make_float2(0.f, 0.f);
      rs[j] = make_float2(0.f, 0.f);
      if (Q.nonlin && c.ok) {
        const uint32_t i = c.rbase + t + P * j;
        const float2 r0v = fld2(Q.rho0, Q.rho0_s, i);
        float2 sr = ld2(Q.rho[0], i);
        for (int a = 1; a < D; ++a) {
          const float2 ra = ld2(Q.rho[a], i);
          sr = make_float2(__fadd_rn(sr.x, ra.x), __fadd_rn(sr.y, ra.y));
        }
        nl[j] = make_float2(__fdiv_rn(__fadd_rn(__fmul_rn(2.f, sr.x), r0v.x), r0v.x),
                            __fdiv_rn(__fadd_rn(__fmul_rn(2.f, sr.y), r0v.y), r0v.y));
      }
    }
    float2 cp[EXTRA ? E : 1];
    if constexpr (EXTRA) {
      if (Q.srcp_on) c.c2r(Q.S[B_SRCP], cp);
    }
    for (int a = 0; a < D; ++a) {
      if (threadIdx.x < 32) prefetch_block<STAGE>(Q, blockIdx.x * (blockDim.x / P), threadIdx.x, a + 1);
      c.c2r(Q.S[a], v);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        const int n = t + P * j;
        const uint32_t i = c.rbase + n;
        const float2 du = v[j];
        div[j] = make_float2(__fadd_rn(div[j].x, du.x), __fadd_rn(div[j].y, du.y));
        if (!c.ok) continue;
        const float2 r0v = fld2(Q.rho0, Q.rho0_s, i);
        const float2 pm = c.pml2(Q.pml[a], a, n);
        const float2 ro = ld2(Q.rho[a], i);
        const float tx = __fmul_rn(__fmul_rn(__fmul_rn(Q.dt, r0v.x), du.x), nl[j].x);
        const float ty = __fmul_rn(__fmul_rn(__fmul_rn(Q.dt, r0v.y), du.y), nl[j].y);
        v[j] = make_float2(__fmul_rn(pm.x, __fsub_rn(__fmul_rn(pm.x, ro.x), tx)),
                           __fmul_rn(pm.y, __fsub_rn(__fmul_rn(pm.y, ro.y), ty)));
      }
      bool corrected = false;
      if constexpr (EXTRA) {
        if (Q.srcp_on) {
          // rho_i += Re F^-1[source_kappa F[s]] / d_i (kspace_solver.py:91-98, scale :619-624)
          const float id = Q.inv_d[a];
#pragma unroll
          for (int j = 0; j < E; ++j)
            v[j] = make_float2(__fadd_rn(v[j].x, __fmul_rn(cp[j].x, id)), __fadd_rn(v[j].y, __fmul_rn(cp[j].y, id)));
          corrected = true;
        }
      }
      if (!corrected) c.source(Q.src[a], v);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        if (c.ok) st2(Q.rho[a], c.rbase + t + P * j, v[j]);
        rs[j] = (a == 0) ? v[j] : make_float2(__fadd_rn(rs[j].x, v[j].x), __fadd_rn(rs[j].y, v[j].y));
      }
    }
    if (Q.absorb == 1) {
      // power law: transform rho0 * div and the density sum (kspace_solver.py:498, :524)
#pragma unroll
      for (int j = 0; j < E; ++j) {
        const uint32_t i = c.rbase + t + P * j;
        if (c.ok) {
          st2(Q.rho_sum, i, rs[j]);
          const float2 r0v = fld2(Q.rho0, Q.rho0_s, i);
          v[j] = make_float2(__fmul_rn(r0v.x, div[j].x), __fmul_rn(r0v.y, div[j].y));
        } else {
          v[j] = make_float2(0.f, 0.f);
        }
      }
      c.r2c(v, Q.S[0]);
      if (Q.disp) c.r2c(rs, Q.S[1]);
      if constexpr (EXTRA) record_unstaggered(c, Q, v);
      return;
    }
    // equation of state without fractional Laplacians (kspace_solver.py:719-723)
#pragma unroll
    for (int j = 0; j < E; ++j) {
      const uint32_t i = c.rbase + t + P * j;
      float2 pv = make_float2(0.f, 0.f);
      if (c.ok) {
        const float2 cc = fld2(Q.c0, Q.c0_s, i);
        const float2 r0v = fld2(Q.rho0, Q.rho0_s, i);
        float ax = rs[j].x, ay = rs[j].y;
        if (Q.absorb == 2) {
          const float2 tau = fld2(Q.tau, Q.tau_s, i);
          ax = __fadd_rn(ax, __fmul_rn(__fmul_rn(tau.x, r0v.x), div[j].x));
          ay = __fadd_rn(ay, __fmul_rn(__fmul_rn(tau.y, r0v.y), div[j].y));
        }
        if (Q.nonlin) {
          const float2 b = fld2(Q.bona, Q.bona_s, i);
          ax = __fadd_rn(ax, __fdiv_rn(__fmul_rn(b.x, __fmul_rn(rs[j].x, rs[j].x)), __fmul_rn(2.f, r0v.x)));
          ay = __fadd_rn(ay, __fdiv_rn(__fmul_rn(b.y, __fmul_rn(rs[j].y, rs[j].y)), __fmul_rn(2.f, r0v.y)));
        }
        pv = make_float2(__fmul_rn(__fmul_rn(cc.x, cc.x), ax), __fmul_rn(__fmul_rn(cc.y, cc.y), ay));
        if (Q.write_p) st2(Q.p, i, pv);
      }
      v[j] = pv;
    }
    c.record(v, Q.rec[0]);
    c.r2c(v, Q.S[3]);
    if constexpr (EXTRA) record_unstaggered(c, Q, v);
    return;
  }

  if constexpr (STAGE == ST_RHO_PL) {
    // mass conservation with split density and power-law absorption
    // (kspace_solver.py:709-717, :498, :524).  The nonlinear factor
    // (2 sum_a rho_a + rho0) / rho0 uses the sum stored by the previous step,
    // which is the same float sum of the same values; it is folded with
    // dt rho0 into one factor per pair (the reference multiplies the three in
    // the order dt rho0 du nl, so results can differ in the last bit).  Only the divergence
    // stays in registers across the components; the new density sum is
    // formed afterwards from the just-written rho_a (cache hits), and the
    // divergence accumulates in this thread's slots of shared memory
    // (dsm[j * blockDim + thread], after the exchange regions), which keeps
    // this stage at one register array.
    float2* dsm = ex + Q.R * Q.ex_stride;
    const int nthr = blockDim.x;
    // w = dt rho0 (2 sum_a rho_a + rho0) / rho0 per pair, loaded and formed
    // once for the three components (all loads issued together)
    float2 w[E];
#pragma unroll
    for (int j = 0; j < E; ++j) {
      const uint32_t i = c.rbase + t + P * j;
      w[j] = make_float2(0.f, 0.f);
      if (c.ok) {
        const float2 r0v = fld2(Q.rho0, Q.rho0_s, i);
        w[j] = make_float2(__fmul_rn(Q.dt, r0v.x), __fmul_rn(Q.dt, r0v.y));
        if (Q.nonlin) {
          const float2 sr = ld2(Q.rho_sum, i);
          w[j] = make_float2(__fmul_rn(w[j].x, __fdiv_rn(__fadd_rn(__fmul_rn(2.f, sr.x), r0v.x), r0v.x)),
                             __fmul_rn(w[j].y, __fdiv_rn(__fadd_rn(__fmul_rn(2.f, sr.y), r0v.y), r0v.y)));
        }
      }
    }
    float2 cp[EXTRA ? E : 1];
    if constexpr (EXTRA) {
      if (Q.srcp_on) c.c2r(Q.S[B_SRCP], cp);
    }
    for (int a = 0; a < D; ++a) {
      if (threadIdx.x < 32) prefetch_block<STAGE>(Q, blockIdx.x * (blockDim.x / P), threadIdx.x, a + 1);
      c.c2r(Q.S[a], v);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        const int n = t + P * j;
        const uint32_t i = c.rbase + n;
        const float2 du = v[j];
        float2* dp = dsm + j * nthr + threadIdx.x;
        const float2 d0 = (a == 0) ? make_float2(0.f, 0.f) : *dp;
        *dp = make_float2(__fadd_rn(d0.x, du.x), __fadd_rn(d0.y, du.y));
        if (!c.ok) continue;
        const float2 pm = c.pml2(Q.pml[a], a, n);
        const float2 ro = ld2(Q.rho[a], i);
        const float tx = __fmul_rn(w[j].x, du.x);
        const float ty = __fmul_rn(w[j].y, du.y);
        v[j] = make_float2(__fmul_rn(pm.x, __fsub_rn(__fmul_rn(pm.x, ro.x), tx)),
                           __fmul_rn(pm.y, __fsub_rn(__fmul_rn(pm.y, ro.y), ty)));
      }
      bool corrected = false;
      if constexpr (EXTRA) {
        if (Q.srcp_on) {
          const float id = Q.inv_d[a];
#pragma unroll
          for (int j = 0; j < E; ++j)
            v[j] = make_float2(__fadd_rn(v[j].x, __fmul_rn(cp[j].x, id)), __fadd_rn(v[j].y, __fmul_rn(cp[j].y, id)));
          corrected = true;
        }
      }
      if (!corrected) c.source(Q.src[a], v);
      if (c.ok) {
#pragma unroll
        for (int j = 0; j < E; ++j) st2(Q.rho[a], c.rbase + t + P * j, v[j]);
      }
    }
    // rho0 * div -> spectrum 0
#pragma unroll
    for (int j = 0; j < E; ++j) {
      const uint32_t i = c.rbase + t + P * j;
      const float2 dv = dsm[j * nthr + threadIdx.x];
      if (c.ok) {
        const float2 r0v = fld2(Q.rho0, Q.rho0_s, i);
        v[j] = make_float2(__fmul_rn(r0v.x, dv.x), __fmul_rn(r0v.y, dv.y));
      } else {
        v[j] = make_float2(0.f, 0.f);
      }
    }
    c.r2c(v, Q.S[0]);
    if constexpr (EXTRA) record_unstaggered(c, Q, v);
    // the new density sum (components added in order), kept for the equation
    // of state and the next step's nonlinear factor, and its spectrum
#pragma unroll
    for (int j = 0; j < E; ++j) {
      const uint32_t i = c.rbase + t + P * j;
      float2 rs = make_float2(0.f, 0.f);
      if (c.ok) {
        rs = ld2(Q.rho[0], i);
        for (int a = 1; a < D; ++a) {
          const float2 ra = ld2(Q.rho[a], i);
          rs = make_float2(__fadd_rn(rs.x, ra.x), __fadd_rn(rs.y, ra.y));
        }
        st2(Q.rho_sum, i, rs);
      }
      v[j] = rs;
    }
    if (Q.disp) c.r2c(v, Q.S[1]);
    return;
  }

  if constexpr (STAGE == ST_SRC) {
    // scattered source fields of this step, transformed for the source-kappa pass
    if (Q.srcp_on) {
      c.scatter(Q.src[0], v);
      c.r2c(v, Q.S[B_SRCP]);
    }
    for (int a = 0; a < D; ++a)
      if (Q.srcu_on[a]) {
        c.scatter(Q.src[3 + a], v);
        c.r2c(v, Q.S[B_SRCU0 + a]);
      }
    return;
  }

  if constexpr (STAGE == ST_P0FFT) {
    // spectrum of p0 for the smoothing window
#pragma unroll
    for (int j = 0; j < E; ++j) v[j] = c.ok ? ld2(Q.p0w, c.rbase + t + P * j) : make_float2(0.f, 0.f);
    c.r2c(v, Q.S[B_P]);
    return;
  }

  if constexpr (STAGE == ST_P0BACK) {
    c.c2r(Q.S[B_P], v);
    if (c.ok) {
#pragma unroll
      for (int j = 0; j < E; ++j) st2(Q.p0w, c.rbase + t + P * j, v[j]);
    }
    return;
  }

  if constexpr (STAGE == ST_UREC) {
    record_unstaggered(c, Q, v);
    return;
  }

  if constexpr (STAGE >= ST_ADJ_A) {
    // transposed step of the lossless, source-free loop: the arithmetic of
    // the generic row kernels' adjoint stages (kw_generic.cuh: adjoint_body),
    // on register-resident rows
    if constexpr (STAGE == ST_ADJ_A || STAGE == ST_ADJ_D) {
      float2 lp[E];
#pragma unroll
      for (int j = 0; j < E; ++j) lp[j] = c.ok ? ld2(Q.p, c.rbase + t + P * j) : make_float2(0.f, 0.f);
      c.add_residual(lp);
      for (int a = 0; a < D; ++a) {
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const int n = t + P * j;
          const uint32_t i = c.rbase + n;
          v[j] = make_float2(0.f, 0.f);
          if (!c.ok) continue;
          if constexpr (STAGE == ST_ADJ_A) {
            if (a == 0 && Q.gacc) {
              const float2 fs = ld2(Q.fsum, i), ga = ld2(Q.gacc, i);
              st2(Q.gacc, i, make_float2(__fmaf_rn(fs.x, lp[j].x, ga.x), __fmaf_rn(fs.y, lp[j].y, ga.y)));
            }
            const float2 cc = fld2(Q.c0, Q.c0_s, i);
            const float2 r0v = fld2(Q.rho0, Q.rho0_s, i);
            const float2 pm = c.pml2(Q.pml[a], a, n);
            const float2 rho = ld2(Q.rho[a], i);
            const float c2x = __fmul_rn(cc.x, cc.x), c2y = __fmul_rn(cc.y, cc.y);
            const float bx = __fmul_rn(Q.dt, r0v.x), by = __fmul_rn(Q.dt, r0v.y);
            const float lrx = __fadd_rn(rho.x, __fmul_rn(c2x, lp[j].x));
            const float lry = __fadd_rn(rho.y, __fmul_rn(c2y, lp[j].y));
            st2(Q.rho[a], i, make_float2(__fmul_rn(__fmul_rn(pm.x, pm.x), lrx), __fmul_rn(__fmul_rn(pm.y, pm.y), lry)));
            v[j] = make_float2(__fmul_rn(__fmul_rn(bx, pm.x), lrx), __fmul_rn(__fmul_rn(by, pm.y), lry));
          } else {
            if (a == 0) st2(Q.p, i, lp[j]);
            const float2 dtr = fld2(Q.dtrsg[a], Q.dtrsg_s[a], i);
            const float2 u = ld2(Q.u[a], i);
            v[j] = make_float2(__fmul_rn(__fmul_rn(dtr.x, 0.5f), u.x), __fmul_rn(__fmul_rn(dtr.y, 0.5f), u.y));
          }
        }
        c.r2c(v, Q.S[a]);
      }
    } else if constexpr (STAGE == ST_ADJ_B) {
      for (int a = 0; a < D; ++a) {
        c.c2r(Q.S[a], v);
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const int n = t + P * j;
          const uint32_t i = c.rbase + n;
          if (!c.ok) continue;
          const float2 sg = c.pml2(Q.pmlsg[a], a, n);
          const float2 u = ld2(Q.u[a], i);
          const float2 dtr = fld2(Q.dtrsg[a], Q.dtrsg_s[a], i);
          const float lux = __fadd_rn(u.x, v[j].x), luy = __fadd_rn(u.y, v[j].y);
          st2(Q.u[a], i, make_float2(__fmul_rn(__fmul_rn(sg.x, sg.x), lux), __fmul_rn(__fmul_rn(sg.y, sg.y), luy)));
          v[j] = make_float2(__fmul_rn(__fmul_rn(dtr.x, sg.x), lux), __fmul_rn(__fmul_rn(dtr.y, sg.y), luy));
        }
        c.r2c(v, Q.S[a]);
      }
    } else {
      // ST_ADJ_C / ST_ADJ_E: sum_i F^-1 S_i
      float2 sum[E];
      for (int a = 0; a < D; ++a) {
        c.c2r(Q.S[a], v);
#pragma unroll
        for (int j = 0; j < E; ++j)
          sum[j] = a == 0 ? v[j] : make_float2(__fadd_rn(sum[j].x, v[j].x), __fadd_rn(sum[j].y, v[j].y));
      }
      if (c.ok) {
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const uint32_t i = c.rbase + t + P * j;
          if constexpr (STAGE == ST_ADJ_C) {
            st2(Q.p, i, sum[j]);
          } else {
            const float2 cc = fld2(Q.c0, Q.c0_s, i);
            const float denx = __fmul_rn(__fmul_rn(cc.x, cc.x), (float)D);
            const float deny = __fmul_rn(__fmul_rn(cc.y, cc.y), (float)D);
            const float2 pv = ld2(Q.p, i);
            float accx = pv.x, accy = pv.y;
            float2 lr = make_float2(0.f, 0.f);
            for (int a = 0; a < D; ++a) {
              const float2 rho = ld2(Q.rho[a], i);
              accx = __fadd_rn(accx, __fdiv_rn(rho.x, denx));
              accy = __fadd_rn(accy, __fdiv_rn(rho.y, deny));
              lr = a == 0 ? rho : make_float2(__fadd_rn(lr.x, rho.x), __fadd_rn(lr.y, rho.y));
            }
            st2(Q.p, i, make_float2(__fsub_rn(accx, sum[j].x), __fsub_rn(accy, sum[j].y)));
            if (Q.gacc) {
              const float2 p0 = ld2(Q.p0, i), ga = ld2(Q.gacc, i);
              const float ovx = __fdiv_rn(__fmul_rn(p0.x, lr.x), __fmul_rn(denx, __fmul_rn(cc.x, cc.x)));
              const float ovy = __fdiv_rn(__fmul_rn(p0.y, lr.y), __fmul_rn(deny, __fmul_rn(cc.y, cc.y)));
              st2(Q.gacc, i, make_float2(__fmul_rn(__fmul_rn(2.f, cc.x), __fsub_rn(ga.x, ovx)),
                                         __fmul_rn(__fmul_rn(2.f, cc.y), __fsub_rn(ga.y, ovy))));
            }
          }
        }
      }
    }
    return;
  }

  if constexpr (STAGE == ST_EOS) {
  // p = c0^2 (rho + tau F^-1[nabla1 F[rho0 div]] - eta F^-1[nabla2 F[rho]] + B/A rho^2 / (2 rho0))
  float2 w[E];
  c.c2r(Q.S[0], v);
  if (Q.disp) c.c2r(Q.S[1], w);
#pragma unroll
  for (int j = 0; j < E; ++j) {
    const uint32_t i = c.rbase + t + P * j;
    float2 pv = make_float2(0.f, 0.f);
    if (c.ok) {
      const float2 rsum = ld2(Q.rho_sum, i);
      const float2 cc = fld2(Q.c0, Q.c0_s, i);
      const float2 tau = fld2(Q.tau, Q.tau_s, i);
      float ax = __fadd_rn(rsum.x, __fmul_rn(tau.x, v[j].x));
      float ay = __fadd_rn(rsum.y, __fmul_rn(tau.y, v[j].y));
      if (Q.disp) {
        const float2 eta = fld2(Q.eta, Q.eta_s, i);
        ax = __fsub_rn(ax, __fmul_rn(eta.x, w[j].x));
        ay = __fsub_rn(ay, __fmul_rn(eta.y, w[j].y));
      }
      if (Q.nonlin) {
        const float2 r0v = fld2(Q.rho0, Q.rho0_s, i);
        const float2 b = fld2(Q.bona, Q.bona_s, i);
        ax = __fadd_rn(ax, __fdiv_rn(__fmul_rn(b.x, __fmul_rn(rsum.x, rsum.x)), __fmul_rn(2.f, r0v.x)));
        ay = __fadd_rn(ay, __fdiv_rn(__fmul_rn(b.y, __fmul_rn(rsum.y, rsum.y)), __fmul_rn(2.f, r0v.y)));
      }
      pv = make_float2(__fmul_rn(__fmul_rn(cc.x, cc.x), ax), __fmul_rn(__fmul_rn(cc.y, cc.y), ay));
      if (Q.write_p) st2(Q.p, i, pv);
    }
    v[j] = pv;
  }
  c.record(v, Q.rec[0]);
  c.r2c(v, Q.S[3]);
  }
}

// Launch and attribute helpers for one stage (instantiated by the translation
// unit that owns the stage: kw_rows_reg.cu or kw_rows_reg2.cu).
// Q.R rows of P threads per block (128 threads, or fewer for small grids).
template <int E, int P, int STAGE>
static cudaError_t rows_v2_launch_stage(dim3 grid, size_t smem, cudaStream_t st, const RowsParams& Q) {
  const bool extra = Q.srcp_on || Q.srcu_on[0] || Q.srcu_on[1] || Q.srcu_on[2] || Q.rec_us;
  const dim3 block(Q.R * P);
  if (extra)
    k_rows_v2<E, P, STAGE, true><<<grid, block, smem, st>>>(Q);
  else
    k_rows_v2<E, P, STAGE, false><<<grid, block, smem, st>>>(Q);
  return cudaGetLastError();
}

template <int E, int P, int STAGE>
static cudaError_t rows_v2_attr_stage() {
  const int lim = 100 * 1024;
  cudaError_t e = cudaFuncSetAttribute(k_rows_v2<E, P, STAGE, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_rows_v2<E, P, STAGE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  return e;
}

#define KW_V2_SWITCH(m, CALL)              \
  switch (m) {                             \
    case 64: return CALL(16, 4);           \
    case 128: return CALL(16, 8);          \
    case 256: return CALL(16, 16);         \
    case 512: return CALL(32, 16);         \
    case 1024: return CALL(32, 32);        \
    default: return cudaErrorInvalidValue; \
  }

// second stage group (kw_rows_reg2.cu)
cudaError_t kw_rows_v2_attr_b(int m);
cudaError_t kw_rows_v2_launch_b(int m, int stage, dim3 grid, size_t smem, cudaStream_t st, const RowsParams& Q);
// third stage group: the adjoint stages (kw_rows_reg3.cu)
cudaError_t kw_rows_v2_attr_c(int m);
cudaError_t kw_rows_v2_launch_c(int m, int stage, dim3 grid, size_t smem, cudaStream_t st, const RowsParams& Q);
