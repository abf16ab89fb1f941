// Register row stages, first group: the stages of every time step (initial
// condition, velocity, density) and the public launch/attribute dispatch.
// The kernel template is kw_rows_reg.cuh; the other stages are instantiated
// in kw_rows_reg2.cu.
#include "kw_rows_reg.cuh"

template <int E, int P>
static cudaError_t rows_a_launch(int stage, dim3 grid, size_t smem, cudaStream_t st, const RowsParams& Q) {
  switch (stage) {
    case ST_INIT: return rows_v2_launch_stage<E, P, ST_INIT>(grid, smem, st, Q);
    case ST_U: return rows_v2_launch_stage<E, P, ST_U>(grid, smem, st, Q);
    case ST_RHO:
      if (Q.absorb == 1 && Q.rho_sum) return rows_v2_launch_stage<E, P, ST_RHO_PL>(grid, smem, st, Q);
      return rows_v2_launch_stage<E, P, ST_RHO>(grid, smem, st, Q);
    default: return cudaErrorInvalidValue;
  }
}

template <int E, int P>
static cudaError_t rows_a_attr() {
  cudaError_t e = rows_v2_attr_stage<E, P, ST_INIT>();
  if (e == cudaSuccess) e = rows_v2_attr_stage<E, P, ST_U>();
  if (e == cudaSuccess) e = rows_v2_attr_stage<E, P, ST_RHO>();
  if (e == cudaSuccess) e = rows_v2_attr_stage<E, P, ST_RHO_PL>();
  return e;
}

static cudaError_t kw_rows_v2_attr_a(int m) {
#define KW_R(E, P) rows_a_attr<E, P>()
  KW_V2_SWITCH(m, KW_R)
#undef KW_R
}

cudaError_t kw_rows_v2_attr(int m) {
  cudaError_t e = kw_rows_v2_attr_a(m);
  if (e == cudaSuccess) e = kw_rows_v2_attr_b(m);
  return e == cudaSuccess ? kw_rows_v2_attr_c(m) : e;
}

cudaError_t kw_rows_v2_launch(int m, int stage, dim3 grid, size_t smem, cudaStream_t st, const RowsParams& Q) {
  if (stage >= ST_ADJ_A) return kw_rows_v2_launch_c(m, stage, grid, smem, st, Q);
  if (stage != ST_INIT && stage != ST_U && stage != ST_RHO) return kw_rows_v2_launch_b(m, stage, grid, smem, st, Q);
#define KW_R(E, P) rows_a_launch<E, P>(stage, grid, smem, st, Q)
  KW_V2_SWITCH(m, KW_R)
#undef KW_R
}
