// Register row stages, third group: the stages of the transposed time loop
// (adjoint of the lossless, source-free loop; see kw_generic.cuh:
// adjoint_body for the arithmetic and kw_plan.cu: kw_plan_adjoint for the
// sequence).
#include "kw_rows_reg.cuh"

// The transposed loop has no sources and no unstaggered records: only the
// EXTRA = false form of each stage is compiled.
template <int E, int P, int STAGE>
static cudaError_t adj_launch(dim3 grid, size_t smem, cudaStream_t st, const RowsParams& Q) {
  k_rows_v2<E, P, STAGE, false><<<grid, dim3(Q.R * P), smem, st>>>(Q);
  return cudaGetLastError();
}

template <int E, int P, int STAGE>
static cudaError_t adj_attr() {
  return cudaFuncSetAttribute(k_rows_v2<E, P, STAGE, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
}

template <int E, int P>
static cudaError_t rows_c_launch(int stage, dim3 grid, size_t smem, cudaStream_t st, const RowsParams& Q) {
  switch (stage) {
    case ST_ADJ_A: return adj_launch<E, P, ST_ADJ_A>(grid, smem, st, Q);
    case ST_ADJ_B: return adj_launch<E, P, ST_ADJ_B>(grid, smem, st, Q);
    case ST_ADJ_C: return adj_launch<E, P, ST_ADJ_C>(grid, smem, st, Q);
    case ST_ADJ_D: return adj_launch<E, P, ST_ADJ_D>(grid, smem, st, Q);
    case ST_ADJ_E: return adj_launch<E, P, ST_ADJ_E>(grid, smem, st, Q);
    default: return cudaErrorInvalidValue;
  }
}

template <int E, int P>
static cudaError_t rows_c_attr() {
  cudaError_t e = adj_attr<E, P, ST_ADJ_A>();
  if (e == cudaSuccess) e = adj_attr<E, P, ST_ADJ_B>();
  if (e == cudaSuccess) e = adj_attr<E, P, ST_ADJ_C>();
  if (e == cudaSuccess) e = adj_attr<E, P, ST_ADJ_D>();
  if (e == cudaSuccess) e = adj_attr<E, P, ST_ADJ_E>();
  return e;
}

cudaError_t kw_rows_v2_attr_c(int m) {
#define KW_R(E, P) rows_c_attr<E, P>()
  KW_V2_SWITCH(m, KW_R)
#undef KW_R
}

cudaError_t kw_rows_v2_launch_c(int m, int stage, dim3 grid, size_t smem, cudaStream_t st, const RowsParams& Q) {
#define KW_R(E, P) rows_c_launch<E, P>(stage, grid, smem, st, Q)
  KW_V2_SWITCH(m, KW_R)
#undef KW_R
}
