// Register row stages, second group: equation of state with fractional
// Laplacians, source scattering, recording of the velocity on the pressure
// grid and the p0 smoothing transforms.
#include "kw_rows_reg.cuh"

template <int E, int P>
static cudaError_t rows_b_launch(int stage, dim3 grid, size_t smem, cudaStream_t st, const RowsParams& Q) {
  switch (stage) {
    case ST_EOS: return rows_v2_launch_stage<E, P, ST_EOS>(grid, smem, st, Q);
    case ST_SRC: return rows_v2_launch_stage<E, P, ST_SRC>(grid, smem, st, Q);
    case ST_P0FFT: return rows_v2_launch_stage<E, P, ST_P0FFT>(grid, smem, st, Q);
    case ST_P0BACK: return rows_v2_launch_stage<E, P, ST_P0BACK>(grid, smem, st, Q);
    case ST_UREC: return rows_v2_launch_stage<E, P, ST_UREC>(grid, smem, st, Q);
    default: return cudaErrorInvalidValue;
  }
}

template <int E, int P>
static cudaError_t rows_b_attr() {
  cudaError_t e = rows_v2_attr_stage<E, P, ST_EOS>();
  if (e == cudaSuccess) e = rows_v2_attr_stage<E, P, ST_SRC>();
  if (e == cudaSuccess) e = rows_v2_attr_stage<E, P, ST_P0FFT>();
  if (e == cudaSuccess) e = rows_v2_attr_stage<E, P, ST_P0BACK>();
  if (e == cudaSuccess) e = rows_v2_attr_stage<E, P, ST_UREC>();
  return e;
}

cudaError_t kw_rows_v2_attr_b(int m) {
#define KW_R(E, P) rows_b_attr<E, P>()
  KW_V2_SWITCH(m, KW_R)
#undef KW_R
}

cudaError_t kw_rows_v2_launch_b(int m, int stage, dim3 grid, size_t smem, cudaStream_t st, const RowsParams& Q) {
#define KW_R(E, P) rows_b_launch<E, P>(stage, grid, smem, st, Q)
  KW_V2_SWITCH(m, KW_R)
#undef KW_R
}
