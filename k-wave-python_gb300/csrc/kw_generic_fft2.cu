// The generic-length row and axis kernels (kw_generic.cuh) on the two-level
// FFT schedule (kw_fft.cuh: fft2_smem), for plans whose lengths take it.
#include "kw_generic.cuh"

KW_GENERIC_DEFINE(1)
