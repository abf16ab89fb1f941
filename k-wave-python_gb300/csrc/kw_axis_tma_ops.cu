// Operator instantiations of the TMA-fed axis pass: generic job lists and
// the gradient pass.
#include "kw_axis_tma.cuh"

KW_TMA_DEFINE_KIND(gen, KK_GEN)
KW_TMA_DEFINE_KIND(grad, KK_GRAD)
