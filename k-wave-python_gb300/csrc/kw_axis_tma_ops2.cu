// Operator instantiations of the TMA-fed axis pass: the divergence pass and
// the fractional-Laplacian pass.
#include "kw_axis_tma.cuh"

KW_TMA_DEFINE_KIND(div, KK_DIV)
KW_TMA_DEFINE_KIND(nab, KK_NAB)
