// Plain (operator-free) instantiations of the TMA-fed axis pass.
#include "kw_axis_tma.cuh"

KW_TMA_DEFINE_KIND(plain, KK_PLAIN)
