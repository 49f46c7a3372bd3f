// In-place (AA-pattern) step kernels with 16-bit fixed-point (shifted) population storage.
#include "lbm_fused_aa.cuh"
LBM_AA_INSTANTIATE(LBM_STORE_I16S, 4, 8)
