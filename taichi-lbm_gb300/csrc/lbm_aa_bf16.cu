// In-place (AA-pattern) step kernels with bf16 (shifted) population storage.
#include "lbm_fused_aa.cuh"
LBM_AA_INSTANTIATE(LBM_STORE_BF16S, 4, 8)
