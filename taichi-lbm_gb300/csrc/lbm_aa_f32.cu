// In-place (AA-pattern) step kernels with fp32 population storage.
#include "lbm_fused_aa.cuh"
LBM_AA_INSTANTIATE(LBM_STORE_F32, 2, 4)
