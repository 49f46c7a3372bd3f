// Fused kernels with bf16 shifted storage (f - w_k), fp32 arithmetic.
#include "lbm_fused_launch.cuh"
LBM_INSTANTIATE_STORAGE(LBM_STORE_BF16S, 4, 8)
