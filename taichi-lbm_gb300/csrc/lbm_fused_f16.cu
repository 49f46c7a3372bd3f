// Fused kernels with fp16 shifted storage (f - w_k), fp32 arithmetic.
#include "lbm_fused_launch.cuh"
#include "lbm_batch.cuh"
LBM_INSTANTIATE_STORAGE(LBM_STORE_F16S, 4, 8)
LBM_BATCH_INSTANTIATE(LBM_STORE_F16S, 4, 8)
