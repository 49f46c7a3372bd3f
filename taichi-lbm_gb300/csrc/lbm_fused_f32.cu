// Fused kernels with fp32 population storage (2 or 4 nodes per thread).
#include "lbm_fused_launch.cuh"
#include "lbm_batch.cuh"
LBM_INSTANTIATE_STORAGE(LBM_STORE_F32, 2, 4)
LBM_BATCH_INSTANTIATE(LBM_STORE_F32, 2, 4)
