// Fused kernels with int16 fixed-point shifted storage (steps of 2^-fixed_exp
// of f - w_k rho_ref), fp32 arithmetic, mass-conserving stores.
#include "lbm_fused_launch.cuh"
#include "lbm_batch.cuh"
LBM_INSTANTIATE_STORAGE(LBM_STORE_I16S, 4, 8)
LBM_BATCH_INSTANTIATE(LBM_STORE_I16S, 4, 8)
