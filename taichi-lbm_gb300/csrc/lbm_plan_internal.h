// Plan state shared by the plan and batch translation units (not part of the
// C ABI: callers hold an opaque LbmPlan*).
#pragma once

#include "lbm_fused.cuh"

struct LbmPlan {
  LbmPlanDesc d;
  LbmPlanBuffers b;
  bool bound = false;
  int parity = 0;
  lbm::FusedParams base;
  // two-pass direct step: the flagged segments run on this plan-owned
  // high-priority stream, forked from and joined back to the caller's stream
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  int side_dev = -1;
};

// the parameters of the plan's current step (parity-dependent buffers)
lbm::FusedParams lbm_plan_params(const LbmPlan* pl);
