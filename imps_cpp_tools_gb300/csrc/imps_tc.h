// Tensor-core (tcgen05) execution of planner stages: split-BF16 operands, FP32 TMEM
// accumulation (kernels_tc.cu).
#pragma once
#include <cuda_runtime.h>

#include "imps_internal.h"

namespace imps {
struct TcPlan;
int tc_create(TcPlan** out, const Plan& P, cudaStream_t st);
int tc_destroy(TcPlan* t);
int tc_invalidate(TcPlan* t);  // operator slots changed: re-pack cached operands
int tc_run_stage(TcPlan* t, const Stage& S, const imps_dslots& slots, cudaStream_t st);
}  // namespace imps
